// cgs_fft.cu -- oversampled FFT passes of the NFFT, one axis per launch.
//
// Each CTA transforms B columns of data[outer][L][inner] along L entirely in
// one shared buffer (mixed-radix Stockham, radices 2/4/8 in registers, 3/5/7
// through the twiddle table).  Zero padding (image side ->
// oversampled grid) and cropping (grid -> image side) are index maps in the
// load / store phases, so padded zeros are never read from or written to HBM.
// The first forward pass also fuses the coil expansion S_c . x, the damping
// mask and the deapodisation 1/phihut (NFFT3's PRE_PHI_HUT step), and the last
// inverse pass fuses the deapodisation: the FFT-side work of the reference's
// nfft_trafo / nfft_adjoint (src/matrix/ft/NFFTTraits.hpp:176-204).
#include <atomic>
#include <type_traits>

#include "cgs_internal.cuh"

#include <initializer_list>

namespace cgs {

namespace {

constexpr int kThreads = 256;

// Kernel attributes hold per device: `devs` has bit d set once device d's
// attributes are set (a process may drive plans on several devices, from
// several threads).
inline bool attr_needed(const std::atomic<uint64_t> &devs)
{
    int dev = 0;
    cudaGetDevice(&dev);
    return !(devs.load(std::memory_order_acquire) & (1ull << (dev & 63)));
}

inline void attr_done(std::atomic<uint64_t> &devs)
{
    int dev = 0;
    cudaGetDevice(&dev);
    devs.fetch_or(1ull << (dev & 63), std::memory_order_release);
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// c + w * v on both FP32 lanes with one paired FMA (fma.rn.f32x2)
__device__ __forceinline__ float2 pfma(float2 w, float2 v, float2 c)
{
    unsigned long long r;
    const unsigned long long a = *reinterpret_cast<const unsigned long long *>(&w);
    const unsigned long long b = *reinterpret_cast<const unsigned long long *>(&v);
    const unsigned long long d = *reinterpret_cast<const unsigned long long *>(&c);
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(d));
    return *reinterpret_cast<const float2 *>(&r);
}
// complex add and subtract as one paired FMA each: b * (+-1) is exact, so the
// result has the rounding of the two FP32 adds, in half the instructions
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return pfma(b, make_float2(1.f, 1.f), a); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return pfma(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by -i (sign<0) or +i (sign>0)
__device__ __forceinline__ float2 mul_i(float2 a, int sign)
{
    return sign < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}

template <int R>
__device__ __forceinline__ void bfly(float2 *v, int sign, const float2 *tw, int nR)
{
    if constexpr (R == 2) {
        float2 a = v[0], b = v[1];
        v[0] = cadd(a, b); v[1] = csub(a, b);
    } else if constexpr (R == 4) {
        float2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
        float2 b0 = cadd(v[1], v[3]), b1 = mul_i(csub(v[1], v[3]), sign);
        v[0] = cadd(a0, b0); v[2] = csub(a0, b0);
        v[1] = cadd(a1, b1); v[3] = csub(a1, b1);
    } else if constexpr (R == 8) {
        // two radix-4 on even/odd samples, then the radix-2 combine with w8^k
        float2 e[4] = {v[0], v[2], v[4], v[6]};
        float2 o[4] = {v[1], v[3], v[5], v[7]};
        bfly<4>(e, sign, tw, nR);
        bfly<4>(o, sign, tw, nR);
        const float h = 0.70710678118654752f;
        // w8^1 = (1 - i)/sqrt2 for sign -1, (1 + i)/sqrt2 for sign +1
        float2 o1 = o[1], o2 = o[2], o3 = o[3];
        o1 = sign < 0 ? make_float2(h * (o1.x + o1.y), h * (o1.y - o1.x))
                      : make_float2(h * (o1.x - o1.y), h * (o1.y + o1.x));
        o2 = mul_i(o2, sign);
        o3 = sign < 0 ? make_float2(h * (-o3.x + o3.y), h * (-o3.y - o3.x))
                      : make_float2(h * (-o3.x - o3.y), h * (-o3.y + o3.x));
        v[0] = cadd(e[0], o[0]); v[4] = csub(e[0], o[0]);
        v[1] = cadd(e[1], o1);   v[5] = csub(e[1], o1);
        v[2] = cadd(e[2], o2);   v[6] = csub(e[2], o2);
        v[3] = cadd(e[3], o3);   v[7] = csub(e[3], o3);
    } else {
        // generic radix through the length-n twiddle table: W_R^{rq} = tw[(rq mod R) * nR]
        float2 out[R];
#pragma unroll
        for (int q = 0; q < R; ++q) {
            float2 acc = v[0];
#pragma unroll
            for (int r = 1; r < R; ++r) {
                float2 w = tw[((r * q) % R) * nR];
                if (sign > 0) w.y = -w.y;
                acc = cadd(acc, cmul(v[r], w));
            }
            out[q] = acc;
        }
#pragma unroll
        for (int q = 0; q < R; ++q) v[q] = out[q];
    }
}

// Elements of one CTA's column block: n * B <= kElems, so every thread holds at
// most kElems / kThreads values of a pass in registers.
constexpr int kElems = 2048;

// One in-place Stockham pass: every thread first reads and transforms all of
// its butterflies into registers, then (after a barrier) writes them back, so
// a single shared buffer serves as source and destination.
template <int R> struct Log2R { static constexpr int v = R == 8 ? 3 : (R == 4 ? 2 : (R == 2 ? 1 : 0)); };

template <int R, bool POW2>
__device__ __forceinline__ void stockham_pass(float2 *buf, const float2 *tw, int n, int Ns, int logNs, int B,
                                              int logB, int P, int sign)
{
    constexpr int NB = (kElems / kThreads + R - 1) / R;
    const int nR = n / R;
    const int step = POW2 ? (n >> (logNs + Log2R<R>::v)) : n / (Ns * R);
    const int total = B * nR;
    float2 v[NB][R];
#pragma unroll
    for (int t = 0; t < NB; ++t) {
        const int q = threadIdx.x + t * kThreads;
        if (q < total) {
            const int b = POW2 ? (q & (B - 1)) : q % B;
            const int j = POW2 ? (q >> logB) : q / B;
            const int k = POW2 ? (j & (Ns - 1)) : j % Ns;
#pragma unroll
            for (int r = 0; r < R; ++r) v[t][r] = buf[(j + r * nR) * P + b];
            if (Ns > 1) {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    float2 w = tw[k * r * step];
                    if (sign > 0) w.y = -w.y;
                    v[t][r] = cmul(v[t][r], w);
                }
            }
            bfly<R>(v[t], sign, tw, nR);
        }
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < NB; ++t) {
        const int q = threadIdx.x + t * kThreads;
        if (q < total) {
            const int b = POW2 ? (q & (B - 1)) : q % B;
            const int j = POW2 ? (q >> logB) : q / B;
            const int k = POW2 ? (j & (Ns - 1)) : j % Ns;
            const int base = (POW2 ? ((j >> logNs) << (logNs + Log2R<R>::v)) : (j / Ns) * Ns * R) + k;
#pragma unroll
            for (int r = 0; r < R; ++r) buf[(base + r * Ns) * P + b] = v[t][r];
        }
    }
    __syncthreads();
}

__device__ __forceinline__ int in_pos_to_axis(int pos, int Lin, int n, int centred)
{
    if (!centred) return pos;
    const int h = Lin >> 1;
    if (pos < h) return pos + h;
    if (pos >= n - h) return pos - n + h;
    return -1;
}

__device__ __forceinline__ int out_axis_to_pos(int a, int Lout, int n, int centred)
{
    if (!centred) return a;
    const int h = Lout >> 1;
    return a < h ? n - h + a : a - h;
}

// MIXED = false: radices 8/4/2 only, every size a power of two, index math by
// shifts; MIXED = true: also radices 3/5/7 with general division
template <bool MIXED>
__global__ void __launch_bounds__(kThreads, MIXED ? 1 : 3)
axis_fft_kernel(const __grid_constant__ AxisPass p, int BO, int BI, int64_t nib)
{
    extern __shared__ float2 smem[];
    constexpr bool POW2 = !MIXED;
    const int n = p.n;
    const int B = BO * BI;
    const int P = B + 1;
    const int logB = 31 - __clz(B), logBI = 31 - __clz(BI), logn = 31 - __clz(n);
    float2 *tw = smem;
    float2 *bufA = smem + n;
    float *dcol = reinterpret_cast<float *>(bufA + (size_t)n * P);  // [B] outer deapodisation per column

    const int64_t blk = blockIdx.x;
    const int64_t ib0 = (blk % nib) * BI;
    const int64_t ob0 = (blk / nib) * BO;

    for (int t = threadIdx.x; t < n; t += kThreads) tw[t] = p.tw[t];
    const bool fused = (p.load_mode == LOAD_IMAGE) || (p.store_mode == STORE_DEAPOD);
    if (fused) {
        for (int b = threadIdx.x; b < B; b += kThreads) {
            const int64_t o = ob0 + (POW2 ? (b >> logBI) : b / BI);
            float d = 1.f;
            if (o < p.outer) {
                if (p.deap_o1) d *= p.deap_o1[o % p.o1_len];
                if (p.deap_o0) d *= p.deap_o0[o / p.o1_len];
            }
            dcol[b] = d;
        }
        __syncthreads();
    }

    // ---- load: fill all n positions of every column (zeros where padded) ----
    const int tot = n * B;
    const bool pos_fast = (BI == 1);
    // batches of kUnroll independent global loads per thread keep enough bytes
    // in flight to stream at HBM rate
    constexpr int kUnroll = 8;
    for (int e0 = threadIdx.x; e0 < tot; e0 += kThreads * kUnroll) {
        float2 v[kUnroll];
        int slot[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const int e = e0 + u * kThreads;
            v[u] = make_float2(0.f, 0.f);
            slot[u] = -1;
            if (e >= tot) continue;
            int pos, b;
            if (pos_fast) { b = POW2 ? (e >> logn) : e / n; pos = POW2 ? (e & (n - 1)) : e % n; }
            else { pos = POW2 ? (e >> logB) : e / B; b = POW2 ? (e & (B - 1)) : e % B; }
            slot[u] = pos * P + b;
            const int64_t o = ob0 + (POW2 ? (b >> logBI) : b / BI);
            const int64_t i = ib0 + (POW2 ? (b & (BI - 1)) : b % BI);
            if (o < p.outer && i < p.inner) {
                const int a = in_pos_to_axis(pos, p.Lin, n, p.in_centred);
                if (a >= 0) {
                    const int64_t pix = o * p.Lin + a;
                    if (p.load_mode == LOAD_PLAIN) {
                        v[u] = p.src[pix * p.inner + i];
                    } else {
                        float2 x = p.img_per_coil ? (p.coil_major ? p.img[i * p.coil_major + pix] : p.img[pix * p.inner + i])
                                                  : p.img[pix];
                        if (p.sens) x = cmul(x, p.sens[pix * p.inner + i]);
                        float sc = dcol[b] * (p.deap_ax ? p.deap_ax[a] : 1.f);
                        if (p.mask) sc *= p.mask[pix];
                        v[u] = cscale(x, sc);
                    }
                }
            }
        }
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
            if (slot[u] >= 0) bufA[slot[u]] = v[u];
    }
    __syncthreads();

    // ---- Stockham passes, in place in shared memory ----
    const int rounds = p.toep_k ? 2 : 1;
    for (int round = 0; round < rounds; ++round) {
        const int sign = round == 0 ? p.sign : +1;
        int Ns = 1, logNs = 0;
        for (int s = 0; s < p.nfac; ++s) {
            const int R = p.fac[s];
            switch (R) {
                case 8: stockham_pass<8, POW2>(bufA, tw, n, Ns, logNs, B, logB, P, sign); logNs += 3; break;
                case 4: stockham_pass<4, POW2>(bufA, tw, n, Ns, logNs, B, logB, P, sign); logNs += 2; break;
                case 2: stockham_pass<2, POW2>(bufA, tw, n, Ns, logNs, B, logB, P, sign); logNs += 1; break;
                case 3: if (MIXED) stockham_pass<3, false>(bufA, tw, n, Ns, logNs, B, logB, P, sign); break;
                case 5: if (MIXED) stockham_pass<5, false>(bufA, tw, n, Ns, logNs, B, logB, P, sign); break;
                case 7: if (MIXED) stockham_pass<7, false>(bufA, tw, n, Ns, logNs, B, logB, P, sign); break;
                default: break;  // host rejects other primes
            }
            Ns *= R;
        }
        if (round == 0 && p.toep_k) {
            // pointwise multiply by the real Toeplitz kernel of this column block
            const int64_t kstride = p.inner / p.toep_nc;
            for (int e = threadIdx.x; e < tot; e += kThreads) {
                int pos, b;
                if (pos_fast) { b = POW2 ? (e >> logn) : e / n; pos = POW2 ? (e & (n - 1)) : e % n; }
                else { pos = POW2 ? (e >> logB) : e / B; b = POW2 ? (e & (B - 1)) : e % B; }
                const int64_t i = ib0 + (POW2 ? (b & (BI - 1)) : b % BI);
                if (i < p.inner) bufA[pos * P + b] = cscale(bufA[pos * P + b], p.toep_k[pos * kstride + i / p.toep_nc]);
            }
            __syncthreads();
        }
    }
    const float2 *src = bufA;

    // ---- store: Lout positions of every column ----
    const int totO = p.Lout * B;
    for (int e = threadIdx.x; e < totO; e += kThreads) {
        int a, b;
        if (pos_fast) { b = e / p.Lout; a = e % p.Lout; }
        else { a = POW2 ? (e >> logB) : e / B; b = POW2 ? (e & (B - 1)) : e % B; }
        const int64_t o = ob0 + (POW2 ? (b >> logBI) : b / BI);
        const int64_t i = ib0 + (POW2 ? (b & (BI - 1)) : b % BI);
        if (o >= p.outer || i >= p.inner) continue;
        const int pos = out_axis_to_pos(a, p.Lout, n, p.out_centred);
        float2 v = src[pos * P + b];
        const int64_t pix = o * p.Lout + a;
        if (p.store_mode == STORE_DEAPOD) v = cscale(v, dcol[b] * (p.deap_ax ? p.deap_ax[a] : 1.f));
        if (p.coil_major && p.store_mode == STORE_DEAPOD) p.dst[i * p.coil_major + pix] = v;
        else p.dst[pix * p.inner + i] = v;
    }
}

// ---------------------------------------------------------------------------
// Passes with the length N and the column count B = 2^LOGB fixed at compile
// time (N B <= 4096 values per CTA and a multiple of 256, so every thread
// holds the same number).  Every thread owns one column of the block and the
// rows r0, r0 + 256/B, ..., so its global addresses are one column base plus
// a row stride; the Stockham passes (radix 7, 5, 3 for the odd part of N,
// then 8, 4, 2) index shared memory with compile-time arithmetic.  Same
// fusions as axis_fft_kernel: pad/crop index maps, the image-side load (coil
// expansion, mask, deapodisation), the deapodising store and the Toeplitz
// round.  Instantiated for the powers of two 64..1024 and the grid sizes with
// small odd factors that 2N oversampling of N = 48..480 produces.
// ---------------------------------------------------------------------------
constexpr int kCtElems = 4096;

__host__ __device__ constexpr int ct_next_radix(int rem)
{
    return rem % 7 == 0 ? 7 : rem % 5 == 0 ? 5 : rem % 3 == 0 ? 3 : rem % 8 == 0 ? 8 : rem % 4 == 0 ? 4 : 2;
}

__host__ __device__ constexpr int ct_logb(int n)
{
    int lb = 6;
    while (lb > 0 && (n << lb) > kCtElems) --lb;
    return lb;
}

// Shared-memory slot of (row, column): rows of B values with no padding; for
// B <= 8 (a row fills at most half the banks) one spare row after every 8, so
// that both consecutive rows and rows 8 apart (the first pass writes stride
// R = 8) fall in different bank groups.
template <int LOGB>
__device__ __forceinline__ int ct_slot(int row, int b)
{
    if constexpr (LOGB <= 3) return ((row + (row >> 3)) << LOGB) + b;
    else return (row << LOGB) + b;
}

template <int N, int LOGB>
__host__ __device__ constexpr int ct_rows()
{
    return LOGB <= 3 ? N + (N + 7) / 8 : N;
}

// Butterfly with the transform direction fixed at compile time (S = -1
// forward, +1 inverse): no selects between the two directions' constants.
template <int R, int S>
__device__ __forceinline__ void ct_bfly(float2 *v, const float2 *tw, int nR)
{
    if constexpr (R == 2) {
        float2 a = v[0], b = v[1];
        v[0] = cadd(a, b); v[1] = csub(a, b);
    } else if constexpr (R == 4) {
        float2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
        float2 b0 = cadd(v[1], v[3]), d = csub(v[1], v[3]);
        float2 b1 = S < 0 ? make_float2(d.y, -d.x) : make_float2(-d.y, d.x);   // S i d
        v[0] = cadd(a0, b0); v[2] = csub(a0, b0);
        v[1] = cadd(a1, b1); v[3] = csub(a1, b1);
    } else if constexpr (R == 8) {
        float2 e[4] = {v[0], v[2], v[4], v[6]};
        float2 o[4] = {v[1], v[3], v[5], v[7]};
        ct_bfly<4, S>(e, tw, nR);
        ct_bfly<4, S>(o, tw, nR);
        const float h = 0.70710678118654752f;
        float2 o1 = o[1], o2 = o[2], o3 = o[3];
        if constexpr (S < 0) {   // w8 = (1 - i)/sqrt2
            o1 = make_float2(h * (o1.x + o1.y), h * (o1.y - o1.x));
            o2 = make_float2(o2.y, -o2.x);
            o3 = make_float2(h * (-o3.x + o3.y), h * (-o3.y - o3.x));
        } else {                 // w8 = (1 + i)/sqrt2
            o1 = make_float2(h * (o1.x - o1.y), h * (o1.y + o1.x));
            o2 = make_float2(-o2.y, o2.x);
            o3 = make_float2(h * (-o3.x - o3.y), h * (-o3.y + o3.x));
        }
        v[0] = cadd(e[0], o[0]); v[4] = csub(e[0], o[0]);
        v[1] = cadd(e[1], o1);   v[5] = csub(e[1], o1);
        v[2] = cadd(e[2], o2);   v[6] = csub(e[2], o2);
        v[3] = cadd(e[3], o3);   v[7] = csub(e[3], o3);
    } else {
        bfly<R>(v, S, tw, nR);
    }
}

// Slot of rows row0 + r * D (r = 0..R-1) as slot(row0) + r * stride when the
// padding (a spare row after every 8, ct_slot) shifts them uniformly: D a
// multiple of 8, or D = 1 with row0 a multiple of 8 and R <= 8.  0: no
// uniform stride (the caller computes each slot).
template <int LOGB, int D, int R>
__host__ __device__ constexpr int ct_stride(bool row0_mult8)
{
    if constexpr (LOGB > 3) return D << LOGB;
    else if constexpr (D % 8 == 0) return (D + D / 8) << LOGB;
    else return (D == 1 && R <= 8 && row0_mult8) ? (1 << LOGB) : 0;
}

template <int N, int LOGB, int R, int NS, int S>
__device__ __forceinline__ void ct_pass_s(float2 *buf, const float2 *tw)
{
    constexpr int B = 1 << LOGB;
    constexpr int NR = N / R;
    constexpr int TB = B * NR;
    constexpr int NBF = (TB + kThreads - 1) / kThreads;
    constexpr int STEP = N / (NS * R);
    constexpr int SL = ct_stride<LOGB, NR, R>(false);         // load rows j + r NR
    constexpr int SS = ct_stride<LOGB, NS, R>(NS == 1 && R == 8);  // store rows base + r NS (base = 8 j when NS = 1)
    float2 v[NBF][R];
#pragma unroll
    for (int t = 0; t < NBF; ++t) {
        const int q = threadIdx.x + t * kThreads;
        if (TB % kThreads != 0 && q >= TB) continue;
        const int b = q & (B - 1), j = q >> LOGB, k = j % NS;
        if constexpr (SL > 0) {
            const float2 *src = buf + ct_slot<LOGB>(j, b);
#pragma unroll
            for (int r = 0; r < R; ++r) v[t][r] = src[r * SL];
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) v[t][r] = buf[ct_slot<LOGB>(j + r * NR, b)];
        }
        if constexpr (NS > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                float2 w = tw[k * r * STEP];
                if constexpr (S > 0) w.y = -w.y;
                v[t][r] = cmul(v[t][r], w);
            }
        }
        ct_bfly<R, S>(v[t], tw, NR);
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < NBF; ++t) {
        const int q = threadIdx.x + t * kThreads;
        if (TB % kThreads != 0 && q >= TB) continue;
        const int b = q & (B - 1), j = q >> LOGB, k = j % NS;
        const int base = (j / NS) * NS * R + k;
        if constexpr (SS > 0) {
            float2 *dst = buf + ct_slot<LOGB>(base, b);
#pragma unroll
            for (int r = 0; r < R; ++r) dst[r * SS] = v[t][r];
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) buf[ct_slot<LOGB>(base + r * NS, b)] = v[t][r];
        }
    }
    __syncthreads();
}

// A pass whose butterfly inputs (IN) or outputs (OUT) stay in the thread's
// registers instead of shared memory.  Butterfly t of a thread covers rows
// j + r N/R with j = r0 + t RSTEP, the rows the thread loads from and stores
// to global memory (r0 + u RSTEP): register u = t + r NBF.  IN holds for the
// first pass (NS = 1), OUT for the last (NS R = N), where the stored row of
// butterfly output r is j + r NS = j + r N/R as well.
template <int N, int LOGB, int R, int NS, int S, bool IN, bool OUT, int EPT>
__device__ __forceinline__ void ct_pass_r(float2 *buf, const float2 *tw, float2 (&reg)[EPT])
{
    constexpr int B = 1 << LOGB;
    constexpr int NR = N / R;
    constexpr int TB = B * NR;
    constexpr int NBF = (TB + kThreads - 1) / kThreads;
    constexpr int STEP = N / (NS * R);
    constexpr int SL = ct_stride<LOGB, NR, R>(false);
    constexpr int SS = ct_stride<LOGB, NS, R>(NS == 1 && R == 8);
    static_assert(!(IN || OUT) || (TB % kThreads == 0 && NBF * R == EPT), "register pass layout");
    static_assert(!IN || NS == 1, "registers in: the first pass only");
    static_assert(!OUT || NS * R == N, "registers out: the last pass only");
    float2 v[NBF][R];
#pragma unroll
    for (int t = 0; t < NBF; ++t) {
        const int q = threadIdx.x + t * kThreads;
        if (TB % kThreads != 0 && q >= TB) continue;
        const int b = q & (B - 1), j = q >> LOGB, k = j % NS;
        if constexpr (IN) {
#pragma unroll
            for (int r = 0; r < R; ++r) v[t][r] = reg[t + r * NBF];
        } else if constexpr (SL > 0) {
            const float2 *src = buf + ct_slot<LOGB>(j, b);
#pragma unroll
            for (int r = 0; r < R; ++r) v[t][r] = src[r * SL];
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) v[t][r] = buf[ct_slot<LOGB>(j + r * NR, b)];
        }
        if constexpr (NS > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                float2 w = tw[k * r * STEP];
                if constexpr (S > 0) w.y = -w.y;
                v[t][r] = cmul(v[t][r], w);
            }
        }
        ct_bfly<R, S>(v[t], tw, NR);
    }
    if constexpr (OUT) {
#pragma unroll
        for (int t = 0; t < NBF; ++t)
#pragma unroll
            for (int r = 0; r < R; ++r) reg[t + r * NBF] = v[t][r];
        return;
    }
    if constexpr (!IN) __syncthreads();  // this pass's reads are done before the in-place stores
#pragma unroll
    for (int t = 0; t < NBF; ++t) {
        const int q = threadIdx.x + t * kThreads;
        if (TB % kThreads != 0 && q >= TB) continue;
        const int b = q & (B - 1), j = q >> LOGB, k = j % NS;
        const int base = (j / NS) * NS * R + k;
        if constexpr (SS > 0) {
            float2 *dst = buf + ct_slot<LOGB>(base, b);
#pragma unroll
            for (int r = 0; r < R; ++r) dst[r * SS] = v[t][r];
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) buf[ct_slot<LOGB>(base + r * NS, b)] = v[t][r];
        }
    }
    __syncthreads();
}

template <int N, int LOGB, int NS, int S, bool IN, bool OUT, int EPT>
__device__ __forceinline__ void ct_passes_r(float2 *buf, const float2 *tw, float2 (&reg)[EPT])
{
    if constexpr (NS < N) {
        constexpr int R = ct_next_radix(N / NS);
        ct_pass_r<N, LOGB, R, NS, S, IN && NS == 1, OUT && NS * R == N, EPT>(buf, tw, reg);
        ct_passes_r<N, LOGB, NS * R, S, IN, OUT, EPT>(buf, tw, reg);
    }
}

// whether the first and last passes can keep their data in registers (every
// thread holds whole butterflies: B N / R a multiple of the block size)
template <int N, int LOGB, int NS = 1>
__host__ __device__ constexpr bool ct_reg_ok()
{
    if constexpr (NS >= N) {
        return true;
    } else {
        constexpr int R = ct_next_radix(N / NS);
        constexpr bool edge = NS == 1 || NS * R == N;
        return (!edge || (((N / R) << LOGB) % kThreads == 0)) && ct_reg_ok<N, LOGB, NS * R>();
    }
}

template <int N, int LOGB, int NS, int S>
__device__ __forceinline__ void ct_passes_s(float2 *buf, const float2 *tw)
{
    if constexpr (NS < N) {
        constexpr int R = ct_next_radix(N / NS);
        ct_pass_s<N, LOGB, R, NS, S>(buf, tw);
        ct_passes_s<N, LOGB, NS * R, S>(buf, tw);
    }
}

template <int N, int LOGB, int R, int NS>
__device__ __forceinline__ void ct_pass(float2 *buf, const float2 *tw, int sign)
{
    constexpr int B = 1 << LOGB;
    constexpr int NR = N / R;
    constexpr int TB = B * NR;                           // butterflies in the block
    constexpr int NBF = (TB + kThreads - 1) / kThreads;  // per thread
    constexpr int STEP = N / (NS * R);                   // twiddle index stride
    float2 v[NBF][R];
#pragma unroll
    for (int t = 0; t < NBF; ++t) {
        const int q = threadIdx.x + t * kThreads;
        if (TB % kThreads != 0 && q >= TB) continue;
        const int b = q & (B - 1), j = q >> LOGB, k = j % NS;
#pragma unroll
        for (int r = 0; r < R; ++r) v[t][r] = buf[ct_slot<LOGB>(j + r * NR, b)];
        if constexpr (NS > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                float2 w = tw[k * r * STEP];
                if (sign > 0) w.y = -w.y;
                v[t][r] = cmul(v[t][r], w);
            }
        }
        bfly<R>(v[t], sign, tw, NR);
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < NBF; ++t) {
        const int q = threadIdx.x + t * kThreads;
        if (TB % kThreads != 0 && q >= TB) continue;
        const int b = q & (B - 1), j = q >> LOGB, k = j % NS;
        const int base = (j / NS) * NS * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) buf[ct_slot<LOGB>(base + r * NS, b)] = v[t][r];
    }
    __syncthreads();
}

template <int N, int LOGB, int NS>
__device__ __forceinline__ void ct_passes(float2 *buf, const float2 *tw, int sign)
{
    if constexpr (NS < N) {
        constexpr int R = ct_next_radix(N / NS);
        ct_pass<N, LOGB, R, NS>(buf, tw, sign);
        ct_passes<N, LOGB, NS * R>(buf, tw, sign);
    }
}

template <int N, int LOGB, int S>
__global__ void __launch_bounds__(kThreads, ((N & (N - 1)) == 0) ? 4 : 3)
axis_fft_ct_kernel(const __grid_constant__ AxisPass p, int logBI, int64_t nib)
{
    constexpr int B = 1 << LOGB;
    constexpr int EPT = (N * B) / kThreads;    // values per thread
    constexpr int RSTEP = kThreads / B;        // rows between a thread's values
    static_assert((N * B) % kThreads == 0 && EPT * RSTEP == N, "rows must tile the transform");
    extern __shared__ float2 smem[];
    float2 *tw = smem;                          // [N]
    float2 *buf = smem + N;                     // [rows][B], see ct_slot
    const int b = threadIdx.x & (B - 1), r0 = threadIdx.x >> LOGB;
    const int64_t blk = blockIdx.x;
    const int64_t o = ((blk / nib) << (LOGB - logBI)) + (b >> logBI);
    const int64_t i = ((blk % nib) << logBI) + (b & ((1 << logBI) - 1));
    const bool col_ok = (o < p.outer) && (i < p.inner);
    // the twiddle table comes in by cp.async, so the column loads below are
    // issued without waiting for it (it is waited for before the barrier that
    // precedes the first butterfly)
    if constexpr (N % 2 == 0) {
        for (int t = threadIdx.x; t < N / 2; t += kThreads) {
            const unsigned d = (unsigned)__cvta_generic_to_shared(tw + 2 * t);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(p.tw + 2 * t) : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    } else {
        for (int t = threadIdx.x; t < N; t += kThreads) tw[t] = p.tw[t];
    }
    // the twiddles are plan constants; everything below uses the previous
    // kernel's output or buffers it may still read
    pdl_wait();
    pdl_trigger();
    float dcol = 1.f;  // outer-dimension deapodisation of this column (fused passes)
    if (col_ok && (p.load_mode == LOAD_IMAGE || p.store_mode == STORE_DEAPOD)) {
        if (p.deap_o1) dcol *= p.deap_o1[o % p.o1_len];
        if (p.deap_o0) dcol *= p.deap_o0[o / p.o1_len];
    }
    {
        // a thread's values differ only in the axis index a: the column's base
        // pointers and strides are set once, the load mode is branched on once
        float2 v[EPT];
#pragma unroll
        for (int u = 0; u < EPT; ++u) v[u] = make_float2(0.f, 0.f);
        if (col_ok && p.load_mode == LOAD_PLAIN) {
            const float2 *src = p.src + (o * p.Lin) * p.inner + i;
            const int64_t sst = p.inner;
#pragma unroll
            for (int u = 0; u < EPT; ++u) {
                const int a = in_pos_to_axis(r0 + u * RSTEP, p.Lin, N, p.in_centred);
                if (a >= 0) v[u] = src[a * sst];
            }
        } else if (col_ok) {
            const bool cm = p.img_per_coil && p.coil_major;
            const float2 *img = !p.img_per_coil ? p.img + o * p.Lin
                                : cm ? p.img + i * p.coil_major + o * p.Lin
                                     : p.img + (o * p.Lin) * p.inner + i;
            const int64_t ist = (p.img_per_coil && !cm) ? p.inner : 1;
            const float2 *sens = p.sens ? p.sens + (o * p.Lin) * p.inner + i : nullptr;
            const float *mask = p.mask ? p.mask + o * p.Lin : nullptr;
            const float *dax = p.deap_ax;
            const int64_t inner = p.inner;
#pragma unroll
            for (int u = 0; u < EPT; ++u) {
                const int a = in_pos_to_axis(r0 + u * RSTEP, p.Lin, N, p.in_centred);
                if (a < 0) continue;
                float2 x = img[a * ist];
                if (sens) x = cmul(x, sens[a * inner]);
                float sc = dax ? dcol * dax[a] : dcol;
                if (mask) sc *= mask[a];
                v[u] = cscale(x, sc);
            }
        }
        if constexpr (N % 2 == 0) asm volatile("cp.async.wait_group 0;" ::: "memory");
        if constexpr (ct_reg_ok<N, LOGB>()) {
            // The first pass takes its inputs from these registers.  Without a
            // Toeplitz round the last pass leaves its outputs in them: row
            // r0 + u RSTEP in v[u], which is what an uncentred store wants; a
            // centred crop to Lout = N/2 (twofold oversampling) stores row
            // a + 3N/4 (a < N/4) or a - N/4 at a = r0 + u RSTEP, which is
            // v[(u + 3 EPT/4) mod EPT] of the same thread.
            const bool rot_ok = (EPT % 4 == 0) && 2 * p.Lout == N;
            // the twiddle table is complete before any butterfly reads it (the
            // radix 3, 5 and 7 butterflies take their roots from it)
            __syncthreads();
            if (!p.toep_k && (!p.out_centred || rot_ok)) {
                ct_passes_r<N, LOGB, 1, S, true, true, EPT>(buf, tw, v);
                if (!col_ok) return;
                const bool dp = p.store_mode == STORE_DEAPOD;
                const bool cm = dp && p.coil_major;
                float2 *dst = cm ? p.dst + i * p.coil_major + o * p.Lout : p.dst + (o * p.Lout) * p.inner + i;
                const int64_t dstr = cm ? 1 : p.inner;
                const float *dax = dp ? p.deap_ax : nullptr;
                auto store = [&](auto rot) {
                    constexpr int ROT = decltype(rot)::value;
#pragma unroll
                    for (int u = 0; u < EPT; ++u) {
                        const int a = r0 + u * RSTEP;
                        if (a >= p.Lout) continue;
                        float2 x = v[(u + ROT) % EPT];
                        if (dp) x = cscale(x, dax ? dcol * dax[a] : dcol);
                        dst[a * dstr] = x;
                    }
                };
                if (p.out_centred) store(std::integral_constant<int, (3 * EPT / 4) % EPT>{});
                else store(std::integral_constant<int, 0>{});
                return;
            }
            ct_passes_r<N, LOGB, 1, S, true, false, EPT>(buf, tw, v);
        } else {
#pragma unroll
            for (int u = 0; u < EPT; ++u) buf[ct_slot<LOGB>(r0 + u * RSTEP, b)] = v[u];
            __syncthreads();
            ct_passes_s<N, LOGB, 1, S>(buf, tw);
        }
    }
    if (p.toep_k) {
        // pointwise multiply by the real Toeplitz kernel, then transform back
        const int64_t kstride = p.inner / p.toep_nc;
        if (i < p.inner) {
#pragma unroll
            for (int u = 0; u < EPT; ++u) {
                const int pos = r0 + u * RSTEP;
                buf[ct_slot<LOGB>(pos, b)] = cscale(buf[ct_slot<LOGB>(pos, b)], p.toep_k[pos * kstride + i / p.toep_nc]);
            }
        }
        __syncthreads();
        ct_passes_s<N, LOGB, 1, +1>(buf, tw);
    }
    if (!col_ok) return;
    const bool dp = p.store_mode == STORE_DEAPOD;
    const bool cm = dp && p.coil_major;
    float2 *dst = cm ? p.dst + i * p.coil_major + o * p.Lout : p.dst + (o * p.Lout) * p.inner + i;
    const int64_t dstr = cm ? 1 : p.inner;
    const float *dax = dp ? p.deap_ax : nullptr;
#pragma unroll
    for (int u = 0; u < EPT; ++u) {
        const int a = r0 + u * RSTEP;
        if (a >= p.Lout) continue;
        const int pos = out_axis_to_pos(a, p.Lout, N, p.out_centred);
        float2 v = buf[ct_slot<LOGB>(pos, b)];
        if (dp) v = cscale(v, dax ? dcol * dax[a] : dcol);
        dst[a * dstr] = v;
    }
}

// A narrower column block (1024 values, 4 per thread) for the power-of-two
// lengths up to 256: a pass over few columns (the 256^2 image of the
// circulant preconditioner: 16 blocks of 16 columns) then spreads over 4x as
// many blocks.  Each column's butterflies are the same, so the results are too.
__host__ __device__ constexpr int ct_logb_small(int n)
{
    if (n > 256 || (n & (n - 1)) != 0) return -1;
    int lb = 0;
    while ((n << (lb + 1)) <= 1024) ++lb;
    return lb < ct_logb(n) ? lb : -1;
}
constexpr int64_t kCtFewBlocks = 152;  // below this many blocks (one per SM) take the narrow block

// column blocks of a pass with 2^LOGB columns per block
struct CtGrid {
    int logBI;
    int64_t nib, nblocks;
};
inline CtGrid ct_grid(const AxisPass &p, int LOGB)
{
    const int B = 1 << LOGB;
    CtGrid g{};
    g.logBI = 0;  // largest power of two <= min(inner, B)
    while ((1 << (g.logBI + 1)) <= B && (int64_t)(1 << (g.logBI + 1)) <= p.inner) ++g.logBI;
    g.nib = (p.inner + (1 << g.logBI) - 1) >> g.logBI;
    const int64_t BO = B >> g.logBI;
    const int64_t nob = (p.outer + BO - 1) / BO;
    g.nblocks = g.nib * nob;
    return g;
}

template <int N, int LOGB>
cgs_status launch_ct_b(const AxisPass &p, cudaStream_t st)
{
    constexpr int B = 1 << LOGB;
    static_assert(N * B <= kCtElems && (N * B) % kThreads == 0, "column block");
    const CtGrid cg = ct_grid(p, LOGB);
    const int logBI = cg.logBI;
    const int64_t nib = cg.nib, nblocks = cg.nblocks;
    if (nblocks > 0x7fffffffLL) { set_error("axis pass grid too large"); return CGS_ERR_BAD_ARG; }
    const size_t smem = ((size_t)N + (size_t)ct_rows<N, LOGB>() * B) * sizeof(float2);
    static std::atomic<uint64_t> attr_devs{0};
    if (attr_needed(attr_devs)) {
        CGS_CUDA(cudaFuncSetAttribute(axis_fft_ct_kernel<N, LOGB, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
        CGS_CUDA(cudaFuncSetAttribute(axis_fft_ct_kernel<N, LOGB, +1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
        attr_done(attr_devs);
    }
    CGS_CUDA(launch_pdl(p.sign < 0 ? axis_fft_ct_kernel<N, LOGB, -1> : axis_fft_ct_kernel<N, LOGB, +1>,
                        dim3((unsigned)nblocks), dim3(kThreads), smem, st, p, logBI, nib));
    return CGS_OK;
}

template <int N>
cgs_status launch_ct(const AxisPass &p, cudaStream_t st)
{
    constexpr int LOGB = ct_logb(N);
    constexpr int LS = ct_logb_small(N);
    if constexpr (LS >= 0) {
        if (ct_grid(p, LOGB).nblocks < kCtFewBlocks) return launch_ct_b<N, LS>(p, st);
    }
    return launch_ct_b<N, LOGB>(p, st);
}

bool ct_supported(int n)
{
    for (int c : {64, 96, 128, 160, 192, 224, 256, 288, 320, 384, 448, 512, 576, 640, 768, 896, 960, 1024})
        if (n == c) return true;
    return false;
}

// the compile-time pass for length n (ct_supported(n) must hold)
cgs_status launch_ct_any(int n, const AxisPass &p, cudaStream_t st)
{
    switch (n) {
        case 64: return launch_ct<64>(p, st);
        case 96: return launch_ct<96>(p, st);
        case 128: return launch_ct<128>(p, st);
        case 160: return launch_ct<160>(p, st);
        case 192: return launch_ct<192>(p, st);
        case 224: return launch_ct<224>(p, st);
        case 256: return launch_ct<256>(p, st);
        case 288: return launch_ct<288>(p, st);
        case 320: return launch_ct<320>(p, st);
        case 384: return launch_ct<384>(p, st);
        case 448: return launch_ct<448>(p, st);
        case 512: return launch_ct<512>(p, st);
        case 576: return launch_ct<576>(p, st);
        case 640: return launch_ct<640>(p, st);
        case 768: return launch_ct<768>(p, st);
        case 896: return launch_ct<896>(p, st);
        case 960: return launch_ct<960>(p, st);
        case 1024: return launch_ct<1024>(p, st);
        default: set_error("no compile-time FFT pass for this length"); return CGS_ERR_BAD_ARG;
    }
}

}  // namespace

cgs_status launch_axis_pass(const AxisPass &p, cudaStream_t st)
{
    if (p.outer <= 0 || p.inner <= 0) return CGS_OK;
    const int n = p.n;
    // columns per CTA: n * B <= kElems values (one shared buffer + twiddles)
    int B = 0;
    for (int c = 1; c <= 32 && (int64_t)n * c <= kElems; c *= 2) B = c;
    if (B < 1) {
        set_error("FFT length too large for the shared-memory axis pass");
        return CGS_ERR_BAD_ARG;
    }
    int BI = 1;  // largest power of two <= min(inner, B)
    while (BI * 2 <= B && BI * 2 <= p.inner) BI *= 2;
    const int BO = B / BI;
    const int64_t nib = (p.inner + BI - 1) / BI;
    const int64_t nob = (p.outer + BO - 1) / BO;
    const size_t smem = ((size_t)n + (size_t)n * (BO * BI + 1)) * sizeof(float2) + (size_t)B * sizeof(float);
    bool mixed = false;
    for (int i = 0; i < p.nfac; ++i) mixed = mixed || (p.fac[i] != 2 && p.fac[i] != 4 && p.fac[i] != 8);
    if (ct_supported(n)) {
        prof_begin(PROF_FFT, st);
        const cgs_status r = launch_ct_any(n, p, st);
        prof_end(PROF_FFT, st);
        return r;
    }
    static std::atomic<uint64_t> attr_devs{0};
    if (attr_needed(attr_devs)) {
        CGS_CUDA(cudaFuncSetAttribute(axis_fft_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      110 * 1024));
        CGS_CUDA(cudaFuncSetAttribute(axis_fft_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      110 * 1024));
        attr_done(attr_devs);
    }
    const int64_t nblocks = nib * nob;
    if (nblocks > 0x7fffffffLL) { set_error("axis pass grid too large"); return CGS_ERR_BAD_ARG; }
    prof_begin(PROF_FFT, st);
    if (mixed) axis_fft_kernel<true><<<(unsigned)nblocks, kThreads, smem, st>>>(p, BO, BI, nib);
    else axis_fft_kernel<false><<<(unsigned)nblocks, kThreads, smem, st>>>(p, BO, BI, nib);
    prof_end(PROF_FFT, st);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

}  // namespace cgs
