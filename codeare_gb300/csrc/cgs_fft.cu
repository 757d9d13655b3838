// cgs_fft.cu -- oversampled FFT passes of the NFFT, one axis per launch.
//
// Each CTA transforms B columns of data[outer][L][inner] along L entirely in
// shared memory (mixed-radix Stockham, radices 2/4/8 in registers, 3/5/7
// through the twiddle table).  Zero padding (image side ->
// oversampled grid) and cropping (grid -> image side) are index maps in the
// load / store phases, so padded zeros are never read from or written to HBM.
// The first forward pass also fuses the coil expansion S_c . x, the damping
// mask and the deapodisation 1/phihut (NFFT3's PRE_PHI_HUT step), and the last
// inverse pass fuses the deapodisation: the FFT-side work of the reference's
// nfft_trafo / nfft_adjoint (src/matrix/ft/NFFTTraits.hpp:176-204).
#include "cgs_internal.cuh"

namespace cgs {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
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

template <int R>
__device__ __forceinline__ void stockham_pass(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                              const float2 *tw, int n, int Ns, int B, int P, int sign)
{
    const int nR = n / R;
    const int step = n / (Ns * R);
    const int total = B * nR;
    for (int q = threadIdx.x; q < total; q += kThreads) {
        const int b = q % B, j = q / B;
        const int k = j % Ns;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = src[(j + r * nR) * P + b];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                float2 w = tw[k * r * step];
                if (sign > 0) w.y = -w.y;
                v[r] = cmul(v[r], w);
            }
        }
        bfly<R>(v, sign, tw, nR);
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) dst[(base + r * Ns) * P + b] = v[r];
    }
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

__device__ __forceinline__ float deapod(const AxisPass &p, int64_t o, int a)
{
    float d = p.deap_ax ? p.deap_ax[a] : 1.f;
    if (p.deap_o1) d *= p.deap_o1[o % p.o1_len];
    if (p.deap_o0) d *= p.deap_o0[o / p.o1_len];
    return d;
}

__global__ void __launch_bounds__(kThreads)
axis_fft_kernel(const __grid_constant__ AxisPass p, int BO, int BI, int64_t nib)
{
    extern __shared__ float2 smem[];
    const int n = p.n;
    const int B = BO * BI;
    const int P = B + 1;
    float2 *tw = smem;
    float2 *bufA = smem + n;
    float2 *bufB = bufA + (size_t)n * P;

    const int64_t blk = blockIdx.x;
    const int64_t ib0 = (blk % nib) * BI;
    const int64_t ob0 = (blk / nib) * BO;

    for (int t = threadIdx.x; t < n; t += kThreads) tw[t] = p.tw[t];

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
            if (pos_fast) { b = e / n; pos = e % n; }
            else { pos = e / B; b = e % B; }
            slot[u] = pos * P + b;
            const int64_t o = ob0 + b / BI;
            const int64_t i = ib0 + b % BI;
            if (o < p.outer && i < p.inner) {
                const int a = in_pos_to_axis(pos, p.Lin, n, p.in_centred);
                if (a >= 0) {
                    const int64_t pix = o * p.Lin + a;
                    if (p.load_mode == LOAD_PLAIN) {
                        v[u] = p.src[pix * p.inner + i];
                    } else {
                        float2 x = p.img_per_coil ? p.img[pix * p.inner + i] : p.img[pix];
                        if (p.sens) x = cmul(x, p.sens[pix * p.inner + i]);
                        float s = deapod(p, o, a);
                        if (p.mask) s *= p.mask[pix];
                        v[u] = cscale(x, s);
                    }
                }
            }
        }
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
            if (slot[u] >= 0) bufA[slot[u]] = v[u];
    }
    __syncthreads();

    // ---- Stockham passes, ping-pong in shared memory ----
    float2 *src = bufA, *dst = bufB;
    int Ns = 1;
    for (int s = 0; s < p.nfac; ++s) {
        const int R = p.fac[s];
        switch (R) {
            case 8: stockham_pass<8>(src, dst, tw, n, Ns, B, P, p.sign); break;
            case 4: stockham_pass<4>(src, dst, tw, n, Ns, B, P, p.sign); break;
            case 2: stockham_pass<2>(src, dst, tw, n, Ns, B, P, p.sign); break;
            case 3: stockham_pass<3>(src, dst, tw, n, Ns, B, P, p.sign); break;
            case 5: stockham_pass<5>(src, dst, tw, n, Ns, B, P, p.sign); break;
            case 7: stockham_pass<7>(src, dst, tw, n, Ns, B, P, p.sign); break;
            default: break;  // host rejects other primes
        }
        __syncthreads();
        float2 *t = src; src = dst; dst = t;
        Ns *= R;
    }

    // ---- store: Lout positions of every column ----
    const int totO = p.Lout * B;
    for (int e = threadIdx.x; e < totO; e += kThreads) {
        int a, b;
        if (pos_fast) { b = e / p.Lout; a = e % p.Lout; }
        else { a = e / B; b = e % B; }
        const int64_t o = ob0 + b / BI;
        const int64_t i = ib0 + b % BI;
        if (o >= p.outer || i >= p.inner) continue;
        const int pos = out_axis_to_pos(a, p.Lout, n, p.out_centred);
        float2 v = src[pos * P + b];
        const int64_t pix = o * p.Lout + a;
        if (p.store_mode == STORE_DEAPOD) v = cscale(v, deapod(p, o, a));
        p.dst[pix * p.inner + i] = v;
    }
}

}  // namespace

cgs_status launch_axis_pass(const AxisPass &p, cudaStream_t st)
{
    if (p.outer <= 0 || p.inner <= 0) return CGS_OK;
    const int n = p.n;
    // shared memory budget ~100 KB: twiddles + two n x (B+1) buffers
    const int budget = 100 * 1024 / 8;
    int B = (budget - n) / (2 * n) - 1;
    int Bp = 1;
    while (Bp * 2 <= B && Bp * 2 <= 32) Bp *= 2;
    B = Bp;
    if (B < 1) {
        set_error("FFT length too large for the shared-memory axis pass");
        return CGS_ERR_BAD_ARG;
    }
    const int BI = (int)(p.inner < B ? p.inner : B);
    const int BO = B / BI;
    const int64_t nib = (p.inner + BI - 1) / BI;
    const int64_t nob = (p.outer + BO - 1) / BO;
    const size_t smem = ((size_t)n + 2 * (size_t)n * (BO * BI + 1)) * sizeof(float2);
    static bool attr_set = false;
    if (!attr_set) {
        CGS_CUDA(cudaFuncSetAttribute(axis_fft_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      110 * 1024));
        attr_set = true;
    }
    const int64_t nblocks = nib * nob;
    if (nblocks > 0x7fffffffLL) { set_error("axis pass grid too large"); return CGS_ERR_BAD_ARG; }
    prof_begin(PROF_FFT, st);
    axis_fft_kernel<<<(unsigned)nblocks, kThreads, smem, st>>>(p, BO, BI, nib);
    prof_end(PROF_FFT, st);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

}  // namespace cgs
