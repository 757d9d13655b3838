// cgs_cnn.cu -- the learned preconditioner: a 5-layer 3x3 CNN on a complex
// image held as 2 real channels (2 -> 32 -> 32 -> 32 -> 32 -> 2, ReLU between
// layers, no biases, so the map is positively homogeneous: M(c r) = c M(r)
// for c > 0).  Activations and weights in BF16, accumulation in FP32.
//
//   conv32_tc05_kernel   32 -> 32 layers on the 5th-generation tensor cores
//                        (tcgen05.mma, TMEM accumulator), used for the forward
//                        pass and, with flipped/transposed weights, for the
//                        input gradients of the backward pass
//   conv32_mma_kernel    the same layers with warp-level mma.sync m16n8k16
//                        (selectable, cgs_net_set_conv_kernel)
//   conv_in / conv_out_v the thin 2 -> 32 and 32 -> 2 layers on CUDA cores
//   wgrad_kernel         weight gradients (reduction over pixels, CUDA cores)
//   adam_kernel          Adam update of the FP32 master weights
//
// Layouts: activations NHWC ([B][H][W][C], C innermost); layer weights
// [9 taps][Cout][Cin] with tap = 3*(dy) + dx for offsets (dy-1, dx-1); the
// convolution is the usual cross-correlation y[p][co] = sum x[p+off][ci] w.
// No reference counterpart (the reference has no learned component).
#include "cgs_internal.cuh"
#include "cgs_tc05.cuh"

#include <atomic>

#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

namespace cgs {
namespace {

constexpr int kC = 32;            // hidden channels
constexpr int kLayers = 5;
constexpr int kCin[kLayers] = {2, kC, kC, kC, kC};
constexpr int kCout[kLayers] = {kC, kC, kC, kC, 2};

constexpr int layer_params(int l) { return 9 * kCin[l] * kCout[l]; }
constexpr int layer_offset(int l)
{
    int o = 0;
    for (int i = 0; i < l; ++i) o += layer_params(i);
    return o;
}
constexpr int kParams = layer_offset(kLayers);  // 28800

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }

// ---------------------------------------------------------------------------
// 32 -> 32 convolution on the tensor cores.  CTA: 8 x 16 output pixels x 32
// output channels, 4 warps, each warp two rows of 16 pixels (two m16 tiles)
// by four n8 tiles, K = 9 taps x 32 channels = 18 k16 steps.  Input tile with
// a one-pixel halo and the weights sit in shared memory with a channel stride
// of 40 bf16 (20 words), which makes every fragment load conflict-free.
// EPI: 0 ReLU, 1 multiply by (mask > 0), 2 none.
// ---------------------------------------------------------------------------
constexpr int kTH = 8, kTW = 16, kCS = 40;

__device__ __forceinline__ void mma_bf16(float *d, const uint32_t *a, const uint32_t *b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <int EPI>
__global__ void __launch_bounds__(128)
conv32_mma_kernel(const __nv_bfloat16 *__restrict__ X, const __nv_bfloat16 *__restrict__ Wt,
                  __nv_bfloat16 *__restrict__ Y, const __nv_bfloat16 *__restrict__ Mask, int H, int W)
{
    __shared__ __align__(16) __nv_bfloat16 xs[(kTH + 2) * (kTW + 2) * kCS];
    __shared__ __align__(16) __nv_bfloat16 ws[9 * kC * kCS];
    const int b = blockIdx.z;
    const int y0 = blockIdx.y * kTH, x0 = blockIdx.x * kTW;
    const __nv_bfloat16 *Xb = X + (size_t)b * H * W * kC;
    // weights: 9 x 32 rows of 32 channels, 16-byte chunks
    for (int e = threadIdx.x; e < 9 * kC * 4; e += 128) {
        const int row = e >> 2, q = e & 3;
        *reinterpret_cast<uint4 *>(&ws[row * kCS + q * 8]) = *reinterpret_cast<const uint4 *>(&Wt[row * kC + q * 8]);
    }
    // input tile with halo, zero outside the image
    for (int e = threadIdx.x; e < (kTH + 2) * (kTW + 2) * 4; e += 128) {
        const int pix = e >> 2, q = e & 3;
        const int ty = pix / (kTW + 2), tx = pix % (kTW + 2);
        const int gy = y0 + ty - 1, gx = x0 + tx - 1;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (gy >= 0 && gy < H && gx >= 0 && gx < W)
            v = *reinterpret_cast<const uint4 *>(&Xb[((size_t)gy * W + gx) * kC + q * 8]);
        *reinterpret_cast<uint4 *>(&xs[pix * kCS + q * 8]) = v;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
        const int dy = tap / 3, dx = tap % 3;
#pragma unroll
        for (int cib = 0; cib < kC; cib += 16) {
            uint32_t bfr[4][2];
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const __nv_bfloat16 *wr = &ws[(tap * kC + nt * 8 + g) * kCS + cib + 2 * t];
                bfr[nt][0] = *reinterpret_cast<const uint32_t *>(wr);
                bfr[nt][1] = *reinterpret_cast<const uint32_t *>(wr + 8);
            }
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const int row = warp * 2 + mt + dy;
                const __nv_bfloat16 *p0 = &xs[(row * (kTW + 2) + g + dx) * kCS + cib + 2 * t];
                const __nv_bfloat16 *p1 = p0 + 8 * kCS;
                uint32_t afr[4];
                afr[0] = *reinterpret_cast<const uint32_t *>(p0);
                afr[1] = *reinterpret_cast<const uint32_t *>(p1);
                afr[2] = *reinterpret_cast<const uint32_t *>(p0 + 8);
                afr[3] = *reinterpret_cast<const uint32_t *>(p1 + 8);
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[mt][nt], afr, bfr[nt]);
            }
        }
    }
    // epilogue: fragment (row g / g+8, cols 2t, 2t+1) of each n8 tile
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        const int gy = y0 + warp * 2 + mt;
        if (gy >= H) continue;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int gx = x0 + g + half * 8;
            if (gx >= W) continue;
            const size_t pix = ((size_t)b * H + gy) * W + gx;
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int co = nt * 8 + 2 * t;
                float v0 = acc[mt][nt][half * 2], v1 = acc[mt][nt][half * 2 + 1];
                if (EPI == 0) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
                if (EPI == 1) {
                    const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162 *>(&Mask[pix * kC + co]);
                    if (!(bf(mk.x) > 0.f)) v0 = 0.f;
                    if (!(bf(mk.y) > 0.f)) v1 = 0.f;
                }
                *reinterpret_cast<__nv_bfloat162 *>(&Y[pix * kC + co]) = __floats2bfloat162_rn(v0, v1);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// 32 -> 32 convolution on the 5th-generation tensor cores (tcgen05).  A CTA
// computes an 8 x 16-pixel tile (M = 128 pixels) x 32 output channels (N):
// one thread issues 18 tcgen05.mma.kind::f16 (BF16 operands, K = 16: 9 taps
// x 2 channel halves) whose FP32 accumulator lives in 32 TMEM columns, and a
// tcgen05.commit arrives on an mbarrier when they are done.  Operands sit in
// shared memory in the canonical K-major layout without swizzle: "core
// matrices" of 8 rows x 16 bytes (8 BF16 values of K), each 128 contiguous
// bytes, adjacent core matrices along K `lbo` bytes apart and along M / N
// `sbo` bytes apart.
//   A: the tile's pixels are ordered m = 8 x + y (column-major), and the
//     input halo tile (10 rows x 18 columns x 32 channels) is stored as
//     [column][channel group of 8][row][16 bytes] (640 bytes per column).
//     The 8 rows of a core matrix (pixels y = 0..7 of column x) are then 8
//     consecutive 16-byte rows of the halo column x + dx starting at row dy,
//     so the A matrix of tap (dy, dx) is a descriptor into the halo tile
//     itself: start dx * 640 + dy * 16 (+ 320 for the upper channel half),
//     lbo = 160 (next channel group), sbo = 640 (next column).  No im2col
//     copy is made.
//   B (32 output channels x 288 = 9 taps x 32 input channels): core
//     (n / 8, k / 8) at (k / 8) * 512 + (n / 8) * 128, so lbo = 512,
//     sbo = 128; the k-step of (tap t, half j) starts (4 t + 2 j) * 512 in.
// The threads store the halo tile and the weights with ordinary stores, then
// a proxy fence makes them visible to the tensor cores.  Each warp reads its
// 32 TMEM lanes (pixels m = 32 w .. 32 w + 31, 32 channels each) with
// tcgen05.ld for the epilogue.  The mbarrier wait is bounded: past the limit
// the CTA sets *err, skips the epilogue and still frees its TMEM.
// ---------------------------------------------------------------------------
constexpr int kTcB = kC * 9 * kC * 2;           // 32 x 288 BF16
constexpr int kTcCol = 4 * (kTH + 2) * 16;      // one halo column: 4 channel groups x 10 rows x 16 B
constexpr int kTcHalo = (kTW + 2) * kTcCol;
constexpr int kTcSmem = kTcB + kTcHalo + 16;
constexpr uint32_t kTcWaitLimit = 1u << 22;

using tc05::smem_u32;

template <int EPI>
__global__ void __launch_bounds__(128)
conv32_tc05_kernel(const __nv_bfloat16 *__restrict__ X, const __nv_bfloat16 *__restrict__ Wt,
                   __nv_bfloat16 *__restrict__ Y, const __nv_bfloat16 *__restrict__ Mask, int H, int W,
                   int *__restrict__ err)
{
    extern __shared__ __align__(128) uint8_t tsm[];
    uint8_t *sB = tsm;
    uint8_t *sX = sB + kTcB;                                  // halo tile, column-major (see above)
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sX + kTcHalo);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int b = blockIdx.z;
    const int y0 = blockIdx.y * kTH, x0 = blockIdx.x * kTW;
    const __nv_bfloat16 *Xb = X + (size_t)b * H * W * kC;

    if (warp == 0) tc05::alloc<32>(tslot);   // 32 TMEM columns: the 128 x 32 FP32 accumulator
    if (tid == 0) tc05::mbar_init(mbar, 1);
    // weights: (tap, co, 8-channel chunk) -> core (co / 8, (32 tap + ci) / 8)
    for (int e = tid; e < 9 * kC * 4; e += 128) {
        const int q = e & 3, co = (e >> 2) % kC, tap = (e >> 2) / kC;
        const uint4 v = *reinterpret_cast<const uint4 *>(&Wt[(tap * kC + co) * kC + q * 8]);
        *reinterpret_cast<uint4 *>(sB + ((tap * 4 + q) * 4 + (co >> 3)) * 128 + (co & 7) * 16) = v;
    }
    // input tile with a one-pixel halo, zero outside the image: row r, column cx,
    // channel group q at cx * 640 + q * 160 + r * 16
    for (int e = tid; e < (kTH + 2) * (kTW + 2) * 4; e += 128) {
        const int pix = e >> 2, q = e & 3;
        const int r = pix / (kTW + 2), cx = pix % (kTW + 2);
        const int gy = y0 + r - 1, gx = x0 + cx - 1;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (gy >= 0 && gy < H && gx >= 0 && gx < W)
            v = *reinterpret_cast<const uint4 *>(&Xb[((size_t)gy * W + gx) * kC + q * 8]);
        *reinterpret_cast<uint4 *>(sX + cx * kTcCol + q * (kTcCol / 4) + r * 16) = v;
    }
    tc05::fence_proxy_async();
    tc05::fence_before();
    __syncthreads();
    tc05::fence_after();
    const uint32_t tmem = *tslot;
    if (tid == 0) {
        // D FP32, A and B BF16, both K-major, N = 32, M = 128
        constexpr uint32_t idesc = tc05::idesc_bf16(128, kC);
        const uint32_t a0 = smem_u32(sX), b0 = smem_u32(sB);
#pragma unroll 1
        for (int tap = 0; tap < 9; ++tap)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int dy = tap / 3, dx = tap % 3;
                const uint64_t ad = tc05::desc(a0 + dx * kTcCol + dy * 16 + j * 2 * (kTcCol / 4), kTcCol / 4, kTcCol);
                const uint64_t bd = tc05::desc(b0 + (tap * 4 + j * 2) * 512, 512, 128);
                tc05::mma_bf16(tmem, ad, bd, idesc, (tap | j) ? 1u : 0u);
            }
        tc05::commit(mbar);
    }
    // bounded wait for the MMAs; tcgen05.ld is warp-collective: the whole
    // warp reads, or none of it does
    const uint32_t done = __all_sync(0xffffffffu, tc05::mbar_wait(mbar, 0, kTcWaitLimit) ? 1u : 0u);
    tc05::fence_after();
    if (!done) {
        if (lane == 0) atomicOr(err, 1);
    } else {
        float v[32];
        tc05::ld32(tmem + ((uint32_t)(warp * 32) << 16), v);
        tc05::wait_ld();
        const int m = tid;                                     // TMEM lane = pixel m = 8 x + y
        const int gy = y0 + (m & 7), gx = x0 + (m >> 3);
        if (gy < H && gx < W) {
            const size_t pix = ((size_t)b * H + gy) * W + gx;
            __align__(16) __nv_bfloat162 o[kC / 2];
#pragma unroll
            for (int c = 0; c < kC; c += 2) {
                float a = v[c], d = v[c + 1];
                if (EPI == 0) { a = fmaxf(a, 0.f); d = fmaxf(d, 0.f); }
                if (EPI == 1) {
                    const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162 *>(&Mask[pix * kC + c]);
                    if (!(bf(mk.x) > 0.f)) a = 0.f;
                    if (!(bf(mk.y) > 0.f)) d = 0.f;
                }
                o[c / 2] = __floats2bfloat162_rn(a, d);
            }
            uint4 *dst = reinterpret_cast<uint4 *>(&Y[pix * kC]);
#pragma unroll
            for (int q = 0; q < 4; ++q) dst[q] = reinterpret_cast<const uint4 *>(o)[q];
        }
    }
    tc05::fence_before();
    __syncthreads();
    if (warp == 0) {
        tc05::fence_after();
        tc05::dealloc<32>(tmem);
    }
}

// 32 -> 2 layer (linear): thread per pixel, each tap's 32 channels read as
// four 16-byte vectors; output fp32 [B][H][W][2]
__global__ void conv_out_v_kernel(const __nv_bfloat16 *__restrict__ X, const float *__restrict__ Wf,
                                  float *__restrict__ Y, int B, int H, int W)
{
    __shared__ float w[9 * 2 * kC];
    for (int e = threadIdx.x; e < 9 * 2 * kC; e += blockDim.x) w[e] = Wf[e];
    __syncthreads();
    const int64_t tot = (int64_t)B * H * W;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < tot; p += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(p % W), y = (int)((p / W) % H);
        const int64_t base = p - (int64_t)y * W - x;
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
            const int yy = y + tap / 3 - 1, xx = x + tap % 3 - 1;
            if (yy < 0 || yy >= H || xx < 0 || xx >= W) continue;
            const uint4 *xr = reinterpret_cast<const uint4 *>(&X[(base + (int64_t)yy * W + xx) * kC]);
            const float *w0 = &w[(tap * 2 + 0) * kC], *w1 = &w[(tap * 2 + 1) * kC];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint4 u = __ldg(xr + q);
                const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const float2 v = __bfloat1622float2(h[c]);
                    const int ch = q * 8 + 2 * c;
                    s0 = fmaf(v.x, w0[ch], fmaf(v.y, w0[ch + 1], s0));
                    s1 = fmaf(v.x, w1[ch], fmaf(v.y, w1[ch + 1], s1));
                }
            }
        }
        *reinterpret_cast<float2 *>(&Y[p * 2]) = make_float2(s0, s1);
    }
}

// 2 -> 32 layer (+ReLU): thread per pixel; input fp32 [B][H][W][2]
__global__ void conv_in_kernel(const float *__restrict__ X, const float *__restrict__ Wf,
                               __nv_bfloat16 *__restrict__ Y, int B, int H, int W)
{
    __shared__ float w[9 * kC * 2];
    for (int e = threadIdx.x; e < 9 * kC * 2; e += blockDim.x) w[e] = Wf[e];
    __syncthreads();
    const int64_t tot = (int64_t)B * H * W;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < tot; p += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(p % W), y = (int)((p / W) % H);
        const int64_t base = p - (int64_t)y * W - x;
        float in[18];
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
            const int yy = y + tap / 3 - 1, xx = x + tap % 3 - 1;
            const bool ok = yy >= 0 && yy < H && xx >= 0 && xx < W;
            const float2 v = ok ? *reinterpret_cast<const float2 *>(&X[(base + (int64_t)yy * W + xx) * 2])
                                : make_float2(0.f, 0.f);
            in[2 * tap] = v.x; in[2 * tap + 1] = v.y;
        }
        __align__(16) __nv_bfloat162 out[kC / 2];
#pragma unroll
        for (int co = 0; co < kC; co += 2) {
            float s0 = 0.f, s1 = 0.f;
#pragma unroll
            for (int tap = 0; tap < 9; ++tap) {
                s0 = fmaf(in[2 * tap], w[(tap * kC + co) * 2], fmaf(in[2 * tap + 1], w[(tap * kC + co) * 2 + 1], s0));
                s1 = fmaf(in[2 * tap], w[(tap * kC + co + 1) * 2], fmaf(in[2 * tap + 1], w[(tap * kC + co + 1) * 2 + 1], s1));
            }
            out[co / 2] = __floats2bfloat162_rn(fmaxf(s0, 0.f), fmaxf(s1, 0.f));
        }
        uint4 *dst = reinterpret_cast<uint4 *>(&Y[p * kC]);
#pragma unroll
        for (int q = 0; q < 4; ++q) dst[q] = reinterpret_cast<const uint4 *>(out)[q];
    }
}

// input gradient of the 32 -> 2 layer, times the ReLU mask of its input:
// dX[p][ci] = (X[p][ci] > 0) * sum_tap sum_co W[tap][co][ci] dY[p - off(tap)][co]
__global__ void conv_out_back_kernel(const float *__restrict__ dY, const float *__restrict__ Wf,
                                     const __nv_bfloat16 *__restrict__ Xmask, __nv_bfloat16 *__restrict__ dX,
                                     int B, int H, int W)
{
    __shared__ float w[9 * 2 * kC];
    for (int e = threadIdx.x; e < 9 * 2 * kC; e += blockDim.x) w[e] = Wf[e];
    __syncthreads();
    const int64_t tot = (int64_t)B * H * W;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < tot; p += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(p % W), y = (int)((p / W) % H);
        const int64_t base = p - (int64_t)y * W - x;
        float acc[kC];
#pragma unroll
        for (int c = 0; c < kC; ++c) acc[c] = 0.f;
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
            const int yy = y - (tap / 3 - 1), xx = x - (tap % 3 - 1);
            if (yy < 0 || yy >= H || xx < 0 || xx >= W) continue;
            const float2 d = *reinterpret_cast<const float2 *>(&dY[(base + (int64_t)yy * W + xx) * 2]);
#pragma unroll
            for (int c = 0; c < kC; ++c) acc[c] = fmaf(d.x, w[(tap * 2) * kC + c], fmaf(d.y, w[(tap * 2 + 1) * kC + c], acc[c]));
        }
        const __nv_bfloat162 *m = reinterpret_cast<const __nv_bfloat162 *>(&Xmask[p * kC]);
        __align__(16) __nv_bfloat162 out[kC / 2];
#pragma unroll
        for (int c = 0; c < kC / 2; ++c) {
            const float2 mk = __bfloat1622float2(m[c]);
            out[c] = __floats2bfloat162_rn(mk.x > 0.f ? acc[2 * c] : 0.f, mk.y > 0.f ? acc[2 * c + 1] : 0.f);
        }
        uint4 *dst = reinterpret_cast<uint4 *>(&dX[p * kC]);
#pragma unroll
        for (int q = 0; q < 4; ++q) dst[q] = reinterpret_cast<const uint4 *>(out)[q];
    }
}

// weights for the input gradient of a 32 -> 32 layer: Wt'[tap'][ci][co] = W[8 - tap'][co][ci]
__global__ void flip_weights_kernel(const float *__restrict__ Wf, __nv_bfloat16 *__restrict__ Wt)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 9 * kC * kC; e += gridDim.x * blockDim.x) {
        const int co = e % kC, ci = (e / kC) % kC, tap = e / (kC * kC);
        Wt[e] = __float2bfloat16(Wf[((8 - tap) * kC + co) * kC + ci]);
    }
}

__global__ void to_bf16_kernel(const float *__restrict__ a, __nv_bfloat16 *__restrict__ b, int n)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) b[e] = __float2bfloat16(a[e]);
}

// Weight gradient dW[tap][co][ci] += sum_p X[p + off(tap)][ci] * D[p][co] over
// one 8 x 8 pixel tile per CTA (CUDA cores, FP32 accumulation, one atomic add
// per weight per CTA).
template <typename TX, typename TD, int CIN, int COUT>
__global__ void __launch_bounds__(256)
wgrad_kernel(const TX *__restrict__ X, const TD *__restrict__ D, float *__restrict__ dW, int H, int W)
{
    constexpr int T = 8;
    __shared__ float xs[(T + 2) * (T + 2)][CIN + 1];
    __shared__ float ds[T * T][COUT];
    const int b = blockIdx.z, y0 = blockIdx.y * T, x0 = blockIdx.x * T;
    for (int e = threadIdx.x; e < (T + 2) * (T + 2) * CIN; e += 256) {
        const int ci = e % CIN, pix = e / CIN;
        const int gy = y0 + pix / (T + 2) - 1, gx = x0 + pix % (T + 2) - 1;
        float v = 0.f;
        if (gy >= 0 && gy < H && gx >= 0 && gx < W) v = (float)X[(((size_t)b * H + gy) * W + gx) * CIN + ci];
        xs[pix][ci] = v;
    }
    for (int e = threadIdx.x; e < T * T * COUT; e += 256) {
        const int co = e % COUT, pix = e / COUT;
        const int gy = y0 + pix / T, gx = x0 + pix % T;
        float v = 0.f;
        if (gy < H && gx < W) v = (float)D[(((size_t)b * H + gy) * W + gx) * COUT + co];
        ds[pix][co] = v;
    }
    __syncthreads();
    for (int o = threadIdx.x; o < 9 * CIN * COUT; o += 256) {
        const int ci = o % CIN, co = (o / CIN) % COUT, tap = o / (CIN * COUT);
        const int dy = tap / 3, dx = tap % 3;
        float acc = 0.f;
#pragma unroll 8
        for (int p = 0; p < T * T; ++p) acc = fmaf(xs[(p / T + dy) * (T + 2) + p % T + dx][ci], ds[p][co], acc);
        atomicAdd(&dW[o], acc);
    }
}

__global__ void mse_kernel(const float *__restrict__ y, const float *__restrict__ t, float *__restrict__ d, int64_t n,
                           float scale, float *__restrict__ loss)
{
    float s = 0.f;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float r = y[e] - t[e];
        d[e] = 2.f * r * scale;
        s = fmaf(r, r, s);
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s * scale);
}

__global__ void adam_kernel(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const float gg = g[e];
        const float mm = b1 * m[e] + (1.f - b1) * gg;
        const float vv = b2 * v[e] + (1.f - b2) * gg * gg;
        m[e] = mm; v[e] = vv;
        w[e] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    }
}

// complex image (float2) -> network input [H][W][2] scaled by 1/s, and back
__global__ void img_to_net_kernel(const float2 *__restrict__ r, const double *__restrict__ nrm2, int64_t n,
                                  float *__restrict__ x, float *__restrict__ scale_out)
{
    const double rms = sqrt(*nrm2 / (double)(2 * n));
    const float inv = rms > 0.0 ? (float)(1.0 / rms) : 0.f;
    if (blockIdx.x == 0 && threadIdx.x == 0) *scale_out = (float)rms;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float2 v = r[e];
        reinterpret_cast<float2 *>(x)[e] = make_float2(v.x * inv, v.y * inv);
    }
}

__global__ void net_to_img_kernel(const float *__restrict__ y, const float *__restrict__ scale, int64_t n,
                                  float2 *__restrict__ z)
{
    const float s = *scale;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float2 v = reinterpret_cast<const float2 *>(y)[e];
        z[e] = make_float2(v.x * s, v.y * s);
    }
}

// z = dsc . (s y) + csq . vc: the network's output back on the image scale,
// times the pixel scaling, plus the circulant's output csq . vc (the same
// products and add, in the same order, as net_to_img, the circulant's output
// scaling and scale_add one after another)
__global__ void net_combine_kernel(const float *__restrict__ y, const float *__restrict__ scale, int64_t n,
                                   const float *__restrict__ dsc, const float *__restrict__ csq,
                                   const float2 *__restrict__ vc, float2 *__restrict__ z)
{
    const float s = *scale;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float2 v = reinterpret_cast<const float2 *>(y)[e];
        float2 o = make_float2(v.x * s, v.y * s);
        const float a = dsc[e];
        o.x *= a; o.y *= a;
        const float f = csq[e];
        const float2 c = vc[e];
        const float2 u = make_float2(c.x * f, c.y * f);
        o.x = fmaf(1.f, u.x, o.x); o.y = fmaf(1.f, u.y, o.y);
        z[e] = o;
    }
}

unsigned blocks_for(int64_t n)
{
    int64_t b = (n + 255) / 256;
    if (b > 152 * 8) b = 152 * 8;
    if (b < 1) b = 1;
    return (unsigned)b;
}

}  // namespace
}  // namespace cgs

using namespace cgs;

struct cgs_net {
    int maxB = 0, maxH = 0, maxW = 0;
    float *w = nullptr;               // fp32 master weights [kParams]
    float *g = nullptr, *m = nullptr, *v = nullptr;  // gradient, Adam moments
    __nv_bfloat16 *wb = nullptr;      // bf16 copies of the 32 -> 32 layers [3][9*32*32]
    __nv_bfloat16 *wflip = nullptr;   // flipped/transposed bf16 weights for input gradients
    float *x0 = nullptr, *y5 = nullptr, *d5 = nullptr, *target = nullptr;  // [B][H][W][2]
    __nv_bfloat16 *act[4] = {nullptr, nullptr, nullptr, nullptr};         // x1..x4 [B][H][W][32]
    __nv_bfloat16 *dA = nullptr, *dB = nullptr;                           // gradient ping-pong
    float *loss = nullptr, *scale = nullptr;
    int64_t step = 0;
    uint64_t serial = 0;              // unique per created network (graphs key on it, not the address)
    int conv_kind = 1;                // 32 -> 32 layers: 1 tcgen05 (default), 0 mma.sync
    int *err = nullptr;               // set by a tcgen05 layer whose MMA wait ran out
};

namespace {

// one 32 -> 32 layer with the network's kernel choice; EPI 0 ReLU, 1 the input-gradient mask
template <int EPI>
cgs_status conv32(cgs_net *n, const __nv_bfloat16 *x, const __nv_bfloat16 *w, __nv_bfloat16 *y,
                  const __nv_bfloat16 *mask, int B, int H, int W, cudaStream_t st)
{
    dim3 grd((W + kTW - 1) / kTW, (H + kTH - 1) / kTH, B);
    if (n->conv_kind == 1) {
        static std::atomic<uint64_t> attr_devs{0};
        int dev = 0;
        CGS_CUDA(cudaGetDevice(&dev));
        const uint64_t bit = dev < 64 ? (1ull << dev) : 0ull;
        if (!(attr_devs.load() & bit)) {
            CGS_CUDA(cudaFuncSetAttribute(conv32_tc05_kernel<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
            attr_devs.fetch_or(bit);
        }
        conv32_tc05_kernel<EPI><<<grd, 128, kTcSmem, st>>>(x, w, y, mask, H, W, n->err);
    } else {
        conv32_mma_kernel<EPI><<<grd, 128, 0, st>>>(x, w, y, mask, H, W);
    }
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status net_refresh_bf16(cgs_net *n, cudaStream_t st)
{
    for (int l = 1; l <= 3; ++l) {
        to_bf16_kernel<<<36, 256, 0, st>>>(n->w + layer_offset(l), n->wb + (l - 1) * 9 * kC * kC, 9 * kC * kC);
        CGS_LAUNCH_CHECK();
    }
    return CGS_OK;
}

cgs_status net_forward_dev(cgs_net *n, int B, int H, int W, cudaStream_t st)
{
    const int64_t P = (int64_t)B * H * W;
    conv_in_kernel<<<blocks_for(P), 256, 0, st>>>(n->x0, n->w + layer_offset(0), n->act[0], B, H, W);
    CGS_LAUNCH_CHECK();
    for (int l = 1; l <= 3; ++l)
        CGS_TRY(conv32<0>(n, n->act[l - 1], n->wb + (l - 1) * 9 * kC * kC, n->act[l], nullptr, B, H, W, st));
    conv_out_v_kernel<<<blocks_for(P), 256, 0, st>>>(n->act[3], n->w + layer_offset(4), n->y5, B, H, W);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

// gradients of the mean squared error into n->g (zeroed here); loss into n->loss
cgs_status net_backward_dev(cgs_net *n, int B, int H, int W, cudaStream_t st)
{
    const int64_t P = (int64_t)B * H * W;
    CGS_CUDA(cudaMemsetAsync(n->g, 0, sizeof(float) * kParams, st));
    CGS_CUDA(cudaMemsetAsync(n->loss, 0, sizeof(float), st));
    mse_kernel<<<blocks_for(P * 2), 256, 0, st>>>(n->y5, n->target, n->d5, P * 2, 1.f / (float)(P * 2), n->loss);
    CGS_LAUNCH_CHECK();
    dim3 wg((W + 7) / 8, (H + 7) / 8, B);
    // layer 5 (32 -> 2)
    wgrad_kernel<__nv_bfloat16, float, kC, 2><<<wg, 256, 0, st>>>(n->act[3], n->d5, n->g + layer_offset(4), H, W);
    CGS_LAUNCH_CHECK();
    conv_out_back_kernel<<<blocks_for(P), 256, 0, st>>>(n->d5, n->w + layer_offset(4), n->act[3], n->dA, B, H, W);
    CGS_LAUNCH_CHECK();
    // layers 4..2 (32 -> 32): dA holds the gradient at the layer's output (pre-activation)
    __nv_bfloat16 *cur = n->dA, *nxt = n->dB;
    for (int l = 3; l >= 1; --l) {
        wgrad_kernel<__nv_bfloat16, __nv_bfloat16, kC, kC><<<wg, 256, 0, st>>>(n->act[l - 1], cur, n->g + layer_offset(l), H, W);
        CGS_LAUNCH_CHECK();
        flip_weights_kernel<<<36, 256, 0, st>>>(n->w + layer_offset(l), n->wflip);
        CGS_LAUNCH_CHECK();
        CGS_TRY(conv32<1>(n, cur, n->wflip, nxt, n->act[l - 1], B, H, W, st));
        __nv_bfloat16 *tmp = cur; cur = nxt; nxt = tmp;
    }
    // layer 1 (2 -> 32): weight gradient only
    wgrad_kernel<float, __nv_bfloat16, 2, kC><<<wg, 256, 0, st>>>(n->x0, cur, n->g + layer_offset(0), H, W);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

std::atomic<uint64_t> g_net_serial{0};

// a tcgen05 layer that gave up waiting for its MMAs sets the flag: report it once
cgs_status net_check_err(cgs_net *n)
{
    int e = 0;
    CGS_CUDA(cudaMemcpy(&e, n->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        cudaMemset(n->err, 0, sizeof(int));
        set_error("a tcgen05 convolution timed out waiting for its MMAs");
        return CGS_ERR_TIMEOUT;
    }
    return CGS_OK;
}

cgs_status net_check(cgs_net *n, int B, int H, int W)
{
    if (!n) { set_error("null net"); return CGS_ERR_BAD_ARG; }
    if (B < 1 || H < 1 || W < 1 || B > n->maxB || (int64_t)H * W > (int64_t)n->maxH * n->maxW) {
        set_error("network batch or image size exceeds what the net was created for");
        return CGS_ERR_BAD_ARG;
    }
    return CGS_OK;
}

}  // namespace

// internal use by the flexible-CG solver: z = M(r) for one complex image
namespace cgs {
uint64_t net_serial(const cgs_net *n) { return n ? n->serial : 0; }

cgs_status net_apply_image(cgs_net *n, const float2 *r, const double *nrm2, int H, int W, float2 *z, cudaStream_t st)
{
    CGS_TRY(net_check(n, 1, H, W));
    const int64_t P = (int64_t)H * W;
    img_to_net_kernel<<<blocks_for(P), 256, 0, st>>>(r, nrm2, P, n->x0, n->scale);
    CGS_LAUNCH_CHECK();
    CGS_TRY(net_forward_dev(n, 1, H, W, st));
    net_to_img_kernel<<<blocks_for(P), 256, 0, st>>>(n->y5, n->scale, P, z);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status net_apply_image_combine(cgs_net *n, const float2 *r, const double *nrm2, int H, int W, const float *dsc,
                                   const float *csq, const float2 *vc, float2 *z, cudaStream_t st)
{
    CGS_TRY(net_check(n, 1, H, W));
    const int64_t P = (int64_t)H * W;
    img_to_net_kernel<<<blocks_for(P), 256, 0, st>>>(r, nrm2, P, n->x0, n->scale);
    CGS_LAUNCH_CHECK();
    CGS_TRY(net_forward_dev(n, 1, H, W, st));
    net_combine_kernel<<<blocks_for(P), 256, 0, st>>>(n->y5, n->scale, P, dsc, csq, vc, z);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}
}  // namespace cgs

extern "C" {

int64_t cgs_net_num_params(void) { return kParams; }

cgs_status cgs_net_create(cgs_net **out, int max_batch, int max_h, int max_w)
{
    if (!out || max_batch < 1 || max_h < 1 || max_w < 1) { set_error("bad net size"); return CGS_ERR_BAD_ARG; }
    cgs_net *n = new cgs_net();
    n->serial = ++g_net_serial;
    n->maxB = max_batch; n->maxH = max_h; n->maxW = max_w;
    const int64_t P = (int64_t)max_batch * max_h * max_w;
    bool ok = true;
    auto al = [&ok](void **p, size_t bytes) { if (ok && cudaMalloc(p, bytes) != cudaSuccess) { ok = false; *p = nullptr; } };
    al((void **)&n->w, sizeof(float) * kParams);
    al((void **)&n->g, sizeof(float) * kParams);
    al((void **)&n->m, sizeof(float) * kParams);
    al((void **)&n->v, sizeof(float) * kParams);
    al((void **)&n->wb, sizeof(__nv_bfloat16) * 3 * 9 * kC * kC);
    al((void **)&n->wflip, sizeof(__nv_bfloat16) * 9 * kC * kC);
    al((void **)&n->x0, sizeof(float) * P * 2);
    al((void **)&n->y5, sizeof(float) * P * 2);
    al((void **)&n->d5, sizeof(float) * P * 2);
    al((void **)&n->target, sizeof(float) * P * 2);
    for (int i = 0; i < 4; ++i) al((void **)&n->act[i], sizeof(__nv_bfloat16) * P * kC);
    al((void **)&n->dA, sizeof(__nv_bfloat16) * P * kC);
    al((void **)&n->dB, sizeof(__nv_bfloat16) * P * kC);
    al((void **)&n->loss, sizeof(float));
    al((void **)&n->scale, sizeof(float));
    al((void **)&n->err, sizeof(int));
    if (!ok) { cgs_net_destroy(n); set_error("cudaMalloc failed for the network"); return CGS_ERR_OOM; }
    cudaMemset(n->m, 0, sizeof(float) * kParams);
    cudaMemset(n->v, 0, sizeof(float) * kParams);
    cudaMemset(n->err, 0, sizeof(int));
    // He-style initialisation (fixed seed, host)
    std::vector<float> w(kParams);
    uint64_t s = 0x9e3779b97f4a7c15ull;
    auto rnd = [&s]() {
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        return ((s >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
    };
    for (int l = 0; l < kLayers; ++l) {
        const double a = std::sqrt(6.0 / (9.0 * kCin[l])) * (l == kLayers - 1 ? 0.5 : 1.0);
        for (int i = 0; i < layer_params(l); ++i) w[layer_offset(l) + i] = (float)(a * rnd());
    }
    cudaMemcpy(n->w, w.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice);
    if (net_refresh_bf16(n, nullptr) != CGS_OK || cudaDeviceSynchronize() != cudaSuccess) {
        cgs_net_destroy(n);
        return CGS_ERR_CUDA;
    }
    *out = n;
    return CGS_OK;
}

cgs_status cgs_net_destroy(cgs_net *n)
{
    if (!n) return CGS_OK;
    void *b[] = {n->w, n->g, n->m, n->v, n->wb, n->wflip, n->x0, n->y5, n->d5, n->target, n->act[0], n->act[1],
                 n->act[2], n->act[3], n->dA, n->dB, n->loss, n->scale, n->err};
    for (void *p : b)
        if (p) cudaFree(p);
    delete n;
    return CGS_OK;
}

cgs_status cgs_net_set_weights(cgs_net *n, const float *w)
{
    if (!n || !w) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    CGS_CUDA(cudaMemcpy(n->w, w, sizeof(float) * kParams, cudaMemcpyDefault));
    CGS_CUDA(cudaMemset(n->m, 0, sizeof(float) * kParams));
    CGS_CUDA(cudaMemset(n->v, 0, sizeof(float) * kParams));
    n->step = 0;
    CGS_TRY(net_refresh_bf16(n, nullptr));
    CGS_CUDA(cudaDeviceSynchronize());
    return CGS_OK;
}

cgs_status cgs_net_get_weights(cgs_net *n, float *w)
{
    if (!n || !w) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    CGS_CUDA(cudaMemcpy(w, n->w, sizeof(float) * kParams, cudaMemcpyDefault));
    return CGS_OK;
}

cgs_status cgs_net_forward(cgs_net *n, const float *x, float *y, int B, int H, int W, void *stream)
{
    CGS_TRY(net_check(n, B, H, W));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t bytes = sizeof(float) * (size_t)B * H * W * 2;
    CGS_CUDA(cudaMemcpyAsync(n->x0, x, bytes, cudaMemcpyDefault, st));
    CGS_TRY(net_forward_dev(n, B, H, W, st));
    CGS_CUDA(cudaMemcpyAsync(y, n->y5, bytes, cudaMemcpyDefault, st));
    CGS_CUDA(cudaStreamSynchronize(st));
    return net_check_err(n);
}

cgs_status cgs_net_set_conv_kernel(cgs_net *n, int kind)
{
    if (!n || (kind != 0 && kind != 1)) { set_error("conv kernel kind must be 0 (mma.sync) or 1 (tcgen05)"); return CGS_ERR_BAD_ARG; }
    n->conv_kind = kind;
    n->serial = ++g_net_serial;   // captured solve graphs hold the kernels by launch: rebuild them
    return CGS_OK;
}

cgs_status cgs_net_gradients(cgs_net *n, const float *x, const float *target, int B, int H, int W, float *grad,
                             float *loss, void *stream)
{
    CGS_TRY(net_check(n, B, H, W));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t bytes = sizeof(float) * (size_t)B * H * W * 2;
    CGS_CUDA(cudaMemcpyAsync(n->x0, x, bytes, cudaMemcpyDefault, st));
    CGS_CUDA(cudaMemcpyAsync(n->target, target, bytes, cudaMemcpyDefault, st));
    CGS_TRY(net_forward_dev(n, B, H, W, st));
    CGS_TRY(net_backward_dev(n, B, H, W, st));
    if (grad) CGS_CUDA(cudaMemcpyAsync(grad, n->g, sizeof(float) * kParams, cudaMemcpyDefault, st));
    if (loss) CGS_CUDA(cudaMemcpyAsync(loss, n->loss, sizeof(float), cudaMemcpyDefault, st));
    CGS_CUDA(cudaStreamSynchronize(st));
    return net_check_err(n);
}

cgs_status cgs_net_train_step(cgs_net *n, const float *x, const float *target, int B, int H, int W, float lr,
                              float *loss, void *stream)
{
    CGS_TRY(net_check(n, B, H, W));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t bytes = sizeof(float) * (size_t)B * H * W * 2;
    if (x != n->x0) CGS_CUDA(cudaMemcpyAsync(n->x0, x, bytes, cudaMemcpyDefault, st));
    if (target != n->target) CGS_CUDA(cudaMemcpyAsync(n->target, target, bytes, cudaMemcpyDefault, st));
    CGS_TRY(net_forward_dev(n, B, H, W, st));
    CGS_TRY(net_backward_dev(n, B, H, W, st));
    n->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)n->step), c2 = 1.f - std::pow(b2, (float)n->step);
    adam_kernel<<<(kParams + 255) / 256, 256, 0, st>>>(n->w, n->g, n->m, n->v, kParams, lr, b1, b2, 1e-8f, c1, c2);
    CGS_LAUNCH_CHECK();
    CGS_TRY(net_refresh_bf16(n, st));
    if (loss) {
        CGS_CUDA(cudaMemcpyAsync(loss, n->loss, sizeof(float), cudaMemcpyDefault, st));
        CGS_CUDA(cudaStreamSynchronize(st));
    }
    return CGS_OK;
}

}  // extern "C"
