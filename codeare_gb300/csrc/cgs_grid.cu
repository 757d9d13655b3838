// cgs_grid.cu -- Kaiser-Bessel interpolation (type 2) and spreading (type 1)
// between k-space nodes and the oversampled grid: the convolution step of
// NFFT3's nfft_trafo / nfft_adjoint that the reference calls per coil
// (src/matrix/ft/NFFTTraits.hpp:176-204, PRE_PSI window of :659-673).
//
// Nodes are sorted once per trajectory into bins of T^d footprint starts.  One
// CTA takes one work item (a bin, or a slice of a crowded bin) and a chunk of
// CC coils: it stages the padded grid tile ((T+2m+1)^d points x CC coils) in
// shared memory, computes the 2m+2 separable window weights of each node once,
// and then applies them to all CC coils.  Interpolation reads the tile only;
// spreading accumulates into the shared tile and adds it to the grid once per
// work item, so global atomics touch each tile point once instead of once per
// node and tap.  Grid and k-space data keep the coil index innermost.
#include "cgs_internal.cuh"
#include "cgs_tc05.cuh"

#include <algorithm>

namespace cgs {

namespace {

constexpr int kThreads = 256;
constexpr int kChunk = 128;   // nodes whose weights are staged at once
constexpr int kMaxTaps = 18;  // 2m+2 with m <= 8

struct GridCfg {
    int CC;     // coils per CTA
    int E;      // padded tile side T + 2m + 1
};

template <int D>
__device__ __forceinline__ void node_read(const float4 *nodes, int64_t s, float *frac, int *c)
{
    if (D == 2) {
        float4 a = nodes[s];
        frac[0] = a.x; frac[1] = a.y;
        c[0] = __float_as_int(a.z); c[1] = __float_as_int(a.w);
    } else {
        float4 a = nodes[2 * s], b = nodes[2 * s + 1];
        frac[0] = a.x; frac[1] = a.y; frac[2] = a.z;
        c[0] = __float_as_int(b.x); c[1] = __float_as_int(b.y); c[2] = __float_as_int(b.z);
    }
}

__device__ __forceinline__ int wrapi(int v, int n)
{
    v %= n;
    return v < 0 ? v + n : v;
}

// stage weights and local footprint origins of nodes [s0, s0+cnt)
template <int D>
__device__ __forceinline__ void stage_weights(const GridGeom &g, const NodeSet &ns, int64_t s0, int cnt,
                                              const int *org, float *wts, int *loc)
{
    const int taps = 2 * g.m + 2;
    const float mf = (float)g.m;
    for (int i = threadIdx.x; i < cnt; i += kThreads) {
        float frac[3]; int c[3];
        node_read<D>(ns.nodes, s0 + i, frac, c);
#pragma unroll
        for (int t = 0; t < D; ++t) {
            const int u = wrapi(c[t] - g.m, g.n[t]);
            loc[i * 3 + t] = u - org[t];
            float *w = wts + (i * 3 + t) * kMaxTaps;
            for (int q = 0; q < taps; ++q) w[q] = kb_phi(frac[t] + mf - (float)q, mf, g.b[t]);
        }
    }
}

template <int D>
__global__ void __launch_bounds__(kThreads)
interp_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ NodeSet ns,
              const float2 *__restrict__ grid, float2 *__restrict__ ks, int CC)
{
    extern __shared__ float4 smem4[];
    const int E = g.T + 2 * g.m + 1;
    const int taps = 2 * g.m + 2;
    const int4 wk = ns.work[blockIdx.x];
    const int c0 = blockIdx.y * CC;
    const int ccn = min(CC, g.nc - c0);
    int tidx[3], org[3];
    {
        int t = wk.x;
        for (int d = D - 1; d >= 0; --d) { tidx[d] = t % g.nt[d]; t /= g.nt[d]; }
        for (int d = 0; d < D; ++d) org[d] = tidx[d] * g.T;
    }
    int Et = 1;
    for (int d = 0; d < D; ++d) Et *= E;
    float2 *tile = reinterpret_cast<float2 *>(smem4);
    float *wts = reinterpret_cast<float *>(tile + (size_t)Et * CC);
    int *loc = reinterpret_cast<int *>(wts + kChunk * 3 * kMaxTaps);

    // 1. stage the padded tile for coils [c0, c0+ccn)
    for (int e = threadIdx.x; e < Et * ccn; e += kThreads) {
        const int cc = e % ccn;
        int r = e / ccn;
        int64_t off = 0;
        int l[3];
        for (int d = D - 1; d >= 0; --d) { l[d] = r % E; r /= E; }
        for (int d = 0; d < D; ++d) off = off * g.n[d] + wrapi(org[d] + l[d], g.n[d]);
        tile[(e / ccn) * CC + cc] = grid[off * g.nc + c0 + cc];
    }
    __syncthreads();

    for (int base = 0; base < wk.z; base += kChunk) {
        const int cnt = min(kChunk, wk.z - base);
        const int64_t s0 = (int64_t)wk.y + base;
        stage_weights<D>(g, ns, s0, cnt, org, wts, loc);
        __syncthreads();
        for (int q = threadIdx.x; q < cnt * ccn; q += kThreads) {
            const int i = q / ccn, cc = q % ccn;
            const float *w0 = wts + (i * 3 + 0) * kMaxTaps;
            const float *w1 = wts + (i * 3 + 1) * kMaxTaps;
            float ax = 0.f, ay = 0.f;
            if (D == 2) {
                const int y0 = loc[i * 3], x0 = loc[i * 3 + 1];
                for (int a = 0; a < taps; ++a) {
                    const float2 *row = tile + ((size_t)(y0 + a) * E + x0) * CC + cc;
                    float rx = 0.f, ry = 0.f;
                    for (int b = 0; b < taps; ++b) {
                        const float2 v = row[b * CC];
                        rx = fmaf(w1[b], v.x, rx); ry = fmaf(w1[b], v.y, ry);
                    }
                    ax = fmaf(w0[a], rx, ax); ay = fmaf(w0[a], ry, ay);
                }
            } else {
                const float *w2 = wts + (i * 3 + 2) * kMaxTaps;
                const int z0 = loc[i * 3], y0 = loc[i * 3 + 1], x0 = loc[i * 3 + 2];
                for (int a = 0; a < taps; ++a) {
                    float px = 0.f, py = 0.f;
                    for (int b = 0; b < taps; ++b) {
                        const float2 *row = tile + (((size_t)(z0 + a) * E + y0 + b) * E + x0) * CC + cc;
                        float rx = 0.f, ry = 0.f;
                        for (int c = 0; c < taps; ++c) {
                            const float2 v = row[c * CC];
                            rx = fmaf(w2[c], v.x, rx); ry = fmaf(w2[c], v.y, ry);
                        }
                        px = fmaf(w1[b], rx, px); py = fmaf(w1[b], ry, py);
                    }
                    ax = fmaf(w0[a], px, ax); ay = fmaf(w0[a], py, ay);
                }
            }
            ks[(s0 + i) * g.nc + c0 + cc] = make_float2(ax, ay);
        }
        __syncthreads();
    }
}

template <int D>
__global__ void __launch_bounds__(kThreads)
spread_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ NodeSet ns,
              const float2 *__restrict__ ks, int weighted, float2 *__restrict__ grid, int CC)
{
    extern __shared__ float4 smem4[];
    const int E = g.T + 2 * g.m + 1;
    const int taps = 2 * g.m + 2;
    const int4 wk = ns.work[blockIdx.x];
    const int c0 = blockIdx.y * CC;
    const int ccn = min(CC, g.nc - c0);
    int tidx[3], org[3];
    {
        int t = wk.x;
        for (int d = D - 1; d >= 0; --d) { tidx[d] = t % g.nt[d]; t /= g.nt[d]; }
        for (int d = 0; d < D; ++d) org[d] = tidx[d] * g.T;
    }
    int Et = 1;
    for (int d = 0; d < D; ++d) Et *= E;
    float2 *tile = reinterpret_cast<float2 *>(smem4);
    float *wts = reinterpret_cast<float *>(tile + (size_t)Et * CC);
    int *loc = reinterpret_cast<int *>(wts + kChunk * 3 * kMaxTaps);

    for (int e = threadIdx.x; e < Et * CC; e += kThreads) tile[e] = make_float2(0.f, 0.f);
    __syncthreads();

    for (int base = 0; base < wk.z; base += kChunk) {
        const int cnt = min(kChunk, wk.z - base);
        const int64_t s0 = (int64_t)wk.y + base;
        stage_weights<D>(g, ns, s0, cnt, org, wts, loc);
        __syncthreads();
        for (int q = threadIdx.x; q < cnt * ccn; q += kThreads) {
            const int i = q / ccn, cc = q % ccn;
            float2 v = ks[(s0 + i) * g.nc + c0 + cc];
            if (weighted && ns.w) { const float ww = ns.w[s0 + i]; v.x *= ww; v.y *= ww; }
            const float *w0 = wts + (i * 3 + 0) * kMaxTaps;
            const float *w1 = wts + (i * 3 + 1) * kMaxTaps;
            if (D == 2) {
                const int y0 = loc[i * 3], x0 = loc[i * 3 + 1];
                for (int a = 0; a < taps; ++a) {
                    const float vx = w0[a] * v.x, vy = w0[a] * v.y;
                    float2 *row = tile + ((size_t)(y0 + a) * E + x0) * CC + cc;
                    for (int b = 0; b < taps; ++b) {
                        atomicAdd(&row[b * CC].x, w1[b] * vx);
                        atomicAdd(&row[b * CC].y, w1[b] * vy);
                    }
                }
            } else {
                const float *w2 = wts + (i * 3 + 2) * kMaxTaps;
                const int z0 = loc[i * 3], y0 = loc[i * 3 + 1], x0 = loc[i * 3 + 2];
                for (int a = 0; a < taps; ++a)
                    for (int b = 0; b < taps; ++b) {
                        const float wab = w0[a] * w1[b];
                        const float vx = wab * v.x, vy = wab * v.y;
                        float2 *row = tile + (((size_t)(z0 + a) * E + y0 + b) * E + x0) * CC + cc;
                        for (int c = 0; c < taps; ++c) {
                            atomicAdd(&row[c * CC].x, w2[c] * vx);
                            atomicAdd(&row[c * CC].y, w2[c] * vy);
                        }
                    }
            }
        }
        __syncthreads();
    }

    // add the tile to the grid (wrapped)
    for (int e = threadIdx.x; e < Et * ccn; e += kThreads) {
        const int cc = e % ccn;
        int r = e / ccn;
        int64_t off = 0;
        int l[3];
        for (int d = D - 1; d >= 0; --d) { l[d] = r % E; r /= E; }
        for (int d = 0; d < D; ++d) off = off * g.n[d] + wrapi(org[d] + l[d], g.n[d]);
        const float2 v = tile[(e / ccn) * CC + cc];
        if (v.x != 0.f || v.y != 0.f) {
            float2 *dst = grid + off * g.nc + c0 + cc;
            atomicAdd(&dst->x, v.x);
            atomicAdd(&dst->y, v.y);
        }
    }
}

// window weights and wrapped footprint starts of every node (once per trajectory)
__global__ void node_weights_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ NodeSet ns,
                                    int2 *__restrict__ nodeU, float *__restrict__ nodeW)
{
    const int taps = 2 * g.m + 2;
    const float mf = (float)g.m;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < ns.M; s += (int64_t)gridDim.x * blockDim.x) {
        float frac[3]; int c[3];
        node_read<2>(ns.nodes, s, frac, c);
        nodeU[s] = make_int2(wrapi(c[0] - g.m, g.n[0]), wrapi(c[1] - g.m, g.n[1]));
        float *w = nodeW + s * 2 * taps;
        for (int t = 0; t < 2; ++t)
            for (int q = 0; q < taps; ++q) w[t * taps + q] = kb_phi(frac[t] + mf - (float)q, mf, g.b[t]);
    }
}

// ---------------------------------------------------------------------------
// Output-stationary 2-D spreading.  A warp owns a PH x PW patch of grid
// points: its 32 lanes form G = 32 / (PH PW) coil groups, lane l serves point
// l mod (PH PW) for the group's CPL coils, accumulated in registers, while
// the warp walks the patch's node list.  Batches of kSpreadBatch list entries
// (node values of the warp's CC = G CPL coils, window weights, footprint
// start, density weight) are staged in shared memory by cp.async, double
// buffered, so the next batch streams in while the current one is summed;
// each node value reaches its group by a broadcast load.  Two FP32 lanes of a
// complex accumulator update with one paired FMA (fma.rn.f32x2, the same
// rounding as two fmaf).  No atomics anywhere: a crowded patch is split into
// several work items whose partial sums land in `partial` and are added in
// slot order by patch_reduce_kernel, so results are bitwise reproducible.
// ---------------------------------------------------------------------------
constexpr int kSpreadBatch = 8;

__device__ __forceinline__ void cp_async4(void *dst, const void *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void *dst, const void *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// acc + w * v on both FP32 lanes of a complex value
__device__ __forceinline__ float2 ffma2(float2 w, float2 v, float2 acc)
{
    unsigned long long r;
    const unsigned long long a = *reinterpret_cast<const unsigned long long *>(&w);
    const unsigned long long b = *reinterpret_cast<const unsigned long long *>(&v);
    const unsigned long long c = *reinterpret_cast<const unsigned long long *>(&acc);
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return *reinterpret_cast<float2 *>(&r);
}

template <int PH, int PW, int CPL, int BY, int BX>
struct SpreadShape {
    static constexpr int NPT = PH * PW;                        // points per patch
    static constexpr int L = (PH / BY) * (PW / BX);            // lanes per coil group (BY x BX points each)
    static constexpr int G = 32 / L;                           // coil groups per warp
    static constexpr int CC = G * CPL;                         // coils per warp
    static constexpr int GS = (CPL % 2 == 0) ? CPL + 2 : CPL;  // group stride (float2): groups 16 B apart in banks
    static constexpr int VR = G * GS;                          // staged value row per entry (float2)
    static_assert(L * G == 32 && PH % BY == 0 && PW % BX == 0, "a patch must tile the warp");
    // one staging buffer: values, weights, footprint starts, density weights
    __host__ __device__ static size_t buf_bytes(int taps)
    {
        return (size_t)kSpreadBatch * (VR * sizeof(float2) + 2 * taps * sizeof(float) + sizeof(int2) + sizeof(float));
    }
};

// TAPS > 0 fixes the footprint width at compile time (0: 2m + 2 at run time)
template <int PH, int PW, int CPL, int BY, int BX, int TAPS = 0>
__global__ void __launch_bounds__(256, (BY * BX <= 2) ? 3 : 2)
spread_patch_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ PatchSet ps,
                    const float2 *__restrict__ ks, const float *__restrict__ dens, int weighted,
                    float2 *__restrict__ grid)
{
    using S = SpreadShape<PH, PW, CPL, BY, BX>;
    constexpr int NB = BY * BX;                            // points per lane
    extern __shared__ float4 smem4[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wi = blockIdx.x * 8 + warp;
    if (wi >= ps.nwork) return;
    const int taps = TAPS > 0 ? TAPS : 2 * g.m + 2;
    const int WS = 2 * taps;                               // weights per entry (a multiple of 4)
    const size_t bb = S::buf_bytes(taps);
    char *wbase = reinterpret_cast<char *>(smem4) + (size_t)warp * 2 * bb;
    const int c0 = blockIdx.y * S::CC;
    const int ccn = min(S::CC, g.nc - c0);
    const bool v16 = ((g.nc & 1) == 0);                    // node rows 16-byte aligned: two coils per copy
    const int4 wk = ps.work[wi];
    const int n0 = g.n[0], n1 = g.n[1];
    const int pt = lane % S::L, cg = lane / S::L;
    const int by = (pt / (PW / BX)) * BY, bx = (pt % (PW / BX)) * BX;   // block origin in the patch
    const int py = (wk.x / ps.npx) * PH + by;
    const int px = (wk.x % ps.npx) * PW + bx;
    const bool wide = (n0 >= taps) && (n1 >= taps);        // no footprint wraps onto itself

    auto buffers = [&](int buf, float2 *&sv, float *&sw, int2 *&su, float *&sd) {
        char *b = wbase + (size_t)buf * bb;
        sv = reinterpret_cast<float2 *>(b);
        sw = reinterpret_cast<float *>(sv + kSpreadBatch * S::VR);
        su = reinterpret_cast<int2 *>(sw + kSpreadBatch * WS);
        sd = reinterpret_cast<float *>(su + kSpreadBatch);
    };
    // queue the copies of entries [e0, e0 + cnt) into buffer `buf`
    auto issue = [&](int e0, int cnt, int buf) {
        float2 *sv; float *sw; int2 *su; float *sd;
        buffers(buf, sv, sw, su, sd);
        const int s_l = (lane < cnt) ? ps.entries[e0 + lane] : 0;
        if (lane < cnt) {
            cp_async8(&su[lane], &ps.nodeU[s_l]);
            if (weighted) cp_async4(&sd[lane], &dens[s_l]);
            else sd[lane] = 1.f;
            const float *W = ps.nodeW + (size_t)s_l * WS;
            for (int q = 0; q < WS; q += 4) cp_async16(&sw[lane * WS + q], W + q);
        }
        for (int j = 0; j < cnt; ++j) {
            const int s = __shfl_sync(0xffffffffu, s_l, j);
            const float2 *v = ks + (size_t)s * g.nc + c0;
            float2 *dv = sv + j * S::VR;
            if (v16 && (S::CC % 2 == 0)) {
                const int c = 2 * lane;
                if (c < S::CC) {
                    float2 *d = dv + (c / CPL) * S::GS + (c % CPL);
                    if (c + 1 < ccn) cp_async16(d, v + c);
                    else if (c < ccn) { cp_async8(d, v + c); d[1] = make_float2(0.f, 0.f); }
                    else { d[0] = make_float2(0.f, 0.f); d[1] = make_float2(0.f, 0.f); }
                }
            } else {
                for (int c = lane; c < S::CC; c += 32) {
                    float2 *d = dv + (c / CPL) * S::GS + (c % CPL);
                    if (c < ccn) cp_async8(d, v + c);
                    else *d = make_float2(0.f, 0.f);
                }
            }
        }
        cp_async_commit();
    };

    float2 acc[NB][CPL];
#pragma unroll
    for (int q = 0; q < NB; ++q)
#pragma unroll
        for (int k = 0; k < CPL; ++k) acc[q][k] = make_float2(0.f, 0.f);
    const int end = wk.y + wk.z;
    int e0 = wk.y, cnt = min(kSpreadBatch, end - e0), buf = 0;
    issue(e0, cnt, 0);
    while (true) {
        const int e1 = e0 + cnt;
        const int cnt1 = min(kSpreadBatch, end - e1);
        if (cnt1 > 0) { issue(e1, cnt1, buf ^ 1); cp_async_wait<1>(); }
        else cp_async_wait<0>();
        __syncwarp();
        float2 *sv; float *sw; int2 *su; float *sd;
        buffers(buf, sv, sw, su, sd);
        for (int i = 0; i < cnt; ++i) {
            const int2 u = su[i];
            const float *W = sw + i * WS;
            const float d = sd[i];
            float wy[BY], wx[BX];
#pragma unroll
            for (int yy = 0; yy < BY; ++yy) {
                wy[yy] = 0.f;
                if (py + yy < n0) {
                    int dy = py + yy - u.x; if (dy < 0) dy += n0;
                    if (wide) wy[yy] = (dy < taps) ? W[dy] : 0.f;
                    else for (int q = dy; q < taps; q += n0) wy[yy] += W[q];
                }
            }
#pragma unroll
            for (int xx = 0; xx < BX; ++xx) {
                wx[xx] = 0.f;
                if (px + xx < n1) {
                    int dx = px + xx - u.y; if (dx < 0) dx += n1;
                    if (wide) wx[xx] = (dx < taps) ? W[taps + dx] : 0.f;
                    else for (int q = dx; q < taps; q += n1) wx[xx] += W[taps + q];
                }
            }
            float2 ww[NB];
#pragma unroll
            for (int yy = 0; yy < BY; ++yy)
#pragma unroll
                for (int xx = 0; xx < BX; ++xx) {
                    const float w = wy[yy] * wx[xx] * d;
                    ww[yy * BX + xx] = make_float2(w, w);
                }
            const float2 *vr = sv + i * S::VR + cg * S::GS;
            if constexpr (CPL % 2 == 0) {
                const float4 *v4 = reinterpret_cast<const float4 *>(vr);
#pragma unroll
                for (int k = 0; k < CPL / 2; ++k) {
                    const float4 q = v4[k];
#pragma unroll
                    for (int b = 0; b < NB; ++b) {
                        acc[b][2 * k] = ffma2(ww[b], make_float2(q.x, q.y), acc[b][2 * k]);
                        acc[b][2 * k + 1] = ffma2(ww[b], make_float2(q.z, q.w), acc[b][2 * k + 1]);
                    }
                }
            } else {
#pragma unroll
                for (int k = 0; k < CPL; ++k) {
                    const float2 q = vr[k];
#pragma unroll
                    for (int b = 0; b < NB; ++b) acc[b][k] = ffma2(ww[b], q, acc[b][k]);
                }
            }
        }
        __syncwarp();
        if (cnt1 <= 0) break;
        e0 = e1; cnt = cnt1; buf ^= 1;
    }
    const int cb = c0 + cg * CPL;                          // first coil of this lane's group
#pragma unroll
    for (int yy = 0; yy < BY; ++yy)
#pragma unroll
        for (int xx = 0; xx < BX; ++xx) {
            if (py + yy >= n0 || px + xx >= n1) continue;
            const int ppt = (by + yy) * PW + bx + xx;       // point index within the patch
            float2 *dst = (wk.w < 0) ? grid + ((size_t)(py + yy) * n1 + px + xx) * g.nc + cb
                                     : ps.partial + ((size_t)wk.w * S::NPT + ppt) * g.nc + cb;
#pragma unroll
            for (int k = 0; k < CPL; ++k)
                if (cg * CPL + k < ccn) dst[k] = acc[yy * BX + xx][k];
        }
}

// ---------------------------------------------------------------------------
// Spreading on the tensor cores.  A warp owns a 4 x 4 patch and 4 NT coils;
// each batch of kSpreadBatch = 8 list entries is one k-step of
// mma.m16n8k8 (TF32 operands, FP32 accumulation):
//   D[16 points][8 NT cols] += W[16 points][8 entries] V[8 entries][8 NT cols]
// W holds the entries' window weights at the patch points (wy * wx *
// density), V their coil values (column 2c and 2c + 1: Re and Im of coil c).
// Both operands are split into a TF32 value and its TF32 remainder and the
// products lo*hi, hi*lo, hi*hi are accumulated (the dropped lo*lo is below
// 2^-22 relative), which keeps the accuracy of FP32 fused multiply-adds.
// Fragments follow the PTX ISA layout of m16n8k8 .tf32: thread (g = lane/4,
// t = lane%4) holds A rows g, g+8 x columns t, t+4; B rows t, t+4 x column g;
// D rows g, g+8 x columns 2t, 2t+1.  Patch point r is row r (row-major 4 x 4),
// so rows g and g+8 are the same column, two rows apart.
// ---------------------------------------------------------------------------
// staged value row in floats: at least 8 NT and 8 or 24 mod 32, so the B
// loads of entry rows t and t + 4 (t = 0..3) fall in distinct banks
__host__ __device__ constexpr int spread_mma_row(int nt)
{
    int r = 8 * nt;
    while (r % 32 != 8 && r % 32 != 24) r += 8;
    return r;
}

template <int NT, int MT = 1> struct SpreadMma {
    static constexpr int R = spread_mma_row(NT);
    static constexpr int WPE = 4 * MT + 4;                 // patch weights per entry: 4 MT rows, 4 columns
    // one staging buffer: values, window taps, footprint starts, density weights
    __host__ __device__ static size_t buf_bytes(int taps)
    {
        return (size_t)kSpreadBatch * (R * sizeof(float) + 2 * taps * sizeof(float) + sizeof(int2) + sizeof(float));
    }
    // per warp: two buffers and the batch's patch weights
    __host__ __device__ static size_t warp_bytes(int taps) { return 2 * buf_bytes(taps) + kSpreadBatch * WPE * sizeof(float); }
};

// TF32 split: hi = x rounded to the nearest TF32 value (half a TF32 unit,
// bit 12, added to the magnitude bits, then the 13 low mantissa bits
// cleared), lo = x - hi (exact in FP32, |lo| <= 2^-11 |x|, either sign)
// passed as is; the tensor cores read the upper 19 bits of a .tf32 operand,
// so lo loses its low bits there and hi*hi + hi*lo + lo*hi carries ~2^-21
// relative error per product, without bias because lo takes both signs
// (a truncated hi would give lo the sign of x and bias every product low).
// Two full-rate integer ops instead of a rounding conversion keep the split
// off the conversion pipe.
__device__ __forceinline__ void tf32_split(float x, uint32_t &hi, uint32_t &lo)
{
    hi = (__float_as_uint(x) + 0x1000u) & 0xffffe000u;
    lo = __float_as_uint(x - __uint_as_float(hi));
}

// x * y on both FP32 lanes (the rounding of two FP32 multiplies)
__device__ __forceinline__ float2 fmul2(float2 x, float2 y) { return ffma2(x, y, make_float2(0.f, 0.f)); }

// tf32_split on two values; the remainders x - hi (exact) with one paired
// FMA, so the result is the same as two tf32_split calls
__device__ __forceinline__ void tf32_split2(float2 x, uint32_t &h0, uint32_t &h1, uint32_t &l0, uint32_t &l1)
{
    h0 = (__float_as_uint(x.x) + 0x1000u) & 0xffffe000u;
    h1 = (__float_as_uint(x.y) + 0x1000u) & 0xffffe000u;
    const float2 lo = ffma2(make_float2(-1.f, -1.f), make_float2(__uint_as_float(h0), __uint_as_float(h1)), x);
    l0 = __float_as_uint(lo.x);
    l1 = __float_as_uint(lo.y);
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// MT m-tiles: a (4 MT) x 4 patch, each m-tile four patch rows
template <int NT, int TAPS = 0, int MT = 1>
__global__ void __launch_bounds__(256, MT == 1 ? 3 : 2)
spread_mma_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ PatchSet ps,
                  const float2 *__restrict__ ks, const float *__restrict__ dens, int weighted,
                  float2 *__restrict__ grid)
{
    using S = SpreadMma<NT, MT>;
    constexpr int WPE = S::WPE;
    constexpr int R = S::R, CC = 4 * NT, CH = 2 * NT;     // coils per warp; 16-byte chunks per entry row
    extern __shared__ float4 smem4[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wi = blockIdx.x * 8 + warp;
    if (wi >= ps.nwork) return;
    const int taps = TAPS > 0 ? TAPS : 2 * g.m + 2;
    const int WS = 2 * taps;
    const size_t bb = S::buf_bytes(taps);                  // a multiple of 16 bytes
    char *wbase = reinterpret_cast<char *>(smem4) + (size_t)warp * S::warp_bytes(taps);
    float *swt = reinterpret_cast<float *>(wbase + 2 * bb);   // [entry][wy 0..4MT-1, wx 0..3]
    const int c0 = blockIdx.y * CC;
    const int ccn = min(CC, g.nc - c0);
    const bool v16 = ((g.nc & 1) == 0);
    const int4 wk = ps.work[wi];
    const int n0 = g.n[0], n1 = g.n[1];
    const int gq = lane >> 2, tq = lane & 3;
    const int py0 = (wk.x / ps.npx) * (4 * MT), px0 = (wk.x % ps.npx) * 4;
    const bool wide = (n0 >= taps) && (n1 >= taps);
    // zero both buffers once: padding columns and rows past a short batch stay finite
    {
        float4 *z = reinterpret_cast<float4 *>(wbase);
        const int n16 = (int)(2 * bb / 16);
        for (int i = lane; i < n16; i += 32) z[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        __syncwarp();
    }
    auto buffers = [&](int buf, float *&sv, float *&sw, int2 *&su, float *&sd) {
        char *b = wbase + (size_t)buf * bb;
        sv = reinterpret_cast<float *>(b);
        sw = sv + kSpreadBatch * R;
        su = reinterpret_cast<int2 *>(sw + kSpreadBatch * WS);
        sd = reinterpret_cast<float *>(su + kSpreadBatch);
    };
    auto issue = [&](int e0, int cnt, int buf) {
        float *sv, *sw, *sd; int2 *su;
        buffers(buf, sv, sw, su, sd);
        const int s_l = (lane < cnt) ? ps.entries[e0 + lane] : 0;
        if (lane < cnt) {
            cp_async8(&su[lane], &ps.nodeU[s_l]);
            if (weighted) cp_async4(&sd[lane], &dens[s_l]);
            else sd[lane] = 1.f;
            const float *W = ps.nodeW + (size_t)s_l * WS;
            for (int q = 0; q < WS; q += 4) cp_async16(&sw[lane * WS + q], W + q);
        }
        if (v16) {
            // all lanes: chunk ch = entry ch / CH, coils 2 (ch % CH) and 2 (ch % CH) + 1
#pragma unroll
            for (int i = 0; i < (kSpreadBatch * CH + 31) / 32; ++i) {
                const int ch = lane + 32 * i;
                const int e = ch / CH, c = 2 * (ch % CH);
                const int s = __shfl_sync(0xffffffffu, s_l, e & (kSpreadBatch - 1));
                if (ch < kSpreadBatch * CH && e < cnt && c < ccn) {
                    const float2 *v = ks + (size_t)s * g.nc + c0 + c;
                    float2 *d = reinterpret_cast<float2 *>(sv + e * R) + c;
                    if (c + 1 < ccn) cp_async16(d, v);
                    else cp_async8(d, v);
                }
            }
        } else {
            for (int j = 0; j < cnt; ++j) {
                const int s = __shfl_sync(0xffffffffu, s_l, j);
                const float2 *v = ks + (size_t)s * g.nc + c0;
                float2 *dv = reinterpret_cast<float2 *>(sv + j * R);
                for (int c = lane; c < ccn; c += 32) cp_async8(dv + c, v + c);
            }
        }
        cp_async_commit();
    };
    // window weight of one axis at offset q from the footprint start
    auto wgt = [&](const float *W, int q, int n) -> float {
        if (q < 0) q += n;
        if (wide) return q < taps ? W[q] : 0.f;
        float w = 0.f;
        for (int r = q; r < taps; r += n) w += W[r];
        return w;
    };

    float acc[MT][NT][4];
#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
#pragma unroll
        for (int t = 0; t < NT; ++t) acc[mt][t][0] = acc[mt][t][1] = acc[mt][t][2] = acc[mt][t][3] = 0.f;
    const int end = wk.y + wk.z;
    int e0 = wk.y, cnt = min(kSpreadBatch, end - e0), buf = 0;
    issue(e0, cnt, 0);
    while (true) {
        const int e1 = e0 + cnt;
        const int cnt1 = min(kSpreadBatch, end - e1);
        if (cnt1 > 0) { issue(e1, cnt1, buf ^ 1); cp_async_wait<1>(); }
        else cp_async_wait<0>();
        __syncwarp();
        float *sv, *sw, *sd; int2 *su;
        buffers(buf, sv, sw, su, sd);
        // the batch's patch weights: (entry e, row or column r) per lane; zero past cnt
#pragma unroll
        for (int idx = lane; idx < kSpreadBatch * WPE; idx += 32) {
            const int e = idx / WPE, r = idx % WPE;
            float w = 0.f;
            if (e < cnt) {
                const int2 u = su[e];
                const float *W = sw + e * WS;
                if (r < 4 * MT) {
                    if (py0 + r < n0) w = wgt(W, py0 + r - u.x, n0);
                } else if (px0 + r - 4 * MT < n1) {
                    w = wgt(W + taps, px0 + r - 4 * MT - u.y, n1) * sd[e];
                }
            }
            swt[idx] = w;
        }
        __syncwarp();
        // A of m-tile mt: entries tq and tq + 4 at patch rows 4 mt + gq / 4 (+ 2), column gq % 4
        uint32_t ah[MT][4], al[MT][4];
#pragma unroll
        for (int mt = 0; mt < MT; ++mt)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const float *wr = swt + (tq + 4 * h) * WPE;
                const float wx = wr[4 * MT + (gq & 3)];
                tf32_split(wr[4 * mt + (gq >> 2)] * wx, ah[mt][2 * h], al[mt][2 * h]);
                tf32_split(wr[4 * mt + (gq >> 2) + 2] * wx, ah[mt][2 * h + 1], al[mt][2 * h + 1]);
            }
        const float *r0 = sv + tq * R + gq, *r1 = sv + (tq + 4) * R + gq;
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            uint32_t bh0, bl0, bh1, bl1;
            tf32_split2(make_float2(r0[8 * t], r1[8 * t]), bh0, bh1, bl0, bl1);
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) {
                mma_tf32(acc[mt][t], al[mt], bh0, bh1);
                mma_tf32(acc[mt][t], ah[mt], bl0, bl1);
                mma_tf32(acc[mt][t], ah[mt], bh0, bh1);
            }
        }
        __syncwarp();
        if (cnt1 <= 0) break;
        e0 = e1; cnt = cnt1; buf ^= 1;
    }
    const int px = px0 + (gq & 3);
#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int yy = py0 + 4 * mt + (gq >> 2) + 2 * h;
            if (yy >= n0 || px >= n1) continue;
            const int ppt = 16 * mt + gq + 8 * h;           // point index within the patch (row-major, 4 wide)
            float2 *dst = (wk.w < 0) ? grid + ((size_t)yy * n1 + px) * g.nc + c0
                                     : ps.partial + ((size_t)wk.w * 16 * MT + ppt) * g.nc + c0;
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                const int c = 4 * t + tq;
                if (c < ccn) dst[c] = make_float2(acc[mt][t][2 * h], acc[mt][t][2 * h + 1]);
            }
        }
}

// ---------------------------------------------------------------------------
// 2-D spreading on the 5th-generation tensor cores (tcgen05), output-
// stationary over 8 x 16 grid patches (spread_block 64).  A 256-thread CTA
// owns one work item (a patch, or a slice of a crowded patch's node list) and
// NCOL / 2 coils: D[128 points][NCOL columns] = W[128][K entries] .
// V[K entries][NCOL], columns = (coil, re/im), accumulated in FP32 in NCOL
// tensor-memory columns.  The entries stream in stages of kSpTcKS:
//   * once per trajectory, spread_tc_weights_kernel stores every stage's
//     patch weights (8 row and 16 column window values per entry, entries
//     innermost) and node indices as one contiguous block, so a stage needs
//     no per-node lookups;
//   * cp.async brings a stage's weight block three stages ahead and its
//     k-space values and density weights two stages ahead (rings of four and
//     three slots, one commit group per kind and stage);
//   * A = W, TF32-split into hi and lo (tf32_split2), lives in tensor memory
//     (row m in lane m, entries along the columns): thread m % 128 of warps
//     m / 32 and m / 32 + 4 (point m = 16 r + c of the patch) multiplies its
//     row and column weights for 8 of the stage's 16 entries and stores them
//     with tcgen05.st;
//   * B = V^T (the values times the density weights), split the same way:
//     a thread per (coil, 4 entries), stored K-major in shared memory in the
//     canonical no-swizzle layout (core matrices of 8 rows x 4 values);
//   * both in one of two stage buffers; a ninth warp waits for a buffer's
//     "full" mbarrier, issues per K = 8 step lo.hi + hi.lo + hi.hi as three
//     tcgen05.mma.kind::tf32 and commits them to the buffer's "empty"
//     mbarrier, while the builders fill the other buffer.
// Before a buffer is rebuilt its mbarrier is waited on, with a bounded wait:
// past the limit the CTA sets *ps.err, stores nothing and still frees its
// tensor memory.  The epilogue reads the accumulator with tcgen05.ld (warps w
// and w + 4: points 32 (w % 4) .., the lower and the upper half of the
// columns) and stores each point's coils to the grid, or to the work item's
// partial slot, reduced in slot order by patch_reduce_kernel as for the other
// kernels.  Entries past the list end and coils past the chunk are zero in A
// and B.
// ---------------------------------------------------------------------------
constexpr int kSpTcPH = 8, kSpTcPW = 16;     // patch rows and columns: 128 points = the MMA's M
constexpr int kSpTcKS = 16;                  // entries per stage: two K = 8 steps
constexpr int kSpTcWPE = kSpTcPH + kSpTcPW;  // patch weights per entry
constexpr int kSpTcWS = kSpTcKS + 4;         // weight row stride in shared memory (floats), bank-spread
constexpr int kSpTcThreads = 256;
constexpr uint64_t kSpTcWaitNs = 1000000000ull;   // a bounded mbarrier wait gives up after 1 s

template <int NCOL> struct SpreadTc {
    static constexpr int B = NCOL * kSpTcKS * 4;        // one of hi / lo
    static constexpr int LBO_B = (NCOL / 8) * 128;     // next 4 entries: past the NCOL / 8 column groups
    static constexpr int OPER = 2 * B;                 // B hi, lo (A lives in tensor memory)
    static constexpr int WSLOT = kSpTcWPE * kSpTcWS * 4 + kSpTcKS * 4;   // weights, node indices
    static constexpr int VSLOT = kSpTcKS * NCOL * 4 + kSpTcKS * 4;       // values, density weights
    static constexpr int NW = 4, NV = 3;                                // ring slots
    static constexpr int SMEM = 2 * OPER + NW * WSLOT + NV * VSLOT + 48;  // + four mbarriers, TMEM slot, flag
    // tensor memory: the accumulator in columns 0 .. NCOL - 1, then per stage
    // buffer 16 hi and 16 lo columns of A
    static constexpr int ACOL = 64;
    static constexpr int TCOLS = 128;
};


// the stage blocks of one work item per CTA: patch weights [24][16] and node
// indices [16] of entries j * 16 .. j * 16 + 15 of the item's list
__global__ void spread_tc_weights_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ PatchSet ps,
                                         float *__restrict__ pw16, int *__restrict__ ps16)
{
    const int4 wk = ps.work[blockIdx.x];
    const int base = ps.pstage[blockIdx.x];
    const int nst = (wk.z + kSpTcKS - 1) / kSpTcKS;
    const int n0 = g.n[0], n1 = g.n[1], taps = 2 * g.m + 2;
    const bool wide = (n0 >= taps) && (n1 >= taps);
    const int py0 = (wk.x / ps.npx) * kSpTcPH, px0 = (wk.x % ps.npx) * kSpTcPW;
    auto wgt = [&](const float *W, int q, int n) -> float {
        if (q < 0) q += n;
        if (wide) return q < taps ? W[q] : 0.f;
        float w = 0.f;
        for (int r = q; r < taps; r += n) w += W[r];
        return w;
    };
    constexpr int PER = kSpTcKS * (kSpTcWPE + 1);
    for (int idx = threadIdx.x; idx < nst * PER; idx += blockDim.x) {
        const int j = idx / PER, rem = idx % PER, q = rem / kSpTcKS, e = rem % kSpTcKS;
        const int ei = j * kSpTcKS + e;
        const int s = ei < wk.z ? ps.entries[wk.y + ei] : -1;
        const int64_t blk = (int64_t)base + j;
        if (q == kSpTcWPE) {
            ps16[blk * kSpTcKS + e] = s;
            continue;
        }
        float w = 0.f;
        if (s >= 0) {
            const int2 u = ps.nodeU[s];
            const float *W = ps.nodeW + (size_t)s * 2 * taps;
            if (q < kSpTcPH) {
                if (py0 + q < n0) w = wgt(W, py0 + q - u.x, n0);
            } else if (px0 + q - kSpTcPH < n1) {
                w = wgt(W + taps, px0 + q - kSpTcPH - u.y, n1);
            }
        }
        pw16[(blk * kSpTcWPE + q) * kSpTcKS + e] = w;
    }
}

// named barrier 1 over the 256 builder threads (warps 0..7); the second form
// also returns the OR of `v` over them, the same value in every thread
__device__ __forceinline__ void builders_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kSpTcThreads) : "memory"); }
__device__ __forceinline__ bool builders_sync_or(bool v)
{
    uint32_t r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, 1, %2, p;\n\t"
                 "selp.u32 %0, 1, 0, q;\n\t}" : "=r"(r) : "r"((uint32_t)v), "n"(kSpTcThreads) : "memory");
    return r != 0;
}
// mbarrier arrive (one count), release at CTA scope
__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc05::smem_u32(bar)) : "memory");
}

template <int NCOL>
__global__ void __launch_bounds__(kSpTcThreads + 32, 4)
spread_tc05_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ PatchSet ps,
                   const float2 *__restrict__ ks, const float *__restrict__ dens, int weighted,
                   float2 *__restrict__ grid)
{
    using S = SpreadTc<NCOL>;
    constexpr int CC = NCOL / 2;
    extern __shared__ __align__(128) uint8_t tsm[];
    uint8_t *wring = tsm + 2 * S::OPER;
    uint8_t *vring = wring + S::NW * S::WSLOT;
    uint64_t *full = reinterpret_cast<uint64_t *>(vring + S::NV * S::VSLOT);   // operands of buffer b built
    uint64_t *empty = full + 2;                                                  // MMAs of buffer b done
    uint32_t *tslot = reinterpret_cast<uint32_t *>(empty + 2);
    volatile int *sfail = reinterpret_cast<volatile int *>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int4 wk = ps.work[blockIdx.x];
    const int64_t base = ps.pstage[blockIdx.x];
    const int c0 = blockIdx.y * CC;
    const int ccn = min(CC, g.nc - c0);
    const int n0 = g.n[0], n1 = g.n[1];
    const bool v16 = (g.nc & 1) == 0;
    const int py0 = (wk.x / ps.npx) * kSpTcPH, px0 = (wk.x % ps.npx) * kSpTcPW;
    const int nst = (wk.z + kSpTcKS - 1) / kSpTcKS;

    auto wslot = [&](int j) { return reinterpret_cast<float *>(wring + (j % S::NW) * S::WSLOT); };
    auto vslot = [&](int j) { return reinterpret_cast<float *>(vring + (j % S::NV) * S::VSLOT); };
    // stage j's weight block (24 rows of 16 entries -> rows kSpTcWS apart) and
    // node indices: threads 0..99
    auto fetch_w = [&](int j) {
        float *d = wslot(j);
        const int64_t blk = base + j;
        if (tid < kSpTcWPE * 4) {
            const int q = tid >> 2, k = tid & 3;
            cp_async16(d + q * kSpTcWS + 4 * k, ps.pw16 + (blk * kSpTcWPE + q) * kSpTcKS + 4 * k);
        } else if (tid < kSpTcWPE * 4 + 4) {
            const int k = tid - kSpTcWPE * 4;
            cp_async16(d + kSpTcWPE * kSpTcWS + 4 * k, ps.ps16 + blk * kSpTcKS + 4 * k);
        }
    };
    // stage j's values and density weights (its node indices are in
    // wslot(j)): threads 0..127
    auto fetch_v = [&](int j) {
        const int *sidx = reinterpret_cast<const int *>(wslot(j) + kSpTcWPE * kSpTcWS);
        float *sv = vslot(j), *sd = sv + kSpTcKS * NCOL;
        if (tid < kSpTcKS) {
            const int s = sidx[tid];
            if (s >= 0 && weighted) cp_async4(&sd[tid], &dens[s]);
            else sd[tid] = 1.f;
        }
        if (v16) {                                                  // two coils per 16-byte piece
            for (int it = tid; it < kSpTcKS * (CC / 2); it += 128) {
                const int e = it / (CC / 2), q = it % (CC / 2);
                const int s = sidx[e];
                float *d = sv + e * NCOL + 4 * q;
                if (s >= 0 && 2 * q < ccn) cp_async16(d, ks + (size_t)s * g.nc + c0 + 2 * q);
                else *reinterpret_cast<float4 *>(d) = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        } else {
            for (int it = tid; it < kSpTcKS * CC; it += 128) {
                const int e = it / CC, q = it % CC;
                const int s = sidx[e];
                float *d = sv + e * NCOL + 2 * q;
                if (s >= 0 && q < ccn) cp_async8(d, ks + (size_t)s * g.nc + c0 + q);
                else *reinterpret_cast<float2 *>(d) = make_float2(0.f, 0.f);
            }
        }
    };

    if (warp == kSpTcThreads / 32) tc05::alloc<S::TCOLS>(tslot);
    if (tid == 0) {
        for (int k = 0; k < 2; ++k) {
            tc05::mbar_init(&full[k], 1);
            tc05::mbar_init(&empty[k], 1);
        }
        tc05::fence_mbar_init();
        *sfail = 0;
    }
    tc05::fence_before();
    __syncthreads();
    tc05::fence_after();
    const uint32_t tmem = *tslot;

    if (warp == kSpTcThreads / 32) {
        // the MMA warp: one thread issues each stage once its operands are built
        if ((tid & 31) == 0) {
            constexpr uint32_t idesc = tc05::idesc_tf32(128, NCOL);
            for (int i = 0; i < nst; ++i) {
                const int b = i & 1;
                if (!tc05::mbar_wait_ns(&full[b], (i >> 1) & 1, kSpTcWaitNs)) { *sfail = 1; break; }
                tc05::fence_after();
                const uint32_t bh = tc05::smem_u32(tsm + b * S::OPER), bl = bh + S::B;
                const uint32_t ah = tmem + S::ACOL + 32 * b, al = ah + 16;
#pragma unroll
                for (int kk = 0; kk < kSpTcKS / 8; ++kk) {
                    const uint32_t ob = kk * 2 * S::LBO_B;
                    const uint64_t dbh = tc05::desc(bh + ob, S::LBO_B, 128), dbl = tc05::desc(bl + ob, S::LBO_B, 128);
                    tc05::mma_tf32_ta(tmem, al + 8 * kk, dbh, idesc, (i | kk) ? 1u : 0u);
                    tc05::mma_tf32_ta(tmem, ah + 8 * kk, dbl, idesc, 1u);
                    tc05::mma_tf32_ta(tmem, ah + 8 * kk, dbh, idesc, 1u);
                }
                tc05::commit(&empty[b]);
            }
        }
        __syncwarp();
    } else {
        // the builders: prologue, then per stage fetch ahead, build, publish
        for (int j = 0; j < 3; ++j)
            if (j < nst) fetch_w(j);
        cp_async_commit();
        cp_async_wait<0>();
        builders_sync();
        // the weight blocks are plan constants; the samples and the grid are
        // the previous kernels' data
        pdl_wait();
        pdl_trigger();
        if (nst > 0 && tid < 128) fetch_v(0);
        cp_async_commit();
        if (nst > 1 && tid < 128) fetch_v(1);
        cp_async_commit();
        cp_async_wait<1>();
        builders_sync();
        bool lf = false;      // this thread's bounded wait ran out
        bool failed = false;  // some builder's did (the same in every builder)
        for (int i = 0; i < nst; ++i) {
            const int b = i & 1;
            uint8_t *bH = tsm + b * S::OPER, *bL = bH + S::B;
            // the MMAs of stage i - 2 read this operand buffer
            if (i >= 2 && !tc05::mbar_wait_ns(&empty[b], ((i - 2) >> 1) & 1, kSpTcWaitNs)) lf = true;
            if (i + 3 < nst) fetch_w(i + 3);
            cp_async_commit();
            if (i + 2 < nst && tid < 128) fetch_v(i + 2);
            cp_async_commit();
            if (tid >= 128) {
                // B: the values times the density weights, a thread per
                // (column, 4 entries): a warp stores 32 consecutive 16-byte rows
                const float *sv = vslot(i), *sd = sv + kSpTcKS * NCOL;
                for (int it = tid - 128; it < NCOL * (kSpTcKS / 4); it += 128) {
                    const int n = it % NCOL, kg = it / NCOL;
                    const float4 d4 = *reinterpret_cast<const float4 *>(sd + 4 * kg);
                    uint32_t h[4], l[4];
                    tf32_split2(fmul2(make_float2(sv[(4 * kg) * NCOL + n], sv[(4 * kg + 1) * NCOL + n]),
                                      make_float2(d4.x, d4.y)), h[0], h[1], l[0], l[1]);
                    tf32_split2(fmul2(make_float2(sv[(4 * kg + 2) * NCOL + n], sv[(4 * kg + 3) * NCOL + n]),
                                      make_float2(d4.z, d4.w)), h[2], h[3], l[2], l[3]);
                    const int off = kg * S::LBO_B + (n >> 3) * 128 + (n & 7) * 16;
                    *reinterpret_cast<uint4 *>(bH + off) = make_uint4(h[0], h[1], h[2], h[3]);
                    *reinterpret_cast<uint4 *>(bL + off) = make_uint4(l[0], l[1], l[2], l[3]);
                }
            }
            // A: point m = tid % 128 (row m / 16, column m % 16; tensor-memory
            // lane m), entries 8 h .. 8 h + 7 for h = tid / 128
            {
                const int m = tid & 127, h = tid >> 7;
                const float *sw = wslot(i);
                const float4 *wr = reinterpret_cast<const float4 *>(sw + (m >> 4) * kSpTcWS);
                const float4 *wc = reinterpret_cast<const float4 *>(sw + (kSpTcPH + (m & 15)) * kSpTcWS);
                uint32_t hv[8], lv[8];
#pragma unroll
                for (int t = 0; t < 2; ++t) {
                    const float4 a = wr[2 * h + t], c = wc[2 * h + t];
                    tf32_split2(fmul2(make_float2(a.x, a.y), make_float2(c.x, c.y)), hv[4 * t], hv[4 * t + 1],
                                lv[4 * t], lv[4 * t + 1]);
                    tf32_split2(fmul2(make_float2(a.z, a.w), make_float2(c.z, c.w)), hv[4 * t + 2], hv[4 * t + 3],
                                lv[4 * t + 2], lv[4 * t + 3]);
                }
                const uint32_t ta = tmem + ((uint32_t)((warp & 3) * 32) << 16) + S::ACOL + 32 * b + 8 * h;
                tc05::st8(ta, hv);
                tc05::st8(ta + 16, lv);
                tc05::wait_st();
            }
            // publish: operands to the tensor cores, and the next stage's data
            // (all groups but the newest landed) to the builders
            tc05::fence_proxy_async();
            tc05::fence_before();
            cp_async_wait<1>();
            if (builders_sync_or(lf)) { failed = true; break; }
            if (tid == 0) mbar_arrive(&full[b]);
        }
        cp_async_wait<0>();
        if (nst > 0 && !failed && !tc05::mbar_wait_ns(&empty[(nst - 1) & 1], ((nst - 1) >> 1) & 1, kSpTcWaitNs))
            failed = true;
        if (failed) *sfail = 1;
    }
    __syncthreads();
    tc05::fence_after();
    if (*sfail) {
        if (tid == 0 && ps.err) *reinterpret_cast<volatile int *>(ps.err) = 1;   // mapped host flag
    } else if (warp < kSpTcThreads / 32) {
        constexpr int HC = NCOL / 2;
        const int m = tid & 127, half = tid >> 7, pr = m >> 4, pc = m & 15;
        const int py = py0 + pr, px = px0 + pc;
        float v[HC];
        if (nst > 0) {
            const uint32_t ta = tmem + ((uint32_t)((warp & 3) * 32) << 16) + half * HC;
            if (HC == 32) tc05::ld32(ta, *reinterpret_cast<float(*)[32]>(v));
            else if (HC == 16) tc05::ld16(ta, *reinterpret_cast<float(*)[16]>(v));
            else tc05::ld8(ta, *reinterpret_cast<float(*)[8]>(v));
            tc05::wait_ld();
        } else {
#pragma unroll
            for (int q = 0; q < HC; ++q) v[q] = 0.f;
        }
        if (py < n0 && px < n1) {
            const int cb = half * (CC / 2);               // first coil of this half
            float2 *dst = (wk.w < 0) ? grid + ((size_t)py * n1 + px) * g.nc + c0 + cb
                                     : ps.partial + ((size_t)wk.w * (kSpTcPH * kSpTcPW) + m) * g.nc + c0 + cb;
            if (v16 && ccn == CC) {
                float4 *d4 = reinterpret_cast<float4 *>(dst);
#pragma unroll
                for (int q = 0; q < CC / 4; ++q) d4[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            } else {
#pragma unroll
                for (int q = 0; q < CC / 2; ++q)
                    if (cb + q < ccn) dst[q] = make_float2(v[2 * q], v[2 * q + 1]);
            }
        }
    }
    tc05::fence_before();
    __syncthreads();
    if (warp == kSpTcThreads / 32) {
        tc05::fence_after();
        tc05::dealloc<S::TCOLS>(tmem);
    }
}

// ---------------------------------------------------------------------------
// 2-D interpolation on the 5th-generation tensor cores (interp_block 64),
// row by row over the region.  Nodes are grouped by the 8 x 16 bin of their
// footprint start, so the footprints of a bin's nodes lie in one UY x UX
// region of the grid (UY = 7 + taps, UX = 15 + taps <= 25).  The window is
// separable: for up to 128 nodes of a bin and NCOL / 2 coils
//   D_y[node][col] = sum_x wx_node(x) G[y][x][col]     (tensor cores, per region row y)
//   f[node][col]   = sum_y wy_node(y) D_y[node][col]   (CUDA cores, FP32)
// and the A operand Wx[node][x] (x padded to kIsK) is the same for every row:
// it is built once per tile, TF32-split, into tensor memory.  Per row:
//   * warps 4..7 bring the row's grid values (cp.async, two rows ahead, a
//     ring of three slots) and store them TF32-split as B, K-major in the
//     canonical no-swizzle layout, in one of two shared-memory buffers;
//   * the MMA warp issues lo.hi + hi.lo + hi.hi per K = 8 step into one of
//     two tensor-memory accumulators and commits to the row's mbarrier;
//   * warps 0..3 (thread m: node m) read the accumulator (tcgen05.ld) and
//     add wy_node(y - oy) times it to their FP32 sums in registers.
// Every handoff is an mbarrier wait bounded by the global timer; a group of
// warps whose wait ran out stops together (an OR over its named barrier), the
// CTA sets *ns.err, stores nothing and frees its tensor memory.  The nodes'
// sums go to the bin-ordered k-space, or with `user` straight into the
// caller's coil-major layout.
// ---------------------------------------------------------------------------
constexpr int kItNodes = 128;                    // nodes per tile (the MMA's M)
constexpr int kIsBH = 8, kIsBW = 16;             // footprint-start bin rows, columns
constexpr int kIsK = 32;                         // region columns padded to the MMA's K
constexpr int kIsWY = 16;                        // floats per node's y window row in shared memory

template <int NCOL, int TAPS> struct InterpSep {
    static constexpr int UY = kIsBH - 1 + TAPS, UX = kIsBW - 1 + TAPS;
    static_assert(UX <= kIsK && NCOL <= 32, "region wider than K, or too many columns");
    static constexpr int B = NCOL * kIsK * 4;                  // one of hi / lo
    static constexpr int LBO_B = (NCOL / 8) * 128;             // next 4 region columns
    static constexpr int RAW = kIsK * NCOL * 4, NR = 3;        // one region row's values
    static constexpr int SMEM = 2 * 2 * B + NR * RAW + kItNodes * kIsWY * 4 + 64;
    // tensor memory: A hi in columns 0..31, A lo 32..63, the row accumulators
    // at 64 and 96
    static constexpr int TCOLS = 128;
};

// named barriers over 128 threads (ids 1 and 2); the second form returns the
// OR of `v` over them, the same value in every participating thread
template <int ID>
__device__ __forceinline__ void group_sync() { asm volatile("bar.sync %0, 128;" ::"n"(ID) : "memory"); }
template <int ID>
__device__ __forceinline__ bool group_sync_or(bool v)
{
    uint32_t r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, %2, 128, p;\n\t"
                 "selp.u32 %0, 1, 0, q;\n\t}" : "=r"(r) : "r"((uint32_t)v), "n"(ID) : "memory");
    return r != 0;
}

template <int NCOL, int TAPS>
__global__ void __launch_bounds__(kSpTcThreads + 32, 3)
interp_sep_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ NodeSet ns,
                  const float2 *__restrict__ grid, float2 *__restrict__ ks, float2 *__restrict__ user)
{
    using I = InterpSep<NCOL, TAPS>;
    constexpr int CC = NCOL / 2;
    extern __shared__ __align__(128) uint8_t tsm[];
    uint8_t *bbuf = tsm;                                                // [buffer][hi, lo]
    uint8_t *raw0 = tsm + 4 * I::B;
    float *wys = reinterpret_cast<float *>(raw0 + I::NR * I::RAW);      // [node][kIsWY]
    uint64_t *bfull = reinterpret_cast<uint64_t *>(wys + kItNodes * kIsWY);   // B of buffer b built
    uint64_t *rdone = bfull + 2;                                         // row's MMAs done
    uint64_t *dempty = rdone + 2;                                        // accumulator read
    uint64_t *afull = dempty + 2;                                        // A in tensor memory
    uint32_t *tslot = reinterpret_cast<uint32_t *>(afull + 1);
    volatile int *sfail = reinterpret_cast<volatile int *>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int4 wk = ns.iwork[blockIdx.x];                  // {bin, first, count <= 128, 0}
    const int c0 = blockIdx.y * CC;
    const int ccn = min(CC, g.nc - c0);
    const int n0 = g.n[0], n1 = g.n[1];
    const bool v16 = (g.nc & 1) == 0;
    const int by0 = (wk.x / ns.ibx) * kIsBH, bx0 = (wk.x % ns.ibx) * kIsBW;
    const int cnt = wk.z;

    if (warp == kSpTcThreads / 32) tc05::alloc<I::TCOLS>(tslot);
    if (tid == 0) {
        for (int k = 0; k < 2; ++k) {
            tc05::mbar_init(&bfull[k], 1);
            tc05::mbar_init(&rdone[k], 1);
            tc05::mbar_init(&dempty[k], 1);
        }
        tc05::mbar_init(afull, 1);
        tc05::fence_mbar_init();
        *sfail = 0;
    }
    tc05::fence_before();
    __syncthreads();
    tc05::fence_after();
    const uint32_t tmem = *tslot;
    float acc[NCOL];
#pragma unroll
    for (int c = 0; c < NCOL; ++c) acc[c] = 0.f;
    int snode = -1;

    if (warp == kSpTcThreads / 32) {
        // the MMA warp: one thread issues each row once A, its B and its accumulator are ready
        if ((tid & 31) == 0) {
            constexpr uint32_t idesc = tc05::idesc_tf32(128, NCOL);
            bool ok = tc05::mbar_wait_ns(afull, 0, kSpTcWaitNs);
            for (int y = 0; ok && y < I::UY; ++y) {
                const int b = y & 1;
                if (!tc05::mbar_wait_ns(&bfull[b], (y >> 1) & 1, kSpTcWaitNs) ||
                    (y >= 2 && !tc05::mbar_wait_ns(&dempty[b], ((y - 2) >> 1) & 1, kSpTcWaitNs))) {
                    ok = false;
                    break;
                }
                tc05::fence_after();
                const uint32_t bh = tc05::smem_u32(bbuf + b * 2 * I::B), bl = bh + I::B;
                const uint32_t d = tmem + 64 + 32 * b;
#pragma unroll
                for (int kk = 0; kk < kIsK / 8; ++kk) {
                    const uint32_t ob = kk * 2 * I::LBO_B;
                    const uint64_t dbh = tc05::desc(bh + ob, I::LBO_B, 128), dbl = tc05::desc(bl + ob, I::LBO_B, 128);
                    tc05::mma_tf32_ta(d, tmem + 32 + 8 * kk, dbh, idesc, kk ? 1u : 0u);
                    tc05::mma_tf32_ta(d, tmem + 8 * kk, dbl, idesc, 1u);
                    tc05::mma_tf32_ta(d, tmem + 8 * kk, dbh, idesc, 1u);
                }
                tc05::commit(&rdone[b]);
            }
            if (!ok) *sfail = 1;
        }
        __syncwarp();
    } else if (tid >= kItNodes) {
        // warps 4..7: each region row's values -> B
        const int bt = tid - kItNodes;
        auto raw = [&](int y) { return reinterpret_cast<float *>(raw0 + (y % I::NR) * I::RAW); };
        // region row y: columns 0 .. kIsK - 1, zero past UX and past the coils
        auto fetch = [&](int y) {
            float *sv = raw(y);
            int gy = by0 + y;
            if (gy >= n0) gy -= n0;
            const int per = v16 ? CC / 2 : CC;
            for (int it = bt; it < kIsK * per; it += kItNodes) {
                const int x = it / per, q = it % per;
                int gx = bx0 + x;
                if (gx >= n1) gx -= n1;
                const float2 *src = grid + ((size_t)gy * n1 + (x < I::UX ? gx : 0)) * g.nc + c0;
                if (v16) {
                    float *d = sv + x * NCOL + 4 * q;
                    if (x < I::UX && 2 * q < ccn) cp_async16(d, src + 2 * q);
                    else *reinterpret_cast<float4 *>(d) = make_float4(0.f, 0.f, 0.f, 0.f);
                } else {
                    float *d = sv + x * NCOL + 2 * q;
                    if (x < I::UX && q < ccn) cp_async8(d, src + q);
                    else *reinterpret_cast<float2 *>(d) = make_float2(0.f, 0.f);
                }
            }
        };
        fetch(0);
        cp_async_commit();
        fetch(1);
        cp_async_commit();
        cp_async_wait<1>();
        group_sync<1>();
        bool lf = false, failed = false;
        for (int y = 0; y < I::UY; ++y) {
            const int b = y & 1;
            // the MMAs of row y - 2 read this B buffer
            if (y >= 2 && !tc05::mbar_wait_ns(&rdone[b], ((y - 2) >> 1) & 1, kSpTcWaitNs)) lf = true;
            if (y + 2 < I::UY) fetch(y + 2);
            cp_async_commit();
            const float *sv = raw(y);
            uint8_t *bH = bbuf + b * 2 * I::B, *bL = bH + I::B;
            // a thread per (column, 4 region columns): a warp stores 32
            // consecutive 16-byte rows
            for (int it = bt; it < NCOL * (kIsK / 4); it += kItNodes) {
                const int n = it % NCOL, kg = it / NCOL;
                uint32_t h[4], l[4];
                tf32_split2(make_float2(sv[(4 * kg) * NCOL + n], sv[(4 * kg + 1) * NCOL + n]), h[0], h[1], l[0], l[1]);
                tf32_split2(make_float2(sv[(4 * kg + 2) * NCOL + n], sv[(4 * kg + 3) * NCOL + n]), h[2], h[3], l[2], l[3]);
                const int off = kg * I::LBO_B + (n >> 3) * 128 + (n & 7) * 16;
                *reinterpret_cast<uint4 *>(bH + off) = make_uint4(h[0], h[1], h[2], h[3]);
                *reinterpret_cast<uint4 *>(bL + off) = make_uint4(l[0], l[1], l[2], l[3]);
            }
            tc05::fence_proxy_async();
            cp_async_wait<1>();
            if (group_sync_or<1>(lf)) { failed = true; break; }
            if (bt == 0) mbar_arrive(&bfull[b]);
        }
        cp_async_wait<0>();
        if (failed) *sfail = 1;
    } else {
        // warps 0..3: node m = tid
        const int m = tid;
        int oy = 0, ox = 0;
        if (m < cnt) {
            snode = ns.ilist[wk.y + m];
            const int2 u = ns.nodeU[snode];
            oy = u.x - by0;
            ox = u.y - bx0;
        }
        const float *W = ns.nodeW + (size_t)max(snode, 0) * 2 * TAPS;
        for (int t = 0; t < kIsWY; ++t) wys[m * kIsWY + t] = (snode >= 0 && t < TAPS) ? W[t] : 0.f;
        // A = Wx: region column x holds tap x - ox of the node's x window
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
#pragma unroll
        for (int k8 = 0; k8 < kIsK / 8; ++k8) {
            float w[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int tp = 8 * k8 + t - ox;
                w[t] = (snode >= 0 && tp >= 0 && tp < TAPS) ? W[TAPS + tp] : 0.f;
            }
            uint32_t hv[8], lv[8];
#pragma unroll
            for (int t = 0; t < 8; t += 2)
                tf32_split2(make_float2(w[t], w[t + 1]), hv[t], hv[t + 1], lv[t], lv[t + 1]);
            tc05::st8(tmem + lane_base + 8 * k8, hv);
            tc05::st8(tmem + lane_base + 32 + 8 * k8, lv);
        }
        tc05::wait_st();
        tc05::fence_before();
        group_sync<2>();
        if (m == 0) mbar_arrive(afull);
        bool lf = false, failed = false;
        for (int y = 0; y < I::UY; ++y) {
            const int b = y & 1;
            if (!tc05::mbar_wait_ns(&rdone[b], (y >> 1) & 1, kSpTcWaitNs)) lf = true;
            tc05::fence_after();
            const int t = y - oy;
            const float wv = (t >= 0 && t < TAPS) ? wys[m * kIsWY + t] : 0.f;
            const float2 w2 = make_float2(wv, wv);
            // 16 accumulator columns at a time (fewer live registers)
#pragma unroll
            for (int h = 0; h < NCOL / 16; ++h) {
                float v[16];
                tc05::ld16(tmem + lane_base + 64 + 32 * b + 16 * h, v);
                tc05::wait_ld();
#pragma unroll
                for (int c = 0; c < 16; c += 2) {
                    const float2 r = ffma2(w2, make_float2(v[c], v[c + 1]),
                                           make_float2(acc[16 * h + c], acc[16 * h + c + 1]));
                    acc[16 * h + c] = r.x;
                    acc[16 * h + c + 1] = r.y;
                }
            }
            tc05::fence_before();
            if (group_sync_or<2>(lf)) { failed = true; break; }
            if (m == 0) mbar_arrive(&dempty[b]);
        }
        if (failed) *sfail = 1;
    }
    __syncthreads();
    tc05::fence_after();
    if (*sfail) {
        if (tid == 0 && ns.err) *reinterpret_cast<volatile int *>(ns.err) = 1;   // mapped host flag
    } else if (tid < kItNodes && tid < cnt && snode >= 0) {
        if (user) {
            const int j = ns.perm[snode];
#pragma unroll
            for (int q = 0; q < CC; ++q)
                if (q < ccn) user[(size_t)(c0 + q) * ns.M + j] = make_float2(acc[2 * q], acc[2 * q + 1]);
        } else {
            float2 *dst = ks + (size_t)snode * g.nc + c0;
            if (v16 && ccn == CC) {
                float4 *d4 = reinterpret_cast<float4 *>(dst);
#pragma unroll
                for (int q = 0; q < CC / 2; ++q)
                    d4[q] = make_float4(acc[4 * q], acc[4 * q + 1], acc[4 * q + 2], acc[4 * q + 3]);
            } else {
#pragma unroll
                for (int q = 0; q < CC; ++q)
                    if (q < ccn) dst[q] = make_float2(acc[2 * q], acc[2 * q + 1]);
            }
        }
    }
    tc05::fence_before();
    __syncthreads();
    if (warp == kSpTcThreads / 32) {
        tc05::fence_after();
        tc05::dealloc<I::TCOLS>(tmem);
    }
}

template <int TAPS>
static cgs_status launch_interp_tc_taps(const GridGeom &g, const NodeSet &ns, const float2 *grid, float2 *ks,
                                        float2 *user, cudaStream_t st)
{
    const int ncol = g.nc > 8 ? 32 : 16;
    dim3 grd(ns.niwork, (g.nc + ncol / 2 - 1) / (ncol / 2));
#define CGS_ITC(NCV)                                                                                        \
    do {                                                                                                    \
        using IT = InterpSep<NCV, TAPS>;                                                                    \
        CGS_CUDA(cudaFuncSetAttribute(interp_sep_kernel<NCV, TAPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                      IT::SMEM));                                                           \
        interp_sep_kernel<NCV, TAPS><<<grd, kSpTcThreads + 32, IT::SMEM, st>>>(g, ns, grid, ks, user);      \
    } while (0)
    if (ncol == 32) CGS_ITC(32);
    else CGS_ITC(16);
#undef CGS_ITC
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

// ---------------------------------------------------------------------------
// 2-D interpolation on the tensor cores.  Nodes are grouped by the 4 x 4 bin
// of their footprint start, so the footprints of a bin's nodes lie in one
// U x U region of the grid (U = 3 + taps).  A warp takes up to 16 nodes of
// one bin and computes with mma.m16n8k8 over the region's points:
//   f[16 nodes][8 NT cols] = W[16 nodes][U^2 points] G[U^2 points][8 NT cols]
// W[j][p] = wy_j[dy] wx_j[dx] for p inside node j's footprint, else 0; G is
// read from the grid through the read-only path (8 consecutive floats per
// column group, one 32-byte sector), warps of neighbouring bins sharing it in
// L1.  Both operands are split into TF32 value and remainder and three
// products are accumulated in FP32, as in the spreading.
// ---------------------------------------------------------------------------
template <int NT, int TAPS> struct InterpMma {
    static constexpr int U = 3 + TAPS, KP = (U * U + 7) / 8 * 8;
    // zero-padded window rows: entry 3 + i is tap i, so a region coordinate
    // minus the footprint offset (in [-3, U]) indexes them without checks
    static constexpr int PL = U + 4;
    static constexpr size_t warp_bytes = (size_t)kInterpGroup * 2 * PL * sizeof(float) + (size_t)KP * sizeof(int);
    static constexpr size_t smem = 8 * warp_bytes;
};

template <int NT, int TAPS>
__global__ void __launch_bounds__(256, 3)
interp_mma_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ NodeSet ns,
                  const float2 *__restrict__ grid, float2 *__restrict__ ks, float2 *__restrict__ user)
{
    using I = InterpMma<NT, TAPS>;
    constexpr int U = I::U, KP = I::KP, CC = 4 * NT, PL = I::PL;
    extern __shared__ float4 smem4[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wi = blockIdx.x * 8 + warp;
    if (wi >= ns.niwork) return;
    float *wpad = reinterpret_cast<float *>(reinterpret_cast<char *>(smem4) + warp * I::warp_bytes);  // [16][2][PL]
    int *spt = reinterpret_cast<int *>(wpad + kInterpGroup * 2 * PL);                                // [KP] grid points
    // the work item's padded window rows ([16][wy, wx][PL]) and node offsets,
    // precomputed once per trajectory (interp_windows_kernel), come in by
    // cp.async without waiting on the node list
    {
        const float *src = ns.iwin + (size_t)wi * kInterpGroup * 2 * PL;
        for (int q = lane; q < kInterpGroup * 2 * PL / 4; q += 32) cp_async16(wpad + 4 * q, src + 4 * q);
        cp_async_commit();
    }
    int s_l = -1, oy_l = 0, ox_l = 0;
    if (lane < kInterpGroup) {
        const int4 mt = ns.imeta[(size_t)wi * kInterpGroup + lane];
        s_l = mt.x; oy_l = mt.y; ox_l = mt.z;
    }
    const int4 wk = ns.iwork[wi];                           // {bin, first, count <= 16, 0}
    const int c0 = blockIdx.y * CC;
    const int ccn = min(CC, g.nc - c0);
    const int n0 = g.n[0], n1 = g.n[1];
    const int by0 = (wk.x / ns.ibx) * 4, bx0 = (wk.x % ns.ibx) * 4;
    // region points (rows and columns wrap once: n0, n1 >= U); -1 past the region
    for (int q = lane; q < KP; q += 32) {
        int pt = -1;
        if (q < U * U) {
            int gy = by0 + q / U, gx = bx0 + q % U;
            if (gy >= n0) gy -= n0;
            if (gx >= n1) gx -= n1;
            pt = gy * n1 + gx;
        }
        spt[q] = pt;
    }
    cp_async_wait<0>();
    __syncwarp();
    // the window blocks and work lists are plan constants; the grid is the
    // previous kernel's output
    pdl_wait();
    pdl_trigger();
    const int gq = lane >> 2, tq = lane & 3;
    const int na = gq, nb = gq + 8;
    const int oya = __shfl_sync(0xffffffffu, oy_l, na), oxa = __shfl_sync(0xffffffffu, ox_l, na);
    const int oyb = __shfl_sync(0xffffffffu, oy_l, nb), oxb = __shfl_sync(0xffffffffu, ox_l, nb);
    // row pointers shifted so that [qy] / [qx] is tap qy - oy / qx - ox (zero outside)
    const float *Wya = wpad + na * 2 * PL + 3 - oya, *Wxa = wpad + na * 2 * PL + PL + 3 - oxa;
    const float *Wyb = wpad + nb * 2 * PL + 3 - oyb, *Wxb = wpad + nb * 2 * PL + PL + 3 - oxb;
    const float *gf = reinterpret_cast<const float *>(grid) + (size_t)c0 * 2 + gq;
    const size_t rs = (size_t)g.nc * 2;                     // floats per grid point
    float acc[NT][4];
#pragma unroll
    for (int t = 0; t < NT; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
    const bool full = (ccn == CC);
    // region coordinates of the thread's two points q0 = k0 + tq and q1 = q0 + 4
    int qy0 = tq / U, qx0 = tq % U, qy1 = (tq + 4) / U, qx1 = (tq + 4) % U;
#pragma unroll 1
    for (int k0 = 0; k0 < KP; k0 += 8) {
        const int p0 = spt[k0 + tq], p1 = spt[k0 + tq + 4];
        float b0v[NT], b1v[NT];
        const float *g0 = gf + (size_t)max(p0, 0) * rs, *g1 = gf + (size_t)max(p1, 0) * rs;
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            const bool ok = full || (8 * t + gq < 2 * ccn);
            b0v[t] = (p0 >= 0 && ok) ? __ldg(g0 + 8 * t) : 0.f;
            b1v[t] = (p1 >= 0 && ok) ? __ldg(g1 + 8 * t) : 0.f;
        }
        uint32_t ah[4], al[4];
        tf32_split(Wya[qy0] * Wxa[qx0], ah[0], al[0]);
        tf32_split(Wyb[qy0] * Wxb[qx0], ah[1], al[1]);
        tf32_split(Wya[qy1] * Wxa[qx1], ah[2], al[2]);
        tf32_split(Wyb[qy1] * Wxb[qx1], ah[3], al[3]);
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            uint32_t bh0, bl0, bh1, bl1;
            tf32_split2(make_float2(b0v[t], b1v[t]), bh0, bh1, bl0, bl1);
            mma_tf32(acc[t], al, bh0, bh1);
            mma_tf32(acc[t], ah, bl0, bl1);
            mma_tf32(acc[t], ah, bh0, bh1);
        }
        qx0 += 8; while (qx0 >= U) { qx0 -= U; ++qy0; }
        qx1 += 8; while (qx1 >= U) { qx1 -= U; ++qy1; }
    }
    // rows gq and gq + 8: nodes na and nb, columns 2 tq, 2 tq + 1 of each n-tile.
    // With `user`, straight into the caller's layout (coil-major, trajectory
    // order): a bin's nodes are mostly runs of consecutive trajectory samples,
    // so each coil row's stores stay close to sector-dense.
    const int sa = __shfl_sync(0xffffffffu, s_l, na), sb = __shfl_sync(0xffffffffu, s_l, nb);
    if (user) {
        const int ja = sa >= 0 ? ns.perm[sa] : 0, jb = sb >= 0 ? ns.perm[sb] : 0;
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            const int c = 4 * t + tq;
            if (c < ccn) {
                float2 *row = user + (size_t)(c0 + c) * ns.M;
                if (sa >= 0) row[ja] = make_float2(acc[t][0], acc[t][1]);
                if (sb >= 0) row[jb] = make_float2(acc[t][2], acc[t][3]);
            }
        }
        return;
    }
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        const int c = 4 * t + tq;
        if (c < ccn) {
            if (sa >= 0) ks[(size_t)sa * g.nc + c0 + c] = make_float2(acc[t][0], acc[t][1]);
            if (sb >= 0) ks[(size_t)sb * g.nc + c0 + c] = make_float2(acc[t][2], acc[t][3]);
        }
    }
}

// one warp per interpolation work item: the padded window rows and footprint
// offsets that interp_mma_kernel would build itself, in its shared-memory
// layout ([16 nodes][wy, wx][PL]) and {node, oy, ox, 0} per node
template <int TAPS>
__global__ void interp_windows_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ NodeSet ns,
                                      float *__restrict__ iwin, int4 *__restrict__ imeta)
{
    constexpr int PL = InterpMma<1, TAPS>::PL, WS = 2 * TAPS;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wi = blockIdx.x * 8 + warp;
    if (wi >= ns.niwork || lane >= kInterpGroup) return;
    const int4 wk = ns.iwork[wi];
    const int by0 = (wk.x / ns.ibx) * 4, bx0 = (wk.x % ns.ibx) * 4;
    float *wy = iwin + ((size_t)wi * kInterpGroup + lane) * 2 * PL, *wx = wy + PL;
    int sv = -1, oy = 0, ox = 0;
    if (lane < wk.z) {
        sv = ns.ilist[wk.y + lane];
        const int2 u = ns.nodeU[sv];
        oy = u.x - by0;
        ox = u.y - bx0;
        const float *W = ns.nodeW + (size_t)sv * WS;
        for (int i = 0; i < PL; ++i) {
            const int t = i - 3;
            wy[i] = (t >= 0 && t < TAPS) ? W[t] : 0.f;
            wx[i] = (t >= 0 && t < TAPS) ? W[TAPS + t] : 0.f;
        }
    } else {
        for (int i = 0; i < PL; ++i) wy[i] = wx[i] = 0.f;
    }
    imeta[(size_t)wi * kInterpGroup + lane] = make_int4(sv, oy, ox, 0);
}

template <int NT, int TAPS>
static cgs_status launch_interp_mma_t(const GridGeom &g, const NodeSet &ns, const float2 *grid, float2 *ks,
                                      float2 *user, cudaStream_t st)
{
    using I = InterpMma<NT, TAPS>;
    CGS_CUDA(cudaFuncSetAttribute(interp_mma_kernel<NT, TAPS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)I::smem));
    dim3 grd((ns.niwork + 7) / 8, (g.nc + 4 * NT - 1) / (4 * NT));
    CGS_CUDA(launch_pdl(interp_mma_kernel<NT, TAPS>, grd, dim3(256), I::smem, st, g, ns, grid, ks, user));
    return CGS_OK;
}

template <int TAPS>
static cgs_status launch_interp_mma_taps(const GridGeom &g, const NodeSet &ns, const float2 *grid, float2 *ks,
                                         float2 *user, cudaStream_t st)
{
    switch (std::min(8, (2 * g.nc + 7) / 8)) {
        case 8: return launch_interp_mma_t<8, TAPS>(g, ns, grid, ks, user, st);
        case 7: return launch_interp_mma_t<7, TAPS>(g, ns, grid, ks, user, st);
        case 6: return launch_interp_mma_t<6, TAPS>(g, ns, grid, ks, user, st);
        case 5: return launch_interp_mma_t<5, TAPS>(g, ns, grid, ks, user, st);
        case 4: return launch_interp_mma_t<4, TAPS>(g, ns, grid, ks, user, st);
        case 3: return launch_interp_mma_t<3, TAPS>(g, ns, grid, ks, user, st);
        case 2: return launch_interp_mma_t<2, TAPS>(g, ns, grid, ks, user, st);
        default: return launch_interp_mma_t<1, TAPS>(g, ns, grid, ks, user, st);
    }
}

// sum the partial slots of split patches in slot order and store them; with
// an even coil count two coils per thread (16-byte loads and stores)
__global__ void patch_reduce2_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ PatchSet ps,
                                     float2 *__restrict__ grid)
{
    pdl_wait();
    pdl_trigger();
    const int nh = g.nc / 2, npt = ps.ph * ps.pw;
    const int64_t total = (int64_t)ps.nmulti * npt * nh;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int c = 2 * (int)(e % nh);
        const int pt = (int)((e / nh) % npt);
        const int4 mu = ps.multi[e / ((int64_t)npt * nh)];
        const int py = (mu.x / ps.npx) * ps.ph + pt / ps.pw;
        const int px = (mu.x % ps.npx) * ps.pw + pt % ps.pw;
        if (py >= g.n[0] || px >= g.n[1]) continue;
        float4 s4 = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int k = 0; k < mu.z; ++k) {
            const float4 v = *reinterpret_cast<const float4 *>(&ps.partial[((size_t)(mu.y + k) * npt + pt) * g.nc + c]);
            s4.x += v.x; s4.y += v.y; s4.z += v.z; s4.w += v.w;
        }
        *reinterpret_cast<float4 *>(&grid[((size_t)py * g.n[1] + px) * g.nc + c]) = s4;
    }
}

__global__ void patch_reduce_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ PatchSet ps,
                                    float2 *__restrict__ grid)
{
    const int nc = g.nc, npt = ps.ph * ps.pw;
    const int64_t total = (int64_t)ps.nmulti * npt * nc;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(e % nc);
        const int pt = (int)((e / nc) % npt);
        const int4 mu = ps.multi[e / ((int64_t)npt * nc)];
        const int py = (mu.x / ps.npx) * ps.ph + pt / ps.pw;
        const int px = (mu.x % ps.npx) * ps.pw + pt % ps.pw;
        if (py >= g.n[0] || px >= g.n[1]) continue;
        float sx = 0.f, sy = 0.f;
        for (int k = 0; k < mu.z; ++k) {
            const float2 v = ps.partial[((size_t)(mu.y + k) * npt + pt) * nc + c];
            sx += v.x; sy += v.y;
        }
        grid[((size_t)py * g.n[1] + px) * nc + c] = make_float2(sx, sy);
    }
}

// ---------------------------------------------------------------------------
// 2-D interpolation with the coil index on the lanes.  A CTA stages the padded
// (T+2m+1)^2 tile of CC coils ([point][coil], coil innermost); a group of
// CC / CPL lanes serves one node, each lane CPL consecutive coils, so every
// tap is one read of CC consecutive complex values (for CC = 16, CPL = 2: one
// full 128-byte bank row per node, conflict-free), and the node's 2 x TAPS
// weights (precomputed once per trajectory) sit in registers.  The complex
// multiply-adds are paired FP32 FMAs (the rounding of two fmaf).
// ---------------------------------------------------------------------------
template <int TAPS, int CC, int CPL>
__global__ void __launch_bounds__(256)
interp2_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ NodeSet ns,
               const int2 *__restrict__ nodeU, const float *__restrict__ nodeW,
               const float2 *__restrict__ grid, float2 *__restrict__ ks)
{
    static_assert(CC % CPL == 0 && 32 % (CC / CPL) == 0, "coil lanes must tile the warp");
    extern __shared__ float4 smem4[];
    float2 *tile = reinterpret_cast<float2 *>(smem4);
    const int E = g.T + TAPS - 1;
    const int4 wk = ns.work[blockIdx.x];
    const int c0 = blockIdx.y * CC;
    const int ccn = min(CC, g.nc - c0);
    const int o0 = (wk.x / g.nt[1]) * g.T, o1 = (wk.x % g.nt[1]) * g.T;
    constexpr int kUnroll = 8;  // independent loads in flight per thread
    const int tot = E * E * CC;
    for (int e0 = threadIdx.x; e0 < tot; e0 += 256 * kUnroll) {
        float2 v[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const int e = e0 + u * 256;
            const int c = e % CC, pt = e / CC;
            const int ly = pt / E, lx = pt % E;
            v[u] = make_float2(0.f, 0.f);
            if (e < tot && c < ccn)
                v[u] = grid[((size_t)wrapi(o0 + ly, g.n[0]) * g.n[1] + wrapi(o1 + lx, g.n[1])) * g.nc + c0 + c];
        }
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
            if (e0 + u * 256 < tot) tile[e0 + u * 256] = v[u];
    }
    __syncthreads();
    constexpr int LPN = CC / CPL;          // lanes per node
    constexpr int NPW = 32 / LPN;          // nodes served by one warp at a time
    const int lane = threadIdx.x & 31, cl = lane % LPN, slot = lane / LPN;
    const int warp = threadIdx.x >> 5;
    for (int i = warp * NPW + slot; i < wk.z; i += 8 * NPW) {
        const int64_t s = (int64_t)wk.y + i;
        const int2 u = nodeU[s];
        const int y0 = u.x - o0, x0 = u.y - o1;
        const float *W = nodeW + s * 2 * TAPS;
        float w0[TAPS], w1[TAPS];
#pragma unroll
        for (int q = 0; q < TAPS; ++q) { w0[q] = W[q]; w1[q] = W[TAPS + q]; }
        float2 acc[CPL];
#pragma unroll
        for (int k = 0; k < CPL; ++k) acc[k] = make_float2(0.f, 0.f);
#pragma unroll
        for (int a = 0; a < TAPS; ++a) {
            const float2 *row = tile + ((y0 + a) * E + x0) * CC + cl * CPL;
            float2 r[CPL];
#pragma unroll
            for (int k = 0; k < CPL; ++k) r[k] = make_float2(0.f, 0.f);
#pragma unroll
            for (int b = 0; b < TAPS; ++b) {
                const float2 wb = make_float2(w1[b], w1[b]);
                if constexpr (CPL == 2) {
                    const float4 q = *reinterpret_cast<const float4 *>(row + b * CC);
                    r[0] = ffma2(wb, make_float2(q.x, q.y), r[0]);
                    r[1] = ffma2(wb, make_float2(q.z, q.w), r[1]);
                } else {
#pragma unroll
                    for (int k = 0; k < CPL; ++k) r[k] = ffma2(wb, row[b * CC + k], r[k]);
                }
            }
            const float2 wa = make_float2(w0[a], w0[a]);
#pragma unroll
            for (int k = 0; k < CPL; ++k) acc[k] = ffma2(wa, r[k], acc[k]);
        }
#pragma unroll
        for (int k = 0; k < CPL; ++k)
            if (cl * CPL + k < ccn) ks[s * g.nc + c0 + cl * CPL + k] = acc[k];
    }
}

// ---------------------------------------------------------------------------
// 3-D gridding on the tensor cores (taps <= 10, every grid side >= 3 + taps).
//
// Node tables (once per trajectory): the wrapped footprint start of every
// node and its 3 x taps window weights, zero padded to kW3 floats (128 B, so
// one node's row is eight 16-byte copies).
//
// Spreading is output-stationary over 4 x 4 x 4 patches of grid points.  A
// warp owns one patch as four m-tiles (its z-planes, 16 (y, x) points each)
// and NT n-tiles of 8 float columns (4 NT coils), and walks the list of nodes
// whose footprint covers the patch in batches of 8 entries, each batch one
// mma.m16n8k8 k-step per (m-tile, n-tile):
//   D[plane z][16 points][8 NT cols] += W[16 points][8 entries] V[8 entries][8 NT cols],
//   W = wz(entry, z) wy(entry, y) (wx(entry, x) density(entry)).
// Entries (values, window rows, starts, density weights) are staged by
// cp.async, double buffered, as in the 2-D kernel; the B fragments and the
// (y, x) weight products are formed once per batch and shared by the four
// planes.  Operands are split into TF32 value and remainder, three products
// accumulate in FP32.  Crowded patches are split into partial slots that
// patch_reduce3_kernel adds in slot order: no atomics, reproducible results.
//
// Interpolation groups up to 16 nodes of one 4 x 4 x 4 footprint-start bin
// per warp; their footprints lie in one U^3 region (U = 3 + taps) and
//   f[16 nodes][8 NT cols] = W[16 nodes][U^3 points] G[U^3 points][8 NT cols]
// runs over the region 8 points per k-step, W = wz wy wx from zero-padded
// window rows (no bounds checks), G read through L1 (8 consecutive floats per
// column group, one 32-byte sector).
// ---------------------------------------------------------------------------
__global__ void node_weights3_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ NodeSet ns,
                                     int4 *__restrict__ nodeU3, float *__restrict__ nodeW)
{
    const int taps = 2 * g.m + 2;
    const float mf = (float)g.m;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < ns.M; s += (int64_t)gridDim.x * blockDim.x) {
        float frac[3]; int c[3];
        node_read<3>(ns.nodes, s, frac, c);
        nodeU3[s] = make_int4(wrapi(c[0] - g.m, g.n[0]), wrapi(c[1] - g.m, g.n[1]), wrapi(c[2] - g.m, g.n[2]), 0);
        float *w = nodeW + s * kW3;
        for (int i = 0; i < kW3; ++i) {
            const int t = i / taps, q = i % taps;
            w[i] = (t < 3) ? kb_phi(frac[t] + mf - (float)q, mf, g.b[t]) : 0.f;
        }
    }
}

template <int NT> struct Spread3Mma {
    static constexpr int R = spread_mma_row(NT);
    // one staging buffer: values, window rows, footprint starts, density weights (a multiple of 16 B)
    static constexpr size_t buf_bytes =
        (size_t)kSpreadBatch * (R * sizeof(float) + kW3 * sizeof(float) + sizeof(int4) + sizeof(float));
    // per warp: two buffers and the batch's patch weights (4 wz, 4 wy, 4 wx per entry)
    static constexpr size_t warp_bytes = 2 * buf_bytes + (size_t)kSpreadBatch * 12 * sizeof(float);
};

template <int NT, int TAPS>
__global__ void __launch_bounds__(256, 2)
spread3_mma_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ PatchSet ps,
                   const float2 *__restrict__ ks, const float *__restrict__ dens, int weighted,
                   float2 *__restrict__ grid)
{
    using S = Spread3Mma<NT>;
    constexpr int R = S::R, CC = 4 * NT, CH = 2 * NT;
    extern __shared__ float4 smem4[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wi = blockIdx.x * 8 + warp;
    if (wi >= ps.nwork) return;
    char *wbase = reinterpret_cast<char *>(smem4) + (size_t)warp * S::warp_bytes;
    float *swt = reinterpret_cast<float *>(wbase + 2 * S::buf_bytes);   // [entry][wz 0..3 | wy 0..3 | wx 0..3]
    const int c0 = blockIdx.y * CC;
    const int ccn = min(CC, g.nc - c0);
    const bool v16 = ((g.nc & 1) == 0);
    const int4 wk = ps.work[wi];
    const int n0 = g.n[0], n1 = g.n[1], n2 = g.n[2];
    const int gq = lane >> 2, tq = lane & 3;
    const int yr = gq >> 2, xc = gq & 3;
    const int pz0 = (wk.x / (ps.npx * ps.npy)) * 4, py0 = ((wk.x / ps.npx) % ps.npy) * 4, px0 = (wk.x % ps.npx) * 4;
    float acc[4][NT][4];
#pragma unroll
    for (int mt = 0; mt < 4; ++mt)
#pragma unroll
        for (int t = 0; t < NT; ++t) acc[mt][t][0] = acc[mt][t][1] = acc[mt][t][2] = acc[mt][t][3] = 0.f;
    if (wk.z > 0) {
        {   // zero both buffers once: padding columns and rows past a short batch stay finite
            float4 *z = reinterpret_cast<float4 *>(wbase);
            const int n16 = (int)(2 * S::buf_bytes / 16);
            for (int i = lane; i < n16; i += 32) z[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            __syncwarp();
        }
        auto buffers = [&](int buf, float *&sv, float *&sw, int4 *&su, float *&sd) {
            char *b = wbase + (size_t)buf * S::buf_bytes;
            sv = reinterpret_cast<float *>(b);
            sw = sv + kSpreadBatch * R;
            su = reinterpret_cast<int4 *>(sw + kSpreadBatch * kW3);
            sd = reinterpret_cast<float *>(su + kSpreadBatch);
        };
        auto issue = [&](int e0, int cnt, int buf) {
            float *sv, *sw, *sd; int4 *su;
            buffers(buf, sv, sw, su, sd);
            const int s_l = (lane < cnt) ? ps.entries[e0 + lane] : 0;
            if (lane < cnt) {
                cp_async16(&su[lane], &ps.nodeU3[s_l]);
                if (weighted) cp_async4(&sd[lane], &dens[s_l]);
                else sd[lane] = 1.f;
            }
            // window rows: 8 entries x 8 chunks of 16 bytes
#pragma unroll
            for (int i = 0; i < (kSpreadBatch * (kW3 / 4)) / 32; ++i) {
                const int ch = lane + 32 * i;
                const int e = ch / (kW3 / 4), q = ch % (kW3 / 4);
                const int s = __shfl_sync(0xffffffffu, s_l, e);
                if (e < cnt) cp_async16(sw + e * kW3 + 4 * q, ps.nodeW + (size_t)s * kW3 + 4 * q);
            }
            if (v16) {
#pragma unroll
                for (int i = 0; i < (kSpreadBatch * CH + 31) / 32; ++i) {
                    const int ch = lane + 32 * i;
                    const int e = ch / CH, c = 2 * (ch % CH);
                    const int s = __shfl_sync(0xffffffffu, s_l, e & (kSpreadBatch - 1));
                    if (ch < kSpreadBatch * CH && e < cnt && c < ccn) {
                        const float2 *v = ks + (size_t)s * g.nc + c0 + c;
                        float2 *d = reinterpret_cast<float2 *>(sv + e * R) + c;
                        if (c + 1 < ccn) cp_async16(d, v);
                        else cp_async8(d, v);
                    }
                }
            } else {
                for (int j = 0; j < cnt; ++j) {
                    const int s = __shfl_sync(0xffffffffu, s_l, j);
                    const float2 *v = ks + (size_t)s * g.nc + c0;
                    float2 *dv = reinterpret_cast<float2 *>(sv + j * R);
                    for (int c = lane; c < ccn; c += 32) cp_async8(dv + c, v + c);
                }
            }
            cp_async_commit();
        };
        const int end = wk.y + wk.z;
        int e0 = wk.y, cnt = min(kSpreadBatch, end - e0), buf = 0;
        issue(e0, cnt, 0);
        while (true) {
            const int e1 = e0 + cnt;
            const int cnt1 = min(kSpreadBatch, end - e1);
            if (cnt1 > 0) { issue(e1, cnt1, buf ^ 1); cp_async_wait<1>(); }
            else cp_async_wait<0>();
            __syncwarp();
            float *sv, *sw, *sd; int4 *su;
            buffers(buf, sv, sw, su, sd);
            // the batch's patch weights: entry e, axis a (z, y, x), offset r in the patch; zero past cnt
#pragma unroll
            for (int i = 0; i < (kSpreadBatch * 12) / 32; ++i) {
                const int idx = lane + 32 * i;
                const int e = idx / 12, a = (idx % 12) >> 2, r = idx & 3;
                float w = 0.f;
                if (e < cnt) {
                    const int4 u = su[e];
                    const int pa = (a == 0 ? pz0 : (a == 1 ? py0 : px0)) + r;
                    const int na = a == 0 ? n0 : (a == 1 ? n1 : n2);
                    if (pa < na) {
                        int q = pa - (a == 0 ? u.x : (a == 1 ? u.y : u.z));
                        if (q < 0) q += na;
                        w = q < TAPS ? sw[e * kW3 + a * TAPS + q] : 0.f;
                        if (a == 2) w *= sd[e];
                    }
                }
                swt[idx] = w;
            }
            __syncwarp();
            const float *we0 = swt + tq * 12, *we1 = swt + (tq + 4) * 12;
            // rows gq and gq + 8 of an m-tile: points (y, x) = (yr, xc) and (yr + 2, xc)
            const float wyx00 = we0[4 + yr] * we0[8 + xc], wyx01 = we0[6 + yr] * we0[8 + xc];
            const float wyx10 = we1[4 + yr] * we1[8 + xc], wyx11 = we1[6 + yr] * we1[8 + xc];
            uint32_t bh0[NT], bl0[NT], bh1[NT], bl1[NT];
            const float *r0 = sv + tq * R + gq, *r1 = sv + (tq + 4) * R + gq;
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                tf32_split2(make_float2(r0[8 * t], r1[8 * t]), bh0[t], bh1[t], bl0[t], bl1[t]);
            }
#pragma unroll
            for (int mt = 0; mt < 4; ++mt) {
                uint32_t ah[4], al[4];
                const float z0 = we0[mt], z1 = we1[mt];
                tf32_split(z0 * wyx00, ah[0], al[0]);
                tf32_split(z0 * wyx01, ah[1], al[1]);
                tf32_split(z1 * wyx10, ah[2], al[2]);
                tf32_split(z1 * wyx11, ah[3], al[3]);
#pragma unroll
                for (int t = 0; t < NT; ++t) {
                    mma_tf32(acc[mt][t], al, bh0[t], bh1[t]);
                    mma_tf32(acc[mt][t], ah, bl0[t], bl1[t]);
                    mma_tf32(acc[mt][t], ah, bh0[t], bh1[t]);
                }
            }
            __syncwarp();
            if (cnt1 <= 0) break;
            e0 = e1; cnt = cnt1; buf ^= 1;
        }
    }
    const int xx = px0 + xc;
#pragma unroll
    for (int mt = 0; mt < 4; ++mt)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int zz = pz0 + mt, yy = py0 + yr + 2 * h;
            if (zz >= n0 || yy >= n1 || xx >= n2) continue;
            const int ppt = 16 * mt + gq + 8 * h;            // point index within the patch (z, y, x row-major)
            float2 *dst = (wk.w < 0) ? grid + (((size_t)zz * n1 + yy) * n2 + xx) * g.nc + c0
                                     : ps.partial + ((size_t)wk.w * 64 + ppt) * g.nc + c0;
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                const int c = 4 * t + tq;
                if (c < ccn) dst[c] = make_float2(acc[mt][t][2 * h], acc[mt][t][2 * h + 1]);
            }
        }
}

// sum the partial slots of split 3-D patches in slot order and store them
__global__ void patch_reduce3_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ PatchSet ps,
                                     float2 *__restrict__ grid)
{
    const int nc = g.nc;
    const int64_t total = (int64_t)ps.nmulti * 64 * nc;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(e % nc);
        const int pt = (int)((e / nc) % 64);
        const int4 mu = ps.multi[e / ((int64_t)64 * nc)];
        const int z = (mu.x / (ps.npx * ps.npy)) * 4 + pt / 16;
        const int y = ((mu.x / ps.npx) % ps.npy) * 4 + (pt / 4) % 4;
        const int x = (mu.x % ps.npx) * 4 + pt % 4;
        if (z >= g.n[0] || y >= g.n[1] || x >= g.n[2]) continue;
        float sx = 0.f, sy = 0.f;
        for (int k = 0; k < mu.z; ++k) {
            const float2 v = ps.partial[((size_t)(mu.y + k) * 64 + pt) * nc + c];
            sx += v.x; sy += v.y;
        }
        grid[(((size_t)z * g.n[1] + y) * g.n[2] + x) * nc + c] = make_float2(sx, sy);
    }
}

template <int NT, int TAPS> struct Interp3Mma {
    static constexpr int U = 3 + TAPS, UU = U * U, KP = (U * U * U + 7) / 8 * 8, NK = KP / 8;
    // zero-padded window rows per axis: entry 3 + i is tap i, so a region
    // coordinate in [0, U] minus the node's offset (0..3) indexes them unchecked
    static constexpr int PL = U + 4;
    static constexpr int R = spread_mma_row(NT);   // staged point row (floats): conflict-free B reads
    static constexpr int S = 4;                    // cp.async stages of 8 points each
    static constexpr size_t stage_bytes = (size_t)8 * R * sizeof(float);
    static constexpr size_t warp_bytes =
        (S * stage_bytes + (size_t)kInterpGroup * 3 * PL * sizeof(float) + (size_t)(UU + U) * sizeof(int) + 15) / 16 * 16;
    static constexpr size_t smem = 8 * warp_bytes;
};

template <int NT, int TAPS>
__global__ void __launch_bounds__(256, 2)
interp3_mma_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ NodeSet ns,
                   const float2 *__restrict__ grid, float2 *__restrict__ ks)
{
    using I = Interp3Mma<NT, TAPS>;
    constexpr int U = I::U, UU = I::UU, NK = I::NK, CC = 4 * NT, PL = I::PL, R = I::R, S = I::S;
    constexpr int CH = 2 * NT, NCH = 8 * CH, NI = (NCH + 31) / 32;   // 16-byte chunks per point / per k-step
    extern __shared__ float4 smem4[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wi = blockIdx.x * 8 + warp;
    if (wi >= ns.niwork) return;
    char *wbase = reinterpret_cast<char *>(smem4) + warp * I::warp_bytes;
    float *sbase = reinterpret_cast<float *>(wbase);                          // [S][8 points][R]
    float *wpad = reinterpret_cast<float *>(wbase + S * I::stage_bytes);     // [16][3][PL]
    int *roff = reinterpret_cast<int *>(wpad + kInterpGroup * 3 * PL);       // [U z][U y] first point of each region row
    int *xoff = roff + UU;                                                    // [U] wrapped x
    const int4 wk = ns.iwork[wi];                          // {bin, first, count <= 16, 0}
    const int c0 = blockIdx.y * CC;
    const int ccn = min(CC, g.nc - c0);
    const bool v16 = ((g.nc & 1) == 0);
    const int n0 = g.n[0], n1 = g.n[1], n2 = g.n[2];
    const int z0 = (wk.x / (ns.ibx * ns.iby)) * 4, y0 = ((wk.x / ns.ibx) % ns.iby) * 4, x0 = (wk.x % ns.ibx) * 4;
    const int cnt = wk.z;
    {   // zero the stages once: columns past the coils and points past the region stay finite
        float4 *z = reinterpret_cast<float4 *>(sbase);
        for (int i = lane; i < (int)(S * I::stage_bytes / 16); i += 32) z[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    // region rows and columns wrap at most once (every side >= U)
    for (int q = lane; q < UU; q += 32) {
        int gz = z0 + q / U, gy = y0 + q % U;
        if (gz >= n0) gz -= n0;
        if (gy >= n1) gy -= n1;
        roff[q] = (gz * n1 + gy) * n2;
    }
    if (lane < U) {
        int gx = x0 + lane;
        if (gx >= n2) gx -= n2;
        xoff[lane] = gx;
    }
    // the group's padded window rows and footprint offsets within the bin (0..3)
    int s_l = -1, oz_l = 0, oy_l = 0, ox_l = 0;
    if (lane < kInterpGroup) {
        float *wr = wpad + lane * 3 * PL;
        if (lane < cnt) {
            s_l = ns.ilist[wk.y + lane];
            const int4 u = ns.nodeU3[s_l];
            oz_l = u.x - z0; oy_l = u.y - y0; ox_l = u.z - x0;
            const float *W = ns.nodeW + (size_t)s_l * kW3;
            for (int i = 0; i < PL; ++i) {
                const int t = i - 3;
                const bool in = (t >= 0 && t < TAPS);
                wr[i] = in ? W[t] : 0.f;
                wr[PL + i] = in ? W[TAPS + t] : 0.f;
                wr[2 * PL + i] = in ? W[2 * TAPS + t] : 0.f;
            }
        } else {
            for (int i = 0; i < 3 * PL; ++i) wr[i] = 0.f;
        }
    }
    __syncwarp();
    // staging: chunk ch of a k-step is point ch / CH, coils 2 (ch % CH) and 2 (ch % CH) + 1;
    // this lane's chunks keep their point slot, so their region coordinates advance by 8 per k-step
    int cz[NI], cy[NI], cx[NI];
#pragma unroll
    for (int i = 0; i < NI; ++i) {
        const int ch = lane + 32 * i;
        const int q = ch < NCH ? ch / CH : 0;
        cz[i] = q / UU; cy[i] = (q / U) % U; cx[i] = q % U;
    }
    const float2 *gsrc = grid + c0;
    auto issue = [&](int stage) {
        float *sb = sbase + stage * 8 * R;
#pragma unroll
        for (int i = 0; i < NI; ++i) {
            const int ch = lane + 32 * i;
            if (ch < NCH) {
                const int pi = ch / CH, c = 2 * (ch % CH);
                if (cz[i] < U && c < ccn) {
                    const float2 *src = gsrc + (size_t)(roff[cz[i] * U + cy[i]] + xoff[cx[i]]) * g.nc + c;
                    float2 *dst = reinterpret_cast<float2 *>(sb + pi * R) + c;
                    if (v16 && c + 1 < ccn) {
                        cp_async16(dst, src);
                    } else {
                        cp_async8(dst, src);
                        if (c + 1 < ccn) cp_async8(dst + 1, src + 1);
                    }
                }
                cx[i] += 8;
                while (cx[i] >= U) { cx[i] -= U; if (++cy[i] == U) { cy[i] = 0; ++cz[i]; } }
            }
        }
        cp_async_commit();
    };
    const int gq = lane >> 2, tq = lane & 3;
    const int na = gq, nb = gq + 8;
    const int oza = __shfl_sync(0xffffffffu, oz_l, na), oya = __shfl_sync(0xffffffffu, oy_l, na),
              oxa = __shfl_sync(0xffffffffu, ox_l, na);
    const int ozb = __shfl_sync(0xffffffffu, oz_l, nb), oyb = __shfl_sync(0xffffffffu, oy_l, nb),
              oxb = __shfl_sync(0xffffffffu, ox_l, nb);
    // row pointers shifted so that [q] is tap q - offset (zero outside)
    const float *Wza = wpad + na * 3 * PL + 3 - oza, *Wya = wpad + na * 3 * PL + PL + 3 - oya,
                *Wxa = wpad + na * 3 * PL + 2 * PL + 3 - oxa;
    const float *Wzb = wpad + nb * 3 * PL + 3 - ozb, *Wyb = wpad + nb * 3 * PL + PL + 3 - oyb,
                *Wxb = wpad + nb * 3 * PL + 2 * PL + 3 - oxb;
    float acc[NT][4];
#pragma unroll
    for (int t = 0; t < NT; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
    // region coordinates of the thread's two A points q0 = 8 k + tq and q1 = q0 + 4
    int qz0 = tq / UU, qy0 = (tq / U) % U, qx0 = tq % U;
    int qz1 = (tq + 4) / UU, qy1 = ((tq + 4) / U) % U, qx1 = (tq + 4) % U;
    __syncwarp();   // zeroed stages and the row tables before the first copies
#pragma unroll
    for (int st = 0; st < S - 1; ++st) {
        if (st < NK) issue(st);
        else cp_async_commit();
    }
#pragma unroll 1
    for (int k = 0; k < NK; ++k) {
        if (k + S - 1 < NK) issue((k + S - 1) % S);
        else cp_async_commit();
        cp_async_wait<S - 1>();
        __syncwarp();
        const float *sb = sbase + (k % S) * 8 * R;
        uint32_t ah[4], al[4];
        tf32_split(Wza[qz0] * (Wya[qy0] * Wxa[qx0]), ah[0], al[0]);
        tf32_split(Wzb[qz0] * (Wyb[qy0] * Wxb[qx0]), ah[1], al[1]);
        tf32_split(Wza[qz1] * (Wya[qy1] * Wxa[qx1]), ah[2], al[2]);
        tf32_split(Wzb[qz1] * (Wyb[qy1] * Wxb[qx1]), ah[3], al[3]);
        const float *r0 = sb + tq * R + gq, *r1 = sb + (tq + 4) * R + gq;
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            uint32_t bh0, bl0, bh1, bl1;
            tf32_split2(make_float2(r0[8 * t], r1[8 * t]), bh0, bh1, bl0, bl1);
            mma_tf32(acc[t], al, bh0, bh1);
            mma_tf32(acc[t], ah, bl0, bl1);
            mma_tf32(acc[t], ah, bh0, bh1);
        }
        qx0 += 8; while (qx0 >= U) { qx0 -= U; if (++qy0 == U) { qy0 = 0; ++qz0; } }
        qx1 += 8; while (qx1 >= U) { qx1 -= U; if (++qy1 == U) { qy1 = 0; ++qz1; } }
        __syncwarp();   // every lane is done with this stage before it is refilled
    }
    cp_async_wait<0>();
    // rows gq and gq + 8: nodes na and nb, columns 2 tq, 2 tq + 1 of each n-tile
    const int sa = __shfl_sync(0xffffffffu, s_l, na), sb_ = __shfl_sync(0xffffffffu, s_l, nb);
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        const int c = 4 * t + tq;
        if (c < ccn) {
            if (na < cnt) ks[(size_t)sa * g.nc + c0 + c] = make_float2(acc[t][0], acc[t][1]);
            if (nb < cnt) ks[(size_t)sb_ * g.nc + c0 + c] = make_float2(acc[t][2], acc[t][3]);
        }
    }
}

template <int NT, int TAPS>
static cgs_status launch_interp3_mma_t(const GridGeom &g, const NodeSet &ns, const float2 *grid, float2 *ks,
                                       cudaStream_t st)
{
    using I = Interp3Mma<NT, TAPS>;
    CGS_CUDA(cudaFuncSetAttribute(interp3_mma_kernel<NT, TAPS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)I::smem));
    dim3 grd((ns.niwork + 7) / 8, (g.nc + 4 * NT - 1) / (4 * NT));
    interp3_mma_kernel<NT, TAPS><<<grd, 256, I::smem, st>>>(g, ns, grid, ks);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

template <int TAPS>
static cgs_status launch_interp3_mma_taps(const GridGeom &g, const NodeSet &ns, const float2 *grid, float2 *ks,
                                          cudaStream_t st)
{
    switch (std::min(8, (2 * g.nc + 7) / 8)) {
        case 8: return launch_interp3_mma_t<8, TAPS>(g, ns, grid, ks, st);
        case 7: return launch_interp3_mma_t<7, TAPS>(g, ns, grid, ks, st);
        case 6: return launch_interp3_mma_t<6, TAPS>(g, ns, grid, ks, st);
        case 5: return launch_interp3_mma_t<5, TAPS>(g, ns, grid, ks, st);
        case 4: return launch_interp3_mma_t<4, TAPS>(g, ns, grid, ks, st);
        case 3: return launch_interp3_mma_t<3, TAPS>(g, ns, grid, ks, st);
        case 2: return launch_interp3_mma_t<2, TAPS>(g, ns, grid, ks, st);
        default: return launch_interp3_mma_t<1, TAPS>(g, ns, grid, ks, st);
    }
}

template <int NT, int TAPS>
static cgs_status launch_spread3_mma_t(const GridGeom &g, const PatchSet &ps, const float2 *ks, const float *dens,
                                       int weighted, float2 *grid, cudaStream_t st)
{
    using S = Spread3Mma<NT>;
    const size_t sm = 8 * S::warp_bytes;
    CGS_CUDA(cudaFuncSetAttribute(spread3_mma_kernel<NT, TAPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    dim3 grd((ps.nwork + 7) / 8, (g.nc + 4 * NT - 1) / (4 * NT));
    spread3_mma_kernel<NT, TAPS><<<grd, 256, sm, st>>>(g, ps, ks, dens, weighted, grid);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

template <int TAPS>
static cgs_status launch_spread3_mma_taps(const GridGeom &g, const PatchSet &ps, const float2 *ks, const float *dens,
                                          int weighted, float2 *grid, cudaStream_t st)
{
    // at most 16 coils per warp: four m-tiles of 4 NT accumulators each
    switch (std::min(4, (2 * g.nc + 7) / 8)) {
        case 4: return launch_spread3_mma_t<4, TAPS>(g, ps, ks, dens, weighted, grid, st);
        case 3: return launch_spread3_mma_t<3, TAPS>(g, ps, ks, dens, weighted, grid, st);
        case 2: return launch_spread3_mma_t<2, TAPS>(g, ps, ks, dens, weighted, grid, st);
        default: return launch_spread3_mma_t<1, TAPS>(g, ps, ks, dens, weighted, grid, st);
    }
}

// ---------------------------------------------------------------------------
// 3-D gridding, one warp per node.  A CTA owns a bin of footprint starts (T^3)
// and its padded E^3 tile (E = T + 2m + 1) for CC coils in shared memory,
// stored as planes of real and imaginary parts, [coil][part][z][y][x] with an
// x pitch PX >= E chosen on the host so that the TAPS x (32 / TAPS) points a
// warp touches in one step fall in distinct banks.  A warp takes one node at
// a time: its lanes evaluate the node's 3 x TAPS window weights (one per
// lane), then lane (row, x) of every y-step walks the TAPS z-planes of its
// (y, x) column with the z weights in registers.
//   interpolation: each lane accumulates its taps, then a warp reduction;
//   spreading: shared-memory atomics into the tile (conflict-free within a
//   step; other warps may hit the same point), then one atomic flush of the
//   tile into the grid per work item.
// ---------------------------------------------------------------------------
template <bool SPREAD, int TAPS, int CC>
__global__ void __launch_bounds__(256)
grid3_warp_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ NodeSet ns,
                  const float2 *__restrict__ in, int weighted, float2 *__restrict__ out, int PX)
{
    constexpr int RPI = 32 / TAPS;                     // x-rows per step
    constexpr int NSTEP = (TAPS + RPI - 1) / RPI;      // steps over the y taps
    extern __shared__ float4 smem4[];
    const int E = g.T + TAPS - 1;
    const int EE = E * E * E;
    const int plane = E * E * PX;                      // floats per (coil, part) plane
    const int4 wk = ns.work[blockIdx.x];
    const int c0 = blockIdx.y * CC;
    const int ccn = min(CC, g.nc - c0);
    const int org2 = (wk.x % g.nt[2]) * g.T;
    const int org1 = ((wk.x / g.nt[2]) % g.nt[1]) * g.T;
    const int org0 = (wk.x / (g.nt[2] * g.nt[1])) * g.T;
    float *tile = reinterpret_cast<float *>(smem4);
    float *wsm = tile + (size_t)CC * 2 * plane;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *W = wsm + warp * 3 * TAPS;
    auto grid_off = [&](int r) {
        const int lz = r / (E * E), ly = (r / E) % E, lx = r % E;
        return ((int64_t)wrapi(org0 + lz, g.n[0]) * g.n[1] + wrapi(org1 + ly, g.n[1])) * g.n[2] + wrapi(org2 + lx, g.n[2]);
    };
    auto tile_off = [&](int r) {
        const int lz = r / (E * E), ly = (r / E) % E, lx = r % E;
        return (lz * E + ly) * PX + lx;
    };

    // tile: zeros (spreading) or the grid values (interpolation), batches of
    // kUnroll independent loads per thread in flight
    constexpr int kUnroll = 8;
    for (int e0 = threadIdx.x; e0 < EE * CC; e0 += 256 * kUnroll) {
        float2 v[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const int e = e0 + u * 256;
            const int cc = e % CC;
            v[u] = make_float2(0.f, 0.f);
            if (!SPREAD && e < EE * CC && cc < ccn) v[u] = in[grid_off(e / CC) * g.nc + c0 + cc];
        }
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const int e = e0 + u * 256;
            if (e < EE * CC) {
                const int cc = e % CC, t = tile_off(e / CC);
                tile[(2 * cc) * plane + t] = v[u].x;
                tile[(2 * cc + 1) * plane + t] = v[u].y;
            }
        }
    }
    __syncthreads();

    const float mf = (float)g.m;
    const int ry = lane / TAPS, rx = lane % TAPS;
    const bool act = ry < RPI;
    for (int i = warp; i < wk.z; i += 8) {
        const int64_t s = (int64_t)wk.y + i;
        const float4 na = ns.nodes[2 * s], nb = ns.nodes[2 * s + 1];
        const int l0 = wrapi(__float_as_int(nb.x) - g.m, g.n[0]) - org0;
        const int l1 = wrapi(__float_as_int(nb.y) - g.m, g.n[1]) - org1;
        const int l2 = wrapi(__float_as_int(nb.z) - g.m, g.n[2]) - org2;
        for (int e = lane; e < 3 * TAPS; e += 32) {
            const int t = e / TAPS, q = e % TAPS;
            const float ft = t == 0 ? na.x : (t == 1 ? na.y : na.z);
            const float bt = t == 0 ? g.b[0] : (t == 1 ? g.b[1] : g.b[2]);
            W[e] = kb_phi(ft + mf - (float)q, mf, bt);
        }
        __syncwarp();
        float wz[TAPS];
#pragma unroll
        for (int q = 0; q < TAPS; ++q) wz[q] = W[q];
        const float wx = act ? W[2 * TAPS + rx] : 0.f;
        float2 v[CC];
        if (SPREAD) {
            const float dw = (weighted && ns.w) ? ns.w[s] : 1.f;
#pragma unroll
            for (int cc = 0; cc < CC; ++cc) {
                v[cc] = cc < ccn ? in[s * g.nc + c0 + cc] : make_float2(0.f, 0.f);
                v[cc].x *= dw; v[cc].y *= dw;
            }
        } else {
#pragma unroll
            for (int cc = 0; cc < CC; ++cc) v[cc] = make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int st = 0; st < NSTEP; ++st) {
            const int b = st * RPI + ry;
            if (act && b < TAPS) {
                const float wyx = W[TAPS + b] * wx;
                const int base = (l0 * E + l1 + b) * PX + l2 + rx;
#pragma unroll
                for (int a = 0; a < TAPS; ++a) {
                    const float w = wz[a] * wyx;
                    const int t = base + a * E * PX;
#pragma unroll
                    for (int cc = 0; cc < CC; ++cc) {
                        float *re = tile + (2 * cc) * plane + t;
                        float *im = tile + (2 * cc + 1) * plane + t;
                        if (SPREAD) {
                            atomicAdd(re, w * v[cc].x);
                            atomicAdd(im, w * v[cc].y);
                        } else {
                            v[cc].x = fmaf(w, *re, v[cc].x);
                            v[cc].y = fmaf(w, *im, v[cc].y);
                        }
                    }
                }
            }
        }
        if (!SPREAD) {
#pragma unroll
            for (int cc = 0; cc < CC; ++cc) {
                float x = v[cc].x, y = v[cc].y;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    x += __shfl_down_sync(0xffffffffu, x, o);
                    y += __shfl_down_sync(0xffffffffu, y, o);
                }
                if (lane == 0 && cc < ccn) out[s * g.nc + c0 + cc] = make_float2(x, y);
            }
        }
        __syncwarp();
    }
    if (!SPREAD) return;
    __syncthreads();
    // add the tile to the grid (wrapped)
    for (int e = threadIdx.x; e < EE * CC; e += 256) {
        const int cc = e % CC;
        if (cc >= ccn) continue;
        const int t = tile_off(e / CC);
        const float vx = tile[(2 * cc) * plane + t], vy = tile[(2 * cc + 1) * plane + t];
        if (vx == 0.f && vy == 0.f) continue;
        float2 *dst = out + grid_off(e / CC) * g.nc + c0 + cc;
        atomicAdd(&dst->x, vx);
        atomicAdd(&dst->y, vy);
    }
}

// 3-D spreading without atomics in shared memory: the tile's z-planes are
// dealt round-robin to the CTA's 8 warps, every warp walks every staged node
// and adds only the node's taps in its own planes (plain read-modify-write:
// no two warps share a plane, no two lanes of a step share a point).  Batches
// of kStage3 nodes (window weights, footprint starts, density-weighted
// values) are staged for the whole CTA; the tile is flushed into the grid
// with one atomic add per point and coil.
constexpr int kStage3 = 32;

template <int TAPS, int CC>
__global__ void __launch_bounds__(256)
spread3_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ NodeSet ns,
               const float2 *__restrict__ ks, int weighted, float2 *__restrict__ grid, int PX)
{
    constexpr int RPI = 32 / TAPS;
    constexpr int NSTEP = (TAPS + RPI - 1) / RPI;
    extern __shared__ float4 smem4[];
    const int E = g.T + TAPS - 1;
    const int EE = E * E * E;
    const int plane = E * E * PX;
    const int4 wk = ns.work[blockIdx.x];
    const int c0 = blockIdx.y * CC;
    const int ccn = min(CC, g.nc - c0);
    const int org2 = (wk.x % g.nt[2]) * g.T;
    const int org1 = ((wk.x / g.nt[2]) % g.nt[1]) * g.T;
    const int org0 = (wk.x / (g.nt[2] * g.nt[1])) * g.T;
    float *tile = reinterpret_cast<float *>(smem4);
    float *sW = tile + (size_t)CC * 2 * plane;                   // [kStage3][3 TAPS]
    float2 *sV = reinterpret_cast<float2 *>(sW + kStage3 * 3 * TAPS);  // [kStage3][CC]
    int *sL = reinterpret_cast<int *>(sV + kStage3 * CC);        // [kStage3][3]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int e = threadIdx.x; e < CC * 2 * plane; e += 256) tile[e] = 0.f;

    const float mf = (float)g.m;
    const int ry = lane / TAPS, rx = lane % TAPS;
    const bool act = ry < RPI;
    for (int j0 = 0; j0 < wk.z; j0 += kStage3) {
        const int cnt = min(kStage3, wk.z - j0);
        __syncthreads();   // the previous batch is consumed (and the tile zeroed)
        for (int e = threadIdx.x; e < cnt * 3 * TAPS; e += 256) {
            const int j = e / (3 * TAPS), r = e % (3 * TAPS), t = r / TAPS, q = r % TAPS;
            const int64_t s = (int64_t)wk.y + j0 + j;
            const float4 na = ns.nodes[2 * s];
            const float ft = t == 0 ? na.x : (t == 1 ? na.y : na.z);
            const float bt = t == 0 ? g.b[0] : (t == 1 ? g.b[1] : g.b[2]);
            sW[e] = kb_phi(ft + mf - (float)q, mf, bt);
        }
        for (int e = threadIdx.x; e < cnt * CC; e += 256) {
            const int j = e / CC, cc = e % CC;
            const int64_t s = (int64_t)wk.y + j0 + j;
            float2 v = cc < ccn ? ks[s * g.nc + c0 + cc] : make_float2(0.f, 0.f);
            const float dw = (weighted && ns.w) ? ns.w[s] : 1.f;
            v.x *= dw; v.y *= dw;
            sV[e] = v;
        }
        for (int j = threadIdx.x; j < cnt; j += 256) {
            const int64_t s = (int64_t)wk.y + j0 + j;
            const float4 nb = ns.nodes[2 * s + 1];
            sL[3 * j] = wrapi(__float_as_int(nb.x) - g.m, g.n[0]) - org0;
            sL[3 * j + 1] = wrapi(__float_as_int(nb.y) - g.m, g.n[1]) - org1;
            sL[3 * j + 2] = wrapi(__float_as_int(nb.z) - g.m, g.n[2]) - org2;
        }
        __syncthreads();
        for (int j = 0; j < cnt; ++j) {
            const int l0 = sL[3 * j], l1 = sL[3 * j + 1], l2 = sL[3 * j + 2];
            const float *W = sW + j * 3 * TAPS;
            const float wx = act ? W[2 * TAPS + rx] : 0.f;
            float2 v[CC];
#pragma unroll
            for (int cc = 0; cc < CC; ++cc) v[cc] = sV[j * CC + cc];
            // this warp's planes z = l0 + a with z % 8 == warp
            for (int a = ((warp - l0) % 8 + 8) % 8; a < TAPS; a += 8) {
                const float wz = W[a];
#pragma unroll
                for (int st = 0; st < NSTEP; ++st) {
                    const int b = st * RPI + ry;
                    if (act && b < TAPS) {
                        const float w = wz * W[TAPS + b] * wx;
                        const int t = ((l0 + a) * E + l1 + b) * PX + l2 + rx;
#pragma unroll
                        for (int cc = 0; cc < CC; ++cc) {
                            float *re = tile + (2 * cc) * plane + t;
                            float *im = tile + (2 * cc + 1) * plane + t;
                            *re = fmaf(w, v[cc].x, *re);
                            *im = fmaf(w, v[cc].y, *im);
                        }
                    }
                }
            }
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < EE * CC; e += 256) {
        const int cc = e % CC;
        if (cc >= ccn) continue;
        const int r = e / CC;
        const int lz = r / (E * E), ly = (r / E) % E, lx = r % E;
        const int t = (lz * E + ly) * PX + lx;
        const float vx = tile[(2 * cc) * plane + t], vy = tile[(2 * cc + 1) * plane + t];
        if (vx == 0.f && vy == 0.f) continue;
        const int64_t off = ((int64_t)wrapi(org0 + lz, g.n[0]) * g.n[1] + wrapi(org1 + ly, g.n[1])) * g.n[2] +
                            wrapi(org2 + lx, g.n[2]);
        float2 *dst = grid + off * g.nc + c0 + cc;
        atomicAdd(&dst->x, vx);
        atomicAdd(&dst->y, vy);
    }
}

// x pitch of the 3-D tile planes: the smallest PX >= E for which the
// (32 / taps) rows x taps points of one warp step fall in distinct banks
int grid3_pitch(int E, int taps)
{
    const int rpi = 32 / taps;
    for (int px = E; px < E + 32; ++px) {
        bool used[32] = {false};
        bool ok = true;
        for (int r = 0; r < rpi && ok; ++r)
            for (int x = 0; x < taps && ok; ++x) {
                const int bank = (r * px + x) % 32;
                ok = !used[bank];
                used[bank] = true;
            }
        if (ok) return px;
    }
    return E;
}

size_t grid3_smem(int E, int PX, int taps, int CC)
{
    // tile planes + the larger of the interpolation per-warp weights and the
    // spreading node batch (weights, values, footprint starts)
    const size_t stage = std::max<size_t>((size_t)8 * 3 * taps * sizeof(float),
                                          (size_t)kStage3 * (3 * taps * sizeof(float) + CC * sizeof(float2) + 3 * sizeof(int)));
    return (size_t)CC * 2 * E * E * PX * sizeof(float) + stage;
}

template <bool SPREAD, int TAPS>
cgs_status launch_grid3_taps(const GridGeom &g, const NodeSet &ns, const float2 *in, int weighted, float2 *out,
                             cudaStream_t st)
{
    const int E = g.T + TAPS - 1;
    const int PX = grid3_pitch(E, TAPS);
    const int CC = (g.nc >= 2 && grid3_smem(E, PX, TAPS, 2) <= 110 * 1024) ? 2 : 1;
    const size_t smem = grid3_smem(E, PX, TAPS, CC);
    if (smem > 200 * 1024) { set_error("3-D gridding tile does not fit in shared memory"); return CGS_ERR_BAD_ARG; }
    dim3 grd(ns.nwork, (g.nc + CC - 1) / CC);
#define CGS_G3(CCV)                                                                                         \
    do {                                                                                                  \
        if (SPREAD) {                                                                                     \
            CGS_CUDA(cudaFuncSetAttribute(spread3_kernel<TAPS, CCV>,                                       \
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));       \
            spread3_kernel<TAPS, CCV><<<grd, 256, smem, st>>>(g, ns, in, weighted, out, PX);               \
        } else {                                                                                          \
            CGS_CUDA(cudaFuncSetAttribute(grid3_warp_kernel<false, TAPS, CCV>,                             \
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));       \
            grid3_warp_kernel<false, TAPS, CCV><<<grd, 256, smem, st>>>(g, ns, in, weighted, out, PX);     \
        }                                                                                                 \
    } while (0)
    if (CC == 2) CGS_G3(2);
    else CGS_G3(1);
#undef CGS_G3
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

template <bool SPREAD>
cgs_status launch_grid3(const GridGeom &g, const NodeSet &ns, const float2 *in, int weighted, float2 *out,
                        cudaStream_t st)
{
    switch (2 * g.m + 2) {
        case 4: return launch_grid3_taps<SPREAD, 4>(g, ns, in, weighted, out, st);
        case 6: return launch_grid3_taps<SPREAD, 6>(g, ns, in, weighted, out, st);
        case 8: return launch_grid3_taps<SPREAD, 8>(g, ns, in, weighted, out, st);
        case 10: return launch_grid3_taps<SPREAD, 10>(g, ns, in, weighted, out, st);
        case 12: return launch_grid3_taps<SPREAD, 12>(g, ns, in, weighted, out, st);
        case 14: return launch_grid3_taps<SPREAD, 14>(g, ns, in, weighted, out, st);
        case 16: return launch_grid3_taps<SPREAD, 16>(g, ns, in, weighted, out, st);
        default: set_error("m too large for 3-D gridding"); return CGS_ERR_BAD_ARG;
    }
}

GridCfg pick_cfg(const GridGeom &g)
{
    GridCfg c;
    c.E = g.T + 2 * g.m + 1;
    size_t Et = 1;
    for (int d = 0; d < g.d; ++d) Et *= (size_t)c.E;
    const size_t fixed = (size_t)kChunk * 3 * kMaxTaps * 4 + (size_t)kChunk * 3 * 4;
    const size_t budget = 100 * 1024;
    int CC = (int)((budget - fixed) / (Et * 8));
    if (CC > g.nc) CC = g.nc;
    if (CC > 8) CC = 8;
    if (CC < 1) CC = 1;
    c.CC = CC;
    return c;
}

size_t smem_bytes(const GridGeom &g, const GridCfg &c)
{
    size_t Et = 1;
    for (int d = 0; d < g.d; ++d) Et *= (size_t)c.E;
    return Et * c.CC * 8 + (size_t)kChunk * 3 * kMaxTaps * 4 + (size_t)kChunk * 3 * 4;
}

}  // namespace

template <int TAPS>
cgs_status launch_interp2_taps(const GridGeom &g, const NodeSet &ns, const float2 *grid, float2 *ks, int CC,
                               cudaStream_t st)
{
    const int E = g.T + TAPS - 1;
    const size_t smem = (size_t)E * E * CC * sizeof(float2);
    dim3 grd(ns.nwork, (g.nc + CC - 1) / CC);
#define CGS_I2(CCV, CPLV)                                                                                   \
    do {                                                                                                  \
        CGS_CUDA(cudaFuncSetAttribute(interp2_kernel<TAPS, CCV, CPLV>,                                     \
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));           \
        interp2_kernel<TAPS, CCV, CPLV><<<grd, 256, smem, st>>>(g, ns, ns.nodeU, ns.nodeW, grid, ks);      \
    } while (0)
    if (CC == 32) CGS_I2(32, 2);
    else if (CC == 16) CGS_I2(16, 2);
    else if (CC == 8) CGS_I2(8, 2);
    else if (CC == 4) CGS_I2(4, 2);
    else CGS_I2(1, 1);
#undef CGS_I2
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_interp_windows(const GridGeom &g, const NodeSet &ns, float *iwin, int4 *imeta, cudaStream_t st)
{
    const int taps = 2 * g.m + 2;
    if (ns.niwork == 0 || g.d != 2 || taps > 10 || (taps & 1)) return CGS_OK;
    const unsigned blocks = (unsigned)((ns.niwork + 7) / 8);
    switch (taps) {
        case 4: interp_windows_kernel<4><<<blocks, 256, 0, st>>>(g, ns, iwin, imeta); break;
        case 6: interp_windows_kernel<6><<<blocks, 256, 0, st>>>(g, ns, iwin, imeta); break;
        case 8: interp_windows_kernel<8><<<blocks, 256, 0, st>>>(g, ns, iwin, imeta); break;
        default: interp_windows_kernel<10><<<blocks, 256, 0, st>>>(g, ns, iwin, imeta); break;
    }
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_interp(const GridGeom &g, const NodeSet &ns, const float2 *grid, float2 *ks,
                         cudaStream_t st, float2 *user, bool *wrote_user)
{
    if (wrote_user) *wrote_user = false;
    if (ns.nwork == 0 || g.nc == 0) return CGS_OK;
    if (2 * g.m + 2 > kMaxTaps) { set_error("m too large"); return CGS_ERR_BAD_ARG; }
    const int taps = 2 * g.m + 2;
    if (g.d == 2 && g.imma == 2 && ns.ilist && ns.niwork > 0 && ns.nodeU && ns.nodeW && taps <= 10 &&
        g.n[0] >= kIsBH - 1 + taps && g.n[1] >= kIsBW - 1 + taps) {
        cgs_status r;
        float2 *u = (user && ns.perm) ? user : nullptr;
        prof_begin(PROF_INTERP, st);
        switch (taps) {
            case 4: r = launch_interp_tc_taps<4>(g, ns, grid, ks, u, st); break;
            case 6: r = launch_interp_tc_taps<6>(g, ns, grid, ks, u, st); break;
            case 8: r = launch_interp_tc_taps<8>(g, ns, grid, ks, u, st); break;
            default: r = launch_interp_tc_taps<10>(g, ns, grid, ks, u, st); break;
        }
        prof_end(PROF_INTERP, st);
        if (r == CGS_OK && wrote_user) *wrote_user = (u != nullptr);
        return r;
    }
    if (g.d == 2 && g.imma == 1 && ns.ilist && ns.niwork > 0 && ns.iwin && ns.imeta && taps <= 10 &&
        g.n[0] >= 3 + taps && g.n[1] >= 3 + taps) {
        cgs_status r;
        float2 *u = (user && ns.perm) ? user : nullptr;
        prof_begin(PROF_INTERP, st);
        switch (taps) {
            case 4: r = launch_interp_mma_taps<4>(g, ns, grid, ks, u, st); break;
            case 6: r = launch_interp_mma_taps<6>(g, ns, grid, ks, u, st); break;
            case 8: r = launch_interp_mma_taps<8>(g, ns, grid, ks, u, st); break;
            default: r = launch_interp_mma_taps<10>(g, ns, grid, ks, u, st); break;
        }
        prof_end(PROF_INTERP, st);
        if (r == CGS_OK && wrote_user) *wrote_user = (u != nullptr);
        return r;
    }
    if (g.d == 2 && ns.nodeU && ns.nodeW && taps <= 10) {
        // 16 coils per CTA by default: a 46 KB tile (T = 16, m = 4) leaves room
        // for 4 CTAs per SM, and each node reads one full bank row per tap
        const int CC = g.icc > 0 ? g.icc : (g.nc >= 16 ? 16 : (g.nc >= 8 ? 8 : (g.nc >= 4 ? 4 : 1)));
        const int E = g.T + taps - 1;
        if ((size_t)E * E * CC * sizeof(float2) <= 200 * 1024) {
            cgs_status r;
            prof_begin(PROF_INTERP, st);
            switch (taps) {
                case 4: r = launch_interp2_taps<4>(g, ns, grid, ks, CC, st); break;
                case 6: r = launch_interp2_taps<6>(g, ns, grid, ks, CC, st); break;
                case 8: r = launch_interp2_taps<8>(g, ns, grid, ks, CC, st); break;
                default: r = launch_interp2_taps<10>(g, ns, grid, ks, CC, st); break;
            }
            prof_end(PROF_INTERP, st);
            return r;
        }
    }
    if (g.d == 3 && g.imma && grid3_mma_ok(g) && ns.ilist && ns.nodeU3 && ns.nodeW && ns.niwork > 0) {
        cgs_status r;
        prof_begin(PROF_INTERP, st);
        switch (taps) {
            case 4: r = launch_interp3_mma_taps<4>(g, ns, grid, ks, st); break;
            case 6: r = launch_interp3_mma_taps<6>(g, ns, grid, ks, st); break;
            case 8: r = launch_interp3_mma_taps<8>(g, ns, grid, ks, st); break;
            default: r = launch_interp3_mma_taps<10>(g, ns, grid, ks, st); break;
        }
        prof_end(PROF_INTERP, st);
        return r;
    }
    if (g.d == 3) {
        prof_begin(PROF_INTERP, st);
        const cgs_status r = launch_grid3<false>(g, ns, grid, 0, ks, st);
        prof_end(PROF_INTERP, st);
        return r;
    }
    GridCfg c = pick_cfg(g);
    size_t smem = smem_bytes(g, c);
    if (smem > 200 * 1024) { set_error("gridding tile does not fit in shared memory"); return CGS_ERR_BAD_ARG; }
    dim3 grd(ns.nwork, (g.nc + c.CC - 1) / c.CC);
    prof_begin(PROF_INTERP, st);
    if (g.d == 2) {
        CGS_CUDA(cudaFuncSetAttribute(interp_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        interp_kernel<2><<<grd, kThreads, smem, st>>>(g, ns, grid, ks, c.CC);
    } else {
        CGS_CUDA(cudaFuncSetAttribute(interp_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        interp_kernel<3><<<grd, kThreads, smem, st>>>(g, ns, grid, ks, c.CC);
    }
    prof_end(PROF_INTERP, st);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_node_weights(const GridGeom &g, const NodeSet &ns, int2 *nodeU, float *nodeW,
                               cudaStream_t st)
{
    if (g.d != 2) { set_error("node weight tables are 2-D only"); return CGS_ERR_BAD_ARG; }
    if (ns.M == 0) return CGS_OK;
    const int64_t blocks = std::min<int64_t>((ns.M + 255) / 256, 152 * 16);
    node_weights_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, ns, nodeU, nodeW);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

bool grid3_mma_ok(const GridGeom &g)
{
    const int taps = 2 * g.m + 2;
    return g.d == 3 && taps <= 10 && g.n[0] >= 3 + taps && g.n[1] >= 3 + taps && g.n[2] >= 3 + taps;
}

cgs_status launch_node_weights3(const GridGeom &g, const NodeSet &ns, int4 *nodeU3, float *nodeW,
                                cudaStream_t st)
{
    if (!grid3_mma_ok(g)) { set_error("3-D node tables need taps <= 10 and every side >= 3 + taps"); return CGS_ERR_BAD_ARG; }
    if (ns.M == 0) return CGS_OK;
    const int64_t blocks = std::min<int64_t>((ns.M + 255) / 256, 152 * 16);
    node_weights3_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, ns, nodeU3, nodeW);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_spread_patch3(const GridGeom &g, const PatchSet &ps, const float2 *ks, const float *dens,
                                int weighted, float2 *grid, cudaStream_t st)
{
    if (ps.nwork == 0 || g.nc == 0) return CGS_OK;
    if (!grid3_mma_ok(g) || ps.pd != 4 || !ps.nodeU3) { set_error("3-D patch lists missing"); return CGS_ERR_BAD_ARG; }
    cgs_status r;
    prof_begin(PROF_SPREAD, st);
    switch (2 * g.m + 2) {
        case 4: r = launch_spread3_mma_taps<4>(g, ps, ks, dens, weighted, grid, st); break;
        case 6: r = launch_spread3_mma_taps<6>(g, ps, ks, dens, weighted, grid, st); break;
        case 8: r = launch_spread3_mma_taps<8>(g, ps, ks, dens, weighted, grid, st); break;
        default: r = launch_spread3_mma_taps<10>(g, ps, ks, dens, weighted, grid, st); break;
    }
    if (r == CGS_OK && ps.nmulti > 0) {
        const int64_t total = (int64_t)ps.nmulti * 64 * g.nc;
        const int64_t blocks = std::min<int64_t>((total + 255) / 256, 152 * 16);
        patch_reduce3_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, ps, grid);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) { set_error(std::string("kernel launch: ") + cudaGetErrorString(e)); r = CGS_ERR_CUDA; }
        else count_launch();
    }
    prof_end(PROF_SPREAD, st);
    return r;
}

cgs_status launch_spread_tc_weights(const GridGeom &g, const PatchSet &ps, float *pw16, int *ps16, cudaStream_t st)
{
    if (ps.nwork == 0) return CGS_OK;
    spread_tc_weights_kernel<<<ps.nwork, 256, 0, st>>>(g, ps, pw16, ps16);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_spread_patch(const GridGeom &g, const PatchSet &ps, const float2 *ks, const float *dens,
                               int weighted, float2 *grid, cudaStream_t st)
{
    if (ps.nwork == 0) return CGS_OK;
    const int taps = 2 * g.m + 2;
    if (taps > kMaxTaps) { set_error("m too large"); return CGS_ERR_BAD_ARG; }
    // coils per warp: the next power of two >= coils (at most 32), or the tuned value
    int CC = 1;
    if (ps.pw == 8 && ps.blk == 1) {
        CC = 1;
    } else if (ps.blk == 8) {
        CC = 2;
        while (CC < g.nc && CC < 16) CC *= 2;
        if (g.scc > 0) CC = g.scc < 2 ? 2 : (g.scc > 16 ? 16 : g.scc);
    } else {
        const int lo = ps.blk >= 2 ? 4 : 2;
        CC = lo;
        while (CC < g.nc && CC < 32) CC *= 2;
        if (g.scc > 0) CC = g.scc < lo ? lo : g.scc;
    }
    dim3 grd((ps.nwork + 7) / 8, (g.nc + CC - 1) / CC);
    prof_begin(PROF_SPREAD, st);
#define CGS_SPT(PHV, PWV, CPLV, BYV, BXV, TV)                                                               \
    do {                                                                                                  \
        const size_t sm = 8 * 2 * SpreadShape<PHV, PWV, CPLV, BYV, BXV>::buf_bytes(taps);                 \
        CGS_CUDA(cudaFuncSetAttribute(spread_patch_kernel<PHV, PWV, CPLV, BYV, BXV, TV>,                   \
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));             \
        spread_patch_kernel<PHV, PWV, CPLV, BYV, BXV, TV><<<grd, 256, sm, st>>>(g, ps, ks, dens, weighted, grid); \
    } while (0)
#define CGS_SP(PHV, PWV, CPLV, BYV, BXV) CGS_SPT(PHV, PWV, CPLV, BYV, BXV, 0)
    // the common footprint (m = 4) with one point per lane on 4 x 4 patches: compile-time taps
#define CGS_SP1(CPLV)                                           \
    do {                                                        \
        if (taps == 10) CGS_SPT(4, 4, CPLV, 1, 1, 10);          \
        else CGS_SP(4, 4, CPLV, 1, 1);                          \
    } while (0)
    if (ps.blk == 64) {   // tcgen05: 8 x 16 patches, 32 coils per CTA (16 or 8 for fewer coils)
        if (ps.ph != kSpTcPH || ps.pw != kSpTcPW) { set_error("unsupported spreading patch"); return CGS_ERR_BAD_ARG; }
        const int ncol = g.nc > 8 ? (g.nc > 16 ? 64 : 32) : 16;
        dim3 grt(ps.nwork, (g.nc + ncol / 2 - 1) / (ncol / 2));
#define CGS_SPTC(NCV)                                                                                     \
    do {                                                                                                  \
        CGS_CUDA(cudaFuncSetAttribute(spread_tc05_kernel<NCV>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                      SpreadTc<NCV>::SMEM));                                              \
        CGS_CUDA(launch_pdl(spread_tc05_kernel<NCV>, grt, dim3(kSpTcThreads + 32), (size_t)SpreadTc<NCV>::SMEM, st, g, ps, \
                            ks, dens, weighted, grid));                                                   \
    } while (0)
        if (!ps.pw16 || !ps.ps16 || !ps.pstage) { set_error("tcgen05 spreading blocks missing"); return CGS_ERR_STATE; }
        if (ncol == 64) CGS_SPTC(64);
        else if (ncol == 32) CGS_SPTC(32);
        else CGS_SPTC(16);
#undef CGS_SPTC
    } else if ((ps.ph != 4 && !(ps.ph == 8 && ps.blk == 32)) || (ps.pw != 4 && ps.pw != 8)) {
        set_error("unsupported spreading patch");
        return CGS_ERR_BAD_ARG;
    } else if (ps.blk == 16 || ps.blk == 32) {  // tensor cores: 4 NT coils per warp, 4 x 4 or 8 x 4 patches
        if (ps.pw != 4 || ps.ph != (ps.blk == 32 ? 8 : 4)) { set_error("unsupported spreading patch"); return CGS_ERR_BAD_ARG; }
        const int nt = std::min(8, (2 * g.nc + 7) / 8);
        dim3 grm((ps.nwork + 7) / 8, (g.nc + 4 * nt - 1) / (4 * nt));
#define CGS_SPMM(NTV, TV, MTV)                                                                           \
    do {                                                                                                 \
        const size_t sm = 8 * SpreadMma<NTV, MTV>::warp_bytes(taps);                                     \
        CGS_CUDA(cudaFuncSetAttribute(spread_mma_kernel<NTV, TV, MTV>,                                   \
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));            \
        spread_mma_kernel<NTV, TV, MTV><<<grm, 256, sm, st>>>(g, ps, ks, dens, weighted, grid);          \
    } while (0)
#define CGS_SPM(NTV, TV)                                  \
    do {                                                  \
        if (ps.blk == 32) CGS_SPMM(NTV, TV, 2);           \
        else CGS_SPMM(NTV, TV, 1);                        \
    } while (0)
#define CGS_SPM1(NTV)                                     \
    do {                                                  \
        if (taps == 10) CGS_SPM(NTV, 10);                 \
        else CGS_SPM(NTV, 0);                             \
    } while (0)
        switch (nt) {
            case 8: CGS_SPM1(8); break;
            case 7: CGS_SPM1(7); break;
            case 6: CGS_SPM1(6); break;
            case 5: CGS_SPM1(5); break;
            case 4: CGS_SPM1(4); break;
            case 3: CGS_SPM1(3); break;
            case 2: CGS_SPM1(2); break;
            default: CGS_SPM1(1); break;
        }
#undef CGS_SPM1
#undef CGS_SPM
#undef CGS_SPMM
    } else if (ps.pw == 8 && ps.blk == 1) {
        CGS_SP(4, 8, 1, 1, 1);
    } else if (ps.blk == 8) {
        switch (CC) {
            case 16: CGS_SP(4, 8, 16, 1, 1); break;
            case 8: CGS_SP(4, 8, 8, 1, 1); break;
            case 4: CGS_SP(4, 8, 4, 1, 1); break;
            default: CGS_SP(4, 8, 2, 1, 1); break;
        }
    } else if (ps.blk == 2) {
        switch (CC) {
            case 32: CGS_SP(4, 4, 8, 2, 1); break;
            case 16: CGS_SP(4, 4, 4, 2, 1); break;
            case 8: CGS_SP(4, 4, 2, 2, 1); break;
            default: CGS_SP(4, 4, 1, 2, 1); break;
        }
    } else if (ps.pw == 8) {
        switch (CC) {
            case 32: CGS_SP(4, 8, 8, 2, 2); break;
            case 16: CGS_SP(4, 8, 4, 2, 2); break;
            case 8: CGS_SP(4, 8, 2, 2, 2); break;
            default: CGS_SP(4, 8, 1, 2, 2); break;
        }
    } else {
        switch (CC) {
            case 32: CGS_SP1(16); break;
            case 16: CGS_SP1(8); break;
            case 8: CGS_SP1(4); break;
            case 4: CGS_SP1(2); break;
            default: CGS_SP1(1); break;
        }
    }
#undef CGS_SP1
#undef CGS_SP
#undef CGS_SPT
    CGS_LAUNCH_CHECK();
    if (ps.nmulti > 0) {
        const bool v2 = (g.nc % 2) == 0;
        const int64_t total = (int64_t)ps.nmulti * ps.ph * ps.pw * (v2 ? g.nc / 2 : g.nc);
        const int64_t blocks = std::min<int64_t>((total + 255) / 256, 152 * 16);
        if (v2) CGS_CUDA(launch_pdl(patch_reduce2_kernel, dim3((unsigned)blocks), dim3(256), 0, st, g, ps, grid));
        else patch_reduce_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, ps, grid);
        CGS_LAUNCH_CHECK();
    }
    prof_end(PROF_SPREAD, st);
    return CGS_OK;
}

cgs_status launch_spread(const GridGeom &g, const NodeSet &ns, const float2 *ks, int weighted,
                         float2 *grid, cudaStream_t st)
{
    if (ns.nwork == 0 || g.nc == 0) return CGS_OK;
    if (2 * g.m + 2 > kMaxTaps) { set_error("m too large"); return CGS_ERR_BAD_ARG; }
    if (g.d == 3) {
        prof_begin(PROF_SPREAD, st);
        const cgs_status r = launch_grid3<true>(g, ns, ks, weighted, grid, st);
        prof_end(PROF_SPREAD, st);
        return r;
    }
    GridCfg c = pick_cfg(g);
    size_t smem = smem_bytes(g, c);
    if (smem > 200 * 1024) { set_error("gridding tile does not fit in shared memory"); return CGS_ERR_BAD_ARG; }
    dim3 grd(ns.nwork, (g.nc + c.CC - 1) / c.CC);
    prof_begin(PROF_SPREAD, st);
    if (g.d == 2) {
        CGS_CUDA(cudaFuncSetAttribute(spread_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        spread_kernel<2><<<grd, kThreads, smem, st>>>(g, ns, ks, weighted, grid, c.CC);
    } else {
        CGS_CUDA(cudaFuncSetAttribute(spread_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        spread_kernel<3><<<grd, kThreads, smem, st>>>(g, ns, ks, weighted, grid, c.CC);
    }
    prof_end(PROF_SPREAD, st);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

}  // namespace cgs
