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

cgs_status launch_interp(const GridGeom &g, const NodeSet &ns, const float2 *grid, float2 *ks,
                         cudaStream_t st)
{
    if (ns.nwork == 0 || g.nc == 0) return CGS_OK;
    if (2 * g.m + 2 > kMaxTaps) { set_error("m too large"); return CGS_ERR_BAD_ARG; }
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

cgs_status launch_spread(const GridGeom &g, const NodeSet &ns, const float2 *ks, int weighted,
                         float2 *grid, cudaStream_t st)
{
    if (ns.nwork == 0 || g.nc == 0) return CGS_OK;
    if (2 * g.m + 2 > kMaxTaps) { set_error("m too large"); return CGS_ERR_BAD_ARG; }
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
