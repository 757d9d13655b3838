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

// ---------------------------------------------------------------------------
// Output-stationary 2-D spreading.  Lane l of a warp owns grid point
// (py0 + l/8, px0 + l%8) of a 4 x 8 patch and accumulates CC coils in
// registers while the warp walks the patch's node list; every node value is
// one uniform (broadcast) load per coil, no atomics anywhere.  A crowded patch
// is split into several work items whose partial sums land in `partial` and
// are added in slot order by patch_reduce_kernel, so results are bitwise
// reproducible.
// ---------------------------------------------------------------------------
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

// Per-warp staging in shared memory of a batch of 32 list entries: lane l
// fetches entry l's node weights, values and density weight with independent
// loads, so one global round trip serves 32 entries; the accumulation loop
// then reads only shared memory (broadcasts and conflict-free rows).  The
// value rows are padded to a 16-byte multiple so two coils come per load.
template <int CC> struct SpreadRow { static constexpr int v = CC + ((CC & 1) ? 1 : 2); };

template <int CC>
__host__ __device__ __forceinline__ size_t spread_patch_smem_per_warp(int taps)
{
    return (size_t)32 * ((2 * taps + 1) * sizeof(float) + SpreadRow<CC>::v * sizeof(float2) + sizeof(int2) +
                         sizeof(float));
}

template <int CC>
__global__ void __launch_bounds__(256)
spread_patch_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ PatchSet ps,
                    const float2 *__restrict__ ks, const float *__restrict__ dens, int weighted,
                    float2 *__restrict__ grid)
{
    extern __shared__ float4 smem4[];
    constexpr int RS = SpreadRow<CC>::v;                  // value row stride (float2)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wi = blockIdx.x * 8 + warp;
    if (wi >= ps.nwork) return;
    const int taps = 2 * g.m + 2;
    const int WS = 2 * taps + 1;                          // padded weight row (conflict-free fill)
    char *base = reinterpret_cast<char *>(smem4) + warp * spread_patch_smem_per_warp<CC>(taps);
    float2 *sv = reinterpret_cast<float2 *>(base);        // [32][RS]
    float *sw = reinterpret_cast<float *>(sv + 32 * RS);  // [32][WS]
    int2 *su = reinterpret_cast<int2 *>(sw + 32 * WS);    // [32]
    float *sd = reinterpret_cast<float *>(su + 32);       // [32]
    const int c0 = blockIdx.y * CC;
    const int ccn = min(CC, g.nc - c0);
    const int4 wk = ps.work[wi];
    const int n0 = g.n[0], n1 = g.n[1];
    const int py = (wk.x / ps.npx) * kPatchH + (lane >> 3);
    const int px = (wk.x % ps.npx) * kPatchW + (lane & 7);
    const bool inside = (py < n0) && (px < n1);
    const bool wide = (n0 >= taps) && (n1 >= taps);       // no footprint wraps onto itself
    float ax[CC], ay[CC];
#pragma unroll
    for (int c = 0; c < CC; ++c) { ax[c] = 0.f; ay[c] = 0.f; }
    const int end = wk.y + wk.z;
    for (int e0 = wk.y; e0 < end; e0 += 32) {
        const int cnt = min(32, end - e0);
        // ---- stage: lane l fetches entry e0 + l ----
        if (lane < cnt) {
            const int s = ps.entries[e0 + lane];
            su[lane] = ps.nodeU[s];
            sd[lane] = weighted ? dens[s] : 1.f;
            const float2 *W2 = reinterpret_cast<const float2 *>(ps.nodeW + (size_t)s * 2 * taps);
            for (int q = 0; q < taps; ++q) {
                const float2 w = W2[q];
                sw[lane * WS + 2 * q] = w.x;
                sw[lane * WS + 2 * q + 1] = w.y;
            }
            const float2 *v = ks + (size_t)s * g.nc + c0;
#pragma unroll
            for (int c = 0; c < CC; ++c)
                sv[lane * RS + c] = (c < ccn) ? v[c] : make_float2(0.f, 0.f);
        }
        __syncwarp();
        // ---- accumulate ----
        for (int i = 0; i < cnt; ++i) {
            const int2 u = su[i];
            float w = 0.f;
            if (inside) {
                int dy = py - u.x; if (dy < 0) dy += n0;
                int dx = px - u.y; if (dx < 0) dx += n1;
                const float *W = sw + i * WS;
                float wy = 0.f, wx = 0.f;
                if (wide) {
                    wy = (dy < taps) ? W[dy] : 0.f;
                    wx = (dx < taps) ? W[taps + dx] : 0.f;
                } else {
                    for (int q = dy; q < taps; q += n0) wy += W[q];
                    for (int q = dx; q < taps; q += n1) wx += W[taps + q];
                }
                w = wy * wx * sd[i];
            }
            if constexpr ((CC & 1) == 0) {
                const float4 *v = reinterpret_cast<const float4 *>(sv + i * RS);
#pragma unroll
                for (int c = 0; c < CC / 2; ++c) {
                    const float4 q = v[c];
                    ax[2 * c] = fmaf(w, q.x, ax[2 * c]); ay[2 * c] = fmaf(w, q.y, ay[2 * c]);
                    ax[2 * c + 1] = fmaf(w, q.z, ax[2 * c + 1]); ay[2 * c + 1] = fmaf(w, q.w, ay[2 * c + 1]);
                }
            } else {
                const float2 *v = sv + i * RS;
#pragma unroll
                for (int c = 0; c < CC; ++c) {
                    const float2 q = v[c];
                    ax[c] = fmaf(w, q.x, ax[c]); ay[c] = fmaf(w, q.y, ay[c]);
                }
            }
        }
        __syncwarp();
    }
    if (!inside) return;
    float2 *dst = (wk.w < 0) ? grid + ((size_t)py * n1 + px) * g.nc + c0
                             : ps.partial + ((size_t)wk.w * 32 + lane) * g.nc + c0;
#pragma unroll
    for (int c = 0; c < CC; ++c)
        if (c < ccn) dst[c] = make_float2(ax[c], ay[c]);
}

// sum the partial slots of split patches in slot order and store them
__global__ void patch_reduce_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ PatchSet ps,
                                    float2 *__restrict__ grid)
{
    const int nc = g.nc;
    const int64_t total = (int64_t)ps.nmulti * 32 * nc;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(e % nc);
        const int lane = (int)((e / nc) % 32);
        const int4 mu = ps.multi[e / ((int64_t)32 * nc)];
        const int py = (mu.x / ps.npx) * kPatchH + (lane >> 3);
        const int px = (mu.x % ps.npx) * kPatchW + (lane & 7);
        if (py >= g.n[0] || px >= g.n[1]) continue;
        float sx = 0.f, sy = 0.f;
        for (int k = 0; k < mu.z; ++k) {
            const float2 v = ps.partial[((size_t)(mu.y + k) * 32 + lane) * nc + c];
            sx += v.x; sy += v.y;
        }
        grid[((size_t)py * g.n[1] + px) * nc + c] = make_float2(sx, sy);
    }
}

// ---------------------------------------------------------------------------
// 2-D interpolation with the coil index on the lanes.  A CTA stages the padded
// (T+2m+1)^2 tile of CC coils ([point][coil], coil innermost); a group of CC
// lanes serves one node, so every tap is one conflict-free read of CC
// consecutive complex values, and the node's 2 x TAPS weights (precomputed
// once per trajectory) sit in registers.
// ---------------------------------------------------------------------------
template <int TAPS, int CC>
__global__ void __launch_bounds__(256)
interp2_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ NodeSet ns,
               const int2 *__restrict__ nodeU, const float *__restrict__ nodeW,
               const float2 *__restrict__ grid, float2 *__restrict__ ks)
{
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
    constexpr int NPW = 32 / CC;           // nodes served by one warp at a time
    const int lane = threadIdx.x & 31, c = lane % CC, slot = lane / CC;
    const int warp = threadIdx.x >> 5;
    for (int i = warp * NPW + slot; i < wk.z; i += 8 * NPW) {
        const int64_t s = (int64_t)wk.y + i;
        const int2 u = nodeU[s];
        const int y0 = u.x - o0, x0 = u.y - o1;
        const float *W = nodeW + s * 2 * TAPS;
        float w0[TAPS], w1[TAPS];
#pragma unroll
        for (int q = 0; q < TAPS; ++q) { w0[q] = W[q]; w1[q] = W[TAPS + q]; }
        float ax = 0.f, ay = 0.f;
#pragma unroll
        for (int a = 0; a < TAPS; ++a) {
            const float2 *row = tile + ((y0 + a) * E + x0) * CC + c;
            float rx = 0.f, ry = 0.f;
#pragma unroll
            for (int b = 0; b < TAPS; ++b) {
                const float2 v = row[b * CC];
                rx = fmaf(w1[b], v.x, rx); ry = fmaf(w1[b], v.y, ry);
            }
            ax = fmaf(w0[a], rx, ax); ay = fmaf(w0[a], ry, ay);
        }
        if (c < ccn) ks[s * g.nc + c0 + c] = make_float2(ax, ay);
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
#define CGS_I2(CCV)                                                                                         \
    do {                                                                                                  \
        CGS_CUDA(cudaFuncSetAttribute(interp2_kernel<TAPS, CCV>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                      (int)smem));                                                         \
        interp2_kernel<TAPS, CCV><<<grd, 256, smem, st>>>(g, ns, ns.nodeU, ns.nodeW, grid, ks);            \
    } while (0)
    if (CC == 16) CGS_I2(16);
    else if (CC == 8) CGS_I2(8);
    else if (CC == 4) CGS_I2(4);
    else CGS_I2(1);
#undef CGS_I2
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_interp(const GridGeom &g, const NodeSet &ns, const float2 *grid, float2 *ks,
                         cudaStream_t st)
{
    if (ns.nwork == 0 || g.nc == 0) return CGS_OK;
    if (2 * g.m + 2 > kMaxTaps) { set_error("m too large"); return CGS_ERR_BAD_ARG; }
    const int taps = 2 * g.m + 2;
    if (g.d == 2 && ns.nodeU && ns.nodeW && taps <= 10) {
        // 8 coils per CTA by default: 40 KB tiles leave room for 4 CTAs per SM
        const int CC = g.icc > 0 ? g.icc : (g.nc >= 8 ? 8 : (g.nc >= 4 ? 4 : 1));
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

cgs_status launch_spread_patch(const GridGeom &g, const PatchSet &ps, const float2 *ks, const float *dens,
                               int weighted, float2 *grid, cudaStream_t st)
{
    if (ps.nwork == 0) return CGS_OK;
    const int CC = g.scc > 0 ? g.scc
                             : (g.nc >= 32 ? 32 : (g.nc >= 16 ? 16 : (g.nc >= 8 ? 8 : (g.nc >= 4 ? 4 : (g.nc >= 2 ? 2 : 1)))));
    const int taps = 2 * g.m + 2;
    if (taps > kMaxTaps) { set_error("m too large"); return CGS_ERR_BAD_ARG; }
    dim3 grd((ps.nwork + 7) / 8, (g.nc + CC - 1) / CC);
    prof_begin(PROF_SPREAD, st);
#define CGS_SP(CCV)                                                                                        \
    do {                                                                                                 \
        const size_t sm = 8 * spread_patch_smem_per_warp<CCV>(taps);                                     \
        CGS_CUDA(cudaFuncSetAttribute(spread_patch_kernel<CCV>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                      (int)sm));                                                          \
        spread_patch_kernel<CCV><<<grd, 256, sm, st>>>(g, ps, ks, dens, weighted, grid);                   \
    } while (0)
    switch (CC) {
        case 32: CGS_SP(32); break;
        case 16: CGS_SP(16); break;
        case 8: CGS_SP(8); break;
        case 4: CGS_SP(4); break;
        case 2: CGS_SP(2); break;
        default: CGS_SP(1); break;
    }
#undef CGS_SP
    CGS_LAUNCH_CHECK();
    if (ps.nmulti > 0) {
        const int64_t total = (int64_t)ps.nmulti * 32 * g.nc;
        const int64_t blocks = std::min<int64_t>((total + 255) / 256, 152 * 16);
        patch_reduce_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, ps, grid);
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
