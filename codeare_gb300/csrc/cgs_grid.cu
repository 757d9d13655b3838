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

template <int PH, int PW, int CPL>
struct SpreadShape {
    static constexpr int NPT = PH * PW;                        // points per patch
    static constexpr int G = 32 / NPT;                         // coil groups per warp
    static constexpr int CC = G * CPL;                         // coils per warp
    static constexpr int GS = (CPL % 2 == 0) ? CPL + 2 : CPL;  // group stride (float2): groups 16 B apart in banks
    static constexpr int VR = G * GS;                          // staged value row per entry (float2)
    static_assert(NPT * G == 32, "a patch must tile the warp");
    // one staging buffer: values, weights, footprint starts, density weights
    __host__ __device__ static size_t buf_bytes(int taps)
    {
        return (size_t)kSpreadBatch * (VR * sizeof(float2) + 2 * taps * sizeof(float) + sizeof(int2) + sizeof(float));
    }
};

template <int PH, int PW, int CPL>
__global__ void __launch_bounds__(256, 3)
spread_patch_kernel(const __grid_constant__ GridGeom g, const __grid_constant__ PatchSet ps,
                    const float2 *__restrict__ ks, const float *__restrict__ dens, int weighted,
                    float2 *__restrict__ grid)
{
    using S = SpreadShape<PH, PW, CPL>;
    extern __shared__ float4 smem4[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wi = blockIdx.x * 8 + warp;
    if (wi >= ps.nwork) return;
    const int taps = 2 * g.m + 2;
    const int WS = 2 * taps;                               // weights per entry (a multiple of 4)
    const size_t bb = S::buf_bytes(taps);
    char *wbase = reinterpret_cast<char *>(smem4) + (size_t)warp * 2 * bb;
    const int c0 = blockIdx.y * S::CC;
    const int ccn = min(S::CC, g.nc - c0);
    const bool v16 = ((g.nc & 1) == 0);                    // node rows 16-byte aligned: two coils per copy
    const int4 wk = ps.work[wi];
    const int n0 = g.n[0], n1 = g.n[1];
    const int pt = lane % S::NPT, cg = lane / S::NPT;
    const int py = (wk.x / ps.npx) * PH + pt / PW;
    const int px = (wk.x % ps.npx) * PW + pt % PW;
    const bool inside = (py < n0) && (px < n1);
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

    float2 acc[CPL];
#pragma unroll
    for (int k = 0; k < CPL; ++k) acc[k] = make_float2(0.f, 0.f);
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
            const float2 ww = make_float2(w, w);
            const float2 *vr = sv + i * S::VR + cg * S::GS;
            if constexpr (CPL % 2 == 0) {
                const float4 *v4 = reinterpret_cast<const float4 *>(vr);
#pragma unroll
                for (int k = 0; k < CPL / 2; ++k) {
                    const float4 q = v4[k];
                    acc[2 * k] = ffma2(ww, make_float2(q.x, q.y), acc[2 * k]);
                    acc[2 * k + 1] = ffma2(ww, make_float2(q.z, q.w), acc[2 * k + 1]);
                }
            } else {
#pragma unroll
                for (int k = 0; k < CPL; ++k) acc[k] = ffma2(ww, vr[k], acc[k]);
            }
        }
        __syncwarp();
        if (cnt1 <= 0) break;
        e0 = e1; cnt = cnt1; buf ^= 1;
    }
    if (!inside) return;
    const int cb = c0 + cg * CPL;                          // first coil of this lane's group
    float2 *dst = (wk.w < 0) ? grid + ((size_t)py * n1 + px) * g.nc + cb
                             : ps.partial + ((size_t)wk.w * S::NPT + pt) * g.nc + cb;
#pragma unroll
    for (int k = 0; k < CPL; ++k)
        if (cg * CPL + k < ccn) dst[k] = acc[k];
}

// sum the partial slots of split patches in slot order and store them
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
    const int taps = 2 * g.m + 2;
    if (taps > kMaxTaps) { set_error("m too large"); return CGS_ERR_BAD_ARG; }
    // coils per warp: the next power of two >= coils (at most 32), or the tuned value
    int CC = 1;
    if (ps.pw == 8) {
        CC = 1;
    } else {
        CC = 2;
        while (CC < g.nc && CC < 32) CC *= 2;
        if (g.scc > 0) CC = g.scc < 2 ? 2 : g.scc;
    }
    dim3 grd((ps.nwork + 7) / 8, (g.nc + CC - 1) / CC);
    prof_begin(PROF_SPREAD, st);
#define CGS_SP(PHV, PWV, CPLV)                                                                              \
    do {                                                                                                  \
        const size_t sm = 8 * 2 * SpreadShape<PHV, PWV, CPLV>::buf_bytes(taps);                           \
        CGS_CUDA(cudaFuncSetAttribute(spread_patch_kernel<PHV, PWV, CPLV>,                                 \
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));             \
        spread_patch_kernel<PHV, PWV, CPLV><<<grd, 256, sm, st>>>(g, ps, ks, dens, weighted, grid);        \
    } while (0)
    if (ps.pw == 8) {
        if (ps.ph != 4) { set_error("unsupported spreading patch"); return CGS_ERR_BAD_ARG; }
        CGS_SP(4, 8, 1);
    } else {
        if (ps.ph != 4 || ps.pw != 4) { set_error("unsupported spreading patch"); return CGS_ERR_BAD_ARG; }
        switch (CC) {
            case 32: CGS_SP(4, 4, 16); break;
            case 16: CGS_SP(4, 4, 8); break;
            case 8: CGS_SP(4, 4, 4); break;
            case 4: CGS_SP(4, 4, 2); break;
            default: CGS_SP(4, 4, 1); break;
        }
    }
#undef CGS_SP
    CGS_LAUNCH_CHECK();
    if (ps.nmulti > 0) {
        const int64_t total = (int64_t)ps.nmulti * ps.ph * ps.pw * g.nc;
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
