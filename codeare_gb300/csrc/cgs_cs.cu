// cgs_cs.cu -- compressed-sensing terms over the NCSENSE operator on sm_103a:
// the objective and gradient of codeare's CS_XSENSE (TV and L1 penalties,
// src/matrix/ft/CS_XSENSE.hpp:197-405) with the TV operators of
// src/matrix/TVOP.hpp, and the vector steps of its NLCG minimiser
// (src/optimisation/NLCG.hpp:84-125).
//
// Images are codeare-ordered (axis 0 fastest, extents D0, D1, D2).  Nothing
// TV-shaped is stored: each kernel takes its forward differences from the
// image on the fly (a 2-point stencil per axis), so one objective pass reads
// x and dx once for every TV term, the L1 term and all trial step sizes.
// Sums accumulate in FP64 per thread, then per block in a fixed order, then
// per column in a fixed order: every result is deterministic.
#include "cgs_internal.cuh"

namespace cgs {

namespace {

constexpr int kT = 256;

__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// Component c of the forward TV of u at (i0, i1, i2).  mode 1: TV2D (two
// components, TVOP.hpp:39-50); mode 2: TV3D over all axes as the reference
// computes it -- its third loop overwrites component 1 with the axis-2
// difference wherever that exists and leaves component 2 zero
// (TVOP.hpp:83-99); mode 3: axis-2 difference only (TVOP.hpp:135-144).
// Differences past the last index are zero.
__device__ __forceinline__ float2 tv_comp(const float2 *__restrict__ u, int mode, int c, int i0, int i1, int i2,
                                          const CsTerms &g)
{
    const float2 z = make_float2(0.f, 0.f);
    const int64_t s1 = g.D0, s2 = (int64_t)g.D0 * g.D1;
    const int64_t q = i0 + s1 * i1 + s2 * i2;
    if (mode == 3) return (i2 < g.D2 - 1) ? sub2(u[q + s2], u[q]) : z;
    if (c == 0) return (i0 < g.D0 - 1) ? sub2(u[q + 1], u[q]) : z;
    if (c == 1) {
        if (mode == 2 && i2 < g.D2 - 1) return sub2(u[q + s2], u[q]);
        return (i1 < g.D1 - 1) ? sub2(u[q + s1], u[q]) : z;
    }
    return z;
}

__device__ __forceinline__ int tv_ncomp(int mode) { return mode == 1 ? 2 : (mode == 2 ? 3 : 1); }

// (|v|^2 + l1)^e
__device__ __forceinline__ float pw(float2 v, float l1, float e) { return powf(fmaf(v.x, v.x, v.y * v.y) + l1, e); }

// p * v * (|v|^2 + l1)^(p/2 - 1), the pointwise factor of dTV (CS_XSENSE.hpp:395-402)
__device__ __forceinline__ float2 tv_g(float2 v, const CsTerms &g)
{
    const float f = pw(v, g.l1, 0.5f * g.pnorm - 1.0f);
    return make_float2(v.x * f * g.pnorm, v.y * f * g.pnorm);
}

__device__ __forceinline__ float2 tv_gc(const float2 *__restrict__ x, int mode, int c, int i0, int i1, int i2,
                                        const CsTerms &g)
{
    return tv_g(tv_comp(x, mode, c, i0, i1, i2, g), g);
}

// The reference's TV adjoint of G = tv_g(TV x) at one pixel: interior ranges
// only for modes 1 and 2 (TVOP.hpp:52-63, 101-118; square D0 == D1), the
// exact adjoint for mode 3 (TVOP.hpp:146-165).
__device__ float2 tv_adj_at(const float2 *__restrict__ x, int mode, int i0, int i1, int i2, const CsTerms &g)
{
    float2 r = make_float2(0.f, 0.f);
    if (mode == 3) {
        if (i2 >= 1 && i2 <= g.D2 - 2) {
            r = sub2(tv_gc(x, 3, 0, i0, i1, i2 - 1, g), tv_gc(x, 3, 0, i0, i1, i2, g));
        } else if (i2 == 0) {
            const float2 a = tv_gc(x, 3, 0, i0, i1, 0, g);
            r = make_float2(-a.x, -a.y);
        } else {
            r = tv_gc(x, 3, 0, i0, i1, g.D2 - 2, g);
        }
        return r;
    }
    if (i0 >= 1 && i0 <= g.D1 - 2) r = sub2(tv_gc(x, mode, 0, i0 - 1, i1, i2, g), tv_gc(x, mode, 0, i0, i1, i2, g));
    if (i1 >= 1 && i1 <= g.D0 - 2) {
        const float2 d = sub2(tv_gc(x, mode, 1, i0, i1 - 1, i2, g), tv_gc(x, mode, 1, i0, i1, i2, g));
        r.x += d.x;
        r.y += d.y;
    }
    if (mode == 2 && i2 >= 1 && i2 <= g.D2 - 2) {
        const float2 d = sub2(tv_gc(x, 2, 2, i0, i1, i2 - 1, g), tv_gc(x, 2, 2, i0, i1, i2, g));
        r.x += d.x;
        r.y += d.y;
    }
    return r;
}

// K sums of a block into partial[blockIdx.x * K + k], in a fixed order
template <int K>
__device__ __forceinline__ void block_sums(double (&acc)[K], double *__restrict__ partial)
{
    __shared__ double ws[K][kT / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) ws[k][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double s = 0.0;
#pragma unroll
        for (int i = 0; i < kT / 32; ++i) s += ws[threadIdx.x][i];
        partial[(int64_t)blockIdx.x * K + threadIdx.x] = s;
    }
}

// data term per step: sum |a + t b - y|^2 (t > 0), sum |a - y|^2 (t = 0)
// (CS_XSENSE.hpp:329-335)
__global__ void __launch_bounds__(kT) cs_obj_ks_kernel(const float2 *__restrict__ a, const float2 *__restrict__ b,
                                                       const float2 *__restrict__ y, int64_t n, CsSteps st,
                                                       double *__restrict__ partial)
{
    double acc[kCsSteps];
#pragma unroll
    for (int k = 0; k < kCsSteps; ++k) acc[k] = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT) {
        const float2 av = a[i], bv = b[i], yv = y[i];
#pragma unroll
        for (int k = 0; k < kCsSteps; ++k) {
            if (k < st.n) {
                const float t = st.t[k];
                float2 om = av;
                if (t > 0.f) om = make_float2(av.x + t * bv.x, av.y + t * bv.y);
                om = sub2(om, yv);
                acc[k] += (double)om.x * om.x + (double)om.y * om.y;
            }
        }
    }
    block_sums<kCsSteps>(acc, partial);
}

// TV and L1 terms per step (CS_XSENSE.hpp:337-365): for each TV term
// tvw * sum (|TV x + t TV dx|^2 + l1)^(p/2) over every component (zeros
// included), and xfmw * sum (|lx + t ldx|^2 + l1)^(p/2).  With a wavelet
// transform x, dx are the images and lx, ldx the NLCG variables (wavelet
// coefficients); without one they are the same arrays.
__global__ void __launch_bounds__(kT) cs_obj_img_kernel(const float2 *__restrict__ x, const float2 *__restrict__ dx,
                                                        const float2 *__restrict__ lx, const float2 *__restrict__ ldx,
                                                        CsTerms g, CsSteps st, double *__restrict__ partial)
{
    double acc[kCsSteps];
#pragma unroll
    for (int k = 0; k < kCsSteps; ++k) acc[k] = 0.0;
    const int64_t n = (int64_t)g.D0 * g.D1 * g.D2;
    const float e = 0.5f * g.pnorm;
    for (int64_t q = (int64_t)blockIdx.x * kT + threadIdx.x; q < n; q += (int64_t)gridDim.x * kT) {
        const int i0 = (int)(q % g.D0);
        const int64_t r = q / g.D0;
        const int i1 = (int)(r % g.D1), i2 = (int)(r / g.D1);
        for (int term = 0; term < 2; ++term) {
            const int mode = g.tvmode[term];
            if (!mode) continue;
            const float w = g.tvw[term];
            for (int c = 0; c < tv_ncomp(mode); ++c) {
                const float2 u = tv_comp(x, mode, c, i0, i1, i2, g), v = tv_comp(dx, mode, c, i0, i1, i2, g);
#pragma unroll
                for (int k = 0; k < kCsSteps; ++k) {
                    if (k < st.n) {
                        const float t = st.t[k];
                        const float2 om = t > 0.f ? make_float2(u.x + t * v.x, u.y + t * v.y) : u;
                        acc[k] += (double)w * pw(om, g.l1, e);
                    }
                }
            }
        }
        if (g.xfmw != 0.f) {
            const float2 u = lx[q], v = ldx[q];
#pragma unroll
            for (int k = 0; k < kCsSteps; ++k) {
                if (k < st.n) {
                    const float t = st.t[k];
                    const float2 om = t > 0.f ? make_float2(u.x + t * v.x, u.y + t * v.y) : u;
                    acc[k] += (double)g.xfmw * pw(om, g.l1, e);
                }
            }
        }
    }
    block_sums<kCsSteps>(acc, partial);
}

// (Re, Im) of sum conj(a) b
__global__ void __launch_bounds__(kT) cs_dot_kernel(const float2 *__restrict__ a, const float2 *__restrict__ b,
                                                    int64_t n, double *__restrict__ partial)
{
    double acc[2] = {0.0, 0.0};
    for (int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT) {
        const float2 u = a[i], v = b[i];
        acc[0] += (double)u.x * v.x + (double)u.y * v.y;
        acc[1] += (double)u.x * v.y - (double)u.y * v.x;
    }
    block_sums<2>(acc, partial);
}

// number of non-zero entries
__global__ void __launch_bounds__(kT) cs_nnz_kernel(const float2 *__restrict__ a, int64_t n,
                                                    double *__restrict__ partial)
{
    double acc[1] = {0.0};
    for (int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT) {
        const float2 u = a[i];
        if (u.x != 0.f || u.y != 0.f) acc[0] += 1.0;
    }
    block_sums<1>(acc, partial);
}

// out[c] = sum over blocks of partial[b * K + c], one block per column
__global__ void __launch_bounds__(kT) cs_colsum_kernel(const double *__restrict__ partial, int nblk, int K,
                                                       double *__restrict__ out)
{
    __shared__ double s[kT];
    const int c = blockIdx.x;
    double v = 0.0;
    for (int b = threadIdx.x; b < nblk; b += kT) v += partial[(int64_t)b * K + c];
    s[threadIdx.x] = v;
    __syncthreads();
    for (int h = kT / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = s[0];
}

// max |x| as float bits (non-negative floats order like their bit patterns)
__global__ void __launch_bounds__(kT) cs_absmax_kernel(const float2 *__restrict__ x, int64_t n,
                                                       unsigned int *__restrict__ out)
{
    float m = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT)
        m = fmaxf(m, hypotf(x[i].x, x[i].y));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// gradient (CS_XSENSE.hpp:223-232): g = 2 ehr + xfmw x (|x|^2 + l1)^(p/2-1)
//                                       + sum_i tvw_i TV_i^H G_i(TV_i x)
__global__ void __launch_bounds__(kT) cs_grad_kernel(const float2 *__restrict__ x, const float2 *__restrict__ ehr,
                                                     CsTerms g, float2 *__restrict__ out)
{
    const int64_t n = (int64_t)g.D0 * g.D1 * g.D2;
    for (int64_t q = (int64_t)blockIdx.x * kT + threadIdx.x; q < n; q += (int64_t)gridDim.x * kT) {
        const float2 e = ehr[q];
        float2 r = make_float2(2.0f * e.x, 2.0f * e.y);
        if (g.xfmw != 0.f) {
            const float2 u = x[q];
            const float f = pw(u, g.l1, 0.5f * g.pnorm - 1.0f);
            r.x += g.xfmw * (u.x * f);
            r.y += g.xfmw * (u.y * f);
        }
        const int i0 = (int)(q % g.D0);
        const int64_t rr = q / g.D0;
        const int i1 = (int)(rr % g.D1), i2 = (int)(rr / g.D1);
        for (int term = 0; term < 2; ++term) {
            const int mode = g.tvmode[term];
            if (!mode) continue;
            const float2 a = tv_adj_at(x, mode, i0, i1, i2, g);
            r.x += g.tvw[term] * a.x;
            r.y += g.tvw[term] * a.y;
        }
        out[q] = r;
    }
}

// g += xfmw x (|x|^2 + l1)^(p/2-1) (dXFM, CS_XSENSE.hpp:383-385)
__global__ void __launch_bounds__(kT) cs_l1grad_kernel(float2 *__restrict__ g, const float2 *__restrict__ x,
                                                       CsTerms t, int64_t n)
{
    for (int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT) {
        const float2 u = x[i];
        const float f = pw(u, t.l1, 0.5f * t.pnorm - 1.0f);
        float2 r = g[i];
        r.x += t.xfmw * (u.x * f);
        r.y += t.xfmw * (u.y * f);
        g[i] = r;
    }
}

// One pass of the periodic wavelet transform along one axis of the n x n
// top-left block of an ld x ld image (DWT.hpp:354-418 per level; filters
// along a line DWT.hpp:644-740): coefficient k < n/2 of a line is
// sum_h lo[h] s[(2k + h) mod n], coefficient n/2 + i is
// sum_h hi[h] s[(2i + 1 - h) mod n].  Thread per output value; axis 1 maps
// consecutive threads to consecutive columns so both axes coalesce.
__global__ void __launch_bounds__(kT) dwt_down_kernel(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                                      int ld, int n, int axis, DwtFilt f)
{
    const int64_t total = (int64_t)n * n;
    for (int64_t t = (int64_t)blockIdx.x * kT + threadIdx.x; t < total; t += (int64_t)gridDim.x * kT) {
        int line, k;
        if (axis == 0) { line = (int)(t / n); k = (int)(t % n); }
        else { k = (int)(t / n); line = (int)(t % n); }
        const int64_t base = axis == 0 ? (int64_t)line * ld : line;
        const int64_t step = axis == 0 ? 1 : ld;
        float2 s = make_float2(0.f, 0.f);
        if (k < n / 2) {
            for (int h = 0; h < f.fl; ++h) {
                int j = 2 * k + h;
                j %= n;
                const float2 v = src[base + j * step];
                s.x += f.lo[h] * v.x;
                s.y += f.lo[h] * v.y;
            }
        } else {
            const int i = k - n / 2;
            for (int h = 0; h < f.fl; ++h) {
                int j = (2 * i + 1 - h) % n;
                if (j < 0) j += n;
                const float2 v = src[base + j * step];
                s.x += f.hi[h] * v.x;
                s.y += f.hi[h] * v.y;
            }
        }
        dst[base + (int64_t)k * step] = s;
    }
}

// One inverse pass along one axis of the n2 x n2 top-left block (n2 = 2 *
// half; DWT.hpp:756-823 per level, DWT.hpp:1046-1180 along a line):
// out[2i + e] = sum_h lo[2h + e] low[(i - h) mod half]
//             + sum_h hi[2h + 1 - e] high[(i + h) mod half]
__global__ void __launch_bounds__(kT) dwt_up_kernel(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                                    int ld, int n2, int axis, DwtFilt f)
{
    const int64_t total = (int64_t)n2 * n2;
    const int half = n2 / 2, m2 = f.fl / 2;
    for (int64_t t = (int64_t)blockIdx.x * kT + threadIdx.x; t < total; t += (int64_t)gridDim.x * kT) {
        int line, m;
        if (axis == 0) { line = (int)(t / n2); m = (int)(t % n2); }
        else { m = (int)(t / n2); line = (int)(t % n2); }
        const int64_t base = axis == 0 ? (int64_t)line * ld : line;
        const int64_t step = axis == 0 ? 1 : ld;
        const int i = m >> 1, e = m & 1;
        float2 lo = make_float2(0.f, 0.f), hi = make_float2(0.f, 0.f);
        for (int h = 0; h < m2; ++h) {
            int j = (i - h) % half;
            if (j < 0) j += half;
            const float2 v = src[base + (int64_t)j * step];
            lo.x += f.lo[2 * h + e] * v.x;
            lo.y += f.lo[2 * h + e] * v.y;
        }
        for (int h = 0; h < m2; ++h) {
            const int j = (i + h) % half;
            const float2 v = src[base + (int64_t)(half + j) * step];
            hi.x += f.hi[2 * h + 1 - e] * v.x;
            hi.y += f.hi[2 * h + 1 - e] * v.y;
        }
        dst[base + (int64_t)m * step] = make_float2(lo.x + hi.x, lo.y + hi.y);
    }
}

__global__ void __launch_bounds__(kT) cs_axpy_kernel(float2 *__restrict__ x, const float2 *__restrict__ dx, float t,
                                                     int64_t n)
{
    for (int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT) {
        const float2 d = dx[i];
        float2 v = x[i];
        v.x += d.x * t;
        v.y += d.y * t;
        x[i] = v;
    }
}

// dx = -g1 + dx * (g1sq / g0sq), or dx = -g1 when g0sq is null
__global__ void __launch_bounds__(kT) cs_dir_kernel(float2 *__restrict__ dx, const float2 *__restrict__ g1,
                                                    const double *__restrict__ g1sq, const double *__restrict__ g0sq,
                                                    int64_t n)
{
    const float bk = g0sq ? (float)(*g1sq / *g0sq) : 0.f;
    for (int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT) {
        const float2 gv = g1[i];
        if (g0sq) {
            const float2 d = dx[i];
            dx[i] = make_float2(-gv.x + d.x * bk, -gv.y + d.y * bk);
        } else {
            dx[i] = make_float2(-gv.x, -gv.y);
        }
    }
}

__global__ void __launch_bounds__(kT) cs_sub_kernel(float2 *__restrict__ out, const float2 *__restrict__ a,
                                                    const float2 *__restrict__ b, int64_t n)
{
    for (int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT)
        out[i] = sub2(a[i], b[i]);
}

// acc[0] += solve iterations, acc[1] |= NaN flag (the loop scalars of one solve)
__global__ void cs_tally_kernel(const CGScalars *__restrict__ sc, int *__restrict__ acc)
{
    acc[0] += sc->iter;
    acc[1] |= sc->nan_flag;
}

int grid_for(int64_t n)
{
    const int64_t b = (n + kT - 1) / kT;
    return (int)(b < kCsBlocks ? (b > 0 ? b : 1) : kCsBlocks);
}

}  // namespace

cgs_status launch_cs_obj(const float2 *ksA, const float2 *ksB, const float2 *ksY, int64_t nks, const float2 *x,
                         const float2 *dx, const float2 *lx, const float2 *ldx, const CsTerms &terms,
                         const CsSteps &steps, double *partial, double *out, cudaStream_t st)
{
    const int gk = grid_for(nks);
    cs_obj_ks_kernel<<<gk, kT, 0, st>>>(ksA, ksB, ksY, nks, steps, partial);
    CGS_LAUNCH_CHECK();
    cs_colsum_kernel<<<kCsSteps, kT, 0, st>>>(partial, gk, kCsSteps, out);
    CGS_LAUNCH_CHECK();
    const int64_t nimg = (int64_t)terms.D0 * terms.D1 * terms.D2;
    const int gi = grid_for(nimg);
    double *pimg = partial + (int64_t)kCsBlocks * kCsSteps;
    cs_obj_img_kernel<<<gi, kT, 0, st>>>(x, dx, lx, ldx, terms, steps, pimg);
    CGS_LAUNCH_CHECK();
    cs_colsum_kernel<<<kCsSteps, kT, 0, st>>>(pimg, gi, kCsSteps, out + kCsSteps);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cs_dot(const float2 *a, const float2 *b, int64_t n, double *partial, double *out2,
                         cudaStream_t st)
{
    const int g = grid_for(n);
    cs_dot_kernel<<<g, kT, 0, st>>>(a, b, n, partial);
    CGS_LAUNCH_CHECK();
    cs_colsum_kernel<<<2, kT, 0, st>>>(partial, g, 2, out2);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cs_nnz(const float2 *a, int64_t n, double *partial, double *out, cudaStream_t st)
{
    const int g = grid_for(n);
    cs_nnz_kernel<<<g, kT, 0, st>>>(a, n, partial);
    CGS_LAUNCH_CHECK();
    cs_colsum_kernel<<<1, kT, 0, st>>>(partial, g, 1, out);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cs_absmax(const float2 *x, int64_t n, unsigned int *out, cudaStream_t st)
{
    CGS_CUDA(cudaMemsetAsync(out, 0, sizeof(unsigned int), st));
    cs_absmax_kernel<<<grid_for(n), kT, 0, st>>>(x, n, out);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cs_grad(const float2 *x, const float2 *ehr, const CsTerms &terms, float2 *g, cudaStream_t st)
{
    const int64_t n = (int64_t)terms.D0 * terms.D1 * terms.D2;
    cs_grad_kernel<<<grid_for(n), kT, 0, st>>>(x, ehr, terms, g);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cs_l1grad(float2 *g, const float2 *x, const CsTerms &terms, int64_t n, cudaStream_t st)
{
    cs_l1grad_kernel<<<grid_for(n), kT, 0, st>>>(g, x, terms, n);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_dwt_pass(const float2 *src, float2 *dst, int ld, int n, int axis, int inverse, const DwtFilt &f,
                           cudaStream_t st)
{
    const int64_t total = (int64_t)n * n;
    const int64_t b = (total + kT - 1) / kT;
    const int grid = (int)(b < 4 * kCsBlocks ? b : 4 * kCsBlocks);
    if (inverse) dwt_up_kernel<<<grid, kT, 0, st>>>(src, dst, ld, n, axis, f);
    else dwt_down_kernel<<<grid, kT, 0, st>>>(src, dst, ld, n, axis, f);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cs_axpy(float2 *x, const float2 *dx, float t, int64_t n, cudaStream_t st)
{
    cs_axpy_kernel<<<grid_for(n), kT, 0, st>>>(x, dx, t, n);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cs_dir(float2 *dx, const float2 *g1, const double *g1sq, const double *g0sq, int64_t n,
                         cudaStream_t st)
{
    cs_dir_kernel<<<grid_for(n), kT, 0, st>>>(dx, g1, g1sq, g0sq, n);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cs_sub(float2 *out, const float2 *a, const float2 *b, int64_t n, cudaStream_t st)
{
    cs_sub_kernel<<<grid_for(n), kT, 0, st>>>(out, a, b, n);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cs_tally(const CGScalars *sc, int *acc, cudaStream_t st)
{
    cs_tally_kernel<<<1, 1, 0, st>>>(sc, acc);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

}  // namespace cgs
