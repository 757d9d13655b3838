// cgs_vec.cu -- memory-bound vector kernels of the CG-SENSE path.
//
// Dot products take FP32 operands and accumulate in FP64 per thread, then in a
// fixed-shape block tree and a fixed-order final pass, so results do not depend
// on scheduling (the reference's dotc accumulates sequentially in
// complex<float>, src/matrix/linalg/Lapack.hpp:619-624).
#include "cgs_internal.cuh"

#include <algorithm>

namespace cgs {

namespace {

constexpr int kThreads = 256;
constexpr int kDotBlocks = 304;  // 2 x 152 SMs

// Caller layout (coil-major, trajectory order) <-> device layout (bin order,
// coil innermost) through 32 x 32 shared-memory tiles.  The gather
// (user[c][j] -> ks[iperm[j]][c]) reads 32 consecutive trajectory nodes of a
// coil and writes each node's run of coils at its sorted position; the
// scatter (ks[s][c] -> user[c][perm[s]]) reads contiguous coil runs and
// writes 32 sorted positions of a coil, whose trajectory indices come in runs
// (the bin sort is stable, so a spoke's consecutive samples stay together).
__global__ void gather_ks_kernel(const float2 *__restrict__ user, const int *__restrict__ iperm,
                                 int64_t M, int nc, float2 *__restrict__ ks)
{
    // 32 x 32 tiles of (coil, node in trajectory order): read along the
    // trajectory (coalesced), written as one contiguous run of the tile's
    // coils per node at the node's sorted position
    __shared__ float2 t[32][33];
    const int64_t tj_n = (M + 31) / 32, tc_n = (nc + 31) / 32;
    for (int64_t tile = blockIdx.x; tile < tj_n * tc_n; tile += gridDim.x) {
        const int64_t j0 = (tile / tc_n) * 32;
        const int c0 = (int)(tile % tc_n) * 32;
        const int64_t j = j0 + threadIdx.x;
        for (int k = threadIdx.y; k < 32; k += 8) {
            const int c = c0 + k;
            if (j < M && c < nc) t[k][threadIdx.x] = user[(int64_t)c * M + j];
        }
        __syncthreads();
        for (int k = threadIdx.y; k < 32; k += 8) {
            const int64_t jj = j0 + k;
            const int c = c0 + threadIdx.x;
            if (jj < M && c < nc) ks[(int64_t)iperm[jj] * nc + c] = t[threadIdx.x][k];
        }
        __syncthreads();
    }
}

// The same gather with 16-byte accesses (even M and coil count, 16-byte
// aligned buffers): tiles of 64 nodes x 32 coils; a warp reads a coil's 64
// consecutive nodes as 32 float4 (512 contiguous bytes) and writes two
// nodes' 32-coil runs (2 x 256 bytes) per instruction.
__global__ void gather_ks_v_kernel(const float2 *__restrict__ user, const int *__restrict__ iperm, int64_t M,
                                   int nc, float2 *__restrict__ ks)
{
    __shared__ float2 t[32][65];
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t tj_n = (M + 63) / 64, tc_n = (nc + 31) / 32;
    for (int64_t tile = blockIdx.x; tile < tj_n * tc_n; tile += gridDim.x) {
        const int64_t j0 = (tile / tc_n) * 64;
        const int c0 = (int)(tile % tc_n) * 32;
        const int64_t j = j0 + 2 * lane;
#pragma unroll
        for (int k = warp; k < 32; k += 8) {
            const int c = c0 + k;
            if (c < nc && j < M) {
                const float4 v = *reinterpret_cast<const float4 *>(user + (int64_t)c * M + j);
                t[k][2 * lane] = make_float2(v.x, v.y);
                t[k][2 * lane + 1] = make_float2(v.z, v.w);
            }
        }
        __syncthreads();
        const int q = lane & 15;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int jj = 16 * r + 2 * warp + (lane >> 4);
            const int c = c0 + 2 * q;
            if (j0 + jj < M && c < nc) {
                const float2 a = t[2 * q][jj], b2 = t[2 * q + 1][jj];
                *reinterpret_cast<float4 *>(ks + (int64_t)iperm[j0 + jj] * nc + c) = make_float4(a.x, a.y, b2.x, b2.y);
            }
        }
        __syncthreads();
    }
}

__global__ void scatter_ks_kernel(const float2 *__restrict__ ks, const int *__restrict__ perm,
                                  int64_t M, int nc, float2 *__restrict__ user)
{
    __shared__ float2 t[32][33];
    const int64_t ts_n = (M + 31) / 32, tc_n = (nc + 31) / 32;
    for (int64_t tile = blockIdx.x; tile < ts_n * tc_n; tile += gridDim.x) {
        const int64_t s0 = (tile / tc_n) * 32;
        const int c0 = (int)(tile % tc_n) * 32;
        for (int k = threadIdx.y; k < 32; k += 8) {
            const int64_t ss = s0 + k;
            const int c = c0 + threadIdx.x;
            if (ss < M && c < nc) t[k][threadIdx.x] = ks[ss * nc + c];
        }
        __syncthreads();
        const int64_t s = s0 + threadIdx.x;
        const int64_t j = s < M ? perm[s] : 0;
        for (int k = threadIdx.y; k < 32; k += 8) {
            const int c = c0 + k;
            if (s < M && c < nc) user[(int64_t)c * M + j] = t[threadIdx.x][k];
        }
        __syncthreads();
    }
}

// tiled transpose between (nc, P) and (P, nc): 32 x 32 tiles, a 1-D grid
// striding over all tiles (P can exceed the 65535 limit of a grid's y extent)
__global__ void transpose_kernel(const float2 *__restrict__ a, int64_t rows, int64_t cols,
                                 float2 *__restrict__ out)
{
    __shared__ float2 t[32][33];
    const int64_t tr_n = (rows + 31) / 32, tc_n = (cols + 31) / 32;
    for (int64_t tile = blockIdx.x; tile < tr_n * tc_n; tile += gridDim.x) {
        const int64_t r0 = (tile / tc_n) * 32, c0 = (tile % tc_n) * 32;
        for (int k = threadIdx.y; k < 32; k += 8) {
            const int64_t r = r0 + k, c = c0 + threadIdx.x;
            if (r < rows && c < cols) t[k][threadIdx.x] = a[r * cols + c];
        }
        __syncthreads();
        for (int k = threadIdx.y; k < 32; k += 8) {
            const int64_t c = c0 + k, r = r0 + threadIdx.x;
            if (r < rows && c < cols) out[c * rows + r] = t[threadIdx.x][k];
        }
        __syncthreads();
    }
}

// per-column partial dots; block b handles a contiguous row range
__global__ void __launch_bounds__(kThreads)
coldot_partial_kernel(const float2 *__restrict__ a, const float2 *__restrict__ b,
                      const float *__restrict__ wr, int64_t rows, int nc, double *__restrict__ partial)
{
    extern __shared__ double sred[];
    const int64_t per = (rows + gridDim.x - 1) / gridDim.x;
    const int64_t rbeg = (int64_t)blockIdx.x * per;
    const int64_t rend = min(rows, rbeg + per);
    // thread layout: column c = t % ncl, row lane = t / ncl, with ncl = min(nc, 256)
    const int ncl = nc < kThreads ? nc : kThreads;
    const int lanes = kThreads / ncl;
    const int t = threadIdx.x;
    const int lr = t / ncl;
    for (int cb = 0; cb < nc; cb += ncl) {
        const int c = cb + t % ncl;
        double acc = 0.0;
        if (lr < lanes && c < nc) {
            for (int64_t r = rbeg + lr; r < rend; r += lanes) {
                const float2 x = a[r * nc + c], y = b[r * nc + c];
                float v = fmaf(x.x, y.x, x.y * y.y);
                double dv = (double)v;
                if (wr) dv *= (double)wr[r];
                acc += dv;
            }
        }
        sred[t] = (lr < lanes) ? acc : 0.0;
        __syncthreads();
        // reduce over the row lanes of each column (fixed order)
        if (t < ncl) {
            double s = 0.0;
            for (int l = 0; l < lanes; ++l) s += sred[l * ncl + t];
            if (cb + t < nc) partial[(int64_t)blockIdx.x * nc + cb + t] = s;
        }
        __syncthreads();
    }
}

// one block per column: a fixed strided split of the block partials and a
// fixed tree (deterministic; a single thread per column would serialise on
// the load latency of nblk dependent adds)
__global__ void __launch_bounds__(kThreads)
coldot_final_kernel(const double *__restrict__ partial, int nblk, int nc, double *__restrict__ out)
{
    __shared__ double sred[kThreads];
    const int c = blockIdx.x;
    double s = 0.0;
    for (int b = threadIdx.x; b < nblk; b += kThreads) s += partial[(int64_t)b * nc + c];
    sred[threadIdx.x] = s;
    __syncthreads();
    for (int h = kThreads / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) sred[threadIdx.x] += sred[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = sred[0];
}

__global__ void cgnr_scalars_kernel(int mode, int nc, double eps, int *active, const double *dot_r,
                                    double *dot_z, const double *dot_v, const double *dz_new,
                                    double *alpha, double *beta)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    if (mode == 0) {
        active[c] = active[c] && !(dot_r[c] < eps);
    } else if (mode == 1) {
        alpha[c] = active[c] ? dot_z[c] / dot_v[c] : 0.0;
    } else {
        if (active[c]) {
            beta[c] = dz_new[c] / dot_z[c];
            dot_z[c] = dz_new[c];
        } else {
            beta[c] = 0.0;
        }
    }
}

// ---- fused per-coil steps of the batched CGNR inverse NFFT ------------------
// Per-column weighted squared norms of a [rows][nc] array, reduced in a fixed
// order: per block (thread column c = t % ncl, row lanes t / ncl, then the
// lanes in order) into partial[block][c]; the last block to finish (atomic
// ticket) adds the block partials per column in block order, one warp per
// column, and runs the scalar step of its coil.
//   MODE 1: dot_v = |ksV|_w^2;  alpha = active ? dot_z / dot_v : 0
//   MODE 2: img += alpha mask imgp (image side, no norm); vec -= alpha other;
//           dot_r = |vec|_w^2; active &= !(dot_r < eps)
//   MODE 3: dz_new = |cZ|_mask^2; beta = active ? dz_new / dot_z : 0, dot_z = dz_new
struct CgnrArgs {
    int64_t rows;
    int nc;
    const float *wr;       // row weights of the norm (nullable)
    float2 *vec;           // the array whose column norms are taken (MODE 2 updates it)
    const float2 *other;   // MODE 2: vec -= alpha * other
    float2 *img;           // MODE 2: image estimate [img_rows][nc]
    const float2 *imgp;    // MODE 2: search direction
    const float *mask;     // MODE 2: damping mask per image row
    int64_t img_rows;
    double *partial;       // [gridDim.x][nc]
    unsigned int *ticket;
    double *dot_r, *dot_z, *dot_v, *dz_new, *alpha, *beta;
    int *active;
    double eps;
};

template <int MODE>
__global__ void __launch_bounds__(kThreads) cgnr_fused_kernel(CgnrArgs a)
{
    __shared__ double sred[kThreads];
    __shared__ bool last;
    const int nc = a.nc, t = threadIdx.x;
    if (MODE == 2) {
        const int64_t total = a.img_rows * nc;
        for (int64_t e = blockIdx.x * (int64_t)blockDim.x + t; e < total; e += (int64_t)gridDim.x * blockDim.x) {
            const int64_t r = e / nc;
            const int c = (int)(e % nc);
            const double al = a.alpha[c];
            if (al == 0.0) continue;
            float sc = (float)al;
            if (a.mask) sc *= a.mask[r];
            const float2 v = a.imgp[e];
            float2 y = a.img[e];
            y.x = fmaf(sc, v.x, y.x); y.y = fmaf(sc, v.y, y.y);
            a.img[e] = y;
        }
    }
    const int64_t per = (a.rows + gridDim.x - 1) / gridDim.x;
    const int64_t rbeg = (int64_t)blockIdx.x * per;
    const int64_t rend = min(a.rows, rbeg + per);
    const int ncl = nc < kThreads ? nc : kThreads;
    const int lanes = kThreads / ncl;
    const int lr = t / ncl;
    for (int cb = 0; cb < nc; cb += ncl) {
        const int c = cb + t % ncl;
        double acc = 0.0;
        if (lr < lanes && c < nc) {
            const float ms = (MODE == 2) ? (float)(-a.alpha[c]) : 0.f;
            for (int64_t r = rbeg + lr; r < rend; r += lanes) {
                float2 x = a.vec[r * nc + c];
                if (MODE == 2 && ms != 0.f) {
                    const float2 o = a.other[r * nc + c];
                    x.x = fmaf(ms, o.x, x.x); x.y = fmaf(ms, o.y, x.y);
                    a.vec[r * nc + c] = x;
                }
                double dv = (double)fmaf(x.x, x.x, x.y * x.y);
                if (a.wr) dv *= (double)a.wr[r];
                acc += dv;
            }
        }
        sred[t] = (lr < lanes) ? acc : 0.0;
        __syncthreads();
        if (t < ncl) {
            double sum = 0.0;
            for (int l = 0; l < lanes; ++l) sum += sred[l * ncl + t];
            if (cb + t < nc) a.partial[(int64_t)blockIdx.x * nc + cb + t] = sum;
        }
        __syncthreads();
    }
    if (t == 0) {
        __threadfence();
        last = atomicAdd(a.ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int warp = t >> 5, lane = t & 31;
    for (int c = warp; c < nc; c += kThreads / 32) {
        double sum = 0.0;
        for (int b = lane; b < (int)gridDim.x; b += 32) sum += ((volatile double *)a.partial)[(int64_t)b * nc + c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
        if (lane == 0) {
            if (MODE == 1) {
                a.dot_v[c] = sum;
                a.alpha[c] = a.active[c] ? a.dot_z[c] / sum : 0.0;
            } else if (MODE == 2) {
                a.dot_r[c] = sum;
                a.active[c] = a.active[c] && !(sum < a.eps);
            } else {
                a.dz_new[c] = sum;
                if (a.active[c]) {
                    a.beta[c] = sum / a.dot_z[c];
                    a.dot_z[c] = sum;
                } else {
                    a.beta[c] = 0.0;
                }
            }
        }
    }
    if (t == 0) *a.ticket = 0u;
}

// ---- the same CGNR with A^H W A applied in image space -----------------------
// When codeare's inner CGNR runs on data y = A u (the CGLS step E^H(E p), u =
// S_c p), every quantity of NFFT3's loop is reachable from the image side
// through T = A^H W A (the Toeplitz kernel): z = A^H W r starts as T u and is
// updated as z -= alpha T(mask p); |r|_W^2 starts as Re <u, T u> and follows
// |r - alpha v|_W^2 = |r|_W^2 - 2 alpha Re <mask p, z> + alpha^2 |v|_W^2 with
// |v|_W^2 = Re <mask p, T(mask p)>.  Three fused kernels per step, each with
// two per-coil reductions in the fixed order of cgnr_fused_kernel:
//   MODE 0: dot_r = Re <S bimg, z>, dot_z = |z|_mask^2          (prologue)
//   MODE 1: dot_v = Re <mask p, g>, cross = Re <mask p, z>; alpha = active ?
//           dot_z / dot_v : 0; dot_r += alpha^2 dot_v - 2 alpha cross;
//           active &= !(dot_r < eps)                            (g = T(mask p))
//   MODE 2: img += alpha mask p, z -= alpha g, dz_new = |z|_mask^2;
//           beta = active ? dz_new / dot_z : 0, dot_z = dz_new
struct CgnrImgArgs {
    int64_t rows;
    int nc;
    const float *mask;      // damping mask per image row
    const float2 *bimg;     // MODE 0: the broadcast image p
    const float2 *sens;     // MODE 0: sensitivities [rows][nc]
    float2 *z;              // A^H W r per coil [rows][nc]
    const float2 *g;        // MODES 1, 2: T(mask p)
    const float2 *pv;       // MODES 1, 2: search direction
    float2 *img;            // MODE 2: the estimate
    double *partial, *partial2;
    unsigned int *ticket;
    double *dot_r, *dot_z, *dot_v, *dz_new, *alpha, *beta;
    int *active;
    double eps;
};

template <int MODE>
__global__ void __launch_bounds__(kThreads) cgnr_img_kernel(CgnrImgArgs a)
{
    __shared__ double sred[kThreads], sred2[kThreads];
    __shared__ bool last;
    const int nc = a.nc, t = threadIdx.x;
    const int64_t per = (a.rows + gridDim.x - 1) / gridDim.x;
    const int64_t rbeg = (int64_t)blockIdx.x * per;
    const int64_t rend = min(a.rows, rbeg + per);
    const int ncl = nc < kThreads ? nc : kThreads;
    const int lanes = kThreads / ncl;
    const int lr = t / ncl;
    for (int cb = 0; cb < nc; cb += ncl) {
        const int c = cb + t % ncl;
        double acc1 = 0.0, acc2 = 0.0;
        if (lr < lanes && c < nc) {
            const float al = (MODE == 2) ? (float)a.alpha[c] : 0.f;
            for (int64_t r = rbeg + lr; r < rend; r += lanes) {
                const int64_t e = r * nc + c;
                const float m = a.mask ? a.mask[r] : 1.f;
                if (MODE == 0) {
                    const float2 b = a.bimg[r], sv = a.sens[e], zv = a.z[e];
                    const float ux = sv.x * b.x - sv.y * b.y, uy = sv.x * b.y + sv.y * b.x;
                    acc1 += (double)fmaf(ux, zv.x, uy * zv.y);
                    acc2 += (double)m * (double)fmaf(zv.x, zv.x, zv.y * zv.y);
                } else if (MODE == 1) {
                    const float2 pv = a.pv[e], gv = a.g[e], zv = a.z[e];
                    acc1 += (double)m * (double)fmaf(pv.x, gv.x, pv.y * gv.y);
                    acc2 += (double)m * (double)fmaf(pv.x, zv.x, pv.y * zv.y);
                } else {
                    float2 zv = a.z[e];
                    if (al != 0.f) {
                        const float2 pv = a.pv[e], gv = a.g[e];
                        const float sm = al * m;
                        float2 y = a.img[e];
                        y.x = fmaf(sm, pv.x, y.x); y.y = fmaf(sm, pv.y, y.y);
                        a.img[e] = y;
                        zv.x = fmaf(-al, gv.x, zv.x); zv.y = fmaf(-al, gv.y, zv.y);
                        a.z[e] = zv;
                    }
                    acc1 += (double)m * (double)fmaf(zv.x, zv.x, zv.y * zv.y);
                }
            }
        }
        sred[t] = (lr < lanes) ? acc1 : 0.0;
        sred2[t] = (lr < lanes) ? acc2 : 0.0;
        __syncthreads();
        if (t < ncl) {
            double s1 = 0.0, s2 = 0.0;
            for (int l = 0; l < lanes; ++l) { s1 += sred[l * ncl + t]; s2 += sred2[l * ncl + t]; }
            if (cb + t < nc) {
                a.partial[(int64_t)blockIdx.x * nc + cb + t] = s1;
                a.partial2[(int64_t)blockIdx.x * nc + cb + t] = s2;
            }
        }
        __syncthreads();
    }
    if (t == 0) {
        __threadfence();
        last = atomicAdd(a.ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int warp = t >> 5, lane = t & 31;
    for (int c = warp; c < nc; c += kThreads / 32) {
        double s1 = 0.0, s2 = 0.0;
        for (int b = lane; b < (int)gridDim.x; b += 32) {
            s1 += ((volatile double *)a.partial)[(int64_t)b * nc + c];
            s2 += ((volatile double *)a.partial2)[(int64_t)b * nc + c];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s1 += __shfl_down_sync(0xffffffffu, s1, o);
            s2 += __shfl_down_sync(0xffffffffu, s2, o);
        }
        if (lane == 0) {
            if (MODE == 0) {
                a.dot_r[c] = s1;
                a.dot_z[c] = s2;
            } else if (MODE == 1) {
                a.dot_v[c] = s1;
                if (a.active[c]) {
                    const double al = a.dot_z[c] / s1;
                    a.alpha[c] = al;
                    a.dot_r[c] = a.dot_r[c] + al * al * s1 - 2.0 * al * s2;
                    a.active[c] = !(a.dot_r[c] < a.eps);
                } else {
                    a.alpha[c] = 0.0;
                }
            } else {
                a.dz_new[c] = s1;
                if (a.active[c]) {
                    a.beta[c] = s1 / a.dot_z[c];
                    a.dot_z[c] = s1;
                } else {
                    a.beta[c] = 0.0;
                }
            }
        }
    }
    if (t == 0) *a.ticket = 0u;
}

__global__ void axpy_cols_kernel(float2 *__restrict__ x, const double *__restrict__ alpha, double sgn,
                                 const float *__restrict__ mask, const float2 *__restrict__ p,
                                 int64_t rows, int nc)
{
    const int64_t total = rows * nc;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / nc;
        const int c = (int)(e % nc);
        const double a = sgn * alpha[c];
        if (a == 0.0) continue;
        float s = (float)a;
        if (mask) s *= mask[r];
        const float2 v = p[e];
        float2 y = x[e];
        y.x = fmaf(s, v.x, y.x); y.y = fmaf(s, v.y, y.y);
        x[e] = y;
    }
}

__global__ void xpby_cols_kernel(float2 *__restrict__ p, const float2 *__restrict__ z,
                                 const double *__restrict__ beta, const int *__restrict__ active,
                                 int64_t rows, int nc)
{
    const int64_t total = rows * nc;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(e % nc);
        if (active && !active[c]) continue;
        const float bb = (float)beta[c];
        const float2 v = z[e];
        float2 y = p[e];
        y.x = fmaf(bb, y.x, v.x); y.y = fmaf(bb, y.y, v.y);
        p[e] = y;
    }
}

__global__ void add_scaled_kernel(float2 *__restrict__ q, const float2 *__restrict__ p,
                                  const CGScalars *__restrict__ sc, int64_t n)
{
    if (sc->done) return;
    const float l = (float)sc->lambda;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x) {
        float2 a = q[e];
        const float2 b = p[e];
        a.x = fmaf(l, b.x, a.x); a.y = fmaf(l, b.y, a.y);
        q[e] = a;
    }
}

__global__ void cg_update_xr_kernel(float2 *__restrict__ x, float2 *__restrict__ r,
                                    const float2 *__restrict__ p, const float2 *__restrict__ q,
                                    CGScalars *__restrict__ sc, int64_t n)
{
    if (sc->done) return;
    const double tsd = sc->rn / sc->pq;
    const float ts = (float)tsd;
    if (blockIdx.x == 0 && threadIdx.x == 0) sc->ts = tsd;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x) {
        const float2 pv = p[e], qv = q[e];
        float2 xv = x[e], rv = r[e];
        xv.x = fmaf(ts, pv.x, xv.x); xv.y = fmaf(ts, pv.y, xv.y);
        rv.x = fmaf(-ts, qv.x, rv.x); rv.y = fmaf(-ts, qv.y, rv.y);
        x[e] = xv; r[e] = rv;
    }
}

__global__ void cg_update_p_kernel(float2 *__restrict__ p, const float2 *__restrict__ r,
                                   const CGScalars *__restrict__ sc, int64_t n)
{
    if (sc->done) return;
    const float bb = (float)(sc->rn / sc->rno);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x) {
        const float2 rv = r[e];
        float2 pv = p[e];
        pv.x = fmaf(bb, pv.x, rv.x); pv.y = fmaf(bb, pv.y, rv.y);
        p[e] = pv;
    }
}

// loop test of the CG-SENSE solvers on the device: records the residual
// measure, sets done; returns whether another iteration runs
__device__ unsigned int cg_check_logic(CGScalars *sc)
{
    unsigned int go = 0;
    if (!sc->done) {
        if (sc->iter >= sc->maxit) {
            sc->done = 1;
        } else if (sc->sqrt_mode && sc->xn == 0.0) {
            // zero right-hand side: x = 0 is the solution
            if (sc->iter < 256) sc->hist[sc->iter] = 0.0;
            sc->done = 1;
        } else {
            const double ratio = sc->rn / sc->xn;
            const double res = sc->sqrt_mode ? sqrt(ratio) : ratio;
            if (sc->iter < 256) sc->hist[sc->iter] = res;
            if (isnan(res)) { sc->nan_flag = 1; sc->done = 1; }
            else if (res <= sc->tol) { sc->done = 1; }
            else { sc->iter += 1; go = 1; }
        }
    }
    return go;
}

__global__ void cg_check_kernel(CGScalars *sc, cudaGraphConditionalHandle h)
{
    cudaGraphSetConditional(h, cg_check_logic(sc));
}

// ---- fused vector updates with a dot product --------------------------------
// Each block reduces its share in a fixed tree into partial[block]; the last
// block to finish (an atomic ticket) adds the partials in block order, so the
// value does not depend on scheduling, writes it and runs the loop's scalar
// step.  The grid is always kDotBlocks blocks.
__device__ __forceinline__ double block_reduce(double v, double *sred)
{
    __syncthreads();
    sred[threadIdx.x] = v;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sred[threadIdx.x] += sred[threadIdx.x + s];
        __syncthreads();
    }
    return sred[0];
}

// true in every thread of the last block, which then holds the total in *tot
__device__ __forceinline__ bool finish_reduce(double v, double *partial, unsigned int *ticket, double *tot)
{
    __shared__ double sred[kThreads];
    __shared__ bool last;
    const double bs = block_reduce(v, sred);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = bs;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double sum = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads) sum += ((volatile double *)partial)[b];
    const double t = block_reduce(sum, sred);
    if (threadIdx.x == 0) *ticket = 0u;
    *tot = t;
    return true;
}

// the same for two sums at once (partial_a and partial_b, gridDim.x each)
__device__ __forceinline__ bool finish_reduce2(double va, double vb, double *partial_a, double *partial_b,
                                               unsigned int *ticket, double *ta, double *tb)
{
    __shared__ double sred[kThreads];
    __shared__ bool last;
    const double ba = block_reduce(va, sred);
    const double bb = block_reduce(vb, sred);
    if (threadIdx.x == 0) {
        partial_a[blockIdx.x] = ba;
        partial_b[blockIdx.x] = bb;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double sa = 0.0, sb = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads) {
        sa += ((volatile double *)partial_a)[b];
        sb += ((volatile double *)partial_b)[b];
    }
    const double a = block_reduce(sa, sred);
    const double b = block_reduce(sb, sred);
    if (threadIdx.x == 0) *ticket = 0u;
    *ta = a;
    *tb = b;
    return true;
}

// q += lambda p (lambda nullable: no update), *out = Re <p, q>; skipped when *done
__global__ void __launch_bounds__(kThreads)
axpy_dot_kernel(float2 *__restrict__ q, const float2 *__restrict__ p, const double *lambda, const int *done,
                int64_t n, double *partial, unsigned int *ticket, double *out)
{
    if (done && *done) return;
    const float l = lambda ? (float)*lambda : 0.f;
    double acc = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        float2 a = q[e];
        const float2 b = p[e];
        if (lambda) {
            a.x = fmaf(l, b.x, a.x); a.y = fmaf(l, b.y, a.y);
            q[e] = a;
        }
        acc += (double)fmaf(b.x, a.x, b.y * a.y);
    }
    double t;
    if (finish_reduce(acc, partial, ticket, &t) && threadIdx.x == 0) *out = t;
}

// CG / CGLS: ts = rn / pq; x += ts p; r -= ts q; rno = rn, rn = |r|^2; loop test
__global__ void __launch_bounds__(kThreads)
cg_xr_rr_kernel(float2 *__restrict__ x, float2 *__restrict__ r, const float2 *__restrict__ p,
                const float2 *__restrict__ q, CGScalars *sc, int64_t n, double *partial, unsigned int *ticket,
                cudaGraphConditionalHandle h)
{
    if (sc->done) return;
    const double tsd = sc->rn / sc->pq;
    const float ts = (float)tsd;
    double acc = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float2 pv = p[e], qv = q[e];
        float2 xv = x[e], rv = r[e];
        xv.x = fmaf(ts, pv.x, xv.x); xv.y = fmaf(ts, pv.y, xv.y);
        rv.x = fmaf(-ts, qv.x, rv.x); rv.y = fmaf(-ts, qv.y, rv.y);
        x[e] = xv; r[e] = rv;
        acc += (double)fmaf(rv.x, rv.x, rv.y * rv.y);
    }
    double t;
    if (finish_reduce(acc, partial, ticket, &t) && threadIdx.x == 0) {
        sc->ts = tsd;
        sc->rno = sc->rn;
        sc->rn = t;
        cudaGraphSetConditional(h, cg_check_logic(sc));
    }
}

// ---- flexible CG ----------------------------------------------------------
__global__ void fcg_init_kernel(FCGScalars *fs)
{
    fs->rr0 = fs->rr;
    fs->best = fs->rr;
    fs->stall = 0;
    fs->restart = 1;
    fs->use_r = 0;
    fs->fallback_at = -1;
}

// stall bookkeeping on the new residual (network mode only): kStallChecks
// checks without a new best residual switch to plain CG (restarted)
constexpr int kStallChecks = 6;
__device__ __forceinline__ void fcg_decide_logic(FCGScalars *fs)
{
    if (fs->rr < fs->best) { fs->best = fs->rr; fs->stall = 0; }
    else fs->stall += 1;
    if ((fs->mode == 2 || fs->mode == 4) && !fs->fallback && fs->stall >= kStallChecks) {
        fs->fallback = 1;
        fs->restart = 1;
        fs->fallback_at = fs->cg.iter;
    }
}

__global__ void fcg_select_kernel(const FCGScalars *fs, float2 *__restrict__ z, const float2 *__restrict__ r, int64_t n)
{
    if (!fs->fallback && fs->mode != 0) return;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) z[e] = r[e];
}

// Polak-Ribiere beta from zr and zro, with the fallback when <z, r> <= 0
__device__ __forceinline__ void fcg_beta_logic(FCGScalars *fs)
{
    if ((fs->mode == 2 || fs->mode == 4) && !fs->fallback && !(fs->zr > 0.0)) {   // no descent direction
        fs->fallback = 1;
        fs->restart = 1;
        fs->use_r = 1;
        fs->fallback_at = fs->cg.iter;
    }
    const double zr = fs->use_r ? fs->rr : fs->zr;
    if (fs->restart) { fs->beta = 0.0; fs->restart = 0; }
    else fs->beta = (fs->zr - fs->zro) / fs->rz;
    fs->rz = zr;
}
__global__ void fcg_beta_kernel(FCGScalars *fs) { fcg_beta_logic(fs); }

// p = (use_r ? r : z) + beta p
__global__ void fcg_p_kernel(const FCGScalars *fs, float2 *__restrict__ p, const float2 *__restrict__ z,
                             const float2 *__restrict__ r, int64_t n)
{
    const float b = (float)fs->beta;
    const float2 *src = fs->use_r ? r : z;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float2 s = src[e];
        float2 pv = p[e];
        p[e] = make_float2(fmaf(b, pv.x, s.x), fmaf(b, pv.y, s.y));
    }
}

// residual check ||r|| / ||r0|| as the plain standard-mode loop
__device__ unsigned int fcg_check_logic(FCGScalars *fs)
{
    CGScalars *sc = &fs->cg;
    unsigned int go = 0;
    if (!sc->done) {
        if (sc->iter >= sc->maxit) {
            sc->done = 1;
        } else if (fs->rr0 == 0.0) {
            if (sc->iter < 256) sc->hist[sc->iter] = 0.0;
            sc->done = 1;
        } else {
            const double res = sqrt(fs->rr / fs->rr0);
            if (sc->iter < 256) sc->hist[sc->iter] = res;
            if (isnan(res)) { sc->nan_flag = 1; sc->done = 1; }
            else if (res <= sc->tol) { sc->done = 1; }
            else { sc->iter += 1; go = 1; }
        }
    }
    return go;
}

__global__ void fcg_check_kernel(FCGScalars *fs, cudaGraphConditionalHandle h)
{
    fs->use_r = 0;
    cudaGraphSetConditional(h, fcg_check_logic(fs));
}

// plain (mode 0), Jacobi (mode 1) and circulant (mode 3) loops, where z = M r
// with a fixed M: a = rz / pq; x += a p; r -= a q; rr = |r|^2; with csq also
// vc = csq . r (the circulant's input scaling).  Mode 0 (z = r) also takes the
// Fletcher-Reeves beta = rr / rz here and runs the loop test.
__global__ void __launch_bounds__(kThreads)
fcg_xr_rr_kernel(FCGScalars *fs, float2 *__restrict__ x, float2 *__restrict__ r, const float2 *__restrict__ p,
                 const float2 *__restrict__ q, int64_t n, double *partial, unsigned int *ticket,
                 cudaGraphConditionalHandle h, const float *__restrict__ csq, float2 *__restrict__ vc)
{
    const float a = (float)(fs->rz / fs->pq);
    double acc = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float2 pv = p[e], qv = q[e], rv = r[e];
        float2 xv = x[e];
        xv.x = fmaf(a, pv.x, xv.x); xv.y = fmaf(a, pv.y, xv.y);
        x[e] = xv;
        const float2 rn = make_float2(fmaf(-a, qv.x, rv.x), fmaf(-a, qv.y, rv.y));
        r[e] = rn;
        if (vc) { const float f = csq[e]; vc[e] = make_float2(rn.x * f, rn.y * f); }
        acc += (double)fmaf(rn.x, rn.x, rn.y * rn.y);
    }
    double t;
    if (finish_reduce(acc, partial, ticket, &t) && threadIdx.x == 0) {
        fs->rr = t;
        if (fs->mode == 0) {
            fs->zr = t;
            fs->beta = t / fs->rz;
            fs->rz = t;
            fs->use_r = 1;
            cudaGraphSetConditional(h, fcg_check_logic(fs));
        }
    }
}

// Jacobi loop: z = d^2 . r, zr = Re <z, r>, Fletcher-Reeves beta = zr / rz, loop test
__global__ void __launch_bounds__(kThreads)
fcg_jacobi_z_kernel(FCGScalars *fs, float2 *__restrict__ z, const float2 *__restrict__ r,
                    const float *__restrict__ d, int64_t n, double *partial, unsigned int *ticket,
                    cudaGraphConditionalHandle h)
{
    double acc = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        float f = d[e];
        f *= f;
        const float2 rv = r[e];
        const float2 zv = make_float2(rv.x * f, rv.y * f);
        z[e] = zv;
        acc += (double)fmaf(zv.x, rv.x, zv.y * rv.y);
    }
    double t;
    if (finish_reduce(acc, partial, ticket, &t) && threadIdx.x == 0) {
        fs->zr = t;
        fs->beta = t / fs->rz;
        fs->rz = t;
        fs->use_r = 0;
        cudaGraphSetConditional(h, fcg_check_logic(fs));
    }
}

// fixed preconditioner given z (or, with csq, z = csq . vc written here: the
// circulant's output scaling): zr = Re <z, r>, Fletcher-Reeves beta = zr / rz,
// loop test
__global__ void __launch_bounds__(kThreads)
fcg_zr_check_kernel(FCGScalars *fs, float2 *__restrict__ z, const float2 *__restrict__ r, int64_t n,
                    double *partial, unsigned int *ticket, cudaGraphConditionalHandle h, const float *__restrict__ csq,
                    const float2 *__restrict__ vc)
{
    double acc = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        float2 zv;
        if (csq) {
            const float f = csq[e];
            const float2 c = vc[e];
            zv = make_float2(c.x * f, c.y * f);
            z[e] = zv;
        } else {
            zv = z[e];
        }
        const float2 rv = r[e];
        acc += (double)fmaf(zv.x, rv.x, zv.y * rv.y);
    }
    double t;
    if (finish_reduce(acc, partial, ticket, &t) && threadIdx.x == 0) {
        fs->zr = t;
        fs->beta = t / fs->rz;
        fs->rz = t;
        fs->use_r = 0;
        cudaGraphSetConditional(h, fcg_check_logic(fs));
    }
}

// ---- flexible CG with a changing preconditioner (modes 2 and 4), fused ------
// alpha = rz / pq; x += alpha p; rold = r; r -= alpha q; rr = |r|^2; then the
// stall bookkeeping (the update, the rr dot and the decision in one kernel).
// The preconditioner's scaled copies of the new residual come out of the same
// pass: with csq, vc = csq . r (the circulant's input); with dsc, vt = dsc . r
// and fs->tt = |vt|^2 (the network's input and its scale; partial_b then
// holds the second sums).
__global__ void __launch_bounds__(kThreads)
fcg_xr_rr_decide_kernel(FCGScalars *fs, float2 *__restrict__ x, float2 *__restrict__ r, float2 *__restrict__ rold,
                        const float2 *__restrict__ p, const float2 *__restrict__ q, int64_t n, double *partial,
                        unsigned int *ticket, const float *__restrict__ csq, float2 *__restrict__ vc,
                        const float *__restrict__ dsc, float2 *__restrict__ vt, double *partial_b)
{
    const float a = (float)(fs->rz / fs->pq);
    double acc = 0.0, acc_t = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float2 pv = p[e], qv = q[e], rv = r[e];
        float2 xv = x[e];
        xv.x = fmaf(a, pv.x, xv.x); xv.y = fmaf(a, pv.y, xv.y);
        x[e] = xv;
        rold[e] = rv;
        const float2 rn = make_float2(fmaf(-a, qv.x, rv.x), fmaf(-a, qv.y, rv.y));
        r[e] = rn;
        acc += (double)fmaf(rn.x, rn.x, rn.y * rn.y);
        if (vc) { const float f = csq[e]; vc[e] = make_float2(rn.x * f, rn.y * f); }
        if (vt) {
            const float f = dsc[e];
            const float2 o = make_float2(rn.x * f, rn.y * f);
            vt[e] = o;
            acc_t += (double)fmaf(o.x, o.x, o.y * o.y);
        }
    }
    double t, tt;
    if (vt) {
        if (finish_reduce2(acc, acc_t, partial, partial_b, ticket, &t, &tt) && threadIdx.x == 0) {
            fs->rr = t;
            fs->tt = tt;
            fcg_decide_logic(fs);
        }
    } else if (finish_reduce(acc, partial, ticket, &t) && threadIdx.x == 0) {
        fs->rr = t;
        fcg_decide_logic(fs);
    }
}

// z = r where the loop has fallen back (fcg_select's rule), zr = Re <z, r>,
// zro = Re <z, rold>, then the Polak-Ribiere beta and the no-descent fallback
// (fcg_beta's rule).  Every block reads fs->fallback before the ticket; only
// the last block, after every ticket, may change it.  The two block sums go
// to partial_a and partial_b (kDotBlocks each) and are added in block order.
__global__ void __launch_bounds__(kThreads)
fcg_zsel_dots_beta_kernel(FCGScalars *fs, float2 *__restrict__ z, const float2 *__restrict__ r,
                          const float2 *__restrict__ rold, int64_t n, double *partial_a, double *partial_b,
                          unsigned int *ticket)
{
    const bool sel = fs->fallback || fs->mode == 0;
    double acc_r = 0.0, acc_o = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float2 rv = r[e], ov = rold[e];
        float2 zv;
        if (sel) { zv = rv; z[e] = zv; }
        else zv = z[e];
        acc_r += (double)fmaf(zv.x, rv.x, zv.y * rv.y);
        acc_o += (double)fmaf(zv.x, ov.x, zv.y * ov.y);
    }
    double ta, tb;
    if (finish_reduce2(acc_r, acc_o, partial_a, partial_b, ticket, &ta, &tb) && threadIdx.x == 0) {
        fs->zr = ta;
        fs->zro = tb;
        fcg_beta_logic(fs);
    }
}

// out = d . in and *nrm = |out|^2 (the network's input and its scale)
__global__ void __launch_bounds__(kThreads)
diag_scale_nrm_kernel(const float2 *__restrict__ in, const float *__restrict__ d, int64_t n, float2 *__restrict__ out,
                      double *partial, unsigned int *ticket, double *nrm)
{
    double acc = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float f = d[e];
        const float2 v = in[e];
        const float2 o = make_float2(v.x * f, v.y * f);
        out[e] = o;
        acc += (double)fmaf(o.x, o.x, o.y * o.y);
    }
    double t;
    if (finish_reduce(acc, partial, ticket, &t) && threadIdx.x == 0) *nrm = t;
}

// T. Chan fold of the 2N point-spread function onto the N-periodic grid
__global__ void circ_fold_kernel(const float2 *__restrict__ T, int N0, int N1, float2 *__restrict__ cN)
{
    const int64_t P = (int64_t)N0 * N1;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < P; e += (int64_t)gridDim.x * blockDim.x) {
        const int i0 = (int)(e / N1), i1 = (int)(e % N1);
        float sx = 0.f, sy = 0.f;
        for (int a = 0; a < 2; ++a) {
            const int j0 = i0 + a * N0;                   // index in T, offset d0 = j0 - N0
            const float w0 = fmaxf(0.f, 1.f - fabsf((float)(j0 - N0)) / (float)N0);
            for (int b = 0; b < 2; ++b) {
                const int j1 = i1 + b * N1;
                const float w = w0 * fmaxf(0.f, 1.f - fabsf((float)(j1 - N1)) / (float)N1);
                const float2 v = T[(int64_t)j0 * (2 * N1) + j1];
                sx = fmaf(w, v.x, sx); sy = fmaf(w, v.y, sy);
            }
        }
        cN[e] = make_float2(sx, sy);
    }
}

__global__ void coil_rsqrt_kernel(const float2 *__restrict__ S, int64_t P, int nc, float *__restrict__ csq)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < nc; ++c) {
            const float2 v = S[p * nc + c];
            s += (double)v.x * v.x + (double)v.y * v.y;
        }
        csq[p] = s > 0.0 ? (float)(1.0 / sqrt(s)) : 0.f;
    }
}

__global__ void circ_kinv_kernel(const float *__restrict__ spec, const FCGScalars *fs, int64_t P,
                                 float *__restrict__ kinv)
{
    const double mu = fs->dsum > 0.0 ? fs->cg.lambda * (double)P / fs->dsum : 0.0;   // lambda / mean sum|S|^2
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < P; e += (int64_t)gridDim.x * blockDim.x) {
        const double den = (double)P * ((double)spec[e] + mu);
        kinv[e] = den > 0.0 ? (float)(1.0 / den) : 0.f;
    }
}

__global__ void scale_add_kernel(float2 *out, const float2 *x, const float *__restrict__ dx, const float2 *y,
                                 const float *__restrict__ dy, int64_t n)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float a = dx ? dx[e] : 1.f;
        float2 v = x[e];
        v.x *= a; v.y *= a;
        if (y) {
            const float b = dy ? dy[e] : 1.f;
            const float2 u = y[e];
            v.x = fmaf(b, u.x, v.x); v.y = fmaf(b, u.y, v.y);
        }
        out[e] = v;
    }
}

// op 0: rn = xn = *src; 1: pq = *src; 2: rno = rn, rn = *src
__global__ void scalar_op_kernel(CGScalars *sc, const double *src, int op)
{
    if (op == 0) { sc->rn = *src; sc->xn = *src; }
    else if (op == 1) { sc->pq = *src; }
    else if (op == 2) { sc->rno = sc->rn; sc->rn = *src; }
}

__global__ void intensity_kernel(const float2 *__restrict__ S, int64_t P, int nc, float *__restrict__ I)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P;
         p += (int64_t)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int c = 0; c < nc; ++c) {
            const float2 v = S[p * nc + c];
            s = fmaf(v.x, v.x, fmaf(v.y, v.y, s));
        }
        I[p] = 1.f / (sqrtf(s) + 1.0e-9f);
    }
}

__global__ void coil_combine_kernel(const float2 *__restrict__ F, const float2 *__restrict__ S,
                                    const float *__restrict__ I, int64_t P, int nc, float2 *__restrict__ x)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P;
         p += (int64_t)gridDim.x * blockDim.x) {
        float ax = 0.f, ay = 0.f;
        for (int c = 0; c < nc; ++c) {
            const float2 f = F[p * nc + c], s = S[p * nc + c];
            // conj(s) * f
            ax = fmaf(s.x, f.x, fmaf(s.y, f.y, ax));
            ay = fmaf(s.x, f.y, fmaf(-s.y, f.x, ay));
        }
        const float g = I ? I[p] : 1.f;
        x[p] = make_float2(ax * g, ay * g);
    }
}

// The same combine with coalesced loads, for coil counts 2, 4, .., 64: L =
// nc / 2 lanes share a pixel, each loads two coils of F and S as one 16-byte
// vector, and the lanes' partial sums meet in a fixed shuffle tree (the
// same order on every run).  A warp reads 512 contiguous bytes of F and of S.
template <int L>
__global__ void __launch_bounds__(kThreads)
coil_combine_v_kernel(const float4 *__restrict__ F, const float4 *__restrict__ S, const float *__restrict__ I,
                      int64_t P, float2 *__restrict__ x)
{
    constexpr int PPW = 32 / L;   // pixels per warp and step
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t p0 = warp * PPW; p0 < P; p0 += nwarps * PPW) {   // warp-uniform loop
        const int64_t p = p0 + lane / L;
        float ax = 0.f, ay = 0.f;
        if (p < P) {
            const int64_t e = p * L + lane % L;
            const float4 f = F[e], s = S[e];
            ax = fmaf(s.x, f.x, fmaf(s.y, f.y, ax));          // conj(s) * f, coil 2q
            ay = fmaf(s.x, f.y, fmaf(-s.y, f.x, ay));
            ax = fmaf(s.z, f.z, fmaf(s.w, f.w, ax));          // coil 2q + 1
            ay = fmaf(s.z, f.w, fmaf(-s.w, f.z, ay));
        }
#pragma unroll
        for (int off = L / 2; off > 0; off >>= 1) {
            ax += __shfl_xor_sync(0xffffffffu, ax, off);
            ay += __shfl_xor_sync(0xffffffffu, ay, off);
        }
        if (p < P && lane % L == 0) {
            const float g = I ? I[p] : 1.f;
            x[p] = make_float2(ax * g, ay * g);
        }
    }
}

__global__ void scale_real_kernel(float2 *__restrict__ x, const float *__restrict__ s, int64_t n)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x) {
        const float f = s[e];
        float2 v = x[e];
        v.x *= f; v.y *= f;
        x[e] = v;
    }
}

unsigned grid_for(int64_t n)
{
    int64_t b = (n + kThreads - 1) / kThreads;
    if (b > 152 * 16) b = 152 * 16;
    if (b < 1) b = 1;
    return (unsigned)b;
}

}  // namespace

int dot_blocks() { return kDotBlocks; }

cgs_status launch_gather_ks(const float2 *user, const int *iperm, int64_t M, int nc, float2 *ks,
                            cudaStream_t st)
{
    if (M * nc == 0) return CGS_OK;
    if ((M & 1) == 0 && (nc & 1) == 0 && ((uintptr_t)user & 15) == 0 && ((uintptr_t)ks & 15) == 0) {
        const int64_t tiles = ((M + 63) / 64) * ((nc + 31) / 32);
        CGS_CUDA(launch_pdl(gather_ks_v_kernel, dim3((unsigned)std::min<int64_t>(tiles, 152 * 16)), dim3(256), 0, st,
                            user, iperm, M, nc, ks));
        return CGS_OK;
    }
    const int64_t tiles = ((M + 31) / 32) * ((nc + 31) / 32);
    gather_ks_kernel<<<(unsigned)std::min<int64_t>(tiles, 152 * 32), dim3(32, 8), 0, st>>>(user, iperm, M, nc, ks);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_scatter_ks(const float2 *ks, const int *perm, int64_t M, int nc, float2 *user,
                             cudaStream_t st)
{
    if (M * nc == 0) return CGS_OK;
    const int64_t tiles = ((M + 31) / 32) * ((nc + 31) / 32);
    scatter_ks_kernel<<<(unsigned)std::min<int64_t>(tiles, 152 * 32), dim3(32, 8), 0, st>>>(ks, perm, M, nc, user);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_to_coil_minor(const float2 *a, int64_t P, int nc, float2 *out, cudaStream_t st)
{
    // a: (nc rows, P cols) -> out: (P rows, nc cols)
    if (P * nc == 0) return CGS_OK;
    const int64_t tiles = ((P + 31) / 32) * ((nc + 31) / 32);
    transpose_kernel<<<(unsigned)std::min<int64_t>(tiles, 152 * 32), dim3(32, 8), 0, st>>>(a, nc, P, out);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_to_coil_major(const float2 *a, int64_t P, int nc, float2 *out, cudaStream_t st)
{
    if (P * nc == 0) return CGS_OK;
    const int64_t tiles = ((P + 31) / 32) * ((nc + 31) / 32);
    transpose_kernel<<<(unsigned)std::min<int64_t>(tiles, 152 * 32), dim3(32, 8), 0, st>>>(a, P, nc, out);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_axpy_dot(float2 *q, const float2 *p, const double *lambda, const int *done, int64_t n,
                           double *partial, unsigned int *ticket, double *out, cudaStream_t st)
{
    axpy_dot_kernel<<<kDotBlocks, kThreads, 0, st>>>(q, p, lambda, done, n, partial, ticket, out);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cg_xr_rr(float2 *x, float2 *r, const float2 *p, const float2 *q, CGScalars *sc, int64_t n,
                           double *partial, unsigned int *ticket, cudaGraphConditionalHandle h, cudaStream_t st)
{
    cg_xr_rr_kernel<<<kDotBlocks, kThreads, 0, st>>>(x, r, p, q, sc, n, partial, ticket, h);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_fcg_xr_rr(FCGScalars *fs, float2 *x, float2 *r, const float2 *p, const float2 *q, int64_t n,
                            double *partial, unsigned int *ticket, cudaGraphConditionalHandle h, cudaStream_t st,
                            const float *csq, float2 *vc)
{
    fcg_xr_rr_kernel<<<kDotBlocks, kThreads, 0, st>>>(fs, x, r, p, q, n, partial, ticket, h, csq, vc);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_fcg_jacobi_z(FCGScalars *fs, float2 *z, const float2 *r, const float *d, int64_t n,
                               double *partial, unsigned int *ticket, cudaGraphConditionalHandle h,
                               cudaStream_t st)
{
    fcg_jacobi_z_kernel<<<kDotBlocks, kThreads, 0, st>>>(fs, z, r, d, n, partial, ticket, h);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cgnr_fused(int mode, int64_t rows, int nc, const float *wr, float2 *vec, const float2 *other,
                             float2 *img, const float2 *imgp, const float *mask, int64_t img_rows, double *partial,
                             unsigned int *ticket, double *dots6, int *active, double eps, cudaStream_t st)
{
    CgnrArgs a;
    a.rows = rows; a.nc = nc; a.wr = wr; a.vec = vec; a.other = other;
    a.img = img; a.imgp = imgp; a.mask = mask; a.img_rows = img_rows;
    a.partial = partial; a.ticket = ticket;
    a.dot_r = dots6; a.dot_z = dots6 + nc; a.dot_v = dots6 + 2 * nc; a.dz_new = dots6 + 3 * nc;
    a.alpha = dots6 + 4 * nc; a.beta = dots6 + 5 * nc;
    a.active = active; a.eps = eps;
    if (mode == 1) cgnr_fused_kernel<1><<<kDotBlocks, kThreads, 0, st>>>(a);
    else if (mode == 2) cgnr_fused_kernel<2><<<kDotBlocks, kThreads, 0, st>>>(a);
    else cgnr_fused_kernel<3><<<kDotBlocks, kThreads, 0, st>>>(a);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cgnr_img(int mode, int64_t rows, int nc, const float *mask, const float2 *bimg,
                           const float2 *sens, float2 *z, const float2 *g, const float2 *pv, float2 *img,
                           double *partial, double *partial2, unsigned int *ticket, double *dots6, int *active,
                           double eps, cudaStream_t st)
{
    CgnrImgArgs a;
    a.rows = rows; a.nc = nc; a.mask = mask; a.bimg = bimg; a.sens = sens; a.z = z; a.g = g; a.pv = pv;
    a.img = img; a.partial = partial; a.partial2 = partial2; a.ticket = ticket;
    a.dot_r = dots6; a.dot_z = dots6 + nc; a.dot_v = dots6 + 2 * nc; a.dz_new = dots6 + 3 * nc;
    a.alpha = dots6 + 4 * nc; a.beta = dots6 + 5 * nc;
    a.active = active; a.eps = eps;
    if (mode == 0) cgnr_img_kernel<0><<<kDotBlocks, kThreads, 0, st>>>(a);
    else if (mode == 1) cgnr_img_kernel<1><<<kDotBlocks, kThreads, 0, st>>>(a);
    else cgnr_img_kernel<2><<<kDotBlocks, kThreads, 0, st>>>(a);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_coldot(const float2 *a, const float2 *b, const float *wr, int64_t rows, int nc,
                         double *partial, double *out, cudaStream_t st)
{
    coldot_partial_kernel<<<kDotBlocks, kThreads, kThreads * sizeof(double), st>>>(a, b, wr, rows, nc,
                                                                                  partial);
    CGS_LAUNCH_CHECK();
    coldot_final_kernel<<<nc, kThreads, 0, st>>>(partial, kDotBlocks, nc, out);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cgnr_scalars(int mode, int nc, double eps, int *active, const double *dot_r,
                               double *dot_z, const double *dot_v, const double *dz_new,
                               double *alpha, double *beta, cudaStream_t st)
{
    cgnr_scalars_kernel<<<(nc + 127) / 128, 128, 0, st>>>(mode, nc, eps, active, dot_r, dot_z, dot_v,
                                                         dz_new, alpha, beta);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_axpy_cols(float2 *x, const double *alpha, double alpha_sign, const float *mask,
                            const float2 *p, int64_t rows, int nc, cudaStream_t st)
{
    axpy_cols_kernel<<<grid_for(rows * nc), kThreads, 0, st>>>(x, alpha, alpha_sign, mask, p, rows, nc);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_xpby_cols(float2 *p, const float2 *z, const double *beta, const int *active,
                            int64_t rows, int nc, cudaStream_t st)
{
    xpby_cols_kernel<<<grid_for(rows * nc), kThreads, 0, st>>>(p, z, beta, active, rows, nc);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_zero(void *p, size_t bytes, cudaStream_t st)
{
    if (bytes) CGS_CUDA(cudaMemsetAsync(p, 0, bytes, st));
    return CGS_OK;
}

cgs_status launch_add_scaled(float2 *q, const float2 *p, const CGScalars *sc, int64_t n,
                             cudaStream_t st)
{
    add_scaled_kernel<<<grid_for(n), kThreads, 0, st>>>(q, p, sc, n);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cg_update_xr(float2 *x, float2 *r, const float2 *p, const float2 *q,
                               CGScalars *sc, int64_t n, cudaStream_t st)
{
    cg_update_xr_kernel<<<grid_for(n), kThreads, 0, st>>>(x, r, p, q, sc, n);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cg_update_p(float2 *p, const float2 *r, const CGScalars *sc, int64_t n,
                              cudaStream_t st)
{
    cg_update_p_kernel<<<grid_for(n), kThreads, 0, st>>>(p, r, sc, n);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_scalar_op(CGScalars *sc, const double *src, int op, cudaStream_t st)
{
    scalar_op_kernel<<<1, 1, 0, st>>>(sc, src, op);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

__global__ void jacobi_scale_kernel(const float2 *__restrict__ S, int64_t P, int nc, const FCGScalars *fs,
                                    float *__restrict__ d)
{
    const double sw = fs->sumw, lam = fs->cg.lambda;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < nc; ++c) {
            const float2 v = S[p * nc + c];
            s += (double)v.x * v.x + (double)v.y * v.y;
        }
        const double D = s * sw + lam;
        d[p] = D > 0.0 ? (float)(1.0 / sqrt(D)) : 0.f;
    }
}

__global__ void diag_scale_kernel(const float2 *in, const float2 *add, const float *__restrict__ d, int power,
                                  int64_t n, float2 *out)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        float f = d[e];
        if (power == 2) f *= f;
        float2 v = in[e];
        if (add) { const float2 a = add[e]; v.x += a.x; v.y += a.y; }
        out[e] = make_float2(v.x * f, v.y * f);
    }
}

cgs_status launch_jacobi_scale(const float2 *sens, int64_t P, int nc, const FCGScalars *fs, float *d,
                               cudaStream_t st)
{
    jacobi_scale_kernel<<<grid_for(P), kThreads, 0, st>>>(sens, P, nc, fs, d);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_diag_scale(const float2 *in, const float2 *add, const float *d, int power, int64_t n,
                             float2 *out, cudaStream_t st)
{
    diag_scale_kernel<<<grid_for(n), kThreads, 0, st>>>(in, add, d, power, n, out);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_fcg_zr_check(FCGScalars *fs, float2 *z, const float2 *r, int64_t n, double *partial,
                               unsigned int *ticket, cudaGraphConditionalHandle h, cudaStream_t st, const float *csq,
                               const float2 *vc)
{
    fcg_zr_check_kernel<<<kDotBlocks, kThreads, 0, st>>>(fs, z, r, n, partial, ticket, h, csq, vc);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_diag_scale_nrm(const float2 *in, const float *d, int64_t n, float2 *out, double *partial,
                                 unsigned int *ticket, double *nrm, cudaStream_t st)
{
    diag_scale_nrm_kernel<<<kDotBlocks, kThreads, 0, st>>>(in, d, n, out, partial, ticket, nrm);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_fcg_xr_rr_decide(FCGScalars *fs, float2 *x, float2 *r, float2 *rold, const float2 *p,
                                   const float2 *q, int64_t n, double *partial, unsigned int *ticket, cudaStream_t st,
                                   const float *csq, float2 *vc, const float *dsc, float2 *vt, double *partial_b)
{
    fcg_xr_rr_decide_kernel<<<kDotBlocks, kThreads, 0, st>>>(fs, x, r, rold, p, q, n, partial, ticket, csq, vc, dsc,
                                                             vt, partial_b);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_fcg_zsel_dots_beta(FCGScalars *fs, float2 *z, const float2 *r, const float2 *rold, int64_t n,
                                     double *partial_a, double *partial_b, unsigned int *ticket, cudaStream_t st)
{
    fcg_zsel_dots_beta_kernel<<<kDotBlocks, kThreads, 0, st>>>(fs, z, r, rold, n, partial_a, partial_b, ticket);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_circ_fold(const float2 *T, int N0, int N1, float2 *cN, cudaStream_t st)
{
    circ_fold_kernel<<<grid_for((int64_t)N0 * N1), kThreads, 0, st>>>(T, N0, N1, cN);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_coil_rsqrt(const float2 *sens, int64_t P, int nc, float *csq, cudaStream_t st)
{
    coil_rsqrt_kernel<<<grid_for(P), kThreads, 0, st>>>(sens, P, nc, csq);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_circ_kinv(const float *spec, const FCGScalars *fs, int64_t P, float *kinv, cudaStream_t st)
{
    circ_kinv_kernel<<<grid_for(P), kThreads, 0, st>>>(spec, fs, P, kinv);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_scale_add(float2 *out, const float2 *x, const float *dx, const float2 *y, const float *dy,
                            int64_t n, cudaStream_t st)
{
    scale_add_kernel<<<grid_for(n), kThreads, 0, st>>>(out, x, dx, y, dy, n);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_fcg_kernels(int which, FCGScalars *fs, float2 *x, float2 *r, float2 *rold, float2 *p,
                              const float2 *q, float2 *z, int64_t n, cudaGraphConditionalHandle h,
                              cudaStream_t st)
{
    switch (which) {
        case FCG_INIT: fcg_init_kernel<<<1, 1, 0, st>>>(fs); break;
        case FCG_SELECT: fcg_select_kernel<<<grid_for(n), kThreads, 0, st>>>(fs, z, r, n); break;
        case FCG_BETA: fcg_beta_kernel<<<1, 1, 0, st>>>(fs); break;
        case FCG_P: fcg_p_kernel<<<grid_for(n), kThreads, 0, st>>>(fs, p, z, r, n); break;
        default: fcg_check_kernel<<<1, 1, 0, st>>>(fs, h); break;
    }
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

__global__ void cg_init_kernel(CGScalars *sc, double lambda, double tol, int maxit, int sqrt_mode)
{
    for (int i = threadIdx.x; i < 256; i += blockDim.x) sc->hist[i] = 0.0;
    if (threadIdx.x == 0) {
        sc->rn = sc->xn = sc->rno = sc->pq = sc->ts = sc->beta = 0.0;
        sc->lambda = lambda;
        sc->done = 0;
        sc->tol = tol;
        sc->iter = 0;
        sc->maxit = maxit;
        sc->sqrt_mode = sqrt_mode;
        sc->nan_flag = 0;
    }
}

cgs_status launch_cg_init(CGScalars *sc, double lambda, double tol, int maxit, int sqrt_mode, cudaStream_t st)
{
    cg_init_kernel<<<1, 256, 0, st>>>(sc, lambda, tol, maxit, sqrt_mode);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_cg_check(CGScalars *sc, cudaGraphConditionalHandle h, cudaStream_t st)
{
    cg_check_kernel<<<1, 1, 0, st>>>(sc, h);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_intensity(const float2 *sens_cm, int64_t P, int nc, float *I, cudaStream_t st)
{
    intensity_kernel<<<grid_for(P), kThreads, 0, st>>>(sens_cm, P, nc, I);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_coil_combine(const float2 *F, const float2 *S, const float *I, int64_t P, int nc,
                               float2 *x, cudaStream_t st)
{
    const bool v16 = ((uintptr_t)F & 15) == 0 && ((uintptr_t)S & 15) == 0;
    const int L = nc / 2;
    if (v16 && nc >= 2 && nc <= 64 && (nc & (nc - 1)) == 0) {
        const float4 *F4 = reinterpret_cast<const float4 *>(F), *S4 = reinterpret_cast<const float4 *>(S);
        const unsigned blocks = grid_for(P * L);
        switch (L) {
            case 1: coil_combine_v_kernel<1><<<blocks, kThreads, 0, st>>>(F4, S4, I, P, x); break;
            case 2: coil_combine_v_kernel<2><<<blocks, kThreads, 0, st>>>(F4, S4, I, P, x); break;
            case 4: coil_combine_v_kernel<4><<<blocks, kThreads, 0, st>>>(F4, S4, I, P, x); break;
            case 8: coil_combine_v_kernel<8><<<blocks, kThreads, 0, st>>>(F4, S4, I, P, x); break;
            case 16: coil_combine_v_kernel<16><<<blocks, kThreads, 0, st>>>(F4, S4, I, P, x); break;
            default: coil_combine_v_kernel<32><<<blocks, kThreads, 0, st>>>(F4, S4, I, P, x); break;
        }
    } else {
        coil_combine_kernel<<<grid_for(P), kThreads, 0, st>>>(F, S, I, P, nc, x);
    }
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

cgs_status launch_scale_real(float2 *x, const float *s, int64_t n, cudaStream_t st)
{
    scale_real_kernel<<<grid_for(n), kThreads, 0, st>>>(x, s, n);
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}

}  // namespace cgs
