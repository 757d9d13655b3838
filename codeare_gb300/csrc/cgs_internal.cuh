// cgs_internal.cuh -- shared declarations of the sm_103a kernels and the plan.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/cgs.h"

namespace cgs {

// ---------------------------------------------------------------------------
// error plumbing (host)
// ---------------------------------------------------------------------------
void set_error(const std::string &msg);
void count_launch(int n = 1);

// Optional per-kernel timing with CUDA events on the launching stream
// (cgs_profile_enable / cgs_profile_collect).  Categories:
enum ProfCat { PROF_FFT = 0, PROF_INTERP = 1, PROF_SPREAD = 2, PROF_NCAT = 3 };
void prof_begin(int cat, cudaStream_t st);
void prof_end(int cat, cudaStream_t st);

#define CGS_CUDA(call)                                                              \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            ::cgs::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));  \
            return CGS_ERR_CUDA;                                                    \
        }                                                                           \
    } while (0)

#define CGS_LAUNCH_CHECK()                                                          \
    do {                                                                            \
        cudaError_t e_ = cudaGetLastError();                                        \
        if (e_ != cudaSuccess) {                                                    \
            ::cgs::set_error(std::string("kernel launch: ") + cudaGetErrorString(e_)); \
            return CGS_ERR_CUDA;                                                    \
        }                                                                           \
        ::cgs::count_launch();                                                      \
    } while (0)

#define CGS_TRY(expr)                         \
    do {                                      \
        cgs_status s_ = (expr);               \
        if (s_ != CGS_OK) return s_;          \
    } while (0)

// ---------------------------------------------------------------------------
// Kaiser-Bessel window, FP32 device version.
// phi(tau) = (b/pi) * sinh(z)/z,  z = b*sqrt(m^2 - tau^2)  (|tau| < m)
//          = (b/pi) * sin(z)/z,   z = b*sqrt(tau^2 - m^2)  (|tau| > m)
//          = b/pi                                           (|tau| = m)
// tau is the distance node - grid point in grid units.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float kb_phi(float tau, float m, float b)
{
    const float s2 = fmaf(-tau, tau, m * m);
    const float bp = b * 0.31830988618379067f;  // b/pi
    if (s2 > 0.f) {
        const float z = b * sqrtf(s2);
        if (z < 1e-3f) return bp * (1.f + z * z * (1.f / 6.f));
        const float E = expm1f(z);             // sinh(z) = E (2+E) / (2 (1+E))
        return bp * (0.5f * E * ((2.f + E) / (1.f + E))) / z;
    } else if (s2 < 0.f) {
        const float z = b * sqrtf(-s2);
        if (z < 1e-3f) return bp * (1.f - z * z * (1.f / 6.f));
        return bp * sinf(z) / z;
    }
    return bp;
}

// ---------------------------------------------------------------------------
// FFT axis pass descriptors
// ---------------------------------------------------------------------------
enum LoadMode : int {
    LOAD_PLAIN = 0,     // src[o][a][i]
    LOAD_IMAGE = 1,     // image-side first pass: img (broadcast or per-coil) * sens * mask * deapod
};
enum StoreMode : int {
    STORE_PLAIN = 0,    // dst[o][a][i]
    STORE_DEAPOD = 1,   // dst[o][a][i] * deapod(o,a)
    STORE_COMBINE = 2,  // out[o][a] = scale(o,a) * deapod * sum_i conj(S[o][a][i]) val_i
};

struct AxisPass {
    // geometry: data[outer][L][inner]; transform length n along L
    int64_t outer, inner;
    int n;            // FFT length
    int Lin, Lout;    // axis lengths of src and dst
    int in_centred;   // src axis is image side: index a holds frequency a - Lin/2 (pad into n)
    int out_centred;  // dst axis is image side: index a takes frequency a - Lout/2 (crop from n)
    int sign;         // -1 forward, +1 inverse
    const float2 *src;
    float2 *dst;
    const float2 *tw; // twiddles exp(-2 pi i t / n), t < n
    int nfac, fac[12];
    // fused image-side terms (first forward pass / last inverse pass)
    int load_mode, store_mode;
    const float2 *img;     // LOAD_IMAGE: image [outer][Lin] (broadcast) or [outer][Lin][inner]
    int img_per_coil;
    int64_t coil_major;    // nonzero: the per-coil images of a LOAD_IMAGE pass and the output of a
                           // STORE_DEAPOD pass are coil-major, img / dst[i * coil_major + pix]
    const float2 *sens;    // [outer][Lin|Lout][inner] sensitivities (coil innermost), nullable
    const float *mask;     // [outer][Lin] real pixel mask (nullable)
    const float *scale;    // STORE_COMBINE: per-pixel real scale (intensity map), nullable
    const float *deap_ax;  // 1/phihut along the axis, length N of the axis
    const float *deap_o1;  // 1/phihut along outer dim closest to the axis (2-D: y; 3-D: y)
    const float *deap_o0;  // 1/phihut along the outermost dim (3-D: z), nullable
    int o1_len;            // length of the o1 image dim (to split outer = o0 * o1_len + o1)
    int64_t combine_stride;// STORE_COMBINE output: out[o*Lout + a]
    float2 *combine_out;
    // Toeplitz: after the forward transform, multiply by a real kernel and
    // transform back (sign +1) before the store: K[pos][i / toep_nc] with
    // row stride inner / toep_nc (outer must be 1)
    const float *toep_k;
    int toep_nc;
};

cgs_status launch_axis_pass(const AxisPass &p, cudaStream_t st);

// Programmatic dependent launch.  A kernel launched by launch_pdl may start
// while the previous kernel on the stream finishes: it first does the work
// that reads only plan constants (twiddles, window tables, work lists, shared
// and tensor memory set-up), then pdl_wait() before it reads or writes any
// buffer that earlier work uses (the wait returns once the previous grid has
// completed and its memory is visible), and pdl_trigger() lets the next such
// kernel start.  Launched the ordinary way both are no-ops.  Stream capture
// and the legacy default stream get ordinary launches.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e;
    if (st == nullptr || cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        kern<<<grid, block, smem, st>>>(args...);
        e = cudaGetLastError();
    } else {
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = grid;
        cfg.blockDim = block;
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        e = cudaLaunchKernelEx(&cfg, kern, args...);
    }
    if (e == cudaSuccess) count_launch();   // the library's own launch count, as for CGS_LAUNCH_CHECK
    return e;
}

// ---------------------------------------------------------------------------
// Gridding (KB interpolation / spreading) over tiles of the oversampled grid
// ---------------------------------------------------------------------------
struct GridGeom {
    int d;            // 2 or 3
    int n[3];         // oversampled grid per dim (dim 0 slowest)
    int m;            // KB cut-off; 2m+2 taps per dim
    float b[3];       // KB shape per dim
    int T;            // tile side (footprint-start bins)
    int nt[3];        // tiles per dim
    int nc;           // coils (innermost in grid and k-space)
    int icc;          // coils per interpolation CTA (1, 4, 8, 16; 0 = automatic)
    int scc;          // coils per spreading warp (1, 2, 4, 8, 16, 32; 0 = automatic)
    int imma;         // interpolation on the tensor cores (needs the NodeSet's bin lists): 2-D 1 mma.sync on
                      // 4 x 4 bins, 2 tcgen05 on 8 x 16 bins; 3-D 1
};

constexpr int kInterpGroup = 16;     // tensor-core interpolation: nodes per warp (the m16)

struct NodeSet {
    int64_t M;          // nodes
    const float4 *nodes;// per node: 2-D {frac0, frac1, c0 bits, c1 bits}; 3-D two float4 per node
    const int *perm;    // sorted position -> original node index
    const float *w;     // density weights in sorted order (nullable)
    int nwork;          // work items
    const int4 *work;   // {tile index, first node, node count, 0}
    const int2 *nodeU;  // 2-D: per node wrapped footprint start (nullable)
    const float *nodeW; // 2-D: per node [2][2m+2] window weights (nullable)
    // 2-D tensor-core interpolation: sorted node indices grouped by the 4 x 4
    // bin of their footprint start, and work items {bin, first, count, 0}
    const int *ilist;
    const int4 *iwork;
    int niwork;
    int ibx;            // bins per grid row
    // 3-D tensor-core gridding: per node its wrapped footprint start
    // {u0, u1, u2, 0}; nodeW then holds kW3 window weights per node (3 x taps,
    // zero padded), and ilist / iwork group the nodes by 4 x 4 x 4 start bin
    const int4 *nodeU3;
    int iby;            // 3-D: bins per grid column (bins per plane = iby * ibx)
    int *err;           // set by a tensor-core kernel whose MMA wait ran out (nullable)
    // 2-D mma.sync interpolation: per work item its nodes' padded window rows
    // ([16][2][taps + 7] floats) and {node, footprint offsets in the bin}
    // (nullable: the kernel then builds them itself)
    const float *iwin;
    const int4 *imeta;
};
constexpr int kW3 = 32;  // floats per node in the 3-D window table

// Output-stationary 2-D spreading: one warp per work item over a ph x pw patch
// of grid points, its lanes split into coil groups (lane = one point or a 2 x 2
// block of points within its group), FP32 accumulators for the group's coils
// in registers, walking the list of nodes whose footprint covers the patch.
// Patches are 4 x 4 single points (two groups) for several coils, 4 x 4 of
// 2 x 1 or 4 x 8 of 2 x 2 blocks (four groups) when tuned so, and 4 x 8 single
// points for one coil.
struct PatchSet {
    int ph, pw;            // patch rows and columns
    int blk;               // 1: a point per lane; 2, 4: 2 x 1, 2 x 2 blocks; 8: 4 x 8 patch, one coil group;
                           // 16, 32: mma.sync on 4 x 4, 8 x 4 patches; 64: tcgen05 on 8 x 16 patches
    int npx;               // patches per grid row
    int nwork;             // work items
    const int *entries;    // node (sorted index) lists, patch after patch
    const int4 *work;      // {patch, first entry, count, partial slot or -1}
    const int2 *nodeU;     // per node: wrapped footprint start (u0, u1)
    const float *nodeW;    // per node: [2][2m+2] window weights
    float2 *partial;       // [slot][ph pw points][nc] partial sums of split patches
    int nmulti;            // patches split into several slots
    const int4 *multi;     // {patch, first slot, slots, 0}
    // 3-D (pd = 4): 4 x 4 x 4 patches, npy patches per grid column; node
    // starts in nodeU3 and kW3 window weights per node in nodeW; partial
    // slots hold 64 points each
    int pd, npy;
    const int4 *nodeU3;
    int *err;              // set by a tensor-core kernel whose MMA wait ran out (nullable)
    // tcgen05 spreading (blk 64): each work item's entries in blocks of 16
    // from block pstage[item]: the entries' patch weights ([24][16]: 8 row
    // then 16 column window values, entries innermost) and node indices
    // ([16], -1 past the list end)
    const float *pw16;
    const int *ps16;
    const int *pstage;
};
// node weights and footprint starts from the node records (once per trajectory)
cgs_status launch_node_weights(const GridGeom &g, const NodeSet &ns, int2 *nodeU, float *nodeW,
                               cudaStream_t st);
// grid[...][c] = sum_s phi * (w_s if weighted) * ks[s][c]; writes every grid point
cgs_status launch_spread_patch(const GridGeom &g, const PatchSet &ps, const float2 *ks, const float *dens,
                               int weighted, float2 *grid, cudaStream_t st);
// the tcgen05 spreading's per-block patch weights and node indices (once per
// trajectory and work list); pw16 / ps16 sized by the blocks of ps.pstage
cgs_status launch_spread_tc_weights(const GridGeom &g, const PatchSet &ps, float *pw16, int *ps16, cudaStream_t st);

// 3-D node tables: wrapped footprint starts and kW3 window weights per node
cgs_status launch_node_weights3(const GridGeom &g, const NodeSet &ns, int4 *nodeU3, float *nodeW,
                                cudaStream_t st);
// 3-D output-stationary spreading over 4 x 4 x 4 patches (writes every grid point)
cgs_status launch_spread_patch3(const GridGeom &g, const PatchSet &ps, const float2 *ks, const float *dens,
                                int weighted, float2 *grid, cudaStream_t st);
// whether the 3-D tensor-core gridding covers this geometry (taps <= 10, every side >= 3 + taps)
bool grid3_mma_ok(const GridGeom &g);

// y[s][c] (sorted, coil innermost) = sum over footprint of grid[...][c]
// With `user` (the caller's layout: coil-major, trajectory order) the
// tensor-core kernel writes there directly and sets *wrote_user; otherwise
// the result is in ks and the caller scatters it.
// the 2-D mma.sync interpolation's per-work-item window blocks (once per trajectory)
cgs_status launch_interp_windows(const GridGeom &g, const NodeSet &ns, float *iwin, int4 *imeta, cudaStream_t st);
cgs_status launch_interp(const GridGeom &g, const NodeSet &ns, const float2 *grid, float2 *ks,
                         cudaStream_t st, float2 *user = nullptr, bool *wrote_user = nullptr);
// grid[...][c] += sum_s phi * (w_s if weighted) * ks[s][c]; grid must be zeroed first
cgs_status launch_spread(const GridGeom &g, const NodeSet &ns, const float2 *ks, int weighted,
                         float2 *grid, cudaStream_t st);

// ---------------------------------------------------------------------------
// vector kernels (cgs_vec.cu)
// ---------------------------------------------------------------------------
// user (NC, M) coil-major unsorted  <->  ks[s][c] sorted coil-minor
// (gather: iperm[j] = sorted position of trajectory node j; scatter: perm[s] =
// trajectory node at sorted position s)
cgs_status launch_gather_ks(const float2 *user, const int *iperm, int64_t M, int nc, float2 *ks,
                            cudaStream_t st);
cgs_status launch_scatter_ks(const float2 *ks, const int *perm, int64_t M, int nc, float2 *user,
                             cudaStream_t st);
// coil-major (NC, P) <-> coil-minor [P][NC]
cgs_status launch_to_coil_minor(const float2 *a, int64_t P, int nc, float2 *out, cudaStream_t st);
cgs_status launch_to_coil_major(const float2 *a, int64_t P, int nc, float2 *out, cudaStream_t st);

// Deterministic FP64-accumulated per-column dots over rows:
// out[c] = sum_r wr[r] * Re(conj(a[r][c]) * b[r][c]), wr nullable (1).
// partial must hold nblk*nc doubles (nblk = dot_blocks()).
int dot_blocks();
cgs_status launch_coldot(const float2 *a, const float2 *b, const float *wr, int64_t rows, int nc,
                         double *partial, double *out, cudaStream_t st);

// scalar CG bookkeeping on device (one thread per coil)
// mode 0: CGNR start of step: active[c] &= (dot_r[c] >= eps)
// mode 1: alpha[c] = active ? dot_z[c] / dot_v[c] : 0
// mode 2: beta[c] = active ? dz_new/dot_z : 0; dot_z = active ? dz_new : dot_z
cgs_status launch_cgnr_scalars(int mode, int nc, double eps, int *active, const double *dot_r,
                               double *dot_z, const double *dot_v, const double *dz_new,
                               double *alpha, double *beta, cudaStream_t st);

// per-column update kernels (coil-minor [rows][nc])
// x[r][c] += alpha[c] * (mask? mask[r] : 1) * p[r][c]
cgs_status launch_axpy_cols(float2 *x, const double *alpha, double alpha_sign, const float *mask,
                            const float2 *p, int64_t rows, int nc, cudaStream_t st);
// p[r][c] = z[r][c] + beta[c] * p[r][c]   (only where active[c])
cgs_status launch_xpby_cols(float2 *p, const float2 *z, const double *beta, const int *active,
                            int64_t rows, int nc, cudaStream_t st);
cgs_status launch_zero(void *p, size_t bytes, cudaStream_t st);

// CGLS (single image) kernels: scalars live in a small device struct
struct CGScalars {
    double rn, xn, rno, pq, ts, beta, lambda;
    int done;
    // device-driven loop control
    double tol;          // break when the residual measure <= tol
    int iter, maxit;     // updates made / allowed
    int sqrt_mode;       // residual measure: 0 rn/xn (codeare), 1 sqrt(rn/xn)
    int nan_flag;
    double hist[256];    // residual measure per check
};
// Flexible CG (preconditioner may change per iteration): Polak-Ribiere beta,
// fallback to plain CG when the residual stalls or <r, z> <= 0.
struct FCGScalars {
    CGScalars cg;        // lambda, done, iter, maxit, tol, hist, nan_flag
    double rr, rr0, rz, pq, zr, zro, beta, best;
    int stall, fallback, use_r, restart, fallback_at;
    int mode;            // 0 plain, 1 Jacobi, 2 scaled network, 3 circulant, 4 circulant + network
    double sumw, tt;     // sum of the density weights; |d . r|^2 for the net
    double dsum;         // sum over pixels and coils of |S|^2 (the circulant's lambda scale)
};
cgs_status launch_fcg_kernels(int which, FCGScalars *fs, float2 *x, float2 *r, float2 *rold, float2 *p,
                              const float2 *q, float2 *z, int64_t n, cudaGraphConditionalHandle h,
                              cudaStream_t st);
enum FcgOp { FCG_INIT = 0, FCG_SELECT = 3, FCG_BETA = 4, FCG_P = 5, FCG_CHECK = 6 };
// flexible-CG loop with a fixed preconditioner (mode 0 plain, 1 Jacobi):
// x, r update and rr (mode 0 also beta and the loop test); z = d^2 r, zr, beta, loop test
// (mode 3: with csq also vc = csq . r, the circulant's input)
cgs_status launch_fcg_xr_rr(FCGScalars *fs, float2 *x, float2 *r, const float2 *p, const float2 *q, int64_t n,
                            double *partial, unsigned int *ticket, cudaGraphConditionalHandle h, cudaStream_t st,
                            const float *csq = nullptr, float2 *vc = nullptr);
cgs_status launch_fcg_jacobi_z(FCGScalars *fs, float2 *z, const float2 *r, const float *d, int64_t n,
                               double *partial, unsigned int *ticket, cudaGraphConditionalHandle h,
                               cudaStream_t st);
// d[p] = 1/sqrt(sum_c |S[p][c]|^2 * sumw + lambda) from the coil-minor sensitivities
cgs_status launch_jacobi_scale(const float2 *sens, int64_t P, int nc, const FCGScalars *fs, float *d,
                               cudaStream_t st);
// out = d^power . (in + add) (power 1 or 2; add may be null), the diagonal
// scaling steps of the preconditioner
cgs_status launch_diag_scale(const float2 *in, const float2 *add, const float *d, int power, int64_t n,
                             float2 *out, cudaStream_t st);
// codeare's inner CGNR with A^H W A applied in image space (cgs_vec.cu,
// cgnr_img_kernel): mode 0 the prologue dots, 1 alpha and the residual-norm
// recurrence after g = T(mask p), 2 the image / z updates and beta.  partial
// and partial2 hold kDotBlocks x nc doubles each.
cgs_status launch_cgnr_img(int mode, int64_t rows, int nc, const float *mask, const float2 *bimg,
                           const float2 *sens, float2 *z, const float2 *g, const float2 *pv, float2 *img,
                           double *partial, double *partial2, unsigned int *ticket, double *dots6, int *active,
                           double eps, cudaStream_t st);
// circulant preconditioner (2-D): the T. Chan fold of the 2N point-spread
// function T[2N0][2N1] (index d + N) onto the N-periodic grid,
//   cN[d mod N] = sum (1 - |d0|/N0)(1 - |d1|/N1) T[d]
cgs_status launch_circ_fold(const float2 *T, int N0, int N1, float2 *cN, cudaStream_t st);
// csq[p] = 1 / sqrt(sum_c |S[p][c]|^2) (0 where the coils vanish)
cgs_status launch_coil_rsqrt(const float2 *sens, int64_t P, int nc, float *csq, cudaStream_t st);
// kinv = 1 / (P (spec + lambda P / dsum)): the spectrum of the inverse circulant,
// with the 1/P of the unnormalised FFT pair folded in
cgs_status launch_circ_kinv(const float *spec, const FCGScalars *fs, int64_t P, float *kinv, cudaStream_t st);
// out = dx . x + (y ? (dy ? dy . y : y) : 0), real per-pixel factors
cgs_status launch_scale_add(float2 *out, const float2 *x, const float *dx, const float2 *y, const float *dy,
                            int64_t n, cudaStream_t st);
// out = d . in and *nrm = sum |out|^2 (partial: dot_blocks() doubles)
cgs_status launch_diag_scale_nrm(const float2 *in, const float *d, int64_t n, float2 *out, double *partial,
                                 unsigned int *ticket, double *nrm, cudaStream_t st);
// flexible-CG loop with a changing preconditioner (modes 2 and 4), two fused
// steps around z = M(r): x, rold, r update with rr and the stall bookkeeping;
// then z = r after a fallback, zr and zro (partials in partial_a and partial_b,
// dot_blocks() each) and the Polak-Ribiere beta
// (with csq also vc = csq . r; with dsc also vt = dsc . r and fs->tt = |vt|^2,
// whose block sums go to partial_b)
cgs_status launch_fcg_xr_rr_decide(FCGScalars *fs, float2 *x, float2 *r, float2 *rold, const float2 *p,
                                   const float2 *q, int64_t n, double *partial, unsigned int *ticket, cudaStream_t st,
                                   const float *csq = nullptr, float2 *vc = nullptr, const float *dsc = nullptr,
                                   float2 *vt = nullptr, double *partial_b = nullptr);
cgs_status launch_fcg_zsel_dots_beta(FCGScalars *fs, float2 *z, const float2 *r, const float2 *rold, int64_t n,
                                     double *partial_a, double *partial_b, unsigned int *ticket, cudaStream_t st);
// fixed-preconditioner loop: zr = Re <z, r>, Fletcher-Reeves beta = zr / rz, loop test
// (with csq, z = csq . vc is formed and written first: the circulant's output)
cgs_status launch_fcg_zr_check(FCGScalars *fs, float2 *z, const float2 *r, int64_t n, double *partial,
                               unsigned int *ticket, cudaGraphConditionalHandle h, cudaStream_t st,
                               const float *csq = nullptr, const float2 *vc = nullptr);
// z = M(r): the learned preconditioner on one complex image (cgs_cnn.cu);
// nrm2 = sum |r|^2 on the device sets the input scale
uint64_t net_serial(const cgs_net *n);   // 0 for null, else unique per created network
cgs_status net_apply_image(cgs_net *n, const float2 *r, const double *nrm2, int H, int W, float2 *z,
                           cudaStream_t st);
// the same with the output step z = dsc . net(r) + csq . vc in one kernel
cgs_status net_apply_image_combine(cgs_net *n, const float2 *r, const double *nrm2, int H, int W, const float *dsc,
                                   const float *csq, const float2 *vc, float2 *z, cudaStream_t st);
// Loop check (one thread): records the residual measure of the current
// iterate, decides whether another update follows, and sets the conditional
// handle of the enclosing while node accordingly.
cgs_status launch_cg_check(CGScalars *sc, cudaGraphConditionalHandle h, cudaStream_t st);
// One fused per-coil step of the batched CGNR inverse NFFT (see cgs_vec.cu):
// mode 1 dot_v and alpha, mode 2 the image and k-space updates with dot_r and
// the early-exit flags, mode 3 dz_new and beta.  dots6 = [dot_r, dot_z, dot_v,
// dz_new, alpha, beta] of nc each; partial holds dot_blocks() x nc doubles.
cgs_status launch_cgnr_fused(int mode, int64_t rows, int nc, const float *wr, float2 *vec, const float2 *other,
                             float2 *img, const float2 *imgp, const float *mask, int64_t img_rows, double *partial,
                             unsigned int *ticket, double *dots6, int *active, double eps, cudaStream_t st);
// Fused updates with a deterministic dot (kDotBlocks blocks, partial[kDotBlocks],
// a ticket that starts at 0 and is reset by the kernel):
// q += lambda p (lambda nullable), *out = Re <p, q>; nothing when *done
cgs_status launch_axpy_dot(float2 *q, const float2 *p, const double *lambda, const int *done, int64_t n,
                           double *partial, unsigned int *ticket, double *out, cudaStream_t st);
// CG / CGLS: x += ts p, r -= ts q (ts = rn / pq), rno = rn, rn = |r|^2, loop test
cgs_status launch_cg_xr_rr(float2 *x, float2 *r, const float2 *p, const float2 *q, CGScalars *sc, int64_t n,
                           double *partial, unsigned int *ticket, cudaGraphConditionalHandle h, cudaStream_t st);
// resets the loop scalars on the device (a graph-resident replacement for the host upload)
cgs_status launch_cg_init(CGScalars *sc, double lambda, double tol, int maxit, int sqrt_mode, cudaStream_t st);
// q += lambda * p ; then pq = Re<p,q> is computed by coldot
cgs_status launch_add_scaled(float2 *q, const float2 *p, const CGScalars *sc, int64_t n,
                             cudaStream_t st);
// x += ts p ; r -= ts q  (ts = rn / pq computed in-kernel)
cgs_status launch_cg_update_xr(float2 *x, float2 *r, const float2 *p, const float2 *q,
                               CGScalars *sc, int64_t n, cudaStream_t st);
// p = r + (rn/rno) p
cgs_status launch_cg_update_p(float2 *p, const float2 *r, const CGScalars *sc, int64_t n,
                              cudaStream_t st);
// sc->field = value (device scalar copy)
cgs_status launch_scalar_op(CGScalars *sc, const double *src, int op, cudaStream_t st);

// x[p] = (I ? I[p] : 1) * sum_c conj(S[p][c]) * F[p][c]   (coil-minor F, S)
cgs_status launch_coil_combine(const float2 *F, const float2 *S, const float *I, int64_t P, int nc,
                               float2 *x, cudaStream_t st);
// intensity map I = 1/(sqrt(sum_c |S_c|^2) + 1e-9) from coil-minor sens
cgs_status launch_intensity(const float2 *sens_cm, int64_t P, int nc, float *I, cudaStream_t st);
// x *= real scale (elementwise, single image)
cgs_status launch_scale_real(float2 *x, const float *s, int64_t n, cudaStream_t st);

// ---------------------------------------------------------------------------
// Compressed sensing over the NCSENSE operator (cgs_cs.cu)
// ---------------------------------------------------------------------------
constexpr int kCsSteps = 16;   // trial step sizes per objective pass
constexpr int kCsBlocks = 304; // reduction grid (2 blocks per SM)
// Penalty terms on a codeare-ordered image (axis 0 fastest).  tvmode: 0 off,
// 1 TV2D, 2 TV3D over all axes, 3 TV3D over the third axis only.
struct CsTerms {
    int D0, D1, D2;
    int tvmode[2];
    float tvw[2];
    float xfmw, l1, pnorm;
};
struct CsSteps {
    float t[kCsSteps];
    int n;
};
// wavelet decomposition filters (high[i] = (-1)^i low[i]), at most 8 taps
struct DwtFilt {
    float lo[8], hi[8];
    int fl;
};
// out[0..15]: data term per step over the k-space arrays (ffdbx = ksA,
// ffdbg = ksB, data = ksY); out[16..31]: TV terms of the images x, dx and
// L1 terms of lx, ldx per step.  partial holds 2 * kCsBlocks * kCsSteps doubles.
cgs_status launch_cs_obj(const float2 *ksA, const float2 *ksB, const float2 *ksY, int64_t nks, const float2 *x,
                         const float2 *dx, const float2 *lx, const float2 *ldx, const CsTerms &terms,
                         const CsSteps &steps, double *partial, double *out, cudaStream_t st);
// g += the L1 gradient at x
cgs_status launch_cs_l1grad(float2 *g, const float2 *x, const CsTerms &terms, int64_t n, cudaStream_t st);
// one wavelet pass along `axis` of the top-left n x n block of an ld x ld
// image: decomposition (inverse 0) or reconstruction (inverse 1); src and
// dst must differ
cgs_status launch_dwt_pass(const float2 *src, float2 *dst, int ld, int n, int axis, int inverse, const DwtFilt &f,
                           cudaStream_t st);
// out2 = (Re, Im) sum conj(a) b
cgs_status launch_cs_dot(const float2 *a, const float2 *b, int64_t n, double *partial, double *out2,
                         cudaStream_t st);
cgs_status launch_cs_nnz(const float2 *a, int64_t n, double *partial, double *out, cudaStream_t st);
// *out = bits of max |x| (a float)
cgs_status launch_cs_absmax(const float2 *x, int64_t n, unsigned int *out, cudaStream_t st);
// g = 2 ehr + the L1 and TV gradients at x
cgs_status launch_cs_grad(const float2 *x, const float2 *ehr, const CsTerms &terms, float2 *g, cudaStream_t st);
cgs_status launch_cs_axpy(float2 *x, const float2 *dx, float t, int64_t n, cudaStream_t st);
// dx = -g1 + dx * (*g1sq / *g0sq); dx = -g1 when g0sq is null
cgs_status launch_cs_dir(float2 *dx, const float2 *g1, const double *g1sq, const double *g0sq, int64_t n,
                         cudaStream_t st);
cgs_status launch_cs_sub(float2 *out, const float2 *a, const float2 *b, int64_t n, cudaStream_t st);
// acc[0] += sc->iter; acc[1] |= sc->nan_flag
cgs_status launch_cs_tally(const CGScalars *sc, int *acc, cudaStream_t st);

}  // namespace cgs
