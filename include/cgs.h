/*
 * cgs.h -- C ABI of the GB300 non-Cartesian CG-SENSE library (libcgs.so).
 *
 * Plain C: opaque plan handle, plain pointers and sizes, status codes, no
 * exceptions and no CUDA or torch types in any signature (a stream is passed
 * as `void*` holding a cudaStream_t; NULL selects the plan's own stream).
 *
 * Every data pointer may be host memory (pageable or pinned) or device memory
 * of the plan's GPU; the library detects which and stages host data itself.
 * Layouts are the reference's (codeare `Matrix` is column-major, first index
 * fastest, src/matrix/Matrix.hpp:165-200):
 *   image      complex float, N^d, codeare x index fastest (== NFFT3 f_hat
 *              order with NFFT dimension 0 slowest, src/matrix/ft/NFFT.hpp:340-346)
 *   coil image complex float, (N^d, NC): coil c is the c-th contiguous image
 *   kspace     float, (d, M): node j at k[d*j .. d*j+d-1], row 0 pairs with the
 *              slowest image axis (NFFT.hpp:267-268), each value in [-0.5, 0.5)
 *   weights    float, (M)
 *   signals    complex float, (M, NC): coil c is the c-th contiguous block
 * Complex values are interleaved (re, im) float pairs.
 *
 * Threading: one plan serves one caller thread at a time (as the reference's
 * NFFT/NCSENSE objects, whose scratch buffers are mutable members,
 * src/matrix/ft/NCSENSE.hpp:485); different plans are independent.
 */
#ifndef CGS_H
#define CGS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    CGS_OK = 0,
    CGS_ERR_BAD_ARG = 1,   /* invalid size, pointer or parameter            */
    CGS_ERR_OOM = 2,       /* device allocation failed                      */
    CGS_ERR_CUDA = 3,      /* a CUDA call failed (cgs_last_error() says which) */
    CGS_ERR_TIMEOUT = 4,   /* a bounded device wait gave up                  */
    CGS_ERR_NAN = 5,       /* the solver met a NaN residual                  */
    CGS_ERR_STATE = 6      /* call out of order (e.g. no k-space set yet)    */
} cgs_status;

typedef struct cgs_plan cgs_plan;

/* Geometry of one NFFT / NCSENSE operator.
 * Replaces the Params consumed by NFFT::NFFT (src/matrix/ft/NFFT.hpp:66-191:
 * keys nk, imsz, m, alpha; n_i = ceil(alpha * N_i)) and NCSENSE::NCSENSE
 * (src/matrix/ft/NCSENSE.hpp:69-184: sensitivities give NC). */
typedef struct {
    int rank;        /* 2 or 3                                             */
    int N[3];        /* image side per NFFT dimension (dimension 0 slowest); even */
    double alpha;    /* oversampling factor sigma (reference default 1.0)  */
    int m;           /* Kaiser-Bessel cut-off (reference default 1)        */
    int64_t M;       /* k-space nodes per coil ("nk")                      */
    int ncoils;      /* NC; 1 for a plain NFFT                             */
    int frames;      /* 0 or 1: one trajectory.  F > 1: NCSENSE's dim4 x dim5
                        batch (NCSENSE.hpp:141-166, 204-348): F frames with a
                        trajectory of M nodes each (k-space (d, M, F)) and the
                        same sensitivities and weights; images (N^d, F),
                        signals (M, NC, F); solves and CS run over the
                        stacked frames.  Not for Toeplitz, FCG or batches. */
} cgs_plan_desc;

/* Create / destroy.  Allocates all device scratch up front. */
cgs_status cgs_plan_create(cgs_plan **plan, const cgs_plan_desc *desc);
cgs_status cgs_plan_destroy(cgs_plan *plan);

/* K-space trajectory, (d, M) floats.  Replaces NFFT::KSpace
 * (src/matrix/ft/NFFT.hpp:258-273) and NCSENSE::KSpace (NCSENSE.hpp:204-236).
 * Sorts the nodes into grid tiles (done once per trajectory). */
cgs_status cgs_set_kspace(cgs_plan *plan, const float *k);

/* Density weights (M).  Replaces NFFT::Weights (NFFT.hpp:281-296) together
 * with the damping mask it builds (NFFTTraits.hpp:225-260). */
cgs_status cgs_set_weights(cgs_plan *plan, const float *w);

/* Coil sensitivities, (N^d, NC) complex; also builds the intensity map
 * I = 1/(sqrt(sum|S|^2)+1e-9).  Replaces NCSENSE::Sensitivities
 * (NCSENSE.hpp:192-196) and IntensityMap (src/matrix/mri/MRI.hpp:7-29). */
cgs_status cgs_set_sensitivities(cgs_plan *plan, const float *sens);

/* Per-coil NFFT trafo: f_c = A fhat_c for every coil (NC images in, (M,NC) out).
 * Replaces NFFT::Trafo (NFFT.hpp:305-361) / NFFT3 nfft_trafo. */
cgs_status cgs_nfft_trafo(cgs_plan *plan, const float *fhat, float *f, void *stream);

/* Per-coil true adjoint NFFT: fhat_c = A^H f_c (no iteration).
 * The operation NFFT3's nfft_adjoint computes (called inside NFFTTraits.hpp:201-204). */
cgs_status cgs_nfft_adjoint(cgs_plan *plan, const float *f, float *fhat, void *stream);

/* Per-coil inverse NFFT by CGNR with the density weights and damping mask:
 * what codeare's NFFT::Adjoint returns (NFFT.hpp:370-436 ->
 * NFFTTraits::ITrafo, NFFTTraits.hpp:122-138): zero start, at most `maxit`
 * steps, a coil stops once its W-weighted squared residual is below `eps`. */
cgs_status cgs_nfft_itrafo(cgs_plan *plan, const float *f, float *fhat, int maxit,
                           double eps, void *stream);

/* SENSE encoding E: y_c = A (S_c . x).  Replaces NCSENSE::Trafo / operator*
 * (NCSENSE.hpp:310-348, 421-423). */
cgs_status cgs_sense_trafo(cgs_plan *plan, const float *x, float *y, void *stream);

/* codeare's E^H: x = I . sum_c conj(S_c) . itrafo_c(y_c).  Replaces
 * NCSENSE::operator/ (NCSENSE.hpp:251-301). */
cgs_status cgs_sense_adjoint_codeare(cgs_plan *plan, const float *y, float *x, int ftiter,
                                     double fteps, void *stream);

/* True adjoint with weights: x = sum_c conj(S_c) . A^H (w . y_c)
 * (w = 1 when `weighted` is 0).  No reference counterpart: the building block
 * of the standard (Pruessmann) CG-SENSE normal equations. */
cgs_status cgs_sense_adjoint(cgs_plan *plan, const float *y, float *x, int weighted,
                             void *stream);

/* Solver options and report. */
typedef enum {
    CGS_MODE_CODEARE = 0,   /* CGLS over codeare's E^H (bit-for-bit semantics of the reference) */
    CGS_MODE_STANDARD = 1   /* CG on (E^H W E + lambda) x = E^H W y, true adjoint      */
} cgs_mode;

typedef struct {
    int mode;          /* cgs_mode                                           */
    int cgiter;        /* outer iterations (reference "cgmaxit", default 10) */
    double cgeps;      /* codeare mode: break when rn/xn <= cgeps (squared ratio);
                          standard mode: break when ||r||/||r0|| <= cgeps      */
    double lambda;     /* Tikhonov weight (reference "lambda")               */
    int ftiter;        /* inner CGNR steps (reference "ftmaxit", default 3)  */
    double fteps;      /* inner CGNR threshold (reference "fteps", 1e-3)     */
    int weighted;      /* standard mode: use the density weights W           */
    int toeplitz;      /* standard mode: apply E^H W E by Toeplitz embedding
                          (2N-grid FFT convolution with the weighted point-spread
                          function, computed once per trajectory and weights);
                          codeare mode: run each CG step's inner CGNR in image
                          space on the same kernel (same steps and early exits
                          as with the NFFT pair; needs alpha >= 2 and m >= 4,
                          else CGS_ERR_BAD_ARG); no reference counterpart     */
    int jacobi;        /* cgs_solve_fcg preconditioner kind (no reference
                          counterpart): 0 none; 1 the exact diagonal D of
                          E^H W E + lambda (D^-1 r); 2 the circulant C (see
                          cgs_precond_apply), with a net the base that the net
                          corrects                                            */
} cgs_solve_opts;

typedef struct {
    int iterations;        /* outer iterations performed                     */
    double res_first;      /* first residual measure (rn/xn or ||r||/||r0||) */
    double res_last;       /* residual measure at exit                       */
    double seconds;        /* device time of the solve                       */
    double res_hist[256];  /* residual measure per check, up to 256          */
    int fallback_at;       /* flexible CG: iteration at which it fell back to
                              plain CG, -1 if it never did                   */
} cgs_solve_report;

/* Full CG-SENSE solve (signals -> image).  CGS_MODE_CODEARE replaces
 * NCSENSE::Adjoint -> CGLS::Solve (NCSENSE.hpp:408-414, 434-436;
 * src/optimisation/CGLS.hpp:30-59) and the body of CGSENSE::Process
 * (src/modules/CGSENSE.cpp:165-179).  `report` may be NULL. */
cgs_status cgs_solve(cgs_plan *plan, const float *y, float *x, const cgs_solve_opts *opts,
                     cgs_solve_report *report, void *stream);

/* ---------------------------------------------------------------------------
 * Learned preconditioner (no reference counterpart): a 5-layer 3x3 CNN on a
 * complex image held as 2 real channels, 2 -> 32 -> 32 -> 32 -> 32 -> 2, ReLU
 * between layers, no biases (so M(c r) = c M(r) for c > 0), BF16 weights and
 * activations with FP32 accumulation.  Tensors are [B][H][W][2] float
 * (channel 0 real, 1 imaginary); weights are cgs_net_num_params() floats,
 * layer after layer, each [9 taps][Cout][Cin], tap = 3*dy + dx for the
 * offset (dy-1, dx-1).
 * ------------------------------------------------------------------------- */
typedef struct cgs_net cgs_net;
int64_t cgs_net_num_params(void);
cgs_status cgs_net_create(cgs_net **net, int max_batch, int max_h, int max_w);
cgs_status cgs_net_destroy(cgs_net *net);
cgs_status cgs_net_set_weights(cgs_net *net, const float *w);
cgs_status cgs_net_get_weights(cgs_net *net, float *w);
cgs_status cgs_net_forward(cgs_net *net, const float *x, float *y, int B, int H, int W, void *stream);
/* The kernel of the 32 -> 32 layers (forward and input gradients): 1 (the
 * default) the 5th-generation tensor cores (tcgen05.mma with the accumulator
 * in tensor memory), 0 the warp-level mma.sync kernel.  Both compute the same
 * BF16 products with FP32 accumulation.  A tcgen05 layer whose bounded wait
 * for its MMAs runs out makes the next forward / gradients call return
 * CGS_ERR_TIMEOUT. */
cgs_status cgs_net_set_conv_kernel(cgs_net *net, int kind);
/* mean-squared-error gradients w.r.t. all weights (for checks) */
cgs_status cgs_net_gradients(cgs_net *net, const float *x, const float *target, int B, int H, int W,
                             float *grad, float *loss, void *stream);
/* one Adam step on the mean-squared error between net(x) and target */
cgs_status cgs_net_train_step(cgs_net *net, const float *x, const float *target, int B, int H, int W,
                              float lr, float *loss, void *stream);

/* Batched solves (no reference counterpart; codeare runs one CGSENSE module
 * per process): one CUDA graph holds the solves of `count` plans as
 * independent branches, each a device-driven CG loop (opts[i] as in
 * cgs_solve, cgiter >= 1), so uneven problems of any size, coil count and
 * trajectory run concurrently from a single graph launch.  A plan may belong
 * to one batch at a time and must not be used elsewhere while the batch
 * solves; changing its k-space, weights or tuning afterwards makes
 * cgs_batch_solve return CGS_ERR_STATE (build a new batch). */
typedef struct cgs_batch cgs_batch;
cgs_status cgs_batch_create(cgs_batch **out, cgs_plan *const *plans, const cgs_solve_opts *opts, int count,
                            void *stream);
/* y[i]: plan i's samples (M x NC complex, host or device); x[i]: its image.
 * reports (nullable) gets one report per plan; seconds (nullable) the device
 * time of the graph launch. */
cgs_status cgs_batch_solve(cgs_batch *b, const float *const *y, float *const *x, cgs_solve_report *reports,
                           double *seconds);
cgs_status cgs_batch_destroy(cgs_batch *b);

/* Gridding work decomposition of a plan (no reference counterpart: NFFT3
 * has no tunable bins).  0 in a field means the built-in default. */
typedef struct {
    int tile;          /* 2-D interpolation bin side in grid points (8, 16, 32; default 8) */
    int work_slice;    /* most nodes per interpolation work item (default 512) */
    int spread_chunk;  /* most nodes per spreading work item (default 2x the mean patch list, 64..1024) */
    int interp_coils;  /* coils per interpolation CTA: 1, 4, 8, 16 or 32 (default 16, fewer for fewer coils) */
    int spread_coils;  /* coils per spreading warp: 1, 2, 4, 8, 16 or 32 (default: coils, at most 32) */
    int spread_block;  /* spreading lanes: 1 (a point each on 4 x 4 patches, two coil groups),
                          2 / 4 (2 x 1 / 2 x 2 blocks, four coil groups, 4 or more coils),
                          8 (a point each on 4 x 8 patches, one coil group, 2..16 coils),
                          16 (4 x 4 patches on the tensor cores, TF32-split operands
                          with FP32 accumulation), 32 (8 x 4 patches on the tensor
                          cores), 64 (8 x 16 patches on the 5th-generation tensor
                          cores, tcgen05.mma kind::tf32 with a tensor-memory
                          accumulator); default 64 from 8 coils, 16 from 4, else 1 */
    int interp_block;  /* 2-D interpolation: 1 CUDA cores (tiles of `tile`), 16 tensor
                          cores (16 nodes of a 4 x 4 footprint-start bin per warp,
                          TF32-split operands, FP32 accumulation), 64 the 5th-generation
                          tensor cores (tcgen05.mma kind::tf32, up to 128 nodes of an
                          8 x 16 footprint-start bin per CTA, the weights in tensor
                          memory); default 16 from 4 coils for m <= 4, else 1 */
    int host_chunks;   /* cgs_nfft_trafo / cgs_nfft_adjoint with a host input or output,
                          cgs_sense_trafo with a host output (one frame): the coils
                          are split into this many contiguous
                          chunks, each run by a child plan (sharing the plan's node
                          tables) on its own stream, so one chunk's host copies
                          overlap another's kernels; 1 = one pass; default, when
                          the k-space holds 8 MiB or more, 4 chunks for the forward
                          and 2 for the adjoint, else 1; at least 4 coils per chunk
                          (no chunks below 8 coils).  Up to 32. */
} cgs_tuning;

cgs_status cgs_get_tuning(const cgs_plan *plan, cgs_tuning *out);
/* Applies `t`; a change of tile, work_slice or spread_chunk re-bins the
 * trajectory (the k-space and weights already set are kept). */
cgs_status cgs_set_tuning(cgs_plan *plan, const cgs_tuning *t);
/* Autotuner: times the plan's own interpolation and spreading launches on
 * scratch data for each candidate decomposition (tile x work_slice x
 * interp_coils, spread_block x spread_chunk x spread_coils), applies the fastest and returns
 * it with its interpolation + spreading time in milliseconds.  Needs the
 * k-space; leaves the plan's data and the Toeplitz kernel to be rebuilt on
 * their next use.  2-D plans only. */
cgs_status cgs_autotune(cgs_plan *plan, cgs_tuning *chosen, double *ms, void *stream);

/* Autotune cache (no reference counterpart): cgs_autotune keeps, per problem
 * class (grid, cut-off m, coil count and nodes per grid point in steps of
 * 2^(1/4)), the decomposition it measured, and applies it to later plans of
 * the same class without timing again (`ms` then reports the cached time).
 * Process-wide and thread-safe.  mode 0: off (and cleared), 1: on (and
 * cleared; the default state is on), 2: clear, keep the current state. */
cgs_status cgs_autotune_cache(int mode);

/* Flexible CG-SENSE with the learned preconditioner (no reference
 * counterpart): standard-mode normal equations (E^H W E + lambda) x = b with
 * z = d . net(d . r) as a variable preconditioner, d = D^-1/2 the exact
 * diagonal scaling (D = sum_c |S_c|^2 sum_j w_j + lambda, so the network
 * works on the unit-diagonal system), Polak-Ribiere beta, and a fallback
 * to plain CG (restarted) once the residual stalls for three iterations or the
 * network gives <r, z> <= 0.  Stops at ||r||/||r0|| <= cgeps.  The right-hand
 * side is b = E^H W y from k-space data y, or the image `rhs` when y is NULL.
 * net == NULL runs the same loop as plain CG (Polak-Ribiere beta), or
 * preconditioned CG with the exact diagonal (opts->jacobi 1) or the circulant
 * of cgs_precond_apply (opts->jacobi 2).  With a net and opts->jacobi 2 the
 * preconditioner is z = C r + d . net(d . r): the network corrects the
 * circulant step instead of the diagonal one.  The plan's
 * image must be 2-D and fit the net's maximum image size. */
cgs_status cgs_solve_fcg(cgs_plan *plan, const float *y, const float *rhs, float *x,
                         const cgs_solve_opts *opts, cgs_net *net, cgs_solve_report *report,
                         void *stream);

/* Circulant preconditioner of the standard-mode normal equations (no
 * reference counterpart): z = C r with
 *   C = Q F^-1 diag(1 / (c + lambda / mean(sum_c |S_c|^2))) F Q,  Q = diag(1 / sqrt(sum_c |S_c|^2)),
 * F the 2-D DFT on the N x N image and c the T. Chan spectrum of the
 * weighted point-spread function (the Toeplitz kernel of cgs_solve's
 * toeplitz option, folded onto the N-periodic grid), floored at 0.2 of its
 * mean.  lambda and the weighting come from opts.  2-D single-frame plans
 * with k-space, sensitivities and (if weighted) weights set. */
cgs_status cgs_precond_apply(cgs_plan *plan, const float *r, float *z, const cgs_solve_opts *opts, void *stream);

/* out = (E^H W E + lambda) x for an image x (Toeplitz or NFFT pair as opts say). */
cgs_status cgs_normal_apply(cgs_plan *plan, const float *x, float *out, const cgs_solve_opts *opts,
                            void *stream);

/* Sizes of the plan (for host wrappers). */
cgs_status cgs_plan_info(const cgs_plan *plan, int *rank, int *N, int *n, int64_t *M,
                         int *ncoils);

/* Sensitivities of one frame of a framed plan (frames > 1), NC x N.. complex,
 * coil-major: the maps of a stack of 2-D slices along a Cartesian third axis
 * (NCSENSE's 3rd_dim_cart, src/matrix/ft/NCSENSE.hpp:81-97, 105: each slice is
 * a frame with the shared trajectory and its own slice of the 3-D maps).
 * cgs_set_sensitivities sets the same maps for every frame instead. */
cgs_status cgs_set_frame_sensitivities(cgs_plan *plan, int frame, const float *sens);

/* Synchronise the plan's stream. */
cgs_status cgs_sync(cgs_plan *plan);

/* Number of this library's kernels launched since load (a launch counter). */
int64_t cgs_kernel_launches(void);

/* Allocation-free 2-D NFFT forward for one coil: f = A fhat.
 * No counterpart in the reference.  It exists for callers that must not
 * allocate device memory while they run: a real-time reconstruction loop
 * next to an acquisition stream (cudaMalloc / cudaFree synchronise the
 * device and would stall it), or a host that owns a fixed device-memory
 * budget through its own pool.  It uses no plan; its scratch is one static
 * device array of 2^19 complex floats (4 MiB) that every GPU loading this
 * library keeps until exit.  Limit: N*n + n*n + 2n + N <= 2^19 with
 * n = ceil(alpha*N) (square N x N image; N = 256 at alpha = 2); larger
 * sizes return CGS_ERR_BAD_ARG.  k (M x 2 floats), fhat (N x N complex) and
 * f (M complex) must be device pointers.  All calls share the array, so
 * calls that overlap on the GPU race; the first call on a device resolves
 * the array's address and should come before any stream capture.  The
 * address is kept until exit, so a cudaDeviceReset invalidates it: do not
 * call this again on a device that was reset.  k is not read on the host:
 * a node outside [-0.5, 0.5) in either coordinate gets NaN in f and the call
 * still returns CGS_OK (the plan entry points reject such a trajectory). */
cgs_status cgs_nfft2d_trafo_noalloc(int N, double alpha, int m, int64_t M, const float *k,
                                    const float *fhat, float *f, void *stream);

/* Per-kernel timing with CUDA events recorded on the launching stream around
 * every FFT pass, interpolation and spreading launch (instrumentation; no
 * reference counterpart -- the reference times whole modules with
 * SimpleTimer, src/core/Queue.cpp:59-60).  cgs_profile_collect waits for the
 * recorded events, writes the accumulated milliseconds and launch counts per
 * category (0 = FFT axis passes, 1 = interpolation, 2 = spreading) into
 * ms[3] / count[3] (either may be NULL) and resets them. */
void cgs_profile_enable(int on);
void cgs_profile_collect(double *ms, int64_t *count);

/* Text of the last error on this thread ("" if none). */
const char *cgs_last_error(void);

/* Diagnostic of the bounded device waits (no reference counterpart: the
 * reference has no device code).  The tensor-core kernels wait for their
 * MMAs on an mbarrier with a time limit; when a wait runs out the kernel
 * skips its epilogue, frees its tensor memory, returns and sets a
 * process-wide flag, and the library's next call reports CGS_ERR_TIMEOUT
 * once.  This call runs that wait in a one-thread kernel on a barrier that
 * nothing completes, for limit_ns nanoseconds (at most 1 s), waits for the
 * kernel on `stream` and returns what the check reports: CGS_ERR_TIMEOUT,
 * with the flag cleared and the context still usable. */
cgs_status cgs_diag_wait_timeout(int64_t limit_ns, void *stream);

/* ------------------------------------------------------------------------
 * Compressed sensing over the NCSENSE operator: codeare's CS_XSENSE with
 * ft = 3 (src/matrix/ft/CS_XSENSE.hpp:73-140), its TV and L1 penalties
 * (TVOP.hpp, CS_XSENSE.hpp:329-405) and the NLCG minimiser
 * (src/optimisation/NLCG.hpp:42-125), as the CompressedSensing module
 * configures them (src/modules/CompressedSensing.cpp:86-136).  A handle
 * borrows a plan that has k-space, weights and sensitivities; the plan must
 * not be used by anyone else while a CS call runs.
 * ------------------------------------------------------------------------ */
typedef struct cgs_cs cgs_cs;

typedef struct {
    /* the NCSENSE inverse (ft ->*): codeare CGLS (keys cgmaxit, cgeps,
     * lambda, ftmaxit, fteps) */
    int cgiter;
    double cgeps, lambda;
    int ftiter;
    double fteps;
    /* minimiser: nlopt 0 = NLCG, 2 = Split Bregman (the reference's is
     * empty: the result is the CGLS image); 1 (L-BFGS) is not supported */
    int nlopt, csiter, nliter, lsiter;
    float lsa, lsb, cgconv;
    int parallel_linesearch;   /* the reference's parallel rule (NLCG.hpp:56-80) */
    /* objective: TV weights (scaled by max |x0| in every cgs_cs_adjoint, as
     * the reference's mutable _tvw), TV'ed axes per term (codeare order;
     * ntvdims 0 = every axis), L1 weight, smoothing l1, p-norm */
    float tvw[2];
    int tvdims[2][3], ntvdims[2];
    float xfmw, l1, pnorm;
    /* wavelet (DWT.hpp): -1 none; 0 Daubechies with member 4 or 8 taps, 2
     * Haar with member 2 (the reference's only initialised filters); the
     * NLCG variable is then the image's wavelet coefficients.  Needs a
     * square 2-D image with dyadic sides; levels down to 16 x 16. */
    int wl_family, wl_member;
    /* operator (CS_XSENSE.hpp:98-110): 3 (or 0) NCSENSE, whose ->* is the
     * CGLS above; 2 plain NFFT (a single-coil plan, no sensitivities), whose
     * ->* is the plan's CGNR inverse NFFT with ftiter steps and threshold
     * fteps (NFFT.hpp:370-436) */
    int ft;
} cgs_cs_opts;

typedef struct {
    int iterations;            /* NLCG iterations over all repetitions */
    int ls_index[256];         /* accepted line-search index per iteration
                                  (lsiter when the search gave up) */
    double rmse[256];          /* sqrt(data term / nnz(data)) per iteration */
    int solves;                /* CGLS solves run */
    int solve_iterations;      /* their CG iterations */
    float tvw_used[2];         /* TV weights after the scaling */
    double seconds;
} cgs_cs_report;

cgs_status cgs_cs_create(cgs_cs **cs, cgs_plan *plan, const cgs_cs_opts *opts);
/* May be called before or after the plan is destroyed. */
cgs_status cgs_cs_destroy(cgs_cs *cs);

/* x = CS reconstruction of data y ((M, NC) complex): CS_XSENSE::Adjoint /
 * operator->* (CS_XSENSE.hpp:283-322). */
cgs_status cgs_cs_adjoint(cgs_cs *cs, const float *y, float *x, cgs_cs_report *report, void *stream);

/* g = gradient of the objective at x for data y (CS_XSENSE::df,
 * CS_XSENSE.hpp:223-232), with the current TV weights.  x, g (and dx below)
 * are wavelet coefficients when the handle has a wavelet. */
cgs_status cgs_cs_df(cgs_cs *cs, const float *y, const float *x, float *g, void *stream);

/* The handle's wavelet transform: out = W in (DWT::operator*, inverse 0)
 * or W^-1 in (DWT::operator->*, inverse 1); a copy without a wavelet. */
cgs_status cgs_cs_wavelet(cgs_cs *cs, const float *in, float *out, int inverse, void *stream);

/* Objective at x + t dx for data y (CS_XSENSE::obj after df(x) and
 * Update(dx), CS_XSENSE.hpp:197-221); *rmse = sqrt(data term / nnz(y)). */
cgs_status cgs_cs_obj(cgs_cs *cs, const float *y, const float *x, const float *dx, float t, double *obj,
                      double *rmse, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CGS_H */
