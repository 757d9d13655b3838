/*
 * cgs_oracle.c -- FP64 CPU oracle for the non-Cartesian CG-SENSE path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this library; the GPU
 * product never calls it.
 *
 * PARITY UNPINNED.  The reference (kvahed/codeare) delegates all NFFT
 * arithmetic to the third-party NFFT3 library (TU Chemnitz; version not pinned
 * by the reference: its CMakeLists.txt:220-246 probes the >= 3.2 naming
 * `nfft_mv_plan_complex`).  Neither NFFT3 nor FFTW is present, and the
 * reference ships no golden vectors for this path.  This file restates, in
 * its own code:
 *   - the Kaiser-Bessel NFFT as published for NFFT3 (Keiner, Kunis, Potts,
 *     "Using NFFT 3", ACM TOMS 36(4), 2009): window
 *        phi(x)  = sinh(b sqrt(m^2 - (n x)^2)) / (pi sqrt(m^2 - (n x)^2))
 *                  (sin-branch beyond |n x| > m, limit b/pi at |n x| = m),
 *        phihat(k) = I0(m sqrt(b^2 - (2 pi k / n)^2)),  b = pi (2 - 1/sigma),
 *     2m+2 taps per dimension starting at floor(n x) - m, deapodisation by
 *     1/prod phihat, unnormalised FFTs with sign -1 (trafo) / +1 (adjoint);
 *     these are the formulas the reference keeps beside its wrapper
 *     (src/matrix/ft/NFFTTraits.hpp:659-673);
 *   - the CGNR inverse NFFT with density weights W and frequency damping
 *     mask What, which the reference runs as its NFFT "Adjoint"
 *     (src/matrix/ft/NFFTTraits.hpp:122-138, solver flags at :66-68,
 *     mask at :225-260; src/matrix/ft/NFFT.hpp:370-436);
 *   - the NCSENSE encoding E and codeare's E^H composition with the
 *     intensity map (src/matrix/ft/NCSENSE.hpp:251-348,
 *     src/matrix/mri/MRI.hpp:7-29);
 *   - the CGLS outer loop (src/optimisation/CGLS.hpp:30-59);
 *   - a direct FP64 NDFT, the exact operator that the NFFT approximates,
 *     which pins the NFFT restatement to its mathematical definition.
 *
 * Layouts follow the reference: an image is stored with the first NFFT
 * dimension slowest (codeare's column-major image copied flat into NFFT3's
 * f_hat, NFFT.hpp:340-346), node j has coordinates x[d*j + t], t = 0 being
 * the slowest image axis, and coil c of a multi-coil array occupies the
 * c-th contiguous block.  Complex data is interleaved (re, im) doubles.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ */
/* Modified Bessel function I0 from its power series                   */
/*   I0(x) = sum_k ((x/2)^2)^k / (k!)^2                                */
/* ------------------------------------------------------------------ */
static double bessel_i0(double x)
{
    double y = 0.25 * x * x, term = 1.0, sum = 1.0;
    for (int k = 1; k < 1000; ++k) {
        term *= y / ((double)k * (double)k);
        sum += term;
        if (term < 1e-18 * sum) break;
    }
    return sum;
}

/* Kaiser-Bessel window in grid units: tau = n*x - l, see header. */
double orc_kb_phi(double tau, int m, double b)
{
    double m2 = (double)m * (double)m, t2 = tau * tau;
    if (m2 > t2) { double s = sqrt(m2 - t2); return sinh(b * s) / (M_PI * s); }
    if (m2 < t2) { double s = sqrt(t2 - m2); return sin(b * s) / (M_PI * s); }
    return b / M_PI;
}

double orc_kb_phihut(int k, int n, int m, double b)
{
    double w = 2.0 * M_PI * (double)k / (double)n;
    double a = b * b - w * w;
    if (a < 0) a = 0; /* cannot happen for |k| <= N/2 <= n/2 */
    return bessel_i0((double)m * sqrt(a));
}

/* ------------------------------------------------------------------ */
/* FP64 mixed-radix Stockham FFT (own implementation; FFTW is absent)  */
/* ------------------------------------------------------------------ */
typedef struct {
    int n, nf, f[40];
    cplx *tw; /* tw[t] = exp(-2 pi i t / n) */
} fftplan;

static void fft_plan_init(fftplan *p, int n)
{
    p->n = n; p->nf = 0;
    int r = n;
    while (r % 4 == 0) { p->f[p->nf++] = 4; r /= 4; }
    while (r % 2 == 0) { p->f[p->nf++] = 2; r /= 2; }
    for (int q = 3; r > 1; q += 2)
        while (r % q == 0) { p->f[p->nf++] = q; r /= q; }
    p->tw = (cplx *)malloc(sizeof(cplx) * (size_t)(n > 0 ? n : 1));
    for (int t = 0; t < n; ++t) {
        double a = -2.0 * M_PI * (double)t / (double)n;
        p->tw[t] = cos(a) + I * sin(a);
    }
}

static void fft_plan_free(fftplan *p) { free(p->tw); p->tw = NULL; }

/* in-place transform of contiguous x (length n) using work (length n). */
static void fft_exec(const fftplan *p, cplx *x, cplx *work, int sign)
{
    const int n = p->n;
    if (n <= 1) return;
    cplx *src = x, *dst = work;
    int Ns = 1;
    cplx v[64], V[64];
    for (int s = 0; s < p->nf; ++s) {
        const int R = p->f[s], nR = n / R, step = n / (Ns * R);
        for (int j = 0; j < nR; ++j) {
            const int k = j % Ns;
            for (int r = 0; r < R; ++r) {
                cplx a = src[j + r * nR];
                const int t = k * r * step;  /* < Ns R step = n */
                cplx w = (sign < 0) ? p->tw[t] : conj(p->tw[t]);
                v[r] = a * w;
            }
            if (R == 2) {
                V[0] = v[0] + v[1]; V[1] = v[0] - v[1];
            } else if (R == 4) {
                cplx a0 = v[0] + v[2], a1 = v[0] - v[2];
                cplx b0 = v[1] + v[3], b1 = v[1] - v[3];
                cplx jb1 = (sign < 0) ? (-I * b1) : (I * b1);
                V[0] = a0 + b0; V[2] = a0 - b0; V[1] = a1 + jb1; V[3] = a1 - jb1;
            } else {
                for (int q = 0; q < R; ++q) {
                    cplx acc = 0;
                    for (int r = 0; r < R; ++r) {
                        int t = ((r * q) % R) * nR;
                        cplx w = (sign < 0) ? p->tw[t] : conj(p->tw[t]);
                        acc += v[r] * w;
                    }
                    V[q] = acc;
                }
            }
            const int base = (j / Ns) * Ns * R + k;
            for (int r = 0; r < R; ++r) dst[base + r * Ns] = V[r];
        }
        cplx *tmp = src; src = dst; dst = tmp;
        Ns *= R;
    }
    if (src != x) memcpy(x, src, sizeof(cplx) * (size_t)n);
}

/* Multi-dimensional unnormalised FFT over an array with dims n[0..d-1]
 * (n[0] slowest). */
static void fft_nd(cplx *a, int d, const int *n, int sign)
{
    size_t total = 1;
    for (int t = 0; t < d; ++t) total *= (size_t)n[t];
    for (int t = 0; t < d; ++t) {
        size_t inner = 1, outer = 1;
        for (int u = t + 1; u < d; ++u) inner *= (size_t)n[u];
        for (int u = 0; u < t; ++u) outer *= (size_t)n[u];
        const int L = n[t];
        fftplan p; fft_plan_init(&p, L);
        /* up to CB adjacent columns are gathered per pass, so every strided
         * row access reads CB consecutive values instead of one */
        enum { CB = 8 };
        cplx *line = (cplx *)malloc(sizeof(cplx) * (size_t)L * (CB + 1));
        cplx *work = line + (size_t)L * CB;
        for (size_t o = 0; o < outer; ++o)
            for (size_t i0 = 0; i0 < inner; i0 += CB) {
                const int cb = (int)((inner - i0) < CB ? (inner - i0) : CB);
                cplx *base = a + o * (size_t)L * inner + i0;
                for (int l = 0; l < L; ++l)
                    for (int c = 0; c < cb; ++c) line[(size_t)c * L + l] = base[(size_t)l * inner + c];
                for (int c = 0; c < cb; ++c) fft_exec(&p, line + (size_t)c * L, work, sign);
                for (int l = 0; l < L; ++l)
                    for (int c = 0; c < cb; ++c) base[(size_t)l * inner + c] = line[(size_t)c * L + l];
            }
        free(line);
        fft_plan_free(&p);
        (void)total;
    }
}

/* exported for tests: 1-D/ND FFT of interleaved doubles */
void orc_fft_nd(double *a, int d, const int *n, int sign)
{
    fft_nd((cplx *)a, d, n, sign);
}

/* ------------------------------------------------------------------ */
/* NFFT plan                                                            */
/* ------------------------------------------------------------------ */
typedef struct {
    int d, N[3], n[3], m;
    long M;
    double b[3];
    double *phihut_inv[3]; /* 1/phihut(k) for k = -N/2 .. N/2-1 */
    double *x;             /* M*d */
    size_t Ntot, ntot;
    /* per node and dimension, the 2m+2 window values and wrapped grid indices,
     * computed once per trajectory as NFFT3's PRE_PSI does for codeare's plans
     * (src/matrix/ft/NFFTTraits.hpp:68-69); NULL when they would exceed 1 GiB */
    double *psi;
    int *psi_idx;
} orc_nfft;

orc_nfft *orc_nfft_create(int d, const int *N, const int *n, int m, long M)
{
    if (d < 1 || d > 3 || m < 0 || M < 0) return NULL;
    orc_nfft *p = (orc_nfft *)calloc(1, sizeof(orc_nfft));
    p->d = d; p->m = m; p->M = M; p->Ntot = 1; p->ntot = 1;
    for (int t = 0; t < d; ++t) {
        p->N[t] = N[t]; p->n[t] = n[t];
        p->Ntot *= (size_t)N[t]; p->ntot *= (size_t)n[t];
        double sigma = (double)n[t] / (double)N[t];
        p->b[t] = M_PI * (2.0 - 1.0 / sigma);
        p->phihut_inv[t] = (double *)malloc(sizeof(double) * (size_t)N[t]);
        for (int i = 0; i < N[t]; ++i)
            p->phihut_inv[t][i] = 1.0 / orc_kb_phihut(i - N[t] / 2, n[t], m, p->b[t]);
    }
    p->x = (double *)calloc((size_t)(M > 0 ? M : 1) * (size_t)d, sizeof(double));
    return p;
}

void orc_nfft_destroy(orc_nfft *p)
{
    if (!p) return;
    for (int t = 0; t < p->d; ++t) free(p->phihut_inv[t]);
    free(p->x);
    free(p->psi);
    free(p->psi_idx);
    free(p);
}

/* tap positions and weights of node j along dimension t, evaluated */
static void node_taps_eval(const orc_nfft *p, long j, int t, int *idx, double *w)
{
    const int n = p->n[t], m = p->m;
    const double nx = (double)n * p->x[(size_t)j * p->d + t];
    const long c = (long)floor(nx);
    for (int i = 0; i < 2 * m + 2; ++i) {
        long l = c - m + i;
        w[i] = orc_kb_phi(nx - (double)l, m, p->b[t]);
        long q = l % n; if (q < 0) q += n;
        idx[i] = (int)q;
    }
}

void orc_nfft_set_x(orc_nfft *p, const double *x)
{
    memcpy(p->x, x, sizeof(double) * (size_t)p->M * (size_t)p->d);
    free(p->psi); free(p->psi_idx);
    p->psi = NULL; p->psi_idx = NULL;
    const size_t T = (size_t)(2 * p->m + 2), cnt = (size_t)p->M * (size_t)p->d * T;
    if (cnt * (sizeof(double) + sizeof(int)) > ((size_t)1 << 30)) return;
    p->psi = (double *)malloc(sizeof(double) * (cnt > 0 ? cnt : 1));
    p->psi_idx = (int *)malloc(sizeof(int) * (cnt > 0 ? cnt : 1));
    if (!p->psi || !p->psi_idx) { free(p->psi); free(p->psi_idx); p->psi = NULL; p->psi_idx = NULL; return; }
#pragma omp parallel for schedule(static)
    for (long j = 0; j < p->M; ++j)
        for (int t = 0; t < p->d; ++t) {
            const size_t o = ((size_t)j * (size_t)p->d + (size_t)t) * T;
            node_taps_eval(p, j, t, p->psi_idx + o, p->psi + o);
        }
}

/* tap positions and weights of node j along dimension t: the precomputed
 * tables, or evaluated into the caller's buffers */
static void node_taps(const orc_nfft *p, long j, int t, const int **idx, const double **w, int *ib, double *wb)
{
    if (p->psi) {
        const size_t o = ((size_t)j * (size_t)p->d + (size_t)t) * (size_t)(2 * p->m + 2);
        *idx = p->psi_idx + o;
        *w = p->psi + o;
        return;
    }
    node_taps_eval(p, j, t, ib, wb);
    *idx = ib;
    *w = wb;
}

static void unravel(size_t flat, int d, const int *dims, int *out)
{
    for (int t = d - 1; t >= 0; --t) { out[t] = (int)(flat % (size_t)dims[t]); flat /= (size_t)dims[t]; }
}

static size_t grid_pos(const orc_nfft *p, const int *i)
{
    size_t pos = 0;
    for (int t = 0; t < p->d; ++t) {
        int k = i[t] - p->N[t] / 2;
        int q = ((k % p->n[t]) + p->n[t]) % p->n[t];
        pos = pos * (size_t)p->n[t] + (size_t)q;
    }
    return pos;
}

/* f = A fhat  (NFFT trafo, sign -1) */
void orc_nfft_trafo(const orc_nfft *p, const double *fhat_in, double *f_out)
{
    const cplx *fhat = (const cplx *)fhat_in;
    cplx *f = (cplx *)f_out;
    cplx *g = (cplx *)calloc(p->ntot, sizeof(cplx));
    int i[3];
    for (size_t k = 0; k < p->Ntot; ++k) {
        unravel(k, p->d, p->N, i);
        double s = 1.0;
        for (int t = 0; t < p->d; ++t) s *= p->phihut_inv[t][i[t]];
        g[grid_pos(p, i)] = fhat[k] * s;
    }
    fft_nd(g, p->d, p->n, -1);
    const int T = 2 * p->m + 2;
    int ib[3][64]; double wb[3][64];
    const int *idx[3]; const double *w[3];
    for (long j = 0; j < p->M; ++j) {
        for (int t = 0; t < p->d; ++t) node_taps(p, j, t, &idx[t], &w[t], ib[t], wb[t]);
        cplx acc = 0;
        if (p->d == 1) {
            for (int a = 0; a < T; ++a) acc += g[idx[0][a]] * w[0][a];
        } else if (p->d == 2) {
            for (int a = 0; a < T; ++a) {
                cplx row = 0;
                const cplx *gr = g + (size_t)idx[0][a] * p->n[1];
                for (int b = 0; b < T; ++b) row += gr[idx[1][b]] * w[1][b];
                acc += row * w[0][a];
            }
        } else {
            for (int a = 0; a < T; ++a) {
                cplx pl = 0;
                for (int b = 0; b < T; ++b) {
                    cplx row = 0;
                    const cplx *gr = g + ((size_t)idx[0][a] * p->n[1] + idx[1][b]) * p->n[2];
                    for (int c = 0; c < T; ++c) row += gr[idx[2][c]] * w[2][c];
                    pl += row * w[1][b];
                }
                acc += pl * w[0][a];
            }
        }
        f[j] = acc;
    }
    free(g);
}

/* fhat = A^H f  (NFFT adjoint, sign +1) */
void orc_nfft_adjoint(const orc_nfft *p, const double *f_in, double *fhat_out)
{
    const cplx *f = (const cplx *)f_in;
    cplx *fhat = (cplx *)fhat_out;
    cplx *g = (cplx *)calloc(p->ntot, sizeof(cplx));
    const int T = 2 * p->m + 2;
    int ib[3][64]; double wb[3][64];
    const int *idx[3]; const double *w[3];
    for (long j = 0; j < p->M; ++j) {
        for (int t = 0; t < p->d; ++t) node_taps(p, j, t, &idx[t], &w[t], ib[t], wb[t]);
        const cplx fj = f[j];
        if (p->d == 1) {
            for (int a = 0; a < T; ++a) g[idx[0][a]] += fj * w[0][a];
        } else if (p->d == 2) {
            for (int a = 0; a < T; ++a) {
                cplx va = fj * w[0][a];
                cplx *gr = g + (size_t)idx[0][a] * p->n[1];
                for (int b = 0; b < T; ++b) gr[idx[1][b]] += va * w[1][b];
            }
        } else {
            for (int a = 0; a < T; ++a)
                for (int b = 0; b < T; ++b) {
                    cplx vb = fj * (w[0][a] * w[1][b]);
                    cplx *gr = g + ((size_t)idx[0][a] * p->n[1] + idx[1][b]) * p->n[2];
                    for (int c = 0; c < T; ++c) gr[idx[2][c]] += vb * w[2][c];
                }
        }
    }
    fft_nd(g, p->d, p->n, +1);
    int i[3];
    for (size_t k = 0; k < p->Ntot; ++k) {
        unravel(k, p->d, p->N, i);
        double s = 1.0;
        for (int t = 0; t < p->d; ++t) s *= p->phihut_inv[t][i[t]];
        fhat[k] = g[grid_pos(p, i)] * s;
    }
    free(g);
}

/* ------------------------------------------------------------------ */
/* Direct NDFT (exact operator)                                         */
/*   f_j = sum_k fhat_k exp(-2 pi i k.x_j),  fhat_k = sum_j f_j exp(+..)*/
/* ------------------------------------------------------------------ */
void orc_ndft_trafo(int d, const int *N, long M, const double *x,
                    const double *fhat_in, double *f_out, int nthreads)
{
    const cplx *fhat = (const cplx *)fhat_in;
    cplx *f = (cplx *)f_out;
    size_t Ntot = 1; for (int t = 0; t < d; ++t) Ntot *= (size_t)N[t];
    (void)nthreads;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads > 0 ? nthreads : 1)
    for (long j = 0; j < M; ++j) {
        cplx *e[3];
        for (int t = 0; t < d; ++t) {
            e[t] = (cplx *)malloc(sizeof(cplx) * (size_t)N[t]);
            for (int i = 0; i < N[t]; ++i) {
                double a = -2.0 * M_PI * (double)(i - N[t] / 2) * x[(size_t)j * d + t];
                e[t][i] = cos(a) + I * sin(a);
            }
        }
        cplx acc = 0;
        if (d == 1) {
            for (int a = 0; a < N[0]; ++a) acc += fhat[a] * e[0][a];
        } else if (d == 2) {
            for (int a = 0; a < N[0]; ++a) {
                cplx row = 0; const cplx *fr = fhat + (size_t)a * N[1];
                for (int b = 0; b < N[1]; ++b) row += fr[b] * e[1][b];
                acc += row * e[0][a];
            }
        } else {
            for (int a = 0; a < N[0]; ++a) {
                cplx pl = 0;
                for (int b = 0; b < N[1]; ++b) {
                    cplx row = 0; const cplx *fr = fhat + ((size_t)a * N[1] + b) * N[2];
                    for (int c = 0; c < N[2]; ++c) row += fr[c] * e[2][c];
                    pl += row * e[1][b];
                }
                acc += pl * e[0][a];
            }
        }
        f[j] = acc;
        for (int t = 0; t < d; ++t) free(e[t]);
    }
    (void)Ntot;
}

void orc_ndft_adjoint(int d, const int *N, long M, const double *x,
                      const double *f_in, double *fhat_out, int nthreads)
{
    const cplx *f = (const cplx *)f_in;
    cplx *fhat = (cplx *)fhat_out;
    size_t Ntot = 1; for (int t = 0; t < d; ++t) Ntot *= (size_t)N[t];
    (void)nthreads;
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
    for (size_t k = 0; k < Ntot; ++k) {
        int i[3]; size_t r = k;
        for (int t = d - 1; t >= 0; --t) { i[t] = (int)(r % (size_t)N[t]); r /= (size_t)N[t]; }
        cplx acc = 0;
        for (long j = 0; j < M; ++j) {
            double ph = 0;
            for (int t = 0; t < d; ++t) ph += (double)(i[t] - N[t] / 2) * x[(size_t)j * d + t];
            double a = 2.0 * M_PI * ph;
            acc += f[j] * (cos(a) + I * sin(a));
        }
        fhat[k] = acc;
    }
}

/* ------------------------------------------------------------------ */
/* Damping mask What (NFFTTraits.hpp:225-260): 1 inside the circle or  */
/* sphere of radius N/2 around index N/2 (N = N[0] for every axis).    */
/* ------------------------------------------------------------------ */
void orc_damp_mask(int d, const int *N, double *what)
{
    const int n0 = N[0], NH = (int)(0.5 * n0);
    size_t tot = 1; for (int t = 0; t < d; ++t) tot *= (size_t)n0;
    int i[3];
    int dims[3] = {n0, n0, n0};
    for (size_t k = 0; k < tot; ++k) {
        unravel(k, d, dims, i);
        double s = 0;
        for (int t = 0; t < d; ++t) { double q = (double)(i[t] - NH); s += q * q; }
        what[k] = (sqrt(s) > (double)NH) ? 0.0 : 1.0;
    }
}

/* ------------------------------------------------------------------ */
/* CGNR inverse NFFT (the reference's NFFT::Adjoint)                   */
/* Minimises ||y - A fhat||_W with damping What on the search          */
/* directions; zero start; stops before a step when the W-weighted     */
/* squared residual is below eps (absolute).                           */
/* ------------------------------------------------------------------ */
static double wdot(const cplx *a, const double *w, size_t n)
{
    double s = 0;
    for (size_t i = 0; i < n; ++i) {
        double q = creal(a[i]) * creal(a[i]) + cimag(a[i]) * cimag(a[i]);
        s += (w ? w[i] : 1.0) * q;
    }
    return s;
}

int orc_itrafo(const orc_nfft *p, const double *y_in, const double *w,
               const double *what, int maxit, double eps, double *fhat_out,
               double *dot_r_out)
{
    const size_t M = (size_t)p->M, Nt = p->Ntot;
    const cplx *y = (const cplx *)y_in;
    cplx *f = (cplx *)fhat_out;
    cplx *r = (cplx *)malloc(sizeof(cplx) * (M ? M : 1));
    cplx *v = (cplx *)malloc(sizeof(cplx) * (M ? M : 1));
    cplx *wr = (cplx *)malloc(sizeof(cplx) * (M ? M : 1));
    cplx *z = (cplx *)malloc(sizeof(cplx) * Nt);
    cplx *pp = (cplx *)malloc(sizeof(cplx) * Nt);
    cplx *tmp = (cplx *)malloc(sizeof(cplx) * Nt);
    for (size_t k = 0; k < Nt; ++k) f[k] = 0;
    /* r = y - A*0 = y */
    for (size_t j = 0; j < M; ++j) r[j] = y[j];
    double dot_r = wdot(r, w, M);
    for (size_t j = 0; j < M; ++j) wr[j] = r[j] * (w ? w[j] : 1.0);
    orc_nfft_adjoint(p, (const double *)wr, (double *)z);
    for (size_t k = 0; k < Nt; ++k) pp[k] = z[k];
    double dot_z = wdot(z, what, Nt);
    int steps = 0;
    for (int l = 0; l < maxit; ++l) {
        if (dot_r < eps) break;
        for (size_t k = 0; k < Nt; ++k) tmp[k] = pp[k] * (what ? what[k] : 1.0);
        orc_nfft_trafo(p, (const double *)tmp, (double *)v);
        double dot_v = wdot(v, w, M);
        double alpha = dot_z / dot_v;
        for (size_t k = 0; k < Nt; ++k) f[k] += alpha * tmp[k];
        for (size_t j = 0; j < M; ++j) r[j] -= alpha * v[j];
        dot_r = wdot(r, w, M);
        for (size_t j = 0; j < M; ++j) wr[j] = r[j] * (w ? w[j] : 1.0);
        orc_nfft_adjoint(p, (const double *)wr, (double *)z);
        double dot_z_old = dot_z;
        dot_z = wdot(z, what, Nt);
        double beta = dot_z / dot_z_old;
        for (size_t k = 0; k < Nt; ++k) pp[k] = beta * pp[k] + z[k];
        ++steps;
    }
    if (dot_r_out) *dot_r_out = dot_r;
    free(r); free(v); free(wr); free(z); free(pp); free(tmp);
    return steps;
}

/* ------------------------------------------------------------------ */
/* SENSE operators over NC coils sharing one trajectory                 */
/* ------------------------------------------------------------------ */

/* I = 1 / (sqrt(sum_c |S_c|^2) + 1e-9)   (MRI.hpp:7-29, sqroot = true) */
void orc_intensity_map(long nvox, int nc, const double *S_in, double *I_out)
{
    const cplx *S = (const cplx *)S_in;
    for (long i = 0; i < nvox; ++i) {
        double s = 0;
        for (int c = 0; c < nc; ++c) {
            cplx v = S[(size_t)c * nvox + i];
            s += creal(v) * creal(v) + cimag(v) * cimag(v);
        }
        I_out[i] = 1.0 / (sqrt(s) + 1.0e-9);
    }
}

/* y_c = A (S_c . x)   (NCSENSE.hpp:310-348) */
void orc_sense_trafo(const orc_nfft *p, int nc, const double *S_in,
                     const double *x_in, double *y_out, int nthreads)
{
    const cplx *S = (const cplx *)S_in, *x = (const cplx *)x_in;
    cplx *y = (cplx *)y_out;
    const size_t Nt = p->Ntot, M = (size_t)p->M;
    (void)nthreads;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
    for (int c = 0; c < nc; ++c) {
        cplx *t = (cplx *)malloc(sizeof(cplx) * Nt);
        for (size_t k = 0; k < Nt; ++k) t[k] = S[(size_t)c * Nt + k] * x[k];
        orc_nfft_trafo(p, (const double *)t, (double *)(y + (size_t)c * M));
        free(t);
    }
}

/* codeare's E^H:  x = I . sum_c conj(S_c) . itrafo_c(y_c)   (NCSENSE.hpp:289-299) */
void orc_sense_adjoint_codeare(const orc_nfft *p, int nc, const double *S_in,
                               const double *Imap, const double *w,
                               const double *what, int maxit, double eps,
                               const double *y_in, double *x_out, int nthreads)
{
    const cplx *S = (const cplx *)S_in, *y = (const cplx *)y_in;
    cplx *x = (cplx *)x_out;
    const size_t Nt = p->Ntot, M = (size_t)p->M;
    cplx *b = (cplx *)malloc(sizeof(cplx) * Nt * (size_t)nc);
    (void)nthreads;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
    for (int c = 0; c < nc; ++c)
        orc_itrafo(p, (const double *)(y + (size_t)c * M), w, what, maxit, eps,
                   (double *)(b + (size_t)c * Nt), NULL);
    for (size_t k = 0; k < Nt; ++k) {
        cplx acc = 0;
        for (int c = 0; c < nc; ++c) acc += b[(size_t)c * Nt + k] * conj(S[(size_t)c * Nt + k]);
        x[k] = acc * Imap[k];
    }
    free(b);
}

/* true adjoint E^H W:  x = sum_c conj(S_c) . A^H (w . y_c) */
void orc_sense_adjoint(const orc_nfft *p, int nc, const double *S_in,
                       const double *w, const double *y_in, double *x_out,
                       int nthreads)
{
    const cplx *S = (const cplx *)S_in, *y = (const cplx *)y_in;
    cplx *x = (cplx *)x_out;
    const size_t Nt = p->Ntot, M = (size_t)p->M;
    cplx *b = (cplx *)malloc(sizeof(cplx) * Nt * (size_t)nc);
    (void)nthreads;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
    for (int c = 0; c < nc; ++c) {
        cplx *t = (cplx *)malloc(sizeof(cplx) * (M ? M : 1));
        for (size_t j = 0; j < M; ++j) t[j] = y[(size_t)c * M + j] * (w ? w[j] : 1.0);
        orc_nfft_adjoint(p, (const double *)t, (double *)(b + (size_t)c * Nt));
        free(t);
    }
    for (size_t k = 0; k < Nt; ++k) {
        cplx acc = 0;
        for (int c = 0; c < nc; ++c) acc += b[(size_t)c * Nt + k] * conj(S[(size_t)c * Nt + k]);
        x[k] = acc;
    }
    free(b);
}

/* ------------------------------------------------------------------ */
/* CGLS outer loop in codeare semantics (CGLS.hpp:30-59):              */
/*   p = A/b; r = p; rn = xn = Re<r,p>; loop: res = rn/xn, break on     */
/*   NaN or res <= cgeps; q = A/(A*p) + lambda p; ts = rn/Re<p,q>;      */
/*   x += ts p; r -= ts q; p = r + (rn_new/rn) p.                       */
/* refprec != 0 rounds every vector to FP32 after each step and         */
/* accumulates the dot products sequentially in complex<float>, as the  */
/* reference does (Lapack.hpp:619-624); refprec = 0 keeps FP64.          */
/* Returns the number of residual checks made; res_hist gets them.      */
/* ------------------------------------------------------------------ */
static void round_f32(cplx *a, size_t n)
{
    for (size_t i = 0; i < n; ++i) a[i] = (double)(float)creal(a[i]) + I * (double)(float)cimag(a[i]);
}

static double re_dotc(const cplx *a, const cplx *b, size_t n, int refprec)
{
    if (refprec) {
        float sr = 0.f, si = 0.f;
        for (size_t i = 0; i < n; ++i) {
            float ar = (float)creal(a[i]), ai = -(float)cimag(a[i]);
            float br = (float)creal(b[i]), bi = (float)cimag(b[i]);
            float pr = ar * br - ai * bi, pi = ar * bi + ai * br;
            sr += pr; si += pi;
        }
        (void)si;
        return (double)sr;
    }
    double s = 0;
    for (size_t i = 0; i < n; ++i) s += creal(a[i]) * creal(b[i]) + cimag(a[i]) * cimag(b[i]);
    return s;
}

int orc_cgls_codeare(const orc_nfft *p, int nc, const double *S, const double *Imap,
                     const double *w, const double *what, int ftiter, double fteps,
                     int cgiter, double cgeps, double lambda, const double *y,
                     double *x_out, double *res_hist, int refprec, int nthreads)
{
    const size_t Nt = p->Ntot, M = (size_t)p->M;
    cplx *x = (cplx *)x_out;
    cplx *pp = (cplx *)malloc(sizeof(cplx) * Nt);
    cplx *r = (cplx *)malloc(sizeof(cplx) * Nt);
    cplx *q = (cplx *)malloc(sizeof(cplx) * Nt);
    cplx *ks = (cplx *)malloc(sizeof(cplx) * M * (size_t)nc);
    orc_sense_adjoint_codeare(p, nc, S, Imap, w, what, ftiter, fteps, y, (double *)pp, nthreads);
    if (refprec) round_f32(pp, Nt);
    if (cgiter == 0) { memcpy(x, pp, sizeof(cplx) * Nt); free(pp); free(r); free(q); free(ks); return 0; }
    memcpy(r, pp, sizeof(cplx) * Nt);
    double rn = re_dotc(r, pp, Nt, refprec), xn = rn;
    if (refprec) { rn = (float)rn; xn = (float)xn; }
    for (size_t k = 0; k < Nt; ++k) x[k] = 0;
    int nres = 0;
    for (int i = 0; i < cgiter; ++i) {
        double res = rn / xn;
        if (refprec) res = (float)res;
        if (res_hist) res_hist[i] = res;
        nres = i + 1;
        if (isnan(res) || res <= cgeps) break;
        orc_sense_trafo(p, nc, S, (const double *)pp, (double *)ks, nthreads);
        if (refprec) round_f32(ks, M * (size_t)nc);
        orc_sense_adjoint_codeare(p, nc, S, Imap, w, what, ftiter, fteps, (const double *)ks, (double *)q, nthreads);
        if (refprec) round_f32(q, Nt);
        if (lambda != 0.0) for (size_t k = 0; k < Nt; ++k) q[k] += lambda * pp[k];
        if (refprec) round_f32(q, Nt);
        double ts = rn / re_dotc(pp, q, Nt, refprec);
        if (refprec) ts = (float)ts;
        for (size_t k = 0; k < Nt; ++k) { x[k] += ts * pp[k]; r[k] -= ts * q[k]; }
        if (refprec) { round_f32(x, Nt); round_f32(r, Nt); }
        double rno = rn;
        rn = re_dotc(r, r, Nt, refprec);
        if (refprec) rn = (float)rn;
        double beta = rn / rno;
        if (refprec) beta = (float)beta;
        for (size_t k = 0; k < Nt; ++k) pp[k] = r[k] + beta * pp[k];
        if (refprec) round_f32(pp, Nt);
    }
    free(pp); free(r); free(q); free(ks);
    return nres;
}

/* ------------------------------------------------------------------ */
/* Standard CG-SENSE: CG on (E^H W E + lambda) x = E^H W y, zero start, */
/* stop when ||r||/||r0|| <= tol or after maxit iterations.             */
/* Returns iterations performed; res_hist[i] = ||r_i||/||r_0||.          */
/* ------------------------------------------------------------------ */
int orc_cg_sense(const orc_nfft *p, int nc, const double *S, const double *w,
                 double lambda, int maxit, double tol, const double *y,
                 double *x_out, double *res_hist, int nthreads)
{
    const size_t Nt = p->Ntot, M = (size_t)p->M;
    cplx *x = (cplx *)x_out;
    cplx *r = (cplx *)malloc(sizeof(cplx) * Nt);
    cplx *pp = (cplx *)malloc(sizeof(cplx) * Nt);
    cplx *q = (cplx *)malloc(sizeof(cplx) * Nt);
    cplx *ks = (cplx *)malloc(sizeof(cplx) * M * (size_t)nc);
    orc_sense_adjoint(p, nc, S, w, y, (double *)r, nthreads);
    for (size_t k = 0; k < Nt; ++k) { x[k] = 0; pp[k] = r[k]; }
    double rr = re_dotc(r, r, Nt, 0), rr0 = rr;
    int it = 0;
    if (res_hist) res_hist[0] = 1.0;
    while (it < maxit && rr0 > 0 && sqrt(rr / rr0) > tol) {
        orc_sense_trafo(p, nc, S, (const double *)pp, (double *)ks, nthreads);
        orc_sense_adjoint(p, nc, S, w, (const double *)ks, (double *)q, nthreads);
        if (lambda != 0.0) for (size_t k = 0; k < Nt; ++k) q[k] += lambda * pp[k];
        double alpha = rr / re_dotc(pp, q, Nt, 0);
        for (size_t k = 0; k < Nt; ++k) { x[k] += alpha * pp[k]; r[k] -= alpha * q[k]; }
        double rr_new = re_dotc(r, r, Nt, 0);
        double beta = rr_new / rr;
        rr = rr_new;
        for (size_t k = 0; k < Nt; ++k) pp[k] = r[k] + beta * pp[k];
        ++it;
        if (res_hist) res_hist[it] = sqrt(rr / rr0);
    }
    free(r); free(pp); free(q); free(ks);
    return it;
}

/* ------------------------------------------------------------------ */
/* Per-coil batches (one OpenMP thread per coil, as the reference's    */
/* NCSENSE runs one NFFT plan per thread, NCSENSE.hpp:290, 335).       */
/* ------------------------------------------------------------------ */
void orc_nfft_trafo_batch(const orc_nfft *p, int nc, const double *fhat, double *f, int nthreads)
{
    (void)nthreads;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
    for (int c = 0; c < nc; ++c)
        orc_nfft_trafo(p, fhat + 2 * (size_t)c * p->Ntot, f + 2 * (size_t)c * (size_t)p->M);
}

void orc_nfft_adjoint_batch(const orc_nfft *p, int nc, const double *f, double *fhat, int nthreads)
{
    (void)nthreads;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
    for (int c = 0; c < nc; ++c)
        orc_nfft_adjoint(p, f + 2 * (size_t)c * (size_t)p->M, fhat + 2 * (size_t)c * p->Ntot);
}
