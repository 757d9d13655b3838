// cgs_plan.cu -- the plan object and the C ABI (include/cgs.h).
//
// Host orchestration only: every arithmetic step runs in the kernels of
// cgs_fft.cu, cgs_grid.cu and cgs_vec.cu on the plan's stream.  Device data
// layouts (all complex float):
//   grid       [n0][n1][n2][NC]       oversampled grid, coil innermost
//   k-space    [s][NC]                nodes in tile-sorted order s, coil innermost
//   coil image [p][NC]                image pixel p (NFFT order), coil innermost
//   image      [p]
// The caller's layouts (coil slowest, nodes in trajectory order) are converted
// at the boundary only.
#include "cgs_internal.cuh"
#include "cgs_tc05.cuh"

#include <algorithm>
#include <thread>
#include <initializer_list>
#include <atomic>
#include <chrono>
#include <complex>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

namespace cgs {

static thread_local std::string g_last_error;
static std::atomic<int64_t> g_launches{0};

void set_error(const std::string &msg) { g_last_error = msg; }
void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// per-kernel event profiler (off unless cgs_profile_enable(1))
namespace {
struct ProfRec { int cat; cudaEvent_t a, b; };
std::mutex g_prof_mu;
bool g_prof_on = false;
std::vector<ProfRec> g_prof_recs;
std::vector<cudaEvent_t> g_prof_pool;
int g_prof_open = -1;
double g_prof_ms[PROF_NCAT] = {0, 0, 0};
int64_t g_prof_cnt[PROF_NCAT] = {0, 0, 0};

cudaEvent_t prof_event()
{
    if (!g_prof_pool.empty()) { cudaEvent_t e = g_prof_pool.back(); g_prof_pool.pop_back(); return e; }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void prof_drain()
{
    for (auto &r : g_prof_recs) {
        float ms = 0.f;
        if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
            g_prof_ms[r.cat] += ms;
            g_prof_cnt[r.cat] += 1;
        }
        g_prof_pool.push_back(r.a);
        g_prof_pool.push_back(r.b);
    }
    g_prof_recs.clear();
}
}  // namespace

static bool capturing(cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
}

void prof_begin(int cat, cudaStream_t st)
{
    if (!g_prof_on || capturing(st)) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (g_prof_recs.size() > 4096) prof_drain();
    ProfRec r{cat, prof_event(), prof_event()};
    cudaEventRecord(r.a, st);
    g_prof_recs.push_back(r);
    g_prof_open = (int)g_prof_recs.size() - 1;
}

void prof_end(int cat, cudaStream_t st)
{
    if (!g_prof_on || capturing(st)) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (g_prof_open >= 0 && g_prof_recs[g_prof_open].cat == cat) cudaEventRecord(g_prof_recs[g_prof_open].b, st);
    g_prof_open = -1;
}

// modified Bessel I0 by its power series, FP64 (host; used for 1/phihut tables)
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

static bool factorize(int n, int *fac, int *nf)
{
    int r = n, k = 0;
    while (r % 8 == 0 && k < 12) { fac[k++] = 8; r /= 8; }
    while (r % 4 == 0 && k < 12) { fac[k++] = 4; r /= 4; }
    while (r % 2 == 0 && k < 12) { fac[k++] = 2; r /= 2; }
    const int primes[] = {3, 5, 7};
    for (int q : primes)
        while (r % q == 0 && k < 12) { fac[k++] = q; r /= q; }
    *nf = k;
    return r == 1;
}

namespace tunek {
// deterministic scratch values in [-0.5, 0.5) for timing runs
__global__ void fill_pattern_kernel(float2 *a, int64_t n, uint32_t seed)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t h = (uint32_t)i * 2654435761u ^ seed;
        h ^= h >> 15; h *= 2246822519u; h ^= h >> 13; h *= 3266489917u; h ^= h >> 16;
        a[i] = make_float2((float)(h & 0xffff) / 65536.f - 0.5f, (float)(h >> 16) / 65536.f - 0.5f);
    }
}
}  // namespace tunek

namespace toepk {
__global__ void toep_prepare_kernel(float2 *T, int d, int n0, int n1, int n2)
{
    const int64_t tot = (int64_t)n0 * n1 * n2;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
        const int i2 = (int)(e % n2), i1 = (int)((e / n2) % n1), i0 = (int)(e / ((int64_t)n1 * n2));
        bool edge = (i0 == 0) || (i1 == 0);
        if (d == 3) edge = edge || (i2 == 0);
        if (edge) T[e] = make_float2(0.f, 0.f);
    }
}

__global__ void toep_real_kernel(const float2 *K, float *out, int64_t tot, float scale)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x)
        out[e] = K[e].x * scale;
}

}  // namespace toepk

}  // namespace cgs

using namespace cgs;

// Coil chunks of a host-buffer per-coil NFFT call: child plans, each holding
// a contiguous range of the caller's coil-major coils and sharing the parent's
// node tables, so that one chunk's host copies overlap the other chunks'
// kernels.  Copies to the device run in order on `in`, copies to the host on
// `out`, each chunk's kernels on its child's stream.  Built on the first
// host-buffer call, dropped whenever the trajectory, the weights or the tuning
// change.
struct HostChunks {
    std::vector<cgs_plan *> plans;
    std::vector<int> c0;  // first coil of each chunk (plans.size() + 1 entries)
    cudaStream_t in = nullptr, out = nullptr;
    cudaEvent_t fork = nullptr, done = nullptr;
    std::vector<cudaEvent_t> copied, computed;
    bool sens = false;    // the children hold their coils of the parent's sensitivities
};

struct cgs_plan {
    int d = 0, N[3] = {1, 1, 1}, n[3] = {1, 1, 1}, m = 1, nc = 1;
    // frames (NCSENSE dim4 x dim5, NCSENSE.hpp:141-166): F child plans with one
    // trajectory each and the same sensitivities and weights.  The parent's
    // vectors stack the frames (image Nt = F * Ntf, k-space M = F * Mf nodes,
    // frame-major); the operator building blocks run per child on the parent's
    // stream, so the CG machinery above them is unchanged.
    int F = 1;
    int64_t Mf = 0, Ntf = 0;
    std::vector<cgs_plan *> fr;
    // host-buffer pipeline of the per-coil NFFT (one frame): one chunk set for
    // the forward and one for the adjoint (their best chunk counts differ)
    HostChunks hcf, hca;
    bool shared_nodes = false;   // a coil chunk: the node tables belong to its parent
    double alpha = 1.0;
    int64_t M = 0, Nt = 1, ntot = 1;
    int device = 0;
    cudaStream_t stream = nullptr;

    // per-dimension FFT twiddles and deapodisation 1/phihut
    float2 *tw[3] = {nullptr, nullptr, nullptr};
    int fac[3][12] = {}, nfac[3] = {0, 0, 0};
    float *deap[3] = {nullptr, nullptr, nullptr};

    // trajectory
    bool have_k = false, have_w = false, have_s = false;
    float4 *nodes = nullptr;
    int *perm = nullptr;   // trajectory node at each sorted position
    int *iperm = nullptr;  // sorted position of each trajectory node
    float *w = nullptr;
    int4 *work = nullptr;
    int nwork = 0;
    GridGeom geom{};
    // 2-D output-stationary spreading: per-patch node lists and weight tables
    int2 *nodeU = nullptr;
    float *nodeW = nullptr;
    int *pentries = nullptr;
    int4 *pwork = nullptr, *pmulti = nullptr;
    // tcgen05 spreading: per work item, blocks of 16 entries (patch weights, node indices)
    float *pw16 = nullptr;
    int *ps16 = nullptr, *pstage = nullptr;
    float2 *ppartial = nullptr;
    int pslots = 1;  // partial slots of the split patches (at least 1)
    PatchSet pset{};
    // 2-D tensor-core interpolation: node lists by 4 x 4 footprint-start bin
    int *ilist = nullptr;
    int4 *iwork = nullptr;
    int niwork = 0, ibx = 0;
    // mma.sync interpolation: per work item the nodes' padded window rows and offsets
    float *iwin = nullptr;
    int4 *imeta = nullptr;
    // 3-D tensor-core gridding: wrapped footprint starts per node (nodeW then
    // holds kW3 window weights per node, ilist / iwork the 4 x 4 x 4 bins,
    // pentries / pwork / pmulti the 4 x 4 x 4 patch lists)
    int4 *nodeU3 = nullptr;
    int iby = 0;

    // host copies of the trajectory and weights (the Toeplitz kernel is built from them)
    std::vector<float> k_host, w_host;
    cgs_tuning tune{};     // gridding decomposition (zeros: defaults)
    uint64_t gen = 0;      // bumped whenever captured graphs of this plan become stale
    // Toeplitz embedding of E^H W E (standard mode)
    bool toep_valid = false;
    int toep_weighted = -1;
    int n2[3] = {1, 1, 1};
    float2 *tw2[3] = {nullptr, nullptr, nullptr};
    int fac2[3][12] = {}, nfac2[3] = {0, 0, 0};
    float *toepK = nullptr;
    float2 *tA = nullptr, *tB = nullptr;

    // image-side maps
    float *mask = nullptr;   // damping mask What (N^d)
    float *imap = nullptr;   // intensity map I (N^d)
    float2 *sens = nullptr;  // [p][NC]

    // scratch
    float2 *grid = nullptr, *t1 = nullptr, *t2 = nullptr;
    float2 *ksY = nullptr, *ksR = nullptr, *ksV = nullptr;
    float2 *cF = nullptr, *cP = nullptr, *cZ = nullptr;
    float2 *vX = nullptr, *vR = nullptr, *vP = nullptr, *vQ = nullptr;
    float2 *ioA = nullptr, *ioB = nullptr;
    double *partial = nullptr, *dots = nullptr;  // dots: 8 arrays of NC
    int *active = nullptr;
    CGScalars *sc = nullptr;
    double *fpart = nullptr;        // per-block partials of the fused update-and-dot kernels
    unsigned int *ftick = nullptr;  // their completion ticket (zero between launches)
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // flexible CG state and graph
    float2 *vB = nullptr, *vZ = nullptr, *vO = nullptr, *vT = nullptr;
    float *dscale = nullptr;
    FCGScalars *fs = nullptr;
    // circulant preconditioner (2-D): floored T. Chan spectrum of the weighted
    // point-spread function, its lambda-dependent inverse, 1/sqrt(sum |S|^2),
    // two scratch images and N-point FFT twiddles per axis
    float *circ = nullptr, *circ_inv = nullptr, *csq = nullptr;
    float2 *vC = nullptr, *vCo = nullptr;
    float2 *twN[2] = {nullptr, nullptr};
    int facN[2][12] = {}, nfacN[2] = {0, 0};
    bool circ_valid = false;
    // codeare-mode CGLS with the Toeplitz kernel: T (mask p) per coil and the
    // second partial-sum buffer of the image-space CGNR
    float2 *cG = nullptr;
    double *partial2 = nullptr;
    cudaGraphExec_t fcg_exec = nullptr;
    int fg_src = -1, fg_toep = -1, fg_weighted = -1, fg_mode = -1;
    uint64_t fg_net = 0;
    int64_t fg_kpro = 0, fg_kbody = 0;
    // captured solve: prologue + while(iteration) as one CUDA graph
    cudaGraphExec_t solve_exec = nullptr;
    int sg_mode = -1, sg_toep = -1, sg_weighted = -1, sg_ftiter = -1;
    double sg_fteps = -1.0;
    int64_t sg_kpro = 0, sg_kbody = 0;

    double *dot_r() { return dots; }
    double *dot_z() { return dots + nc; }
    double *dot_v() { return dots + 2 * nc; }
    double *dz_new() { return dots + 3 * nc; }
    double *alpha_c() { return dots + 4 * nc; }
    double *beta_c() { return dots + 5 * nc; }
    double *scal() { return dots + 6 * nc; }  // single-image dots
};

namespace {

template <class T>
cgs_status dev_alloc(T **p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
    if (e != cudaSuccess) {
        set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
        *p = nullptr;
        return CGS_ERR_OOM;
    }
    return CGS_OK;
}

void dev_free(void *p)
{
    if (p) cudaFree(p);
}

// the gridding kernels' view of a plan's node tables
int *tc_flag();

NodeSet node_set(const cgs_plan *p)
{
    NodeSet ns{p->M, p->nodes, p->perm, p->w, p->nwork, p->work, p->nodeU, p->nodeW, p->ilist, p->iwork,
               p->niwork, p->ibx, p->nodeU3, p->iby, tc_flag(), p->iwin, p->imeta};
    return ns;
}

bool is_device_ptr(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

cudaStream_t pick_stream(cgs_plan *p, void *s) { return s ? (cudaStream_t)s : p->stream; }

// bring caller data onto the device (returns a device pointer)
cgs_status stage_in(const void *src, size_t bytes, void *staging, const void **dev, cudaStream_t st)
{
    if (is_device_ptr(src)) { *dev = src; return CGS_OK; }
    CGS_CUDA(cudaMemcpyAsync(staging, src, bytes, cudaMemcpyHostToDevice, st));
    *dev = staging;
    return CGS_OK;
}

// ---------------------------------------------------------------------------
// NFFT building blocks on device layouts
// ---------------------------------------------------------------------------
AxisPass base_pass(cgs_plan *p, int t)
{
    AxisPass a{};
    a.n = p->n[t];
    a.tw = p->tw[t];
    a.nfac = p->nfac[t];
    for (int i = 0; i < 12; ++i) a.fac[i] = p->fac[t][i];
    a.load_mode = LOAD_PLAIN;
    a.store_mode = STORE_PLAIN;
    a.o1_len = 1;
    return a;
}

// forward NFFT of all coils.  src_img: single image (expand with sens) when
// per_coil == 0, coil-minor per-coil images when 1, coil-major (the caller's
// layout) when 2.  mask may be null.  With
// `user` the result goes to the caller's layout (coil-major, trajectory
// order) instead of ks, by the interpolation itself where it can, else by a
// scatter after it.
// the FFT passes of the forward NFFT (one frame): images -> oversampled grid
cgs_status op_forward_grid(cgs_plan *p, const float2 *src_img, int per_coil, const float *mask, cudaStream_t st)
{
    const int d = p->d, nc = p->nc;
    // pass over the fastest image axis (t = d-1), from the image side
    {
        AxisPass a = base_pass(p, d - 1);
        int64_t outer = 1;
        for (int t = 0; t < d - 1; ++t) outer *= p->N[t];
        a.outer = outer; a.inner = nc; a.Lin = p->N[d - 1]; a.Lout = p->n[d - 1]; a.sign = -1; a.in_centred = 1;
        a.load_mode = LOAD_IMAGE;
        a.img = src_img; a.img_per_coil = per_coil ? 1 : 0;
        a.coil_major = per_coil == 2 ? p->Nt : 0;
        a.sens = per_coil ? nullptr : p->sens;
        a.mask = mask;
        a.deap_ax = p->deap[d - 1];
        a.deap_o1 = p->deap[d - 2]; a.o1_len = p->N[d - 2];
        a.deap_o0 = (d == 3) ? p->deap[0] : nullptr;
        a.dst = (d == 2) ? p->t1 : p->t1;
        CGS_TRY(launch_axis_pass(a, st));
    }
    if (d == 2) {
        AxisPass a = base_pass(p, 0);
        a.outer = 1; a.inner = (int64_t)p->n[1] * nc; a.Lin = p->N[0]; a.Lout = p->n[0]; a.sign = -1; a.in_centred = 1;
        a.src = p->t1; a.dst = p->grid;
        CGS_TRY(launch_axis_pass(a, st));
    } else {
        AxisPass a = base_pass(p, 1);
        a.outer = p->N[0]; a.inner = (int64_t)p->n[2] * nc; a.Lin = p->N[1]; a.Lout = p->n[1]; a.sign = -1; a.in_centred = 1;
        a.src = p->t1; a.dst = p->t2;
        CGS_TRY(launch_axis_pass(a, st));
        AxisPass b = base_pass(p, 0);
        b.outer = 1; b.inner = (int64_t)p->n[1] * p->n[2] * nc; b.Lin = p->N[0]; b.Lout = p->n[0]; b.sign = -1; b.in_centred = 1;
        b.src = p->t2; b.dst = p->grid;
        CGS_TRY(launch_axis_pass(b, st));
    }
    return CGS_OK;
}

// the interpolation of the forward NFFT: p's nodes from `grid` (any plan's
// grid of p's geometry) into ks, or into the caller's layout with `user`
cgs_status op_forward_interp(cgs_plan *p, const float2 *grid, float2 *ks, cudaStream_t st, float2 *user)
{
    NodeSet ns = node_set(p);
    bool direct = false;
    CGS_TRY(launch_interp(p->geom, ns, grid, ks, st, user, &direct));
    if (user && !direct) CGS_TRY(launch_scatter_ks(ks, p->perm, p->M, p->nc, user, st));
    return CGS_OK;
}

cgs_status op_forward(cgs_plan *p, const float2 *src_img, int per_coil, const float *mask, float2 *ks,
                      cudaStream_t st, float2 *user = nullptr)
{
    if (p->F > 1) {
        for (int f = 0; f < p->F; ++f)
            CGS_TRY(op_forward(p->fr[f], src_img + (per_coil ? f * p->Ntf * p->nc : f * p->Ntf), per_coil, mask,
                               ks + f * p->Mf * p->nc, st, user ? user + f * p->Mf * p->nc : nullptr));
        return CGS_OK;
    }
    CGS_TRY(op_forward_grid(p, src_img, per_coil, mask, st));
    return op_forward_interp(p, p->grid, ks, st, user);
}

// the FFT passes of the adjoint NFFT (one frame): p's grid -> per-coil
// images (deapodised), coil-minor or, with coil_major_out, coil-major
cgs_status op_adjoint_fft(cgs_plan *p, float2 *out, cudaStream_t st, bool coil_major_out)
{
    const int d = p->d, nc = p->nc;
    const float2 *cur = p->grid;

    if (d == 3) {
        AxisPass a = base_pass(p, 0);
        a.outer = 1; a.inner = (int64_t)p->n[1] * p->n[2] * nc; a.Lin = p->n[0]; a.Lout = p->N[0]; a.sign = +1; a.out_centred = 1;
        a.src = cur; a.dst = p->t2;
        CGS_TRY(launch_axis_pass(a, st));
        AxisPass b = base_pass(p, 1);
        b.outer = p->N[0]; b.inner = (int64_t)p->n[2] * nc; b.Lin = p->n[1]; b.Lout = p->N[1]; b.sign = +1; b.out_centred = 1;
        b.src = p->t2; b.dst = p->t1;
        CGS_TRY(launch_axis_pass(b, st));
    } else {
        AxisPass a = base_pass(p, 0);
        a.outer = 1; a.inner = (int64_t)p->n[1] * nc; a.Lin = p->n[0]; a.Lout = p->N[0]; a.sign = +1; a.out_centred = 1;
        a.src = cur; a.dst = p->t1;
        CGS_TRY(launch_axis_pass(a, st));
    }
    AxisPass c = base_pass(p, d - 1);
    int64_t outer = 1;
    for (int t = 0; t < d - 1; ++t) outer *= p->N[t];
    c.outer = outer; c.inner = nc; c.Lin = p->n[d - 1]; c.Lout = p->N[d - 1]; c.sign = +1; c.out_centred = 1;
    c.src = p->t1; c.dst = out;
    c.store_mode = STORE_DEAPOD;
    c.coil_major = coil_major_out ? p->Nt : 0;
    c.deap_ax = p->deap[d - 1];
    c.deap_o1 = p->deap[d - 2]; c.o1_len = p->N[d - 2];
    c.deap_o0 = (d == 3) ? p->deap[0] : nullptr;
    return launch_axis_pass(c, st);
}

// adjoint NFFT of all coils into per-coil images (deapodised): coil-minor,
// or coil-major (the caller's layout) with coil_major_out
cgs_status op_adjoint(cgs_plan *p, const float2 *ks, int weighted, float2 *out, cudaStream_t st,
                      bool coil_major_out = false)
{
    if (p->F > 1) {
        for (int f = 0; f < p->F; ++f)
            CGS_TRY(op_adjoint(p->fr[f], ks + f * p->Mf * p->nc, weighted, out + f * p->Ntf * p->nc, st,
                               coil_major_out));
        return CGS_OK;
    }
    const int d = p->d, nc = p->nc;
    NodeSet ns = node_set(p);
    if (d == 2) {
        // writes every grid point: no clearing pass
        CGS_TRY(launch_spread_patch(p->geom, p->pset, ks, p->w, weighted && p->w != nullptr, p->grid, st));
    } else if (p->pset.pd == 4) {
        // 3-D patches on the tensor cores: also writes every grid point
        CGS_TRY(launch_spread_patch3(p->geom, p->pset, ks, p->w, weighted && p->w != nullptr, p->grid, st));
    } else {
        CGS_TRY(launch_zero(p->grid, sizeof(float2) * (size_t)p->ntot * nc, st));
        CGS_TRY(launch_spread(p->geom, ns, ks, weighted && p->w != nullptr, p->grid, st));
    }
    return op_adjoint_fft(p, out, st, coil_major_out);
}

// CGNR inverse NFFT per coil (codeare's NFFT::Adjoint) on sorted k-space ksIn
// into coil-minor images cF.
cgs_status op_itrafo(cgs_plan *p, const float2 *ksIn, int maxit, double eps, cudaStream_t st)
{
    const int nc = p->nc;
    const int64_t M = p->M, Nt = p->Nt;
    const float *w = p->w;
    CGS_TRY(launch_zero(p->cF, sizeof(float2) * Nt * nc, st));
    CGS_CUDA(cudaMemcpyAsync(p->ksR, ksIn, sizeof(float2) * M * nc, cudaMemcpyDeviceToDevice, st));
    CGS_TRY(launch_coldot(p->ksR, p->ksR, w, M, nc, p->partial, p->dot_r(), st));
    CGS_TRY(op_adjoint(p, p->ksR, 1, p->cZ, st));
    CGS_CUDA(cudaMemcpyAsync(p->cP, p->cZ, sizeof(float2) * Nt * nc, cudaMemcpyDeviceToDevice, st));
    CGS_TRY(launch_coldot(p->cZ, p->cZ, p->mask, Nt, nc, p->partial, p->dot_z(), st));
    CGS_CUDA(cudaMemsetAsync(p->active, 0x01, sizeof(int) * nc, st));
    // Per step: A p (masked), alpha; f += alpha p, r -= alpha A p, dot_r and the
    // early-exit flag of the next step; A^H W r, beta; p = z + beta p.  The
    // reductions and their scalar steps are fused into three kernels (a coil
    // leaving after this step's update only skips the beta and p of this step,
    // which no later step reads).
    if (maxit > 0)
        CGS_TRY(launch_cgnr_scalars(0, nc, eps, p->active, p->dot_r(), p->dot_z(), p->dot_v(),
                                    p->dz_new(), p->alpha_c(), p->beta_c(), st));
    for (int l = 0; l < maxit; ++l) {
        CGS_TRY(op_forward(p, p->cP, 1, p->mask, p->ksV, st));
        CGS_TRY(launch_cgnr_fused(1, M, nc, w, p->ksV, nullptr, nullptr, nullptr, nullptr, 0, p->partial, p->ftick,
                                  p->dots, p->active, eps, st));
        CGS_TRY(launch_cgnr_fused(2, M, nc, w, p->ksR, p->ksV, p->cF, p->cP, p->mask, Nt, p->partial, p->ftick,
                                  p->dots, p->active, eps, st));
        CGS_TRY(op_adjoint(p, p->ksR, 1, p->cZ, st));
        CGS_TRY(launch_cgnr_fused(3, Nt, nc, p->mask, p->cZ, nullptr, nullptr, nullptr, nullptr, 0, p->partial,
                                  p->ftick, p->dots, p->active, eps, st));
        CGS_TRY(launch_xpby_cols(p->cP, p->cZ, p->beta_c(), p->active, Nt, nc, st));
    }
    return CGS_OK;
}

// codeare E^H: x = I . sum conj(S) . itrafo(ks)
cgs_status op_eh_codeare(cgs_plan *p, const float2 *ks, int ftiter, double fteps, float2 *x,
                         cudaStream_t st)
{
    if (p->F > 1) {  // per frame (NCSENSE.hpp:254-266)
        for (int f = 0; f < p->F; ++f)
            CGS_TRY(op_eh_codeare(p->fr[f], ks + f * p->Mf * p->nc, ftiter, fteps, x + f * p->Ntf, st));
        return CGS_OK;
    }
    CGS_TRY(op_itrafo(p, ks, ftiter, fteps, st));
    return launch_coil_combine(p->cF, p->sens, p->imap, p->Nt, p->nc, x, st);
}

// true E^H W: x = sum conj(S) . A^H (w ks)
cgs_status op_eh(cgs_plan *p, const float2 *ks, int weighted, float2 *x, cudaStream_t st)
{
    if (p->F > 1) {
        for (int f = 0; f < p->F; ++f)
            CGS_TRY(op_eh(p->fr[f], ks + f * p->Mf * p->nc, weighted, x + f * p->Ntf, st));
        return CGS_OK;
    }
    CGS_TRY(op_adjoint(p, ks, weighted, p->cF, st));
    return launch_coil_combine(p->cF, p->sens, nullptr, p->Nt, p->nc, x, st);
}

// bins and per-launch coil counts from the plan's tuning
void apply_tiles(cgs_plan *p)
{
    GridGeom &g = p->geom;
    g.T = (p->d == 2) ? (p->tune.tile > 0 ? p->tune.tile : 8) : 8;
    for (int t = 0; t < p->d; ++t)
        if (g.T > p->n[t]) g.T = p->n[t];
    for (int t = 0; t < 3; ++t) g.nt[t] = 1;
    for (int t = 0; t < p->d; ++t) g.nt[t] = (p->n[t] + g.T - 1) / g.T;
    g.icc = p->tune.interp_coils;
    g.scc = p->tune.spread_coils;
    const int ib = p->tune.interp_block;
    g.imma = (p->d == 2 && ib == 64) ? 2 : ((p->d == 2 && (ib == 16 || (ib == 0 && p->nc >= 4))) ? 1 : 0);
    if (p->d == 3) g.imma = (ib != 1 && grid3_mma_ok(g)) ? 1 : 0;
}

// Node lists of the 2-D tensor-core interpolation: sorted node indices grouped
// by the 4 x 4 bin (8 x 16 for the tcgen05 kernel) of their wrapped footprint
// start (the same wrap as the device's node tables), work items (one warp, or
// one CTA for tcgen05) of at most kInterpGroup (128) nodes of one bin, in bin
// order so that neighbouring work items read neighbouring grid regions.  `cc`
// holds floor(n x) per node in trajectory order.
cgs_status build_ibins(cgs_plan *p, const std::vector<int> &cc, const std::vector<int> &perm)
{
    const int n0 = p->n[0], n1 = p->n[1], m = p->m;
    // interp_block 64 (tcgen05): 8 x 16 bins, work items of up to 128 nodes
    const bool tc = p->tune.interp_block == 64;
    const int bh = tc ? 8 : 4, bw = tc ? 16 : 4, group = tc ? 128 : kInterpGroup;
    const int nby = (n0 + bh - 1) / bh, nbx = (n1 + bw - 1) / bw;
    const int64_t M = p->M;
    std::vector<int> bin(M), cnt((size_t)nby * nbx + 1, 0);
    auto wrap = [](int v, int n) { v %= n; return v < 0 ? v + n : v; };
    for (int64_t s = 0; s < M; ++s) {
        const int j = perm[s];
        const int u0 = wrap(cc[(size_t)j * 2] - m, n0), u1 = wrap(cc[(size_t)j * 2 + 1] - m, n1);
        bin[s] = (u0 / bh) * nbx + u1 / bw;
        cnt[bin[s] + 1]++;
    }
    for (size_t b = 0; b + 1 < cnt.size(); ++b) cnt[b + 1] += cnt[b];
    std::vector<int> list(M), fill(cnt.begin(), cnt.end() - 1);
    for (int64_t s = 0; s < M; ++s) list[fill[bin[s]]++] = (int)s;
    std::vector<int4> work;
    for (int b = 0; b < nby * nbx; ++b)
        for (int s0 = cnt[b]; s0 < cnt[b + 1]; s0 += group)
            work.push_back(make_int4(b, s0, std::min(group, cnt[b + 1] - s0), 0));
    dev_free(p->ilist);
    dev_free(p->iwork);
    dev_free(p->iwin);
    dev_free(p->imeta);
    p->ilist = nullptr;
    p->iwork = nullptr;
    p->iwin = nullptr;
    p->imeta = nullptr;
    CGS_TRY(dev_alloc(&p->ilist, (size_t)M));
    CGS_TRY(dev_alloc(&p->iwork, std::max<size_t>(work.size(), 1)));
    CGS_CUDA(cudaMemcpy(p->ilist, list.data(), sizeof(int) * M, cudaMemcpyHostToDevice));
    if (!work.empty()) CGS_CUDA(cudaMemcpy(p->iwork, work.data(), sizeof(int4) * work.size(), cudaMemcpyHostToDevice));
    p->niwork = (int)work.size();
    p->ibx = nbx;
    const int taps = 2 * m + 2;
    if (!tc && !work.empty() && taps <= 10 && p->nodeU && p->nodeW) {
        // the mma.sync kernel's window blocks: 16 nodes x 2 rows of taps + 7 floats per item
        CGS_TRY(dev_alloc(&p->iwin, work.size() * kInterpGroup * 2 * (size_t)(taps + 7)));
        CGS_TRY(dev_alloc(&p->imeta, work.size() * kInterpGroup));
        CGS_TRY(launch_interp_windows(p->geom, node_set(p), p->iwin, p->imeta, p->stream));
        CGS_CUDA(cudaStreamSynchronize(p->stream));
    }
    return CGS_OK;
}

// Per 4 x 4 patch (4 x 8 for one coil, 8 x 4 or 8 x 16 for the tensor-core
// variants) of the 2-D grid, the sorted indices of the nodes whose footprint
// (2m+2 taps per axis, wrapped) covers any point of the patch; work items of
// at most `chunk` nodes, crowded patches spread over several partial slots;
// node weights precomputed on the device.  `cc` holds each node's integer
// grid cell floor(n x) in trajectory order.
cgs_status build_patches(cgs_plan *p, const std::vector<int> &cc)
{
    const int n0 = p->n[0], n1 = p->n[1], m = p->m, taps = 2 * m + 2;
    // one coil: 4 x 8 patches, a point per lane; with 4 or more coils, spread_block 4:
    // 4 x 8 patches of 2 x 2 blocks and spread_block 2: 4 x 4 patches of 2 x 1 blocks
    // (four coil groups); spread_block 1: 4 x 4 patches, a point per lane, two coil groups
    // spread_block 8: 4 x 8 patches, one coil group, a point per lane
    // spread_block 16: 4 x 4 patches on the tensor cores (TF32 split, FP32
    // accumulation), the default for 4 to 7 coils; spread_block 64 (tcgen05),
    // the default from 8 coils up, where its coil-independent weight build
    // is shared by enough coils
    const int tb = p->tune.spread_block != 0 ? p->tune.spread_block : (p->nc >= 8 ? 64 : (p->nc >= 4 ? 16 : 1));
    // spread_block 32: 8 x 4 patches on the tensor cores (two m-tiles per warp);
    // spread_block 64: 8 x 16 patches on the 5th-generation tensor cores (tcgen05)
    const int blk = (tb == 16 || tb == 32 || tb == 64)
                        ? tb
                        : (p->nc == 1 ? 1 : ((tb == 8 || (p->nc >= 4 && (tb == 4 || tb == 2))) ? tb : 1));
    const bool tensor = (blk == 16 || blk == 32 || blk == 64);
    const int kPatchH = (blk == 32 || blk == 64) ? 8 : 4;
    const int kPatchW = blk == 64 ? 16 : ((!tensor && (p->nc == 1 || blk == 4 || blk == 8)) ? 8 : 4);
    const int npy = (n0 + kPatchH - 1) / kPatchH, npx = (n1 + kPatchW - 1) / kPatchW;
    const int64_t P = (int64_t)npy * npx, M = p->M;
    std::vector<int> perm(M);
    CGS_CUDA(cudaMemcpy(perm.data(), p->perm, sizeof(int) * M, cudaMemcpyDeviceToHost));
    auto axis_patches = [taps](int u, int n, int ph, int *out) {
        int k = 0;
        for (int i = 0; i < taps; ++i) {
            const int q = ((u + i) % n) / ph;
            bool seen = false;
            for (int j = 0; j < k; ++j) seen = seen || (out[j] == q);
            if (!seen) out[k++] = q;
        }
        return k;
    };
    std::vector<int64_t> cnt(P + 1, 0);
    std::vector<int> ru(M), cu(M);
    int rows[64], cols[64];
    for (int64_t s = 0; s < M; ++s) {
        const int j = perm[s];
        int u0 = (cc[(size_t)j * 2] - m) % n0; if (u0 < 0) u0 += n0;
        int u1 = (cc[(size_t)j * 2 + 1] - m) % n1; if (u1 < 0) u1 += n1;
        ru[s] = u0; cu[s] = u1;
        const int nr = axis_patches(u0, n0, kPatchH, rows), ncl = axis_patches(u1, n1, kPatchW, cols);
        for (int a = 0; a < nr; ++a)
            for (int b = 0; b < ncl; ++b) cnt[(int64_t)rows[a] * npx + cols[b] + 1]++;
    }
    for (int64_t q = 0; q < P; ++q) cnt[q + 1] += cnt[q];
    const int64_t E = cnt[P];
    if (E > 0x7fffffffLL) { set_error("patch lists too long"); return CGS_ERR_BAD_ARG; }
    std::vector<int> entries(E > 0 ? E : 1);
    std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
    for (int64_t s = 0; s < M; ++s) {
        const int nr = axis_patches(ru[s], n0, kPatchH, rows), ncl = axis_patches(cu[s], n1, kPatchW, cols);
        for (int a = 0; a < nr; ++a)
            for (int b = 0; b < ncl; ++b) entries[fill[(int64_t)rows[a] * npx + cols[b]]++] = (int)s;
    }
    // work items: a chunk bound that keeps every warp's list short
    const int64_t avg = std::max<int64_t>(1, E / std::max<int64_t>(P, 1));
    // the tcgen05 kernel (128-point patches, fixed per-item set-up) prefers
    // longer items: 3x the mean list, 256..1024
    const int chunk = p->tune.spread_chunk > 0 ? p->tune.spread_chunk
                      : blk == 64 ? (int)std::min<int64_t>(1024, std::max<int64_t>(256, 3 * avg))
                                  : (int)std::min<int64_t>(1024, std::max<int64_t>(64, 2 * avg));
    std::vector<int4> work, multi;
    int slots = 0;
    for (int64_t q = 0; q < P; ++q) {
        const int64_t a = cnt[q], c = cnt[q + 1] - cnt[q];
        const int64_t nch = std::max<int64_t>(1, (c + chunk - 1) / chunk);
        if (nch == 1) {
            work.push_back(make_int4((int)q, (int)a, (int)c, -1));
        } else {
            multi.push_back(make_int4((int)q, slots, (int)nch, 0));
            for (int64_t k = 0; k < nch; ++k) {
                const int64_t b = a + k * chunk;
                work.push_back(make_int4((int)q, (int)b, (int)std::min<int64_t>(chunk, a + c - b), slots++));
            }
        }
    }
    // longest lists first, so the long ones do not form the tail
    std::stable_sort(work.begin(), work.end(), [](const int4 &x, const int4 &y) { return x.z > y.z; });
    for (void *b : {(void *)p->nodeU, (void *)p->nodeW, (void *)p->pentries, (void *)p->pwork, (void *)p->pmulti,
                    (void *)p->ppartial, (void *)p->pw16, (void *)p->ps16, (void *)p->pstage}) dev_free(b);
    p->nodeU = nullptr; p->nodeW = nullptr; p->pentries = nullptr; p->pwork = nullptr; p->pmulti = nullptr;
    p->ppartial = nullptr; p->pw16 = nullptr; p->ps16 = nullptr; p->pstage = nullptr;
    CGS_TRY(dev_alloc(&p->nodeU, M));
    CGS_TRY(dev_alloc(&p->nodeW, (size_t)M * 2 * taps));
    CGS_TRY(dev_alloc(&p->pentries, entries.size()));
    CGS_TRY(dev_alloc(&p->pwork, work.size()));
    CGS_TRY(dev_alloc(&p->pmulti, std::max<size_t>(1, multi.size())));
    p->pslots = std::max(slots, 1);
    CGS_TRY(dev_alloc(&p->ppartial, (size_t)p->pslots * kPatchH * kPatchW * p->nc));
    CGS_CUDA(cudaMemcpy(p->pentries, entries.data(), sizeof(int) * entries.size(), cudaMemcpyHostToDevice));
    CGS_CUDA(cudaMemcpy(p->pwork, work.data(), sizeof(int4) * work.size(), cudaMemcpyHostToDevice));
    if (!multi.empty())
        CGS_CUDA(cudaMemcpy(p->pmulti, multi.data(), sizeof(int4) * multi.size(), cudaMemcpyHostToDevice));
    NodeSet ns = node_set(p);
    CGS_TRY(launch_node_weights(p->geom, ns, p->nodeU, p->nodeW, p->stream));
    CGS_CUDA(cudaStreamSynchronize(p->stream));
    PatchSet &ps = p->pset;
    ps.ph = kPatchH;
    ps.pw = kPatchW;
    ps.blk = blk;
    ps.npx = npx;
    ps.nwork = (int)work.size();
    ps.entries = p->pentries;
    ps.work = p->pwork;
    ps.nodeU = p->nodeU;
    ps.nodeW = p->nodeW;
    ps.partial = p->ppartial;
    ps.nmulti = (int)multi.size();
    ps.multi = p->pmulti;
    ps.err = tc_flag();
    ps.pw16 = nullptr; ps.ps16 = nullptr; ps.pstage = nullptr;
    if (blk == 64) {
        // the tcgen05 kernel's stage blocks: 16 entries each, per work item in
        // work order (patch weights computed on the device)
        std::vector<int> stage(work.size());
        int64_t blocks = 0;
        for (size_t t = 0; t < work.size(); ++t) {
            stage[t] = (int)blocks;
            blocks += (work[t].z + 15) / 16;
        }
        if (blocks > 0x7fffffffLL / 24) { set_error("patch lists too long"); return CGS_ERR_BAD_ARG; }
        CGS_TRY(dev_alloc(&p->pstage, std::max<size_t>(1, stage.size())));
        CGS_TRY(dev_alloc(&p->pw16, (size_t)std::max<int64_t>(1, blocks) * 24 * 16));
        CGS_TRY(dev_alloc(&p->ps16, (size_t)std::max<int64_t>(1, blocks) * 16));
        if (!stage.empty())
            CGS_CUDA(cudaMemcpy(p->pstage, stage.data(), sizeof(int) * stage.size(), cudaMemcpyHostToDevice));
        ps.pstage = p->pstage;
        CGS_TRY(launch_spread_tc_weights(p->geom, ps, p->pw16, p->ps16, p->stream));
        CGS_CUDA(cudaStreamSynchronize(p->stream));
        ps.pw16 = p->pw16;
        ps.ps16 = p->ps16;
    }
    return CGS_OK;
}

// 3-D tensor-core gridding (taps <= 10, every side >= 3 + taps): the node
// tables, the interpolation bins (nodes grouped by the 4 x 4 x 4 bin of their
// wrapped footprint start, work items of at most kInterpGroup nodes) and,
// unless spread_block 1 asks for the CUDA-core kernel, the spreading patch
// lists (per 4 x 4 x 4 patch the sorted indices of the nodes whose footprint
// covers it; work items of at most `chunk` entries, crowded patches spread
// over partial slots; a patch without nodes still gets an item, which writes
// its zeros).  `cc` holds floor(n x) per node in trajectory order, `perm` the
// trajectory node of each sorted position.
cgs_status build_grid3(cgs_plan *p, const std::vector<int> &cc, const std::vector<int> &perm)
{
    const int n0 = p->n[0], n1 = p->n[1], n2 = p->n[2], m = p->m, taps = 2 * m + 2;
    const int64_t M = p->M;
    auto wrap = [](int v, int n) { v %= n; return v < 0 ? v + n : v; };
    for (void *b : {(void *)p->iwin, (void *)p->imeta, (void *)p->nodeU3, (void *)p->nodeW, (void *)p->ilist, (void *)p->iwork, (void *)p->pentries,
                    (void *)p->pwork, (void *)p->pmulti, (void *)p->ppartial, (void *)p->pw16, (void *)p->ps16,
                    (void *)p->pstage}) dev_free(b);
    p->nodeU3 = nullptr; p->nodeW = nullptr; p->ilist = nullptr; p->iwork = nullptr;
    p->iwin = nullptr; p->imeta = nullptr;
    p->pentries = nullptr; p->pwork = nullptr; p->pmulti = nullptr; p->ppartial = nullptr;
    p->pw16 = nullptr; p->ps16 = nullptr; p->pstage = nullptr;
    p->niwork = 0;
    p->pset = PatchSet{};
    p->pslots = 1;
    std::vector<int> u((size_t)M * 3);
    for (int64_t s = 0; s < M; ++s) {
        const int j = perm[s];
        for (int t = 0; t < 3; ++t) u[(size_t)s * 3 + t] = wrap(cc[(size_t)j * 3 + t] - m, p->n[t]);
    }
    CGS_TRY(dev_alloc(&p->nodeU3, (size_t)M));
    CGS_TRY(dev_alloc(&p->nodeW, (size_t)M * kW3));
    {
        NodeSet ns = node_set(p);
        CGS_TRY(launch_node_weights3(p->geom, ns, p->nodeU3, p->nodeW, p->stream));
    }
    // interpolation bins
    const int nbz = (n0 + 3) / 4, nby = (n1 + 3) / 4, nbx = (n2 + 3) / 4;
    const int64_t NB = (int64_t)nbz * nby * nbx;
    {
        std::vector<int64_t> cnt(NB + 1, 0);
        std::vector<int> bin(M);
        for (int64_t s = 0; s < M; ++s) {
            const int *us = &u[(size_t)s * 3];
            bin[s] = (int)(((int64_t)(us[0] / 4) * nby + us[1] / 4) * nbx + us[2] / 4);
            cnt[bin[s] + 1]++;
        }
        for (int64_t b = 0; b < NB; ++b) cnt[b + 1] += cnt[b];
        std::vector<int> list(M > 0 ? M : 1);
        std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
        for (int64_t s = 0; s < M; ++s) list[fill[bin[s]]++] = (int)s;
        std::vector<int4> work;
        for (int64_t b = 0; b < NB; ++b)
            for (int64_t s0 = cnt[b]; s0 < cnt[b + 1]; s0 += kInterpGroup)
                work.push_back(make_int4((int)b, (int)s0, (int)std::min<int64_t>(kInterpGroup, cnt[b + 1] - s0), 0));
        CGS_TRY(dev_alloc(&p->ilist, list.size()));
        CGS_TRY(dev_alloc(&p->iwork, std::max<size_t>(work.size(), 1)));
        CGS_CUDA(cudaMemcpy(p->ilist, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice));
        if (!work.empty())
            CGS_CUDA(cudaMemcpy(p->iwork, work.data(), sizeof(int4) * work.size(), cudaMemcpyHostToDevice));
        p->niwork = (int)work.size();
        p->ibx = nbx;
        p->iby = nby;
    }
    if (p->tune.spread_block != 1) {
        // patches of the axis covering [u, u + taps) (mod n), each once
        auto axis_patches = [taps](int uu, int n, int *out) {
            int k = 0;
            for (int i = 0; i < taps; ++i) {
                const int q = ((uu + i) % n) / 4;
                bool seen = false;
                for (int j = 0; j < k; ++j) seen = seen || (out[j] == q);
                if (!seen) out[k++] = q;
            }
            return k;
        };
        const int64_t P = NB;  // patches have the bins' shape
        // nodes split into contiguous ranges, one host thread each: per-thread
        // counts, then each thread fills its own positions, so every list
        // keeps the sorted node order whatever the thread count
        const int nth = (int)std::max<int64_t>(1, std::min<int64_t>({16, (int64_t)std::thread::hardware_concurrency(),
                                                                      M / 65536 + 1}));
        std::vector<std::vector<int64_t>> tcnt(nth, std::vector<int64_t>(P, 0));
        auto walk = [&](int th, auto &&visit) {
            const int64_t s0 = M * th / nth, s1 = M * (th + 1) / nth;
            int pz[16], py[16], px[16];
            for (int64_t s = s0; s < s1; ++s) {
                const int *us = &u[(size_t)s * 3];
                const int kz = axis_patches(us[0], n0, pz), ky = axis_patches(us[1], n1, py),
                          kx = axis_patches(us[2], n2, px);
                for (int a = 0; a < kz; ++a)
                    for (int b = 0; b < ky; ++b) {
                        const int64_t row = ((int64_t)pz[a] * nby + py[b]) * nbx;
                        for (int c = 0; c < kx; ++c) visit(row + px[c], s);
                    }
            }
        };
        auto parallel = [&](auto &&body) {
            std::vector<std::thread> ts;
            for (int th = 1; th < nth; ++th) ts.emplace_back(body, th);
            body(0);
            for (auto &t : ts) t.join();
        };
        parallel([&](int th) {
            int64_t *c = tcnt[th].data();
            walk(th, [c](int64_t q, int64_t) { c[q]++; });
        });
        std::vector<int64_t> cnt(P + 1, 0);
        for (int64_t q = 0; q < P; ++q) {
            int64_t sum = 0;
            for (int th = 0; th < nth; ++th) sum += tcnt[th][q];
            cnt[q + 1] = cnt[q] + sum;
        }
        const int64_t E = cnt[P];
        if (E > 0x7fffffffLL) { set_error("3-D patch lists too long"); return CGS_ERR_BAD_ARG; }
        // per-thread start positions within each patch's list
        for (int64_t q = 0; q < P; ++q) {
            int64_t pos = cnt[q];
            for (int th = 0; th < nth; ++th) {
                const int64_t c = tcnt[th][q];
                tcnt[th][q] = pos;
                pos += c;
            }
        }
        std::vector<int> entries(E > 0 ? E : 1);
        parallel([&](int th) {
            int64_t *f = tcnt[th].data();
            int *e = entries.data();
            walk(th, [f, e](int64_t q, int64_t s) { e[f[q]++] = (int)s; });
        });
        const int64_t avg = std::max<int64_t>(1, E / std::max<int64_t>(P, 1));
        const int chunk = p->tune.spread_chunk > 0 ? p->tune.spread_chunk
                                                   : (int)std::min<int64_t>(2048, std::max<int64_t>(64, 2 * avg));
        std::vector<int4> work, multi;
        int slots = 0;
        for (int64_t q = 0; q < P; ++q) {
            const int64_t a = cnt[q], c = cnt[q + 1] - cnt[q];
            const int64_t nch = std::max<int64_t>(1, (c + chunk - 1) / chunk);
            if (nch == 1) {
                work.push_back(make_int4((int)q, (int)a, (int)c, -1));
            } else {
                multi.push_back(make_int4((int)q, slots, (int)nch, 0));
                for (int64_t k = 0; k < nch; ++k) {
                    const int64_t b = a + k * chunk;
                    work.push_back(make_int4((int)q, (int)b, (int)std::min<int64_t>(chunk, a + c - b), slots++));
                }
            }
        }
        std::stable_sort(work.begin(), work.end(), [](const int4 &x, const int4 &y) { return x.z > y.z; });
        CGS_TRY(dev_alloc(&p->pentries, entries.size()));
        CGS_TRY(dev_alloc(&p->pwork, std::max<size_t>(work.size(), 1)));
        CGS_TRY(dev_alloc(&p->pmulti, std::max<size_t>(1, multi.size())));
        p->pslots = std::max(slots, 1);
        CGS_TRY(dev_alloc(&p->ppartial, (size_t)p->pslots * 64 * p->nc));
        CGS_CUDA(cudaMemcpy(p->pentries, entries.data(), sizeof(int) * entries.size(), cudaMemcpyHostToDevice));
        if (!work.empty())
            CGS_CUDA(cudaMemcpy(p->pwork, work.data(), sizeof(int4) * work.size(), cudaMemcpyHostToDevice));
        if (!multi.empty())
            CGS_CUDA(cudaMemcpy(p->pmulti, multi.data(), sizeof(int4) * multi.size(), cudaMemcpyHostToDevice));
        PatchSet &ps = p->pset;
        ps.ph = 4; ps.pw = 4; ps.pd = 4; ps.blk = 16;
        ps.npx = nbx; ps.npy = nby;
        ps.nwork = (int)work.size();
        ps.entries = p->pentries;
        ps.work = p->pwork;
        ps.nodeU = nullptr;
        ps.nodeW = p->nodeW;
        ps.nodeU3 = p->nodeU3;
        ps.partial = p->ppartial;
        ps.nmulti = (int)multi.size();
        ps.multi = p->pmulti;
    }
    CGS_CUDA(cudaStreamSynchronize(p->stream));
    return CGS_OK;
}

// ---------------------------------------------------------------------------
// Toeplitz embedding of A^H W A (per coil, shared kernel):
//   (A^H W A f)_k = sum_k' T[k - k'] f_k',  T[d] = sum_j w_j exp(+2 pi i d.x_j),
// d in [-N, N)^d, computed once as the adjoint NFFT of the weights on a 2N
// image.  The circulant extension C (C = T with the unused d = -N faces
// zeroed, so C is Hermitian) has a real 2N-point DFT K; the operator is then
// pad(N -> 2N) . FFT . (K / (2N)^d) . IFFT . crop(2N -> N).
// ---------------------------------------------------------------------------
AxisPass toep_pass(cgs_plan *p, int t)
{
    AxisPass a{};
    a.n = p->n2[t];
    a.tw = p->tw2[t];
    a.nfac = p->nfac2[t];
    for (int i = 0; i < 12; ++i) a.fac[i] = p->fac2[t][i];
    a.load_mode = LOAD_PLAIN;
    a.store_mode = STORE_PLAIN;
    a.o1_len = 1;
    return a;
}

// Captured solve graphs hold the trajectory's work lists and the Toeplitz
// kernel by address: any change to those drops them (they are rebuilt on the
// next solve).
void drop_graphs(cgs_plan *p)
{
    p->gen++;
    if (p->solve_exec) { cudaGraphExecDestroy(p->solve_exec); p->solve_exec = nullptr; }
    if (p->fcg_exec) { cudaGraphExecDestroy(p->fcg_exec); p->fcg_exec = nullptr; }
}

// N-point FFT pass along axis t of the image grid (circulant preconditioner)
static cgs_status circ_twiddles(cgs_plan *p)
{
    for (int t = 0; t < 2; ++t) {
        if (p->twN[t]) continue;
        if (!factorize(p->N[t], p->facN[t], &p->nfacN[t])) {
            set_error("the circulant preconditioner needs image sides that factor into 2, 3, 5, 7");
            return CGS_ERR_BAD_ARG;
        }
        std::vector<float2> tw(p->N[t]);
        for (int i = 0; i < p->N[t]; ++i) {
            const double a = -2.0 * M_PI * (double)i / (double)p->N[t];
            tw[i] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        CGS_TRY(dev_alloc(&p->twN[t], (size_t)p->N[t]));
        CGS_CUDA(cudaMemcpy(p->twN[t], tw.data(), sizeof(float2) * tw.size(), cudaMemcpyHostToDevice));
    }
    return CGS_OK;
}

static AxisPass circ_pass(cgs_plan *p, int t)
{
    AxisPass a{};
    a.n = p->N[t];
    a.tw = p->twN[t];
    a.nfac = p->nfacN[t];
    for (int i = 0; i < 12; ++i) a.fac[i] = p->facN[t][i];
    a.load_mode = LOAD_PLAIN;
    a.store_mode = STORE_PLAIN;
    a.o1_len = 1;
    a.Lin = a.Lout = p->N[t];
    return a;
}

// in-place 2-D transform of an N0 x N1 image: axis 1 with `sign1`, then axis 0
// (forward; with kinv also multiplied by kinv[pos0][pos1] and transformed back)
static cgs_status circ_fft2(cgs_plan *p, float2 *v, int sign1, const float *kinv, cudaStream_t st)
{
    AxisPass a = circ_pass(p, 1);
    a.outer = p->N[0]; a.inner = 1; a.sign = sign1; a.src = v; a.dst = v;
    CGS_TRY(launch_axis_pass(a, st));
    if (sign1 > 0) return CGS_OK;
    AxisPass b = circ_pass(p, 0);
    b.outer = 1; b.inner = p->N[1]; b.sign = -1; b.src = v; b.dst = v;
    b.toep_k = kinv; b.toep_nc = 1;
    return launch_axis_pass(b, st);
}

// Floored T. Chan spectrum of the point-spread function T[2N0][2N1] (index
// d + N): fold onto the N-periodic grid, 2-D DFT, real part, floor at
// kCircFloor times its mean (the unsampled k-space corners and the gaps
// between spokes would otherwise give near-zero eigenvalues whose inverse
// amplifies noise).  Runs once per Toeplitz kernel.
constexpr double kCircFloor = 0.2;
static cgs_status build_circulant(cgs_plan *p, const float2 *T, cudaStream_t st)
{
    p->circ_valid = false;
    if (p->d != 2) return CGS_OK;
    CGS_TRY(circ_twiddles(p));
    const int64_t P = p->Nt;
    if (!p->vC) CGS_TRY(dev_alloc(&p->vC, (size_t)P));
    if (!p->circ) CGS_TRY(dev_alloc(&p->circ, (size_t)P));
    CGS_TRY(launch_circ_fold(T, p->N[0], p->N[1], p->vC, st));
    CGS_TRY(circ_fft2(p, p->vC, -1, nullptr, st));
    std::vector<float2> spec(P);
    CGS_CUDA(cudaMemcpyAsync(spec.data(), p->vC, sizeof(float2) * P, cudaMemcpyDeviceToHost, st));
    CGS_CUDA(cudaStreamSynchronize(st));
    double mean = 0.0;
    for (const float2 &v : spec) mean += (double)v.x;
    mean /= (double)P;
    const double floor = kCircFloor * std::max(mean, 0.0);
    std::vector<float> c(P);
    for (int64_t i = 0; i < P; ++i) c[i] = (float)std::max((double)spec[i].x, floor);
    CGS_CUDA(cudaMemcpy(p->circ, c.data(), sizeof(float) * P, cudaMemcpyHostToDevice));
    p->circ_valid = true;
    return CGS_OK;
}

// z = C(r) = csq . IFFT(kinv . FFT(csq . r)), kinv and csq set for the current
// lambda and sensitivities (fcg prologue or cgs_precond_apply); out may not alias r
// The transforms alone, in place on vC = csq . r (the flexible-CG loop bodies
// form vC in their residual update and apply the output scaling in their next
// kernel)
static cgs_status op_circ_core(cgs_plan *p, cudaStream_t st)
{
    CGS_TRY(circ_fft2(p, p->vC, -1, p->circ_inv, st));
    return circ_fft2(p, p->vC, +1, nullptr, st);
}

static cgs_status op_circ(cgs_plan *p, const float2 *r, float2 *out, cudaStream_t st)
{
    const int64_t P = p->Nt;
    CGS_TRY(launch_diag_scale(r, nullptr, p->csq, 1, P, p->vC, st));
    CGS_TRY(op_circ_core(p, st));
    return launch_diag_scale(p->vC, nullptr, p->csq, 1, P, out, st);
}

// the circulant's lambda- and coil-dependent factors from fs->cg.lambda
static cgs_status circ_prepare(cgs_plan *p, FCGScalars *fs, cudaStream_t st)
{
    const int64_t P = p->Nt;
    if (!p->csq) CGS_TRY(dev_alloc(&p->csq, (size_t)P));
    if (!p->circ_inv) CGS_TRY(dev_alloc(&p->circ_inv, (size_t)P));
    CGS_TRY(launch_coil_rsqrt(p->sens, P, p->nc, p->csq, st));
    CGS_TRY(launch_coldot(p->sens, p->sens, nullptr, P * p->nc, 1, p->partial, &fs->dsum, st));
    return launch_circ_kinv(p->circ, fs, P, p->circ_inv, st);
}

cgs_status build_toeplitz(cgs_plan *p, int weighted, cudaStream_t st)
{
    drop_graphs(p);
    const int d = p->d;
    int64_t T2 = 1;
    for (int t = 0; t < d; ++t) {
        p->n2[t] = 2 * p->N[t];
        if (!factorize(p->n2[t], p->fac2[t], &p->nfac2[t])) { set_error("2N must factor into 2, 3, 5, 7"); return CGS_ERR_BAD_ARG; }
        T2 *= p->n2[t];
        if (!p->tw2[t]) {
            std::vector<float2> tw(p->n2[t]);
            for (int i = 0; i < p->n2[t]; ++i) {
                const double a = -2.0 * M_PI * (double)i / (double)p->n2[t];
                tw[i] = make_float2((float)std::cos(a), (float)std::sin(a));
            }
            CGS_TRY(dev_alloc(&p->tw2[t], (size_t)p->n2[t]));
            CGS_CUDA(cudaMemcpy(p->tw2[t], tw.data(), sizeof(float2) * tw.size(), cudaMemcpyHostToDevice));
        }
    }
    const int64_t nc = p->nc;
    if (!p->tA) {
        // 2-D: [N0][2N1][NC]; 3-D: [N0][N1][2N2][NC] and [N0][2N1][2N2][NC]
        int64_t a = (d == 2) ? (int64_t)p->N[0] * p->n2[1] : (int64_t)p->N[0] * p->N[1] * p->n2[2];
        CGS_TRY(dev_alloc(&p->tA, (size_t)(a * nc)));
        if (d == 3) CGS_TRY(dev_alloc(&p->tB, (size_t)((int64_t)p->N[0] * p->n2[1] * p->n2[2] * nc)));
        CGS_TRY(dev_alloc(&p->toepK, (size_t)T2));
    }
    // point-spread function through a one-coil plan on the 2N image
    cgs_plan_desc sd{};
    sd.rank = d;
    for (int t = 0; t < d; ++t) sd.N[t] = p->n2[t];
    sd.alpha = p->alpha; sd.m = p->m; sd.M = p->M; sd.ncoils = 1;
    cgs_plan *sub = nullptr;
    CGS_TRY(cgs_plan_create(&sub, &sd));
    float2 *wc = nullptr, *T = nullptr;
    cgs_status r = CGS_OK;
    if (d == 3) {
        // one spreading pass: the CUDA-core kernel, which needs no patch lists
        cgs_tuning once{};
        once.spread_block = 1;
        once.interp_block = 1;
        r = cgs_set_tuning(sub, &once);
    }
    if (r == CGS_OK) r = cgs_set_kspace(sub, p->k_host.data());
    if (r == CGS_OK) r = dev_alloc(&wc, (size_t)p->M);
    if (r == CGS_OK) r = dev_alloc(&T, (size_t)T2);
    if (r == CGS_OK) {
        std::vector<float2> wh(p->M);
        for (int64_t j = 0; j < p->M; ++j) wh[j] = make_float2(weighted ? p->w_host[j] : 1.f, 0.f);
        if (cudaMemcpy(wc, wh.data(), sizeof(float2) * wh.size(), cudaMemcpyHostToDevice) != cudaSuccess) r = CGS_ERR_CUDA;
    }
    if (r == CGS_OK) r = cgs_nfft_adjoint(sub, (const float *)wc, (float *)T, st);
    if (r == CGS_OK && cudaStreamSynchronize(st) != cudaSuccess) r = CGS_ERR_CUDA;
    cgs_plan_destroy(sub);
    if (r == CGS_OK) {
        toepk::toep_prepare_kernel<<<1024, 256, 0, st>>>(T, d, p->n2[0], p->n2[1], d == 3 ? p->n2[2] : 1);
        if (cudaGetLastError() != cudaSuccess) r = CGS_ERR_CUDA;
        count_launch();
    }
    if (r == CGS_OK && d == 2) r = build_circulant(p, T, st);
    // DFT of the circulant kernel: centred input (index d + N <-> position d mod 2N), full output
    for (int t = 0; t < d && r == CGS_OK; ++t) {
        AxisPass a = toep_pass(p, t);
        int64_t outer = 1, inner = 1;
        for (int u = 0; u < t; ++u) outer *= p->n2[u];
        for (int u = t + 1; u < d; ++u) inner *= p->n2[u];
        a.outer = outer; a.inner = inner; a.Lin = p->n2[t]; a.Lout = p->n2[t]; a.sign = -1;
        a.in_centred = 1; a.out_centred = 0;
        a.src = T; a.dst = T;  // in place: every CTA reads its columns before writing them
        r = launch_axis_pass(a, st);
    }
    if (r == CGS_OK) {
        toepk::toep_real_kernel<<<1024, 256, 0, st>>>(T, p->toepK, T2, (float)(1.0 / (double)T2));
        if (cudaGetLastError() != cudaSuccess) r = CGS_ERR_CUDA;
        count_launch();
    }
    if (r == CGS_OK && cudaStreamSynchronize(st) != cudaSuccess) r = CGS_ERR_CUDA;
    dev_free(wc);
    dev_free(T);
    if (r != CGS_OK) return r;
    p->toep_valid = true;
    p->toep_weighted = weighted;
    return CGS_OK;
}

// coil_out[p][c] = (A^H W A)(mask . u_c) through the Toeplitz kernel for all
// coils, u_c = S_c x (per_coil 0, x one image) or x_c (per_coil 1, x coil-minor)
cgs_status op_toeplitz_coils(cgs_plan *p, const float2 *x, int per_coil, const float *mask, float2 *coil_out,
                             cudaStream_t st)
{
    const int d = p->d, nc = p->nc;
    {   // pad the fastest axis: image -> [..][2N][NC], with the coil expansion
        AxisPass a = toep_pass(p, d - 1);
        int64_t outer = 1;
        for (int t = 0; t < d - 1; ++t) outer *= p->N[t];
        a.outer = outer; a.inner = nc; a.Lin = p->N[d - 1]; a.Lout = p->n2[d - 1]; a.sign = -1; a.in_centred = 1;
        a.load_mode = LOAD_IMAGE; a.img = x; a.img_per_coil = per_coil; a.sens = per_coil ? nullptr : p->sens;
        a.mask = mask;
        a.dst = p->tA;
        CGS_TRY(launch_axis_pass(a, st));
    }
    float2 *cur = p->tA;
    if (d == 3) {
        AxisPass a = toep_pass(p, 1);
        a.outer = p->N[0]; a.inner = (int64_t)p->n2[2] * nc; a.Lin = p->N[1]; a.Lout = p->n2[1]; a.sign = -1;
        a.in_centred = 1; a.src = p->tA; a.dst = p->tB;
        CGS_TRY(launch_axis_pass(a, st));
        cur = p->tB;
    }
    {   // slowest axis: FFT, multiply by K, inverse FFT, crop (in place)
        AxisPass a = toep_pass(p, 0);
        int64_t inner = nc;
        for (int t = 1; t < d; ++t) inner *= p->n2[t];
        a.outer = 1; a.inner = inner; a.Lin = p->N[0]; a.Lout = p->N[0]; a.sign = -1;
        a.in_centred = 1; a.out_centred = 1; a.src = cur; a.dst = cur;
        a.toep_k = p->toepK; a.toep_nc = nc;
        CGS_TRY(launch_axis_pass(a, st));
    }
    if (d == 3) {
        AxisPass a = toep_pass(p, 1);
        a.outer = p->N[0]; a.inner = (int64_t)p->n2[2] * nc; a.Lin = p->n2[1]; a.Lout = p->N[1]; a.sign = +1;
        a.out_centred = 1; a.src = p->tB; a.dst = p->tA;
        CGS_TRY(launch_axis_pass(a, st));
    }
    {   // crop the fastest axis back to the image
        AxisPass a = toep_pass(p, d - 1);
        int64_t outer = 1;
        for (int t = 0; t < d - 1; ++t) outer *= p->N[t];
        a.outer = outer; a.inner = nc; a.Lin = p->n2[d - 1]; a.Lout = p->N[d - 1]; a.sign = +1; a.out_centred = 1;
        a.src = p->tA; a.dst = coil_out;
        return launch_axis_pass(a, st);
    }
}

// out = sum_c conj(S_c) (A^H W A)(S_c x) through the Toeplitz kernel
cgs_status op_ehe_toeplitz(cgs_plan *p, const float2 *x, float2 *out, cudaStream_t st)
{
    CGS_TRY(op_toeplitz_coils(p, x, 0, nullptr, p->cF, st));
    return launch_coil_combine(p->cF, p->sens, nullptr, p->Nt, p->nc, out, st);
}

// codeare's E^H applied to E x (the CGLS step), all in image space: the
// per-coil CGNR inverse NFFT of y_c = A (S_c x) with A^H W A from the
// Toeplitz kernel (cgnr_img_kernel states the recurrences), then
// I . sum conj(S_c) f_c.  Same steps, early exits and frozen coils as
// op_itrafo; exact up to the NFFT approximation error (sigma >= 2, m >= 4).
cgs_status op_eh_codeare_ehx_toeplitz(cgs_plan *p, const float2 *x, int ftiter, double fteps, float2 *out,
                                      cudaStream_t st)
{
    const int nc = p->nc;
    const int64_t Nt = p->Nt;
    if (!p->cG) CGS_TRY(dev_alloc(&p->cG, (size_t)Nt * nc));
    if (!p->partial2) CGS_TRY(dev_alloc(&p->partial2, (size_t)dot_blocks() * std::max(nc, 1)));
    CGS_TRY(op_toeplitz_coils(p, x, 0, nullptr, p->cZ, st));           // z = A^H W y_c = T (S_c x)
    CGS_TRY(launch_zero(p->cF, sizeof(float2) * Nt * nc, st));
    CGS_TRY(launch_cgnr_img(0, Nt, nc, p->mask, x, p->sens, p->cZ, nullptr, nullptr, nullptr, p->partial,
                            p->partial2, p->ftick, p->dots, p->active, fteps, st));
    CGS_CUDA(cudaMemcpyAsync(p->cP, p->cZ, sizeof(float2) * Nt * nc, cudaMemcpyDeviceToDevice, st));
    CGS_CUDA(cudaMemsetAsync(p->active, 0x01, sizeof(int) * nc, st));
    if (ftiter > 0)
        CGS_TRY(launch_cgnr_scalars(0, nc, fteps, p->active, p->dot_r(), p->dot_z(), p->dot_v(), p->dz_new(),
                                    p->alpha_c(), p->beta_c(), st));
    for (int l = 0; l < ftiter; ++l) {
        CGS_TRY(op_toeplitz_coils(p, p->cP, 1, p->mask, p->cG, st));   // g = T (mask p)
        CGS_TRY(launch_cgnr_img(1, Nt, nc, p->mask, nullptr, nullptr, p->cZ, p->cG, p->cP, nullptr, p->partial,
                                p->partial2, p->ftick, p->dots, p->active, fteps, st));
        CGS_TRY(launch_cgnr_img(2, Nt, nc, p->mask, nullptr, nullptr, p->cZ, p->cG, p->cP, p->cF, p->partial,
                                p->partial2, p->ftick, p->dots, p->active, fteps, st));
        CGS_TRY(launch_xpby_cols(p->cP, p->cZ, p->beta_c(), p->active, Nt, nc, st));
    }
    return launch_coil_combine(p->cF, p->sens, p->imap, Nt, nc, out, st);
}

// One CG-SENSE iteration (either mode) on the plan's buffers.
// One CG-SENSE iteration (either mode) on the plan's buffers, ending with the
// loop test that sets the graph condition h.
cgs_status cg_iteration(cgs_plan *p, const cgs_solve_opts *o, cudaGraphConditionalHandle h, cudaStream_t st)
{
    const int64_t Nt = p->Nt;
    if (o->mode == CGS_MODE_CODEARE && o->toeplitz) {
        CGS_TRY(op_eh_codeare_ehx_toeplitz(p, p->vP, o->ftiter, o->fteps, p->vQ, st));
    } else if (o->mode == CGS_MODE_CODEARE) {
        CGS_TRY(op_forward(p, p->vP, 0, nullptr, p->ksV, st));
        CGS_TRY(op_eh_codeare(p, p->ksV, o->ftiter, o->fteps, p->vQ, st));
    } else if (o->toeplitz) {
        CGS_TRY(op_ehe_toeplitz(p, p->vP, p->vQ, st));
    } else {
        CGS_TRY(op_forward(p, p->vP, 0, nullptr, p->ksV, st));
        CGS_TRY(op_eh(p, p->ksV, o->weighted, p->vQ, st));
    }
    // q += lambda p, pq = Re <p, q>
    CGS_TRY(launch_axpy_dot(p->vQ, p->vP, &p->sc->lambda, &p->sc->done, Nt, p->fpart, p->ftick, &p->sc->pq, st));
    // x += ts p, r -= ts q, rn = |r|^2, loop test
    CGS_TRY(launch_cg_xr_rr(p->vX, p->vR, p->vP, p->vQ, p->sc, Nt, p->fpart, p->ftick, h, st));
    return launch_cg_update_p(p->vP, p->vR, p->sc, Nt, st);
}

// Capture the whole solve once per (mode, operator, weighting, inner CGNR
// setting): a prologue (E^H of the data, r = p, rn = xn, first check) and a
// while node whose body is one iteration followed by the check.  The check
// kernel decides on the device whether the loop continues, so a solve is one
// graph launch and one read-back.
// Appends one device-driven solve to graph g as an independent branch: the
// prologue (E^H y, r = p = that, first dot, check) and a WHILE node whose body
// is one CG iteration plus the check that sets its condition.  With
// init_in_graph the loop scalars are reset by a kernel (batch graphs);
// otherwise the caller uploads them before each launch.
cgs_status append_solve(cgs_plan *p, const cgs_solve_opts *o, cudaGraph_t g, bool init_in_graph, cudaStream_t st,
                        int64_t *kpro, int64_t *kbody)
{
    const int64_t Nt = p->Nt;
    cudaGraphConditionalHandle h;
    if (cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault) != cudaSuccess) {
        cudaGetLastError();
        set_error("cudaGraphConditionalHandleCreate failed");
        return CGS_ERR_CUDA;
    }
    cgs_status r = CGS_OK;
    const int64_t c0 = cgs_kernel_launches();
    std::vector<cudaGraphNode_t> frontier;
    if (cudaStreamBeginCaptureToGraph(st, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess)
        r = CGS_ERR_CUDA;
    if (r == CGS_OK) {
        cgs_status q = CGS_OK;
        if (init_in_graph)
            q = launch_cg_init(p->sc, o->lambda, o->cgeps, o->cgiter, o->mode == CGS_MODE_CODEARE ? 0 : 1, st);
        if (q == CGS_OK)
            q = (o->mode == CGS_MODE_CODEARE) ? op_eh_codeare(p, p->ksY, o->ftiter, o->fteps, p->vP, st)
                                              : op_eh(p, p->ksY, o->weighted, p->vP, st);
        if (q == CGS_OK && cudaMemcpyAsync(p->vR, p->vP, sizeof(float2) * Nt, cudaMemcpyDeviceToDevice, st) != cudaSuccess) q = CGS_ERR_CUDA;
        if (q == CGS_OK) q = launch_zero(p->vX, sizeof(float2) * Nt, st);
        if (q == CGS_OK) q = launch_coldot(p->vR, p->vP, nullptr, Nt, 1, p->partial, p->scal(), st);
        if (q == CGS_OK) q = launch_scalar_op(p->sc, p->scal(), 0, st);
        if (q == CGS_OK) q = launch_cg_check(p->sc, h, st);
        if (q == CGS_OK) {
            cudaStreamCaptureStatus cs;
            const cudaGraphNode_t *deps = nullptr;
            size_t nd = 0;
            if (cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &nd) != cudaSuccess) q = CGS_ERR_CUDA;
            else frontier.assign(deps, deps + nd);
        }
        cudaGraph_t gg = g;
        if (cudaStreamEndCapture(st, &gg) != cudaSuccess && q == CGS_OK) q = CGS_ERR_CUDA;
        r = q;
    }
    *kpro = cgs_kernel_launches() - c0;
    cudaGraphNode_t cond = nullptr;
    cudaGraph_t body = nullptr;
    if (r == CGS_OK) {
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        if (cudaGraphAddNode(&cond, g, frontier.data(), nullptr, frontier.size(), &cp) != cudaSuccess) r = CGS_ERR_CUDA;
        else body = cp.conditional.phGraph_out[0];
    }
    const int64_t c1 = cgs_kernel_launches();
    if (r == CGS_OK && cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess)
        r = CGS_ERR_CUDA;
    if (r == CGS_OK) {
        cgs_status q = cg_iteration(p, o, h, st);
        cudaGraph_t bb = body;
        if (cudaStreamEndCapture(st, &bb) != cudaSuccess && q == CGS_OK) q = CGS_ERR_CUDA;
        r = q;
    }
    *kbody = cgs_kernel_launches() - c1;
    count_launch((int)-(cgs_kernel_launches() - c0));  // captured launches run only when the graph runs
    cudaGetLastError();
    return r;
}

cgs_status build_solve_graph(cgs_plan *p, const cgs_solve_opts *o, cudaStream_t st)
{
    if (p->solve_exec) { cudaGraphExecDestroy(p->solve_exec); p->solve_exec = nullptr; }
    cudaGraph_t g = nullptr;
    CGS_CUDA(cudaGraphCreate(&g, 0));
    cgs_status r = append_solve(p, o, g, false, st, &p->sg_kpro, &p->sg_kbody);
    if (r == CGS_OK && cudaGraphInstantiate(&p->solve_exec, g, 0) != cudaSuccess) {
        set_error("cudaGraphInstantiate of the solve graph failed");
        r = CGS_ERR_CUDA;
    }
    cudaGraphDestroy(g);
    cudaGetLastError();
    if (r != CGS_OK) { p->solve_exec = nullptr; return r; }
    p->sg_mode = o->mode; p->sg_toep = o->toeplitz; p->sg_weighted = o->weighted;
    p->sg_ftiter = o->ftiter; p->sg_fteps = o->fteps;
    return CGS_OK;
}

// q = (E^H W E + lambda) p on the device buffers (lambda from the scalars;
// with sc null only E^H W E p)
cgs_status op_normal(cgs_plan *p, const float2 *x, float2 *q, int toeplitz, int weighted, CGScalars *sc,
                     cudaStream_t st)
{
    if (toeplitz) {
        CGS_TRY(op_ehe_toeplitz(p, x, q, st));
    } else {
        CGS_TRY(op_forward(p, x, 0, nullptr, p->ksV, st));
        CGS_TRY(op_eh(p, p->ksV, weighted, q, st));
    }
    return sc ? launch_add_scaled(q, x, sc, p->Nt, st) : CGS_OK;  // null sc: the caller adds lambda x
}

cgs_status fcg_alloc(cgs_plan *p)
{
    if (!p->vB) CGS_TRY(dev_alloc(&p->vB, (size_t)p->Nt));
    if (!p->vZ) CGS_TRY(dev_alloc(&p->vZ, (size_t)p->Nt));
    if (!p->vO) CGS_TRY(dev_alloc(&p->vO, (size_t)p->Nt));
    if (!p->vT) CGS_TRY(dev_alloc(&p->vT, (size_t)p->Nt));
    if (!p->dscale) CGS_TRY(dev_alloc(&p->dscale, (size_t)p->Nt));
    if (!p->fs) CGS_TRY(dev_alloc(&p->fs, 1));
    if (p->d == 2 && !p->vCo) CGS_TRY(dev_alloc(&p->vCo, (size_t)p->Nt));
    return CGS_OK;
}

// z = M(r): mode 2 d . (t + net(t)) with t = d . r (the network corrects the
// Jacobi step); mode 1 d^2 . r; mode 3 the circulant C(r); mode 4
// C(r) + d . net(t) (the network corrects the circulant step); mode 0 (or
// after the fallback) z = r.  The fused loop body passes `in_body`: its
// residual update has already formed vC = csq . r and vT = dscale . r with
// fs->tt, the network's output step adds the circulant's scaled output, and
// the caller makes the fallback's z = r itself (with its dots).
cgs_status fcg_precondition(cgs_plan *p, cgs_net *net, int mode, cudaStream_t st, bool in_body = false)
{
    const int64_t Nt = p->Nt;
    if (in_body && mode == 4) {
        CGS_TRY(op_circ_core(p, st));
        return net_apply_image_combine(net, p->vT, &p->fs->tt, p->N[0], p->N[1], p->dscale, p->csq, p->vC, p->vZ,
                                       st);
    }
    if (in_body && mode == 2) {
        CGS_TRY(net_apply_image(net, p->vT, &p->fs->tt, p->N[0], p->N[1], p->vZ, st));
        return launch_diag_scale(p->vZ, p->vT, p->dscale, 1, Nt, p->vZ, st);
    }
    if (mode == 4) {
        CGS_TRY(op_circ(p, p->vR, p->vCo, st));
        CGS_TRY(launch_diag_scale_nrm(p->vR, p->dscale, Nt, p->vT, p->fpart, p->ftick, &p->fs->tt, st));
        CGS_TRY(net_apply_image(net, p->vT, &p->fs->tt, p->N[0], p->N[1], p->vZ, st));
        CGS_TRY(launch_scale_add(p->vZ, p->vZ, p->dscale, p->vCo, nullptr, Nt, st));
    } else if (mode == 3) {
        CGS_TRY(op_circ(p, p->vR, p->vZ, st));
    } else if (mode == 2) {
        CGS_TRY(launch_diag_scale_nrm(p->vR, p->dscale, Nt, p->vT, p->fpart, p->ftick, &p->fs->tt, st));
        CGS_TRY(net_apply_image(net, p->vT, &p->fs->tt, p->N[0], p->N[1], p->vZ, st));
        CGS_TRY(launch_diag_scale(p->vZ, p->vT, p->dscale, 1, Nt, p->vZ, st));
    } else if (mode == 1) {
        CGS_TRY(launch_diag_scale(p->vR, nullptr, p->dscale, 2, Nt, p->vZ, st));
    }
    if (in_body) return CGS_OK;
    return launch_fcg_kernels(FCG_SELECT, p->fs, p->vX, p->vR, p->vO, p->vP, p->vQ, p->vZ, Nt,
                              cudaGraphConditionalHandle(), st);
}

// Capture flexible CG: prologue (b, r = b, x = 0, z = M(r), p = z) and a
// while node over one iteration plus the device-side check.
cgs_status build_fcg_graph(cgs_plan *p, int from_data, int toeplitz, int weighted, cgs_net *net, int mode,
                           cudaStream_t st)
{
    if (p->fcg_exec) { cudaGraphExecDestroy(p->fcg_exec); p->fcg_exec = nullptr; }
    const int64_t Nt = p->Nt;
    FCGScalars *fs = p->fs;
    auto K = [&](int which, cudaGraphConditionalHandle h) {
        return launch_fcg_kernels(which, fs, p->vX, p->vR, p->vO, p->vP, p->vQ, p->vZ, Nt, h, st);
    };
    cudaGraph_t g = nullptr;
    CGS_CUDA(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    cgs_status r = CGS_OK;
    if (cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault) != cudaSuccess) r = CGS_ERR_CUDA;
    const int64_t c0 = cgs_kernel_launches();
    std::vector<cudaGraphNode_t> frontier;
    if (r == CGS_OK && cudaStreamBeginCaptureToGraph(st, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess)
        r = CGS_ERR_CUDA;
    if (r == CGS_OK) {
        cgs_status q = CGS_OK;
        if (from_data) q = op_eh(p, p->ksY, weighted, p->vR, st);
        else if (cudaMemcpyAsync(p->vR, p->vB, sizeof(float2) * Nt, cudaMemcpyDeviceToDevice, st) != cudaSuccess) q = CGS_ERR_CUDA;
        if (q == CGS_OK) q = launch_zero(p->vX, sizeof(float2) * Nt, st);
        if (q == CGS_OK) q = launch_zero(p->vP, sizeof(float2) * Nt, st);
        if (q == CGS_OK) q = launch_zero(p->vO, sizeof(float2) * Nt, st);
        if (q == CGS_OK && mode != 0) q = launch_jacobi_scale(p->sens, Nt, p->nc, fs, p->dscale, st);
        if (q == CGS_OK && mode >= 3) q = circ_prepare(p, fs, st);
        if (q == CGS_OK) q = launch_coldot(p->vR, p->vR, nullptr, Nt, 1, p->partial, &fs->rr, st);
        if (q == CGS_OK) q = K(FCG_INIT, h);
        if (q == CGS_OK) q = fcg_precondition(p, net, mode, st);
        if (q == CGS_OK) q = launch_coldot(p->vZ, p->vR, nullptr, Nt, 1, p->partial, &fs->zr, st);
        if (q == CGS_OK) q = K(FCG_BETA, h);
        if (q == CGS_OK) q = K(FCG_P, h);
        if (q == CGS_OK) q = K(FCG_CHECK, h);
        if (q == CGS_OK) {
            cudaStreamCaptureStatus cs;
            const cudaGraphNode_t *deps = nullptr;
            size_t nd = 0;
            if (cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &nd) != cudaSuccess) q = CGS_ERR_CUDA;
            else frontier.assign(deps, deps + nd);
        }
        cudaGraph_t gg = g;
        if (cudaStreamEndCapture(st, &gg) != cudaSuccess && q == CGS_OK) q = CGS_ERR_CUDA;
        r = q;
    }
    p->fg_kpro = cgs_kernel_launches() - c0;
    cudaGraph_t body = nullptr;
    if (r == CGS_OK) {
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t cond;
        if (cudaGraphAddNode(&cond, g, frontier.data(), nullptr, frontier.size(), &cp) != cudaSuccess) r = CGS_ERR_CUDA;
        else body = cp.conditional.phGraph_out[0];
    }
    const int64_t c1 = cgs_kernel_launches();
    if (r == CGS_OK && cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess)
        r = CGS_ERR_CUDA;
    if (r == CGS_OK) {
        cgs_status q = CGS_OK;
        if (mode < 2 || mode == 3) {
            // fixed preconditioner: fused updates, Fletcher-Reeves beta
            q = op_normal(p, p->vP, p->vQ, toeplitz, weighted, nullptr, st);
            if (q == CGS_OK) q = launch_axpy_dot(p->vQ, p->vP, &fs->cg.lambda, nullptr, Nt, p->fpart, p->ftick, &fs->pq, st);
            // (mode 3: the update also forms csq . r, and the <z, r> kernel
            // applies the circulant's output scaling)
            if (q == CGS_OK)
                q = launch_fcg_xr_rr(fs, p->vX, p->vR, p->vP, p->vQ, Nt, p->fpart, p->ftick, h, st,
                                     mode == 3 ? p->csq : nullptr, mode == 3 ? p->vC : nullptr);
            if (q == CGS_OK && mode == 1)
                q = launch_fcg_jacobi_z(fs, p->vZ, p->vR, p->dscale, Nt, p->fpart, p->ftick, h, st);
            if (q == CGS_OK && mode == 3) q = op_circ_core(p, st);
            if (q == CGS_OK && mode == 3)
                q = launch_fcg_zr_check(fs, p->vZ, p->vR, Nt, p->fpart, p->ftick, h, st, p->csq, p->vC);
            if (q == CGS_OK) q = K(FCG_P, h);
            cudaGraph_t bb = body;
            if (cudaStreamEndCapture(st, &bb) != cudaSuccess && q == CGS_OK) q = CGS_ERR_CUDA;
            r = q;
        } else {
        // changing preconditioner: the lambda term with <p, q>; the x / r update
        // with <r, r>, the stall test and the preconditioner's scaled copies of
        // r (csq . r for the circulant, dscale . r with its norm for the
        // network); the fallback's z = r with <z, r>, <z, r_old> and beta: one
        // kernel each
        q = op_normal(p, p->vP, p->vQ, toeplitz, weighted, nullptr, st);
        if (q == CGS_OK) q = launch_axpy_dot(p->vQ, p->vP, &fs->cg.lambda, nullptr, Nt, p->fpart, p->ftick, &fs->pq, st);
        if (q == CGS_OK)
            q = launch_fcg_xr_rr_decide(fs, p->vX, p->vR, p->vO, p->vP, p->vQ, Nt, p->fpart, p->ftick, st,
                                        mode == 4 ? p->csq : nullptr, mode == 4 ? p->vC : nullptr, p->dscale, p->vT,
                                        p->partial);
        if (q == CGS_OK) q = fcg_precondition(p, net, mode, st, true);
        if (q == CGS_OK) q = launch_fcg_zsel_dots_beta(fs, p->vZ, p->vR, p->vO, Nt, p->fpart, p->partial, p->ftick, st);
        if (q == CGS_OK) q = K(FCG_P, h);
        if (q == CGS_OK) q = K(FCG_CHECK, h);
        cudaGraph_t bb = body;
        if (cudaStreamEndCapture(st, &bb) != cudaSuccess && q == CGS_OK) q = CGS_ERR_CUDA;
        r = q;
        }
    }
    p->fg_kbody = cgs_kernel_launches() - c1;
    count_launch((int)-(cgs_kernel_launches() - c0));
    if (r == CGS_OK && cudaGraphInstantiate(&p->fcg_exec, g, 0) != cudaSuccess) {
        set_error("cudaGraphInstantiate of the flexible-CG graph failed");
        r = CGS_ERR_CUDA;
    }
    cudaGraphDestroy(g);
    cudaGetLastError();
    if (r != CGS_OK) { p->fcg_exec = nullptr; return r; }
    p->fg_src = from_data; p->fg_toep = toeplitz; p->fg_weighted = weighted; p->fg_net = net_serial(net); p->fg_mode = mode;
    return CGS_OK;
}

// A process-wide flag in mapped pinned host memory (one address for every
// device) that a tensor-core gridding kernel sets when its bounded MMA wait
// runs out; the next call that checks it reports CGS_ERR_TIMEOUT once.
int *g_tc_flag = nullptr;
std::once_flag g_tc_once;

int *tc_flag()
{
    std::call_once(g_tc_once, [] {
        void *h = nullptr;
        if (cudaHostAlloc(&h, sizeof(int), cudaHostAllocMapped | cudaHostAllocPortable) == cudaSuccess) {
            *static_cast<volatile int *>(h) = 0;
            g_tc_flag = static_cast<int *>(h);
        }
    });
    return g_tc_flag;
}

cgs_status tc_check()
{
    volatile int *f = g_tc_flag;
    if (f && *f) {
        *f = 0;
        set_error("a tensor-core gridding kernel timed out waiting for its MMAs; its output is incomplete");
        return CGS_ERR_TIMEOUT;
    }
    return CGS_OK;
}

cgs_status check_ready(cgs_plan *p, bool need_w, bool need_s)
{
    if (!p) { set_error("null plan"); return CGS_ERR_BAD_ARG; }
    CGS_TRY(tc_check());
    if (!p->have_k) { set_error("k-space not set"); return CGS_ERR_STATE; }
    if (need_w && !p->have_w) { set_error("weights not set"); return CGS_ERR_STATE; }
    if (need_s && !p->have_s) { set_error("sensitivities not set"); return CGS_ERR_STATE; }
    if (cudaSetDevice(p->device) != cudaSuccess) { set_error("cudaSetDevice failed"); return CGS_ERR_CUDA; }
    return CGS_OK;
}

cgs_status read_scalars(cgs_plan *p, CGScalars *h, cudaStream_t st)
{
    CGS_CUDA(cudaMemcpyAsync(h, p->sc, sizeof(CGScalars), cudaMemcpyDeviceToHost, st));
    CGS_CUDA(cudaStreamSynchronize(st));
    return tc_check();
}

}  // namespace

// One thread waits, with the bounded mbarrier wait of the tensor-core
// kernels, for the first phase of a barrier that expects one arrival and
// never gets it; when the wait gives up it raises the timeout flag as those
// kernels do.  Nothing else is waited on, held or written.
namespace cgs {
namespace diagk {
__global__ void wait_kernel(int64_t limit_ns, int *flag)
{
    __shared__ uint64_t bar;
    if (threadIdx.x != 0) return;
    tc05::mbar_init(&bar, 1);
    tc05::fence_mbar_init();
    if (!tc05::mbar_wait_ns(&bar, 0, (uint64_t)limit_ns)) *reinterpret_cast<volatile int *>(flag) = 1;
}
}  // namespace diagk
}  // namespace cgs

extern "C" cgs_status cgs_diag_wait_timeout(int64_t limit_ns, void *stream)
{
    if (limit_ns <= 0 || limit_ns > 1000000000LL) {
        set_error("cgs_diag_wait_timeout: the limit must be in (0, 1 s]");
        return CGS_ERR_BAD_ARG;
    }
    int *f = tc_flag();
    if (!f) { set_error("cgs_diag_wait_timeout: no mapped host flag"); return CGS_ERR_CUDA; }
    cudaStream_t st = (cudaStream_t)stream;
    cgs::diagk::wait_kernel<<<1, 32, 0, st>>>(limit_ns, f);
    CGS_LAUNCH_CHECK();
    CGS_CUDA(cudaStreamSynchronize(st));
    return tc_check();
}

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char *cgs_last_error(void) { return g_last_error.c_str(); }

int64_t cgs_kernel_launches(void) { return g_launches.load(); }

void cgs_profile_enable(int on)
{
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (!on) prof_drain();
    g_prof_on = (on != 0);
}

void cgs_profile_collect(double *ms, int64_t *count)
{
    std::lock_guard<std::mutex> lk(g_prof_mu);
    prof_drain();
    for (int c = 0; c < PROF_NCAT; ++c) {
        if (ms) ms[c] = g_prof_ms[c];
        if (count) count[c] = g_prof_cnt[c];
        g_prof_ms[c] = 0.0;
        g_prof_cnt[c] = 0;
    }
}

cgs_status cgs_plan_create(cgs_plan **out, const cgs_plan_desc *desc)
{
    if (!out || !desc) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    *out = nullptr;
    if (desc->frames < 0 || desc->frames > 4096) { set_error("frames must be 0..4096"); return CGS_ERR_BAD_ARG; }
    if (desc->frames > 1) {
        // one child plan per frame; the parent holds the stacked vectors only
        cgs_plan_desc one = *desc;
        one.frames = 1;
        cgs_plan *p = new cgs_plan();
        p->F = desc->frames;
        cgs_status st = CGS_OK;
        for (int f = 0; f < p->F && st == CGS_OK; ++f) {
            cgs_plan *c = nullptr;
            st = cgs_plan_create(&c, &one);
            if (st == CGS_OK) p->fr.push_back(c);
        }
        if (st != CGS_OK) { cgs_plan_destroy(p); return st; }
        const cgs_plan *c0 = p->fr[0];
        p->d = c0->d; p->m = c0->m; p->nc = c0->nc; p->alpha = c0->alpha; p->device = c0->device;
        for (int t = 0; t < 3; ++t) { p->N[t] = c0->N[t]; p->n[t] = c0->n[t]; }
        p->geom = c0->geom;
        p->tune = c0->tune;
        p->Mf = c0->M; p->Ntf = c0->Nt;
        p->M = p->F * p->Mf; p->Nt = p->F * p->Ntf; p->ntot = c0->ntot;
        const int64_t nc = p->nc, M = p->M, Nt = p->Nt;
#define ALLOCF(ptr, cnt) do { st = dev_alloc(&(ptr), (cnt)); if (st != CGS_OK) { cgs_plan_destroy(p); return st; } } while (0)
        if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) {
            cgs_plan_destroy(p); set_error("stream creation failed"); return CGS_ERR_CUDA;
        }
        cudaEventCreate(&p->ev0);
        cudaEventCreate(&p->ev1);
        ALLOCF(p->ksY, M * nc); ALLOCF(p->ksV, M * nc);
        ALLOCF(p->vX, Nt); ALLOCF(p->vR, Nt); ALLOCF(p->vP, Nt); ALLOCF(p->vQ, Nt);
        ALLOCF(p->ioA, std::max(Nt, M * nc)); ALLOCF(p->ioB, std::max(Nt, M * nc));
        ALLOCF(p->partial, (size_t)dot_blocks() * std::max<int64_t>(nc, 1));
        ALLOCF(p->dots, 8 * nc + 8);
        ALLOCF(p->sc, 1);
        ALLOCF(p->fpart, (size_t)dot_blocks());
        ALLOCF(p->ftick, 1);
#undef ALLOCF
        if (cudaMemset(p->ftick, 0, sizeof(unsigned int)) != cudaSuccess) {
            cgs_plan_destroy(p);
            set_error("cudaMemset failed");
            return CGS_ERR_CUDA;
        }
        *out = p;
        return CGS_OK;
    }

    if (desc->rank != 2 && desc->rank != 3) { set_error("rank must be 2 or 3"); return CGS_ERR_BAD_ARG; }
    if (desc->ncoils < 1 || desc->M < 1 || desc->m < 0 || desc->m > 8 || !(desc->alpha >= 1.0)) {
        set_error("bad ncoils / M / m / alpha");
        return CGS_ERR_BAD_ARG;
    }
    if (desc->M > 0x7fffffffLL) { set_error("M too large"); return CGS_ERR_BAD_ARG; }
    cgs_plan *p = new cgs_plan();
    p->d = desc->rank; p->m = desc->m; p->nc = desc->ncoils; p->M = desc->M; p->alpha = desc->alpha;
    for (int t = 0; t < p->d; ++t) {
        if (desc->N[t] < 2 || (desc->N[t] & 1)) { delete p; set_error("N must be even and >= 2"); return CGS_ERR_BAD_ARG; }
        p->N[t] = desc->N[t];
        p->n[t] = (int)std::ceil(desc->alpha * desc->N[t]);
        if (p->n[t] < p->N[t]) p->n[t] = p->N[t];
        if (p->n[t] > 2048) { delete p; set_error("oversampled grid side above 2048"); return CGS_ERR_BAD_ARG; }
        if (!factorize(p->n[t], p->fac[t], &p->nfac[t])) {
            delete p;
            set_error("oversampled size must factor into 2, 3, 5 and 7");
            return CGS_ERR_BAD_ARG;
        }
        p->Nt *= p->N[t];
        p->ntot *= p->n[t];
    }
    cudaGetDevice(&p->device);
    cgs_status st = CGS_OK;
#define ALLOC(ptr, cnt) do { st = dev_alloc(&(ptr), (cnt)); if (st != CGS_OK) { cgs_plan_destroy(p); return st; } } while (0)
    if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete p; set_error("stream creation failed"); return CGS_ERR_CUDA;
    }
    cudaEventCreate(&p->ev0);
    cudaEventCreate(&p->ev1);
    // twiddles and deapodisation tables
    for (int t = 0; t < p->d; ++t) {
        const int n = p->n[t], N = p->N[t];
        std::vector<float2> tw(n);
        for (int i = 0; i < n; ++i) {
            const double a = -2.0 * M_PI * (double)i / (double)n;
            tw[i] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        const double sigma = (double)n / (double)N;
        const double b = M_PI * (2.0 - 1.0 / sigma);
        p->geom.b[t] = (float)b;
        std::vector<float> dp(N);
        for (int i = 0; i < N; ++i) {
            const double w = 2.0 * M_PI * (double)(i - N / 2) / (double)n;
            double a = b * b - w * w;
            if (a < 0) a = 0;
            dp[i] = (float)(1.0 / bessel_i0((double)p->m * std::sqrt(a)));
        }
        ALLOC(p->tw[t], n);
        ALLOC(p->deap[t], N);
        cudaMemcpy(p->tw[t], tw.data(), sizeof(float2) * n, cudaMemcpyHostToDevice);
        cudaMemcpy(p->deap[t], dp.data(), sizeof(float) * N, cudaMemcpyHostToDevice);
    }
    // geometry of the gridding tiles
    GridGeom &g = p->geom;
    g.d = p->d; g.m = p->m; g.nc = p->nc;
    for (int t = 0; t < 3; ++t) g.n[t] = (t < p->d) ? p->n[t] : 1;
    apply_tiles(p);
    const int64_t nc = p->nc, M = p->M, Nt = p->Nt, nT = p->ntot;
    // damping mask What (NFFTTraits.hpp:225-260): radius N[0]/2 around index N[0]/2
    {
        std::vector<float> mk(Nt);
        const int N0 = p->N[0], NH = (int)(0.5 * N0);
        for (int64_t k = 0; k < Nt; ++k) {
            int64_t r = k;
            double s = 0;
            for (int t = p->d - 1; t >= 0; --t) {
                const int i = (int)(r % p->N[t]);
                r /= p->N[t];
                const double q = (double)(i - NH);
                s += q * q;
            }
            mk[k] = (std::sqrt(s) > (double)NH) ? 0.f : 1.f;
        }
        ALLOC(p->mask, Nt);
        cudaMemcpy(p->mask, mk.data(), sizeof(float) * Nt, cudaMemcpyHostToDevice);
    }
    ALLOC(p->imap, Nt);
    ALLOC(p->sens, Nt * nc);
    ALLOC(p->grid, nT * nc);
    {
        int64_t t1 = 1;
        for (int t = 0; t < p->d - 1; ++t) t1 *= p->N[t];
        t1 *= p->n[p->d - 1];
        ALLOC(p->t1, t1 * nc);
        if (p->d == 3) ALLOC(p->t2, (int64_t)p->N[0] * p->n[1] * p->n[2] * nc);
    }
    ALLOC(p->ksY, M * nc); ALLOC(p->ksR, M * nc); ALLOC(p->ksV, M * nc);
    ALLOC(p->cF, Nt * nc); ALLOC(p->cP, Nt * nc); ALLOC(p->cZ, Nt * nc);
    ALLOC(p->vX, Nt); ALLOC(p->vR, Nt); ALLOC(p->vP, Nt); ALLOC(p->vQ, Nt);
    const int64_t io = std::max(Nt * nc, M * nc);
    ALLOC(p->ioA, io); ALLOC(p->ioB, io);
    ALLOC(p->partial, (size_t)dot_blocks() * std::max<int64_t>(nc, 1));
    ALLOC(p->dots, 8 * nc + 8);
    ALLOC(p->active, nc);
    ALLOC(p->sc, 1);
    ALLOC(p->fpart, (size_t)dot_blocks());
    ALLOC(p->ftick, 1);
    if (cudaMemset(p->ftick, 0, sizeof(unsigned int)) != cudaSuccess) {
        cgs_plan_destroy(p);
        set_error("cudaMemset failed");
        return CGS_ERR_CUDA;
    }
    ALLOC(p->nodes, (size_t)M * (p->d == 2 ? 1 : 2));
    ALLOC(p->perm, M);
    ALLOC(p->iperm, M);
    ALLOC(p->w, M);
#undef ALLOC
    *out = p;
    return CGS_OK;
}

// ---------------------------------------------------------------------------
// Coil chunks of the host-buffer per-coil NFFT
// ---------------------------------------------------------------------------
static void drop_chunk_set(HostChunks &h)
{
    if (h.in) cudaStreamSynchronize(h.in);
    if (h.out) cudaStreamSynchronize(h.out);
    for (cgs_plan *c : h.plans) cgs_plan_destroy(c);
    h.plans.clear();
    h.c0.clear();
    for (cudaEvent_t e : h.copied) cudaEventDestroy(e);
    for (cudaEvent_t e : h.computed) cudaEventDestroy(e);
    h.copied.clear();
    h.computed.clear();
    h.sens = false;
    for (cudaEvent_t *e : {&h.fork, &h.done})
        if (*e) { cudaEventDestroy(*e); *e = nullptr; }
    for (cudaStream_t *st : {&h.in, &h.out})
        if (*st) { cudaStreamDestroy(*st); *st = nullptr; }
}

static void drop_host_chunks(cgs_plan *p)
{
    drop_chunk_set(p->hcf);
    drop_chunk_set(p->hca);
}

// chunks of a host-buffer call (one frame, 8 coils or more): the tuning's
// host_chunks, else, once the caller's k-space reaches 8 MiB (below that the
// copies are too short to hide anything behind), 4 for the forward and 2 for
// the adjoint, whose spreading loses more to smaller coil counts; at least 4
// coils per chunk, so that every chunk grids with the parent's patch shapes
// and node tables
static int host_chunk_count(const cgs_plan *p, bool adjoint)
{
    if (p->F > 1 || p->nc < 8) return 1;
    int c = p->tune.host_chunks;
    if (c == 0) c = (p->M * p->nc * (int64_t)sizeof(float2) >= (8 << 20)) ? (adjoint ? 2 : 4) : 1;
    return std::max(1, std::min(c, p->nc / 4));
}

// C child plans with the parent's geometry and decomposition (coil groups
// left to their defaults), nc / C coils each (the first nc % C chunks one
// more), reading the parent's node tables; each owns its grids, staging and
// the partial sums of split spreading patches
static cgs_status build_host_chunks(cgs_plan *p, HostChunks &h, int C)
{
    if ((int)h.plans.size() == C) return CGS_OK;
    drop_chunk_set(h);
    cgs_plan_desc one{};
    one.rank = p->d;
    for (int t = 0; t < 3; ++t) one.N[t] = p->N[t];
    one.alpha = p->alpha;
    one.m = p->m;
    one.M = p->M;
    one.frames = 1;
    cgs_status st = CGS_OK;
    h.c0.push_back(0);
    for (int q = 0; q < C && st == CGS_OK; ++q) {
        one.ncoils = p->nc / C + (q < p->nc % C ? 1 : 0);
        cgs_plan *c = nullptr;
        st = cgs_plan_create(&c, &one);
        if (st != CGS_OK) break;
        h.plans.push_back(c);
        h.c0.push_back(h.c0.back() + one.ncoils);
        dev_free(c->nodes);
        dev_free(c->perm);
        dev_free(c->w);
        c->shared_nodes = true;
        dev_free(c->iperm);
        c->nodes = p->nodes; c->perm = p->perm; c->iperm = p->iperm; c->w = p->w;
        c->work = p->work; c->nwork = p->nwork;
        c->nodeU = p->nodeU; c->nodeW = p->nodeW;
        c->pentries = p->pentries; c->pwork = p->pwork; c->pmulti = p->pmulti;
        c->pw16 = p->pw16; c->ps16 = p->ps16; c->pstage = p->pstage;
        c->ilist = p->ilist; c->iwork = p->iwork; c->niwork = p->niwork; c->ibx = p->ibx;
        c->iwin = p->iwin; c->imeta = p->imeta;
        c->nodeU3 = p->nodeU3; c->iby = p->iby;
        c->tune = p->tune;
        c->tune.interp_coils = c->tune.spread_coils = 0;
        c->tune.host_chunks = 1;
        apply_tiles(c);
        c->pset = p->pset;
        c->pslots = p->pslots;
        if (p->d == 2) {
            st = dev_alloc(&c->ppartial, (size_t)p->pslots * p->pset.ph * p->pset.pw * c->nc);
            c->pset.partial = c->ppartial;
        } else if (p->pset.pd == 4) {
            st = dev_alloc(&c->ppartial, (size_t)p->pslots * 64 * c->nc);
            c->pset.partial = c->ppartial;
        }
        c->have_k = p->have_k;
        c->have_w = p->have_w;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        const bool ok0 = cudaEventCreateWithFlags(&e0, cudaEventDisableTiming) == cudaSuccess;
        if (ok0) h.copied.push_back(e0);
        const bool ok1 = cudaEventCreateWithFlags(&e1, cudaEventDisableTiming) == cudaSuccess;
        if (ok1) h.computed.push_back(e1);
        if (st == CGS_OK && (!ok0 || !ok1)) {
            set_error("event creation failed");
            st = CGS_ERR_CUDA;
        }
    }
    if (st == CGS_OK && (cudaEventCreateWithFlags(&h.fork, cudaEventDisableTiming) != cudaSuccess ||
                         cudaEventCreateWithFlags(&h.done, cudaEventDisableTiming) != cudaSuccess ||
                         cudaStreamCreateWithFlags(&h.in, cudaStreamNonBlocking) != cudaSuccess ||
                         cudaStreamCreateWithFlags(&h.out, cudaStreamNonBlocking) != cudaSuccess)) {
        set_error("event or stream creation failed");
        st = CGS_ERR_CUDA;
    }
    if (st != CGS_OK) drop_chunk_set(h);
    return st;
}

// each chunk's coils of the parent's sensitivities ([p][NC] -> [p][nq])
static cgs_status chunk_sensitivities(cgs_plan *p, HostChunks &h)
{
    if (h.sens) return CGS_OK;
    for (size_t q = 0; q < h.plans.size(); ++q) {
        cgs_plan *c = h.plans[q];
        CGS_CUDA(cudaMemcpy2DAsync(c->sens, sizeof(float2) * c->nc, p->sens + h.c0[q], sizeof(float2) * p->nc,
                                   sizeof(float2) * c->nc, p->Nt, cudaMemcpyDeviceToDevice, p->stream));
        c->have_s = true;
    }
    CGS_CUDA(cudaStreamSynchronize(p->stream));
    h.sens = true;
    return CGS_OK;
}

cgs_status cgs_plan_destroy(cgs_plan *p)
{
    if (!p) return CGS_OK;
    cudaSetDevice(p->device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    for (cgs_plan *c : p->fr) cgs_plan_destroy(c);
    drop_host_chunks(p);
    if (p->shared_nodes) {  // the parent frees these
        p->nodes = nullptr; p->perm = nullptr; p->iperm = nullptr; p->w = nullptr; p->work = nullptr;
        p->nodeU = nullptr; p->nodeW = nullptr; p->pentries = nullptr; p->pwork = nullptr; p->pmulti = nullptr;
        p->ilist = nullptr; p->iwork = nullptr; p->nodeU3 = nullptr;
        p->pw16 = nullptr; p->ps16 = nullptr; p->pstage = nullptr;
        p->iwin = nullptr; p->imeta = nullptr;
    }
    void *bufs[] = {p->tw[0], p->tw[1], p->tw[2], p->deap[0], p->deap[1], p->deap[2], p->nodes, p->perm, p->iperm,
                    p->w, p->work, p->nodeU, p->nodeW, p->pentries, p->pwork, p->pmulti, p->ppartial, p->pw16, p->ps16, p->pstage, p->ilist, p->iwork, p->iwin, p->imeta, p->nodeU3, p->mask, p->imap, p->sens, p->grid, p->t1, p->t2, p->ksY, p->ksR, p->ksV,
                    p->cF, p->cP, p->cZ, p->vX, p->vR, p->vP, p->vQ, p->ioA, p->ioB, p->partial, p->dots,
                    p->active, p->sc, p->fpart, p->ftick};
    for (void *b : bufs) dev_free(b);
    for (void *b : {(void *)p->tw2[0], (void *)p->tw2[1], (void *)p->tw2[2], (void *)p->toepK, (void *)p->tA,
                    (void *)p->tB}) dev_free(b);
    if (p->solve_exec) cudaGraphExecDestroy(p->solve_exec);
    if (p->fcg_exec) cudaGraphExecDestroy(p->fcg_exec);
    for (void *b : {(void *)p->vB, (void *)p->vZ, (void *)p->vO, (void *)p->vT, (void *)p->dscale, (void *)p->fs,
                    (void *)p->circ, (void *)p->circ_inv, (void *)p->csq, (void *)p->vC, (void *)p->vCo,
                    (void *)p->twN[0], (void *)p->twN[1], (void *)p->cG, (void *)p->partial2})
        dev_free(b);
    if (p->ev0) cudaEventDestroy(p->ev0);
    if (p->ev1) cudaEventDestroy(p->ev1);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
    return CGS_OK;
}

cgs_status cgs_plan_info(const cgs_plan *p, int *rank, int *N, int *n, int64_t *M, int *ncoils)
{
    if (!p) { set_error("null plan"); return CGS_ERR_BAD_ARG; }
    if (rank) *rank = p->d;
    for (int t = 0; t < 3; ++t) {
        if (N) N[t] = p->N[t];
        if (n) n[t] = p->n[t];
    }
    if (M) *M = p->M;
    if (ncoils) *ncoils = p->nc;
    return CGS_OK;
}

cgs_status cgs_set_kspace(cgs_plan *p, const float *k_in)
{
    if (!p || !k_in) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    CGS_CUDA(cudaSetDevice(p->device));
    if (p->F > 1) {  // frame f takes k[:, :, f] (NCSENSE.hpp:213-223)
        drop_graphs(p);
        p->have_k = p->have_w = false;
        for (int f = 0; f < p->F; ++f) CGS_TRY(cgs_set_kspace(p->fr[f], k_in + (int64_t)f * p->d * p->Mf));
        p->have_k = true;
        return CGS_OK;
    }
    const int d = p->d;
    const int64_t M = p->M;
    std::vector<float> k((size_t)M * d);
    if (is_device_ptr(k_in)) {
        CGS_CUDA(cudaMemcpy(k.data(), k_in, sizeof(float) * k.size(), cudaMemcpyDeviceToHost));
    } else {
        std::memcpy(k.data(), k_in, sizeof(float) * k.size());
    }
    p->toep_valid = false;
    drop_graphs(p);
    drop_host_chunks(p);
    apply_tiles(p);
    const GridGeom &g = p->geom;
    int ntiles = 1;
    for (int t = 0; t < d; ++t) ntiles *= g.nt[t];
    std::vector<int> tile(M), cnt(ntiles + 1, 0);
    std::vector<float> frac((size_t)M * d);
    std::vector<int> cc((size_t)M * d);
    for (int64_t j = 0; j < M; ++j) {
        int ti = 0;
        for (int t = 0; t < d; ++t) {
            const double x = (double)k[(size_t)j * d + t];
            if (!(x >= -0.5 && x < 0.5)) {
                set_error("k-space coordinate outside [-0.5, 0.5)");
                return CGS_ERR_BAD_ARG;
            }
            const double nx = (double)p->n[t] * x;
            const double c = std::floor(nx);
            frac[(size_t)j * d + t] = (float)(nx - c);
            cc[(size_t)j * d + t] = (int)c;
            int u = ((int)c - p->m) % p->n[t];
            if (u < 0) u += p->n[t];
            ti = ti * g.nt[t] + u / g.T;
        }
        tile[j] = ti;
        cnt[ti + 1]++;
    }
    for (int i = 0; i < ntiles; ++i) cnt[i + 1] += cnt[i];
    std::vector<int> perm(M), fill(cnt.begin(), cnt.end() - 1);
    for (int64_t j = 0; j < M; ++j) perm[fill[tile[j]]++] = (int)j;
    const int per = (d == 2) ? 1 : 2;
    std::vector<float4> nodes((size_t)M * per);
    for (int64_t s = 0; s < M; ++s) {
        const int j = perm[s];
        if (d == 2) {
            float4 a;
            a.x = frac[(size_t)j * 2]; a.y = frac[(size_t)j * 2 + 1];
            int c0 = cc[(size_t)j * 2], c1 = cc[(size_t)j * 2 + 1];
            std::memcpy(&a.z, &c0, 4); std::memcpy(&a.w, &c1, 4);
            nodes[s] = a;
        } else {
            float4 a, b;
            a.x = frac[(size_t)j * 3]; a.y = frac[(size_t)j * 3 + 1]; a.z = frac[(size_t)j * 3 + 2]; a.w = 0.f;
            int c0 = cc[(size_t)j * 3], c1 = cc[(size_t)j * 3 + 1], c2 = cc[(size_t)j * 3 + 2], z = 0;
            std::memcpy(&b.x, &c0, 4); std::memcpy(&b.y, &c1, 4); std::memcpy(&b.z, &c2, 4); std::memcpy(&b.w, &z, 4);
            nodes[2 * s] = a; nodes[2 * s + 1] = b;
        }
    }
    // work items: bins split into slices of at most kWork nodes
    const int kWork = p->tune.work_slice > 0 ? p->tune.work_slice : 512;
    std::vector<int4> work;
    for (int ti = 0; ti < ntiles; ++ti) {
        for (int s0 = cnt[ti]; s0 < cnt[ti + 1]; s0 += kWork) {
            const int c = std::min(kWork, cnt[ti + 1] - s0);
            work.push_back(make_int4(ti, s0, c, 0));
        }
    }
    // longest items first (the crowded k-space centre), so they do not form the tail
    std::stable_sort(work.begin(), work.end(), [](const int4 &x, const int4 &y) { return x.z > y.z; });
    dev_free(p->work);
    p->work = nullptr;
    CGS_TRY(dev_alloc(&p->work, work.size()));
    p->nwork = (int)work.size();
    CGS_CUDA(cudaMemcpy(p->work, work.data(), sizeof(int4) * work.size(), cudaMemcpyHostToDevice));
    CGS_CUDA(cudaMemcpy(p->nodes, nodes.data(), sizeof(float4) * nodes.size(), cudaMemcpyHostToDevice));
    CGS_CUDA(cudaMemcpy(p->perm, perm.data(), sizeof(int) * M, cudaMemcpyHostToDevice));
    {
        std::vector<int> iperm(M);
        for (int64_t q = 0; q < M; ++q) iperm[perm[q]] = (int)q;
        CGS_CUDA(cudaMemcpy(p->iperm, iperm.data(), sizeof(int) * M, cudaMemcpyHostToDevice));
    }
    if (d == 2) {
        CGS_TRY(build_patches(p, cc));
        CGS_TRY(build_ibins(p, cc, perm));
    } else if (grid3_mma_ok(p->geom) && !(p->tune.spread_block == 1 && p->tune.interp_block == 1)) {
        CGS_TRY(build_grid3(p, cc, perm));
    } else {
        for (void *b : {(void *)p->iwin, (void *)p->imeta, (void *)p->nodeU3, (void *)p->nodeW, (void *)p->ilist, (void *)p->iwork, (void *)p->pentries,
                        (void *)p->pwork, (void *)p->pmulti, (void *)p->ppartial, (void *)p->pw16, (void *)p->ps16,
                        (void *)p->pstage}) dev_free(b);
        p->nodeU3 = nullptr; p->nodeW = nullptr; p->ilist = nullptr; p->iwork = nullptr;
        p->iwin = nullptr; p->imeta = nullptr;
        p->pentries = nullptr; p->pwork = nullptr; p->pmulti = nullptr; p->ppartial = nullptr;
        p->pw16 = nullptr; p->ps16 = nullptr; p->pstage = nullptr;
        p->niwork = 0;
        p->pset = PatchSet{};
    }
    p->k_host = k;
    p->have_k = true;
    // weights (if already given) must follow the new order: reset to "unset"
    p->have_w = false;
    CGS_CUDA(cudaMemset(p->w, 0, sizeof(float) * M));
    return CGS_OK;
}

cgs_status cgs_set_weights(cgs_plan *p, const float *w_in)
{
    if (!p || !w_in) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    if (!p->have_k) { set_error("set k-space before weights (NFFT.hpp:281-296 needs the nodes)"); return CGS_ERR_STATE; }
    CGS_CUDA(cudaSetDevice(p->device));
    if (p->F > 1) {  // the same weights for every frame (NCSENSE.hpp:244-248)
        drop_graphs(p);
        for (int f = 0; f < p->F; ++f) CGS_TRY(cgs_set_weights(p->fr[f], w_in));
        p->have_w = true;
        return CGS_OK;
    }
    const int64_t M = p->M;
    std::vector<float> w(M), ws(M);
    std::vector<int> perm(M);
    if (is_device_ptr(w_in)) CGS_CUDA(cudaMemcpy(w.data(), w_in, sizeof(float) * M, cudaMemcpyDeviceToHost));
    else std::memcpy(w.data(), w_in, sizeof(float) * M);
    CGS_CUDA(cudaMemcpy(perm.data(), p->perm, sizeof(int) * M, cudaMemcpyDeviceToHost));
    for (int64_t s = 0; s < M; ++s) ws[s] = w[perm[s]];
    CGS_CUDA(cudaMemcpy(p->w, ws.data(), sizeof(float) * M, cudaMemcpyHostToDevice));
    p->w_host = w;
    p->toep_valid = false;
    drop_graphs(p);
    drop_host_chunks(p);
    p->have_w = true;
    return CGS_OK;
}

cgs_status cgs_set_sensitivities(cgs_plan *p, const float *s_in)
{
    if (!p || !s_in) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    CGS_CUDA(cudaSetDevice(p->device));
    if (p->F > 1) {
        for (int f = 0; f < p->F; ++f) CGS_TRY(cgs_set_sensitivities(p->fr[f], s_in));
        p->have_s = true;
        return CGS_OK;
    }
    cudaStream_t st = p->stream;
    const void *src;
    p->hcf.sens = p->hca.sens = false;  // the chunks copy the new maps on their next use
    CGS_TRY(stage_in(s_in, sizeof(float2) * p->Nt * p->nc, p->ioA, &src, st));
    CGS_TRY(launch_to_coil_minor((const float2 *)src, p->Nt, p->nc, p->sens, st));
    CGS_TRY(launch_intensity(p->sens, p->Nt, p->nc, p->imap, st));
    CGS_CUDA(cudaStreamSynchronize(st));
    p->have_s = true;
    return CGS_OK;
}

cgs_status cgs_set_frame_sensitivities(cgs_plan *p, int frame, const float *s_in)
{
    if (!p || !s_in) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    if (p->F <= 1 || frame < 0 || frame >= p->F) { set_error("frame index out of range (or not a framed plan)"); return CGS_ERR_BAD_ARG; }
    CGS_CUDA(cudaSetDevice(p->device));
    CGS_TRY(cgs_set_sensitivities(p->fr[frame], s_in));
    bool all = true;
    for (int f = 0; f < p->F; ++f) all = all && p->fr[f]->have_s;
    p->have_s = all;
    return CGS_OK;
}

cgs_status cgs_sync(cgs_plan *p)
{
    if (!p) { set_error("null plan"); return CGS_ERR_BAD_ARG; }
    CGS_CUDA(cudaStreamSynchronize(p->stream));
    return CGS_OK;
}

// The coil chunks of a host-buffer call.  Chunk q is copied in on h.in
// (after chunk q-1), transformed on its child's stream once its copy is in,
// and copied out on h.out (after chunk q-1's copy out) once its kernels are
// done; `st` forks the work and waits for all of it.  `copy_in(q, stream)`
// issues chunk q's host-to-device copy, `compute(q, stream)` its kernels and
// `copy_out(q, stream)` its device-to-host copy (each may issue nothing).
// Every chunk's kernels are queued before the first copy out: a copy with
// pageable host memory returns only once it is done (to pageable memory) or
// staged (from it), and the kernels queued before it keep the GPU busy.
extern "C++" {
template <class In, class Run, class Out>
static cgs_status run_host_chunks(HostChunks &h, cudaStream_t st, bool hout, In copy_in, Run compute, Out copy_out)
{
    const size_t C = h.plans.size();
    CGS_CUDA(cudaEventRecord(h.fork, st));
    CGS_CUDA(cudaStreamWaitEvent(h.in, h.fork, 0));
    CGS_CUDA(cudaStreamWaitEvent(h.out, h.fork, 0));
    for (size_t q = 0; q < C; ++q) {
        CGS_TRY(copy_in(q, h.in));
        CGS_CUDA(cudaEventRecord(h.copied[q], h.in));
        cudaStream_t s = h.plans[q]->stream;
        CGS_CUDA(cudaStreamWaitEvent(s, h.copied[q], 0));
        CGS_TRY(compute(q, s));
        CGS_CUDA(cudaEventRecord(h.computed[q], s));
    }
    for (size_t q = 0; q < C; ++q) {
        CGS_CUDA(cudaStreamWaitEvent(h.out, h.computed[q], 0));
        CGS_TRY(copy_out(q, h.out));
    }
    CGS_CUDA(cudaEventRecord(h.done, h.out));
    CGS_CUDA(cudaStreamWaitEvent(st, h.done, 0));
    if (hout) CGS_CUDA(cudaStreamSynchronize(st));
    return CGS_OK;
}
}  // extern "C++"

static cgs_status chunked_trafo(cgs_plan *p, const float *fhat, float *f, bool hin, bool hout, cudaStream_t st)
{
    HostChunks &h = p->hcf;
    auto src = [&](size_t q) { return (const float2 *)fhat + (int64_t)h.c0[q] * p->Nt; };
    auto out = [&](size_t q) { return (float2 *)f + (int64_t)h.c0[q] * p->M; };
    return run_host_chunks(
        h, st, hout,
        [&](size_t q, cudaStream_t s) -> cgs_status {
            cgs_plan *c = h.plans[q];
            if (hin) CGS_CUDA(cudaMemcpyAsync(c->ioA, src(q), sizeof(float2) * c->nc * p->Nt, cudaMemcpyHostToDevice, s));
            return CGS_OK;
        },
        [&](size_t q, cudaStream_t s) -> cgs_status {
            cgs_plan *c = h.plans[q];
            return op_forward(c, hin ? c->ioA : src(q), 2, nullptr, c->ksV, s, hout ? c->ioB : out(q));
        },
        [&](size_t q, cudaStream_t s) -> cgs_status {
            cgs_plan *c = h.plans[q];
            if (hout) CGS_CUDA(cudaMemcpyAsync(out(q), c->ioB, sizeof(float2) * c->nc * p->M, cudaMemcpyDeviceToHost, s));
            return CGS_OK;
        });
}

// per-coil images (coil-major, caller) -> samples (coil-major, caller)
cgs_status cgs_nfft_trafo(cgs_plan *p, const float *fhat, float *f, void *stream)
{
    CGS_TRY(check_ready(p, false, false));
    if (!fhat || !f) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    cudaStream_t st = pick_stream(p, stream);
    if (p->F > 1) {
        for (int q = 0; q < p->F; ++q)
            CGS_TRY(cgs_nfft_trafo(p->fr[q], fhat + 2 * q * p->Ntf * p->nc, f + 2 * q * p->Mf * p->nc, st));
        return CGS_OK;
    }
    {
        const bool hin = !is_device_ptr(fhat), hout = !is_device_ptr(f);
        const int C = host_chunk_count(p, false);
        if ((hin || hout) && C > 1) {
            CGS_TRY(build_host_chunks(p, p->hcf, C));
            return chunked_trafo(p, fhat, f, hin, hout, st);
        }
    }
    const void *src;
    CGS_TRY(stage_in(fhat, sizeof(float2) * p->Nt * p->nc, p->ioA, &src, st));
    const bool dev = is_device_ptr(f);
    float2 *dst = dev ? (float2 *)f : p->ioB;
    CGS_TRY(op_forward(p, (const float2 *)src, 2, nullptr, p->ksV, st, dst));
    if (!dev) {
        CGS_CUDA(cudaMemcpyAsync(f, dst, sizeof(float2) * p->M * p->nc, cudaMemcpyDeviceToHost, st));
        CGS_CUDA(cudaStreamSynchronize(st));
    }
    return CGS_OK;
}

// caller k-space (coil-major, trajectory order; frames stacked) -> sorted layout
static cgs_status gather_ks(cgs_plan *p, const float *y, float2 *dst, cudaStream_t st)
{
    const void *src;
    CGS_TRY(stage_in(y, sizeof(float2) * p->M * p->nc, p->ioA, &src, st));
    if (p->F == 1) return launch_gather_ks((const float2 *)src, p->iperm, p->M, p->nc, dst, st);
    for (int f = 0; f < p->F; ++f) {
        const int64_t off = f * p->Mf * p->nc;
        CGS_TRY(launch_gather_ks((const float2 *)src + off, p->fr[f]->iperm, p->Mf, p->nc, dst + off, st));
    }
    return CGS_OK;
}

static cgs_status ks_in(cgs_plan *p, const float *y, cudaStream_t st) { return gather_ks(p, y, p->ksY, st); }

static cgs_status coil_images_out(cgs_plan *p, const float2 *cm, float *out, cudaStream_t st)
{
    const bool dev = is_device_ptr(out);
    float2 *dst = dev ? (float2 *)out : p->ioB;
    CGS_TRY(launch_to_coil_major(cm, p->Nt, p->nc, dst, st));
    if (!dev) {
        CGS_CUDA(cudaMemcpyAsync(out, dst, sizeof(float2) * p->Nt * p->nc, cudaMemcpyDeviceToHost, st));
        CGS_CUDA(cudaStreamSynchronize(st));
    }
    return CGS_OK;
}

static cgs_status image_out(cgs_plan *p, const float2 *img, float *out, cudaStream_t st)
{
    if (is_device_ptr(out)) {
        if ((const void *)img != (const void *)out)
            CGS_CUDA(cudaMemcpyAsync(out, img, sizeof(float2) * p->Nt, cudaMemcpyDeviceToDevice, st));
    } else {
        CGS_CUDA(cudaMemcpyAsync(out, img, sizeof(float2) * p->Nt, cudaMemcpyDeviceToHost, st));
        CGS_CUDA(cudaStreamSynchronize(st));
    }
    return CGS_OK;
}

static cgs_status chunked_adjoint(cgs_plan *p, const float *f, float *fhat, bool hin, bool hout, cudaStream_t st)
{
    HostChunks &h = p->hca;
    auto src = [&](size_t q) { return (const float2 *)f + (int64_t)h.c0[q] * p->M; };
    auto out = [&](size_t q) { return (float2 *)fhat + (int64_t)h.c0[q] * p->Nt; };
    return run_host_chunks(
        h, st, hout,
        [&](size_t q, cudaStream_t s) -> cgs_status {
            cgs_plan *c = h.plans[q];
            if (hin) CGS_CUDA(cudaMemcpyAsync(c->ioA, src(q), sizeof(float2) * c->nc * p->M, cudaMemcpyHostToDevice, s));
            return CGS_OK;
        },
        [&](size_t q, cudaStream_t s) -> cgs_status {
            cgs_plan *c = h.plans[q];
            CGS_TRY(launch_gather_ks(hin ? c->ioA : src(q), c->iperm, c->M, c->nc, c->ksY, s));
            return op_adjoint(c, c->ksY, 0, hout ? c->ioB : out(q), s, true);
        },
        [&](size_t q, cudaStream_t s) -> cgs_status {
            cgs_plan *c = h.plans[q];
            if (hout) CGS_CUDA(cudaMemcpyAsync(out(q), c->ioB, sizeof(float2) * c->nc * p->Nt, cudaMemcpyDeviceToHost, s));
            return CGS_OK;
        });
}

cgs_status cgs_nfft_adjoint(cgs_plan *p, const float *f, float *fhat, void *stream)
{
    CGS_TRY(check_ready(p, false, false));
    if (!fhat || !f) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    cudaStream_t st = pick_stream(p, stream);
    if (p->F > 1) {
        for (int q = 0; q < p->F; ++q)
            CGS_TRY(cgs_nfft_adjoint(p->fr[q], f + 2 * q * p->Mf * p->nc, fhat + 2 * q * p->Ntf * p->nc, st));
        return CGS_OK;
    }
    {
        const bool hin = !is_device_ptr(f), hout = !is_device_ptr(fhat);
        const int C = host_chunk_count(p, true);
        if ((hin || hout) && C > 1) {
            CGS_TRY(build_host_chunks(p, p->hca, C));
            return chunked_adjoint(p, f, fhat, hin, hout, st);
        }
    }
    CGS_TRY(ks_in(p, f, st));
    // the last FFT pass stores straight into the caller's coil-major layout
    const bool dev = is_device_ptr(fhat);
    float2 *dst = dev ? (float2 *)fhat : p->ioB;
    CGS_TRY(op_adjoint(p, p->ksY, 0, dst, st, true));
    if (!dev) {
        CGS_CUDA(cudaMemcpyAsync(fhat, dst, sizeof(float2) * p->Nt * p->nc, cudaMemcpyDeviceToHost, st));
        CGS_CUDA(cudaStreamSynchronize(st));
    }
    return CGS_OK;
}

cgs_status cgs_nfft_itrafo(cgs_plan *p, const float *f, float *fhat, int maxit, double eps, void *stream)
{
    CGS_TRY(check_ready(p, true, false));
    if (!fhat || !f || maxit < 0) { set_error("bad argument"); return CGS_ERR_BAD_ARG; }
    cudaStream_t st = pick_stream(p, stream);
    if (p->F > 1) {
        for (int q = 0; q < p->F; ++q)
            CGS_TRY(cgs_nfft_itrafo(p->fr[q], f + 2 * q * p->Mf * p->nc, fhat + 2 * q * p->Ntf * p->nc, maxit, eps,
                                    st));
        return CGS_OK;
    }
    CGS_TRY(ks_in(p, f, st));
    CGS_TRY(op_itrafo(p, p->ksY, maxit, eps, st));
    return coil_images_out(p, p->cF, fhat, st);
}

// SENSE forward into the caller's host k-space by coil chunks: the image is
// staged once on `st`, each chunk expands it with its coils' sensitivities
// and interpolates while the previous chunk's samples go to the host.
static cgs_status chunked_sense_trafo(cgs_plan *p, const float2 *xs, float *y, cudaStream_t st)
{
    HostChunks &h = p->hcf;
    auto out = [&](size_t q) { return (float2 *)y + (int64_t)h.c0[q] * p->M; };
    return run_host_chunks(
        h, st, true,
        [&](size_t, cudaStream_t) -> cgs_status { return CGS_OK; },
        [&](size_t q, cudaStream_t s) -> cgs_status {
            cgs_plan *c = h.plans[q];
            return op_forward(c, xs, 0, nullptr, c->ksV, s, c->ioB);
        },
        [&](size_t q, cudaStream_t s) -> cgs_status {
            cgs_plan *c = h.plans[q];
            CGS_CUDA(cudaMemcpyAsync(out(q), c->ioB, sizeof(float2) * c->nc * p->M, cudaMemcpyDeviceToHost, s));
            return CGS_OK;
        });
}

cgs_status cgs_sense_trafo(cgs_plan *p, const float *x, float *y, void *stream)
{
    CGS_TRY(check_ready(p, false, true));
    if (!x || !y) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    cudaStream_t st = pick_stream(p, stream);
    const void *src;
    CGS_TRY(stage_in(x, sizeof(float2) * p->Nt, p->ioA, &src, st));
    if (!is_device_ptr(y)) {
        const int C = host_chunk_count(p, false);
        if (C > 1) {
            CGS_TRY(build_host_chunks(p, p->hcf, C));
            CGS_TRY(chunk_sensitivities(p, p->hcf));
            return chunked_sense_trafo(p, (const float2 *)src, y, st);
        }
    }
    const bool dev = is_device_ptr(y);
    float2 *dst = dev ? (float2 *)y : p->ioB;
    CGS_TRY(op_forward(p, (const float2 *)src, 0, nullptr, p->ksV, st, dst));
    if (!dev) {
        CGS_CUDA(cudaMemcpyAsync(y, dst, sizeof(float2) * p->M * p->nc, cudaMemcpyDeviceToHost, st));
        CGS_CUDA(cudaStreamSynchronize(st));
    }
    return CGS_OK;
}

cgs_status cgs_sense_adjoint_codeare(cgs_plan *p, const float *y, float *x, int ftiter, double fteps,
                                     void *stream)
{
    CGS_TRY(check_ready(p, true, true));
    if (!x || !y || ftiter < 0) { set_error("bad argument"); return CGS_ERR_BAD_ARG; }
    cudaStream_t st = pick_stream(p, stream);
    CGS_TRY(ks_in(p, y, st));
    CGS_TRY(op_eh_codeare(p, p->ksY, ftiter, fteps, p->vX, st));
    return image_out(p, p->vX, x, st);
}

cgs_status cgs_sense_adjoint(cgs_plan *p, const float *y, float *x, int weighted, void *stream)
{
    CGS_TRY(check_ready(p, weighted != 0, true));
    if (!x || !y) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    cudaStream_t st = pick_stream(p, stream);
    CGS_TRY(ks_in(p, y, st));
    CGS_TRY(op_eh(p, p->ksY, weighted, p->vX, st));
    return image_out(p, p->vX, x, st);
}

// codeare mode takes the Toeplitz kernel only where the NFFT is accurate: the
// reference's CGNR composes its own (approximate) NFFT pair, which equals the
// point-spread-function convolution only up to the NFFT error
static cgs_status check_codeare_toeplitz(const cgs_plan *p, const cgs_solve_opts *o)
{
    if (o->mode == CGS_MODE_CODEARE && o->toeplitz && !(p->alpha >= 2.0 - 1e-9 && p->m >= 4)) {
        set_error("codeare mode with the Toeplitz kernel needs sigma >= 2 and m >= 4 (an accurate NFFT)");
        return CGS_ERR_BAD_ARG;
    }
    return CGS_OK;
}

// the density weighting of the Toeplitz kernel: codeare's CGNR always uses W
static int toeplitz_weighting(const cgs_plan *p, const cgs_solve_opts *o)
{
    if (o->mode == CGS_MODE_CODEARE) return p->have_w ? 1 : 0;
    return (o->weighted && p->have_w) ? 1 : 0;
}

cgs_status cgs_solve(cgs_plan *p, const float *y, float *x, const cgs_solve_opts *o,
                     cgs_solve_report *rep, void *stream)
{
    if (!o) { set_error("null options"); return CGS_ERR_BAD_ARG; }
    const bool codeare = (o->mode == CGS_MODE_CODEARE);
    CGS_TRY(check_ready(p, codeare || o->weighted, true));
    if (!x || !y || o->cgiter < 0 || o->ftiter < 0) { set_error("bad argument"); return CGS_ERR_BAD_ARG; }
    if (p->F > 1 && o->toeplitz) { set_error("the Toeplitz operator is not built for frames"); return CGS_ERR_BAD_ARG; }
    CGS_TRY(check_codeare_toeplitz(p, o));
    cudaStream_t st = pick_stream(p, stream);
    if (rep) { std::memset(rep, 0, sizeof(*rep)); rep->fallback_at = -1; }
    if (o->toeplitz) {
        const int wtd = toeplitz_weighting(p, o);
        if (!p->toep_valid || p->toep_weighted != wtd) CGS_TRY(build_toeplitz(p, wtd, st));
    }
    CGS_CUDA(cudaEventRecord(p->ev0, st));
    CGS_TRY(ks_in(p, y, st));
    int iters = 0;
    cgs_status result = CGS_OK;
    if (o->cgiter == 0 && codeare) {
        // CGLS with no iterations returns A/b (CGLS.hpp:32-33)
        CGS_TRY(op_eh_codeare(p, p->ksY, o->ftiter, o->fteps, p->vX, st));
    } else {
        const bool same = p->solve_exec && p->sg_mode == o->mode && p->sg_toep == o->toeplitz &&
                          p->sg_weighted == o->weighted && p->sg_ftiter == o->ftiter && p->sg_fteps == o->fteps;
        if (!same) CGS_TRY(build_solve_graph(p, o, st));
        CGScalars init{};
        init.lambda = o->lambda;
        init.tol = o->cgeps;
        init.maxit = o->cgiter;
        init.sqrt_mode = codeare ? 0 : 1;
        CGS_CUDA(cudaMemcpyAsync(p->sc, &init, sizeof(init), cudaMemcpyHostToDevice, st));
        CGS_CUDA(cudaGraphLaunch(p->solve_exec, st));
        CGScalars h;
        CGS_TRY(read_scalars(p, &h, st));
        iters = h.iter;
        count_launch((int)(p->sg_kpro + (int64_t)h.iter * p->sg_kbody));
        if (h.nan_flag) result = CGS_ERR_NAN;
        if (rep) {
            const int nh = std::min(256, h.iter + 1);
            for (int i = 0; i < nh; ++i) rep->res_hist[i] = h.hist[i];
            rep->res_first = h.hist[0];
            // the measure after the last update (the loop's final check records it unless maxit ended it)
            const double ratio = h.rn / h.xn;
            rep->res_last = codeare ? ratio : std::sqrt(ratio);
            if (!codeare && h.iter < 256) rep->res_hist[h.iter] = rep->res_last;
        }
    }
    CGS_CUDA(cudaEventRecord(p->ev1, st));
    CGS_TRY(image_out(p, p->vX, x, st));
    CGS_CUDA(cudaEventSynchronize(p->ev1));
    if (rep) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p->ev0, p->ev1);
        rep->seconds = ms * 1e-3;
        rep->iterations = iters;
    }
    return result;
}

cgs_status cgs_normal_apply(cgs_plan *p, const float *x, float *out, const cgs_solve_opts *o, void *stream)
{
    if (!o) { set_error("null options"); return CGS_ERR_BAD_ARG; }
    CGS_TRY(check_ready(p, o->weighted != 0, true));
    if (!x || !out) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    if (p->F > 1 && o->toeplitz) { set_error("the Toeplitz operator is not built for frames"); return CGS_ERR_BAD_ARG; }
    cudaStream_t st = pick_stream(p, stream);
    if (o->toeplitz) {
        const int wtd = (o->weighted && p->have_w) ? 1 : 0;
        if (!p->toep_valid || p->toep_weighted != wtd) CGS_TRY(build_toeplitz(p, wtd, st));
    }
    CGScalars init{};
    init.lambda = o->lambda;
    CGS_CUDA(cudaMemcpyAsync(p->sc, &init, sizeof(init), cudaMemcpyHostToDevice, st));
    const void *src;
    CGS_TRY(stage_in(x, sizeof(float2) * p->Nt, p->ioA, &src, st));
    CGS_TRY(fcg_alloc(p));
    CGS_CUDA(cudaMemcpyAsync(p->vZ, src, sizeof(float2) * p->Nt, cudaMemcpyDeviceToDevice, st));
    CGS_TRY(op_normal(p, p->vZ, p->vQ, o->toeplitz, o->weighted, p->sc, st));
    return image_out(p, p->vQ, out, st);
}

cgs_status cgs_solve_fcg(cgs_plan *p, const float *y, const float *rhs, float *x, const cgs_solve_opts *o,
                         cgs_net *net, cgs_solve_report *rep, void *stream)
{
    if (!o) { set_error("null options"); return CGS_ERR_BAD_ARG; }
    CGS_TRY(check_ready(p, o->weighted != 0, true));
    if (!x || (!y && !rhs) || o->cgiter < 0) { set_error("bad argument"); return CGS_ERR_BAD_ARG; }
    if (p->d != 2) { set_error("the learned preconditioner is 2-D"); return CGS_ERR_BAD_ARG; }
    if (p->F > 1) { set_error("flexible CG is not built for frames"); return CGS_ERR_BAD_ARG; }
    cudaStream_t st = pick_stream(p, stream);
    if (rep) std::memset(rep, 0, sizeof(*rep));
    CGS_TRY(fcg_alloc(p));
    if (o->toeplitz) {
        const int wtd = (o->weighted && p->have_w) ? 1 : 0;
        if (!p->toep_valid || p->toep_weighted != wtd) CGS_TRY(build_toeplitz(p, wtd, st));
    }
    const int from_data = y ? 1 : 0;
    if (from_data) {
        CGS_TRY(ks_in(p, y, st));
    } else {
        const void *src;
        CGS_TRY(stage_in(rhs, sizeof(float2) * p->Nt, p->ioA, &src, st));
        CGS_CUDA(cudaMemcpyAsync(p->vB, src, sizeof(float2) * p->Nt, cudaMemcpyDeviceToDevice, st));
    }
    // o->jacobi: 0 none, 1 the exact diagonal, 2 the circulant (with a net: its correction's base)
    if (o->jacobi < 0 || o->jacobi > 2) { set_error("preconditioner kind must be 0, 1 or 2"); return CGS_ERR_BAD_ARG; }
    const int mode = net ? (o->jacobi == 2 ? 4 : 2) : (o->jacobi == 2 ? 3 : (o->jacobi ? 1 : 0));
    if (mode >= 3) {
        const int wtd = (o->weighted && p->have_w) ? 1 : 0;
        if (!p->toep_valid || p->toep_weighted != wtd || !p->circ_valid) CGS_TRY(build_toeplitz(p, wtd, st));
    }
    const bool same = p->fcg_exec && p->fg_src == from_data && p->fg_toep == o->toeplitz &&
                      p->fg_weighted == o->weighted && p->fg_net == net_serial(net) && p->fg_mode == mode;
    if (!same) CGS_TRY(build_fcg_graph(p, from_data, o->toeplitz, o->weighted, net, mode, st));
    double sumw = (double)p->M;
    if (o->weighted && p->have_w) {
        sumw = 0.0;
        for (float v : p->w_host) sumw += (double)v;
    }
    FCGScalars init{};
    init.cg.lambda = o->lambda;
    init.cg.tol = o->cgeps;
    init.cg.maxit = o->cgiter;
    init.cg.sqrt_mode = 1;
    init.fallback = 0;
    init.mode = mode;
    init.sumw = sumw;
    CGS_CUDA(cudaEventRecord(p->ev0, st));
    CGS_CUDA(cudaMemcpyAsync(p->fs, &init, sizeof(init), cudaMemcpyHostToDevice, st));
    CGS_CUDA(cudaGraphLaunch(p->fcg_exec, st));
    CGS_CUDA(cudaEventRecord(p->ev1, st));
    FCGScalars h;
    CGS_CUDA(cudaMemcpyAsync(&h, p->fs, sizeof(h), cudaMemcpyDeviceToHost, st));
    CGS_CUDA(cudaStreamSynchronize(st));
    count_launch((int)(p->fg_kpro + (int64_t)h.cg.iter * p->fg_kbody));
    if (rep) {
        const int nh = std::min(256, h.cg.iter + 1);
        for (int i = 0; i < nh; ++i) rep->res_hist[i] = h.cg.hist[i];
        rep->iterations = h.cg.iter;
        rep->res_first = h.cg.hist[0];
        rep->res_last = h.rr0 > 0 ? std::sqrt(h.rr / h.rr0) : 0.0;
        if (h.cg.iter < 256) rep->res_hist[h.cg.iter] = rep->res_last;
        rep->fallback_at = (net && h.fallback) ? h.fallback_at : -1;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p->ev0, p->ev1);
        rep->seconds = ms * 1e-3;
    }
    CGS_TRY(image_out(p, p->vX, x, st));
    return h.cg.nan_flag ? CGS_ERR_NAN : CGS_OK;
}


cgs_status cgs_precond_apply(cgs_plan *p, const float *r, float *z, const cgs_solve_opts *o, void *stream)
{
    if (!o || !r || !z) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    CGS_TRY(check_ready(p, o->weighted != 0, true));
    if (p->d != 2 || p->F > 1) { set_error("the circulant preconditioner is built for single-frame 2-D plans"); return CGS_ERR_BAD_ARG; }
    cudaStream_t st = pick_stream(p, stream);
    CGS_TRY(fcg_alloc(p));
    const int wtd = (o->weighted && p->have_w) ? 1 : 0;
    if (!p->toep_valid || p->toep_weighted != wtd || !p->circ_valid) CGS_TRY(build_toeplitz(p, wtd, st));
    FCGScalars init{};
    init.cg.lambda = o->lambda;
    CGS_CUDA(cudaMemcpyAsync(p->fs, &init, sizeof(init), cudaMemcpyHostToDevice, st));
    CGS_TRY(circ_prepare(p, p->fs, st));
    const void *src;
    CGS_TRY(stage_in(r, sizeof(float2) * p->Nt, p->ioA, &src, st));
    CGS_CUDA(cudaMemcpyAsync(p->vZ, src, sizeof(float2) * p->Nt, cudaMemcpyDeviceToDevice, st));
    CGS_TRY(op_circ(p, p->vZ, p->vQ, st));
    return image_out(p, p->vQ, z, st);
}

cgs_status cgs_get_tuning(const cgs_plan *p, cgs_tuning *out)
{
    if (!p || !out) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    *out = p->F > 1 ? p->fr[0]->tune : p->tune;
    return CGS_OK;
}

static cgs_status rebin(cgs_plan *p)
{
    if (!p->have_k) return CGS_OK;
    const std::vector<float> k = p->k_host, w = p->w_host;
    const bool hw = p->have_w;
    CGS_TRY(cgs_set_kspace(p, k.data()));
    if (hw) CGS_TRY(cgs_set_weights(p, w.data()));
    return CGS_OK;
}

cgs_status cgs_set_tuning(cgs_plan *p, const cgs_tuning *t)
{
    if (!p || !t) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    auto in = [](int v, std::initializer_list<int> ok) {
        for (int o : ok) if (v == o) return true;
        return false;
    };
    if (!in(t->tile, {0, 8, 16, 32}) || !in(t->interp_coils, {0, 1, 4, 8, 16, 32}) ||
        !in(t->spread_coils, {0, 1, 2, 4, 8, 16, 32}) || !in(t->spread_block, {0, 1, 2, 4, 8, 16, 32, 64}) || !in(t->interp_block, {0, 1, 16, 64}) ||
        (t->work_slice != 0 && (t->work_slice < 32 || t->work_slice > 65536)) ||
        (t->spread_chunk != 0 && (t->spread_chunk < 32 || t->spread_chunk > 65536)) ||
        t->host_chunks < 0 || t->host_chunks > 32) {
        set_error("tuning value out of range");
        return CGS_ERR_BAD_ARG;
    }
    CGS_CUDA(cudaSetDevice(p->device));
    if (p->F > 1) {
        drop_graphs(p);
        for (int f = 0; f < p->F; ++f) CGS_TRY(cgs_set_tuning(p->fr[f], t));
        p->tune = *t;
        return CGS_OK;
    }
    const bool bins = t->tile != p->tune.tile || t->work_slice != p->tune.work_slice ||
                      t->spread_chunk != p->tune.spread_chunk || t->spread_block != p->tune.spread_block ||
                      t->interp_block != p->tune.interp_block;
    p->tune = *t;
    apply_tiles(p);
    drop_graphs(p);
    drop_host_chunks(p);
    if (bins) CGS_TRY(rebin(p));
    return CGS_OK;
}

}  // extern "C"

namespace {
// Autotune results by problem class, process-wide: plans with the same grid,
// cut-off, coil count and sampling density (nodes per grid point, in steps of
// 2^(1/4)) share the decomposition measured on the first of them.
struct TuneKey {
    int n0, n1, m, nc, dens;
    bool operator<(const TuneKey &o) const
    {
        return std::tie(n0, n1, m, nc, dens) < std::tie(o.n0, o.n1, o.m, o.nc, o.dens);
    }
};
std::mutex g_tune_mx;
std::map<TuneKey, std::pair<cgs_tuning, double>> g_tune_cache;
bool g_tune_cache_on = true;

TuneKey tune_key(const cgs_plan *p)
{
    const double dens = (double)p->M / ((double)p->n[0] * (double)p->n[1]);
    return TuneKey{p->n[0], p->n[1], p->m, p->nc, (int)std::lround(4.0 * std::log2(std::max(dens, 1e-12)))};
}
}  // namespace

extern "C" {

cgs_status cgs_autotune_cache(int mode)
{
    if (mode < 0 || mode > 2) { set_error("autotune cache mode must be 0, 1 or 2"); return CGS_ERR_BAD_ARG; }
    std::lock_guard<std::mutex> lk(g_tune_mx);
    g_tune_cache.clear();
    if (mode != 2) g_tune_cache_on = (mode == 1);
    return CGS_OK;
}

cgs_status cgs_autotune(cgs_plan *p, cgs_tuning *chosen, double *ms, void *stream)
{
    if (!p) { set_error("null plan"); return CGS_ERR_BAD_ARG; }
    if (!p->have_k) { set_error("autotune needs the k-space"); return CGS_ERR_STATE; }
    if (p->d != 2) { set_error("the autotuner covers 2-D plans"); return CGS_ERR_BAD_ARG; }
    if (p->F > 1) {  // frames share the geometry: tune the first, apply to all
        cgs_tuning t{};
        CGS_TRY(cgs_autotune(p->fr[0], &t, ms, stream));
        CGS_TRY(cgs_set_tuning(p, &t));
        if (chosen) *chosen = t;
        return CGS_OK;
    }
    const TuneKey key = tune_key(p);
    {
        cgs_tuning t{};
        double t_ms = 0.0;
        bool hit = false;
        {
            std::lock_guard<std::mutex> lk(g_tune_mx);
            auto it = g_tune_cache.find(key);
            if (g_tune_cache_on && it != g_tune_cache.end()) {
                t = it->second.first;
                t_ms = it->second.second;
                hit = true;
            }
        }
        if (hit) {
            CGS_TRY(cgs_set_tuning(p, &t));
            if (chosen) *chosen = t;
            if (ms) *ms = t_ms;
            return CGS_OK;
        }
    }
    CGS_CUDA(cudaSetDevice(p->device));
    cudaStream_t st = pick_stream(p, stream);
    const int64_t gridN = p->ntot * p->nc, ksN = p->M * p->nc;
    auto fill = [&](float2 *a, int64_t n, uint32_t seed) -> cgs_status {
        const unsigned blocks = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 8);
        tunek::fill_pattern_kernel<<<blocks, 256, 0, st>>>(a, n, seed);
        CGS_LAUNCH_CHECK();
        return CGS_OK;
    };
    auto timed = [&](auto &&launch, double *out) -> cgs_status {
        CGS_TRY(launch());
        CGS_CUDA(cudaEventRecord(p->ev0, st));
        for (int i = 0; i < 3; ++i) CGS_TRY(launch());
        CGS_CUDA(cudaEventRecord(p->ev1, st));
        CGS_CUDA(cudaEventSynchronize(p->ev1));
        float t = 0.f;
        CGS_CUDA(cudaEventElapsedTime(&t, p->ev0, p->ev1));
        *out = t / 3.0;
        return CGS_OK;
    };
    auto interp = [&]() -> cgs_status {
        NodeSet ns = node_set(p);
        return launch_interp(p->geom, ns, p->grid, p->ksR, st);
    };
    auto spread = [&]() -> cgs_status {
        return launch_spread_patch(p->geom, p->pset, p->ksV, p->w, 0, p->grid, st);
    };
    std::vector<int> iccs, sccs;
    for (int c : {1, 4, 8, 16, 32})
        if (c == 1 || c <= p->nc) iccs.push_back(c);
    for (int c : {32, 16, 8, 4, 2, 1})
        if (c <= p->nc && (int)sccs.size() < 3) sccs.push_back(c);
    cgs_tuning best = p->tune, cur = p->tune;
    double t_int = 1e30, t_spr = 1e30, t = 0.0;
    // interpolation: the tensor cores, then CUDA-core bin sides and coils per CTA,
    // then the work slice
    CGS_TRY(fill(p->grid, gridN, 0x9e3779b9u));
    bool imma_best = false;
    for (int ib : {16, 64}) {   // mma.sync on 4 x 4 bins, tcgen05 on 8 x 16 bins
        cur = best; cur.interp_block = ib;
        p->tune = cur;
        CGS_TRY(rebin(p));
        if (p->geom.imma == (ib == 64 ? 2 : 1)) {
            CGS_TRY(timed(interp, &t));
            if (t < t_int) { t_int = t; best.interp_block = ib; imma_best = true; }
        }
    }
    for (int tile : {8, 16, 32}) {
        if (tile > p->n[0] || tile > p->n[1]) continue;
        cur = best; cur.tile = tile; cur.work_slice = 512; cur.interp_block = 1;
        p->tune = cur;
        CGS_TRY(rebin(p));
        const int E = std::min(tile, std::min(p->n[0], p->n[1])) + 2 * p->m + 1;
        for (int c : iccs) {
            if ((size_t)E * E * c * sizeof(float2) > 200 * 1024) continue;  // keeps the register-tile kernel
            p->tune.interp_coils = c;
            apply_tiles(p);
            CGS_TRY(timed(interp, &t));
            if (t < t_int) {
                t_int = t; best.tile = tile; best.work_slice = 512; best.interp_coils = c; best.interp_block = 1;
                imma_best = false;
            }
        }
    }
    for (int slice : {128, 256, 1024}) {
        if (imma_best) break;  // the tensor-core kernel does not use the work slices
        cur = best; cur.work_slice = slice;
        p->tune = cur;
        CGS_TRY(rebin(p));
        CGS_TRY(timed(interp, &t));
        if (t < t_int) { t_int = t; best.work_slice = slice; }
    }
    // spreading: points per lane, chunk bound and coils per warp
    CGS_TRY(fill(p->ksV, ksN, 0x85ebca6bu));
    for (int blk : {64, 16, 1, 2, 4, 8}) {
        if ((blk == 2 || blk == 4) && p->nc < 4) continue;
        if (blk == 8 && (p->nc < 2 || p->nc > 16)) continue;
        for (int chunk : {0, 64, 128, 256, 512, 1024}) {
            if (blk > 1 && blk < 16 && chunk != 0 && chunk != 512) continue;  // block variants: two chunk bounds
            if (blk >= 16 && chunk == 64) continue;
            cur = best; cur.spread_chunk = chunk; cur.spread_block = blk;
            p->tune = cur;
            CGS_TRY(rebin(p));
            for (int c : sccs) {
                if (blk >= 16 && c != sccs.front()) continue;  // the tensor-core kernels set their own coil width
                if ((blk == 2 || blk == 4) && c < 4) continue;
                if (blk == 8 && c > 16) continue;
                p->tune.spread_coils = c;
                apply_tiles(p);
                CGS_TRY(timed(spread, &t));
                if (t < t_spr) { t_spr = t; best.spread_chunk = chunk; best.spread_coils = c; best.spread_block = blk; }
            }
        }
    }
    p->tune = best;
    apply_tiles(p);
    CGS_TRY(rebin(p));
    if (chosen) *chosen = best;
    if (ms) *ms = t_int + t_spr;
    {
        std::lock_guard<std::mutex> lk(g_tune_mx);
        if (g_tune_cache_on) g_tune_cache[key] = {best, t_int + t_spr};
    }
    return CGS_OK;
}


}  // extern "C"

struct cgs_batch {
    std::vector<cgs_plan *> plans;
    std::vector<cgs_solve_opts> opts;
    std::vector<uint64_t> gens;
    std::vector<int64_t> kpro, kbody;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    CGScalars *host_sc = nullptr;  // pinned, one per plan
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int device = 0;
};

extern "C" {

cgs_status cgs_batch_destroy(cgs_batch *b)
{
    if (!b) return CGS_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->host_sc) cudaFreeHost(b->host_sc);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return CGS_OK;
}

cgs_status cgs_batch_create(cgs_batch **out, cgs_plan *const *plans, const cgs_solve_opts *opts, int count,
                            void *stream)
{
    if (!out || !plans || !opts || count < 1) { set_error("bad argument"); return CGS_ERR_BAD_ARG; }
    *out = nullptr;
    for (int i = 0; i < count; ++i) {
        cgs_plan *p = plans[i];
        const cgs_solve_opts *o = &opts[i];
        if (!p) { set_error("null plan in batch"); return CGS_ERR_BAD_ARG; }
        if (p->F > 1) { set_error("batches take single-frame plans"); return CGS_ERR_BAD_ARG; }
        if (p->device != plans[0]->device) { set_error("batch plans must share a device"); return CGS_ERR_BAD_ARG; }
        for (int j = 0; j < i; ++j)
            if (plans[j] == p) { set_error("a plan appears twice in the batch"); return CGS_ERR_BAD_ARG; }
        const bool codeare = o->mode == CGS_MODE_CODEARE;
        CGS_TRY(check_ready(p, codeare || o->weighted, true));
        if (o->cgiter < 1 || o->cgiter > 100000 || o->ftiter < 0) { set_error("bad iteration counts"); return CGS_ERR_BAD_ARG; }
    }
    cgs_batch *b = new cgs_batch();
    b->device = plans[0]->device;
    cudaSetDevice(b->device);
    cgs_status r = CGS_OK;
    if (stream) b->stream = (cudaStream_t)stream;
    else if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess) b->own_stream = true;
    else r = CGS_ERR_CUDA;
    if (r == CGS_OK && (cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess)) r = CGS_ERR_CUDA;
    if (r == CGS_OK && cudaMallocHost(&b->host_sc, sizeof(CGScalars) * count) != cudaSuccess) r = CGS_ERR_OOM;
    cudaStream_t st = b->stream;
    // Toeplitz kernels first: building one invalidates the plan's graphs
    for (int i = 0; i < count && r == CGS_OK; ++i) {
        cgs_plan *p = plans[i];
        const cgs_solve_opts &o = opts[i];
        if (o.toeplitz) {
            if (p->F > 1) { set_error("the Toeplitz operator is not built for frames"); r = CGS_ERR_BAD_ARG; break; }
            r = check_codeare_toeplitz(p, &o);
            const int wtd = toeplitz_weighting(p, &o);
            if (r == CGS_OK && (!p->toep_valid || p->toep_weighted != wtd)) r = build_toeplitz(p, wtd, st);
        }
    }
    cudaGraph_t g = nullptr;
    if (r == CGS_OK && cudaGraphCreate(&g, 0) != cudaSuccess) r = CGS_ERR_CUDA;
    for (int i = 0; i < count && r == CGS_OK; ++i) {
        cgs_solve_opts o = opts[i];
        int64_t kp = 0, kb = 0;
        r = append_solve(plans[i], &o, g, true, st, &kp, &kb);
        b->plans.push_back(plans[i]);
        b->opts.push_back(o);
        b->kpro.push_back(kp);
        b->kbody.push_back(kb);
    }
    if (r == CGS_OK && cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) {
        set_error("cudaGraphInstantiate of the batch graph failed");
        r = CGS_ERR_CUDA;
    }
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    if (r != CGS_OK) { b->exec = nullptr; cgs_batch_destroy(b); return r; }
    for (cgs_plan *p : b->plans) b->gens.push_back(p->gen);
    *out = b;
    return CGS_OK;
}

cgs_status cgs_batch_solve(cgs_batch *b, const float *const *y, float *const *x, cgs_solve_report *reports,
                           double *seconds)
{
    if (!b || !y || !x) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    const int count = (int)b->plans.size();
    for (int i = 0; i < count; ++i) {
        if (!y[i] || !x[i]) { set_error("null data pointer in batch"); return CGS_ERR_BAD_ARG; }
        if (b->plans[i]->gen != b->gens[i]) {
            set_error("a plan of the batch changed after the batch was built");
            return CGS_ERR_STATE;
        }
    }
    CGS_CUDA(cudaSetDevice(b->device));
    cudaStream_t st = b->stream;
    for (int i = 0; i < count; ++i) CGS_TRY(ks_in(b->plans[i], y[i], st));
    CGS_CUDA(cudaEventRecord(b->ev0, st));
    CGS_CUDA(cudaGraphLaunch(b->exec, st));
    CGS_CUDA(cudaEventRecord(b->ev1, st));
    for (int i = 0; i < count; ++i)
        CGS_CUDA(cudaMemcpyAsync(&b->host_sc[i], b->plans[i]->sc, sizeof(CGScalars), cudaMemcpyDeviceToHost, st));
    for (int i = 0; i < count; ++i) CGS_TRY(image_out(b->plans[i], b->plans[i]->vX, x[i], st));
    CGS_CUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    CGS_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    if (seconds) *seconds = ms * 1e-3;
    cgs_status result = CGS_OK;
    for (int i = 0; i < count; ++i) {
        const CGScalars &h = b->host_sc[i];
        const bool codeare = b->opts[i].mode == CGS_MODE_CODEARE;
        count_launch((int)(b->kpro[i] + (int64_t)h.iter * b->kbody[i]));
        if (h.nan_flag) result = CGS_ERR_NAN;
        if (reports) {
            cgs_solve_report *rep = &reports[i];
            std::memset(rep, 0, sizeof(*rep));
            rep->fallback_at = -1;
            const int nh = std::min(256, h.iter + 1);
            for (int k = 0; k < nh; ++k) rep->res_hist[k] = h.hist[k];
            rep->res_first = h.hist[0];
            const double ratio = h.rn / h.xn;
            rep->res_last = codeare ? ratio : std::sqrt(ratio);
            if (!codeare && h.iter < 256) rep->res_hist[h.iter] = rep->res_last;
            rep->iterations = h.iter;
            rep->seconds = ms * 1e-3;
        }
    }
    if (result == CGS_ERR_NAN) set_error("NaN in a batch solve");
    return result;
}

}  // extern "C"

// ===========================================================================
// Compressed sensing over the NCSENSE operator (CS_XSENSE with ft = 3)
// ===========================================================================
struct cgs_cs {
    cgs_plan *p = nullptr;
    int device = 0;  // the plan's device (destroy must not touch the plan, which may be gone)
    int ft = 3;      // 3 NCSENSE, 2 plain NFFT
    cgs_cs_opts o{};
    CsTerms tm{};
    cgs_solve_opts so{};
    // image vectors (codeare order) and k-space vectors (the plan's sorted layout)
    float2 *x = nullptr, *g0 = nullptr, *g1 = nullptr, *dx = nullptr;
    float2 *ksData = nullptr, *ksE = nullptr, *ksG = nullptr;
    double *partial = nullptr;   // 2 * kCsBlocks * kCsSteps
    double *sums = nullptr;      // [0..31] objective per step, [32..47] dots, [48] nnz
    unsigned int *amax = nullptr;
    int *tally = nullptr;        // solve iterations, NaN flag
    double *hsums = nullptr;     // pinned copy of sums
    int solves = 0;
    double ndnz = 0.0;
    // wavelet transform (the NLCG variable is the coefficient array when on)
    bool dwt = false;
    int dwt_levels = 0;
    DwtFilt filt{};
    float2 *wx = nullptr, *wdx = nullptr, *wtmp = nullptr, *wu = nullptr;
    const float2 *wxp = nullptr;  // image of the last df's x (x itself without a wavelet)
};

namespace {

// slots in cgs_cs::sums
constexpr int kSumDots = 2 * kCsSteps;  // (re, im) pairs: g0.dx, dx.dx, x.x, gsq[0], gsq[1]
constexpr int kDotG0Dx = kSumDots, kDotDx = kSumDots + 2, kDotX = kSumDots + 4, kDotGsq = kSumDots + 6;
constexpr int kSumNnz = kSumDots + 10;
constexpr int kSumCount = kSumNnz + 1;

// codeare CGLS from p->ksY into p->vX, on the device only (the loop scalars
// stay there; cs_tally adds its iterations and NaN flag)
cgs_status cs_solve(cgs_cs *c, cudaStream_t st)
{
    cgs_plan *p = c->p;
    const cgs_solve_opts *o = &c->so;
    c->solves++;
    if (c->ft == 2) {  // NFFT ->*: the CGNR inverse NFFT of the single coil (NFFT.hpp:370-436)
        CGS_TRY(op_itrafo(p, p->ksY, o->ftiter, o->fteps, st));
        CGS_CUDA(cudaMemcpyAsync(p->vX, p->cF, sizeof(float2) * p->Nt, cudaMemcpyDeviceToDevice, st));
        return CGS_OK;
    }
    if (o->cgiter == 0) return op_eh_codeare(p, p->ksY, o->ftiter, o->fteps, p->vX, st);  // CGLS.hpp:32-33
    const bool same = p->solve_exec && p->sg_mode == CGS_MODE_CODEARE && p->sg_toep == 0 &&
                      p->sg_weighted == o->weighted && p->sg_ftiter == o->ftiter && p->sg_fteps == o->fteps;
    if (!same) CGS_TRY(build_solve_graph(p, o, st));
    CGScalars init{};
    init.lambda = o->lambda;
    init.tol = o->cgeps;
    init.maxit = o->cgiter;
    init.sqrt_mode = 0;
    CGS_CUDA(cudaMemcpyAsync(p->sc, &init, sizeof(init), cudaMemcpyHostToDevice, st));
    CGS_CUDA(cudaGraphLaunch(p->solve_exec, st));
    count_launch((int)p->sg_kpro);
    return launch_cs_tally(p->sc, c->tally, st);
}

// out = W in (inverse 0) or W^-1 in (inverse 1), the reference's DWT
// operator * and ->* (DWT.hpp:354-418, 756-823); a copy without a wavelet
cgs_status cs_dwt(cgs_cs *c, const float2 *in, float2 *out, int inverse, cudaStream_t st)
{
    cgs_plan *p = c->p;
    if (in != out) CGS_CUDA(cudaMemcpyAsync(out, in, sizeof(float2) * p->Nt, cudaMemcpyDeviceToDevice, st));
    if (!c->dwt) return CGS_OK;
    const int S = c->tm.D0;
    if (!inverse) {
        int n = S;
        for (int l = 0; l < c->dwt_levels; ++l, n /= 2) {
            CGS_TRY(launch_dwt_pass(out, c->wtmp, S, n, 0, 0, c->filt, st));
            CGS_TRY(launch_dwt_pass(c->wtmp, out, S, n, 1, 0, c->filt, st));
        }
    } else {
        int n = S >> c->dwt_levels;
        for (int l = 0; l < c->dwt_levels; ++l, n *= 2) {
            CGS_TRY(launch_dwt_pass(out, c->wtmp, S, 2 * n, 1, 1, c->filt, st));
            CGS_TRY(launch_dwt_pass(c->wtmp, out, S, 2 * n, 0, 1, c->filt, st));
        }
    }
    return CGS_OK;
}

// the CS operator's forward (ft * x): E of NCSENSE, or the single-coil NFFT
cgs_status cs_E(cgs_cs *c, const float2 *x, float2 *ks, cudaStream_t st)
{
    return op_forward(c->p, x, c->ft == 2 ? 1 : 0, nullptr, ks, st);
}

// g = df(x) (CS_XSENSE.hpp:223-232); leaves E wx in ksE and wx in wxp for
// the next Update and objective
cgs_status cs_df(cgs_cs *c, const float2 *x, float2 *g, cudaStream_t st)
{
    cgs_plan *p = c->p;
    const int64_t nks = p->M * p->nc;
    if (c->dwt) CGS_TRY(cs_dwt(c, x, c->wx, 1, st));
    c->wxp = c->dwt ? c->wx : x;
    CGS_TRY(cs_E(c, c->wxp, c->ksE, st));
    CGS_TRY(launch_cs_sub(p->ksY, c->ksE, c->ksData, nks, st));
    CGS_TRY(cs_solve(c, st));
    if (!c->dwt) return launch_cs_grad(x, p->vX, c->tm, g, st);
    // W (2 ehr + TV terms of wx) + the L1 term of the coefficients
    CsTerms img = c->tm;
    img.xfmw = 0.f;
    CGS_TRY(launch_cs_grad(c->wxp, p->vX, img, c->wu, st));
    CGS_TRY(cs_dwt(c, c->wu, g, 0, st));
    return c->tm.xfmw != 0.f ? launch_cs_l1grad(g, x, c->tm, p->Nt, st) : CGS_OK;
}

// Update(dx): ffdbg = E W^-1 dx (CS_XSENSE.hpp:234-236); returns the image of dx
cgs_status cs_update(cgs_cs *c, const float2 *dx, const float2 **wdxp, cudaStream_t st)
{
    if (c->dwt) CGS_TRY(cs_dwt(c, dx, c->wdx, 1, st));
    *wdxp = c->dwt ? c->wdx : dx;
    return cs_E(c, *wdxp, c->ksG, st);
}

cgs_status cs_read(cgs_cs *c, cudaStream_t st)
{
    CGS_CUDA(cudaMemcpyAsync(c->hsums, c->sums, sizeof(double) * kSumCount, cudaMemcpyDeviceToHost, st));
    CGS_CUDA(cudaStreamSynchronize(st));
    return CGS_OK;
}

// one NLCG minimisation of x in place (NLCG.hpp:84-125)
cgs_status cs_minimise(cgs_cs *c, cgs_cs_report *rep, cudaStream_t st)
{
    cgs_plan *p = c->p;
    const cgs_cs_opts &o = c->o;
    const int64_t Nt = p->Nt, nks = p->M * p->nc;
    float t0 = 1.f, t = 1.f;
    int cur = 0;  // which gsq slot holds |g0|^2
    CGS_TRY(launch_cs_dot(c->x, c->x, Nt, c->partial, c->sums + kDotX, st));
    CGS_TRY(cs_df(c, c->x, c->g0, st));
    CGS_TRY(launch_cs_dot(c->g0, c->g0, Nt, c->partial, c->sums + kDotGsq, st));
    CGS_TRY(launch_cs_dir(c->dx, c->g0, nullptr, nullptr, Nt, st));
    double xn = -1.0;
    for (int k = 0; k < o.nliter; ++k) {
        // Update(dx): ffdbx = E wx is in ksE from the last df, ffdbg = E wdx
        const float2 *wdxp = nullptr;
        CGS_TRY(cs_update(c, c->dx, &wdxp, st));
        CGS_TRY(launch_cs_dot(c->g0, c->dx, Nt, c->partial, c->sums + kDotG0Dx, st));
        // f0 and the line search (NLCG.hpp:42-54), kCsSteps - 1 candidates per pass
        int li = o.lsiter;
        double rmse = 0.0, f0 = 0.0, g0dx = 0.0;
        const float tprev = t;
        for (int base = 0; base < o.lsiter && li == o.lsiter; base += kCsSteps - 1) {
            CsSteps steps{};
            steps.t[0] = 0.f;
            steps.n = 1;
            for (int i = base; i < o.lsiter && steps.n < kCsSteps; ++i)
                steps.t[steps.n++] = (float)((double)t0 * std::pow((double)o.lsb, (double)(i + 1)));
            CGS_TRY(launch_cs_obj(c->ksE, c->ksG, c->ksData, nks, c->wxp, wdxp, c->x, c->dx, c->tm, steps,
                                  c->partial, c->sums, st));
            CGS_TRY(cs_read(c, st));
            if (xn < 0.0) xn = std::sqrt(c->hsums[kDotX]);
            const double *h = c->hsums;
            f0 = h[0] + h[kCsSteps];
            g0dx = std::hypot(h[kDotG0Dx], h[kDotG0Dx + 1]);
            rmse = std::sqrt(h[0] / c->ndnz);
            for (int j = 1; j < steps.n; ++j) {
                const double tj = steps.t[j];
                const double f1 = h[j] + h[kCsSteps + j];
                const double lim = f0 - (double)o.lsa * (o.parallel_linesearch ? (double)tprev : tj) * g0dx;
                if (f1 <= lim) {
                    li = base + j - 1;
                    t = steps.t[j];
                    rmse = std::sqrt(h[j] / c->ndnz);
                    break;
                }
            }
            if (li == o.lsiter && steps.n > 1) rmse = std::sqrt(h[steps.n - 1] / c->ndnz);
        }
        if (rep && rep->iterations < 256) {
            rep->ls_index[rep->iterations] = li;
            rep->rmse[rep->iterations] = rmse;
        }
        if (rep) rep->iterations++;
        if (li == o.lsiter) return CGS_OK;  // "Reached max line search, exiting"
        if (li > 2) t0 *= o.lsb;
        else if (li < 1) t0 /= o.lsb;
        CGS_TRY(launch_cs_axpy(c->x, c->dx, t, Nt, st));
        CGS_TRY(cs_df(c, c->x, c->g1, st));
        double *gsq0 = c->sums + kDotGsq + 2 * cur, *gsq1 = c->sums + kDotGsq + 2 * (1 - cur);
        CGS_TRY(launch_cs_dot(c->g1, c->g1, Nt, c->partial, gsq1, st));
        CGS_TRY(launch_cs_dir(c->dx, c->g1, gsq1, gsq0, Nt, st));
        std::swap(c->g0, c->g1);
        cur = 1 - cur;
        CGS_TRY(launch_cs_dot(c->dx, c->dx, Nt, c->partial, c->sums + kDotDx, st));
        CGS_TRY(cs_read(c, st));
        if (std::sqrt(c->hsums[kDotDx]) / xn < (double)o.cgconv) break;
    }
    return CGS_OK;
}

cgs_status cs_data_in(cgs_cs *c, const float *y, cudaStream_t st)
{
    cgs_plan *p = c->p;
    CGS_TRY(gather_ks(p, y, c->ksData, st));
    CGS_TRY(launch_cs_nnz(c->ksData, p->M * p->nc, c->partial, c->sums + kSumNnz, st));
    CGS_TRY(cs_read(c, st));
    c->ndnz = c->hsums[kSumNnz];
    return CGS_OK;
}

cgs_status cs_image_in(cgs_plan *p, const float *src, float2 *dst, cudaStream_t st)
{
    CGS_CUDA(cudaMemcpyAsync(dst, src, sizeof(float2) * p->Nt,
                             is_device_ptr(src) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    return CGS_OK;
}

// Minimum-phase Daubechies low-pass filter with p = taps / 2 vanishing
// moments (I. Daubechies, Comm. Pure Appl. Math. 41 (1988) 909-996), by
// spectral factorisation: the roots y_k of P(y) = sum_k C(p-1+k, k) y^k
// (Durand-Kerner iteration), each mapped to the root w_k of
// w + 1/w = 2 - 4 y_k outside the unit circle; h(w) = (1 + w)^p prod (w - w_k)
// in ascending powers, scaled to sum sqrt(2).  p = 1 is the Haar filter.
std::vector<double> daubechies(int taps)
{
    typedef std::complex<double> cd;
    const int p = taps / 2, deg = p - 1;
    std::vector<cd> poly(1, cd(1.0, 0.0));
    auto mul = [&](cd a0, cd a1) {  // poly *= a0 + a1 w
        std::vector<cd> r(poly.size() + 1, cd(0.0, 0.0));
        for (size_t i = 0; i < poly.size(); ++i) {
            r[i] += poly[i] * a0;
            r[i + 1] += poly[i] * a1;
        }
        poly.swap(r);
    };
    for (int i = 0; i < p; ++i) mul(cd(1.0, 0.0), cd(1.0, 0.0));
    if (deg > 0) {
        std::vector<double> c(p);
        for (int k = 0; k < p; ++k) {
            double b = 1.0;  // C(p-1+k, k)
            for (int j = 1; j <= k; ++j) b = b * (p - 1 + j) / j;
            c[k] = b;
        }
        auto eval = [&](cd x) {  // monic P
            cd v(0.0, 0.0);
            for (int k = deg; k >= 0; --k) v = v * x + c[k] / c[deg];
            return v;
        };
        std::vector<cd> z(deg);
        for (int i = 0; i < deg; ++i) z[i] = std::pow(cd(0.4, 0.9), i);
        for (int it = 0; it < 1000; ++it) {
            double delta = 0.0;
            for (int i = 0; i < deg; ++i) {
                cd den(1.0, 0.0);
                for (int j = 0; j < deg; ++j)
                    if (j != i) den *= z[i] - z[j];
                const cd step = eval(z[i]) / den;
                z[i] -= step;
                delta = std::max(delta, std::abs(step));
            }
            if (delta < 1e-16) break;
        }
        for (const cd &y : z) {
            const cd b = 2.0 - 4.0 * y, q = std::sqrt(b * b - 4.0);
            const cd w1 = 0.5 * (b + q), w2 = 0.5 * (b - q);
            mul(-(std::abs(w1) > std::abs(w2) ? w1 : w2), cd(1.0, 0.0));
        }
    }
    std::vector<double> h(poly.size());
    double sum = 0.0;
    for (size_t i = 0; i < h.size(); ++i) sum += (h[i] = poly[i].real());
    for (double &v : h) v *= std::sqrt(2.0) / sum;
    return h;
}

// TVOP::Trafo's choice of operator (TVOP.hpp:277-295) for a rank-d image
int cs_tv_mode(int d, const int *dims, int nd)
{
    if (d == 2 && (nd == 0 || (nd >= 2 && dims[0] == 1 && dims[1] == 1))) return 1;
    if (d == 3 && (nd == 0 || (nd >= 3 && dims[0] == 1 && dims[1] == 1 && dims[2] == 1))) return 2;
    if (d == 3 && nd >= 3 && dims[0] == 0 && dims[1] == 0 && dims[2] == 1) return 3;
    return -1;
}

}  // namespace

extern "C" {

cgs_status cgs_cs_create(cgs_cs **out, cgs_plan *p, const cgs_cs_opts *o)
{
    if (!out || !o) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    *out = nullptr;
    const int ft = o->ft == 0 ? 3 : o->ft;
    if (ft != 2 && ft != 3) { set_error("ft: 2 (NFFT) or 3 (NCSENSE)"); return CGS_ERR_BAD_ARG; }
    CGS_TRY(check_ready(p, true, ft == 3));
    if (ft == 2 && (p->nc != 1 || p->F > 1)) { set_error("ft = 2 takes a single-coil, single-frame plan"); return CGS_ERR_BAD_ARG; }
    if (o->nlopt != 0 && o->nlopt != 2) { set_error("nlopt: only 0 (NLCG) and 2 (Split Bregman)"); return CGS_ERR_BAD_ARG; }
    // the reference initialises filters for Daubechies 4 / 8 and Haar 2 only (Wavelet.hpp:165-200)
    const bool dwt = o->wl_family > -1 && o->wl_family <= 5;
    if (dwt && !((o->wl_family == 0 && (o->wl_member == 4 || o->wl_member == 8)) ||
                 (o->wl_family == 2 && o->wl_member == 2))) {
        set_error("wavelet: families 0 (members 4, 8) and 2 (member 2) have filters");
        return CGS_ERR_BAD_ARG;
    }
    if (o->cgiter < 0 || o->ftiter < 0 || o->csiter < 0 || o->nliter < 0 || o->lsiter < 0) {
        set_error("negative iteration count");
        return CGS_ERR_BAD_ARG;
    }
    if (p->F > 1 && p->d != 2) { set_error("CS over frames takes 2-D frames"); return CGS_ERR_BAD_ARG; }
    CsTerms tm{};
    // codeare order: axis 0 is the plan's fastest axis; frames are the third
    // axis of the image (the dim4 image (N, N, nt), NCSENSE.hpp:173-180)
    const int rank = p->F > 1 ? 3 : p->d;
    tm.D0 = p->N[p->d - 1];
    tm.D1 = p->N[p->d - 2];
    tm.D2 = p->F > 1 ? p->F : (p->d >= 3 ? p->N[p->d - 3] : 1);
    for (int i = 0; i < 2; ++i) {
        tm.tvw[i] = o->tvw[i];
        if (o->tvw[i] == 0.f) continue;
        const int nd = std::max(0, std::min(3, o->ntvdims[i]));
        tm.tvmode[i] = cs_tv_mode(rank, o->tvdims[i], nd);
        if (tm.tvmode[i] < 0) { set_error("no TV operator for these image axes"); return CGS_ERR_BAD_ARG; }
        if (tm.tvmode[i] != 3 && tm.D0 != tm.D1) { set_error("TV over axes 0 and 1 needs a square image"); return CGS_ERR_BAD_ARG; }
        if (tm.tvmode[i] == 3 && tm.D2 < 2) { set_error("TV over axis 2 needs at least 2 slices"); return CGS_ERR_BAD_ARG; }
    }
    tm.xfmw = o->xfmw;
    tm.l1 = o->l1;
    tm.pnorm = o->pnorm;
    int levels = 0;
    if (dwt) {
        // DWT<T>(N) of CS_XSENSE.hpp:133: a square 2-D transform with dyadic
        // sides down to 2^4 (WL_SCALE, DWT.hpp:38-40)
        if (rank != 2 || tm.D0 != tm.D1 || (tm.D0 & (tm.D0 - 1)) != 0) {
            set_error("the wavelet transform needs a square 2-D image with dyadic sides");
            return CGS_ERR_BAD_ARG;
        }
        int L = 0;
        while ((1 << L) < tm.D0) ++L;
        levels = std::max(0, L - 4);
    }
    cgs_cs *c = new cgs_cs;
    c->p = p;
    c->device = p->device;
    c->ft = ft;
    c->o = *o;
    c->tm = tm;
    c->dwt = dwt;
    c->dwt_levels = levels;
    if (dwt) {
        const std::vector<double> h = daubechies(o->wl_member);
        c->filt.fl = (int)h.size();
        for (int i = 0; i < c->filt.fl; ++i) {
            c->filt.lo[i] = (float)h[i];
            c->filt.hi[i] = (float)((i & 1) ? -h[i] : h[i]);  // mirrorfilt, Wavelet.hpp:12-19
        }
    }
    c->so.mode = CGS_MODE_CODEARE;
    c->so.cgiter = o->cgiter;
    c->so.cgeps = o->cgeps;
    c->so.lambda = o->lambda;
    c->so.ftiter = o->ftiter;
    c->so.fteps = o->fteps;
    c->so.weighted = 1;
    const int64_t Nt = p->Nt, nks = p->M * p->nc;
    cgs_status r = CGS_OK;
    if (r == CGS_OK) r = dev_alloc(&c->x, Nt);
    if (r == CGS_OK) r = dev_alloc(&c->g0, Nt);
    if (r == CGS_OK) r = dev_alloc(&c->g1, Nt);
    if (r == CGS_OK) r = dev_alloc(&c->dx, Nt);
    if (r == CGS_OK) r = dev_alloc(&c->ksData, nks);
    if (r == CGS_OK) r = dev_alloc(&c->ksE, nks);
    if (r == CGS_OK) r = dev_alloc(&c->ksG, nks);
    if (r == CGS_OK) r = dev_alloc(&c->partial, (size_t)2 * kCsBlocks * kCsSteps);
    if (r == CGS_OK) r = dev_alloc(&c->sums, kSumCount);
    if (r == CGS_OK) r = dev_alloc(&c->amax, 1);
    if (r == CGS_OK) r = dev_alloc(&c->tally, 2);
    if (r == CGS_OK && dwt) r = dev_alloc(&c->wx, Nt);
    if (r == CGS_OK && dwt) r = dev_alloc(&c->wdx, Nt);
    if (r == CGS_OK && dwt) r = dev_alloc(&c->wtmp, Nt);
    if (r == CGS_OK && dwt) r = dev_alloc(&c->wu, Nt);
    if (r == CGS_OK && cudaMallocHost((void **)&c->hsums, sizeof(double) * kSumCount) != cudaSuccess) {
        set_error("cudaMallocHost failed");
        r = CGS_ERR_OOM;
    }
    if (r == CGS_OK && cudaMemset(c->sums, 0, sizeof(double) * kSumCount) != cudaSuccess) r = CGS_ERR_CUDA;
    if (r != CGS_OK) {
        cgs_cs_destroy(c);
        return r;
    }
    *out = c;
    return CGS_OK;
}

cgs_status cgs_cs_destroy(cgs_cs *c)
{
    if (!c) return CGS_OK;
    cudaSetDevice(c->device);  // cudaFree waits for work still using the buffers
    for (void *q : {(void *)c->x, (void *)c->g0, (void *)c->g1, (void *)c->dx, (void *)c->ksData, (void *)c->ksE,
                    (void *)c->ksG, (void *)c->partial, (void *)c->sums, (void *)c->amax, (void *)c->tally,
                    (void *)c->wx, (void *)c->wdx, (void *)c->wtmp, (void *)c->wu})
        dev_free(q);
    if (c->hsums) cudaFreeHost(c->hsums);
    delete c;
    return CGS_OK;
}

cgs_status cgs_cs_adjoint(cgs_cs *c, const float *y, float *x, cgs_cs_report *rep, void *stream)
{
    if (!c || !y || !x) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    cgs_plan *p = c->p;
    CGS_TRY(check_ready(p, true, c->ft == 3));
    cudaStream_t st = pick_stream(p, stream);
    if (rep) std::memset(rep, 0, sizeof(*rep));
    CGS_CUDA(cudaEventRecord(p->ev0, st));
    c->solves = 0;
    CGS_CUDA(cudaMemsetAsync(c->tally, 0, 2 * sizeof(int), st));
    CGS_TRY(cs_data_in(c, y, st));
    // x0 = ft ->* data, the CG-SENSE solve (CS_XSENSE.hpp:293-297)
    CGS_CUDA(cudaMemcpyAsync(p->ksY, c->ksData, sizeof(float2) * p->M * p->nc, cudaMemcpyDeviceToDevice, st));
    CGS_TRY(cs_solve(c, st));
    CGS_TRY(cs_dwt(c, p->vX, c->x, 0, st));  // x = W x0 (CS_XSENSE.hpp:301-302)
    // TV weights *= max |x| (CS_XSENSE.hpp:303-305; cumulative over calls, as the reference's)
    CGS_TRY(launch_cs_absmax(c->x, p->Nt, c->amax, st));
    unsigned int bits = 0;
    CGS_CUDA(cudaMemcpyAsync(&bits, c->amax, sizeof(bits), cudaMemcpyDeviceToHost, st));
    CGS_CUDA(cudaStreamSynchronize(st));
    float ma;
    std::memcpy(&ma, &bits, sizeof(ma));
    for (int i = 0; i < 2; ++i) c->tm.tvw[i] *= ma;
    if (c->o.nlopt == 0)
        for (int i = 0; i < c->o.csiter; ++i) CGS_TRY(cs_minimise(c, rep, st));
    if (c->dwt) CGS_TRY(cs_dwt(c, c->x, c->wu, 1, st));  // CS_XSENSE.hpp:317-318
    CGS_CUDA(cudaEventRecord(p->ev1, st));
    CGS_TRY(image_out(p, c->dwt ? c->wu : c->x, x, st));
    int tally[2] = {0, 0};
    CGS_CUDA(cudaMemcpyAsync(tally, c->tally, sizeof(tally), cudaMemcpyDeviceToHost, st));
    CGS_CUDA(cudaStreamSynchronize(st));
    count_launch((int)((int64_t)tally[0] * p->sg_kbody));
    if (rep) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p->ev0, p->ev1);
        rep->seconds = ms * 1e-3;
        rep->solves = c->solves;
        rep->solve_iterations = tally[0];
        rep->tvw_used[0] = c->tm.tvw[0];
        rep->tvw_used[1] = c->tm.tvw[1];
    }
    if (tally[1]) { set_error("NaN in a CG-SENSE solve"); return CGS_ERR_NAN; }
    return CGS_OK;
}

cgs_status cgs_cs_df(cgs_cs *c, const float *y, const float *x, float *g, void *stream)
{
    if (!c || !y || !x || !g) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    cgs_plan *p = c->p;
    CGS_TRY(check_ready(p, true, c->ft == 3));
    cudaStream_t st = pick_stream(p, stream);
    c->solves = 0;
    CGS_CUDA(cudaMemsetAsync(c->tally, 0, 2 * sizeof(int), st));
    CGS_TRY(cs_data_in(c, y, st));
    CGS_TRY(cs_image_in(p, x, c->x, st));
    CGS_TRY(cs_df(c, c->x, c->g0, st));
    CGS_TRY(image_out(p, c->g0, g, st));
    int tally[2] = {0, 0};
    CGS_CUDA(cudaMemcpyAsync(tally, c->tally, sizeof(tally), cudaMemcpyDeviceToHost, st));
    CGS_CUDA(cudaStreamSynchronize(st));
    count_launch((int)((int64_t)tally[0] * p->sg_kbody));
    if (tally[1]) { set_error("NaN in a CG-SENSE solve"); return CGS_ERR_NAN; }
    return CGS_OK;
}

cgs_status cgs_cs_wavelet(cgs_cs *c, const float *in, float *out, int inverse, void *stream)
{
    if (!c || !in || !out) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    cgs_plan *p = c->p;
    CGS_TRY(check_ready(p, true, c->ft == 3));
    cudaStream_t st = pick_stream(p, stream);
    CGS_TRY(cs_image_in(p, in, c->dx, st));
    CGS_TRY(cs_dwt(c, c->dx, c->g1, inverse ? 1 : 0, st));
    return image_out(p, c->g1, out, st);
}

cgs_status cgs_cs_obj(cgs_cs *c, const float *y, const float *x, const float *dx, float t, double *obj,
                      double *rmse, void *stream)
{
    if (!c || !y || !x || !dx || !obj) { set_error("null argument"); return CGS_ERR_BAD_ARG; }
    cgs_plan *p = c->p;
    CGS_TRY(check_ready(p, true, c->ft == 3));
    cudaStream_t st = pick_stream(p, stream);
    CGS_TRY(cs_data_in(c, y, st));
    CGS_TRY(cs_image_in(p, x, c->x, st));
    CGS_TRY(cs_image_in(p, dx, c->dx, st));
    if (c->dwt) CGS_TRY(cs_dwt(c, c->x, c->wx, 1, st));
    c->wxp = c->dwt ? c->wx : c->x;
    CGS_TRY(cs_E(c, c->wxp, c->ksE, st));
    const float2 *wdxp = nullptr;
    CGS_TRY(cs_update(c, c->dx, &wdxp, st));
    CsSteps steps{};
    steps.t[0] = t;
    steps.n = 1;
    CGS_TRY(launch_cs_obj(c->ksE, c->ksG, c->ksData, p->M * p->nc, c->wxp, wdxp, c->x, c->dx, c->tm, steps,
                          c->partial, c->sums, st));
    CGS_TRY(cs_read(c, st));
    *obj = c->hsums[0] + c->hsums[kCsSteps];
    if (rmse) *rmse = std::sqrt(c->hsums[0] / c->ndnz);
    return CGS_OK;
}

}  // extern "C"
