// cgs_static.cu -- a 2-D single-coil NFFT forward that allocates no memory.
//
// Who needs it: callers that may not allocate device memory while they run.
// A real-time reconstruction loop beside an acquisition stream is one:
// cudaMalloc / cudaFree synchronise the whole device and would stall it.  A
// host application that owns a fixed device-memory budget through its own
// pool is another.  The plan-based entry points allocate all their scratch
// at cgs_plan_create; this one keeps its scratch (the oversampled grid, the
// half-transformed rows, twiddles and deapodisation factors) in one
// file-scope __device__ array instead, and takes only caller-owned device
// buffers for its inputs and output.
//
// Limits and rules:
//   * scratch capacity kStaticElems complex floats (4 MiB), held by every GPU
//     that loads this library until the process exits;  a call needs
//     N*n + n*n + 2*n + N <= kStaticElems (n = ceil(alpha*N)), so N = 256 at
//     alpha = 2 is the largest square image; larger sizes are rejected;
//   * every call on a device shares the one array and leaves its contents
//     behind: calls that overlap on the GPU (different streams, or threads
//     without ordering) race and corrupt each other's results;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture.  The address is kept for the life of the
//     process: a cudaDeviceReset unloads the module, and calls on that device
//     after a reset are not supported;
//   * a node outside [-0.5, 0.5) in either coordinate gets NaN in f (the plan
//     entry points reject such a trajectory with an error instead; this call
//     does not read k on the host).
// Nothing here sorts the nodes (sorting needs a plan), so the interpolation
// reads the grid per node straight from global memory / L2.
#include "cgs_internal.cuh"

#include <cmath>
#include <mutex>

namespace cgs {
namespace {

constexpr int64_t kStaticElems = int64_t(1) << 19;  // 524288 complex floats = 4 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float2 g_static_scratch[kStaticElems];

std::mutex g_static_mu;
float2 *g_static_ptr[kMaxDevices] = {};
int g_static_sms[kMaxDevices] = {};

// once per device, with the device current: the array's device address and
// the device's SM count (it sizes the interpolation grid)
cgs_status static_scratch(float2 **out, int *sms)
{
    int dev = 0;
    CGS_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) { set_error("device index out of range"); return CGS_ERR_BAD_ARG; }
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!g_static_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) {
            set_error(std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
            return CGS_ERR_CUDA;
        }
        int nsm = 0;
        e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess || nsm <= 0) {
            set_error(std::string("cudaDeviceGetAttribute(SM count): ") + cudaGetErrorString(e));
            return CGS_ERR_CUDA;
        }
        g_static_ptr[dev] = (float2 *)p;
        g_static_sms[dev] = nsm;
    }
    *out = g_static_ptr[dev];
    *sms = g_static_sms[dev];
    return CGS_OK;
}

// I0 by its power series in FP64 (device)
__device__ double dev_bessel_i0(double x)
{
    double y = 0.25 * x * x, term = 1.0, sum = 1.0;
    for (int k = 1; k < 500; ++k) {
        term *= y / ((double)k * (double)k);
        sum += term;
        if (term < 1e-18 * sum) break;
    }
    return sum;
}

// twiddles exp(-2 pi i t / n) and 1/phihut(k), k = -N/2 .. N/2-1
__global__ void static_tables_kernel(float2 *tw, int n, float *deap, int N, int m, double b)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n + N; t += gridDim.x * blockDim.x) {
        if (t < n) {
            double s, c;
            sincospi(-2.0 * (double)t / (double)n, &s, &c);
            tw[t] = make_float2((float)c, (float)s);
        } else {
            const int i = t - n;
            const double w = 2.0 * 3.14159265358979323846 * (double)(i - N / 2) / (double)n;
            double a = b * b - w * w;
            if (a < 0) a = 0;
            deap[i] = (float)(1.0 / dev_bessel_i0((double)m * sqrt(a)));
        }
    }
}

// one thread per node: 2m+2 separable KB taps per dimension from the grid
__global__ void static_interp_kernel(const float *__restrict__ k, int64_t M, const float2 *__restrict__ grid,
                                     int n, int m, float b, float2 *__restrict__ f)
{
    constexpr int kMaxTaps = 18;
    const int taps = 2 * m + 2;
    const float mf = (float)m;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < M; j += (int64_t)gridDim.x * blockDim.x) {
        const float x0 = k[2 * j], x1 = k[2 * j + 1];
        if (!(x0 >= -0.5f && x0 < 0.5f && x1 >= -0.5f && x1 < 0.5f)) {
            f[j] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
            continue;
        }
        const double nx0 = (double)n * (double)x0, nx1 = (double)n * (double)x1;
        const double c0 = floor(nx0), c1 = floor(nx1);
        const float fr0 = (float)(nx0 - c0), fr1 = (float)(nx1 - c1);
        float w0[kMaxTaps], w1[kMaxTaps];
        for (int q = 0; q < taps; ++q) {
            w0[q] = kb_phi(fr0 + mf - (float)q, mf, b);
            w1[q] = kb_phi(fr1 + mf - (float)q, mf, b);
        }
        int u0 = ((int)c0 - m) % n; if (u0 < 0) u0 += n;
        int u1 = ((int)c1 - m) % n; if (u1 < 0) u1 += n;
        float ax = 0.f, ay = 0.f;
        for (int a = 0; a < taps; ++a) {
            int r = u0 + a; if (r >= n) r -= n;
            const float2 *row = grid + (int64_t)r * n;
            float rx = 0.f, ry = 0.f;
            for (int q = 0; q < taps; ++q) {
                int cidx = u1 + q; if (cidx >= n) cidx -= n;
                const float2 v = row[cidx];
                rx = fmaf(w1[q], v.x, rx); ry = fmaf(w1[q], v.y, ry);
            }
            ax = fmaf(w0[a], rx, ax); ay = fmaf(w0[a], ry, ay);
        }
        f[j] = make_float2(ax, ay);
    }
}

bool on_device(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

bool factor(int n, int *fac, int *nf)
{
    int r = n, k = 0;
    while (r % 8 == 0 && k < 12) { fac[k++] = 8; r /= 8; }
    while (r % 4 == 0 && k < 12) { fac[k++] = 4; r /= 4; }
    while (r % 2 == 0 && k < 12) { fac[k++] = 2; r /= 2; }
    for (int q : {3, 5, 7})
        while (r % q == 0 && k < 12) { fac[k++] = q; r /= q; }
    *nf = k;
    return r == 1;
}

}  // namespace
}  // namespace cgs

using namespace cgs;

extern "C" cgs_status cgs_nfft2d_trafo_noalloc(int N, double alpha, int m, int64_t M, const float *k,
                                               const float *fhat, float *f, void *stream)
{
    if (N < 2 || (N & 1) || !(alpha >= 1.0) || m < 0 || m > 8 || M < 0) {
        set_error("cgs_nfft2d_trafo_noalloc: need even N >= 2, alpha >= 1, 0 <= m <= 8, M >= 0");
        return CGS_ERR_BAD_ARG;
    }
    if (!(alpha * (double)N <= 2048.0)) {  // also catches alpha = inf before the cast below
        set_error("cgs_nfft2d_trafo_noalloc: oversampled size ceil(alpha*N) must be at most 2048");
        return CGS_ERR_BAD_ARG;
    }
    const int n = (int)std::ceil(alpha * N);
    const int64_t need = (int64_t)N * n + (int64_t)n * n + 2 * (int64_t)n + N;
    if (need > kStaticElems) {
        set_error("cgs_nfft2d_trafo_noalloc: N x n + n^2 + 2n + N = " + std::to_string(need) +
                  " complex values exceeds the static scratch of " + std::to_string(kStaticElems) +
                  " (largest square image at alpha = 2 is 256)");
        return CGS_ERR_BAD_ARG;
    }
    AxisPass base{};
    if (!factor(n, base.fac, &base.nfac)) {
        set_error("cgs_nfft2d_trafo_noalloc: oversampled size must factor into 2, 3, 5 and 7");
        return CGS_ERR_BAD_ARG;
    }
    if (M == 0) return CGS_OK;
    if (!k || !fhat || !f || !on_device(k) || !on_device(fhat) || !on_device(f)) {
        set_error("cgs_nfft2d_trafo_noalloc: k, fhat and f must be device pointers");
        return CGS_ERR_BAD_ARG;
    }
    float2 *s = nullptr;
    int sms = 0;
    CGS_TRY(static_scratch(&s, &sms));
    cudaStream_t st = (cudaStream_t)stream;
    float2 *t1 = s;                                  // [N][n]  rows transformed along x
    float2 *grid = t1 + (int64_t)N * n;              // [n][n]
    float2 *tw = grid + (int64_t)n * n;              // n twiddles
    float *deap = reinterpret_cast<float *>(tw + n); // N factors (fits in n float2 slots)
    const double b = 3.14159265358979323846 * (2.0 - 1.0 / ((double)n / (double)N));
    static_tables_kernel<<<(n + N + 255) / 256, 256, 0, st>>>(tw, n, deap, N, m, b);
    CGS_LAUNCH_CHECK();

    base.n = n; base.tw = tw; base.sign = -1; base.in_centred = 1;
    base.load_mode = LOAD_PLAIN; base.store_mode = STORE_PLAIN; base.o1_len = 1;
    AxisPass x = base;  // along x from the image, with deapodisation
    x.outer = N; x.inner = 1; x.Lin = N; x.Lout = n;
    x.load_mode = LOAD_IMAGE; x.img = reinterpret_cast<const float2 *>(fhat); x.img_per_coil = 1;
    x.deap_ax = deap; x.deap_o1 = deap; x.o1_len = N;
    x.dst = t1;
    CGS_TRY(launch_axis_pass(x, st));
    AxisPass y = base;  // along y
    y.outer = 1; y.inner = n; y.Lin = N; y.Lout = n;
    y.src = t1; y.dst = grid;
    CGS_TRY(launch_axis_pass(y, st));
    const int64_t blocks = std::min<int64_t>((M + 255) / 256, (int64_t)sms * 8);
    static_interp_kernel<<<(unsigned)blocks, 256, 0, st>>>(k, M, grid, n, m, (float)b,
                                                          reinterpret_cast<float2 *>(f));
    CGS_LAUNCH_CHECK();
    return CGS_OK;
}
