// sparc_grad.cu -- gradient post-processing on the device (grad.py:42-117, 188-364).
//
// After the batched adjoint runs, the per-source kernels are already resident in HBM.  The
// reference writes them to FITS files and grad.py reads them back to sum, precondition, smooth
// and (anti)symmetrise them, and to form the update direction and the line-search models.
// Here those steps run where the kernels are:
//
//   grad_sum_kernel     K = sum_s kernels[s], H = sum_s |hessians[s]| * rho(z), per-block max H
//   grad_row_kernel     per pair of z-rows: K / max(H / max H, floor), Gaussian filter in the
//                       x-wavenumber by a packed complex FFT (two real rows per FFT, the shared
//                       memory Stockham FFT of the wave solver's row pass), (anti)symmetrise in x
//   grad_col_kernel     z filter (scipy's gaussian_filter1d with mode 'reflect', or grad.py's
//                       11-point 'smooth'), one thread per output point
//   vec_reduce_kernel + vec_final_kernel   dot products and maxima: per-block partials over a
//                       fixed grid, summed by one block in a fixed tree order, so results do
//                       not depend on timing or on earlier calls
//   vec_axpby_kernel    y = a x + b z with a, b either host values or ratios of device scalars
//                       (the L-BFGS two-loop recursion runs without a host round trip)
//   ls_models_kernel    model + eps * update / max(update) * rms(model) for every eps
//
// All of it is FP64: the work is 2-D (nz x nx, about 10^5 points) and bound by launch latency
// and by reading the per-source kernels once (2 nsrc nz nx doubles).
#include <cmath>
#include <string>
#include <vector>

#include "sparc_common.cuh"
#include "sparc_gb300.h"

namespace sparc {
int report_error(int code, const std::string &msg);
}
using namespace sparc;

namespace {

constexpr int GRAD_THREADS = 256;
constexpr int GRAD_BLOCKS = 304;        // 2 x 152 SMs; fixed so every reduction has one order
constexpr int GRAD_WPB = 2;             // row pairs (warps) per block of the x pass
constexpr int GRAD_MAX_RADIUS = 32;     // Gaussian z filter taps on each side
constexpr int GRAD_MAX_PAIRS = 64;      // L-BFGS pairs
constexpr int GRAD_MAX_EPS = 32;        // line-search models per call
constexpr int GRAD_NSCALAR = 8 + 4 * GRAD_MAX_PAIRS;

size_t pad32(size_t n) { return (n + 31) & ~size_t(31); }

// Workspace carve-up (doubles): partials, device scalars, FFT tables, three nz x nx fields.
struct GradWork {
    double *part, *sc, *twr, *twi, *gk, *K, *H, *T;
};
size_t grad_work_doubles(int nx, int nz)
{
    const size_t n = (size_t)(nx > 0 ? nx : 0) * (size_t)(nz > 0 ? nz : 0);
    return pad32(GRAD_BLOCKS) + pad32(GRAD_NSCALAR) + 3 * pad32((size_t)(nx > 0 ? nx : 0)) + 3 * pad32(n);
}
GradWork carve(void *work, int nx, int nz)
{
    double *p = static_cast<double *>(work);
    const size_t n = (size_t)nx * nz;
    GradWork w;
    w.part = p; p += pad32(GRAD_BLOCKS);
    w.sc = p; p += pad32(GRAD_NSCALAR);
    w.twr = p; p += pad32(nx);
    w.twi = p; p += pad32(nx);
    w.gk = p; p += pad32(nx);
    w.K = p; p += pad32(n);
    w.H = p; p += pad32(n);
    w.T = p;
    return w;
}

// max that propagates NaN like numpy's max
__device__ __forceinline__ double nanmax(double a, double b)
{
    if (a != a) return a;
    if (b != b) return b;
    return fmax(a, b);
}

// Fixed-order tree reduction over the block (GRAD_THREADS threads); every thread gets the result.
template <bool MAX>
__device__ __forceinline__ double block_reduce(double v)
{
    __shared__ double s[GRAD_THREADS];
    const int t = threadIdx.x;
    s[t] = v;
    __syncthreads();
#pragma unroll
    for (int w = GRAD_THREADS / 2; w > 0; w >>= 1) {
        if (t < w) s[t] = MAX ? nanmax(s[t], s[t + w]) : s[t] + s[t + w];
        __syncthreads();
    }
    const double r = s[0];
    __syncthreads();
    return r;
}

// ---------------------------------------------------------------------------------------------
// Tables: FFT twiddles exp(-2 pi i t / nx) and the x filter exp(-m^2 / (2 nk^2)) / nx of bin t,
// m = min(t, nx - t) (np.fft.rfftfreq(nx, 1/nx) mirrored onto the full spectrum; the 1/nx is
// irfft's normalisation), grad.py:44-51.
__global__ void grad_tables_kernel(int nx, double nk, double *twr, double *twi, double *gk)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nx) return;
    const double u = 2.0 * (double)t / (double)nx;
    twr[t] = cospi(u);
    twi[t] = -sinpi(u);
    const double m = (double)min(t, nx - t);
    gk[t] = exp(-(m * m) / (2.0 * nk * nk)) / (double)nx;
}

// K, H and the per-block maxima of |H| (grad.py:188-195: the sums over sources in source order,
// then hess * rho(z); without preconditioning the plain sum of the hessians).
__global__ void __launch_bounds__(GRAD_THREADS) grad_sum_kernel(const double *__restrict__ kern,
                                                                const double *__restrict__ hess,
                                                                const double *__restrict__ rho, int nsrc, int nx,
                                                                long long n, int precondition, double *K, double *H,
                                                                double *part)
{
    double m = 0.0;
    for (long long i = (long long)blockIdx.x * GRAD_THREADS + threadIdx.x; i < n; i += (long long)GRAD_BLOCKS * GRAD_THREADS) {
        double ks = 0.0, hs = 0.0;
#pragma unroll 8
        for (int s = 0; s < nsrc; s++) {  // unrolled so that eight sources' loads are in flight
            ks += kern[(size_t)s * n + i];
            const double h = hess[(size_t)s * n + i];
            hs += precondition ? fabs(h) : h;
        }
        if (precondition) hs = hs * rho[i / nx];
        K[i] = ks;
        H[i] = hs;
        m = nanmax(m, fabs(hs));
    }
    m = block_reduce<true>(m);
    if (threadIdx.x == 0) part[blockIdx.x] = m;
}

struct GradRowArgs {
    const double *K, *H, *part, *twr, *twi, *gk;
    double *T;
    int nz, sym, precondition;
    double floor;
};

// One warp per pair of z-rows (packed as the real and imaginary parts of one complex FFT):
// kern = K / max(H / max H, floor) (grad.py:110, 195-196; K / H without preconditioning),
// x filter (grad.py:42-52), then
// 0.5 (f +/- f reversed in x) (grad.py:100-101).  Each row is scaled by an exact power of two
// before the FFT so its rounding is relative to itself, not to its partner row.
template <int N>
__global__ void __launch_bounds__(GRAD_WPB *WARP) grad_row_kernel(GradRowArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *sm = reinterpret_cast<double *>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r0 = 2 * (blockIdx.x * GRAD_WPB + warp);
    if (r0 >= a.nz) return;
    const bool two = r0 + 1 < a.nz;
    double *xr = sm + warp * 4 * N, *xi = xr + N, *yr = xi + N, *yi = yr + N;
    double hm = 0.0;
    for (int i = lane; i < GRAD_BLOCKS; i += WARP) hm = nanmax(hm, a.part[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) hm = nanmax(hm, __shfl_xor_sync(0xffffffffu, hm, o));
    double mr = 0.0, mi = 0.0;
    for (int x = lane; x < N; x += WARP) {
        const size_t q0 = (size_t)r0 * N + x;
        double h = a.H[q0];
        if (a.precondition) {
            h = h / hm;
            if (h < a.floor) h = a.floor;
        }
        xr[x] = a.K[q0] / h;
        double v = 0.0;
        if (two) {
            double h1 = a.H[q0 + N];
            if (a.precondition) {
                h1 = h1 / hm;
                if (h1 < a.floor) h1 = a.floor;
            }
            v = a.K[q0 + N] / h1;
        }
        xi[x] = v;
        mr = fmax(mr, fabs(xr[x]));
        mi = fmax(mi, fabs(v));
    }
    double sr, si, isr, isi;
    warp_row_scale(mr, sr, isr);
    warp_row_scale(mi, si, isi);
    __syncwarp();
    double *fr, *fi;
    FFTRun<double, N, 0, 1>::run(xr, xi, yr, yi, a.twr, a.twi, lane, false, sr, si, fr, fi);
    for (int k = lane; k < N; k += WARP) {
        const double g = __ldg(a.gk + k);
        fr[k] *= g;
        fi[k] *= g;
    }
    __syncwarp();
    double *gr = (fr == xr) ? yr : xr, *gi = (fr == xr) ? yi : xi;
    double *orr, *oi;
    FFTRun<double, N, 0, 1>::run(fr, fi, gr, gi, a.twr, a.twi, lane, true, 1.0, 1.0, orr, oi);
    __syncwarp();
    for (int x = lane; x < N; x += WARP) {
        double f0 = orr[x] * isr, f1 = oi[x] * isi;
        if (a.sym != 0) {
            const double s = (double)a.sym;
            f0 = 0.5 * (f0 + s * (orr[N - 1 - x] * isr));
            f1 = 0.5 * (f1 + s * (oi[N - 1 - x] * isi));
        }
        a.T[(size_t)r0 * N + x] = f0;
        if (two) a.T[(size_t)(r0 + 1) * N + x] = f1;
    }
}

struct GradColArgs {
    const double *T;
    double *out;
    int nx, nz, zfilt, radius;
    double w[GRAD_MAX_RADIUS + 1];  // Gaussian taps w[0] (centre) .. w[radius]
    double c[6];                    // 'smooth': c0 and 0.5 c1 .. 0.5 c5
};

__device__ __forceinline__ int reflect(int i, int n)
{
    int p = i % (2 * n);
    if (p < 0) p += 2 * n;
    return p < n ? p : 2 * n - 1 - p;
}

// z filter, one thread per output point (the field is L2-resident: 8 nz nx bytes).
//  gaussian: scipy's correlate1d for a symmetric kernel, w0 a[k] + sum_{j=r..1} (a[k-j] + a[k+j]) w_j
//            with the 'reflect' extension (d c b a | a b c d | d c b a);
//  smooth:   grad.py:66-87, including its rows 4 and nz-1, which the reference leaves at zero.
__global__ void __launch_bounds__(GRAD_THREADS) grad_col_kernel(GradColArgs a)
{
    const long long n = (long long)a.nx * a.nz;
    const long long i = (long long)blockIdx.x * GRAD_THREADS + threadIdx.x;
    if (i >= n) return;
    const int k = (int)(i / a.nx), x = (int)(i - (long long)k * a.nx);
    const double *T = a.T;
    const int nx = a.nx, nz = a.nz;
    auto at = [&](int kk) { return T[(size_t)kk * nx + x]; };
    double v;
    if (a.zfilt == SPARC_ZFILT_GAUSSIAN) {
        v = at(k) * a.w[0];
        for (int j = a.radius; j >= 1; j--) v += (at(reflect(k - j, nz)) + at(reflect(k + j, nz))) * a.w[j];
    } else if (a.zfilt == SPARC_ZFILT_SMOOTH) {
        if (k == 0) v = at(0);
        else if (k >= 5 && k <= nz - 6)
            v = a.c[0] * at(k) + a.c[1] * (at(k - 1) + at(k + 1)) + a.c[2] * (at(k - 2) + at(k + 2)) +
                a.c[3] * (at(k - 3) + at(k + 3)) + a.c[4] * (at(k - 4) + at(k + 4)) + a.c[5] * (at(k - 5) + at(k + 5));
        else if ((k >= 1 && k <= 3) || (k >= nz - 5 && k <= nz - 2)) v = 0.5 * (at(k - 1) + at(k + 1));
        else v = 0.0;  // rows 4 and nz-1
    } else {
        v = at(k);
    }
    a.out[i] = v;
}

// Per-block partials: mode 0 sum a (b - c) (c may be null: sum a b); mode 1 max a (NaN-propagating).
__global__ void __launch_bounds__(GRAD_THREADS) vec_reduce_kernel(int mode, const double *__restrict__ a,
                                                                  const double *__restrict__ b,
                                                                  const double *__restrict__ c, long long n,
                                                                  double *part)
{
    double v = mode == 1 ? -INFINITY : 0.0;
    for (long long i = (long long)blockIdx.x * GRAD_THREADS + threadIdx.x; i < n; i += (long long)GRAD_BLOCKS * GRAD_THREADS) {
        if (mode == 1) v = nanmax(v, a[i]);
        else v += a[i] * (c ? (b[i] - c[i]) : b[i]);
    }
    v = mode == 1 ? block_reduce<true>(v) : block_reduce<false>(v);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
}

// One block: out = the partials reduced in a fixed order.
__global__ void __launch_bounds__(GRAD_THREADS) vec_final_kernel(int mode, const double *part, double *out)
{
    double v = mode == 1 ? -INFINITY : 0.0;
    for (int i = threadIdx.x; i < GRAD_BLOCKS; i += GRAD_THREADS) v = mode == 1 ? nanmax(v, part[i]) : v + part[i];
    v = mode == 1 ? block_reduce<true>(v) : block_reduce<false>(v);
    if (threadIdx.x == 0) *out = v;
}

// Coefficient mult * (num / den) - (snum / sden), each device pointer optional (absent num or
// den: 1; absent snum: no subtraction).
struct Coef {
    double mult = 1.0;
    const double *num = nullptr, *den = nullptr, *snum = nullptr, *sden = nullptr;
};
__device__ __forceinline__ double coef_value(const Coef &c)
{
    double v = c.mult;
    if (c.num) v = v * *c.num;
    if (c.den) v = v / *c.den;
    if (c.snum) v = v - *c.snum / *c.sden;
    return v;
}

__global__ void __launch_bounds__(GRAD_THREADS) vec_axpby_kernel(long long n, Coef ca, const double *x, Coef cb,
                                                                 const double *z, double *y)
{
    const double a = coef_value(ca), b = z ? coef_value(cb) : 0.0;
    for (long long i = (long long)blockIdx.x * GRAD_THREADS + threadIdx.x; i < n; i += (long long)GRAD_BLOCKS * GRAD_THREADS)
        y[i] = z ? a * x[i] + b * z[i] : a * x[i];
}

struct LsArgs {
    const double *model, *update, *sumsq, *umax;
    double *out;
    long long n;
    int neps;
    double eps[GRAD_MAX_EPS];
};

// grad.py:351-364: update / max(update) (unless 0), rms(model) (1 if 0), model + eps u scale.
__global__ void __launch_bounds__(GRAD_THREADS) ls_models_kernel(LsArgs a)
{
    const double umax = *a.umax;
    double scale = sqrt(*a.sumsq / (double)a.n);
    if (scale == 0.0) scale = 1.0;
    for (long long i = (long long)blockIdx.x * GRAD_THREADS + threadIdx.x; i < a.n; i += (long long)GRAD_BLOCKS * GRAD_THREADS) {
        double u = a.update[i];
        if (umax != 0.0) u = u / umax;
        const double m = a.model[i];
        for (int e = 0; e < a.neps; e++) a.out[(size_t)e * a.n + i] = m + a.eps[e] * u * scale;
    }
}

// ---------------------------------------------------------------------------------------------
cudaError_t reduce_to(int mode, const double *a, const double *b, const double *c, long long n, double *part,
                      double *out, cudaStream_t st)
{
    vec_reduce_kernel<<<GRAD_BLOCKS, GRAD_THREADS, 0, st>>>(mode, a, b, c, n, part);
    vec_final_kernel<<<1, GRAD_THREADS, 0, st>>>(mode, part, out);
    return cudaGetLastError();
}

cudaError_t axpby(long long n, Coef ca, const double *x, Coef cb, const double *z, double *y, cudaStream_t st)
{
    vec_axpby_kernel<<<GRAD_BLOCKS, GRAD_THREADS, 0, st>>>(n, ca, x, cb, z, y);
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_grad_row(const GradRowArgs &a, cudaStream_t st)
{
    const int pairs = (a.nz + 1) / 2;
    const int grid = (pairs + GRAD_WPB - 1) / GRAD_WPB;
    const size_t smem = (size_t)GRAD_WPB * 4 * N * sizeof(double);
    auto k = grad_row_kernel<N>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, GRAD_WPB * WARP, smem, st>>>(a);
    return cudaGetLastError();
}

#define GRAD_FFT_SIZES(X) X(64) X(128) X(192) X(256) X(384) X(512) X(768) X(1024)

bool grad_fft_supported(int n)
{
#define CASE(n_) if (n == n_) return true;
    GRAD_FFT_SIZES(CASE)
#undef CASE
    return false;
}

cudaError_t grad_row(const GradRowArgs &a, int nx, cudaStream_t st)
{
#define CASE(n_) if (nx == n_) return launch_grad_row<n_>(a, st);
    GRAD_FFT_SIZES(CASE)
#undef CASE
    return cudaErrorInvalidValue;
}

int cuda_fail(const char *what, cudaError_t e)
{
    return report_error(SPARC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

extern "C" {

unsigned long long sparc_grad_workspace_bytes(int nx, int nz)
{
    return (unsigned long long)(grad_work_doubles(nx, nz) * sizeof(double));
}

int sparc_gradient(const sparc_grad_config_t *cfg, const double *kernels, const double *hessians, const double *rho,
                   double *grad, void *work, void *stream)
{
    if (!cfg || !kernels || !hessians || (cfg->precondition && !rho) || !grad || !work)
        return report_error(SPARC_ERR_ARG, "sparc_gradient: null argument");
    const int nx = cfg->nx, nz = cfg->nz;
    if (nz < 1 || cfg->nsrc < 1) return report_error(SPARC_ERR_ARG, "sparc_gradient: nz and nsrc must be >= 1");
    if (!grad_fft_supported(nx))
        return report_error(SPARC_ERR_SIZE, "sparc_gradient: nx = " + std::to_string(nx) + " not in the FFT table");
    if (!(cfg->nk > 0.0)) return report_error(SPARC_ERR_ARG, "sparc_gradient: nk must be > 0");
    if (cfg->sym < -1 || cfg->sym > 1) return report_error(SPARC_ERR_ARG, "sparc_gradient: sym must be -1, 0 or 1");
    GradColArgs ca{};
    ca.zfilt = cfg->zfilt;
    if (cfg->zfilt == SPARC_ZFILT_GAUSSIAN) {
        if (!(cfg->zsigma > 0.0)) return report_error(SPARC_ERR_ARG, "sparc_gradient: zsigma must be > 0");
        const int r = (int)(4.0 * cfg->zsigma + 0.5);  // scipy: int(truncate * sd + 0.5), truncate 4
        if (r > GRAD_MAX_RADIUS)
            return report_error(SPARC_ERR_SIZE, "sparc_gradient: Gaussian radius " + std::to_string(r) + " > 32");
        std::vector<double> w(2 * r + 1);
        double sum = 0.0;
        for (int j = -r; j <= r; j++) {
            w[j + r] = std::exp(-0.5 / (cfg->zsigma * cfg->zsigma) * (double)(j * j));
            sum += w[j + r];
        }
        for (int j = 0; j <= r; j++) ca.w[j] = w[j + r] / sum;
        ca.radius = r;
    } else if (cfg->zfilt == SPARC_ZFILT_SMOOTH) {
        if (nz < 11) return report_error(SPARC_ERR_SIZE, "sparc_gradient: the 'smooth' z filter needs nz >= 11");
        // grad.py:70-75, exact binary fractions
        const double c[6] = {0.75390625, 0.41015625, -0.234375, 0.087890625, -0.01953125, 0.001953125};
        ca.c[0] = c[0];
        for (int j = 1; j < 6; j++) ca.c[j] = 0.5 * c[j];
    } else if (cfg->zfilt != SPARC_ZFILT_NONE) {
        return report_error(SPARC_ERR_ARG, "sparc_gradient: unknown z filter");
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const GradWork w = carve(work, nx, nz);
    const long long n = (long long)nx * nz;
    grad_tables_kernel<<<(nx + 127) / 128, 128, 0, st>>>(nx, cfg->nk, w.twr, w.twi, w.gk);
    grad_sum_kernel<<<GRAD_BLOCKS, GRAD_THREADS, 0, st>>>(kernels, hessians, rho, cfg->nsrc, nx, n, cfg->precondition,
                                                          w.K, w.H, w.part);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail("sparc_gradient: sum", e);
    GradRowArgs ra{w.K, w.H, w.part, w.twr, w.twi, w.gk, w.T, nz, cfg->sym, cfg->precondition, cfg->hess_floor};
    e = grad_row(ra, nx, st);
    if (e != cudaSuccess) return cuda_fail("sparc_gradient: x pass", e);
    ca.T = w.T;
    ca.out = grad;
    ca.nx = nx;
    ca.nz = nz;
    grad_col_kernel<<<(unsigned)((n + GRAD_THREADS - 1) / GRAD_THREADS), GRAD_THREADS, 0, st>>>(ca);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail("sparc_gradient: z pass", e);
    return SPARC_OK;
}

int sparc_vec_dot(long long n, const double *a, const double *b, const double *c, double *result, void *work,
                  void *stream)
{
    if (n < 0 || !a || !b || !result || !work) return report_error(SPARC_ERR_ARG, "sparc_vec_dot: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const GradWork w = carve(work, 0, 0);
    cudaError_t e = reduce_to(0, a, b, c, n, w.part, w.sc, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(result, w.sc, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? SPARC_OK : cuda_fail("sparc_vec_dot", e);
}

int sparc_vec_axpby(long long n, double alpha, const double *x, double beta, const double *z, double *y,
                    void *stream)
{
    if (n < 0 || !x || !y) return report_error(SPARC_ERR_ARG, "sparc_vec_axpby: bad argument");
    Coef ca, cb;
    ca.mult = alpha;
    cb.mult = beta;
    cudaError_t e = axpby(n, ca, x, cb, z, y, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? SPARC_OK : cuda_fail("sparc_vec_axpby", e);
}

int sparc_update_direction(int algo, long long n, const double *g, const double *g_prev, const double *p_prev,
                           double *p, double *beta, void *work, void *stream)
{
    if (n < 0 || !g || !p || (algo != 0 && (!g_prev || !p_prev || !work)) || algo < 0 || algo > 2)
        return report_error(SPARC_ERR_ARG, "sparc_update_direction: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Coef m1;
    m1.mult = -1.0;
    if (algo == 0) {
        cudaError_t e = axpby(n, m1, g, Coef{}, nullptr, p, st);
        if (e != cudaSuccess) return cuda_fail("sparc_update_direction", e);
        if (beta) *beta = 0.0;
        return SPARC_OK;
    }
    const GradWork w = carve(work, 0, 0);
    double *num = w.sc, *den = w.sc + 1;
    // beta = g.(g - g_prev) / (g_prev.g_prev  or  (g - g_prev).p_prev)
    cudaError_t e = reduce_to(0, g, g, g_prev, n, w.part, num, st);
    if (e == cudaSuccess) {
        if (algo == 1) e = reduce_to(0, g_prev, g_prev, nullptr, n, w.part, den, st);
        else {
            // (g - g_prev).p_prev = p_prev.(g - g_prev)
            e = reduce_to(0, p_prev, g, g_prev, n, w.part, den, st);
        }
    }
    Coef cb;
    cb.num = num;
    cb.den = den;
    if (e == cudaSuccess) e = axpby(n, m1, g, cb, p_prev, p, st);
    if (e == cudaSuccess && beta) {
        double h[2];
        e = cudaMemcpyAsync(h, w.sc, 2 * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) *beta = h[0] / h[1];
    }
    return e == cudaSuccess ? SPARC_OK : cuda_fail("sparc_update_direction", e);
}

int sparc_lbfgs_direction(long long n, int npairs, const double *const *s, const double *const *y, const double *g,
                          double *p, void *work, void *stream)
{
    if (n < 0 || npairs < 0 || npairs > GRAD_MAX_PAIRS || !g || !p || !work || (npairs > 0 && (!s || !y)))
        return report_error(SPARC_ERR_ARG, "sparc_lbfgs_direction: bad argument");
    for (int i = 0; i < npairs; i++)
        if (!s[i] || !y[i] || s[i] == p || y[i] == p)
            return report_error(SPARC_ERR_ARG, "sparc_lbfgs_direction: null or aliased pair");
    if (g == p) return report_error(SPARC_ERR_ARG, "sparc_lbfgs_direction: p aliases g");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const GradWork w = carve(work, 0, 0);
    // scalars: ys[i] = y_i.s_i, sq[i] = s_i.q (first loop), yr[i] = y_i.r (second loop), yy
    double *ys = w.sc + 8, *sq = ys + GRAD_MAX_PAIRS, *yr = sq + GRAD_MAX_PAIRS, *yy = w.sc;
    cudaError_t e = axpby(n, Coef{}, g, Coef{}, nullptr, p, st);  // q = g, held in p
    for (int i = npairs - 1; i >= 0 && e == cudaSuccess; i--) {
        e = reduce_to(0, y[i], s[i], nullptr, n, w.part, ys + i, st);
        if (e == cudaSuccess) e = reduce_to(0, s[i], p, nullptr, n, w.part, sq + i, st);
        Coef ca, cb;
        cb.mult = -1.0;
        cb.num = sq + i;
        cb.den = ys + i;  // q <- q - alpha_i y_i, alpha_i = s_i.q / y_i.s_i
        if (e == cudaSuccess) e = axpby(n, ca, p, cb, y[i], p, st);
    }
    if (npairs > 0 && e == cudaSuccess) {
        const int l = npairs - 1;  // r = gamma q, gamma = s.y / y.y of the newest pair
        e = reduce_to(0, y[l], y[l], nullptr, n, w.part, yy, st);
        Coef ca;
        ca.num = ys + l;
        ca.den = yy;
        if (e == cudaSuccess) e = axpby(n, ca, p, Coef{}, nullptr, p, st);
    }
    for (int i = 0; i < npairs && e == cudaSuccess; i++) {
        e = reduce_to(0, y[i], p, nullptr, n, w.part, yr + i, st);
        Coef ca, cb;
        cb.num = sq + i;
        cb.den = ys + i;
        cb.snum = yr + i;
        cb.sden = ys + i;  // r <- r + s_i (alpha_i - y_i.r / y_i.s_i)
        if (e == cudaSuccess) e = axpby(n, ca, p, cb, s[i], p, st);
    }
    Coef m1;
    m1.mult = -1.0;
    if (e == cudaSuccess) e = axpby(n, m1, p, Coef{}, nullptr, p, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? SPARC_OK : cuda_fail("sparc_lbfgs_direction", e);
}

int sparc_linesearch_models(long long n, const double *model, const double *update, int neps, const double *eps,
                            double *out, void *work, void *stream)
{
    if (n < 1 || !model || !update || !out || !work || neps < 0 || neps > GRAD_MAX_EPS || (neps > 0 && !eps))
        return report_error(SPARC_ERR_ARG, "sparc_linesearch_models: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const GradWork w = carve(work, 0, 0);
    LsArgs a{};
    a.model = model;
    a.update = update;
    a.sumsq = w.sc;
    a.umax = w.sc + 1;
    a.out = out;
    a.n = n;
    a.neps = neps;
    for (int i = 0; i < neps; i++) a.eps[i] = eps[i];
    cudaError_t e = reduce_to(0, model, model, nullptr, n, w.part, w.sc, st);
    if (e == cudaSuccess) e = reduce_to(1, update, nullptr, nullptr, n, w.part, w.sc + 1, st);
    if (e == cudaSuccess) {
        ls_models_kernel<<<GRAD_BLOCKS, GRAD_THREADS, 0, st>>>(a);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? SPARC_OK : cuda_fail("sparc_linesearch_models", e);
}

}  // extern "C"
