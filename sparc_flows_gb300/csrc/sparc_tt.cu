// sparc_tt.cu -- travel-time adjoint source on the device (ADJOINT_SOURCE_FILT,
// driver.f90:1758-2238), FP64, for a batch of sources.
//
// The reference, per ridge filter ("mode") and per measured receiver i, windows the time
// derivative of the filtered synthetic at x_i, transforms it, multiplies by the filter and by
// exp(-i k x_i), transforms the whole (x, t) plane back and adds the result, scaled by
// -tau_i / (sum ccdot^2 dt), time-reversed into the adjoint source: one 2-D transform per
// receiver.  The sum over receivers is linear, and exp(-2 pi i k (i-1)/nx) is the forward DFT
// kernel of a point at x_i, so it equals one transform per mode:
//     adj_mode = Re IDFT2( filter * DFT2(c) ),  c(x_i, t) = con_i w_i(t) ccdot(x_i, t),
// with c zero at unmeasured x.  Per mode and batch: three inverse 2-D transforms (filtered
// synthetic, filtered data, time derivative), the Gizon-Birch derivative of the synthetic along
// t, per-receiver reductions (window pick, travel time, normalisation), and one forward plus
// one inverse 2-D transform of c.
//
// Fields are complex [nb][nt][nx] (x fastest).  x transforms: one warp per row, the shared-
// memory Stockham FFT of the wave solver (nx in its table).  t transforms: any nt (the record
// count, 240 or 241 for 3600 steps -- 241 is prime): Bluestein's chirp-z transform on two
// power-of-two FFTs of length M >= 2 nt - 1 (nt <= 512), a direct DFT over 16-column tiles above
// that.  FFTW's transforms are unnormalised, and so are these.
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

constexpr int TT_THREADS = 256;
constexpr int TT_COLS = 16;      // columns per block of the t transform
constexpr int TT_XWPB = 2;       // rows (warps) per block of the x transform
constexpr double TT_PI = 3.141592653589793;

// x transform of complex rows in place, sign -1 forward, +1 inverse (unnormalised).
template <int N>
__global__ void __launch_bounds__(TT_XWPB *WARP) tt_fft_x_kernel(double2 *data, long long nrows, const double *twr,
                                                                 const double *twi, int inverse)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *sm = reinterpret_cast<double *>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long row = (long long)blockIdx.x * TT_XWPB + warp;
    if (row >= nrows) return;
    double *xr = sm + (size_t)warp * 4 * N, *xi = xr + N, *yr = xi + N, *yi = yr + N;
    double2 *d = data + row * N;
    for (int x = lane; x < N; x += WARP) {
        const double2 v = d[x];
        xr[x] = v.x;
        xi[x] = v.y;
    }
    __syncwarp();
    double *orr, *oi;
    FFTRun<double, N, 0, 1>::run(xr, xi, yr, yi, twr, twi, lane, inverse != 0, 1.0, 1.0, orr, oi);
    __syncwarp();
    for (int x = lane; x < N; x += WARP) d[x] = make_double2(orr[x], oi[x]);
}

// t transform of complex columns in place: column (b, x) of length nt, stride nx.
// wt[m] = exp(-2 pi i m / nt); inverse uses the conjugate.
__global__ void __launch_bounds__(TT_THREADS) tt_dft_t_kernel(double2 *data, int nt, int nx, const double2 *wt,
                                                              int inverse)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2 *tile = reinterpret_cast<double2 *>(smem_raw);  // [nt][TT_COLS]
    double2 *w = tile + (size_t)nt * TT_COLS;                // [nt]
    const int x0 = blockIdx.x * TT_COLS;
    double2 *base = data + (size_t)blockIdx.y * nt * nx + x0;
    for (int idx = threadIdx.x; idx < nt * TT_COLS; idx += TT_THREADS) {
        const int t = idx / TT_COLS, c = idx % TT_COLS;
        tile[idx] = (x0 + c < nx) ? base[(size_t)t * nx + c] : make_double2(0.0, 0.0);
    }
    for (int m = threadIdx.x; m < nt; m += TT_THREADS) {
        double2 v = wt[m];
        if (inverse) v.y = -v.y;
        w[m] = v;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < nt * TT_COLS; idx += TT_THREADS) {
        const int k = idx / TT_COLS, c = idx % TT_COLS;
        double sr = 0.0, si = 0.0;
        int m = 0;
        for (int t = 0; t < nt; t++) {
            const double2 a = tile[t * TT_COLS + c], b = w[m];
            sr += a.x * b.x - a.y * b.y;
            si += a.x * b.y + a.y * b.x;
            m += k;
            if (m >= nt) m -= nt;
        }
        if (x0 + c < nx) base[(size_t)k * nx + c] = make_double2(sr, si);
    }
}

// t transform by Bluestein's chirp-z algorithm: nk = (n^2 + k^2 - (k-n)^2) / 2 turns the length-nt
// DFT into a convolution with the chirp b_m = exp(+i pi m^2 / nt), evaluated with two power-of-two
// FFTs of length M >= 2 nt - 1 (Bluestein, IEEE Trans. Audio Electroacoust. 18 (1970) 451-455):
//   X_k = w_k IFFT_M( FFT_M(x_n w_n) * FFT_M(b) )_k / M,   w_n = exp(-i pi n^2 / nt).
// The inverse transform is the conjugate of the forward one of the conjugate.  A block of WPB warps
// takes WPB consecutive columns (b, x0 .. x0 + WPB - 1): the tile [nt][WPB] is loaded and stored
// row-contiguously (WPB x 16 bytes per record) through shared memory, each warp transforms one
// column with the Stockham FFT of the x transforms.
template <int M, int WPB>
__global__ void __launch_bounds__(WPB *WARP) tt_bluestein_t_kernel(double2 *data, int nt, int nx, const double2 *chirp,
                                                                   const double2 *bhat, const double *twr,
                                                                   const double *twi, int inverse)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *sm = reinterpret_cast<double *>(smem_raw);
    constexpr int SW = 4 * M + 2;  // per-warp stride: the tile rows of 8 warps land on distinct banks
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int x0 = blockIdx.x * WPB;
    double2 *base = data + (size_t)blockIdx.y * nt * nx + x0;
    const double cs = inverse ? -1.0 : 1.0;  // conjugation of the input and output for the inverse
    for (int idx = threadIdx.x; idx < nt * WPB; idx += WPB * WARP) {
        const int t = idx / WPB, c = idx % WPB;
        double *xr = sm + (size_t)c * SW, *xi = xr + M;
        double2 v = (x0 + c < nx) ? base[(size_t)t * nx + c] : make_double2(0.0, 0.0);
        v.y *= cs;
        const double2 w = chirp[t];
        xr[t] = v.x * w.x - v.y * w.y;
        xi[t] = v.x * w.y + v.y * w.x;
    }
    double *xr = sm + (size_t)warp * SW, *xi = xr + M, *yr = xi + M, *yi = yr + M;
    for (int t = nt + lane; t < M; t += WARP) {
        xr[t] = 0.0;
        xi[t] = 0.0;
    }
    __syncthreads();
    double *fr, *fi;
    FFTRun<double, M, 0, 1>::run(xr, xi, yr, yi, twr, twi, lane, false, 1.0, 1.0, fr, fi);
    for (int k = lane; k < M; k += WARP) {
        const double2 b = bhat[k];
        const double ar = fr[k], ai = fi[k];
        fr[k] = ar * b.x - ai * b.y;
        fi[k] = ar * b.y + ai * b.x;
    }
    __syncwarp();
    double *gr = (fr == xr) ? yr : xr, *gi = (fr == xr) ? yi : xi;
    double *cr, *ci;
    FFTRun<double, M, 0, 1>::run(fr, fi, gr, gi, twr, twi, lane, true, 1.0, 1.0, cr, ci);
    __syncwarp();
    const double inv_m = 1.0 / (double)M;
    for (int k = lane; k < nt; k += WARP) {  // X_k = w_k c_k / M, back into the warp's own buffer
        const double2 w = chirp[k];
        const double ar = cr[k] * inv_m, ai = ci[k] * inv_m;
        const double rr = ar * w.x - ai * w.y, ri = ar * w.y + ai * w.x;
        cr[k] = rr;
        ci[k] = ri * cs;
    }
    if (lane == 0) reinterpret_cast<int *>(sm + (size_t)WPB * SW)[warp] = (int)(cr - (sm + (size_t)warp * SW));
    __syncthreads();
    for (int idx = threadIdx.x; idx < nt * WPB; idx += WPB * WARP) {
        const int t = idx / WPB, c = idx % WPB;
        if (x0 + c >= nx) continue;
        const double *wb = sm + (size_t)c * SW;
        const int off = reinterpret_cast<const int *>(sm + (size_t)WPB * SW)[c];
        base[(size_t)t * nx + c] = make_double2(wb[off + t], wb[off + M + t]);
    }
}

// out = in * filter[t][x] (real), optionally times i 2 pi freqnu(t) (the time derivative of
// driver.f90:2015-2017, freqnu = distmat(nt) / (nt dt 60)).
__global__ void __launch_bounds__(TT_THREADS) tt_filter_kernel(const double2 *in, double2 *out, const double *filter,
                                                               int nt, int nx, long long n, int deriv, double dt_min)
{
    const long long stride = (long long)gridDim.x * TT_THREADS;
    for (long long i = (long long)blockIdx.x * TT_THREADS + threadIdx.x; i < n; i += stride) {
        const long long tx = i % ((long long)nt * nx);
        const int t = (int)(tx / nx);
        const double f = filter[tx];
        double2 v = in[i];
        v.x *= f;
        v.y *= f;
        if (deriv) {
            const int d = (t > nt - t) ? -(nt - t) : t;  // distmat: index 0 at 0, upper half negative
            const double om = 2.0 * TT_PI * ((double)d / ((double)nt * dt_min * 60.0));
            v = make_double2(-om * v.y, om * v.x);  // times i om
        }
        out[i] = v;
    }
}

// Real records into complex planes.
__global__ void __launch_bounds__(TT_THREADS) tt_load_kernel(const double *in, double2 *out, long long n)
{
    const long long stride = (long long)gridDim.x * TT_THREADS;
    for (long long i = (long long)blockIdx.x * TT_THREADS + threadIdx.x; i < n; i += stride)
        out[i] = make_double2(in[i], 0.0);
}

// Real part into a complex buffer (imaginary part zero), optional scale.
__global__ void __launch_bounds__(TT_THREADS) tt_real_kernel(const double2 *in, double2 *out, long long n, double s)
{
    const long long stride = (long long)gridDim.x * TT_THREADS;
    for (long long i = (long long)blockIdx.x * TT_THREADS + threadIdx.x; i < n; i += stride)
        out[i] = make_double2(in[i].x * s, 0.0);
}

// Multiplier of COMPUTE_TT_GIZONBIRCH's derivative (driver.f90:913-917) on the full spectrum:
// i 2 pi q / (nt dt) below nt/2, zero at q = nt/2 (and its mirror), the conjugate mirror above.
__global__ void __launch_bounds__(TT_THREADS) tt_gb_kernel(double2 *data, int nt, int nx, long long n, double dt_min)
{
    const int h = nt / 2;
    const long long stride = (long long)gridDim.x * TT_THREADS;
    for (long long i = (long long)blockIdx.x * TT_THREADS + threadIdx.x; i < n; i += stride) {
        const int q = (int)((i / nx) % nt);
        int s = 0;
        if (q < h) s = q;
        else if (q > nt - h) s = -(nt - q);
        const double om = 2.0 * TT_PI * (double)s / ((double)nt * dt_min);
        const double2 v = data[i];
        data[i] = make_double2(-om * v.y, om * v.x);
    }
}

// One measured receiver: b, x (0-based), search range [timest, timefin] (1-based, clipped),
// given window (lef, rig) or picked one; results: lef, rig, loc, tau, con.
struct TTRow {
    int b, x, timest, timefin, lef, rig, loc, pad;
    double tau, con;
};

// One warp per measured receiver (driver.f90:2040-2100): window pick (first maximum of
// |Re acc| over the search range), travel time by Simpson sums (SIMPSON_REGULAR weights over
// the whole record, integrals.f90:107-130) of w u0dot (u0 - u) and w u0dot^2, and the
// normalisation con = Re(-tau / (sum_{lef..rig} ccdot^2 dt)).  u0dot holds nt times the
// derivative (the c2r transform is unnormalised).
__global__ void __launch_bounds__(TT_THREADS) tt_rows_kernel(TTRow *rows, int nrows, const double2 *acc,
                                                             const double2 *dat, const double2 *u0dot,
                                                             const double2 *ccdot, int nt, int nx, int halftime,
                                                             int given, double dt_min)
{
    const int warp = (blockIdx.x * TT_THREADS + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= nrows) return;
    TTRow r = rows[warp];
    const size_t base = (size_t)r.b * nt * nx + r.x;
    auto at = [&](const double2 *f, int t) { return f[base + (size_t)t * nx]; };
    if (!given) {
        const int a = max(r.timest, 1), e = min(r.timefin, nt);
        double best = -1.0;
        int bi = a;
        for (int t = a + lane; t <= e; t += WARP) {
            const double v = fabs(at(acc, t - 1).x);
            if (v > best) { best = v; bi = t; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        r.loc = bi;
        r.lef = max(bi - halftime, 1);
        r.rig = min(bi + halftime, nt);
    }
    double num = 0.0, den = 0.0, sr = 0.0, si = 0.0;
    const double inv_nt = 1.0 / (double)nt;
    for (int t = r.lef + lane; t <= r.rig; t += WARP) {  // 1-based t
        const double wgt = (t == 1 || t == nt) ? 1.0 : ((t % 2 == 0) ? 4.0 : 2.0);
        const double ud = at(u0dot, t - 1).x * inv_nt;
        const double u0 = at(acc, t - 1).x, u = at(dat, t - 1).x;
        num += wgt * (ud * (u0 - u));
        den += wgt * (ud * ud);
        const double2 c = at(ccdot, t - 1);
        sr += c.x * c.x - c.y * c.y;
        si += 2.0 * c.x * c.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        num += __shfl_xor_sync(0xffffffffu, num, o);
        den += __shfl_xor_sync(0xffffffffu, den, o);
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
        si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if (lane == 0) {
        const double tau = num / den;  // both Simpson sums carry the same dt / 3
        const double dr = sr * dt_min, di = si * dt_min;
        r.tau = tau;
        r.con = -tau * dr / (dr * dr + di * di);  // Re(-tau / (dr + i di))
        rows[warp] = r;
    }
}

// MISFIT_ALL (driver.f90:2294-2651), one warp per measured receiver: window pick (first maximum
// of |Re acc| over the search range, window loc -+ halftime, not clipped), then COMPUTE_TT
// (driver.f90:855-890) on the window: the cross-correlation cc(i) = dt sum u0(k) u(k + i) for
// lags i in (-n, n), its first maximum, and the vertex of the parabola through the three samples
// around it.  tau = NaN marks a receiver that is not measured: a window leaving the record or a
// peak at the end of the lag range (the reference reads past its arrays there).
__global__ void __launch_bounds__(TT_THREADS) tt_cc_kernel(TTRow *rows, int nrows, const double2 *acc,
                                                           const double2 *dat, int nt, int nx, int halftime,
                                                           int given, double dt_min)
{
    const int warp = (blockIdx.x * TT_THREADS + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= nrows) return;
    TTRow r = rows[warp];
    const size_t base = (size_t)r.b * nt * nx + r.x;
    auto re = [&](const double2 *f, int t0) { return f[base + (size_t)t0 * nx].x; };  // 0-based record index
    if (!given) {
        const int a = max(r.timest, 1), e = min(r.timefin, nt);  // 1-based, clipped
        double best = -1.0;
        int bi = a;
        for (int t = a + lane; t <= e; t += WARP) {
            const double v = fabs(re(acc, t - 1));
            if (v > best) { best = v; bi = t; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        r.loc = bi;
        r.lef = bi - halftime;
        r.rig = bi + halftime;
    }
    double tau = nan("");
    if (r.lef >= 1 && r.rig <= nt && r.rig >= r.lef) {
        const int n = r.rig - r.lef + 1, w0 = r.lef - 1;  // window sample k (1..n) is record w0 + k - 1
        // cc at lag i = j - (n - 1): dt sum_k u0(k - min(i, 0)) u(k + max(i, 0)) over the overlap
        auto cc = [&](int j) {
            const int i = j - (n - 1);
            double c = 0.0;
            if (i <= 0) {
                for (int k = 1; k <= n + i; k++) c += re(acc, w0 + k - i - 1) * re(dat, w0 + k - 1);
            } else {
                for (int k = 1; k <= n - i; k++) c += re(acc, w0 + k - 1) * re(dat, w0 + k + i - 1);
            }
            return c * dt_min;
        };
        double best = -INFINITY;
        int bl = 2 * n;
        for (int j = lane; j <= 2 * n - 2; j += WARP) {
            const double c = cc(j);
            if (c > best) { best = c; bl = j; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bl, o);
            if (ob > best || (ob == best && oi < bl)) { best = ob; bl = oi; }
        }
        if (bl > 0 && bl < 2 * n - 2) {
            const double cm = cc(bl - 1), c0 = cc(bl), cp = cc(bl + 1);
            const double t0 = (double)(bl - (n - 1)) * dt_min;
            // parabola c = p0 + p1 t + p2 t^2 through (t0 - dt, t0, t0 + dt); tau = -p1 / (2 p2)
            const double p2 = (cm - 2.0 * c0 + cp) / (2.0 * dt_min * dt_min);
            const double p1 = (cp - cm) / (2.0 * dt_min) - 2.0 * p2 * t0;
            tau = -p1 * 0.5 / p2;
        }
    }
    if (lane == 0) {
        r.tau = tau;
        rows[warp] = r;
    }
}

// c(x_i, t) = con_i w_i(t) ccdot(x_i, t) at the measured receivers (the buffer is zeroed first).
__global__ void __launch_bounds__(TT_THREADS) tt_scatter_kernel(const TTRow *rows, int nrows, const double2 *ccdot,
                                                                double2 *c, int nt, int nx)
{
    const int warp = (blockIdx.x * TT_THREADS + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= nrows) return;
    const TTRow r = rows[warp];
    const size_t base = (size_t)r.b * nt * nx + r.x;
    for (int t = r.lef + lane; t <= r.rig; t += WARP) {
        const double2 v = ccdot[base + (size_t)(t - 1) * nx];
        double2 &o = c[base + (size_t)(t - 1) * nx];
        o.x += r.con * v.x;
        o.y += r.con * v.y;
    }
}

// adj[b][nt-1-t][x] += Re(field[b][t][x]) (time reversal, driver.f90:2097-2099).
__global__ void __launch_bounds__(TT_THREADS) tt_accum_kernel(const double2 *f, double *adj, int nt, int nx,
                                                              long long n)
{
    const long long stride = (long long)gridDim.x * TT_THREADS;
    for (long long i = (long long)blockIdx.x * TT_THREADS + threadIdx.x; i < n; i += stride) {
        const long long plane = (long long)nt * nx;
        const long long b = i / plane, r = i - b * plane;
        const int t = (int)(r / nx), x = (int)(r - (long long)t * nx);
        adj[b * plane + (long long)(nt - 1 - t) * nx + x] += f[i].x;
    }
}

__global__ void __launch_bounds__(TT_THREADS) tt_scale_out_kernel(const double *adj, double *out, long long n, double s)
{
    const long long stride = (long long)gridDim.x * TT_THREADS;
    for (long long i = (long long)blockIdx.x * TT_THREADS + threadIdx.x; i < n; i += stride) out[i] = adj[i] * s;
}

unsigned tt_grid(long long n)
{
    const long long g = (n + TT_THREADS - 1) / TT_THREADS;
    return (unsigned)(g < 152LL * 8 ? g : 152LL * 8);
}

}  // namespace

struct sparc_tt_plan {
    int nx = 0, nt = 0, nb = 0;
    std::vector<void *> allocs;
    double2 *S = nullptr, *D = nullptr, *ACC = nullptr, *DAT = nullptr, *CCD = nullptr, *U0D = nullptr, *C = nullptr;
    double *adj = nullptr, *twr = nullptr, *twi = nullptr;
    double2 *wt = nullptr;
    TTRow *rows = nullptr;
    int cap = 0;
    int bm = 0;  // Bluestein length (0: direct DFT along t)
    double2 *chirp = nullptr, *bhat = nullptr;
    double *btwr = nullptr, *btwi = nullptr;
};

namespace {

template <int N>
cudaError_t fft_x_n(sparc_tt_plan *p, double2 *f, int inverse, cudaStream_t st)
{
    const long long nrows = (long long)p->nb * p->nt;
    const size_t smem = (size_t)TT_XWPB * 4 * N * sizeof(double);
    auto k = tt_fft_x_kernel<N>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<(unsigned)((nrows + TT_XWPB - 1) / TT_XWPB), TT_XWPB * WARP, smem, st>>>(f, nrows, p->twr, p->twi, inverse);
    return cudaGetLastError();
}

cudaError_t fft_x(sparc_tt_plan *p, double2 *f, int inverse, cudaStream_t st)
{
#define CASE(n_) if (p->nx == n_) return fft_x_n<n_>(p, f, inverse, st);
    CASE(64) CASE(128) CASE(192) CASE(256) CASE(384) CASE(512) CASE(768) CASE(1024)
#undef CASE
    return cudaErrorInvalidValue;
}

size_t dft_t_smem(int nt) { return ((size_t)nt * TT_COLS + nt) * sizeof(double2); }

template <int M, int WPB>
cudaError_t bluestein_t(sparc_tt_plan *p, double2 *f, int inverse, cudaStream_t st)
{
    const size_t smem = (size_t)WPB * (4 * M + 2) * sizeof(double) + WPB * sizeof(int) + 16;
    auto k = tt_bluestein_t_kernel<M, WPB>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((p->nx + WPB - 1) / WPB, p->nb);
    k<<<grid, WPB * WARP, smem, st>>>(f, p->nt, p->nx, p->chirp, p->bhat, p->btwr, p->btwi, inverse);
    return cudaGetLastError();
}

cudaError_t dft_t(sparc_tt_plan *p, double2 *f, int inverse, cudaStream_t st)
{
    switch (p->bm) {
        case 64: return bluestein_t<64, 8>(p, f, inverse, st);
        case 128: return bluestein_t<128, 8>(p, f, inverse, st);
        case 256: return bluestein_t<256, 8>(p, f, inverse, st);
        case 512: return bluestein_t<512, 8>(p, f, inverse, st);
        case 1024: return bluestein_t<1024, 4>(p, f, inverse, st);
        default: break;
    }
    const size_t smem = dft_t_smem(p->nt);
    cudaError_t e = cudaFuncSetAttribute(tt_dft_t_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((p->nx + TT_COLS - 1) / TT_COLS, p->nb);
    tt_dft_t_kernel<<<grid, TT_THREADS, smem, st>>>(f, p->nt, p->nx, p->wt, inverse);
    return cudaGetLastError();
}

// 2-D transform over (x, t) of every source's plane.
cudaError_t dft2(sparc_tt_plan *p, double2 *f, int inverse, cudaStream_t st)
{
    cudaError_t e = fft_x(p, f, inverse, st);
    if (e == cudaSuccess) e = dft_t(p, f, inverse, st);
    return e;
}

int tt_fail(const char *what, cudaError_t e)
{
    return report_error(SPARC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

bool tt_nx_ok(int nx)
{
    return nx == 64 || nx == 128 || nx == 192 || nx == 256 || nx == 384 || nx == 512 || nx == 768 || nx == 1024;
}

}  // namespace

extern "C" {

int sparc_tt_plan_create(int nx, int nt, int nbatch, int max_rows, sparc_tt_plan_t **out)
{
    if (!out) return report_error(SPARC_ERR_ARG, "sparc_tt_plan_create: null argument");
    *out = nullptr;
    if (!tt_nx_ok(nx)) return report_error(SPARC_ERR_SIZE, "sparc_tt_plan_create: nx not in the FFT table");
    if (nt < 2 || dft_t_smem(nt) > 220 * 1024)
        return report_error(SPARC_ERR_SIZE, "sparc_tt_plan_create: nt must be in 2..860");
    if (nbatch < 1 || nbatch > 65535 || max_rows < 1) return report_error(SPARC_ERR_ARG, "sparc_tt_plan_create: bad batch");
    sparc_tt_plan *p = new sparc_tt_plan();
    p->nx = nx;
    p->nt = nt;
    p->nb = nbatch;
    p->cap = max_rows;
    const size_t n = (size_t)nbatch * nt * nx;
    struct Req { void **ptr; size_t bytes; };
    std::vector<Req> reqs = {
        {(void **)&p->S, n * sizeof(double2)}, {(void **)&p->D, n * sizeof(double2)},
        {(void **)&p->ACC, n * sizeof(double2)}, {(void **)&p->DAT, n * sizeof(double2)},
        {(void **)&p->CCD, n * sizeof(double2)}, {(void **)&p->U0D, n * sizeof(double2)},
        {(void **)&p->C, n * sizeof(double2)}, {(void **)&p->adj, n * sizeof(double)},
        {(void **)&p->twr, nx * sizeof(double)}, {(void **)&p->twi, nx * sizeof(double)},
        {(void **)&p->wt, nt * sizeof(double2)}, {(void **)&p->rows, (size_t)max_rows * sizeof(TTRow)},
    };
    for (auto &r : reqs) {
        cudaError_t e = cudaMalloc(r.ptr, r.bytes);
        if (e != cudaSuccess) {
            sparc_tt_plan_destroy(p);
            return tt_fail("sparc_tt_plan_create: cudaMalloc", e);
        }
        p->allocs.push_back(*r.ptr);
    }
    std::vector<double> tr(nx), ti(nx);
    for (int t = 0; t < nx; t++) {
        tr[t] = std::cos(2.0 * TT_PI * (double)t / (double)nx);
        ti[t] = -std::sin(2.0 * TT_PI * (double)t / (double)nx);
    }
    std::vector<double2> w(nt);
    for (int m = 0; m < nt; m++) w[m] = make_double2(std::cos(2.0 * TT_PI * (double)m / (double)nt),
                                                     -std::sin(2.0 * TT_PI * (double)m / (double)nt));
    cudaError_t e = cudaMemcpy(p->twr, tr.data(), nx * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(p->twi, ti.data(), nx * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(p->wt, w.data(), nt * sizeof(double2), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(p->adj, 0, n * sizeof(double));
    // Bluestein tables: the smallest power of two M >= 2 nt - 1 in the FFT table (64..1024)
    int M = 64;
    while (M < 2 * nt - 1) M *= 2;
    if (e == cudaSuccess && M <= 1024) {
        p->bm = M;
        std::vector<double2> ch(nt), bext(M, make_double2(0.0, 0.0)), bh(M);
        std::vector<double> btr(M), bti(M);
        for (int m = 0; m < nt; m++) {
            // n^2 mod 2 nt keeps the phase argument small (exp(-i pi n^2 / nt) has period 2 nt in n^2)
            const long long q = ((long long)m * m) % (2LL * nt);
            const double ang = TT_PI * (double)q / (double)nt;
            ch[m] = make_double2(std::cos(ang), -std::sin(ang));
            bext[m] = make_double2(std::cos(ang), std::sin(ang));
            if (m > 0) bext[M - m] = bext[m];
        }
        for (int t = 0; t < M; t++) {
            btr[t] = std::cos(2.0 * TT_PI * (double)t / (double)M);
            bti[t] = -std::sin(2.0 * TT_PI * (double)t / (double)M);
        }
        for (int k = 0; k < M; k++) {  // FFT_M(b) by a direct sum on the host (once per plan)
            double sr = 0.0, si = 0.0;
            for (int m = 0; m < M; m++) {
                const long long q = ((long long)k * m) % M;
                const double c = btr[q], sn = bti[q];
                sr += bext[m].x * c - bext[m].y * sn;
                si += bext[m].x * sn + bext[m].y * c;
            }
            bh[k] = make_double2(sr, si);
        }
        struct Req2 { void **ptr; size_t bytes; };
        Req2 r2[4] = {{(void **)&p->chirp, nt * sizeof(double2)}, {(void **)&p->bhat, M * sizeof(double2)},
                      {(void **)&p->btwr, M * sizeof(double)}, {(void **)&p->btwi, M * sizeof(double)}};
        for (auto &r : r2) {
            if (e == cudaSuccess) e = cudaMalloc(r.ptr, r.bytes);
            if (e == cudaSuccess) p->allocs.push_back(*r.ptr);
        }
        if (e == cudaSuccess) e = cudaMemcpy(p->chirp, ch.data(), nt * sizeof(double2), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(p->bhat, bh.data(), M * sizeof(double2), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(p->btwr, btr.data(), M * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(p->btwi, bti.data(), M * sizeof(double), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        sparc_tt_plan_destroy(p);
        return tt_fail("sparc_tt_plan_create: tables", e);
    }
    *out = p;
    return SPARC_OK;
}

int sparc_tt_plan_destroy(sparc_tt_plan_t *p)
{
    if (!p) return SPARC_OK;
    for (void *q : p->allocs) cudaFree(q);
    delete p;
    return SPARC_OK;
}

int sparc_tt_set_records(sparc_tt_plan_t *p, const double *synth, const double *data, void *stream)
{
    if (!p || !synth || !data) return report_error(SPARC_ERR_ARG, "sparc_tt_set_records: null argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const long long n = (long long)p->nb * p->nt * p->nx;
    // real records into complex planes, then forward 2-D transforms (driver.f90:1840-1844)
    tt_load_kernel<<<tt_grid(n), TT_THREADS, 0, st>>>(synth, p->S, n);
    tt_load_kernel<<<tt_grid(n), TT_THREADS, 0, st>>>(data, p->D, n);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = dft2(p, p->S, 0, st);
    if (e == cudaSuccess) e = dft2(p, p->D, 0, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(p->adj, 0, (size_t)n * sizeof(double), st);
    return e == cudaSuccess ? SPARC_OK : tt_fail("sparc_tt_set_records", e);
}

int sparc_tt_mode(sparc_tt_plan_t *p, const double *filter, int nrows, int *rows, int halftime, int given,
                  double dt_min, double *tau, void *stream)
{
    if (!p || !filter || nrows < 0 || nrows > p->cap || (nrows > 0 && (!rows || !tau)) || halftime < 0)
        return report_error(SPARC_ERR_ARG, "sparc_tt_mode: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nt = p->nt, nx = p->nx;
    const long long n = (long long)p->nb * nt * nx;
    for (int r = 0; r < nrows; r++) {
        const int *q = rows + 7 * r;
        if (q[0] < 0 || q[0] >= p->nb || q[1] < 0 || q[1] >= nx || (given && (q[4] < 1 || q[5] > nt || q[4] > q[5])))
            return report_error(SPARC_ERR_ARG, "sparc_tt_mode: row out of range");
        if (!given && (max(q[2], 1) > min(q[3], nt)))
            return report_error(SPARC_ERR_ARG, "sparc_tt_mode: empty search range");
    }
    std::vector<TTRow> h(nrows);
    for (int r = 0; r < nrows; r++) {
        const int *q = rows + 7 * r;
        h[r] = TTRow{q[0], q[1], q[2], q[3], q[4], q[5], 0, 0, 0.0, 0.0};
    }
    cudaError_t e = cudaSuccess;
    // filtered synthetic and data, the time derivative of the filtered synthetic (driver.f90:1990-2017)
    tt_filter_kernel<<<tt_grid(n), TT_THREADS, 0, st>>>(p->S, p->ACC, filter, nt, nx, n, 0, dt_min);
    tt_filter_kernel<<<tt_grid(n), TT_THREADS, 0, st>>>(p->D, p->DAT, filter, nt, nx, n, 0, dt_min);
    tt_filter_kernel<<<tt_grid(n), TT_THREADS, 0, st>>>(p->S, p->CCD, filter, nt, nx, n, 1, dt_min);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = dft2(p, p->ACC, 1, st);
    if (e == cudaSuccess) e = dft2(p, p->DAT, 1, st);
    if (e == cudaSuccess) e = dft2(p, p->CCD, 1, st);
    // Gizon-Birch derivative of every synthetic column along t (driver.f90:905-923)
    if (e == cudaSuccess) {
        tt_real_kernel<<<tt_grid(n), TT_THREADS, 0, st>>>(p->ACC, p->U0D, n, 1.0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = dft_t(p, p->U0D, 0, st);
    if (e == cudaSuccess) {
        tt_gb_kernel<<<tt_grid(n), TT_THREADS, 0, st>>>(p->U0D, nt, nx, n, dt_min);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = dft_t(p, p->U0D, 1, st);
    if (e == cudaSuccess && nrows > 0) {
        e = cudaMemcpyAsync(p->rows, h.data(), nrows * sizeof(TTRow), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) {
            const unsigned g = (unsigned)(((long long)nrows * WARP + TT_THREADS - 1) / TT_THREADS);
            tt_rows_kernel<<<g, TT_THREADS, 0, st>>>(p->rows, nrows, p->ACC, p->DAT, p->U0D, p->CCD, nt, nx, halftime,
                                                     given, dt_min);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemsetAsync(p->C, 0, (size_t)n * sizeof(double2), st);
        if (e == cudaSuccess) {
            const unsigned g = (unsigned)(((long long)nrows * WARP + TT_THREADS - 1) / TT_THREADS);
            tt_scatter_kernel<<<g, TT_THREADS, 0, st>>>(p->rows, nrows, p->CCD, p->C, nt, nx);
            e = cudaGetLastError();
        }
        // adj_mode = Re IDFT2(filter * DFT2(c)), accumulated time-reversed
        if (e == cudaSuccess) e = dft2(p, p->C, 0, st);
        if (e == cudaSuccess) {
            tt_filter_kernel<<<tt_grid(n), TT_THREADS, 0, st>>>(p->C, p->C, filter, nt, nx, n, 0, dt_min);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = dft2(p, p->C, 1, st);
        if (e == cudaSuccess) {
            tt_accum_kernel<<<tt_grid(n), TT_THREADS, 0, st>>>(p->C, p->adj, nt, nx, n);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), p->rows, nrows * sizeof(TTRow), cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return tt_fail("sparc_tt_mode", e);
    for (int r = 0; r < nrows; r++) {
        int *q = rows + 7 * r;
        q[4] = h[r].lef;
        q[5] = h[r].rig;
        q[6] = h[r].loc;
        tau[r] = h[r].tau;
    }
    return SPARC_OK;
}

int sparc_tt_misfit_mode(sparc_tt_plan_t *p, const double *filter, int nrows, int *rows, int halftime, int given,
                         double dt_min, double *tau, void *stream)
{
    if (!p || !filter || nrows < 0 || nrows > p->cap || (nrows > 0 && (!rows || !tau)) || halftime < 0)
        return report_error(SPARC_ERR_ARG, "sparc_tt_misfit_mode: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nt = p->nt, nx = p->nx;
    const long long n = (long long)p->nb * nt * nx;
    std::vector<TTRow> h(nrows);
    for (int r = 0; r < nrows; r++) {
        const int *q = rows + 7 * r;
        if (q[0] < 0 || q[0] >= p->nb || q[1] < 0 || q[1] >= nx)
            return report_error(SPARC_ERR_ARG, "sparc_tt_misfit_mode: row out of range");
        if (!given && (max(q[2], 1) > min(q[3], nt)))
            return report_error(SPARC_ERR_ARG, "sparc_tt_misfit_mode: empty search range");
        h[r] = TTRow{q[0], q[1], q[2], q[3], q[4], q[5], 0, 0, 0.0, 0.0};
    }
    tt_filter_kernel<<<tt_grid(n), TT_THREADS, 0, st>>>(p->S, p->ACC, filter, nt, nx, n, 0, dt_min);
    tt_filter_kernel<<<tt_grid(n), TT_THREADS, 0, st>>>(p->D, p->DAT, filter, nt, nx, n, 0, dt_min);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = dft2(p, p->ACC, 1, st);
    if (e == cudaSuccess) e = dft2(p, p->DAT, 1, st);
    if (e == cudaSuccess && nrows > 0) {
        e = cudaMemcpyAsync(p->rows, h.data(), nrows * sizeof(TTRow), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) {
            const unsigned g = (unsigned)(((long long)nrows * WARP + TT_THREADS - 1) / TT_THREADS);
            tt_cc_kernel<<<g, TT_THREADS, 0, st>>>(p->rows, nrows, p->ACC, p->DAT, nt, nx, halftime, given, dt_min);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), p->rows, nrows * sizeof(TTRow), cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return tt_fail("sparc_tt_misfit_mode", e);
    for (int r = 0; r < nrows; r++) {
        int *q = rows + 7 * r;
        q[4] = h[r].lef;
        q[5] = h[r].rig;
        q[6] = h[r].loc;
        tau[r] = h[r].tau;
    }
    return SPARC_OK;
}

int sparc_tt_adjoint(sparc_tt_plan_t *p, double *adj, void *stream)
{
    if (!p || !adj) return report_error(SPARC_ERR_ARG, "sparc_tt_adjoint: null argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const long long n = (long long)p->nb * p->nt * p->nx;
    tt_scale_out_kernel<<<tt_grid(n), TT_THREADS, 0, st>>>(p->adj, adj, n, (double)p->nt / 60.0);  // driver.f90:2201
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? SPARC_OK : tt_fail("sparc_tt_adjoint", e);
}

}  // extern "C"
