// sparc_capi.cu -- the C ABI of include/sparc_gb300.h: plan life cycle, FP64 construction of
// the compact-derivative and FFT tables, background/source upload, and the step sequence
//   R(1) C(1) R(2) C(2) ... R(5) C(5) R(6) E
// (row pass, column pass of each RK stage, closing row pass, end-of-step update), captured in
// a CUDA graph and replayed once per step.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "sparc_common.cuh"
#include "sparc_gb300.h"
#include "sparc_tma.cuh"

using namespace sparc;

namespace sparc {
template <typename T>
int kernels_accumulate_static_impl(const KAccArgs<T> &proto, cudaStream_t st, std::string &err);
}

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(SPARC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));      \
    } while (0)

// ---------------------------------------------------------------------------------------------
// Compact-derivative tables (FP64).  Coefficients follow dbyd2.f, where d2i, C1..C5, alpha,
// alpha2, gamma2, alpha1, beta1, const and up1 are implicitly REAL(4): they are formed in float
// and used as double.
// ---------------------------------------------------------------------------------------------
struct HostZTab {
    int nz = 0, ibc = 0, nch = 0, L = 0, preset_row = -1;
    double c1 = 0, c2 = 0;
    std::vector<double> w5, ib, lwib, gm, WL, VU, G;
    std::vector<double> lowr, uppr;
};

bool invert(std::vector<double> &M, int n)  // Gauss-Jordan with partial pivoting, in place
{
    std::vector<double> I(n * n, 0.0);
    for (int i = 0; i < n; i++) I[i * n + i] = 1.0;
    for (int col = 0; col < n; col++) {
        int piv = col;
        for (int r = col + 1; r < n; r++)
            if (std::fabs(M[r * n + col]) > std::fabs(M[piv * n + col])) piv = r;
        if (M[piv * n + col] == 0.0) return false;
        if (piv != col)
            for (int c = 0; c < n; c++) {
                std::swap(M[piv * n + c], M[col * n + c]);
                std::swap(I[piv * n + c], I[col * n + c]);
            }
        double d = M[col * n + col];
        for (int c = 0; c < n; c++) { M[col * n + c] /= d; I[col * n + c] /= d; }
        for (int r = 0; r < n; r++) {
            if (r == col) continue;
            double f = M[r * n + col];
            if (f == 0.0) continue;
            for (int c = 0; c < n; c++) { M[r * n + c] -= f * M[col * n + c]; I[r * n + c] -= f * I[col * n + c]; }
        }
    }
    M = I;
    return true;
}

bool chunking(int nz, int lmax, int &nch, int &L)
{
    nch = (nz + lmax - 1) / lmax;
    L = (nz + nch - 1) / nch;
    if (nch > 20) return false;  // block geometry of sparc_col.cu (ColCfg MAXNCH)
    return nz - (nch - 1) * L >= 2 && L >= 2;
}

bool build_ztab(int nz, int ibc, int nch, int L, HostZTab &t)
{
    if (nz < 8) return false;
    t.nz = nz; t.ibc = ibc; t.nch = nch; t.L = L;
    const float d2i = (float)(nz - 1);
    const float C1 = d2i * 7.0f / 9.0f, C2 = d2i / 36.0f;  // dbyd2.f:82-83
    t.c1 = C1; t.c2 = C2;
    const float b1 = -(43.0f / 96.0f * d2i), b2 = -(5.0f / 6.0f * d2i), b3 = 9.0f / 8.0f * d2i,
                b4 = 1.0f / 6.0f * d2i, b5 = -(1.0f / 96.0f * d2i);        // dbyd2.f:101-105
    const float f1 = -(10.0f / 3.0f * d2i), f2 = -(3.0f * d2i), f3 = 6.0f * d2i, f4 = 1.0f / 3.0f * d2i;  // :119-122
    const float alpha = 1.0f / 3.0f, alpha2 = 3.0f / 4.0f, gamma2 = 1.0f / 8.0f, alpha1 = 6.0f, beta1 = 3.0f;
    const float cnst = 1.0f / (alpha2 - beta1 * gamma2);
    const float up1 = (alpha1 * alpha2 - beta1) * cnst;
    t.w5.assign((size_t)nz * 5, 0.0);
    const double r1[5] = {b1, b2, b3, b4, b5};                 // row 1 on b[0..4]
    const double rm2[5] = {-(double)b5, -(double)b4, -(double)b3, -(double)b2, -(double)b1};  // row nz-2 on b[nz-5..]
    for (int j = 0; j < 5; j++) { t.w5[1 * 5 + j] = r1[j]; t.w5[(size_t)(nz - 2) * 5 + j] = rm2[j]; }
    t.preset_row = -1;
    if (ibc == 1 || ibc == 3) {  // row 0: 4-point closure, then preconditioned with row 1 (dbyd2.f:178-182)
        const double r0[5] = {f1, f2, f3, f4, 0.0};
        for (int j = 0; j < 5; j++) t.w5[j] = ((double)alpha2 * r0[j] - (double)beta1 * r1[j]) * (double)cnst;
    }
    if (ibc == 1 || ibc == 2) {  // row nz-1 on b[nz-5..nz-1] (dbyd2.f:139-142, 183-187)
        const double rl[5] = {0.0, -(double)f4, -(double)f3, -(double)f2, -(double)f1};
        for (int j = 0; j < 5; j++)
            t.w5[(size_t)(nz - 1) * 5 + j] = ((double)alpha2 * rl[j] - (double)beta1 * rm2[j]) * (double)cnst;
    }
    if (ibc == 2) t.preset_row = 0;
    if (ibc == 3) t.preset_row = nz - 1;
    // matrix (dbyd2.f:151-196)
    t.uppr.assign(nz, 0.0);
    t.lowr.assign(nz, 0.0);
    for (int k = 2; k <= nz - 3; k++) t.uppr[k] = alpha;
    t.uppr[0] = (ibc % 2 == 0) ? 0.0 : (double)up1;
    t.uppr[1] = alpha2;
    t.uppr[nz - 2] = gamma2;
    for (int k = 0; k < nz; k++) t.lowr[k] = t.uppr[nz - 1 - k];
    t.lowr[nz - 1] = (ibc != 1 && ibc != 2) ? 0.0 : (double)up1;
    t.uppr[nz - 1] = 0.0;
    t.lowr[0] = 0.0;
    // chunk-local factors and spikes
    t.ib.assign(nz, 0.0); t.lwib.assign(nz, 0.0); t.gm.assign(nz, 0.0);
    t.WL.assign(nz, 0.0); t.VU.assign(nz, 0.0);
    std::vector<double> bet(nz), w(nz), v(nz);
    for (int c = 0; c < nch; c++) {
        const int s = c * L, e = std::min(nz, (c + 1) * L) - 1;
        bet[s] = 1.0;
        t.ib[s] = 1.0;
        for (int k = s + 1; k <= e; k++) {
            t.gm[k] = t.uppr[k - 1] / bet[k - 1];
            bet[k] = 1.0 - t.lowr[k] * t.gm[k];
            t.ib[k] = 1.0 / bet[k];
            t.lwib[k] = t.lowr[k] * t.ib[k];
        }
        auto solve = [&](std::vector<double> &y, int unit_row) {
            for (int k = s; k <= e; k++) {
                double r = (k == unit_row) ? 1.0 : 0.0;
                y[k] = r * t.ib[k] - (k > s ? t.lwib[k] * y[k - 1] : 0.0);
            }
            for (int k = e - 1; k >= s; k--) y[k] -= t.gm[k + 1] * y[k + 1];
        };
        solve(w, s);
        solve(v, e);
        const double ls = (s > 0) ? t.lowr[s] : 0.0;
        const double ue = (e < nz - 1) ? t.uppr[e] : 0.0;
        for (int k = s; k <= e; k++) { t.WL[k] = ls * w[k]; t.VU[k] = ue * v[k]; }
    }
    // reduced system for u = (x[s_0], x[e_0], x[s_1], x[e_1], ...)
    const int n2 = 2 * nch;
    std::vector<double> M((size_t)n2 * n2, 0.0);
    for (int c = 0; c < nch; c++) {
        const int s = c * L, e = std::min(nz, (c + 1) * L) - 1;
        const int rows[2] = {s, e};
        for (int h = 0; h < 2; h++) {
            const int r = 2 * c + h, k = rows[h];
            M[(size_t)r * n2 + r] += 1.0;
            if (c > 0) M[(size_t)r * n2 + (2 * c - 1)] += t.WL[k];
            if (c < nch - 1) M[(size_t)r * n2 + (2 * c + 2)] += t.VU[k];
        }
    }
    if (!invert(M, n2)) return false;
    t.G = M;
    return true;
}

// ---------------------------------------------------------------------------------------------
// Geometric-band form of the compact derivative (FP32 column pass).  The right-hand side is
// formed exactly as dbyd2 forms it; the tridiagonal solve x = T^{-1} rhs is replaced by the
// inverse of the infinite Toeplitz operator (1/3, 1, 1/3), whose entries are exactly geometric,
// t0 r^|d| with r = -(3 - sqrt 5)/2, applied with rhs zero outside 0..nz-1.  The boundary rows
// of T (dbyd2.f:151-196) and the finite ends make T^{-1} differ from it only near the two
// corners (elsewhere by < 1e-9 of t0), where the difference has rank 2 on a KC x KC block; it is
// factored by cross approximation with full pivoting.
// ---------------------------------------------------------------------------------------------
struct HostBand {
    int nz = 0, q = 0;
    double t0 = 0, r = 0;
    std::vector<double> uv;  // Ub [KC][Q], Vb [Q][KC], Ut [KC][Q], Vt [Q][KC], then the top-block
                             // Thomas factors ib [KC], lwib [KC], gm [KC] and the coupling lowr
    double err = 0;          // max |T^{-1} - band - corners| / max |T^{-1}|
};

// Cross approximation of the n x n matrix C (row-major) to rank <= qmax: C ~ U V.
static int cross_approx(std::vector<double> C, int n, int qmax, double tol, double *U, double *V)
{
    for (int i = 0; i < n * qmax; i++) { U[i] = 0.0; V[i] = 0.0; }
    int q = 0;
    for (; q < qmax; q++) {
        int pi = 0, pj = 0;
        double best = 0.0;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++)
                if (std::fabs(C[(size_t)i * n + j]) > best) { best = std::fabs(C[(size_t)i * n + j]); pi = i; pj = j; }
        if (best <= tol) break;
        const double piv = C[(size_t)pi * n + pj];
        for (int i = 0; i < n; i++) U[i * qmax + q] = C[(size_t)i * n + pj];
        for (int j = 0; j < n; j++) V[q * n + j] = C[(size_t)pi * n + j] / piv;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) C[(size_t)i * n + j] -= U[i * qmax + q] * V[q * n + j];
    }
    return q;
}

bool build_band(const HostZTab &tz, HostBand &h)
{
    const int nz = tz.nz, KC = BAND_KC, Q = BAND_Q;
    if (nz < 2 * KC + 2 * BAND_W) return false;
    h.nz = nz;
    // T^{-1} column by column (diag 1, sub lowr, super uppr), Thomas on unit vectors
    std::vector<double> gam(nz), bet(nz), Ti((size_t)nz * nz, 0.0), y(nz);
    bet[0] = 1.0;
    for (int k = 1; k < nz; k++) {
        gam[k] = tz.uppr[k - 1] / bet[k - 1];
        bet[k] = 1.0 - tz.lowr[k] * gam[k];
    }
    for (int col = 0; col < nz; col++) {
        for (int k = 0; k < nz; k++) y[k] = ((k == col ? 1.0 : 0.0) - (k > 0 ? tz.lowr[k] * y[k - 1] : 0.0)) / bet[k];
        for (int k = nz - 2; k >= 0; k--) y[k] -= gam[k + 1] * y[k + 1];
        for (int k = 0; k < nz; k++) Ti[(size_t)k * nz + col] = y[k];
    }
    const int kc = nz / 2;
    h.t0 = Ti[(size_t)kc * nz + kc];
    h.r = Ti[(size_t)kc * nz + kc + 1] / h.t0;
    std::vector<double> rp(nz + 1);
    rp[0] = 1.0;
    for (int d = 1; d <= nz; d++) rp[d] = rp[d - 1] * h.r;
    auto band = [&](int k, int j) { return h.t0 * rp[std::abs(k - j)]; };
    double mx = 0.0;
    for (double v : Ti) mx = std::max(mx, std::fabs(v));
    h.uv.assign((size_t)4 * KC * Q, 0.0);
    double *Ub = h.uv.data(), *Vb = Ub + KC * Q, *Ut = Vb + KC * Q, *Vt = Ut + KC * Q;
    std::vector<double> C((size_t)KC * KC);
    for (int i = 0; i < KC; i++)
        for (int j = 0; j < KC; j++) C[(size_t)i * KC + j] = Ti[(size_t)i * nz + j] - band(i, j);
    const int qb = cross_approx(C, KC, Q, 1e-13 * mx, Ub, Vb);
    const int o = nz - KC;
    for (int i = 0; i < KC; i++)
        for (int j = 0; j < KC; j++) C[(size_t)i * KC + j] = Ti[(size_t)(o + i) * nz + o + j] - band(o + i, o + j);
    const int qt = cross_approx(C, KC, Q, 1e-13 * mx, Ut, Vt);
    h.q = std::max(qb, qt);
    double dev = 0.0;
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < nz; j++) {
            double v = band(k, j);
            if (k < KC && j < KC)
                for (int q = 0; q < Q; q++) v += Ub[k * Q + q] * Vb[q * KC + j];
            if (k >= o && j >= o)
                for (int q = 0; q < Q; q++) v += Ut[(k - o) * Q + q] * Vt[q * KC + (j - o)];
            dev = std::max(dev, std::fabs(Ti[(size_t)k * nz + j] - v));
        }
    h.err = dev / mx;
    {  // Thomas factors of T restricted to the top KC rows (x[nz-KC-1] moves to the right-hand side)
        std::vector<double> th((size_t)3 * KC + 1, 0.0);
        double *ib = th.data(), *lwib = ib + KC, *gm = lwib + KC;
        double bprev = 1.0;
        ib[0] = 1.0;
        for (int m = 1; m < KC; m++) {
            const int k = o + m;
            gm[m] = tz.uppr[k - 1] / bprev;
            const double bet = 1.0 - tz.lowr[k] * gm[m];
            ib[m] = 1.0 / bet;
            lwib[m] = tz.lowr[k] * ib[m];
            bprev = bet;
        }
        th[3 * KC] = tz.lowr[o];
        h.uv.insert(h.uv.end(), th.begin(), th.end());
    }
    return h.err < 1e-8;
}

// dbyd2's right-hand side of row k of column i (interior c1/c2 differences, boundary closures,
// caller-set row), the same algebra as zrhs on the device.
static double zrhs_host(const HostZTab &t, const double *b, int n1, int i, int k, double preset)
{
    const int nz = t.nz;
    auto f = [&](int kk) { return b[(size_t)kk * n1 + i]; };
    if (k >= 2 && k <= nz - 3) return t.c1 * (f(k + 1) - f(k - 1)) + t.c2 * (f(k + 2) - f(k - 2));
    if (k == t.preset_row) return preset;
    const int base = (k <= 1) ? 0 : nz - 5;
    double r = 0.0;
    for (int j = 0; j < 5; j++) r += t.w5[(size_t)k * 5 + j] * f(base + j);
    return r;
}

// Host evaluation of the geometric-band form, unstretched: x = t0 sum_d r^|d| rhs[k+d] + corners.
void zband_host(const HostZTab &t, const HostBand &h, const double *b, double *x, const double *preset_v, int n1)
{
    const int nz = h.nz, KC = BAND_KC, Q = BAND_Q, o = nz - KC;
    const double *Ub = h.uv.data(), *Vb = Ub + KC * Q, *Ut = Vb + KC * Q, *Vt = Ut + KC * Q;
    std::vector<double> rhs(nz);
    for (int i = 0; i < n1; i++) {
        for (int k = 0; k < nz; k++) rhs[k] = zrhs_host(t, b, n1, i, k, preset_v ? preset_v[i] : 0.0);
        double sb[BAND_Q] = {}, st[BAND_Q] = {};
        for (int q = 0; q < Q; q++)
            for (int j = 0; j < KC; j++) { sb[q] += Vb[q * KC + j] * rhs[j]; st[q] += Vt[q * KC + j] * rhs[o + j]; }
        for (int k = 0; k < nz; k++) {
            // sum_{d>=1} r^d (rhs[k-d] + rhs[k+d]), accumulated outward from the row
            double v = rhs[k], L = 0.0, U = 0.0, rd = 1.0;
            for (int d = 1; d < nz; d++) {
                rd *= h.r;
                if (k - d >= 0) L += rd * rhs[k - d];
                if (k + d < nz) U += rd * rhs[k + d];
            }
            v = h.t0 * (v + L + U);
            if (k < KC)
                for (int q = 0; q < Q; q++) v += Ub[k * Q + q] * sb[q];
            if (k >= o)
                for (int q = 0; q < Q; q++) v += Ut[(k - o) * Q + q] * st[q];
            x[(size_t)k * n1 + i] = v;
        }
    }
}

// Host evaluation of the partitioned solve (same algebra as the device code).
void zsolve_host(const HostZTab &t, const double *b, double *x, const double *preset_v, int n1)
{
    const int nz = t.nz, nch = t.nch, L = t.L, n2 = 2 * nch;
    std::vector<double> col(nz), y(nz), ub(n2);
    for (int i = 0; i < n1; i++) {
        for (int k = 0; k < nz; k++) col[k] = b[(size_t)k * n1 + i];
        auto rhs = [&](int k) {
            if (k >= 2 && k <= nz - 3) return t.c1 * (col[k + 1] - col[k - 1]) + t.c2 * (col[k + 2] - col[k - 2]);
            if (k == t.preset_row) return preset_v ? preset_v[i] : 0.0;
            const int base = (k <= 1) ? 0 : nz - 5;
            double r = 0.0;
            for (int j = 0; j < 5; j++) r += t.w5[(size_t)k * 5 + j] * col[base + j];
            return r;
        };
        for (int c = 0; c < nch; c++) {
            const int s = c * L, e = std::min(nz, (c + 1) * L) - 1;
            for (int k = s; k <= e; k++) y[k] = rhs(k) * t.ib[k] - (k > s ? t.lwib[k] * y[k - 1] : 0.0);
            for (int k = e - 1; k >= s; k--) y[k] -= t.gm[k + 1] * y[k + 1];
            ub[2 * c] = y[s];
            ub[2 * c + 1] = y[e];
        }
        for (int c = 0; c < nch; c++) {
            const int s = c * L, e = std::min(nz, (c + 1) * L) - 1;
            double xl = 0, xr = 0;
            if (c > 0) for (int q = 0; q < n2; q++) xl += t.G[(size_t)(2 * c - 1) * n2 + q] * ub[q];
            if (c < nch - 1) for (int q = 0; q < n2; q++) xr += t.G[(size_t)(2 * c + 2) * n2 + q] * ub[q];
            for (int k = s; k <= e; k++) x[(size_t)k * n1 + i] = y[k] - t.WL[k] * xl - t.VU[k] * xr;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Device memory helpers
// ---------------------------------------------------------------------------------------------
template <typename T>
__global__ void cast_kernel(const double *__restrict__ src, T *__restrict__ dst, size_t n)
{
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) dst[i] = (T)src[i];
}

template <typename T>
cudaError_t cast_to(const double *src, T *dst, size_t n, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    int blocks = (int)std::min<size_t>((n + 255) / 256, 4096);
    cast_kernel<T><<<blocks, 256, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}

// Sum of squares of v_z per solve (one block per solve), FP64 accumulation.
template <typename T>
__global__ void vz_norm_kernel(const T *__restrict__ A, size_t F, double *__restrict__ out)
{
    const T *vz = A + ((size_t)blockIdx.x * 4 + 3) * F;
    double s = 0.0;
    for (size_t i = threadIdx.x; i < F; i += blockDim.x) {
        const double v = (double)vz[i];
        s += v * v;
    }
    __shared__ double red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

template <typename T>
struct DevZ {
    T *buf = nullptr;
    ZTab<T> tab{};
};

template <typename T>
cudaError_t upload_ztab(const HostZTab &h, DevZ<T> &d, std::vector<void *> &allocs)
{
    const int nz = h.nz, n2 = 2 * h.nch;
    const size_t n = (size_t)nz * 5 + (size_t)nz * 5 + (size_t)n2 * n2;
    std::vector<T> host(n);
    size_t o = 0;
    auto put = [&](const std::vector<double> &v) { for (double x : v) host[o++] = (T)x; };
    put(h.w5); put(h.ib); put(h.lwib); put(h.gm); put(h.WL); put(h.VU); put(h.G);
    cudaError_t e = cudaMalloc(&d.buf, n * sizeof(T));
    if (e != cudaSuccess) return e;
    allocs.push_back(d.buf);
    e = cudaMemcpy(d.buf, host.data(), n * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    T *p = d.buf;
    d.tab.w5 = p; p += (size_t)nz * 5;
    d.tab.ib = p; p += nz;
    d.tab.lwib = p; p += nz;
    d.tab.gm = p; p += nz;
    d.tab.WL = p; p += nz;
    d.tab.VU = p; p += nz;
    d.tab.G = p;
    d.tab.c1 = (T)h.c1;
    d.tab.c2 = (T)h.c2;
    d.tab.preset_row = h.preset_row;
    return cudaSuccess;
}

template <typename T>
struct DevFFT {
    T *buf = nullptr;
    const T *twr = nullptr, *twi = nullptr, *kap = nullptr;
};

template <typename T>
cudaError_t upload_fft(int n, DevFFT<T> &d, std::vector<void *> &allocs)
{
    std::vector<T> host((size_t)3 * n);
    const double pi = 3.141592653589793;
    for (int t = 0; t < n; t++) {
        host[t] = (T)std::cos(2.0 * pi * (double)t / (double)n);
        host[n + t] = (T)(-std::sin(2.0 * pi * (double)t / (double)n));
        double kap;  // eyekx (initialize.f90:206-208) with the Nyquist bin dropped by c2r
        if (2 * t < n) kap = (double)t * (1.0 / (double)n) * 2.0 * pi;
        else if (2 * t == n) kap = 0.0;
        else kap = -(double)(n - t) * (1.0 / (double)n) * 2.0 * pi;
        host[2 * n + t] = (T)kap;
    }
    cudaError_t e = cudaMalloc(&d.buf, host.size() * sizeof(T));
    if (e != cudaSuccess) return e;
    allocs.push_back(d.buf);
    e = cudaMemcpy(d.buf, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice);
    d.twr = d.buf; d.twi = d.buf + n; d.kap = d.buf + 2 * n;
    return e;
}

// 2-D tiled tensor map over rows x nx of an x-fastest field array (box: boxw columns x boxr rows).
bool encode_map(CUtensorMap *m, const void *base, int nx, long long rows, int boxr, size_t esize, int boxw = 8)
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn)
            return false;
        encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }
    const cuuint64_t dims[2] = {(cuuint64_t)nx, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)nx * esize};
    const cuuint32_t box[2] = {(cuuint32_t)boxw, (cuuint32_t)boxr};
    const cuuint32_t estr[2] = {1u, 1u};
    CUresult r = encode(m, esize == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2,
                        const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

template <typename T>
struct Solver {
    StepArgs<T> a{};
    ColMaps maps{};
    bool have_maps = false;
    ColMaps32 maps32{};        // 32-column boxes of nz/2 rows (TMA-staged first phase of the banded pass)
    bool have_maps32 = false;
    DevZ<T> z[4];
    DevFFT<T> fft;
    BandDev band{};    // banded z-derivative tables (FP32 plans, column_impl 2)
    int band_R = 0;    // rows per thread group of the banded column pass (0: not used)
    int band_cw = 0;   // its block width (columns)
    int band_tma_R = 0;  // rows per thread group of the TMA-staged banded pass (0: not used)
    bool end_stream = false;  // streamed end-of-step kernel (32-column tiles) fits this grid
    std::vector<void *> allocs;
    size_t F = 0;
    T *work = nullptr;  // kernel-accumulation scratch [nb][8][nz][nx]
};

}  // namespace

struct sparc_plan {
    sparc_config_t cfg{};
    int nch = 0, L = 0, nch64 = 0, L64 = 0;
    std::vector<void *> allocs;
    HostZTab hz[4], hz64[4];
    DevZ<double> z64[4];
    DevFFT<double> fft64;
    Solver<float> s32;
    Solver<double> s64;
    int *d_time = nullptr;
    int *d_err = nullptr;
    bool have_bg = false, have_src = false;
    double unstretch_top = 1.0;
    cudaGraphExec_t gexec = nullptr;
    cudaGraph_t graph = nullptr;
    const void *g_seis = nullptr, *g_snaps = nullptr;
    int g_cap = -1, g_rec0 = 0;
    double g_fsign = 0.0;
    cudaStream_t g_stream = nullptr;
    double *d_srcw = nullptr;
    int *d_srcidx = nullptr;
};

namespace {

template <typename T>
Solver<T> &solver(sparc_plan *p);
template <>
Solver<float> &solver<float>(sparc_plan *p) { return p->s32; }
template <>
Solver<double> &solver<double>(sparc_plan *p) { return p->s64; }

template <typename T>
int alloc_solver(sparc_plan *p)
{
    Solver<T> &S = solver<T>(p);
    const sparc_config_t &c = p->cfg;
    const int nx = c.nx, nz = c.nz, nb = c.nbatch;
    const int nzpml = c.npmlbot + c.npmltop, nhx = 2 * c.npmlhor;
    const size_t F = (size_t)nx * nz;
    S.F = F;
    const int nbg = c.bg_per_solve ? nb : 1;
    struct Req { T **ptr; size_t n; };
    T *A, *SV, *P, *RVXP, *DX, *FXX, *FXZ, *TOPDX, *PZ, *SPZ, *PX, *SPX;
    T *rhoinv, *rho0, *gp0, *gr0, *g, *stretch, *fdz, *az, *bz, *ax, *bx, *c2rho0, *v0x, *v0z, *inj, *rows;
    std::vector<Req> reqs = {
        {&A, (size_t)nb * 4 * F}, {&SV, (size_t)3 * nb * 2 * F}, {&P, nb * F}, {&RVXP, nb * F}, {&DX, nb * F},
        {&FXX, nb * F}, {&FXZ, nb * F}, {&TOPDX, (size_t)nb * nx},
        {&PZ, (size_t)nb * 2 * nzpml * nx}, {&SPZ, (size_t)3 * nb * 2 * nzpml * nx},
        {&PX, (size_t)nb * 2 * nz * nhx}, {&SPX, (size_t)3 * nb * 2 * nz * nhx},
        {&rhoinv, (size_t)nz}, {&rho0, (size_t)nz}, {&gp0, (size_t)nz}, {&gr0, (size_t)nz}, {&g, (size_t)nz},
        {&stretch, (size_t)nz}, {&fdz, (size_t)nbg * nzpml * nx}, {&az, (size_t)nbg * nzpml * nx},
        {&bz, (size_t)nbg * nzpml * nx}, {&ax, (size_t)nbg * nz * nhx}, {&bx, (size_t)nbg * nz * nhx},
        {&c2rho0, c.c2d ? nbg * F : (size_t)nz}, {&v0x, c.flows ? nbg * F : 1}, {&v0z, c.flows ? nbg * F : 1},
        {&inj, (size_t)nb * nx}, {&rows, (size_t)nb * nx},
    };
    for (auto &r : reqs) {
        void *ptr = nullptr;
        cudaError_t e = cudaMalloc(&ptr, std::max<size_t>(r.n, 1) * sizeof(T));
        if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        S.allocs.push_back(ptr);
        cudaMemset(ptr, 0, std::max<size_t>(r.n, 1) * sizeof(T));
        *r.ptr = (T *)ptr;
    }
    // tables
    for (int ibc = 0; ibc < 4; ibc++) {
        cudaError_t e = upload_ztab<T>(p->hz[ibc], S.z[ibc], S.allocs);
        if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("table upload: ") + cudaGetErrorString(e));
    }
    {
        cudaError_t e = upload_fft<T>(nx, S.fft, S.allocs);
        if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("fft upload: ") + cudaGetErrorString(e));
    }
    StepArgs<T> &a = S.a;
    a.nx = nx; a.nz = nz; a.nb = nb; a.nh = c.npmlhor; a.nhx = nhx; a.nzpml = nzpml;
    a.npmlbot = c.npmlbot; a.npmltop = c.npmltop;
    a.flows = c.flows; a.c2d = c.c2d;
    a.bg2 = c.bg_per_solve ? (long long)F : 0;
    a.bgz = c.bg_per_solve ? (long long)nzpml * nx : 0;
    a.bgx = c.bg_per_solve ? (long long)nz * nhx : 0;
    a.dt = (T)c.deltat; a.stretchx = (T)c.stretchx; a.fsign = T(1);
    a.ALO = nullptr;
    if (sizeof(T) == 4 && c.compensated) {  // low parts of the FP32 state (compensated update)
        void *ptr = nullptr;
        cudaError_t e = cudaMalloc(&ptr, (size_t)nb * 4 * F * sizeof(T));
        if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        S.allocs.push_back(ptr);
        cudaMemset(ptr, 0, (size_t)nb * 4 * F * sizeof(T));
        a.ALO = (T *)ptr;
    }
    a.A = A; a.SV = SV; a.P = P; a.RVXP = RVXP; a.DX = DX; a.FXX = FXX; a.FXZ = FXZ; a.TOPDX = TOPDX;
    a.PZ = PZ; a.SPZ = SPZ; a.PX = PX; a.SPX = SPX;
    a.rhoinv = rhoinv; a.rho0 = rho0; a.gp0 = gp0; a.gr0 = gr0; a.g = g; a.stretch = stretch;
    a.fdz = fdz; a.az = az; a.bz = bz; a.ax = ax; a.bx = bx; a.c2rho0 = c2rho0; a.v0x = v0x; a.v0z = v0z;
    a.twr = S.fft.twr; a.twi = S.fft.twi; a.kap = S.fft.kap;
    a.z1 = S.z[1].tab; a.z2 = S.z[2].tab; a.z3 = S.z[3].tab;
    a.nch = p->nch; a.L = p->L;
    a.d_time = p->d_time;
    a.src_until = c.src_until; a.k_inj = c.k_inj; a.k_obs = c.k_obs; a.steps_out = c.steps_out;
    a.filt_k0 = c.filter_k0; a.filt_xall = c.filter_all_x;
    // partitioned-solve block width: 32, 8 or 4 columns on request; otherwise 32 when those blocks
    // (nx / 32 per solve) fill the 152 SMs, else 8.  One FP64 solve of 256 columns (the plain
    // configuration): column pass 0.66 ms per step at 32 columns (8 blocks), 0.33 at 8 (32
    // blocks), 0.35 at 4 (64 blocks, 76 threads each) on a GB300
    if ((c.column_block == 32 || c.column_block == 8 || c.column_block == 4) && nx % c.column_block == 0) {
        a.colw = c.column_block;
    } else {
        a.colw = (nx % 32 == 0 && (long long)(nx / 32) * nb >= 152) ? 32 : 8;
    }
    a.inj_scale = inj; a.src_rows = rows; a.nrows = 1;
    a.d_err = p->d_err;
    {  // streamed end-of-step kernel: two [nz][32] fields in shared memory
        int maxsm = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        S.end_stream = nx % 32 == 0 && end_stream_smem_bytes<T>(nz) <= (size_t)maxsm;
    }
    // banded column pass (FP32 only: its truncation at 5e-10 is below FP32 rounding, not FP64's)
    S.band_R = 0;
    const int bcw = (c.column_block == 8 || c.column_block == 16 || c.column_block == 32) ? c.column_block : 32;
    if (sizeof(T) == 4 && (c.column_impl == 2 || c.column_impl == 3) && nx % bcw == 0 && col_band_rows(nz, bcw) > 0) {
        const int R = col_band_rows(nz, bcw);
        int maxsm = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        bool ok = col_band_smem_bytes(nz, nzpml, R, bcw) <= (size_t)maxsm;
        HostBand hb[3];
        for (int i = 0; i < 3 && ok; i++) ok = build_band(p->hz[i + 1], hb[i]);
        for (int i = 1; i < 3 && ok; i++)  // the interior operator does not depend on the boundary condition
            ok = std::fabs(hb[i].t0 - hb[0].t0) <= 1e-12 * std::fabs(hb[0].t0) && std::fabs(hb[i].r - hb[0].r) <= 1e-12;
        for (int i = 0; i < 3 && ok; i++) {
            std::vector<float> f(hb[i].uv.begin(), hb[i].uv.end());
            void *ptr = nullptr;
            if (cudaMalloc(&ptr, f.size() * sizeof(float)) != cudaSuccess) return fail(SPARC_ERR_CUDA, "cudaMalloc: band tables");
            S.allocs.push_back(ptr);
            cudaMemcpy(ptr, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice);
            S.band.uv[i] = (const float *)ptr;
        }
        if (ok) {
            for (int i = 0; i < 2; i++)  // Thomas factors of ibc 1, 2 as kernel-parameter copies
                for (int j = 0; j < 3 * BAND_KC + 1; j++)
                    S.band.th[i][j] = (float)hb[i].uv[(size_t)4 * BAND_KC * BAND_Q + j];
            S.band.t0 = (float)hb[0].t0;
            S.band.r = (float)hb[0].r;
            double rp = 1.0;
            for (int d = 0; d < BAND_NPOW; d++) { S.band.rpow[d] = (float)rp; rp *= hb[0].r; }
            S.band_R = R;
            S.band_cw = bcw;
            // specialised grids: the first phase's inputs staged by TMA (boxes of 32 columns x nz/2 rows)
            S.have_maps32 = col_band_specialised(nx, nz, bcw, R) && nz % 2 == 0 && nz / 2 <= 256 &&
                            encode_map(&S.maps32.A, A, nx, (long long)nb * 4 * nz, nz / 2, sizeof(float), 32) &&
                            encode_map(&S.maps32.SV, SV, nx, (long long)3 * nb * 2 * nz, nz / 2, sizeof(float), 32) &&
                            encode_map(&S.maps32.DX, DX, nx, (long long)nb * nz, nz / 2, sizeof(float), 32);
        }
    }
    // TMA tiles: boxes of boxr rows, a multiple of 128 bytes so both boxes of a tile start
    // 128-byte aligned in shared memory; two boxes cover nz
    {
        const int per128 = (int)(128 / (8 * sizeof(T)));
        int boxr = (nz + 1) / 2;
        boxr = ((boxr + per128 - 1) / per128) * per128;
        a.boxr = boxr;
        const size_t es = sizeof(T);
        S.have_maps = boxr <= 256 && nx % 8 == 0 && c.column_impl != 0 &&
                      encode_map(&S.maps.A, A, nx, (long long)nb * 4 * nz, boxr, es) &&
                      encode_map(&S.maps.SV, SV, nx, (long long)3 * nb * 2 * nz, boxr, es) &&
                      encode_map(&S.maps.DX, DX, nx, (long long)nb * nz, boxr, es) &&
                      encode_map(&S.maps.FXX, FXX, nx, (long long)nb * nz, boxr, es) &&
                      encode_map(&S.maps.FXZ, FXZ, nx, (long long)nb * nz, boxr, es);
        if (S.have_maps) {
            const size_t smem = col_tma_smem_bytes<T>(nz, p->nch, boxr);
            int maxsm = 0, dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
            if (smem > (size_t)maxsm) S.have_maps = false;
            // TMA-staged banded pass (FP32): also the 2-D background tiles it stages
            const int Rt = col_band_tma_rows(nz);
            if (sizeof(T) == 4 && c.column_impl == 3 && S.band_R > 0 && Rt > 0 &&
                col_band_tma_smem_bytes(nz, Rt, boxr) <= (size_t)maxsm &&
                (!c.c2d || encode_map(&S.maps.C2R, c2rho0, nx, (long long)nbg * nz, boxr, es)) &&
                (!c.flows || encode_map(&S.maps.V0Z, v0z, nx, (long long)nbg * nz, boxr, es)))
                S.band_tma_R = Rt;
        }
    }
    // stage overlap: the 512-column row pass starts on the SMs that the banded column pass's last
    // wave leaves idle, each row block waiting for its own solve's column tiles only
    // (SPARC_STAGE_OVERLAP=0 turns it off)
    a.tile_cnt = nullptr;
    a.tiles_per_solve = 0;
    {
        const char *ov = std::getenv("SPARC_STAGE_OVERLAP");
        const bool want = !(ov && ov[0] == '0');
        if (want && sizeof(T) == 4 && nx == 512 && S.band_R > 0 && S.band_tma_R == 0 && c.column_impl == 2) {
            void *ptr = nullptr;
            if (cudaMalloc(&ptr, (size_t)5 * nb * sizeof(int)) != cudaSuccess)
                return fail(SPARC_ERR_CUDA, "cudaMalloc: stage-overlap counters");
            S.allocs.push_back(ptr);
            cudaMemset(ptr, 0, (size_t)5 * nb * sizeof(int));
            a.tile_cnt = (int *)ptr;
            a.tiles_per_solve = nx / S.band_cw;
        }
    }
    return SPARC_OK;
}

template <typename T>
void free_solver(Solver<T> &S)
{
    for (void *q : S.allocs) cudaFree(q);
    S.allocs.clear();
}

template <typename T>
cudaError_t col_stage(sparc_plan *p, const StepArgs<T> &a, cudaStream_t st)
{
    Solver<T> &S = solver<T>(p);
    if constexpr (sizeof(T) == 4) {
        switch (S.band_tma_R) {
            case 9: return launch_col_stage_band_tma<9>(S.maps, a, S.band, st);
            case 11: return launch_col_stage_band_tma<11>(S.maps, a, S.band, st);
            case 13: return launch_col_stage_band_tma<13>(S.maps, a, S.band, st);
            default: break;
        }
        const ColMaps32 *m32 = S.have_maps32 ? &S.maps32 : nullptr;
        switch (S.band_cw * 100 + S.band_R) {
            case 3208: return launch_col_stage_band<32, 8>(a, S.band, m32, st);
            case 3210: return launch_col_stage_band<32, 10>(a, S.band, m32, st);
            case 3212: return launch_col_stage_band<32, 12>(a, S.band, m32, st);
            case 1609: return launch_col_stage_band<16, 9>(a, S.band, m32, st);
            case 1611: return launch_col_stage_band<16, 11>(a, S.band, m32, st);
            case 1613: return launch_col_stage_band<16, 13>(a, S.band, m32, st);
            case 809: return launch_col_stage_band<8, 9>(a, S.band, m32, st);
            case 811: return launch_col_stage_band<8, 11>(a, S.band, m32, st);
            case 813: return launch_col_stage_band<8, 13>(a, S.band, m32, st);
            default: break;
        }
    }
    return (S.have_maps && p->cfg.column_impl == 1) ? launch_col_stage_tma<T>(S.maps, a, st)
                                                     : launch_col_stage<T>(a, st);
}

template <typename T>
cudaError_t end_step(sparc_plan *p, const StepArgs<T> &a, cudaStream_t st)
{
    Solver<T> &S = solver<T>(p);
    if (a.ALO) {  // compensated (double-float) update
        if constexpr (sizeof(T) == 4)
            if (p->cfg.nx % 16 == 0 && S.end_stream) return launch_end_step_comp(a, st);
        return launch_end_step<T>(a, st);
    }
    if (S.have_maps && p->cfg.column_impl == 1) return launch_end_step_tma<T>(S.maps, a, st);
    return S.end_stream ? launch_end_step_stream<T>(a, st) : launch_end_step<T>(a, st);
}

template <typename T>
cudaError_t enqueue_step(sparc_plan *p, StepArgs<T> a, cudaStream_t st)
{
    const double *B = p->cfg.betas;  // B[s-1] = beta of stage s (B[0] = 0)
    cudaError_t e;
    if (a.tile_cnt && (e = cudaMemsetAsync(a.tile_cnt, 0, (size_t)5 * a.nb * sizeof(int), st)) != cudaSuccess) return e;
    for (int s = 1; s <= 5; s++) {
        a.stage = s;
        a.bs = (T)B[s - 1];
        a.bsm1 = (s >= 2) ? (T)B[s - 2] : T(0);
        a.slot_s = s % 3; a.slot_sm1 = (s - 1) % 3; a.slot_sm2 = (s + 1) % 3;  // (s-2) mod 3
        if ((e = launch_row_stage<T>(a, st)) != cudaSuccess) return e;
        if ((e = col_stage(p, a, st)) != cudaSuccess) return e;
    }
    a.stage = 6;
    a.bs = (T)0; a.bsm1 = (T)B[4];
    a.slot_s = 0; a.slot_sm1 = 5 % 3; a.slot_sm2 = 4 % 3;
    if ((e = launch_row_stage<T>(a, st)) != cudaSuccess) return e;
    a.stage = 7;
    a.bs = (T)B[4];
    a.slot_s = 5 % 3; a.slot_sm1 = 4 % 3;
    return end_step(p, a, st);
}

template <typename T>
int profile_passes(sparc_plan *p, int nsteps, double *ms, cudaStream_t st)
{
    StepArgs<T> a = solver<T>(p).a;
    a.fsign = T(1);
    a.seis = nullptr; a.snaps = nullptr; a.nrec_cap = 0;
    a.tile_cnt = nullptr;  // passes timed one by one: no stage overlap, whose row pass would wait
    a.unstretch_top = (T)p->unstretch_top;
    const double *B = p->cfg.betas;
    std::vector<cudaEvent_t> ev;
    std::vector<int> cls;
    auto rec = [&](int c) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecord(e, st);
        ev.push_back(e);
        cls.push_back(c);
    };
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < nsteps && e == cudaSuccess; i++) {
        for (int s = 1; s <= 5 && e == cudaSuccess; s++) {
            a.stage = s; a.bs = (T)B[s - 1]; a.bsm1 = (s >= 2) ? (T)B[s - 2] : T(0);
            a.slot_s = s % 3; a.slot_sm1 = (s - 1) % 3; a.slot_sm2 = (s + 1) % 3;
            rec(0); e = launch_row_stage<T>(a, st); rec(-1);
            if (e != cudaSuccess) break;
            rec(1); e = col_stage(p, a, st); rec(-1);
        }
        if (e != cudaSuccess) break;
        a.stage = 6; a.bs = T(0); a.bsm1 = (T)B[4]; a.slot_s = 0; a.slot_sm1 = 2; a.slot_sm2 = 1;
        rec(0); e = launch_row_stage<T>(a, st); rec(-1);
        if (e != cudaSuccess) break;
        a.stage = 7; a.bs = (T)B[4]; a.slot_s = 2; a.slot_sm1 = 1;
        rec(2); e = end_step(p, a, st); rec(-1);
    }
    cudaError_t es = cudaStreamSynchronize(st);
    ms[0] = ms[1] = ms[2] = ms[3] = 0.0;
    if (e == cudaSuccess && es == cudaSuccess && ev.size() >= 2) {
        for (size_t i = 0; i + 1 < ev.size(); i += 2) {
            float t = 0.f;
            cudaEventElapsedTime(&t, ev[i], ev[i + 1]);
            ms[cls[i]] += t;
        }
        float tot = 0.f;
        cudaEventElapsedTime(&tot, ev.front(), ev.back());
        ms[3] = tot;
    }
    for (auto x : ev) cudaEventDestroy(x);
    if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("profile: ") + cudaGetErrorString(e));
    if (es != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("profile sync: ") + cudaGetErrorString(es));
    return SPARC_OK;
}

template <typename T>
int run_forward(sparc_plan *p, int nsteps, double fsign, void *seis, void *snaps, int rec0, int cap, int use_graph,
                cudaStream_t st)
{
    Solver<T> &S = solver<T>(p);
    StepArgs<T> a = S.a;
    a.fsign = (T)fsign;
    a.seis = (T *)seis;
    a.snaps = (T *)snaps;
    a.nrec_cap = cap;
    a.rec0 = rec0;
    a.unstretch_top = (T)p->unstretch_top;
    if (!use_graph) {
        for (int i = 0; i < nsteps; i++) CK(enqueue_step<T>(p, a, st));
        return SPARC_OK;
    }
    const bool same = p->gexec && p->g_seis == seis && p->g_snaps == snaps && p->g_cap == cap &&
                      p->g_rec0 == rec0 && p->g_fsign == fsign && p->g_stream == st;
    if (!same) {
        if (p->gexec) { cudaGraphExecDestroy(p->gexec); p->gexec = nullptr; }
        if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
        // warm the launch attributes outside of capture
        cudaStream_t cap_st;
        CK(cudaStreamCreateWithFlags(&cap_st, cudaStreamNonBlocking));
        cudaError_t e = cudaStreamBeginCapture(cap_st, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) e = enqueue_step<T>(p, a, cap_st);
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(cap_st, &g);
        cudaStreamDestroy(cap_st);
        if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return fail(SPARC_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e)); }
        if (e2 != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e2));
        p->graph = g;
        CK(cudaGraphInstantiate(&p->gexec, g, 0));
        p->g_seis = seis; p->g_snaps = snaps; p->g_cap = cap; p->g_rec0 = rec0; p->g_fsign = fsign; p->g_stream = st;
    }
    for (int i = 0; i < nsteps; i++) CK(cudaGraphLaunch(p->gexec, st));
    return SPARC_OK;
}

template <typename T>
int set_background(sparc_plan *p, const sparc_background_t *bg, cudaStream_t st)
{
    Solver<T> &S = solver<T>(p);
    StepArgs<T> &a = S.a;
    const sparc_config_t &c = p->cfg;
    const int nz = c.nz, nx = c.nx, nzpml = c.npmlbot + c.npmltop, nhx = 2 * c.npmlhor;
    const int nbg = c.bg_per_solve ? c.nbatch : 1;
    if (!bg->stretch || !bg->unstretch || !bg->rhoinv || !bg->rho0 || !bg->gradp0_z || !bg->gradrho0_z || !bg->g ||
        !bg->fdz || !bg->az || !bg->bz || !bg->ax || !bg->bx || !bg->c2rho0)
        return fail(SPARC_ERR_ARG, "sparc_set_background: missing array");
    if (c.flows && (!bg->v0x || !bg->v0z)) return fail(SPARC_ERR_ARG, "sparc_set_background: flows need v0x, v0z");
    CK(cast_to<T>(bg->stretch, (T *)a.stretch, nz, st));
    CK(cast_to<T>(bg->rhoinv, (T *)a.rhoinv, nz, st));
    CK(cast_to<T>(bg->rho0, (T *)a.rho0, nz, st));
    CK(cast_to<T>(bg->gradp0_z, (T *)a.gp0, nz, st));
    CK(cast_to<T>(bg->gradrho0_z, (T *)a.gr0, nz, st));
    CK(cast_to<T>(bg->g, (T *)a.g, nz, st));
    CK(cast_to<T>(bg->fdz, (T *)a.fdz, (size_t)nbg * nzpml * nx, st));
    CK(cast_to<T>(bg->az, (T *)a.az, (size_t)nbg * nzpml * nx, st));
    CK(cast_to<T>(bg->bz, (T *)a.bz, (size_t)nbg * nzpml * nx, st));
    CK(cast_to<T>(bg->ax, (T *)a.ax, (size_t)nbg * nz * nhx, st));
    CK(cast_to<T>(bg->bx, (T *)a.bx, (size_t)nbg * nz * nhx, st));
    CK(cast_to<T>(bg->c2rho0, (T *)a.c2rho0, c.c2d ? (size_t)nbg * nz * nx : (size_t)nz, st));
    if (c.flows) {
        CK(cast_to<T>(bg->v0x, (T *)a.v0x, (size_t)nbg * nz * nx, st));
        CK(cast_to<T>(bg->v0z, (T *)a.v0z, (size_t)nbg * nz * nx, st));
    }
    double ut = 0.0;
    CK(cudaMemcpyAsync(&ut, bg->unstretch + (nz - 1), sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    p->unstretch_top = ut;
    p->have_bg = true;
    // unstretch_top is a launch argument: a captured graph holds a stale copy
    if (p->gexec) { cudaGraphExecDestroy(p->gexec); p->gexec = nullptr; }
    return SPARC_OK;
}

template <typename T>
int set_source(sparc_plan *p, const double *inj, const double *rows, int nrows, const double *wts, const int *idx,
               int ntab, cudaStream_t st)
{
    Solver<T> &S = solver<T>(p);
    StepArgs<T> &a = S.a;
    const int nb = p->cfg.nbatch, nx = p->cfg.nx;
    if (nrows > a.nrows) {
        void *ptr = nullptr;
        CK(cudaMalloc(&ptr, (size_t)nb * nrows * nx * sizeof(T)));
        S.allocs.push_back(ptr);
        a.src_rows = (const T *)ptr;
    }
    a.nrows = nrows;
    CK(cast_to<T>(inj, (T *)a.inj_scale, (size_t)nb * nx, st));
    CK(cast_to<T>(rows, (T *)a.src_rows, (size_t)nb * nrows * nx, st));
    if (p->d_srcw) { cudaFree(p->d_srcw); p->d_srcw = nullptr; }
    if (p->d_srcidx) { cudaFree(p->d_srcidx); p->d_srcidx = nullptr; }
    CK(cudaMalloc(&p->d_srcw, (size_t)std::max(ntab, 1) * 7 * sizeof(double)));
    CK(cudaMalloc(&p->d_srcidx, (size_t)std::max(ntab, 1) * sizeof(int)));
    CK(cudaMemcpyAsync(p->d_srcw, wts, (size_t)ntab * 7 * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(p->d_srcidx, idx, (size_t)ntab * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    a.src_w = p->d_srcw;
    a.src_idx = p->d_srcidx;
    a.ntab = ntab;
    p->have_src = true;
    // a new source invalidates a captured graph (its arguments changed)
    if (p->gexec) { cudaGraphExecDestroy(p->gexec); p->gexec = nullptr; }
    if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
    return SPARC_OK;
}

template <typename T>
int reset_state(sparc_plan *p, int time0, cudaStream_t st)
{
    Solver<T> &S = solver<T>(p);
    StepArgs<T> &a = S.a;
    const sparc_config_t &c = p->cfg;
    const size_t F = S.F;
    const int nb = c.nbatch, nzpml = c.npmlbot + c.npmltop, nhx = 2 * c.npmlhor;
    CK(cudaMemsetAsync(a.A, 0, (size_t)nb * 4 * F * sizeof(T), st));
    if (a.ALO) CK(cudaMemsetAsync(a.ALO, 0, (size_t)nb * 4 * F * sizeof(T), st));
    CK(cudaMemsetAsync(a.SV, 0, (size_t)3 * nb * 2 * F * sizeof(T), st));
    CK(cudaMemsetAsync(a.PZ, 0, (size_t)nb * 2 * nzpml * c.nx * sizeof(T), st));
    CK(cudaMemsetAsync(a.SPZ, 0, (size_t)3 * nb * 2 * nzpml * c.nx * sizeof(T), st));
    CK(cudaMemsetAsync(a.PX, 0, (size_t)nb * 2 * c.nz * nhx * sizeof(T), st));
    CK(cudaMemsetAsync(a.SPX, 0, (size_t)3 * nb * 2 * c.nz * nhx * sizeof(T), st));
    const int tm1 = time0 - 1;  // the first row pass of a step advances the counter
    CK(cudaMemcpyAsync(p->d_time, &tm1, sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    return SPARC_OK;
}

// Checkpoint layout: the step counter (16 bytes), then the persistent device state of the batch
// in this order -- A [nb][4][nz][nx], ALO (compensated FP32 plans only, same shape), PZ
// [nb][2][nzpml][nx], PX [nb][2][nz][2 npmlhor] -- all of the plan precision.  The RHS registers
// (SV, SPZ, SPX) are not part of it: stage 1 of a step reads none of them.
struct CkptPart {
    void *ptr;
    size_t bytes;
};

template <typename T>
int checkpoint_parts(sparc_plan *p, CkptPart (&parts)[4])
{
    Solver<T> &S = solver<T>(p);
    const sparc_config_t &c = p->cfg;
    const size_t nb = c.nbatch, F = S.F, nzpml = c.npmlbot + c.npmltop, nhx = 2 * c.npmlhor;
    parts[0] = {S.a.A, nb * 4 * F * sizeof(T)};
    parts[1] = {S.a.ALO, S.a.ALO ? nb * 4 * F * sizeof(T) : 0};
    parts[2] = {S.a.PZ, nb * 2 * nzpml * c.nx * sizeof(T)};
    parts[3] = {S.a.PX, nb * 2 * c.nz * nhx * sizeof(T)};
    return 4;
}

size_t checkpoint_bytes(sparc_plan *p)
{
    CkptPart parts[4];
    if (p->cfg.precision == 32) checkpoint_parts<float>(p, parts);
    else checkpoint_parts<double>(p, parts);
    size_t n = 16;
    for (auto &q : parts) n += q.bytes;
    return n;
}

bool check_cfg(const sparc_config_t *c, std::string &why)
{
    if (c->precision != 32 && c->precision != 64) { why = "precision must be 32 or 64"; return false; }
    if (c->nbatch < 1) { why = "nbatch < 1"; return false; }
    if (!fft_size_supported(c->nx)) { why = "nx not supported by the FFT (64..1024, 2^a 3^b)"; return false; }
    if (c->nx % 8) { why = "nx must be a multiple of 8 (column block width)"; return false; }
    if (c->nz < 16) { why = "nz < 16"; return false; }
    if (c->npmlbot < 1 || c->npmltop < 1 || c->npmlbot + c->npmltop >= c->nz) { why = "bad vertical PML size"; return false; }
    if (c->npmlhor < 1 || 2 * c->npmlhor >= c->nx) { why = "bad horizontal PML size"; return false; }
    if (c->k_inj < 1 || c->k_inj > c->nz - 2 || c->k_obs < 0 || c->k_obs >= c->nz) { why = "bad injection/observation row"; return false; }
    if (c->steps_out < 1) { why = "steps_out < 1"; return false; }
    if (c->filter_k0 < 1 || c->filter_k0 > 5) { why = "filter_k0 must be 1..5 (5: the reference)"; return false; }
    return true;
}

}  // namespace

// ===============================================================================================
// C ABI
// ===============================================================================================
namespace sparc {
// Error reporting for the entry points defined in other translation units (sparc_grad.cu):
// the same per-thread message sparc_last_error returns.
int report_error(int code, const std::string &msg) { return fail(code, msg); }
}  // namespace sparc

extern "C" {

const char *sparc_last_error(void) { return g_err.c_str(); }

int sparc_plan_create(const sparc_config_t *cfg, sparc_plan_t **out)
{
    if (!cfg || !out) return fail(SPARC_ERR_ARG, "sparc_plan_create: null argument");
    *out = nullptr;
    std::string why;
    if (!check_cfg(cfg, why)) return fail(SPARC_ERR_SIZE, "sparc_plan_create: " + why);
    sparc_plan *p = new sparc_plan();
    p->cfg = *cfg;
    const int lmax = 16;  // rows per z-chunk (sparc_col.cu ColCfg)
    if (!chunking(cfg->nz, lmax, p->nch, p->L) || !chunking(cfg->nz, 16, p->nch64, p->L64)) {
        delete p;
        return fail(SPARC_ERR_SIZE, "sparc_plan_create: nz too large for the column chunking");
    }
    for (int ibc = 0; ibc < 4; ibc++) {
        if (!build_ztab(cfg->nz, ibc, p->nch, p->L, p->hz[ibc]) ||
            !build_ztab(cfg->nz, ibc, p->nch64, p->L64, p->hz64[ibc])) {
            delete p;
            return fail(SPARC_ERR_SIZE, "sparc_plan_create: singular reduced system");
        }
    }
    cudaError_t e = cudaMalloc(&p->d_time, sizeof(int));
    if (e != cudaSuccess) { delete p; return fail(SPARC_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e)); }
    p->allocs.push_back(p->d_time);
    e = cudaMalloc(&p->d_err, sizeof(int));
    if (e != cudaSuccess) { sparc_plan_destroy(p); return fail(SPARC_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e)); }
    p->allocs.push_back(p->d_err);
    cudaMemset(p->d_err, 0, sizeof(int));
    int zero = -1;
    cudaMemcpy(p->d_time, &zero, sizeof(int), cudaMemcpyHostToDevice);
    for (int ibc = 0; ibc < 4; ibc++) {
        e = upload_ztab<double>(p->hz64[ibc], p->z64[ibc], p->allocs);
        if (e != cudaSuccess) { sparc_plan_destroy(p); return fail(SPARC_ERR_CUDA, std::string("tables: ") + cudaGetErrorString(e)); }
    }
    e = upload_fft<double>(cfg->nx, p->fft64, p->allocs);
    if (e != cudaSuccess) { sparc_plan_destroy(p); return fail(SPARC_ERR_CUDA, std::string("fft: ") + cudaGetErrorString(e)); }
    int rc = cfg->precision == 32 ? alloc_solver<float>(p) : alloc_solver<double>(p);
    if (rc != SPARC_OK) { std::string m = g_err; sparc_plan_destroy(p); return fail(rc, m); }
    *out = p;
    return SPARC_OK;
}

int sparc_plan_destroy(sparc_plan_t *p)
{
    if (!p) return SPARC_OK;
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    if (p->graph) cudaGraphDestroy(p->graph);
    free_solver(p->s32);
    free_solver(p->s64);
    for (void *q : p->allocs) cudaFree(q);
    if (p->d_srcw) cudaFree(p->d_srcw);
    if (p->d_srcidx) cudaFree(p->d_srcidx);
    delete p;
    return SPARC_OK;
}

int sparc_ddz(sparc_plan_t *p, const double *var, double *dvar, int n1, int ibc, const double *preset,
              const double *stretch, void *stream)
{
    if (!p || !var || !dvar || n1 < 1) return fail(SPARC_ERR_ARG, "sparc_ddz: bad argument");
    if (ibc < 0 || ibc > 3) return fail(SPARC_ERR_ARG, "sparc_ddz: ibc must be 0..3");
    CK(launch_ddz<double>(p->z64[ibc].tab, p->nch64, p->L64, var, dvar, n1, p->cfg.nz, preset, stretch, 0,
                          (cudaStream_t)stream));
    return SPARC_OK;
}

int sparc_ddzkern(sparc_plan_t *p, const double *var, double *dvar, int n1, int ibc, const double *stretch,
                  void *stream)
{
    if (!p || !var || !dvar || n1 < 1) return fail(SPARC_ERR_ARG, "sparc_ddzkern: bad argument");
    if (ibc < 0 || ibc > 1) return fail(SPARC_ERR_ARG, "sparc_ddzkern: ibc must be 0 or 1");
    CK(launch_ddz<double>(p->z64[ibc].tab, p->nch64, p->L64, var, dvar, n1, p->cfg.nz, nullptr, stretch, 1,
                          (cudaStream_t)stream));
    return SPARC_OK;
}

int sparc_ddx(sparc_plan_t *p, const double *var, double *dvar, int nrows, double stretchx, void *stream)
{
    if (!p || !var || !dvar || nrows < 0) return fail(SPARC_ERR_ARG, "sparc_ddx: bad argument");
    CK(launch_ddx<double>(var, dvar, nrows, p->cfg.nx, stretchx, p->fft64.twr, p->fft64.twi, p->fft64.kap,
                          (cudaStream_t)stream));
    return SPARC_OK;
}

int sparc_set_background(sparc_plan_t *p, const sparc_background_t *bg, void *stream)
{
    if (!p || !bg) return fail(SPARC_ERR_ARG, "sparc_set_background: null argument");
    return p->cfg.precision == 32 ? set_background<float>(p, bg, (cudaStream_t)stream)
                                  : set_background<double>(p, bg, (cudaStream_t)stream);
}

int sparc_set_source(sparc_plan_t *p, const double *inj_scale, const double *rows, int nrows, const double *wts,
                     const int *idx, int ntab, void *stream)
{
    if (!p || !inj_scale || !rows || nrows < 1 || !wts || !idx || ntab < 1)
        return fail(SPARC_ERR_ARG, "sparc_set_source: bad argument");
    return p->cfg.precision == 32 ? set_source<float>(p, inj_scale, rows, nrows, wts, idx, ntab, (cudaStream_t)stream)
                                  : set_source<double>(p, inj_scale, rows, nrows, wts, idx, ntab, (cudaStream_t)stream);
}

int sparc_reset_state(sparc_plan_t *p, int time0, void *stream)
{
    if (!p) return fail(SPARC_ERR_ARG, "sparc_reset_state: null plan");
    return p->cfg.precision == 32 ? reset_state<float>(p, time0, (cudaStream_t)stream)
                                  : reset_state<double>(p, time0, (cudaStream_t)stream);
}

int sparc_forward(sparc_plan_t *p, int nsteps, double flow_sign, void *seis, void *snaps, int nrec_cap,
                  int use_graph, void *stream)
{
    if (!p || nsteps < 0 || nrec_cap < 0) return fail(SPARC_ERR_ARG, "sparc_forward: bad argument");
    if (!p->have_bg || !p->have_src) return fail(SPARC_ERR_STATE, "sparc_forward: background and source must be set first");
    if (nrec_cap > 0 && !seis && !snaps) return fail(SPARC_ERR_ARG, "sparc_forward: nrec_cap without outputs");
    return p->cfg.precision == 32
               ? run_forward<float>(p, nsteps, flow_sign, seis, snaps, 0, nrec_cap, use_graph, (cudaStream_t)stream)
               : run_forward<double>(p, nsteps, flow_sign, seis, snaps, 0, nrec_cap, use_graph, (cudaStream_t)stream);
}

int sparc_forward_window(sparc_plan_t *p, int nsteps, double flow_sign, void *seis, void *snaps, int rec0,
                         int nrec_cap, int use_graph, void *stream)
{
    if (!p || nsteps < 0 || nrec_cap < 0 || rec0 < 0) return fail(SPARC_ERR_ARG, "sparc_forward_window: bad argument");
    if (!p->have_bg || !p->have_src)
        return fail(SPARC_ERR_STATE, "sparc_forward_window: background and source must be set first");
    if (nrec_cap > 0 && !seis && !snaps) return fail(SPARC_ERR_ARG, "sparc_forward_window: nrec_cap without outputs");
    return p->cfg.precision == 32
               ? run_forward<float>(p, nsteps, flow_sign, seis, snaps, rec0, nrec_cap, use_graph, (cudaStream_t)stream)
               : run_forward<double>(p, nsteps, flow_sign, seis, snaps, rec0, nrec_cap, use_graph, (cudaStream_t)stream);
}

size_t sparc_checkpoint_bytes(const sparc_plan_t *p)
{
    return p ? checkpoint_bytes(const_cast<sparc_plan_t *>(p)) : 0;
}

int sparc_checkpoint_save(sparc_plan_t *p, void *dst, void *stream)
{
    if (!p || !dst) return fail(SPARC_ERR_ARG, "sparc_checkpoint_save: bad argument");
    if ((reinterpret_cast<uintptr_t>(dst) & 15) != 0) return fail(SPARC_ERR_ARG, "sparc_checkpoint_save: dst not 16-byte aligned");
    CkptPart parts[4];
    if (p->cfg.precision == 32) checkpoint_parts<float>(p, parts);
    else checkpoint_parts<double>(p, parts);
    cudaStream_t st = (cudaStream_t)stream;
    char *d = static_cast<char *>(dst);
    CK(cudaMemcpyAsync(d, p->d_time, sizeof(int), cudaMemcpyDeviceToDevice, st));
    d += 16;
    for (auto &q : parts) {
        if (q.bytes) CK(cudaMemcpyAsync(d, q.ptr, q.bytes, cudaMemcpyDeviceToDevice, st));
        d += q.bytes;
    }
    return SPARC_OK;
}

int sparc_checkpoint_load(sparc_plan_t *p, const void *src, void *stream)
{
    if (!p || !src) return fail(SPARC_ERR_ARG, "sparc_checkpoint_load: bad argument");
    if ((reinterpret_cast<uintptr_t>(src) & 15) != 0) return fail(SPARC_ERR_ARG, "sparc_checkpoint_load: src not 16-byte aligned");
    CkptPart parts[4];
    if (p->cfg.precision == 32) checkpoint_parts<float>(p, parts);
    else checkpoint_parts<double>(p, parts);
    cudaStream_t st = (cudaStream_t)stream;
    const char *d = static_cast<const char *>(src);
    CK(cudaMemcpyAsync(p->d_time, d, sizeof(int), cudaMemcpyDeviceToDevice, st));
    d += 16;
    for (auto &q : parts) {
        if (q.bytes) CK(cudaMemcpyAsync(q.ptr, d, q.bytes, cudaMemcpyDeviceToDevice, st));
        d += q.bytes;
    }
    return SPARC_OK;
}

int sparc_profile_passes(sparc_plan_t *p, int nsteps, double *ms, void *stream)
{
    if (!p || !ms || nsteps < 1) return fail(SPARC_ERR_ARG, "sparc_profile_passes: bad argument");
    if (!p->have_bg || !p->have_src) return fail(SPARC_ERR_STATE, "sparc_profile_passes: background and source first");
    return p->cfg.precision == 32 ? profile_passes<float>(p, nsteps, ms, (cudaStream_t)stream)
                                  : profile_passes<double>(p, nsteps, ms, (cudaStream_t)stream);
}

int sparc_get_state(sparc_plan_t *p, void *dst, void *stream)
{
    if (!p || !dst) return fail(SPARC_ERR_ARG, "sparc_get_state: bad argument");
    const size_t es = p->cfg.precision == 32 ? 4 : 8;
    const void *src = p->cfg.precision == 32 ? (const void *)p->s32.a.A : (const void *)p->s64.a.A;
    CK(cudaMemcpyAsync(dst, src, (size_t)p->cfg.nbatch * 4 * p->cfg.nx * p->cfg.nz * es, cudaMemcpyDeviceToDevice,
                       (cudaStream_t)stream));
    return SPARC_OK;
}

int sparc_set_state(sparc_plan_t *p, const void *src, void *stream)
{
    if (!p || !src) return fail(SPARC_ERR_ARG, "sparc_set_state: bad argument");
    const size_t es = p->cfg.precision == 32 ? 4 : 8;
    void *dst = p->cfg.precision == 32 ? (void *)p->s32.a.A : (void *)p->s64.a.A;
    const size_t bytes = (size_t)p->cfg.nbatch * 4 * p->cfg.nx * p->cfg.nz * es;
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    if (p->cfg.precision == 32 && p->s32.a.ALO) CK(cudaMemsetAsync(p->s32.a.ALO, 0, bytes, (cudaStream_t)stream));
    return SPARC_OK;
}

int sparc_check_state(sparc_plan_t *p, double *norms, void *stream)
{
    if (!p || !norms) return fail(SPARC_ERR_ARG, "sparc_check_state: bad argument");
    const int nb = p->cfg.nbatch;
    const size_t F = (size_t)p->cfg.nx * p->cfg.nz;
    cudaStream_t st = (cudaStream_t)stream;
    double *d = nullptr;
    CK(cudaMallocAsync((void **)&d, nb * sizeof(double), st));
    if (p->cfg.precision == 32) vz_norm_kernel<float><<<nb, 256, 0, st>>>(p->s32.a.A, F, d);
    else vz_norm_kernel<double><<<nb, 256, 0, st>>>(p->s64.a.A, F, d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(norms, d, nb * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("sparc_check_state: ") + cudaGetErrorString(e));
    bool bad = false;
    for (int b = 0; b < nb; b++) {
        norms[b] = std::sqrt(norms[b]);
        if (!std::isfinite(norms[b])) bad = true;
    }
    int derr = 0;
    CK(cudaMemcpy(&derr, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (derr == SPARC_DEV_ERR_TMA_TIMEOUT)
        return fail(SPARC_ERR_TIMEOUT, "sparc_check_state: a bounded wait for staged column tiles gave up");
    if (derr == SPARC_DEV_ERR_STAGE_WAIT)
        return fail(SPARC_ERR_TIMEOUT, "sparc_check_state: a row pass gave up waiting for its solve's column tiles");
    if (derr == SPARC_DEV_ERR_TMA_ALIGN)
        return fail(SPARC_ERR_CUDA, "sparc_check_state: shared memory of the column pass not 128-byte aligned for TMA");
    if (bad) return fail(SPARC_ERR_NONFINITE, "sparc_check_state: non-finite v_z (the solve diverged)");
    return SPARC_OK;
}

int sparc_plan_describe(const sparc_plan_t *p, char *buf, int len)
{
    if (!p || !buf || len < 1) return fail(SPARC_ERR_ARG, "sparc_plan_describe: bad argument");
    std::string col, end;
    if (p->cfg.precision == 32) {
        const Solver<float> &S = p->s32;
        if (S.band_tma_R) col = "col_band_tma_kernel<" + std::to_string(S.band_tma_R) + ">";
        else if (S.band_R)
            col = "col_band_kernel<" + std::to_string(S.band_cw) + "," + std::to_string(S.band_R) + "," +
                  (col_band_specialised(p->cfg.nx, p->cfg.nz, S.band_cw, S.band_R)
                       ? std::to_string(p->cfg.nx) + "," + std::to_string(p->cfg.nz)
                       : std::string("0,0")) +
                  (S.have_maps32 ? ",1>" : ",0>");
        else if (S.have_maps && p->cfg.column_impl == 1) col = "col_stage_tma_kernel<float>";
        else col = "col_stage_kernel<float," + std::to_string(S.a.colw) + ">";
        end = S.a.ALO ? (S.end_stream ? "end_step_comp_kernel" : "end_step_kernel<float>")
                      : (S.have_maps && p->cfg.column_impl == 1) ? "end_step_tma_kernel<float>"
                      : S.end_stream ? "end_step_stream_kernel<float>" : "end_step_kernel<float>";
    } else {
        const Solver<double> &S = p->s64;
        col = (S.have_maps && p->cfg.column_impl == 1) ? "col_stage_tma_kernel<double>"
                                                        : "col_stage_kernel<double," + std::to_string(S.a.colw) + ">";
        end = (S.have_maps && p->cfg.column_impl == 1) ? "end_step_tma_kernel<double>"
              : S.end_stream ? "end_step_stream_kernel<double>" : "end_step_kernel<double>";
    }
    const bool overlap = p->cfg.precision == 32 && p->s32.a.tile_cnt != nullptr;
    const std::string d = "column=" + col + " end=" + end + " stage_overlap=" + (overlap ? "1" : "0");
    std::snprintf(buf, (size_t)len, "%s", d.c_str());
    return SPARC_OK;
}

int sparc_get_time(sparc_plan_t *p, int *time, void *stream)
{
    if (!p || !time) return fail(SPARC_ERR_ARG, "sparc_get_time: bad argument");
    int t = 0;
    CK(cudaMemcpyAsync(&t, p->d_time, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    *time = t + 1;
    return SPARC_OK;
}

}  // extern "C"

namespace {
template <typename T>
KAccArgs<T> kacc_args(sparc_plan *p, const void *fsn, int nfwd, const void *adj, long long adj_stride, int jf,
                      double *out)
{
    Solver<T> &S = solver<T>(p);
    const sparc_config_t &c = p->cfg;
    const size_t F = S.F;
    KAccArgs<T> k{};
    k.nx = c.nx; k.nz = c.nz; k.nb = c.nbatch;
    k.fsn = (const T *)fsn;
    k.fbase = (long long)jf * 6 * F;
    k.fstride = (long long)nfwd * 6 * F;
    k.adj = (const T *)adj;
    k.astride = adj_stride;
    k.out = out;
    k.work = nullptr;
    k.stretch = S.a.stretch;
    k.twr = S.fft.twr; k.twi = S.fft.twi; k.kap = S.fft.kap;
    k.stretchx = (T)c.stretchx;
    k.z1 = S.z[1].tab;
    k.nch = p->nch; k.L = p->L;
    k.colw = S.a.colw;
    return k;
}

template <typename T>
int kernels_impl(sparc_plan *p, const void *fsn, int nfwd, const void *adj, long long adj_stride, int jf, double *out,
                 cudaStream_t st)
{
    Solver<T> &S = solver<T>(p);
    const sparc_config_t &c = p->cfg;
    const size_t F = S.F;
    if (!S.work) {
        void *ptr = nullptr;
        CK(cudaMalloc(&ptr, (size_t)c.nbatch * 4 * F * sizeof(T)));
        S.allocs.push_back(ptr);
        S.work = (T *)ptr;
    }
    KAccArgs<T> k{};
    k.nx = c.nx; k.nz = c.nz; k.nb = c.nbatch;
    k.fsn = (const T *)fsn;
    k.fbase = (long long)jf * 6 * F;
    k.fstride = (long long)nfwd * 6 * F;
    k.adj = (const T *)adj;
    k.astride = adj_stride;
    k.out = out;
    k.work = S.work;
    k.stretch = S.a.stretch;
    k.twr = S.fft.twr; k.twi = S.fft.twi; k.kap = S.fft.kap;
    k.stretchx = (T)c.stretchx;
    k.z1 = S.z[1].tab;
    k.nch = p->nch; k.L = p->L;
    k.colw = S.a.colw;
    CK(launch_kacc<T>(k, st));
    return SPARC_OK;
}
}  // namespace

extern "C" {

int sparc_kernels(sparc_plan_t *p, const void *fsn, int nfwd, const void *asn, int nadj, int npair, double *out,
                  void *stream)
{
    if (!p || !fsn || !asn || !out || nfwd < 1 || nadj < 1 || npair < 0 || npair > nfwd || npair > nadj)
        return fail(SPARC_ERR_ARG, "sparc_kernels: bad argument");
    if (!p->have_bg) return fail(SPARC_ERR_STATE, "sparc_kernels: background must be set first");
    const size_t F = (size_t)p->cfg.nx * p->cfg.nz;
    const size_t es = p->cfg.precision == 32 ? 4 : 8;
    for (int j = 0; j < npair; j++) {
        const int ja = nadj - 1 - j;
        const char *adj = (const char *)asn + ((size_t)ja * 6 * F + 2 * F) * es;
        int rc = p->cfg.precision == 32
                     ? kernels_impl<float>(p, fsn, nfwd, adj, (long long)nadj * 6 * F, j, out, (cudaStream_t)stream)
                     : kernels_impl<double>(p, fsn, nfwd, adj, (long long)nadj * 6 * F, j, out, (cudaStream_t)stream);
        if (rc != SPARC_OK) return rc;
    }
    return SPARC_OK;
}

int sparc_kernels_accumulate(sparc_plan_t *p, const void *fsn, int nfwd, int jf, double *out, void *stream)
{
    if (!p || !fsn || !out || nfwd < 1 || jf < 0 || jf >= nfwd)
        return fail(SPARC_ERR_ARG, "sparc_kernels_accumulate: bad argument");
    if (!p->have_bg) return fail(SPARC_ERR_STATE, "sparc_kernels_accumulate: background must be set first");
    const size_t F = (size_t)p->cfg.nx * p->cfg.nz;
    if (p->cfg.precision == 32)
        return kernels_impl<float>(p, fsn, nfwd, p->s32.a.A + 2 * F, (long long)4 * F, jf, out, (cudaStream_t)stream);
    return kernels_impl<double>(p, fsn, nfwd, p->s64.a.A + 2 * F, (long long)4 * F, jf, out, (cudaStream_t)stream);
}

int sparc_adjoint(sparc_plan_t *p, const void *fsn, int nfwd, int nsteps, double *out, void *stream)
{
    if (!p || !fsn || !out || nfwd < 1 || nsteps < 1) return fail(SPARC_ERR_ARG, "sparc_adjoint: bad argument");
    if (!p->have_bg || !p->have_src) return fail(SPARC_ERR_STATE, "sparc_adjoint: background and source must be set first");
    const int so = p->cfg.steps_out;
    if (so < 1 || 1 + (long long)(nfwd - 1) * so > nsteps)
        return fail(SPARC_ERR_ARG, "sparc_adjoint: nfwd records need 1 + (nfwd - 1) * steps_out <= nsteps");
    const cudaStream_t st = (cudaStream_t)stream;
    const bool f32 = p->cfg.precision == 32;
    const size_t F = (size_t)p->cfg.nx * p->cfg.nz;
    int rc = f32 ? reset_state<float>(p, 0, st) : reset_state<double>(p, 0, st);
    if (rc != SPARC_OK) return rc;
    CK(cudaMemsetAsync(out, 0, (size_t)p->cfg.nbatch * 4 * F * sizeof(double), st));
    // adjoint record ja (written at time ja * steps_out, the first after one step) pairs with
    // forward record nfwd - 1 - ja (kernels.f90:215, 258)
    int done = 0;
    for (int ja = 0; ja < nfwd; ja++) {
        const int n = ja == 0 ? 1 : so;
        rc = f32 ? run_forward<float>(p, n, -1.0, nullptr, nullptr, 0, 0, 1, st)
                 : run_forward<double>(p, n, -1.0, nullptr, nullptr, 0, 0, 1, st);
        if (rc != SPARC_OK) return rc;
        done += n;
        const int jf = nfwd - 1 - ja;
        rc = f32 ? kernels_impl<float>(p, fsn, nfwd, p->s32.a.A + 2 * F, (long long)4 * F, jf, out, st)
                 : kernels_impl<double>(p, fsn, nfwd, p->s64.a.A + 2 * F, (long long)4 * F, jf, out, st);
        if (rc != SPARC_OK) return rc;
    }
    if (nsteps > done) {
        rc = f32 ? run_forward<float>(p, nsteps - done, -1.0, nullptr, nullptr, 0, 0, 1, st)
                 : run_forward<double>(p, nsteps - done, -1.0, nullptr, nullptr, 0, 0, 1, st);
        if (rc != SPARC_OK) return rc;
    }
    return SPARC_OK;
}

int sparc_kernels_accumulate_static(sparc_plan_t *p, const void *fsn, int nfwd, int jf, double *out, void *stream)
{
    if (!p || !fsn || !out || nfwd < 1 || jf < 0 || jf >= nfwd)
        return fail(SPARC_ERR_ARG, "sparc_kernels_accumulate_static: bad argument");
    if (!p->have_bg) return fail(SPARC_ERR_STATE, "sparc_kernels_accumulate_static: background must be set first");
    const size_t F = (size_t)p->cfg.nx * p->cfg.nz;
    std::string err;
    int rc;
    if (p->cfg.precision == 32)
        rc = kernels_accumulate_static_impl<float>(kacc_args<float>(p, fsn, nfwd, p->s32.a.A + 2 * F, (long long)4 * F, jf, out),
                                                   (cudaStream_t)stream, err);
    else
        rc = kernels_accumulate_static_impl<double>(kacc_args<double>(p, fsn, nfwd, p->s64.a.A + 2 * F, (long long)4 * F, jf, out),
                                                    (cudaStream_t)stream, err);
    if (rc != SPARC_OK) return fail(rc, err);
    return SPARC_OK;
}

// Host evaluation of the partitioned compact-derivative tables (FP64), the same algebra the
// device code applies; used to validate the tables without a GPU.
int sparc_zband_host(int nz, int ibc, const double *b, double *x, const double *preset, int n1, double *band_err)
{
    if (!b || !x || n1 < 1 || ibc < 1 || ibc > 3) return fail(SPARC_ERR_ARG, "sparc_zband_host: bad argument");
    int nch, L;  // chunk factors are not used by the band form
    if (!chunking(nz, std::max(16, (nz + 19) / 20), nch, L)) return fail(SPARC_ERR_SIZE, "sparc_zband_host: bad size");
    HostZTab t;
    HostBand h;
    if (!build_ztab(nz, ibc, nch, L, t) || !build_band(t, h)) return fail(SPARC_ERR_SIZE, "sparc_zband_host: no band form");
    if (band_err) *band_err = h.err;
    zband_host(t, h, b, x, preset, n1);
    return SPARC_OK;
}

int sparc_zsolve_host(int nz, int ibc, int lmax, const double *b, double *x, const double *preset, int n1)
{
    if (!b || !x || n1 < 1 || ibc < 0 || ibc > 3) return fail(SPARC_ERR_ARG, "sparc_zsolve_host: bad argument");
    int nch, L;
    if (!chunking(nz, lmax, nch, L)) return fail(SPARC_ERR_SIZE, "sparc_zsolve_host: bad chunking");
    HostZTab t;
    if (!build_ztab(nz, ibc, nch, L, t)) return fail(SPARC_ERR_SIZE, "sparc_zsolve_host: singular");
    zsolve_host(t, b, x, preset, n1);
    return SPARC_OK;
}

}  // extern "C"

// =============================================================================================
// 3-D plans (option 16): buffers, one time step as a launch sequence, the C ABI.
// =============================================================================================
namespace {

template <typename T>
struct Plan3 {
    std::vector<void *> allocs;
    T *A = nullptr, *SCR = nullptr, *X = nullptr, *PV = nullptr, *SPV = nullptr, *PSI = nullptr;
    T *D1 = nullptr, *D2 = nullptr, *D3 = nullptr, *PP = nullptr, *RHO = nullptr, *GX = nullptr, *GY = nullptr,
      *GZ = nullptr;
    T *prof = nullptr, *v0 = nullptr, *pat = nullptr;
    T *ADJ = nullptr;  // adjoint forcing of the current step at the observation level [nb][ny][nx]
    DevZ<T> z[2];  // ibc 0, 1
    DevFFT<T> fx, fy;
    S3Bg<T> bg{};
    const T *stretch = nullptr;
};

}  // namespace

struct sparc3d_plan {
    sparc3d_config_t cfg{};
    int nch = 0, L = 0;
    HostZTab hz[2];
    Plan3<float> s32;
    Plan3<double> s64;
    std::vector<double> amp;
    // kernel-mode adjoint source (sparc3d_set_adjoint_source): the caller's device slices
    // [nb][nrows][ny][nx] and the per-step LAGRANGE_INTERP table
    bool adj = false;
    const double *adj_rows = nullptr;
    int adj_nrows = 0;
    double adj_scale = 0.0;
    std::vector<double> adj_w;
    std::vector<int> adj_idx;
    int time = 0;
    bool have_bg = false;
    long long F = 0, P = 0, nxy = 0;
};

namespace {

template <typename T>
Plan3<T> &plan3(sparc3d_plan *p);
template <>
Plan3<float> &plan3<float>(sparc3d_plan *p) { return p->s32; }
template <>
Plan3<double> &plan3<double>(sparc3d_plan *p) { return p->s64; }

template <typename T>
int alloc_plan3(sparc3d_plan *p)
{
    Plan3<T> &S = plan3<T>(p);
    const sparc3d_config_t &c = p->cfg;
    const long long F = p->F, P = p->P, nz = c.nz, npml = c.npmlbot + c.npmltop;
    struct Req { T **ptr; size_t n; };
    std::vector<Req> reqs = {
        {&S.A, (size_t)6 * F}, {&S.SCR, (size_t)6 * F}, {&S.X, (size_t)6 * F},
        {&S.PV, (size_t)2 * P}, {&S.SPV, (size_t)2 * P}, {&S.PSI, (size_t)2 * P},
        {&S.D1, (size_t)F}, {&S.D2, (size_t)F}, {&S.D3, (size_t)F}, {&S.PP, (size_t)F}, {&S.RHO, (size_t)F},
        {&S.GX, (size_t)F}, {&S.GY, (size_t)F}, {&S.GZ, (size_t)F},
        {&S.prof, (size_t)(8 * nz + 2 * npml)}, {&S.v0, c.flows ? (size_t)3 * nz * p->nxy : 1},
        {&S.pat, (size_t)c.nbatch * p->nxy}, {&S.ADJ, (size_t)c.nbatch * p->nxy},
    };
    for (auto &r : reqs) {
        void *ptr = nullptr;
        const size_t bytes = std::max<size_t>(r.n, 1) * sizeof(T);
        cudaError_t e = cudaMalloc(&ptr, bytes);
        if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        S.allocs.push_back(ptr);
        e = cudaMemset(ptr, 0, bytes);
        if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("cudaMemset: ") + cudaGetErrorString(e));
        *r.ptr = (T *)ptr;
    }
    for (int ibc = 0; ibc < 2; ibc++) {
        cudaError_t e = upload_ztab<T>(p->hz[ibc], S.z[ibc], S.allocs);
        if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("table upload: ") + cudaGetErrorString(e));
    }
    cudaError_t e = upload_fft<T>(c.nx, S.fx, S.allocs);
    if (e == cudaSuccess) e = upload_fft<T>(c.ny, S.fy, S.allocs);
    if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("fft tables: ") + cudaGetErrorString(e));
    T *q = S.prof;
    S.stretch = q; q += nz;
    S.bg.rhoinv = q; q += nz;
    S.bg.rho0 = q; q += nz;
    S.bg.c2rho0 = q; q += nz;
    S.bg.gradp0_z = q; q += nz;
    S.bg.gradrho0_z = q; q += nz;
    S.bg.g = q; q += nz;
    S.bg.source_dep = q; q += nz;
    S.bg.az = q; q += npml;
    S.bg.bz = q;
    return SPARC_OK;
}

template <typename T>
void free_plan3(Plan3<T> &S)
{
    for (void *q : S.allocs) cudaFree(q);
    S.allocs.clear();
}

// ddxyz (derivatives.f90:175-305) pieces on fields [nz][nb][ny][nx]
template <typename T>
cudaError_t d3x(sparc3d_plan *p, const T *v, T *dv, cudaStream_t st)
{
    const Plan3<T> &S = plan3<T>(p);
    const sparc3d_config_t &c = p->cfg;
    return launch_ddx<T>(v, dv, c.nz * c.nbatch * c.ny, c.nx, (T)c.stretchx, S.fx.twr, S.fx.twi, S.fx.kap, st);
}
template <typename T>
cudaError_t d3y(sparc3d_plan *p, const T *v, T *dv, cudaStream_t st)
{
    const Plan3<T> &S = plan3<T>(p);
    const sparc3d_config_t &c = p->cfg;
    return launch_ddy<T>(v, dv, c.nz * c.nbatch, c.nx, c.ny, (T)c.stretchy, S.fy.twr, S.fy.twi, S.fy.kap, st);
}
template <typename T>
cudaError_t d3z(sparc3d_plan *p, const T *v, T *dv, int ibc, cudaStream_t st, int filter = 0)
{
    const Plan3<T> &S = plan3<T>(p);
    return launch_ddz<T>(S.z[ibc].tab, p->nch, p->L, v, dv, (int)(p->cfg.nbatch * p->nxy), p->cfg.nz, nullptr,
                         S.stretch, filter, st);
}

// MP_FLOWS_PML_3D_DISPL (displacement.f90:377-477) on X (psi: PSI), into SCR and SPV.
template <typename T>
cudaError_t rhs3(sparc3d_plan *p, const T *X, const T *PSI, T amp, cudaStream_t st)
{
    Plan3<T> &S = plan3<T>(p);
    const sparc3d_config_t &c = p->cfg;
    const long long F = p->F, P = p->P;
    const S3Args a{c.nx, c.ny, c.nz, c.nbatch, c.npmlbot, c.npmltop, c.k_src, c.flows, p->nxy};
    cudaError_t e;
#define R3(call) do { e = (call); if (e != cudaSuccess) return e; } while (0)
    R3(d3x<T>(p, X, S.D1, st));
    R3(d3y<T>(p, X + F, S.D2, st));
    R3(d3z<T>(p, X + 2 * F, S.D3, 1, st));
    R3(launch_s3_div<T>(a, S.bg, S.D1, S.D2, S.D3, X + 2 * F, PSI, S.SPV, S.PP, S.RHO, st));
    R3(d3x<T>(p, S.PP, S.GX, st));
    R3(d3y<T>(p, S.PP, S.GY, st));
    R3(d3z<T>(p, S.PP, S.GZ, 0, st));
    if (c.flows) {
        const long long q = (long long)c.nz * p->nxy;
        for (int comp = 0; comp < 3; comp++) {
            const T *v = X + (3 + comp) * F;
            R3(d3x<T>(p, v, S.D1, st));
            R3(d3y<T>(p, v, S.D2, st));
            R3(d3z<T>(p, v, S.D3, 1, st));
            R3(launch_s3_adv<T>(a, S.D1, S.D2, S.D3, S.v0, S.v0 + q, S.v0 + 2 * q, S.SCR + (3 + comp) * F, st));
        }
    }
    R3(launch_s3_rhs<T>(a, S.bg, X, S.SCR, S.GX, S.GY, S.GZ, PSI + P, S.SPV + P, S.RHO, S.pat, amp,
                        p->adj ? S.ADJ : nullptr, c.k_obs, st));
#undef R3
    return cudaSuccess;
}

// STEP (step.f90:43-119) and the record of TIMESTEPPING (driver.f90:388-409).
// Kernel-stage record of the current state into snap ([5][F], see s3_record_kernel).
template <typename T>
cudaError_t record3(sparc3d_plan *p, T *snap, cudaStream_t st)
{
    Plan3<T> &S = plan3<T>(p);
    const long long F = p->F;
    cudaError_t e;
    if ((e = d3x<T>(p, S.A, S.D1, st)) != cudaSuccess) return e;
    if ((e = d3y<T>(p, S.A + F, S.D2, st)) != cudaSuccess) return e;
    if ((e = d3z<T>(p, S.A + 2 * F, S.D3, 1, st, 1)) != cudaSuccess) return e;
    return launch_s3_record<T>(F, S.D1, S.D2, S.D3, S.A, S.SCR, snap, st);
}

template <typename T>
cudaError_t step3(sparc3d_plan *p, T *seis, int cap, int &nrec, cudaStream_t st, T *snaps = nullptr, int rec0 = 0,
                  int snap_cap = 0)
{
    Plan3<T> &S = plan3<T>(p);
    const sparc3d_config_t &c = p->cfg;
    const long long F = p->F, P = p->P;
    const S3Args a{c.nx, c.ny, c.nz, c.nbatch, c.npmlbot, c.npmltop, c.k_src, c.flows, p->nxy};
    const T amp = (T)(p->time >= 0 && p->time < (int)p->amp.size() ? p->amp[p->time] : 0.0);
    cudaError_t e;
    if (p->adj) {  // this step's adjoint forcing (the same in all five stages)
        const long long lvl = (long long)c.nbatch * p->nxy;
        const int t = p->time;
        if (t >= 0 && t < (int)p->adj_idx.size()) {
            S3Lagr w;
            for (int j = 0; j < 7; j++) w.w[j] = p->adj_w[(size_t)t * 7 + j];
            e = launch_s3_adjsrc<T>(lvl, p->nxy, p->adj_rows, p->adj_nrows, p->adj_idx[t], w, p->adj_scale, S.ADJ, st);
        } else {
            e = cudaMemsetAsync(S.ADJ, 0, lvl * sizeof(T), st);
        }
        if (e != cudaSuccess) return e;
    }
    for (int s = 0; s < 5; s++) {
        const T *X = S.A, *PSI = S.PV;
        if (s > 0) {
            e = launch_s3_stage_in<T>(6 * F, S.A, S.SCR, S.X, (T)c.betas[s], 2 * P, S.PV, S.SPV, S.PSI, st);
            if (e != cudaSuccess) return e;
            X = S.X;
            PSI = S.PSI;
        }
        e = rhs3<T>(p, X, PSI, amp, st);
        if (e != cudaSuccess) return e;
    }
    const int filter = (c.filter_every == 2 && (p->time + 1) % 2 == 0) ? 1 : 0;
    e = launch_s3_end<T>(a, S.A, S.SCR, (T)c.deltat, filter, S.PV, S.SPV, st);
    if (e != cudaSuccess) return e;
    if (c.steps_out > 0 && p->time % c.steps_out == 0) {
        if (seis && nrec < cap) {
            const size_t lvl = (size_t)c.nbatch * p->nxy;
            e = cudaMemcpyAsync(seis + (size_t)nrec * lvl, S.A + 5 * F + (size_t)c.k_obs * lvl, lvl * sizeof(T),
                                cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) return e;
        }
        nrec++;
        const int j = p->time / c.steps_out - rec0;  // kernel-stage record j of the window
        if (snaps && j >= 0 && j < snap_cap) {
            e = record3<T>(p, snaps + (size_t)j * 5 * F, st);
            if (e != cudaSuccess) return e;
        }
    }
    p->time++;
    return cudaSuccess;
}

// One record pair of the 3-D kernel integral, the plan's current state as the adjoint fields.
template <typename T>
cudaError_t kacc3(sparc3d_plan *p, const T *snap, double *out, cudaStream_t st)
{
    Plan3<T> &S = plan3<T>(p);
    const long long F = p->F;
    cudaError_t e;
#define K3(call) do { e = (call); if (e != cudaSuccess) return e; } while (0)
    K3(d3x<T>(p, S.A + 3 * F, S.D1, st));
    K3(d3y<T>(p, S.A + 4 * F, S.D2, st));
    K3(d3z<T>(p, S.A + 5 * F, S.D3, 1, st, 1));
    K3(launch_s3_kacc_div<T>(F, S.D1, S.D2, S.D3, snap, out, st));
    for (int j = 0; j < 3; j++) {
        const T *vf = snap + (size_t)(1 + j) * F;
        K3(d3x<T>(p, vf, S.D1, st));
        K3(d3y<T>(p, vf, S.D2, st));
        K3(d3z<T>(p, vf, S.D3, 1, st, 1));
        K3(launch_s3_kacc_v<T>(F, S.D1, S.D2, S.D3, S.A + (size_t)(3 + j) * F, out, st));
    }
#undef K3
    return cudaSuccess;
}

bool check_cfg3(const sparc3d_config_t *c, std::string &why)
{
    if (c->precision != 32 && c->precision != 64) { why = "precision must be 32 or 64"; return false; }
    if (c->nbatch < 1) { why = "nbatch must be >= 1"; return false; }
    if (!fft_size_supported(c->nx) || c->nx % 16) { why = "nx not in the FFT table or not a multiple of 16"; return false; }
    if (!ddy_size_supported(c->ny)) { why = "ny not in 64, 128, 192, 256, 384, 512"; return false; }
    if (c->precision == 64 && c->ny > 384) { why = "ny > 384 needs more shared memory than a block has in FP64"; return false; }
    if (c->npmlbot < 5 || c->npmltop < 5) { why = "npmlbot and npmltop must be >= 5 (filter window)"; return false; }
    if (c->nz < c->npmlbot + c->npmltop + 1 || c->nz < 11) { why = "nz too small for the PML layers"; return false; }
    if (c->k_src < 0 || c->k_src >= c->nz || c->k_obs < 0 || c->k_obs >= c->nz) { why = "k_src / k_obs out of range"; return false; }
    if (c->filter_every != 0 && c->filter_every != 2) { why = "filter_every must be 0 or 2"; return false; }
    if ((long long)c->nz * c->nbatch * c->ny > 2147483647LL || (long long)c->nz * c->nbatch > 65535) {
        why = "nz * nbatch * ny (x-pass rows) or nz * nbatch (y-pass planes) too large";
        return false;
    }
    return true;
}

template <typename T>
int set_bg3(sparc3d_plan *p, const sparc3d_background_t *bg, cudaStream_t st)
{
    Plan3<T> &S = plan3<T>(p);
    const sparc3d_config_t &c = p->cfg;
    const int nz = c.nz, npml = c.npmlbot + c.npmltop;
    const double *prof[8] = {bg->stretch, bg->rhoinv, bg->rho0, bg->c2rho0, bg->gradp0_z, bg->gradrho0_z, bg->g,
                             bg->source_dep};
    for (int i = 0; i < 8; i++) CK(cast_to<T>(prof[i], S.prof + (size_t)i * nz, nz, st));
    CK(cast_to<T>(bg->az, S.prof + (size_t)8 * nz, npml, st));
    CK(cast_to<T>(bg->bz, S.prof + (size_t)8 * nz + npml, npml, st));
    if (c.flows) {
        const size_t q = (size_t)nz * p->nxy;
        CK(cast_to<T>(bg->v0x, S.v0, q, st));
        CK(cast_to<T>(bg->v0y, S.v0 + q, q, st));
        CK(cast_to<T>(bg->v0z, S.v0 + 2 * q, q, st));
    }
    return SPARC_OK;
}

}  // namespace

extern "C" {

int sparc3d_plan_create(const sparc3d_config_t *cfg, sparc3d_plan_t **out)
{
    if (!cfg || !out) return fail(SPARC_ERR_ARG, "sparc3d_plan_create: null argument");
    *out = nullptr;
    std::string why;
    if (!check_cfg3(cfg, why)) return fail(SPARC_ERR_SIZE, "sparc3d_plan_create: " + why);
    sparc3d_plan *p = new sparc3d_plan();
    p->cfg = *cfg;
    p->nxy = (long long)cfg->nx * cfg->ny;
    p->F = p->nxy * cfg->nbatch * cfg->nz;
    p->P = p->nxy * cfg->nbatch * (cfg->npmlbot + cfg->npmltop);
    if (!chunking(cfg->nz, 16, p->nch, p->L)) {
        delete p;
        return fail(SPARC_ERR_SIZE, "sparc3d_plan_create: nz too large for the column chunking");
    }
    for (int ibc = 0; ibc < 2; ibc++)
        if (!build_ztab(cfg->nz, ibc, p->nch, p->L, p->hz[ibc])) {
            delete p;
            return fail(SPARC_ERR_SIZE, "sparc3d_plan_create: singular reduced system");
        }
    const int rc = cfg->precision == 32 ? alloc_plan3<float>(p) : alloc_plan3<double>(p);
    if (rc != SPARC_OK) {
        std::string m = g_err;
        sparc3d_plan_destroy(p);
        return fail(rc, m);
    }
    *out = p;
    return SPARC_OK;
}

int sparc3d_plan_destroy(sparc3d_plan_t *p)
{
    if (!p) return SPARC_OK;
    free_plan3(p->s32);
    free_plan3(p->s64);
    delete p;
    return SPARC_OK;
}

int sparc3d_set_background(sparc3d_plan_t *p, const sparc3d_background_t *bg, void *stream)
{
    if (!p || !bg) return fail(SPARC_ERR_ARG, "sparc3d_set_background: null argument");
    const double *need[10] = {bg->stretch, bg->rhoinv, bg->rho0, bg->c2rho0, bg->gradp0_z, bg->gradrho0_z, bg->g,
                              bg->source_dep, bg->az, bg->bz};
    for (const double *q : need)
        if (!q) return fail(SPARC_ERR_ARG, "sparc3d_set_background: missing profile");
    if (p->cfg.flows && (!bg->v0x || !bg->v0y || !bg->v0z))
        return fail(SPARC_ERR_ARG, "sparc3d_set_background: flows on but v0 missing");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int rc = p->cfg.precision == 32 ? set_bg3<float>(p, bg, st) : set_bg3<double>(p, bg, st);
    if (rc == SPARC_OK) p->have_bg = true;
    return rc;
}

int sparc3d_set_source(sparc3d_plan_t *p, const double *pattern, const double *amp, int namp, void *stream)
{
    if (!p || !pattern || namp < 0 || (namp > 0 && !amp)) return fail(SPARC_ERR_ARG, "sparc3d_set_source: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t n = (size_t)p->cfg.nbatch * p->nxy;
    if (p->cfg.precision == 32) CK(cast_to<float>(pattern, p->s32.pat, n, st));
    else CK(cast_to<double>(pattern, p->s64.pat, n, st));
    p->amp.assign(amp, amp + namp);
    return SPARC_OK;
}

int sparc3d_reset_state(sparc3d_plan_t *p, int time0, void *stream)
{
    if (!p) return fail(SPARC_ERR_ARG, "sparc3d_reset_state: null plan");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t es = p->cfg.precision == 32 ? sizeof(float) : sizeof(double);
    void *A = p->cfg.precision == 32 ? (void *)p->s32.A : (void *)p->s64.A;
    void *SCR = p->cfg.precision == 32 ? (void *)p->s32.SCR : (void *)p->s64.SCR;
    void *PV = p->cfg.precision == 32 ? (void *)p->s32.PV : (void *)p->s64.PV;
    void *SPV = p->cfg.precision == 32 ? (void *)p->s32.SPV : (void *)p->s64.SPV;
    CK(cudaMemsetAsync(A, 0, 6 * p->F * es, st));
    CK(cudaMemsetAsync(SCR, 0, 6 * p->F * es, st));
    CK(cudaMemsetAsync(PV, 0, 2 * p->P * es, st));
    CK(cudaMemsetAsync(SPV, 0, 2 * p->P * es, st));
    p->time = time0;
    return SPARC_OK;
}

int sparc3d_forward(sparc3d_plan_t *p, int nsteps, void *seis, int nrec_cap, int *nrec, void *stream)
{
    if (!p || nsteps < 0 || nrec_cap < 0) return fail(SPARC_ERR_ARG, "sparc3d_forward: bad argument");
    if (!p->have_bg) return fail(SPARC_ERR_STATE, "sparc3d_forward: background not set");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int n = 0;
    for (int i = 0; i < nsteps; i++) {
        cudaError_t e = p->cfg.precision == 32 ? step3<float>(p, (float *)seis, nrec_cap, n, st)
                                               : step3<double>(p, (double *)seis, nrec_cap, n, st);
        if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("sparc3d_forward: ") + cudaGetErrorString(e));
    }
    if (nrec) *nrec = n;
    return SPARC_OK;
}

int sparc3d_get_state(sparc3d_plan_t *p, void *dst, void *stream)
{
    if (!p || !dst) return fail(SPARC_ERR_ARG, "sparc3d_get_state: null argument");
    const size_t es = p->cfg.precision == 32 ? sizeof(float) : sizeof(double);
    const void *A = p->cfg.precision == 32 ? (const void *)p->s32.A : (const void *)p->s64.A;
    CK(cudaMemcpyAsync(dst, A, 6 * p->F * es, cudaMemcpyDeviceToDevice, static_cast<cudaStream_t>(stream)));
    return SPARC_OK;
}

int sparc3d_set_state(sparc3d_plan_t *p, const void *src, void *stream)
{
    if (!p || !src) return fail(SPARC_ERR_ARG, "sparc3d_set_state: null argument");
    const size_t es = p->cfg.precision == 32 ? sizeof(float) : sizeof(double);
    void *A = p->cfg.precision == 32 ? (void *)p->s32.A : (void *)p->s64.A;
    CK(cudaMemcpyAsync(A, src, 6 * p->F * es, cudaMemcpyDeviceToDevice, static_cast<cudaStream_t>(stream)));
    return SPARC_OK;
}

int sparc3d_set_adjoint_source(sparc3d_plan_t *p, const double *rows, int nrows, const double *wts, const int *idx,
                               int ntab, double scale, void *stream)
{
    (void)stream;
    if (!p || !rows || nrows < 1 || !wts || !idx || ntab < 1)
        return fail(SPARC_ERR_ARG, "sparc3d_set_adjoint_source: bad argument");
    p->adj = true;
    p->adj_rows = rows;
    p->adj_nrows = nrows;
    p->adj_scale = scale;
    p->adj_w.assign(wts, wts + (size_t)ntab * 7);
    p->adj_idx.assign(idx, idx + ntab);
    return SPARC_OK;
}

int sparc3d_forward_records(sparc3d_plan_t *p, int nsteps, void *seis, int nrec_cap, int *nrec, void *snaps, int rec0,
                            int snap_cap, void *stream)
{
    if (!p || nsteps < 0 || nrec_cap < 0 || rec0 < 0 || snap_cap < 0 || (snap_cap > 0 && !snaps))
        return fail(SPARC_ERR_ARG, "sparc3d_forward_records: bad argument");
    if (!p->have_bg) return fail(SPARC_ERR_STATE, "sparc3d_forward_records: background not set");
    if (p->cfg.steps_out < 1) return fail(SPARC_ERR_ARG, "sparc3d_forward_records: steps_out must be >= 1");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int n = 0;
    for (int i = 0; i < nsteps; i++) {
        cudaError_t e = p->cfg.precision == 32
                            ? step3<float>(p, (float *)seis, nrec_cap, n, st, (float *)snaps, rec0, snap_cap)
                            : step3<double>(p, (double *)seis, nrec_cap, n, st, (double *)snaps, rec0, snap_cap);
        if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("sparc3d_forward_records: ") + cudaGetErrorString(e));
    }
    if (nrec) *nrec = n;
    return SPARC_OK;
}

int sparc3d_kernels_accumulate(sparc3d_plan_t *p, const void *snaps, int slot, double *out, void *stream)
{
    if (!p || !snaps || slot < 0 || !out) return fail(SPARC_ERR_ARG, "sparc3d_kernels_accumulate: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t off = (size_t)slot * 5 * p->F;
    cudaError_t e = p->cfg.precision == 32 ? kacc3<float>(p, (const float *)snaps + off, out, st)
                                           : kacc3<double>(p, (const double *)snaps + off, out, st);
    if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("sparc3d_kernels_accumulate: ") + cudaGetErrorString(e));
    return SPARC_OK;
}

size_t sparc3d_checkpoint_bytes(const sparc3d_plan_t *p)
{
    if (!p) return 0;
    const size_t es = p->cfg.precision == 32 ? sizeof(float) : sizeof(double);
    return (6 * (size_t)p->F + 2 * (size_t)p->P) * es;
}

int sparc3d_checkpoint_save(sparc3d_plan_t *p, void *dst, int *time, void *stream)
{
    if (!p || !dst || !time) return fail(SPARC_ERR_ARG, "sparc3d_checkpoint_save: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t es = p->cfg.precision == 32 ? sizeof(float) : sizeof(double);
    const void *A = p->cfg.precision == 32 ? (const void *)p->s32.A : (const void *)p->s64.A;
    const void *PV = p->cfg.precision == 32 ? (const void *)p->s32.PV : (const void *)p->s64.PV;
    CK(cudaMemcpyAsync(dst, A, 6 * p->F * es, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync((char *)dst + 6 * p->F * es, PV, 2 * p->P * es, cudaMemcpyDeviceToDevice, st));
    *time = p->time;
    return SPARC_OK;
}

int sparc3d_checkpoint_load(sparc3d_plan_t *p, const void *src, int time, void *stream)
{
    if (!p || !src) return fail(SPARC_ERR_ARG, "sparc3d_checkpoint_load: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t es = p->cfg.precision == 32 ? sizeof(float) : sizeof(double);
    void *A = p->cfg.precision == 32 ? (void *)p->s32.A : (void *)p->s64.A;
    void *PV = p->cfg.precision == 32 ? (void *)p->s32.PV : (void *)p->s64.PV;
    CK(cudaMemcpyAsync(A, src, 6 * p->F * es, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(PV, (const char *)src + 6 * p->F * es, 2 * p->P * es, cudaMemcpyDeviceToDevice, st));
    p->time = time;
    return SPARC_OK;
}

}  // extern "C"

// =============================================================================================
// 2-D sponge plans (option 5): buffers, one time step as a launch sequence, the C ABI.
// =============================================================================================
namespace {

template <typename T>
struct Plan5 {
    std::vector<void *> allocs;
    T *A = nullptr, *SCR = nullptr, *X = nullptr, *DVX = nullptr, *DVZ = nullptr, *GX = nullptr, *GZ = nullptr;
    T *prof = nullptr, *pat = nullptr;
    T *PV = nullptr, *SPV = nullptr, *PSI = nullptr;  // PML auxiliaries [npa][npml][nb][nx] (options 6, 12)
    T *FLUX = nullptr, *DZBX = nullptr, *DZF = nullptr, *DXF = nullptr, *DXBZ = nullptr;  // option 12 work
    T *MAG = nullptr;                                  // option 12: box, boz, curlboy [3][nz][nx]
    DevZ<T> z1;
    DevFFT<T> fx;
    S5Bg<T> bg{};
    const T *stretch = nullptr;
};

}  // namespace

struct sparc5_plan {
    sparc5_config_t cfg{};
    int nch = 0, L = 0;
    HostZTab hz1;
    Plan5<float> s32;
    Plan5<double> s64;
    std::vector<double> amp;
    int time = 0;
    bool have_bg = false;
    long long F = 0;
};

namespace {

template <typename T>
Plan5<T> &plan5(sparc5_plan *p);
template <>
Plan5<float> &plan5<float>(sparc5_plan *p) { return p->s32; }
template <>
Plan5<double> &plan5<double>(sparc5_plan *p) { return p->s64; }

// Fields of the state, PML auxiliaries and PML levels of an option.
int nf5(const sparc5_config_t &c) { return c.option == 12 ? 8 : 5; }
int npa5(const sparc5_config_t &c) { return c.option == 12 ? 4 : (c.option == 6 ? 2 : 0); }
int npml5(const sparc5_config_t &c) { return (c.option == 6 || c.option == 12) ? c.npmlbot + c.npmltop : 0; }

template <typename T>
int alloc_plan5(sparc5_plan *p)
{
    Plan5<T> &S = plan5<T>(p);
    const sparc5_config_t &c = p->cfg;
    const size_t F = (size_t)p->F, nz = c.nz, npml = npml5(c), nf = nf5(c);
    const size_t P2 = (size_t)npa5(c) * npml * c.nbatch * c.nx;
    const size_t FM = c.option == 12 ? F : 0, NM = c.option == 12 ? 3 * nz * (size_t)c.nx : 0;
    struct Req { T **ptr; size_t n; };
    std::vector<Req> reqs = {{&S.A, nf * F}, {&S.SCR, nf * F}, {&S.X, nf * F}, {&S.DVX, F}, {&S.DVZ, F}, {&S.GX, F},
                             {&S.GZ, F}, {&S.prof, 9 * nz + 2 * npml}, {&S.pat, (size_t)c.nbatch * c.nx},
                             {&S.PV, P2}, {&S.SPV, P2}, {&S.PSI, P2}, {&S.FLUX, FM}, {&S.DZBX, FM}, {&S.DZF, FM},
                             {&S.DXF, FM}, {&S.DXBZ, FM}, {&S.MAG, NM}};
    for (auto &r : reqs) {
        void *ptr = nullptr;
        const size_t bytes = std::max<size_t>(r.n, 1) * sizeof(T);
        cudaError_t e = cudaMalloc(&ptr, bytes);
        if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        S.allocs.push_back(ptr);
        e = cudaMemset(ptr, 0, bytes);
        if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("cudaMemset: ") + cudaGetErrorString(e));
        *r.ptr = (T *)ptr;
    }
    cudaError_t e = upload_ztab<T>(p->hz1, S.z1, S.allocs);
    if (e == cudaSuccess) e = upload_fft<T>(c.nx, S.fx, S.allocs);
    if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("tables: ") + cudaGetErrorString(e));
    T *q = S.prof;
    S.stretch = q; q += nz;
    S.bg.rhoinv = q; q += nz;
    S.bg.rho0 = q; q += nz;
    S.bg.c2rho0 = q; q += nz;
    S.bg.gradp0_z = q; q += nz;
    S.bg.gradrho0_z = q; q += nz;
    S.bg.g = q; q += nz;
    S.bg.source_dep = q; q += nz;
    S.bg.sponge = q; q += nz;
    S.bg.az = q; q += npml;
    S.bg.bz = q;
    if (c.option == 12) {
        S.bg.box = S.MAG;
        S.bg.boz = S.MAG + nz * c.nx;
        S.bg.curl = S.MAG + 2 * nz * c.nx;
    }
    return SPARC_OK;
}

// STEP for option 5 (step.f90:43-119, physics2d.f90:1099-1137, FILTER_VARS_2D) and the record.
template <typename T>
cudaError_t step5(sparc5_plan *p, T *seis, int cap, int &nrec, cudaStream_t st)
{
    Plan5<T> &S = plan5<T>(p);
    const sparc5_config_t &c = p->cfg;
    const long long F = p->F, lvl = (long long)c.nbatch * c.nx;
    const bool pml = c.option == 6 || c.option == 12, mhd = c.option == 12;
    const int nf = nf5(c);
    const S5Args a{c.nx, c.nz, c.nbatch, c.k_src, c.filter_all_x ? 0 : c.npmlhor - 1,
                   c.filter_all_x ? c.nx - 1 : c.nx - c.npmlhor, pml ? c.npmlbot : 0, pml ? c.npmltop : 0,
                   nf, npa5(c)};
    const long long P2 = (long long)npa5(c) * npml5(c) * lvl;
    const T amp = (T)(p->time >= 0 && p->time < (int)p->amp.size() ? p->amp[p->time] : 0.0);
    cudaError_t e;
    for (int s = 0; s < 5; s++) {
        const T *X = S.A, *PSI = S.PV;
        if (s > 0) {
            e = launch_s3_stage_in<T>(nf * F, S.A, S.SCR, S.X, (T)c.betas[s], P2, S.PV, S.SPV, S.PSI, st);
            if (e != cudaSuccess) return e;
            X = S.X;
            PSI = S.PSI;
        }
        const int nrows = c.nz * c.nbatch;
        e = launch_ddx<T>(X + F, S.DVX, nrows, c.nx, (T)c.stretchx, S.fx.twr, S.fx.twi, S.fx.kap, st);
        if (e == cudaSuccess) e = launch_ddx<T>(X + 4 * F, S.GX, nrows, c.nx, (T)c.stretchx, S.fx.twr, S.fx.twi, S.fx.kap, st);
        if (e == cudaSuccess) e = launch_ddz<T>(S.z1.tab, p->nch, p->L, X + 3 * F, S.DVZ, (int)lvl, c.nz, nullptr, S.stretch, 0, st);
        if (e == cudaSuccess) e = launch_ddz<T>(S.z1.tab, p->nch, p->L, X + 4 * F, S.GZ, (int)lvl, c.nz, nullptr, S.stretch, 0, st);
        if (e == cudaSuccess && mhd) {  // flux, d flux/dx, d flux/dz, d b_z/dx, d b_x/dz
            e = launch_s12_flux<T>(a, S.bg, X, S.FLUX, st);
            if (e == cudaSuccess) e = launch_ddx<T>(S.FLUX, S.DXF, nrows, c.nx, (T)c.stretchx, S.fx.twr, S.fx.twi, S.fx.kap, st);
            if (e == cudaSuccess) e = launch_ddx<T>(X + 7 * F, S.DXBZ, nrows, c.nx, (T)c.stretchx, S.fx.twr, S.fx.twi, S.fx.kap, st);
            if (e == cudaSuccess) e = launch_ddz<T>(S.z1.tab, p->nch, p->L, S.FLUX, S.DZF, (int)lvl, c.nz, nullptr, S.stretch, 0, st);
            if (e == cudaSuccess) e = launch_ddz<T>(S.z1.tab, p->nch, p->L, X + 5 * F, S.DZBX, (int)lvl, c.nz, nullptr, S.stretch, 0, st);
        }
        if (e == cudaSuccess)
            e = mhd ? launch_s12_rhs<T>(a, S.bg, X, S.SCR, S.DVX, S.DVZ, S.GX, S.GZ, S.DZBX, S.DZF, S.DXF, S.DXBZ, PSI,
                                        S.SPV, S.pat, amp, st)
                : pml ? launch_s6_rhs<T>(a, S.bg, X, S.SCR, S.DVX, S.DVZ, S.GX, S.GZ, PSI, S.SPV, S.pat, amp, st)
                      : launch_s5_rhs<T>(a, S.bg, X, S.SCR, S.DVX, S.DVZ, S.GX, S.GZ, S.pat, amp, st);
        if (e != cudaSuccess) return e;
    }
    e = launch_s5_end<T>(a, S.A, S.SCR, (T)c.deltat, pml ? S.PV : nullptr, S.SPV, st);
    if (e != cudaSuccess) return e;
    if (c.steps_out > 0 && p->time % c.steps_out == 0) {
        if (seis && nrec < cap) {
            e = cudaMemcpyAsync(seis + (size_t)nrec * lvl, S.A + 3 * F + (size_t)c.k_obs * lvl, lvl * sizeof(T),
                                cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) return e;
        }
        nrec++;
    }
    p->time++;
    return cudaSuccess;
}

template <typename T>
int set_bg5(sparc5_plan *p, const sparc5_background_t *bg, cudaStream_t st)
{
    Plan5<T> &S = plan5<T>(p);
    const int nz = p->cfg.nz;
    const double *prof[9] = {bg->stretch, bg->rhoinv, bg->rho0, bg->c2rho0, bg->gradp0_z, bg->gradrho0_z, bg->g,
                             bg->source_dep, bg->sponge};
    for (int i = 0; i < 9; i++) CK(cast_to<T>(prof[i], S.prof + (size_t)i * nz, nz, st));
    if (p->cfg.option == 6 || p->cfg.option == 12) {
        const int npml = p->cfg.npmlbot + p->cfg.npmltop;
        CK(cast_to<T>(bg->az, S.prof + (size_t)9 * nz, npml, st));
        CK(cast_to<T>(bg->bz, S.prof + (size_t)9 * nz + npml, npml, st));
    }
    if (p->cfg.option == 12) {  // box, boz; curlboy = d box/dz - d boz/dx (physics2d.f90:166-168)
        const int nx = p->cfg.nx;
        const size_t NM = (size_t)nz * nx;
        T *box = S.MAG, *boz = S.MAG + NM, *curl = S.MAG + 2 * NM;
        CK(cast_to<T>(bg->box, box, NM, st));
        CK(cast_to<T>(bg->boz, boz, NM, st));
        CK(launch_ddz<T>(S.z1.tab, p->nch, p->L, box, curl, nx, nz, nullptr, S.stretch, 0, st));
        CK(launch_ddx<T>(boz, S.DXBZ, nz, nx, (T)p->cfg.stretchx, S.fx.twr, S.fx.twi, S.fx.kap, st));
        CK(launch_s5_axpy<T>((long long)NM, curl, S.DXBZ, T(-1), st));
    }
    return SPARC_OK;
}

}  // namespace

extern "C" {

int sparc5_plan_create(const sparc5_config_t *cfg, sparc5_plan_t **out)
{
    if (!cfg || !out) return fail(SPARC_ERR_ARG, "sparc5_plan_create: null argument");
    *out = nullptr;
    if (cfg->precision != 32 && cfg->precision != 64) return fail(SPARC_ERR_SIZE, "sparc5_plan_create: precision");
    if (!fft_size_supported(cfg->nx)) return fail(SPARC_ERR_SIZE, "sparc5_plan_create: nx not in the FFT table");
    if (cfg->nz < 11 || cfg->nbatch < 1 || cfg->k_src < 0 || cfg->k_src >= cfg->nz || cfg->k_obs < 0 ||
        cfg->k_obs >= cfg->nz || (!cfg->filter_all_x && (cfg->npmlhor < 1 || 2 * cfg->npmlhor > cfg->nx)) ||
        (long long)cfg->nz * cfg->nbatch > 2147483647LL)
        return fail(SPARC_ERR_SIZE, "sparc5_plan_create: bad grid, batch or rows");
    if ((cfg->option != 5 && cfg->option != 6 && cfg->option != 12) ||
        (cfg->option != 5 && (cfg->npmlbot < 1 || cfg->npmltop < 1 || cfg->npmlbot + cfg->npmltop >= cfg->nz)))
        return fail(SPARC_ERR_ARG, "sparc5_plan_create: option must be 5, 6 or 12 (with PML levels for 6 and 12)");
    sparc5_plan *p = new sparc5_plan();
    p->cfg = *cfg;
    p->F = (long long)cfg->nx * cfg->nbatch * cfg->nz;
    if (!chunking(cfg->nz, 16, p->nch, p->L) || !build_ztab(cfg->nz, 1, p->nch, p->L, p->hz1)) {
        delete p;
        return fail(SPARC_ERR_SIZE, "sparc5_plan_create: nz too large for the column chunking");
    }
    const int rc = cfg->precision == 32 ? alloc_plan5<float>(p) : alloc_plan5<double>(p);
    if (rc != SPARC_OK) {
        std::string m = g_err;
        sparc5_plan_destroy(p);
        return fail(rc, m);
    }
    *out = p;
    return SPARC_OK;
}

int sparc5_plan_destroy(sparc5_plan_t *p)
{
    if (!p) return SPARC_OK;
    for (void *q : p->s32.allocs) cudaFree(q);
    for (void *q : p->s64.allocs) cudaFree(q);
    delete p;
    return SPARC_OK;
}

int sparc5_set_background(sparc5_plan_t *p, const sparc5_background_t *bg, void *stream)
{
    if (!p || !bg) return fail(SPARC_ERR_ARG, "sparc5_set_background: null argument");
    const double *need[9] = {bg->stretch, bg->rhoinv, bg->rho0, bg->c2rho0, bg->gradp0_z, bg->gradrho0_z, bg->g,
                             bg->source_dep, bg->sponge};
    for (const double *q : need)
        if (!q) return fail(SPARC_ERR_ARG, "sparc5_set_background: missing profile");
    if (p->cfg.option != 5 && (!bg->az || !bg->bz)) return fail(SPARC_ERR_ARG, "sparc5_set_background: PML az, bz missing");
    if (p->cfg.option == 12 && (!bg->box || !bg->boz))
        return fail(SPARC_ERR_ARG, "sparc5_set_background: option 12 needs the background field box, boz");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int rc = p->cfg.precision == 32 ? set_bg5<float>(p, bg, st) : set_bg5<double>(p, bg, st);
    if (rc == SPARC_OK) p->have_bg = true;
    return rc;
}

int sparc5_set_source(sparc5_plan_t *p, const double *pattern, const double *amp, int namp, void *stream)
{
    if (!p || !pattern || namp < 0 || (namp > 0 && !amp)) return fail(SPARC_ERR_ARG, "sparc5_set_source: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t n = (size_t)p->cfg.nbatch * p->cfg.nx;
    if (p->cfg.precision == 32) CK(cast_to<float>(pattern, p->s32.pat, n, st));
    else CK(cast_to<double>(pattern, p->s64.pat, n, st));
    p->amp.assign(amp, amp + namp);
    return SPARC_OK;
}

int sparc5_reset_state(sparc5_plan_t *p, int time0, void *stream)
{
    if (!p) return fail(SPARC_ERR_ARG, "sparc5_reset_state: null plan");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t es = p->cfg.precision == 32 ? sizeof(float) : sizeof(double);
    void *A = p->cfg.precision == 32 ? (void *)p->s32.A : (void *)p->s64.A;
    void *SCR = p->cfg.precision == 32 ? (void *)p->s32.SCR : (void *)p->s64.SCR;
    CK(cudaMemsetAsync(A, 0, nf5(p->cfg) * p->F * es, st));
    CK(cudaMemsetAsync(SCR, 0, nf5(p->cfg) * p->F * es, st));
    if (npa5(p->cfg) > 0) {
        const size_t P2 = (size_t)npa5(p->cfg) * npml5(p->cfg) * p->cfg.nbatch * p->cfg.nx;
        void *PV = p->cfg.precision == 32 ? (void *)p->s32.PV : (void *)p->s64.PV;
        void *SPV = p->cfg.precision == 32 ? (void *)p->s32.SPV : (void *)p->s64.SPV;
        CK(cudaMemsetAsync(PV, 0, P2 * es, st));
        CK(cudaMemsetAsync(SPV, 0, P2 * es, st));
    }
    p->time = time0;
    return SPARC_OK;
}

int sparc5_forward(sparc5_plan_t *p, int nsteps, void *seis, int nrec_cap, int *nrec, void *stream)
{
    if (!p || nsteps < 0 || nrec_cap < 0) return fail(SPARC_ERR_ARG, "sparc5_forward: bad argument");
    if (!p->have_bg) return fail(SPARC_ERR_STATE, "sparc5_forward: background not set");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int n = 0;
    for (int i = 0; i < nsteps; i++) {
        cudaError_t e = p->cfg.precision == 32 ? step5<float>(p, (float *)seis, nrec_cap, n, st)
                                               : step5<double>(p, (double *)seis, nrec_cap, n, st);
        if (e != cudaSuccess) return fail(SPARC_ERR_CUDA, std::string("sparc5_forward: ") + cudaGetErrorString(e));
    }
    if (nrec) *nrec = n;
    return SPARC_OK;
}

int sparc5_get_state(sparc5_plan_t *p, void *dst, void *stream)
{
    if (!p || !dst) return fail(SPARC_ERR_ARG, "sparc5_get_state: null argument");
    const size_t es = p->cfg.precision == 32 ? sizeof(float) : sizeof(double);
    const void *A = p->cfg.precision == 32 ? (const void *)p->s32.A : (const void *)p->s64.A;
    CK(cudaMemcpyAsync(dst, A, nf5(p->cfg) * p->F * es, cudaMemcpyDeviceToDevice, static_cast<cudaStream_t>(stream)));
    return SPARC_OK;
}

}  // extern "C"
