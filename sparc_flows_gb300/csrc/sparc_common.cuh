// sparc_common.cuh -- device data structures and building blocks of the GB300 wave solver.
//
//  * warp-level Stockham FFT (radix 4/2/3, shared-memory ping-pong) used for the spectral
//    x-derivative of derivatives.f90:28-58;
//  * SPIKE-partitioned solve of the sixth-order compact z-derivative (dbyd2.f:8-235,
//    mtridag.f:96-112): each column is cut into NCH chunks of at most LMAX rows, every chunk
//    is solved independently with its own Thomas factors, and the coupling between chunks is
//    restored exactly through precomputed spike vectors and the inverse of the small reduced
//    system (all factors precomputed in FP64 on the host).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace sparc {

constexpr int WARP = 32;
constexpr int MAX_NCH = 24;  // chunks per column (nz <= MAX_NCH * LMAX)
constexpr int SPARC_DEV_ERR_TMA_TIMEOUT = 1;  // device error flag: a bounded mbarrier wait gave up
constexpr int SPARC_DEV_ERR_TMA_ALIGN = 2;    // ... a TMA destination in shared memory was not 128-byte aligned
constexpr int SPARC_DEV_ERR_STAGE_WAIT = 3;   // ... a row pass gave up waiting for its solve's column tiles
// Geometric-band form of the compact z-derivative (FP32 column pass): T^{-1} as the inverse of
// the infinite Toeplitz operator, t0 r^|d|, plus rank-BAND_Q corrections on BAND_KC x BAND_KC
// corners.  BAND_W: minimum rows of zero padding / depth margin the host checks for.
constexpr int BAND_W = 20, BAND_KC = 24, BAND_Q = 3, BAND_NPOW = 48;

// Field order of the live state (xi_y and v_y vanish identically in 2-D).
enum { F_XIX = 0, F_XIZ = 1, F_VX = 2, F_VZ = 3 };

// Compact-derivative tables for one boundary condition (device pointers).
template <typename T>
struct ZTab {
    const T *w5;    // [nz][5] stencil weights of rows 0, 1, nz-2, nz-1 (rows 0,1 on b[0..4],
                    // rows nz-2, nz-1 on b[nz-5..nz-1]); interior rows use c1, c2
    const T *ib;    // [nz] 1/beta of the chunk-local Thomas factorisation
    const T *lwib;  // [nz] lower * ib
    const T *gm;    // [nz] gamma (backward sweep)
    const T *WL;    // [nz] lower(s_c) * spike from the chunk's first row
    const T *VU;    // [nz] upper(e_c) * spike from the chunk's last row
    const T *G;     // [2 nch][2 nch] inverse of the reduced system
    T c1, c2;       // interior coefficients (float32 values of dbyd2.f:82-83)
    int preset_row; // row whose right-hand side is supplied by the caller (-1: none)
};

// Everything one stage kernel needs.  Layouts (x fastest everywhere):
//   A    [nb][4][nz][nx]            state xi_x, xi_z, v_x, v_z (ALO: low parts, FP32 plans)
//   SV   [3][nb][2][nz][nx]         ring of stage RHS of v_x, v_z (slot = stage % 3)
//   P, RVXP, DX, FXX, FXZ [nb][nz][nx] stage intermediates, TOPDX [nb][nx]
//   PZ   [nb][2][nzpml][nx]         psi_vz, psi_p;  SPZ [3][nb][2][nzpml][nx]
//   PX   [nb][2][nz][nhx]           psi_vx, psi_gradp_x;  SPX [3][nb][2][nz][nhx]
template <typename T>
struct StepArgs {
    int nx, nz, nb, nh, nhx, nzpml, npmlbot, npmltop;
    int flows, c2d;
    long long bg2, bgz, bgx;  // batch strides of 2-D, PML-layer and x-PML background arrays
    T bs, bsm1, dt, stretchx, fsign, unstretch_top;
    int stage, slot_s, slot_sm1, slot_sm2;
    T *A, *SV, *P, *RVXP, *DX, *FXX, *FXZ, *TOPDX, *PZ, *SPZ, *PX, *SPX;
    T *ALO;  // low parts of the state (FP32 plans): A + ALO carries ~48 significant bits
    const T *rhoinv, *rho0, *gp0, *gr0, *g, *stretch;
    const T *fdz, *az, *bz, *ax, *bx, *c2rho0, *v0x, *v0z;
    const T *twr, *twi, *kap;
    ZTab<T> z1, z2, z3;
    int nch, L;
    int *d_time;
    int src_until, k_inj, k_obs, steps_out;
    int filt_k0, filt_xall;  // FILTER_VARS_2D coverage (rows from filt_k0, all columns if filt_xall)
    int colw;                // column-pass block width (8 or 32 columns)
    int boxr;                // rows per TMA box of the staged column pass (2 boxes cover nz)
    int *d_err;              // device error flag (SPARC_DEV_ERR_*)
    // stage overlap (FP32 banded column pass followed by the 512-column row pass): tile_cnt[s-1][b]
    // counts the column tiles of solve b finished in stage s (tiles_per_solve when complete); the
    // row pass of stage s+1, launched as a programmatic dependent of the column pass, starts on
    // SMs the column pass's last wave leaves idle and waits for its own solve's count only.
    // nullptr: no overlap
    int *tile_cnt;
    int tiles_per_solve;
    const T *inj_scale, *src_rows;
    int nrows;
    const double *src_w;
    const int *src_idx;
    int ntab;
    T *seis, *snaps;
    int nrec_cap;
    int rec0;  // records rec0 .. rec0 + nrec_cap - 1 are written, to slots 0 .. nrec_cap - 1
};

template <typename T>
__device__ __forceinline__ T *svp(const StepArgs<T> &a, int slot, int b, int c)
{
    return a.SV + (((size_t)slot * a.nb + b) * 2 + c) * (size_t)a.nz * a.nx;
}

// Row of the vertical-PML arrays holding depth row k (-1 outside both layers).
template <typename T>
__device__ __forceinline__ int pml_row(const StepArgs<T> &a, int k)
{
    if (k < a.npmlbot) return k;
    if (k >= a.nz - a.npmltop) return a.npmlbot + (k - (a.nz - a.npmltop));
    return -1;
}

// Geometric-band tables (FP32 plans).  x = T^{-1} rhs is evaluated as
//   x[k] = t0 (rhs[k] + sum_{d>=1} r^d (rhs[k-d] + rhs[k+d]))      (rhs zero outside 0..nz-1)
//        + sum_q Ub[k][q] (Vb[q] . rhs[0..KC))                      for k < KC
//        + sum_q Ut[k'][q] (Vt[q] . rhs[nz-KC..nz))                 for k' = k - (nz-KC) >= 0
// uv[i] (boundary condition i+1) holds Ub [KC][Q], Vb [Q][KC], Ut [KC][Q], Vt [Q][KC];
// rpow[n] = r^n.
struct BandDev {
    float t0, r;
    float rpow[BAND_NPOW];
    const float *uv[3];
    // Thomas factors of the top block for ibc 1 and 2 (copies of uv[0], uv[1] from 4 KC Q on:
    // 1/beta, lower/beta, gamma, the coupling to row nz-KC-1): indexed with compile-time
    // offsets, they are constant-bank operands of the sweeps' arithmetic, with no load on the
    // recurrence's chain
    float th[2][3 * BAND_KC + 1];
};


// ------------------------------------------------------------------------------------------
// FFT
// ------------------------------------------------------------------------------------------
// Radix plan: as many radix-8 passes as possible, then 4, 2, 3 (512 = 8.8.8, 384 = 8.8.2.3).
template <int N>
struct Radices {
    static constexpr int count()
    {
        int n = N, c = 0;
        while (n % 8 == 0) { n /= 8; c++; }
        while (n % 4 == 0) { n /= 4; c++; }
        while (n % 2 == 0) { n /= 2; c++; }
        while (n % 3 == 0) { n /= 3; c++; }
        return c;
    }
    static constexpr int at(int i)
    {
        int n = N, c = 0;
        while (n % 8 == 0) { if (c == i) return 8; n /= 8; c++; }
        while (n % 4 == 0) { if (c == i) return 4; n /= 4; c++; }
        while (n % 2 == 0) { if (c == i) return 2; n /= 2; c++; }
        while (n % 3 == 0) { if (c == i) return 3; n /= 3; c++; }
        return 1;
    }
};

template <typename T, int R>
__host__ __device__ __forceinline__ void butterfly(T *vr, T *vi, bool inv)
{
    if constexpr (R == 2) {
        T ar = vr[0], ai = vi[0];
        vr[0] = ar + vr[1]; vi[0] = ai + vi[1];
        vr[1] = ar - vr[1]; vi[1] = ai - vi[1];
    } else if constexpr (R == 4) {
        T s0r = vr[0] + vr[2], s0i = vi[0] + vi[2];
        T d0r = vr[0] - vr[2], d0i = vi[0] - vi[2];
        T s1r = vr[1] + vr[3], s1i = vi[1] + vi[3];
        T d1r = vr[1] - vr[3], d1i = vi[1] - vi[3];
        T jr = inv ? -d1i : d1i, ji = inv ? d1r : -d1r;  // d1 * (inv ? +i : -i)
        vr[0] = s0r + s1r; vi[0] = s0i + s1i;
        vr[1] = d0r + jr;  vi[1] = d0i + ji;
        vr[2] = s0r - s1r; vi[2] = s0i - s1i;
        vr[3] = d0r - jr;  vi[3] = d0i - ji;
    } else if constexpr (R == 8) {
        // out[2q] = DFT4(v_k + v_{k+4})[q], out[2q+1] = DFT4((v_k - v_{k+4}) W8^k)[q]
        const T r2 = T(0.7071067811865475244008443621048490);
        T ar[4], ai[4], br[4], bi[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            ar[k] = vr[k] + vr[k + 4]; ai[k] = vi[k] + vi[k + 4];
            br[k] = vr[k] - vr[k + 4]; bi[k] = vi[k] - vi[k + 4];
        }
        // W8^1 = (1 -/+ i)/sqrt2, W8^2 = -/+ i, W8^3 = (-1 -/+ i)/sqrt2 (forward / inverse)
        const T sg = inv ? T(1) : T(-1);
        {
            T xr = br[1], xi = bi[1];
            br[1] = r2 * (xr - sg * xi); bi[1] = r2 * (xi + sg * xr);
            xr = br[2]; xi = bi[2];
            br[2] = -sg * xi; bi[2] = sg * xr;
            xr = br[3]; xi = bi[3];
            br[3] = r2 * (-xr - sg * xi); bi[3] = r2 * (-xi + sg * xr);
        }
        butterfly<T, 4>(ar, ai, inv);
        butterfly<T, 4>(br, bi, inv);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            vr[2 * q] = ar[q]; vi[2 * q] = ai[q];
            vr[2 * q + 1] = br[q]; vi[2 * q + 1] = bi[q];
        }
    } else {  // R == 3
        const T h = T(0.8660254037844386467637231707529362);
        T tr = vr[1] + vr[2], ti = vi[1] + vi[2];
        T dr = vr[1] - vr[2], di = vi[1] - vi[2];
        T mr = vr[0] - T(0.5) * tr, mi = vi[0] - T(0.5) * ti;
        T sg = inv ? h : -h;  // sigma * sqrt(3)/2
        // i * sg * d = (-sg*di, sg*dr)
        vr[0] = vr[0] + tr; vi[0] = vi[0] + ti;
        vr[1] = mr - sg * di; vi[1] = mi + sg * dr;
        vr[2] = mr + sg * di; vi[2] = mi - sg * dr;
    }
}

// One Stockham autosort stage of radix R after NS points have been combined.  The first stage
// (NS == 1) multiplies the real and imaginary inputs by sr and si.
template <typename T, int N, int R, int NS>
__device__ __forceinline__ void stockham_stage(const T *__restrict__ xr, const T *__restrict__ xi,
                                               T *__restrict__ yr, T *__restrict__ yi,
                                               const T *__restrict__ twr, const T *__restrict__ twi,
                                               int lane, bool inv, T sr, T si)
{
    constexpr int NR = N / R;
    constexpr int TS = N / (NS * R);
#pragma unroll 2
    for (int j = lane; j < NR; j += WARP) {
        const int k = j % NS;
        T vr[R], vi[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
            T ar = xr[j + r * NR], ai = xi[j + r * NR];
            if (NS == 1) {
                vr[r] = ar * sr; vi[r] = ai * si;
            } else if (r == 0) {
                vr[r] = ar; vi[r] = ai;
            } else {
                const int t = r * k * TS;  // < N
                T wr = __ldg(twr + t), wi = __ldg(twi + t);
                if (inv) wi = -wi;
                vr[r] = ar * wr - ai * wi;
                vi[r] = ar * wi + ai * wr;
            }
        }
        butterfly<T, R>(vr, vi, inv);
        const int base = (j / NS) * NS * R + k;
#pragma unroll
        for (int r = 0; r < R; r++) {
            yr[base + r * NS] = vr[r];
            yi[base + r * NS] = vi[r];
        }
    }
}

template <typename T, int N, int I, int NS>
struct FFTRun {
    __device__ static __forceinline__ void run(T *xr, T *xi, T *yr, T *yi, const T *twr, const T *twi,
                                               int lane, bool inv, T sr, T si, T *&outr, T *&outi)
    {
        if constexpr (I == Radices<N>::count()) {
            outr = xr; outi = xi;
        } else {
            constexpr int R = Radices<N>::at(I);
            stockham_stage<T, N, R, NS>(xr, xi, yr, yi, twr, twi, lane, inv, sr, si);
            __syncwarp();
            FFTRun<T, N, I + 1, NS * R>::run(yr, yi, xr, xi, twr, twi, lane, inv, T(1), T(1), outr, outi);
        }
    }
};

// Power of two 2^-e with e the binary exponent of the maximum m of |v| over a row
// (m in [2^(e-1), 2^e)): scales the row's largest value into [0.5, 1) exactly.  Two real rows
// packed in one complex FFT share its rounding, which is relative to the larger row; in FP32 a
// row 1e7 times smaller than its partner (pressure against displacement at the bottom of a
// polytrope) would keep no significant digit.  Scaling each row first makes the rounding
// relative to the row itself.  The exponent is read from the bit pattern and the scale is kept
// a normal number (subnormal rows get the largest scale, 2^125 / 2^1021); zero and non-finite
// rows keep scale 1.
__device__ __forceinline__ float pow2_scale_of(float m)
{
    if (!(m > 0.f) || !isfinite(m)) return 1.f;
    const int E = (int)((__float_as_uint(m) >> 23) & 0xffu);  // biased exponent, 0 for subnormal
    const int f = min(max(253 - max(E, 1), 1), 254);          // biased exponent of 2^(126 - E)
    return __uint_as_float((unsigned)f << 23);
}
__device__ __forceinline__ double pow2_scale_of(double m)
{
    if (!(m > 0.0) || !isfinite(m)) return 1.0;
    const int E = (int)((__double_as_longlong(m) >> 52) & 0x7ff);
    const long long f = min(max(2045 - max(E, 1), 1), 2046);  // biased exponent of 2^(1022 - E)
    return __longlong_as_double(f << 52);
}
// Scale s for a row whose lane-local max |v| is m_lane, and the factor that takes the FFT
// output back (1/s, exact).  A row that is zero gets output factor 0: its partner, scaled to
// O(1), leaks rounding of O(eps) into it, while its derivative is exactly zero.  (A NaN in such
// a row still propagates: 0 * NaN is NaN.)
template <typename T>
__device__ __forceinline__ void warp_row_scale(T m_lane, T &s, T &inv)
{
    T m = m_lane;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    s = pow2_scale_of(m);
    inv = (m == T(0)) ? T(0) : T(1) / s;
}

// Spectral derivative of the complex row (xr + i xi) of length N held in warp-private shared
// memory (yr, yi are scratch of the same size): forward FFT of (sr xr + i si xi), multiply bin
// k by i*kap[k]*scale (kap already carries the 1/N normalisation and a zero Nyquist bin),
// inverse FFT.  Real and imaginary parts of the result are the derivatives of the two real rows
// times sr and si (powers of two from warp_row_scale; 1 for no scaling).
template <typename T, int N>
__device__ __forceinline__ void fft_deriv(T *xr, T *xi, T *yr, T *yi, const T *twr, const T *twi,
                                          const T *kap, T scale, int lane, T *&outr, T *&outi,
                                          T sr = T(1), T si = T(1))
{
    T *fr, *fi;
    FFTRun<T, N, 0, 1>::run(xr, xi, yr, yi, twr, twi, lane, false, sr, si, fr, fi);
    for (int k = lane; k < N; k += WARP) {
        T kk = __ldg(kap + k) * scale;
        T re = fr[k], im = fi[k];
        fr[k] = -kk * im;
        fi[k] = kk * re;
    }
    __syncwarp();
    T *gr = (fr == xr) ? yr : xr, *gi = (fr == xr) ? yi : xi;
    FFTRun<T, N, 0, 1>::run(fr, fi, gr, gi, twr, twi, lane, true, T(1), T(1), outr, outi);
}

// ------------------------------------------------------------------------------------------
// Compact z-derivative, SPIKE-partitioned (see file comment).
// src: shared memory [nz][CWS] (column stride CWS), thread owns rows [k0, k0+n) of column c.
// ------------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T zrhs(const ZTab<T> &tb, const T *src, int CWS, int c, int k, int nz, T preset)
{
    if (k >= 2 && k <= nz - 3)
        return tb.c1 * (src[(k + 1) * CWS + c] - src[(k - 1) * CWS + c]) +
               tb.c2 * (src[(k + 2) * CWS + c] - src[(k - 2) * CWS + c]);
    if (k == tb.preset_row) return preset;
    const int base = (k <= 1) ? 0 : nz - 5;
    const T *w = tb.w5 + 5 * k;
    T r = __ldg(w) * src[base * CWS + c];
#pragma unroll
    for (int j = 1; j < 5; j++) r += __ldg(w + j) * src[(base + j) * CWS + c];
    return r;
}

// Chunk-local forward and backward sweeps; y[m] for m < n.  Returns y[n-1] (kept out of
// the register array so that it is never indexed with a run-time value).
template <typename T, int LMAX>
__device__ __forceinline__ T zlocal(const ZTab<T> &tb, const T *src, int CWS, int c, int k0, int n, int nz,
                                    T preset, T (&y)[LMAX])
{
    T prev = T(0);
#pragma unroll
    for (int m = 0; m < LMAX; m++) {
        if (m < n) {
            const int k = k0 + m;
            T v = zrhs(tb, src, CWS, c, k, nz, preset) * __ldg(tb.ib + k);
            if (m > 0) v -= __ldg(tb.lwib + k) * prev;
            y[m] = v;
            prev = v;
        }
    }
    const T last = prev;
#pragma unroll
    for (int m = LMAX - 2; m >= 0; m--) {
        if (m + 1 < n) y[m] -= __ldg(tb.gm + k0 + m + 1) * y[m + 1];
    }
    return last;
}

// Coupling values from the neighbouring chunks: xl = x[first row - 1], xr = x[last row + 1].
template <typename T>
__device__ __forceinline__ void zcouple(const ZTab<T> &tb, const T *ybnd, int CWS, int c, int j, int nch,
                                        T &xl, T &xr)
{
    const int n2 = 2 * nch;
    xl = T(0); xr = T(0);
    if (j > 0) {
        const T *g = tb.G + (2 * j - 1) * n2;
        for (int q = 0; q < n2; q++) xl += __ldg(g + q) * ybnd[q * CWS + c];
    }
    if (j < nch - 1) {
        const T *g = tb.G + (2 * j + 2) * n2;
        for (int q = 0; q < n2; q++) xr += __ldg(g + q) * ybnd[q * CWS + c];
    }
}

template <typename T>
__device__ __forceinline__ T zcorrect(const ZTab<T> &tb, T y, int k, T xl, T xr)
{
    return y - __ldg(tb.WL + k) * xl - __ldg(tb.VU + k) * xr;
}

// ------------------------------------------------------------------------------------------
// Launchers (defined in sparc_row.cu / sparc_col.cu)
// ------------------------------------------------------------------------------------------
template <typename T>
cudaError_t launch_row_stage(const StepArgs<T> &a, cudaStream_t st);
template <typename T>
cudaError_t launch_col_stage(const StepArgs<T> &a, cudaStream_t st);
template <typename T>
cudaError_t launch_end_step(const StepArgs<T> &a, cudaStream_t st);
template <typename T>
cudaError_t launch_ddx(const T *var, T *dvar, int nrows, int nx, T stretchx, const T *twr, const T *twi,
                       const T *kap, cudaStream_t st);
template <typename T>
cudaError_t launch_ddz(const ZTab<T> &tb, int nch, int L, const T *var, T *dvar, int n1, int nz,
                       const T *preset, const T *stretch, int filter, cudaStream_t st);
// One forward/adjoint record pair of the kernel integral (kernels.f90:209-358).
//   forward fields of solve b: fsn + fbase + b*fstride, six fields of F values each
//                              (xi_x, xi_z, v_x, v_z, acc_x, acc_z);
//   adjoint v_x of solve b:    adj + b*astride (v_z follows F values later);
//   out [nb][4][nz][nx] FP64:  kc, kvx, kvz, hes;  work [nb][4][nz][nx] of T.
template <typename T>
struct KAccArgs {
    int nx, nz, nb;
    const T *fsn;
    long long fbase, fstride;
    const T *adj;
    long long astride;
    double *out;
    T *work;
    const T *stretch, *twr, *twi, *kap;
    T stretchx;
    ZTab<T> z1;
    int nch, L;
    int colw;
};
template <typename T>
cudaError_t launch_kacc(const KAccArgs<T> &k, cudaStream_t st);

bool fft_size_supported(int n);

// ------------------------------------------------------------------------------------------
// 3-D displacement step (sparc_3d.cu).  Fields [nz][nb][ny][nx]; nxy = nx * ny.
struct S3Args {
    int nx, ny, nz, nb, npmlbot, npmltop, e_rad, flows;
    long long nxy;
};
template <typename T>
struct S3Bg {  // profiles in z ([nz]) and PML coefficients ([npmlbot + npmltop])
    const T *rhoinv, *rho0, *c2rho0, *gradp0_z, *gradrho0_z, *g, *source_dep, *az, *bz;
};
bool ddy_size_supported(int ny);
template <typename T>
cudaError_t launch_ddy(const T *var, T *dvar, int nplanes, int nx, int ny, T stretchy, const T *twr, const T *twi,
                       const T *kap, cudaStream_t st);
template <typename T>
cudaError_t launch_s3_stage_in(long long n6, const T *A, const T *SCR, T *X, T beta, long long np, const T *PV,
                               const T *SPV, T *PSI, cudaStream_t st);
template <typename T>
cudaError_t launch_s3_div(const S3Args &a, const S3Bg<T> &bg, const T *D1, const T *D2, T *D3, const T *XIZ,
                          const T *PSIVZ, T *SPSIVZ, T *PP, T *RHO, cudaStream_t st);
template <typename T>
cudaError_t launch_s3_adv(const S3Args &a, const T *D1, const T *D2, const T *D3, const T *V0X, const T *V0Y,
                          const T *V0Z, T *OUT, cudaStream_t st);
struct S3Lagr {  // the 7 LAGRANGE_INTERP weights of one step
    double w[7];
};
template <typename T>
cudaError_t launch_s3_rhs(const S3Args &a, const S3Bg<T> &bg, const T *X, T *SCR, const T *GX, const T *GY,
                          const T *GZ, const T *PSIP, T *SPSIP, const T *RHO, const T *PAT, T amp, const T *ADJ,
                          int k_obs, cudaStream_t st);
template <typename T>
cudaError_t launch_s3_adjsrc(long long lvl, long long nxy, const double *rows, int nrows, int i0, const S3Lagr &w,
                             double scale, T *ADJ, cudaStream_t st);
template <typename T>
cudaError_t launch_s3_record(long long F, const T *D1, const T *D2, const T *D3, const T *A, const T *SCR, T *snap,
                             cudaStream_t st);
template <typename T>
cudaError_t launch_s3_kacc_div(long long F, const T *D1, const T *D2, const T *D3, const T *snap, double *out,
                               cudaStream_t st);
template <typename T>
cudaError_t launch_s3_kacc_v(long long F, const T *D1, const T *D2, const T *D3, const T *va, double *out,
                             cudaStream_t st);
template <typename T>
cudaError_t launch_s3_end(const S3Args &a, T *A, const T *SCR, T dt, int filter, T *PV, const T *SPV,
                          cudaStream_t st);

// 2-D sponge step (option 5, sparc_sponge.cu).  Fields [nz][nb][nx].
struct S5Args {
    int nx, nz, nb, e_rad, i0, i1;  // filter columns [i0, i1]
    int npmlbot, npmltop;           // options 6 and 12
    int nf, npa;                    // fields of the state (5 or 8), PML auxiliaries (0, 2 or 4)
};
template <typename T>
struct S5Bg {  // profiles in z; az, bz [npmlbot + npmltop] (options 6, 12)
    const T *rhoinv, *rho0, *c2rho0, *gradp0_z, *gradrho0_z, *g, *source_dep, *sponge, *az, *bz;
    const T *box, *boz, *curl;  // option 12: background field and curlboy, [nz][nx]
};
template <typename T>
cudaError_t launch_s5_rhs(const S5Args &a, const S5Bg<T> &bg, const T *X, T *SCR, const T *DVX, const T *DVZ,
                          const T *GX, const T *GZ, const T *PAT, T amp, cudaStream_t st);
template <typename T>
cudaError_t launch_s6_rhs(const S5Args &a, const S5Bg<T> &bg, const T *X, T *SCR, const T *DVX, const T *DVZ,
                          const T *GX, const T *GZ, const T *PSI, T *SPSI, const T *PAT, T amp, cudaStream_t st);
template <typename T>
cudaError_t launch_s5_end(const S5Args &a, T *A, const T *SCR, T dt, T *PV, const T *SPV, cudaStream_t st);
template <typename T>
cudaError_t launch_s12_flux(const S5Args &a, const S5Bg<T> &bg, const T *X, T *FLUX, cudaStream_t st);
template <typename T>
cudaError_t launch_s12_rhs(const S5Args &a, const S5Bg<T> &bg, const T *X, T *SCR, const T *DVX, const T *DVZ,
                           const T *GX, const T *GZ, const T *DZBX, const T *DZF, const T *DXF, const T *DXBZ,
                           const T *PSI, T *SPSI, const T *PAT, T amp, cudaStream_t st);
template <typename T>
cudaError_t launch_s5_axpy(long long n, T *Y, const T *X, T a, cudaStream_t st);

struct ColMaps32;
// m32: tensor maps of A and SV with a 32-column box of nz/2 rows, or null; with them the
// specialised grids stage the first phase's inputs with TMA
template <int CW, int R>
cudaError_t launch_col_stage_band(const StepArgs<float> &a, const BandDev &bd, const ColMaps32 *m32, cudaStream_t st);
size_t col_band_smem_bytes(int nz, int nzpml, int R, int cw);
bool col_band_specialised(int nx, int nz, int cw, int R);  // compiled for this grid
int col_band_rows(int nz, int cw);  // rows per thread group (0: no banded pass for this depth / width)

template <typename T>
cudaError_t launch_end_step_stream(const StepArgs<T> &a, cudaStream_t st);
template <typename T>
size_t end_stream_smem_bytes(int nz);
cudaError_t launch_end_step_comp(const StepArgs<float> &a, cudaStream_t st);  // compensated (ALO) FP32

struct ColMaps;
template <int R>
cudaError_t launch_col_stage_band_tma(const ColMaps &maps, const StepArgs<float> &a, const BandDev &bd, cudaStream_t st);
size_t col_band_tma_smem_bytes(int nz, int R, int boxr);
int col_band_tma_rows(int nz);  // rows per thread group of the TMA-staged banded pass (0: unavailable)
template <typename T>
cudaError_t launch_col_stage_tma(const ColMaps &maps, const StepArgs<T> &a, cudaStream_t st);
template <typename T>
size_t col_tma_smem_bytes(int nz, int nch, int boxr);
template <typename T>
cudaError_t launch_end_step_tma(const ColMaps &maps, const StepArgs<T> &a, cudaStream_t st);

}  // namespace sparc
