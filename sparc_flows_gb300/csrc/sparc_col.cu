// sparc_col.cu -- column (z-direction) passes of the RK step.
//
// A block owns CW adjacent x-columns of one solve over the full depth; its threads are CW
// columns x NCH z-chunks.  Fields are staged in shared memory as [nz][CW] so every compact
// derivative (dbyd2.f:8-235) reads its +-2 halo from shared memory, and the chunked Thomas
// solves exchange only two boundary values per chunk (see sparc_common.cuh).
//
// col_stage_kernel, stage s (physics2d.f90:943-1094 in the order the data allow):
//   xi_z(s) -> d/dz (ibc 3, top value -dxi_x/dx * unstretch) + vertical PML psi_vz
//   div = dxi_x/dx + dxi_z/dz;  p = -c2rho0 div - gradp0_z xi_z;  rho = -rho0 div - gradrho0_z xi_z
//   p -> d/dz (ibc 2) + vertical PML psi_p;  RHS v_z = -rhoinv (dp/dz + rho g) - 2 v0 . grad v_z + source
//   v_x(s) -> d/dz (ibc 1): partial RHS v_x = -2 v0x dv_x/dx - 2 v0z dv_x/dz (completed by the next row pass)
// end_step_kernel: a += deltat scr; FILTER_VARS_2D (physics2d.f90:509-556); pmlvars += deltat
// scrpml; seismogram and partial-state records (driver.f90:386-417).
#include "sparc_common.cuh"

namespace sparc {

// Column-block geometry: CW columns per block, at most MAXNCH chunks of at most LMAX rows.
template <typename T>
struct ColCfg;
// Narrow blocks (8 columns = one 32-byte sector per row for FP32) so that several blocks are
// resident per SM and their barrier-separated phases overlap each other's memory latency.
template <>
struct ColCfg<float> {
    static constexpr int LMAX = 16, MAXNCH = 20;
};
template <>
struct ColCfg<double> {
    static constexpr int LMAX = 16, MAXNCH = 20;
};
template <typename T, int CW>
constexpr int min_blocks() { return CW <= 8 ? (sizeof(T) == 4 ? 4 : 2) : 1; }

template <typename T, int CW, int LMAX>
__global__ void __launch_bounds__(CW *ColCfg<T>::MAXNCH, (min_blocks<T, CW>())) col_stage_kernel(StepArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *B0 = reinterpret_cast<T *>(smem_raw);
    const int nz = a.nz, nx = a.nx, nch = a.nch;
    T *B1 = B0 + (size_t)nz * CW;
    T *YB = B1 + (size_t)nz * CW;  // 4 x [2 nch][CW]
    const int c = threadIdx.x % CW, j = threadIdx.x / CW;
    const int x = blockIdx.x * CW + c;
    const int b = blockIdx.y;
    const int k0 = j * a.L;
    const int n = min(a.L, nz - k0);
    const size_t F = (size_t)nz * nx;
    const T *Ab = a.A + (size_t)b * 4 * F;
    const int s = a.stage;
    const T bs = a.bs, bsm1 = a.bsm1;
    const int time = *a.d_time;
    T *yb0 = YB, *yb1 = YB + 2 * nch * CW, *yb2 = YB + 4 * nch * CW, *yb3 = YB + 6 * nch * CW;

    T xz[LMAX];
    // ---- A: xi_z at stage s (scr xi_z = v_z of stage s-1 with the RHS boundary zeros)
#pragma unroll
    for (int m = 0; m < LMAX; m++) {
        if (m < n) {
            const int k = k0 + m;
            const size_t q = (size_t)k * nx + x;
            T v = __ldg(Ab + F_XIZ * F + q);
            if (s >= 2) {
                T avz = __ldg(Ab + F_VZ * F + q);
                T t = (s == 2) ? avz : avz + bsm1 * __ldg(svp(a, a.slot_sm2, b, 1) + q);
                if (k == 0 || x == 0 || x == nx - 1) t = T(0);
                v += bs * t;
            }
            xz[m] = v;
            B0[k * CW + c] = v;
        }
    }
    __syncthreads();
    // ---- B: local solve of d xi_z/dz
    T y[LMAX];
    const T preset3 = -__ldg(a.TOPDX + (size_t)b * nx + x) * a.unstretch_top;
    const T ylast_yb0 = zlocal<T, LMAX>(a.z3, B0, CW, c, k0, n, nz, preset3, y);
    yb0[(2 * j) * CW + c] = y[0];
    yb0[(2 * j + 1) * CW + c] = ylast_yb0;
    __syncthreads();
    // ---- C: correct, vertical PML, divergence, pressure
    {
        T xl, xr;
        zcouple(a.z3, yb0, CW, c, j, nch, xl, xr);
#pragma unroll
        for (int m = 0; m < LMAX; m++) {
            if (m < n) {
                const int k = k0 + m;
                const size_t q = (size_t)k * nx + x;
                T dzz = zcorrect(a.z3, y[m], k, xl, xr) * __ldg(a.stretch + k);
                const int pi = pml_row(a, k);
                T fd = T(1);
                if (pi >= 0) {
                    const size_t qz = ((size_t)b * 2 * a.nzpml + pi) * nx + x;  // psi_vz
                    const size_t qb = (size_t)b * a.bgz + (size_t)pi * nx + x;
                    T ps = __ldg(a.PZ + qz);
                    if (s >= 2) ps += bs * __ldg(a.SPZ + (size_t)a.slot_sm1 * a.nb * 2 * a.nzpml * nx + qz);
                    a.SPZ[(size_t)a.slot_s * a.nb * 2 * a.nzpml * nx + qz] = __ldg(a.az + qb) * dzz + __ldg(a.bz + qb) * ps;
                    dzz += ps;
                    fd = __ldg(a.fdz + qb);
                }
                const T div = __ldg(a.DX + (size_t)b * F + q) + dzz;
                const T c2r = a.c2d ? __ldg(a.c2rho0 + (size_t)b * a.bg2 + q) : __ldg(a.c2rho0 + k);
                const T gp = __ldg(a.gp0 + k) * fd, gr = __ldg(a.gr0 + k) * fd;
                const T p = -c2r * div - gp * xz[m];
                const T rho = -__ldg(a.rho0 + k) * div - gr * xz[m];
                xz[m] = rho * __ldg(a.g + k);
                B1[k * CW + c] = p;
                a.P[(size_t)b * F + q] = p;
                T vx = __ldg(Ab + F_VX * F + q);
                if (s >= 2) vx += bs * __ldg(svp(a, a.slot_sm1, b, 0) + q);
                B0[k * CW + c] = vx;
            }
        }
    }
    __syncthreads();
    // ---- D: local solves of dp/dz (ibc 2, bottom value 0) and dv_x/dz (ibc 1)
    T y2[LMAX];
    const T ylast_yb1 = zlocal<T, LMAX>(a.z2, B1, CW, c, k0, n, nz, T(0), y);
    yb1[(2 * j) * CW + c] = y[0];
    yb1[(2 * j + 1) * CW + c] = ylast_yb1;
    if (a.flows) {
        const T y2last_yb2 = zlocal<T, LMAX>(a.z1, B0, CW, c, k0, n, nz, T(0), y2);
        yb2[(2 * j) * CW + c] = y2[0];
        yb2[(2 * j + 1) * CW + c] = y2last_yb2;
    }
    __syncthreads();
    // ---- E: gradient of p, RHS v_z without advection; advection of v_x along z
    {
        T xl, xr;
        zcouple(a.z2, yb1, CW, c, j, nch, xl, xr);
        T xl2 = T(0), xr2 = T(0);
        if (a.flows) zcouple(a.z1, yb2, CW, c, j, nch, xl2, xr2);
#pragma unroll
        for (int m = 0; m < LMAX; m++) {
            if (m < n) {
                const int k = k0 + m;
                const size_t q = (size_t)k * nx + x;
                T gpz = zcorrect(a.z2, y[m], k, xl, xr) * __ldg(a.stretch + k);
                const int pi = pml_row(a, k);
                if (pi >= 0) {
                    const size_t qz = (((size_t)b * 2 + 1) * a.nzpml + pi) * nx + x;  // psi_p
                    const size_t qb = (size_t)b * a.bgz + (size_t)pi * nx + x;
                    T ps = __ldg(a.PZ + qz);
                    if (s >= 2) ps += bs * __ldg(a.SPZ + (size_t)a.slot_sm1 * a.nb * 2 * a.nzpml * nx + qz);
                    a.SPZ[(size_t)a.slot_s * a.nb * 2 * a.nzpml * nx + qz] = __ldg(a.az + qb) * gpz + __ldg(a.bz + qb) * ps;
                    gpz += ps;
                }
                xz[m] = -__ldg(a.rhoinv + k) * (gpz + xz[m]);
                T rv = T(0);
                if (a.flows) {
                    const T dvxdz = zcorrect(a.z1, y2[m], k, xl2, xr2) * __ldg(a.stretch + k);
                    rv = __ldg(a.FXX + (size_t)b * F + q) - T(2) * a.fsign * __ldg(a.v0z + (size_t)b * a.bg2 + q) * dvxdz;
                }
                a.RVXP[(size_t)b * F + q] = rv;
                T vz = __ldg(Ab + F_VZ * F + q);
                if (s >= 2) vz += bs * __ldg(svp(a, a.slot_sm1, b, 1) + q);
                B1[k * CW + c] = vz;
            }
        }
    }
    __syncthreads();
    // ---- F: local solve of dv_z/dz
    if (a.flows) {
        const T y2last_yb3 = zlocal<T, LMAX>(a.z1, B1, CW, c, k0, n, nz, T(0), y2);
        yb3[(2 * j) * CW + c] = y2[0];
        yb3[(2 * j + 1) * CW + c] = y2last_yb3;
    }
    __syncthreads();
    // ---- G: finish RHS v_z (advection, source, boundary zeros)
    T xl2 = T(0), xr2 = T(0);
    if (a.flows) zcouple(a.z1, yb3, CW, c, j, nch, xl2, xr2);
    T forcing = T(0);
    const bool inject = (time <= a.src_until) && (time >= 0) && (time < a.ntab);
    if (inject && a.k_inj >= k0 && a.k_inj < k0 + n) {
        const double *w = a.src_w + (size_t)time * 7;
        const int i0 = a.src_idx[time];
        double f = 0.0;
        for (int jj = 0; jj < 7; jj++) {
            const int r = i0 + jj;
            if (r >= 0 && r < a.nrows && w[jj] != 0.0)
                f += w[jj] * (double)__ldg(a.src_rows + ((size_t)b * a.nrows + r) * nx + x);
        }
        forcing = T(f) * __ldg(a.inj_scale + (size_t)b * nx + x);
    }
    T *svz = svp(a, a.slot_s, b, 1);
#pragma unroll
    for (int m = 0; m < LMAX; m++) {
        if (m < n) {
            const int k = k0 + m;
            const size_t q = (size_t)k * nx + x;
            T r = xz[m];
            if (k == a.k_inj) r += forcing;
            if (a.flows) {
                const T dvzdz = zcorrect(a.z1, y2[m], k, xl2, xr2) * __ldg(a.stretch + k);
                r += __ldg(a.FXZ + (size_t)b * F + q) - T(2) * a.fsign * __ldg(a.v0z + (size_t)b * a.bg2 + q) * dvzdz;
            }
            if (k == 0 || x == 0 || x == nx - 1) r = T(0);
            svz[q] = r;
        }
    }
}

// FILTER_VARS_2D coefficients (physics2d.f90:517-522), already halved for the neighbours.
template <typename T>
__device__ __forceinline__ T filt11(const T *B, int CW, int c, int k)
{
    const T c0 = T(0.75390625), h1 = T(0.5 * 0.41015625), h2 = T(0.5 * -0.234375), h3 = T(0.5 * 0.087890625),
            h4 = T(0.5 * -0.01953125), h5 = T(0.5 * 0.001953125);
    return c0 * B[k * CW + c] + h1 * (B[(k - 1) * CW + c] + B[(k + 1) * CW + c]) +
           h2 * (B[(k - 2) * CW + c] + B[(k + 2) * CW + c]) + h3 * (B[(k - 3) * CW + c] + B[(k + 3) * CW + c]) +
           h4 * (B[(k - 4) * CW + c] + B[(k + 4) * CW + c]) + h5 * (B[(k - 5) * CW + c] + B[(k + 5) * CW + c]);
}

// Double-float helpers (Knuth TwoSum, FMA-based exact product) for the FP32 state update.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void df_add(float &hi, float &lo, float bh, float bl)
{
    float s, e;
    two_sum(hi, bh, s, e);
    e += lo + bl;
    hi = s + e;
    lo = e - (hi - s);
}

// h * (x + y) for double-float x, y and an exact binary coefficient h, added to (hi, lo).
__device__ __forceinline__ void df_axpy2(float &hi, float &lo, float h, float xh, float xl, float yh, float yl)
{
    float s, e;
    two_sum(xh, yh, s, e);
    e += xl + yl;
    const float p = h * s;
    const float pe = fmaf(h, s, -p) + h * e;
    df_add(hi, lo, p, pe);
}

// End of step for FP32 plans carrying low parts: a + deltat scr and FILTER_VARS_2D evaluated in
// double-float arithmetic, so the state keeps ~48 bits across the 3600 steps instead of
// accumulating one FP32 rounding of |a| per step.
__device__ __forceinline__ float filt11_df(const float *H, const float *Lo, int CW, int c, int k, float &lo)
{
    float hi = 0.f;
    lo = 0.f;
    const float c0 = 0.75390625f, h1 = 0.205078125f, h2 = -0.1171875f, h3 = 0.0439453125f, h4 = -0.009765625f,
                h5 = 0.0009765625f;
    {
        const float p = c0 * H[k * CW + c];
        const float pe = fmaf(c0, H[k * CW + c], -p) + c0 * Lo[k * CW + c];
        df_add(hi, lo, p, pe);
    }
    const float hs[5] = {h1, h2, h3, h4, h5};
#pragma unroll
    for (int j = 1; j <= 5; j++)
        df_axpy2(hi, lo, hs[j - 1], H[(k - j) * CW + c], Lo[(k - j) * CW + c], H[(k + j) * CW + c],
                 Lo[(k + j) * CW + c]);
    return hi;
}

template <int CW>
__device__ void end_step_compensated(const StepArgs<float> &a, float *B0, float *B1, int c, int x, int b, int k0, int n,
                                     bool record, int rec, float *snap)
{
    const int nz = a.nz, nx = a.nx;
    const size_t F = (size_t)nz * nx;
    float *Ab = a.A + (size_t)b * 4 * F;
    float *Lb = a.ALO + (size_t)b * 4 * F;
    const bool xf = a.filt_xall || ((x >= a.nh - 1) && (x <= nx - a.nh));
    for (int f = 0; f < 4; f++) {
        for (int m = 0; m < n; m++) {
            const int k = k0 + m;
            const size_t q = (size_t)k * nx + x;
            float sc;
            if (f == F_XIX || f == F_XIZ) {
                const int cc = (f == F_XIX) ? 0 : 1;
                sc = Ab[(f == F_XIX ? F_VX : F_VZ) * F + q] + a.bs * svp(a, a.slot_sm1, b, cc)[q];
                if (k == 0 || x == 0 || x == nx - 1) sc = 0.f;
            } else {
                sc = svp(a, a.slot_s, b, f == F_VX ? 0 : 1)[q];
            }
            float hi = Ab[f * F + q], lo = Lb[f * F + q];
            const float d = a.dt * sc;
            df_add(hi, lo, d, fmaf(a.dt, sc, -d));
            B0[k * CW + c] = hi;
            B1[k * CW + c] = lo;
        }
        __syncthreads();
        for (int m = 0; m < n; m++) {
            const int k = k0 + m;
            const size_t q = (size_t)k * nx + x;
            float hi = B0[k * CW + c], lo = B1[k * CW + c];
            if (xf && k >= a.filt_k0 && k <= nz - 2) {
                if (k >= 5 && k <= nz - 6) {
                    hi = filt11_df(B0, B1, CW, c, k, lo);
                } else {
                    float h = 0.f, l = 0.f;
                    df_axpy2(h, l, 0.5f, B0[(k + 1) * CW + c], B1[(k + 1) * CW + c], B0[(k - 1) * CW + c],
                             B1[(k - 1) * CW + c]);
                    hi = h;
                    lo = l;
                }
            }
            Ab[f * F + q] = hi;
            Lb[f * F + q] = lo;
            if (snap) snap[(size_t)f * F + q] = hi;
            if (record && f == F_VZ && k == a.k_obs && a.seis) a.seis[((size_t)b * a.nrec_cap + rec) * nx + x] = hi;
        }
        __syncthreads();
    }
}

template <typename T, int CW, int LMAX>
__global__ void __launch_bounds__(CW *ColCfg<T>::MAXNCH, (min_blocks<T, CW>())) end_step_kernel(StepArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *B0 = reinterpret_cast<T *>(smem_raw);
    const int nz = a.nz, nx = a.nx;
    const int c = threadIdx.x % CW, j = threadIdx.x / CW;
    const int x = blockIdx.x * CW + c;
    const int b = blockIdx.y;
    const int k0 = j * a.L;
    const int n = min(a.L, nz - k0);
    const size_t F = (size_t)nz * nx;
    T *Ab = a.A + (size_t)b * 4 * F;
    const int time = *a.d_time;
    const int rec = (a.steps_out > 0) ? time / a.steps_out - a.rec0 : 0;  // slot in the record window
    const bool record = a.steps_out > 0 && time % a.steps_out == 0 && rec >= 0 && rec < a.nrec_cap && time >= 0;
    const bool xf = a.filt_xall || ((x >= a.nh - 1) && (x <= nx - a.nh));
    T *snap = record && a.snaps ? a.snaps + ((size_t)b * a.nrec_cap + rec) * 6 * F : nullptr;
    if constexpr (sizeof(T) == 4) {
        if (a.ALO) {
            end_step_compensated<CW>(a, B0, B0 + (size_t)nz * CW, c, x, b, k0, n, record, rec, snap);
            goto aux;
        }
    }
    for (int f = 0; f < 4; f++) {
        for (int m = 0; m < n; m++) {
            {
                const int k = k0 + m;
                const size_t q = (size_t)k * nx + x;
                T sc;
                if (f == F_XIX || f == F_XIZ) {  // scr xi = v of stage 5 with the RHS boundary zeros
                    const int cc = (f == F_XIX) ? 0 : 1;
                    sc = Ab[(f == F_XIX ? F_VX : F_VZ) * F + q] + a.bs * svp(a, a.slot_sm1, b, cc)[q];
                    if (k == 0 || x == 0 || x == nx - 1) sc = T(0);
                } else {
                    sc = svp(a, a.slot_s, b, f == F_VX ? 0 : 1)[q];
                }
                B0[k * CW + c] = Ab[f * F + q] + a.dt * sc;
            }
        }
        __syncthreads();
        for (int m = 0; m < n; m++) {
            {
                const int k = k0 + m;
                const size_t q = (size_t)k * nx + x;
                T out = B0[k * CW + c];
                if (xf && k >= a.filt_k0 && k <= nz - 2) {
                    if (k >= 5 && k <= nz - 6) out = filt11(B0, CW, c, k);
                    else out = T(0.5) * (B0[(k + 1) * CW + c] + B0[(k - 1) * CW + c]);
                }
                Ab[f * F + q] = out;
                if (snap) snap[(size_t)f * F + q] = out;
                if (record && f == F_VZ && k == a.k_obs && a.seis)
                    a.seis[((size_t)b * a.nrec_cap + rec) * nx + x] = out;
            }
        }
        __syncthreads();
    }
aux:
    for (int m = 0; m < n; m++) {
        {
            const int k = k0 + m;
            const size_t q = (size_t)k * nx + x;
            const int pi = pml_row(a, k);
            if (pi >= 0) {
                for (int cc = 0; cc < 2; cc++) {
                    const size_t qz = (((size_t)b * 2 + cc) * a.nzpml + pi) * nx + x;
                    a.PZ[qz] += a.dt * a.SPZ[(size_t)a.slot_s * a.nb * 2 * a.nzpml * nx + qz];
                }
            }
            if (snap) {
                snap[4 * F + q] = svp(a, a.slot_s, b, 0)[q];
                snap[5 * F + q] = svp(a, a.slot_s, b, 1)[q];
            }
        }
    }
}

// Generic compact derivative of n1 columns: dvar = stretch .* dbyd2(var), optional
// FILTER_VAR_Z (kernels.f90:891-928) afterwards.
template <typename T, int CW, int LMAX>
__global__ void __launch_bounds__(CW *ColCfg<T>::MAXNCH, (min_blocks<T, CW>())) ddz_kernel(ZTab<T> tb, int nch, int L, const T *__restrict__ var,
                                                         T *__restrict__ dvar, int n1, int nz,
                                                         const T *__restrict__ preset,
                                                         const T *__restrict__ stretch, int filter)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *B0 = reinterpret_cast<T *>(smem_raw);
    T *YB = B0 + (size_t)nz * CW;
    const int c = threadIdx.x % CW, j = threadIdx.x / CW;
    const int x = blockIdx.x * CW + c;
    const bool valid = x < n1;
    const int xs = valid ? x : n1 - 1;
    const int k0 = j * L;
    const int n = min(L, nz - k0);
#pragma unroll
    for (int m = 0; m < LMAX; m++)
        if (m < n) B0[(k0 + m) * CW + c] = var[(size_t)(k0 + m) * n1 + xs];
    __syncthreads();
    T y[LMAX];
    const T pre = preset ? preset[xs] : T(0);
    const T ylast_YB = zlocal<T, LMAX>(tb, B0, CW, c, k0, n, nz, pre, y);
    YB[(2 * j) * CW + c] = y[0];
    YB[(2 * j + 1) * CW + c] = ylast_YB;
    __syncthreads();
    T xl, xr;
    zcouple(tb, YB, CW, c, j, nch, xl, xr);
#pragma unroll
    for (int m = 0; m < LMAX; m++) {
        if (m < n) {
            const int k = k0 + m;
            y[m] = zcorrect(tb, y[m], k, xl, xr) * (stretch ? __ldg(stretch + k) : T(1));
        }
    }
    if (filter) {
        __syncthreads();
#pragma unroll
        for (int m = 0; m < LMAX; m++)
            if (m < n) B0[(k0 + m) * CW + c] = y[m];
        __syncthreads();
#pragma unroll
        for (int m = 0; m < LMAX; m++) {
            if (m < n) {
                const int k = k0 + m;
                if (k >= 1 && k <= 4) y[m] = T(0.5) * (B0[(k + 1) * CW + c] + B0[(k - 1) * CW + c]);
                else if (k >= 5 && k <= nz - 6) y[m] = filt11(B0, CW, c, k);
                else if (k >= nz - 5 && k <= nz - 2) y[m] = T(0.5) * (B0[(k + 1) * CW + c] + B0[(k - 1) * CW + c]);
            }
        }
    }
    if (valid) {
#pragma unroll
        for (int m = 0; m < LMAX; m++)
            if (m < n) dvar[(size_t)(k0 + m) * n1 + x] = y[m];
    }
}


// Kernel integral, z-derivatives and FP64 accumulation of one record pair (kernels.f90:293-358):
//   kc  += div(f_xi) div(a_v),  kvx += d_x f_vx a_vx + d_x f_vz a_vz,
//   kvz += d_z f_vx a_vx + d_z f_vz a_vz,  hes += f_acc_x^2 + f_acc_z^2,
// with every z-derivative taken as ddzkern (ibc 1, times stretch, then FILTER_VAR_Z,
// kernels.f90:648-661, 891-928).  The x-derivatives come from kacc_row_kernel (work).
template <typename T, int CW, int LMAX>
__device__ __forceinline__ void kacc_dz(const KAccArgs<T> &a, const T *src, T *B0, T *B1, T *YB, int c, int j,
                                        int x, int k0, int n, T (&out)[LMAX])
{
    const int nz = a.nz, nx = a.nx;
    for (int m = 0; m < n; m++) B0[(k0 + m) * CW + c] = src[(size_t)(k0 + m) * nx + x];
    __syncthreads();
    T y[LMAX];
    const T last = zlocal<T, LMAX>(a.z1, B0, CW, c, k0, n, nz, T(0), y);
    YB[(2 * j) * CW + c] = y[0];
    YB[(2 * j + 1) * CW + c] = last;
    __syncthreads();
    T xl, xr;
    zcouple(a.z1, YB, CW, c, j, a.nch, xl, xr);
#pragma unroll
    for (int m = 0; m < LMAX; m++)
        if (m < n) B1[(k0 + m) * CW + c] = zcorrect(a.z1, y[m], k0 + m, xl, xr) * __ldg(a.stretch + k0 + m);
    __syncthreads();
#pragma unroll
    for (int m = 0; m < LMAX; m++) {
        if (m < n) {
            const int k = k0 + m;
            T v = B1[k * CW + c];
            if ((k >= 1 && k <= 4) || (k >= nz - 5 && k <= nz - 2)) v = T(0.5) * (B1[(k + 1) * CW + c] + B1[(k - 1) * CW + c]);
            else if (k >= 5 && k <= nz - 6) v = filt11(B1, CW, c, k);
            out[m] = v;
        }
    }
    __syncthreads();
}

template <typename T, int CW, int LMAX>
__global__ void __launch_bounds__(CW *ColCfg<T>::MAXNCH, (min_blocks<T, CW>())) kacc_col_kernel(KAccArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *B0 = reinterpret_cast<T *>(smem_raw);
    const int nz = a.nz, nx = a.nx;
    T *B1 = B0 + (size_t)nz * CW;
    T *YB = B1 + (size_t)nz * CW;
    const int c = threadIdx.x % CW, j = threadIdx.x / CW;
    const int x = blockIdx.x * CW + c;
    const int b = blockIdx.y;
    const int k0 = j * a.L;
    const int n = min(a.L, nz - k0);
    const size_t F = (size_t)nz * nx;
    const T *f = a.fsn + a.fbase + (size_t)b * a.fstride;
    const T *avx = a.adj + (size_t)b * a.astride, *avz = avx + F;
    const T *w = a.work + (size_t)b * 4 * F;
    double *o = a.out + (size_t)b * 4 * F;
    T divf[LMAX], d[LMAX];
    kacc_dz<T, CW, LMAX>(a, f + 1 * F, B0, B1, YB, c, j, x, k0, n, divf);  // d_z f_xi_z
#pragma unroll
    for (int m = 0; m < LMAX; m++)
        if (m < n) divf[m] += w[0 * F + (size_t)(k0 + m) * nx + x];
    kacc_dz<T, CW, LMAX>(a, avz, B0, B1, YB, c, j, x, k0, n, d);  // d_z a_vz
#pragma unroll
    for (int m = 0; m < LMAX; m++) {
        if (m < n) {
            const size_t q = (size_t)(k0 + m) * nx + x;
            const T diva = d[m] + w[1 * F + q];
            o[0 * F + q] += (double)divf[m] * (double)diva;
        }
    }
    kacc_dz<T, CW, LMAX>(a, f + 2 * F, B0, B1, YB, c, j, x, k0, n, divf);  // d_z f_vx
    kacc_dz<T, CW, LMAX>(a, f + 3 * F, B0, B1, YB, c, j, x, k0, n, d);     // d_z f_vz
#pragma unroll
    for (int m = 0; m < LMAX; m++) {
        if (m < n) {
            const size_t q = (size_t)(k0 + m) * nx + x;
            const double ax = (double)avx[q], az = (double)avz[q];
            o[1 * F + q] += (double)w[2 * F + q] * ax + (double)w[3 * F + q] * az;
            o[2 * F + q] += (double)divf[m] * ax + (double)d[m] * az;
            const double fx = (double)f[4 * F + q], fz = (double)f[5 * F + q];
            o[3 * F + q] += fz * fz + fx * fx;
        }
    }
}

template <typename T>
cudaError_t launch_kacc_row(const KAccArgs<T> &a, cudaStream_t st);

template <typename T, int CW>
static cudaError_t launch_kacc_cw(const KAccArgs<T> &a, cudaStream_t st)
{
    constexpr int LMAX = ColCfg<T>::LMAX;
    const size_t smem = ((size_t)2 * a.nz * CW + (size_t)2 * a.nch * CW) * sizeof(T);
    auto k = kacc_col_kernel<T, CW, LMAX>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid(a.nx / CW, a.nb);
    k<<<grid, CW * a.nch, smem, st>>>(a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_kacc(const KAccArgs<T> &a, cudaStream_t st)
{
    const int cw = a.colw == 32 ? 32 : 8;
    if (a.nx % cw || a.L > ColCfg<T>::LMAX || a.nch > ColCfg<T>::MAXNCH) return cudaErrorInvalidValue;
    cudaError_t e = launch_kacc_row<T>(a, st);
    if (e != cudaSuccess) return e;
    return cw == 32 ? launch_kacc_cw<T, 32>(a, st) : launch_kacc_cw<T, 8>(a, st);
}
template cudaError_t launch_kacc<float>(const KAccArgs<float> &, cudaStream_t);
template cudaError_t launch_kacc<double>(const KAccArgs<double> &, cudaStream_t);

template <typename T, int CW>
static cudaError_t launch_col_stage_cw(const StepArgs<T> &a, cudaStream_t st)
{
    constexpr int LMAX = ColCfg<T>::LMAX;
    const size_t smem = ((size_t)2 * a.nz * CW + (size_t)8 * a.nch * CW) * sizeof(T);
    auto k = col_stage_kernel<T, CW, LMAX>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid(a.nx / CW, a.nb);
    k<<<grid, CW * a.nch, smem, st>>>(a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_col_stage(const StepArgs<T> &a, cudaStream_t st)
{
    if (a.nx % a.colw || a.L > ColCfg<T>::LMAX || a.nch > ColCfg<T>::MAXNCH) return cudaErrorInvalidValue;
    switch (a.colw) {
        case 32: return launch_col_stage_cw<T, 32>(a, st);
        case 8: return launch_col_stage_cw<T, 8>(a, st);
        case 4: return launch_col_stage_cw<T, 4>(a, st);
        default: return cudaErrorInvalidValue;
    }
}

template <typename T, int CW>
static cudaError_t launch_end_step_cw(const StepArgs<T> &a, cudaStream_t st)
{
    constexpr int LMAX = ColCfg<T>::LMAX;
    const size_t smem = (size_t)a.nz * CW * sizeof(T) * (a.ALO ? 2 : 1);
    auto k = end_step_kernel<T, CW, LMAX>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid(a.nx / CW, a.nb);
    k<<<grid, CW * a.nch, smem, st>>>(a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_end_step(const StepArgs<T> &a, cudaStream_t st)
{
    const int cw = a.colw == 32 ? 32 : 8;
    if (a.nx % cw || a.L > ColCfg<T>::LMAX || a.nch > ColCfg<T>::MAXNCH) return cudaErrorInvalidValue;
    return cw == 32 ? launch_end_step_cw<T, 32>(a, st) : launch_end_step_cw<T, 8>(a, st);
}

template <typename T, int CW>
static cudaError_t launch_ddz_cw(const ZTab<T> &tb, int nch, int L, const T *var, T *dvar, int n1, int nz,
                                 const T *preset, const T *stretch, int filter, cudaStream_t st)
{
    constexpr int LMAX = ColCfg<T>::LMAX;
    const size_t smem = ((size_t)nz * CW + (size_t)2 * nch * CW) * sizeof(T);
    auto k = ddz_kernel<T, CW, LMAX>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid((n1 + CW - 1) / CW);
    k<<<grid, CW * nch, smem, st>>>(tb, nch, L, var, dvar, n1, nz, preset, stretch, filter);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_ddz(const ZTab<T> &tb, int nch, int L, const T *var, T *dvar, int n1, int nz, const T *preset,
                       const T *stretch, int filter, cudaStream_t st)
{
    if (L > ColCfg<T>::LMAX || nch > ColCfg<T>::MAXNCH || n1 <= 0) return cudaErrorInvalidValue;
    // many columns (a 3-D field: nb * ny * nx): 32 columns per block, four 32-byte sectors per
    // row access; few (a 2-D row of nx): 8, so that enough blocks exist
    if (n1 % 32 == 0 && n1 >= 32 * 152 * 8)
        return launch_ddz_cw<T, 32>(tb, nch, L, var, dvar, n1, nz, preset, stretch, filter, st);
    return launch_ddz_cw<T, 8>(tb, nch, L, var, dvar, n1, nz, preset, stretch, filter, st);
}

template cudaError_t launch_col_stage<float>(const StepArgs<float> &, cudaStream_t);
template cudaError_t launch_col_stage<double>(const StepArgs<double> &, cudaStream_t);
template cudaError_t launch_end_step<float>(const StepArgs<float> &, cudaStream_t);
template cudaError_t launch_end_step<double>(const StepArgs<double> &, cudaStream_t);
template cudaError_t launch_ddz<float>(const ZTab<float> &, int, int, const float *, float *, int, int,
                                       const float *, const float *, int, cudaStream_t);
template cudaError_t launch_ddz<double>(const ZTab<double> &, int, int, const double *, double *, int, int,
                                        const double *, const double *, int, cudaStream_t);

}  // namespace sparc
