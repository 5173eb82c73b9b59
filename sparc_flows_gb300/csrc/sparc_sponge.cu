// sparc_sponge.cu -- kernels of the 2-D velocity-pressure-density steps: option 5
// (MP_QUIET_SPONGE_2D, physics2d.f90:1099-1137, a sponge layer), option 6 (MP_QUIET_PML_2D,
// physics2d.f90:662-713, the vertical PML) and option 12 (MP_MHD_PML_2d, physics2d.f90:411-474,
// the same with a background magnetic field: b_x, b_z in the state, the induction equation,
// the Lorentz force, and the magnetic part of PML_BOUNDARY_ACCOUNTING_2D, 1162-1200).
//
// Fields are [nz][nb][nx] (level-major, the batch inside a level, as the 3-D step), the state
// five of them: rho, v_x, v_y (zero in 2-D), v_z, p (initialize.f90:500-504).  One RK stage:
// X = A + beta SCR (s3_stage_in), x passes of v_x and p (the spectral row pass), z passes of
// v_z and p (the compact column solve, ibc 1), then s5_rhs_kernel: continuity, momentum with
// pressure gradient, buoyancy, sponge and source, pressure; the top and bottom rows of the
// momentum and pressure RHS zero.  End of step: s5_end_kernel, a += dt scr and FILTER_VARS_2D
// (physics2d.f90:509-560) down each column from a register window, in place.
#include "sparc_common.cuh"

namespace sparc {

constexpr int S5_THREADS = 256;

template <typename T>
__global__ void __launch_bounds__(S5_THREADS) s5_rhs_kernel(S5Args a, S5Bg<T> bg, const T *__restrict__ X,
                                                            T *__restrict__ SCR, const T *__restrict__ DVX,
                                                            const T *__restrict__ DVZ, const T *__restrict__ GX,
                                                            const T *__restrict__ GZ, const T *__restrict__ PAT, T amp)
{
    const long long lvl = (long long)a.nb * a.nx, n = lvl * a.nz, F = n;
    const long long stride = (long long)gridDim.x * S5_THREADS;
    for (long long i = (long long)blockIdx.x * S5_THREADS + threadIdx.x; i < n; i += stride) {
        const int k = (int)(i / lvl);
        const long long r = i - (long long)k * lvl;
        const T rho = X[i], vx = X[F + i], vz = X[3 * F + i], p = X[4 * F + i];
        const T sp = bg.sponge[k], ri = bg.rhoinv[k];
        const T div = DVX[i] + DVZ[i];
        SCR[i] = -bg.gradrho0_z[k] * vz - bg.rho0[k] * div - sp * rho;
        T rx = -ri * GX[i] - sp * vx;
        T rz = -ri * GZ[i] - sp * vz;
        rz = rz - rho * bg.g[k] * ri;
        if (abs(k - a.e_rad) <= 4) rz = rz + (PAT[r] * amp) * bg.source_dep[k];
        T rp = -bg.c2rho0[k] * div - vz * bg.gradp0_z[k] - sp * p;
        if (k == 0 || k == a.nz - 1) rx = rz = rp = T(0);
        SCR[F + i] = rx;
        SCR[2 * F + i] = T(0);
        SCR[3 * F + i] = rz;
        SCR[4 * F + i] = rp;
    }
}

// Option 6, MP_QUIET_PML_2D (physics2d.f90:662-713): the same formulation with the vertical PML
// (PML_BOUNDARY_ACCOUNTING_2D, physics2d.f90:1142-1160: psi_p and psi_vz on the PML rows,
// stored [2][npml][nb][nx]) and no sponge; the top and bottom rows of all four RHS zero.
template <typename T>
__global__ void __launch_bounds__(S5_THREADS) s6_rhs_kernel(S5Args a, S5Bg<T> bg, const T *__restrict__ X,
                                                            T *__restrict__ SCR, const T *__restrict__ DVX,
                                                            const T *__restrict__ DVZ, const T *__restrict__ GX,
                                                            const T *__restrict__ GZ, const T *__restrict__ PSI,
                                                            T *__restrict__ SPSI, const T *__restrict__ PAT, T amp)
{
    const long long lvl = (long long)a.nb * a.nx, n = lvl * a.nz, F = n;
    const long long P = (long long)(a.npmlbot + a.npmltop) * lvl;
    const long long stride = (long long)gridDim.x * S5_THREADS;
    for (long long i = (long long)blockIdx.x * S5_THREADS + threadIdx.x; i < n; i += stride) {
        const int k = (int)(i / lvl);
        const long long r = i - (long long)k * lvl;
        T gz = GZ[i], dvz = DVZ[i];
        int pi = -1;
        if (k < a.npmlbot) pi = k;
        else if (k >= a.nz - a.npmltop) pi = a.npmlbot + (k - (a.nz - a.npmltop));
        if (pi >= 0) {
            const long long m = (long long)pi * lvl + r;
            const T pp = PSI[m], pv = PSI[P + m];
            SPSI[m] = bg.az[pi] * gz + bg.bz[pi] * pp;
            gz = gz + pp;
            SPSI[P + m] = bg.az[pi] * dvz + bg.bz[pi] * pv;
            dvz = dvz + pv;
        }
        const T rho = X[i], vz = X[3 * F + i];
        const T ri = bg.rhoinv[k];
        const T div = DVX[i] + dvz;
        T rc = -bg.rho0[k] * div - bg.gradrho0_z[k] * vz;
        T rp = -bg.c2rho0[k] * div - vz * bg.gradp0_z[k];
        T rx = -ri * GX[i];
        T rz = -ri * (gz + rho * bg.g[k]);
        if (abs(k - a.e_rad) <= 4) rz = rz + (PAT[r] * amp) * bg.source_dep[k];
        if (k == 0 || k == a.nz - 1) rc = rp = rx = rz = T(0);
        SCR[i] = rc;
        SCR[F + i] = rx;
        SCR[2 * F + i] = T(0);
        SCR[3 * F + i] = rz;
        SCR[4 * F + i] = rp;
    }
}

template <typename T>
__global__ void __launch_bounds__(S5_THREADS) s5_axpy_kernel(long long n, T *__restrict__ Y, const T *__restrict__ X,
                                                             T a)
{
    const long long stride = (long long)gridDim.x * S5_THREADS;
    for (long long i = (long long)blockIdx.x * S5_THREADS + threadIdx.x; i < n; i += stride) Y[i] = Y[i] + a * X[i];
}

// One thread per (field, column): a += dt scr, then FILTER_VARS_2D: the 11-point filter on rows
// 5 .. nz-6 and two-point means on rows nz-5 .. nz-2 (0-based) of the updated column, written
// to rows 5 .. nz-2 for x in [i0, i1] (HORIZONTAL_PMLS) from an 11-value register window.
template <typename T>
__global__ void __launch_bounds__(S5_THREADS) s5_end_kernel(S5Args a, T *__restrict__ A, const T *__restrict__ SCR,
                                                            T dt)
{
    const long long lvl = (long long)a.nb * a.nx;
    const long long cols = (long long)a.nf * lvl, F = lvl * a.nz;
    const long long c = (long long)blockIdx.x * S5_THREADS + threadIdx.x;
    if (c >= cols) return;
    const int v = (int)(c / lvl);
    const long long r = c - (long long)v * lvl;
    const int x = (int)(r % a.nx);
    T *col = A + (long long)v * F + r;
    const T *sc = SCR + (long long)v * F + r;
    const int nz = a.nz;
    for (int k = 0; k < nz; k++) col[(long long)k * lvl] = col[(long long)k * lvl] + dt * sc[(long long)k * lvl];
    if (x < a.i0 || x > a.i1 || nz < 11) return;
    const T c0 = T(0.75390625), h1 = T(0.5 * 0.41015625), h2 = T(0.5 * -0.234375), h3 = T(0.5 * 0.087890625),
            h4 = T(0.5 * -0.01953125), h5 = T(0.5 * 0.001953125);
    T w[11];  // rows k-5 .. k+5 of the updated column, for the row k being written
#pragma unroll
    for (int j = 0; j < 11; j++) w[j] = col[(long long)j * lvl];
    for (int k = 5; k <= nz - 2; k++) {
        T out;
        if (k <= nz - 6)
            out = c0 * w[5] + h1 * (w[4] + w[6]) + h2 * (w[3] + w[7]) + h3 * (w[2] + w[8]) + h4 * (w[1] + w[9]) +
                  h5 * (w[0] + w[10]);
        else
            out = T(0.5) * (w[6] + w[4]);
#pragma unroll
        for (int j = 0; j < 10; j++) w[j] = w[j + 1];
        if (k + 6 < nz) w[10] = col[(long long)(k + 6) * lvl];
        col[(long long)k * lvl] = out;
    }
}

// Option 12: the induction flux -(v_x boz - v_z box) of the stage input (physics2d.f90:421).
template <typename T>
__global__ void __launch_bounds__(S5_THREADS) s12_flux_kernel(S5Args a, S5Bg<T> bg, const T *__restrict__ X,
                                                              T *__restrict__ FLUX)
{
    const long long lvl = (long long)a.nb * a.nx, n = lvl * a.nz, F = n;
    const long long stride = (long long)gridDim.x * S5_THREADS;
    for (long long i = (long long)blockIdx.x * S5_THREADS + threadIdx.x; i < n; i += stride) {
        const int k = (int)(i / lvl);
        const int x = (int)((i - (long long)k * lvl) % a.nx);
        const long long q = (long long)k * a.nx + x;
        FLUX[i] = -(X[F + i] * bg.boz[q] - X[3 * F + i] * bg.box[q]);
    }
}

// Option 12, MP_MHD_PML_2d (physics2d.f90:411-474) with PML_BOUNDARY_ACCOUNTING_2D (1142-1200):
// psi_p, psi_vz as option 6; dv_z/dz (with its PML term) replaced on the PML rows 1..npmlbot-1
// and nz-npmltop..nz-2 (0-based) by the mean of its two neighbours; psi of d flux/dz and of
// d b_x/dz.  PML auxiliaries [4][npml][nb][nx]: psi_p, psi_vz, psi_flux, psi_dzbx.  The top and
// bottom rows of all eight RHS zero.
template <typename T>
__global__ void __launch_bounds__(S5_THREADS) s12_rhs_kernel(S5Args a, S5Bg<T> bg, const T *__restrict__ X,
                                                             T *__restrict__ SCR, const T *__restrict__ DVX,
                                                             const T *__restrict__ DVZ, const T *__restrict__ GX,
                                                             const T *__restrict__ GZ, const T *__restrict__ DZBX,
                                                             const T *__restrict__ DZF, const T *__restrict__ DXF,
                                                             const T *__restrict__ DXBZ, const T *__restrict__ PSI,
                                                             T *__restrict__ SPSI, const T *__restrict__ PAT, T amp)
{
    const long long lvl = (long long)a.nb * a.nx, n = lvl * a.nz, F = n;
    const long long P = (long long)(a.npmlbot + a.npmltop) * lvl;
    const long long stride = (long long)gridDim.x * S5_THREADS;
    auto pml = [&](int k) {
        if (k < a.npmlbot) return k;
        if (k >= a.nz - a.npmltop) return a.npmlbot + (k - (a.nz - a.npmltop));
        return -1;
    };
    for (long long i = (long long)blockIdx.x * S5_THREADS + threadIdx.x; i < n; i += stride) {
        const int k = (int)(i / lvl);
        const long long r = i - (long long)k * lvl;
        const int x = (int)(r % a.nx);
        T gz = GZ[i], dzf = DZF[i], dzbx = DZBX[i];
        T dvz = DVZ[i];
        const int pi = pml(k);
        if (pi >= 0) {
            const long long m = (long long)pi * lvl + r;
            const T pp = PSI[m], pv = PSI[P + m], pf = PSI[2 * P + m], pb = PSI[3 * P + m];
            SPSI[m] = bg.az[pi] * gz + bg.bz[pi] * pp;
            gz = gz + pp;
            SPSI[P + m] = bg.az[pi] * dvz + bg.bz[pi] * pv;
            dvz = dvz + pv;
            SPSI[2 * P + m] = bg.az[pi] * dzf + bg.bz[pi] * pf;
            dzf = dzf + pf;
            SPSI[3 * P + m] = bg.az[pi] * dzbx + bg.bz[pi] * pb;
            dzbx = dzbx + pb;
        }
        if ((k >= 1 && k <= a.npmlbot - 1) || (k >= a.nz - a.npmltop && k <= a.nz - 2)) {
            T nb2[2];
#pragma unroll
            for (int j = 0; j < 2; j++) {
                const int kk = j == 0 ? k - 1 : k + 1;
                const int pk = pml(kk);
                T v = DVZ[i + (j == 0 ? -lvl : lvl)];
                if (pk >= 0) v = v + PSI[P + (long long)pk * lvl + r];
                nb2[j] = v;
            }
            dvz = T(0.5) * (nb2[0] + nb2[1]);
        }
        const long long q = (long long)k * a.nx + x;
        const T rho = X[i], vz = X[3 * F + i], bxs = X[5 * F + i], bzs = X[7 * F + i];
        const T ri = bg.rhoinv[k], cu = bg.curl[q];
        const T div = DVX[i] + dvz;
        const T cur = dzbx - DXBZ[i];
        const T t1 = bg.boz[q] * cur + bzs * cu;
        const T t3 = -bg.box[q] * cur - bxs * cu;
        T rc = -bg.gradrho0_z[k] * vz - bg.rho0[k] * div;
        T rx = ri * (t1 - GX[i]);
        T rz = ri * (t3 - gz);
        rz = rz - ri * rho * bg.g[k];
        if (abs(k - a.e_rad) <= 4) rz = rz + (PAT[r] * amp) * bg.source_dep[k];
        T rp = -bg.c2rho0[k] * div - vz * bg.gradp0_z[k];
        T rbx = -dzf, rbz = DXF[i];
        if (k == 0 || k == a.nz - 1) rc = rx = rz = rp = rbx = rbz = T(0);
        SCR[i] = rc;
        SCR[F + i] = rx;
        SCR[2 * F + i] = T(0);
        SCR[3 * F + i] = rz;
        SCR[4 * F + i] = rp;
        SCR[5 * F + i] = rbx;
        SCR[6 * F + i] = T(0);
        SCR[7 * F + i] = rbz;
    }
}

static unsigned s5_grid(long long n)
{
    const long long g = (n + S5_THREADS - 1) / S5_THREADS;
    return (unsigned)(g < 152LL * 16 ? g : 152LL * 16);
}

template <typename T>
cudaError_t launch_s5_rhs(const S5Args &a, const S5Bg<T> &bg, const T *X, T *SCR, const T *DVX, const T *DVZ,
                          const T *GX, const T *GZ, const T *PAT, T amp, cudaStream_t st)
{
    const long long n = (long long)a.nb * a.nx * a.nz;
    s5_rhs_kernel<T><<<s5_grid(n), S5_THREADS, 0, st>>>(a, bg, X, SCR, DVX, DVZ, GX, GZ, PAT, amp);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_s6_rhs(const S5Args &a, const S5Bg<T> &bg, const T *X, T *SCR, const T *DVX, const T *DVZ,
                          const T *GX, const T *GZ, const T *PSI, T *SPSI, const T *PAT, T amp, cudaStream_t st)
{
    const long long n = (long long)a.nb * a.nx * a.nz;
    s6_rhs_kernel<T><<<s5_grid(n), S5_THREADS, 0, st>>>(a, bg, X, SCR, DVX, DVZ, GX, GZ, PSI, SPSI, PAT, amp);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_s12_flux(const S5Args &a, const S5Bg<T> &bg, const T *X, T *FLUX, cudaStream_t st)
{
    const long long n = (long long)a.nb * a.nx * a.nz;
    s12_flux_kernel<T><<<s5_grid(n), S5_THREADS, 0, st>>>(a, bg, X, FLUX);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_s12_rhs(const S5Args &a, const S5Bg<T> &bg, const T *X, T *SCR, const T *DVX, const T *DVZ,
                           const T *GX, const T *GZ, const T *DZBX, const T *DZF, const T *DXF, const T *DXBZ,
                           const T *PSI, T *SPSI, const T *PAT, T amp, cudaStream_t st)
{
    const long long n = (long long)a.nb * a.nx * a.nz;
    s12_rhs_kernel<T><<<s5_grid(n), S5_THREADS, 0, st>>>(a, bg, X, SCR, DVX, DVZ, GX, GZ, DZBX, DZF, DXF, DXBZ, PSI,
                                                         SPSI, PAT, amp);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_s5_axpy(long long n, T *Y, const T *X, T a, cudaStream_t st)
{
    s5_axpy_kernel<T><<<s5_grid(n), S5_THREADS, 0, st>>>(n, Y, X, a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_s5_end(const S5Args &a, T *A, const T *SCR, T dt, T *PV, const T *SPV, cudaStream_t st)
{
    const long long cols = (long long)a.nf * a.nb * a.nx;
    s5_end_kernel<T><<<(unsigned)((cols + S5_THREADS - 1) / S5_THREADS), S5_THREADS, 0, st>>>(a, A, SCR, dt);
    const long long np = (long long)a.npa * (a.npmlbot + a.npmltop) * a.nb * a.nx;
    if (PV && np > 0) s5_axpy_kernel<T><<<s5_grid(np), S5_THREADS, 0, st>>>(np, PV, SPV, dt);
    return cudaGetLastError();
}

template cudaError_t launch_s5_rhs<float>(const S5Args &, const S5Bg<float> &, const float *, float *, const float *,
                                          const float *, const float *, const float *, const float *, float,
                                          cudaStream_t);
template cudaError_t launch_s5_rhs<double>(const S5Args &, const S5Bg<double> &, const double *, double *,
                                           const double *, const double *, const double *, const double *,
                                           const double *, double, cudaStream_t);
template cudaError_t launch_s6_rhs<float>(const S5Args &, const S5Bg<float> &, const float *, float *, const float *,
                                          const float *, const float *, const float *, const float *, float *,
                                          const float *, float, cudaStream_t);
template cudaError_t launch_s6_rhs<double>(const S5Args &, const S5Bg<double> &, const double *, double *,
                                           const double *, const double *, const double *, const double *,
                                           const double *, double *, const double *, double, cudaStream_t);
#define SPARC_S12_INST(T)                                                                                      \
    template cudaError_t launch_s12_flux<T>(const S5Args &, const S5Bg<T> &, const T *, T *, cudaStream_t);          \
    template cudaError_t launch_s12_rhs<T>(const S5Args &, const S5Bg<T> &, const T *, T *, const T *, const T *,    \
                                           const T *, const T *, const T *, const T *, const T *, const T *,        \
                                           const T *, T *, const T *, T, cudaStream_t);                             \
    template cudaError_t launch_s5_axpy<T>(long long, T *, const T *, T, cudaStream_t);
SPARC_S12_INST(float)
SPARC_S12_INST(double)
#undef SPARC_S12_INST
template cudaError_t launch_s5_end<float>(const S5Args &, float *, const float *, float, float *, const float *,
                                          cudaStream_t);
template cudaError_t launch_s5_end<double>(const S5Args &, double *, const double *, double, double *,
                                           const double *, cudaStream_t);

}  // namespace sparc
