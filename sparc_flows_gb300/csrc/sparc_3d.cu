// sparc_3d.cu -- kernels of the 3-D displacement step (option 16, MP_FLOWS_PML_3D_DISPL,
// displacement.f90:377-477) for a batch of solves.
//
// Layout: every field is [nz][nb][ny][nx] -- level-major with the solves of the batch inside a
// level -- so that a z-derivative is one launch over nb*ny*nx columns of stride nb*ny*nx, an
// x-derivative one launch over nz*nb*ny rows, and a y-derivative one launch over nz*nb planes.
// The state is six such fields (xi_x, xi_y, xi_z, v_x, v_y, v_z), the vertical PML
// auxiliaries two fields of npml levels (psi_vz, psi_p).  Background profiles depend on z
// only; the flow fields v0 are [nz][ny][nx], shared by the batch.
//
// One RK stage (ddxyz, derivatives.f90:175-305, as three passes per differentiated field):
//   s3_stage_in       X = A + beta SCR, psi = PML + beta SCRPML          (step.f90:48-63)
//   x / y / z passes of xi_x, xi_y, xi_z (ibc 1)
//   s3_div_kernel     z-PML psi_vz, div, p, rho'                        (displacement.f90:396-416)
//   x / y / z passes of p (ibc 0)
//   x / y / z passes of v_x, v_y, v_z (ibc 1) + s3_adv_kernel, when the flow is on
//   s3_rhs_kernel     z-PML psi_p, RHS of v (pressure gradient, buoyancy, source), RHS of xi,
//                     top and bottom rows zero                          (displacement.f90:419-474)
// End of step: s3_end_kernel (a += dt scr with FILTER_VARS_3D_HORIZ_PML when due, one thread
// per column with an 11-value window in registers, in place), the PML auxiliaries, the record.
#include "sparc_common.cuh"

namespace sparc {

constexpr int S3_THREADS = 256;

// ---------------------------------------------------------------------------------------------
// y-derivative: a block takes 16 consecutive x-columns of one (level, solve) plane; each warp
// transforms two of them (packed as real and imaginary parts of one complex row of length NY,
// the shared-memory Stockham FFT of the x pass), derivative by i k * stretchy, inverse.  Loads
// and stores go through shared memory so that each global access covers 16 consecutive x
// (64 bytes in FP32) of one y-row.
constexpr int DDY_COLS = 16;
constexpr int DDY_WARPS = DDY_COLS / 2;
// Per-warp region of the shared-memory transform: xr, xi, yr, yi of NY values each, every array
// offset by one more word and the regions DDY_SPAN(NY) words apart (not a multiple of 32), so
// that the 16 columns a warp scatters on load (and gathers on store) fall in different banks.
template <int NY>
constexpr int ddy_span() { return 4 * NY + 5; }

template <typename T, int NY>
__global__ void __launch_bounds__(DDY_WARPS *WARP) ddy_kernel(const T *__restrict__ var, T *__restrict__ dvar,
                                                             int nx, T stretchy, const T *twr, const T *twi,
                                                             const T *kap)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sm = reinterpret_cast<T *>(smem_raw);
    constexpr int S = ddy_span<NY>();
    __shared__ T s_inv[DDY_COLS];
    __shared__ int s_off[DDY_WARPS][2];  // offsets of the result arrays in each warp's region
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t plane = (size_t)blockIdx.y * NY * nx;
    const int x0 = blockIdx.x * DDY_COLS;
    for (int idx = threadIdx.x; idx < NY * DDY_COLS; idx += DDY_WARPS * WARP) {
        const int y = idx / DDY_COLS, c = idx % DDY_COLS;
        sm[(c >> 1) * S + (c & 1) * (NY + 1) + y] = var[plane + (size_t)y * nx + x0 + c];
    }
    __syncthreads();
    T *base = sm + warp * S;
    T *xr = base, *xi = base + (NY + 1), *yr = base + 2 * (NY + 1), *yi = base + 3 * (NY + 1);
    T mr = T(0), mi = T(0);
    for (int y = lane; y < NY; y += WARP) {
        mr = fmax(mr, fabs(xr[y]));
        mi = fmax(mi, fabs(xi[y]));
    }
    T sr, si, isr, isi;
    warp_row_scale(mr, sr, isr);
    warp_row_scale(mi, si, isi);
    T *orr, *oi;
    fft_deriv<T, NY>(xr, xi, yr, yi, twr, twi, kap, stretchy, lane, orr, oi, sr, si);
    if (lane == 0) {
        s_inv[2 * warp] = isr;
        s_inv[2 * warp + 1] = isi;
        s_off[warp][0] = (int)(orr - base);
        s_off[warp][1] = (int)(oi - base);
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < NY * DDY_COLS; idx += DDY_WARPS * WARP) {
        const int y = idx / DDY_COLS, c = idx % DDY_COLS, w = c >> 1;
        dvar[plane + (size_t)y * nx + x0 + c] = sm[w * S + s_off[w][c & 1] + y] * s_inv[c];
    }
}

template <typename T, int NY>
static cudaError_t ddy_n(const T *var, T *dvar, int nplanes, int nx, T stretchy, const T *twr, const T *twi,
                         const T *kap, cudaStream_t st)
{
    const size_t smem = (size_t)DDY_WARPS * ddy_span<NY>() * sizeof(T);
    auto k = ddy_kernel<T, NY>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(nx / DDY_COLS, nplanes);
    k<<<grid, DDY_WARPS * WARP, smem, st>>>(var, dvar, nx, stretchy, twr, twi, kap);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_ddy(const T *var, T *dvar, int nplanes, int nx, int ny, T stretchy, const T *twr, const T *twi,
                       const T *kap, cudaStream_t st)
{
    if (nplanes <= 0) return cudaSuccess;
    if (nx % DDY_COLS) return cudaErrorInvalidValue;
    if (nplanes > 65535) return cudaErrorInvalidValue;
#define CASE(n_) if (ny == n_) return ddy_n<T, n_>(var, dvar, nplanes, nx, stretchy, twr, twi, kap, st);
    CASE(64) CASE(128) CASE(192) CASE(256) CASE(384) CASE(512)
#undef CASE
    return cudaErrorInvalidValue;
}

bool ddy_size_supported(int ny)
{
    return ny == 64 || ny == 128 || ny == 192 || ny == 256 || ny == 384 || ny == 512;
}

// ---------------------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(S3_THREADS) s3_stage_in(long long n6, const T *__restrict__ A,
                                                          const T *__restrict__ SCR, T *__restrict__ X, T beta,
                                                          long long np, const T *__restrict__ PV,
                                                          const T *__restrict__ SPV, T *__restrict__ PSI)
{
    const long long stride = (long long)gridDim.x * S3_THREADS;
    for (long long i = (long long)blockIdx.x * S3_THREADS + threadIdx.x; i < n6 + np; i += stride) {
        if (i < n6) X[i] = A[i] + beta * SCR[i];
        else PSI[i - n6] = PV[i - n6] + beta * SPV[i - n6];
    }
}

// PML level of row k (-1 outside the vertical PML).
__device__ __forceinline__ int s3_pml(const S3Args &a, int k)
{
    if (k < a.npmlbot) return k;
    if (k >= a.nz - a.npmltop) return a.npmlbot + (k - (a.nz - a.npmltop));
    return -1;
}

// displacement.f90:396-416: psi_vz, d xi_z/dz + psi_vz, div, p, rho'.
template <typename T>
__global__ void __launch_bounds__(S3_THREADS) s3_div_kernel(S3Args a, S3Bg<T> bg, const T *__restrict__ D1,
                                                            const T *__restrict__ D2, T *__restrict__ D3,
                                                            const T *__restrict__ XIZ, const T *__restrict__ PSIVZ,
                                                            T *__restrict__ SPSIVZ, T *__restrict__ PP,
                                                            T *__restrict__ RHO)
{
    const long long lvl = (long long)a.nb * a.nxy, n = lvl * a.nz;
    const long long stride = (long long)gridDim.x * S3_THREADS;
    for (long long i = (long long)blockIdx.x * S3_THREADS + threadIdx.x; i < n; i += stride) {
        const int k = (int)(i / lvl);
        const long long r = i - (long long)k * lvl;
        T dz = D3[i];
        const int pi = s3_pml(a, k);
        if (pi >= 0) {
            const long long m = (long long)pi * lvl + r;
            const T ps = PSIVZ[m];
            SPSIVZ[m] = bg.az[pi] * dz + bg.bz[pi] * ps;
            dz = dz + ps;
        }
        const T div = D1[i] + D2[i] + dz;
        const T xz = XIZ[i];
        PP[i] = -bg.c2rho0[k] * div - xz * bg.gradp0_z[k];
        RHO[i] = -bg.rho0[k] * div - xz * bg.gradrho0_z[k];
    }
}

// Advection of one velocity component: OUT = -2 (v0x d_x v + v0y d_y v + v0z d_z v).
template <typename T>
__global__ void __launch_bounds__(S3_THREADS) s3_adv_kernel(S3Args a, const T *__restrict__ D1,
                                                            const T *__restrict__ D2, const T *__restrict__ D3,
                                                            const T *__restrict__ V0X, const T *__restrict__ V0Y,
                                                            const T *__restrict__ V0Z, T *__restrict__ OUT)
{
    const long long lvl = (long long)a.nb * a.nxy, n = lvl * a.nz;
    const long long stride = (long long)gridDim.x * S3_THREADS;
    for (long long i = (long long)blockIdx.x * S3_THREADS + threadIdx.x; i < n; i += stride) {
        const int k = (int)(i / lvl);
        const long long r = i - (long long)k * lvl;
        const long long q = (long long)k * a.nxy + r % a.nxy;  // v0 is shared by the batch
        OUT[i] = T(-2.0) * (V0X[q] * D1[i] + V0Y[q] * D2[i] + V0Z[q] * D3[i]);
    }
}

// displacement.f90:419-474: psi_p, RHS of v_x, v_y, v_z (pressure gradient; buoyancy and the
// source on v_z), RHS of xi = v, and the top and bottom rows of every RHS set to zero.
template <typename T>
__global__ void __launch_bounds__(S3_THREADS) s3_rhs_kernel(S3Args a, S3Bg<T> bg, const T *__restrict__ X,
                                                            T *__restrict__ SCR, const T *__restrict__ GX,
                                                            const T *__restrict__ GY, const T *__restrict__ GZ,
                                                            const T *__restrict__ PSIP, T *__restrict__ SPSIP,
                                                            const T *__restrict__ RHO, const T *__restrict__ PAT,
                                                            T amp, const T *__restrict__ ADJ, int k_obs)
{
    const long long lvl = (long long)a.nb * a.nxy, n = lvl * a.nz, F = n;
    const long long stride = (long long)gridDim.x * S3_THREADS;
    for (long long i = (long long)blockIdx.x * S3_THREADS + threadIdx.x; i < n; i += stride) {
        const int k = (int)(i / lvl);
        const long long r = i - (long long)k * lvl;
        T gz = GZ[i];
        const int pi = s3_pml(a, k);
        if (pi >= 0) {
            const long long m = (long long)pi * lvl + r;
            const T ps = PSIP[m];
            SPSIP[m] = bg.az[pi] * gz + bg.bz[pi] * ps;
            gz = gz + ps;
        }
        if (k == 0 || k == a.nz - 1) {
#pragma unroll
            for (int v = 0; v < 6; v++) SCR[v * F + i] = T(0);
            continue;
        }
        const T ri = bg.rhoinv[k];
        const T ax = a.flows ? SCR[3 * F + i] : T(0);
        const T ay = a.flows ? SCR[4 * F + i] : T(0);
        const T az = a.flows ? SCR[5 * F + i] : T(0);
        T rz = az - ri * gz;
        rz = rz - ri * RHO[i] * bg.g[k];
        if (ADJ) {  // kernel-mode adjoint: forcing / rho0 * delta_width at o_rad (displacement.f90:615-627)
            if (k == k_obs) rz = rz + ADJ[r];
        } else if (abs(k - a.e_rad) <= 4) {
            rz = rz + (PAT[r] * amp) * bg.source_dep[k];
        }
        SCR[3 * F + i] = ax - ri * GX[i];
        SCR[4 * F + i] = ay - ri * GY[i];
        SCR[5 * F + i] = rz;
        SCR[0 * F + i] = X[3 * F + i];
        SCR[1 * F + i] = X[4 * F + i];
        SCR[2 * F + i] = X[5 * F + i];
    }
}

// End of step, one thread per (field, column): a += dt scr over the column, then, when
// filter is set, FILTER_VARS_3D_HORIZ_PML (physics.f90:836-882) on levels
// [npmlbot, nz - npmltop) from an 11-value window of the updated column held in registers,
// written back in place (each write is at a level the window has already read past).
template <typename T>
__global__ void __launch_bounds__(S3_THREADS) s3_end_kernel(S3Args a, T *__restrict__ A, const T *__restrict__ SCR,
                                                            T dt, int filter)
{
    const long long lvl = (long long)a.nb * a.nxy;
    const long long cols = 6 * lvl, F = lvl * a.nz;
    const long long c = (long long)blockIdx.x * S3_THREADS + threadIdx.x;
    if (c >= cols) return;
    const int v = (int)(c / lvl);
    const long long r = c - (long long)v * lvl;
    T *col = A + (long long)v * F + r;
    const T *sc = SCR + (long long)v * F + r;
    for (int k = 0; k < a.nz; k++) col[(long long)k * lvl] = col[(long long)k * lvl] + dt * sc[(long long)k * lvl];
    if (!filter) return;
    const int k0 = a.npmlbot, k1 = a.nz - a.npmltop;
    if (k0 < 5 || k1 + 5 > a.nz || k0 >= k1) return;
    const T c0 = T(0.75390625), h1 = T(0.5 * 0.41015625), h2 = T(0.5 * -0.234375), h3 = T(0.5 * 0.087890625),
            h4 = T(0.5 * -0.01953125), h5 = T(0.5 * 0.001953125);
    T w[11];
#pragma unroll
    for (int j = 0; j < 11; j++) w[j] = col[(long long)(k0 - 5 + j) * lvl];
    for (int k = k0; k < k1; k++) {
        const T out = c0 * w[5] + h1 * (w[4] + w[6]) + h2 * (w[3] + w[7]) + h3 * (w[2] + w[8]) +
                      h4 * (w[1] + w[9]) + h5 * (w[0] + w[10]);
#pragma unroll
        for (int j = 0; j < 10; j++) w[j] = w[j + 1];
        if (k + 6 < a.nz) w[10] = col[(long long)(k + 6) * lvl];
        col[(long long)k * lvl] = out;
    }
}

// Adjoint forcing of one step at the observation level, [nb][ny][nx]: LAGRANGE_INTERP of the
// adjoint-source slices (physics.f90:678-737), forcing = sum_j w[j] rows[b][i0 + j] (rows outside
// 0 .. nrows-1 count as zero), times scale = delta_width / rho0(o_rad).
template <typename T>
__global__ void __launch_bounds__(S3_THREADS) s3_adjsrc_kernel(long long lvl, long long nxy, const double *__restrict__ rows,
                                                               int nrows, int i0, S3Lagr w, double scale,
                                                               T *__restrict__ ADJ)
{
    const long long stride = (long long)gridDim.x * S3_THREADS;
    for (long long i = (long long)blockIdx.x * S3_THREADS + threadIdx.x; i < lvl; i += stride) {
        const long long b = i / nxy, q = i - b * nxy;
        double f = 0.0;
#pragma unroll
        for (int j = 0; j < 7; j++) {
            const int r = i0 + j;
            if (r >= 0 && r < nrows && w.w[j] != 0.0) f += w.w[j] * rows[((size_t)b * nrows + r) * nxy + q];
        }
        ADJ[i] = (T)(f * scale);
    }
}

// Kernel-stage record of the forward state (what PRODUCE_KERNELS reads from the partial states,
// kernels.f90:221-280): div xi = D1 + D2 + D3 (the x, y and filtered z derivatives), v_x, v_y, v_z,
// and |acc|^2 of the last stage's RHS of v (hessian integrand), [5][F].
template <typename T>
__global__ void __launch_bounds__(S3_THREADS) s3_record_kernel(long long F, const T *__restrict__ D1,
                                                               const T *__restrict__ D2, const T *__restrict__ D3,
                                                               const T *__restrict__ A, const T *__restrict__ SCR,
                                                               T *__restrict__ snap)
{
    const long long stride = (long long)gridDim.x * S3_THREADS;
    for (long long i = (long long)blockIdx.x * S3_THREADS + threadIdx.x; i < F; i += stride) {
        snap[i] = D1[i] + D2[i] + D3[i];
        snap[F + i] = A[3 * F + i];
        snap[2 * F + i] = A[4 * F + i];
        snap[3 * F + i] = A[5 * F + i];
        const double ax = SCR[3 * F + i], ay = SCR[4 * F + i], az = SCR[5 * F + i];
        snap[4 * F + i] = (T)(ax * ax + ay * ay + az * az);
    }
}

// Kernel integrands, FP64 accumulation into out [5][F] (kc, kv_x, kv_y, kv_z, hessian):
// kc += div xi_f div v_a (div v_a = D1 + D2 + D3 of the adjoint v), hessian += |acc_f|^2.
template <typename T>
__global__ void __launch_bounds__(S3_THREADS) s3_kacc_div_kernel(long long F, const T *__restrict__ D1,
                                                                 const T *__restrict__ D2, const T *__restrict__ D3,
                                                                 const T *__restrict__ snap, double *__restrict__ out)
{
    const long long stride = (long long)gridDim.x * S3_THREADS;
    for (long long i = (long long)blockIdx.x * S3_THREADS + threadIdx.x; i < F; i += stride) {
        const T diva = D1[i] + D2[i] + D3[i];
        out[i] += (double)snap[i] * (double)diva;
        out[4 * F + i] += (double)snap[4 * F + i];
    }
}

// kv_i += d_i(v_f,j) v_a,j for one component j (D1, D2, D3: x, y, filtered z derivatives of v_f,j).
template <typename T>
__global__ void __launch_bounds__(S3_THREADS) s3_kacc_v_kernel(long long F, const T *__restrict__ D1,
                                                               const T *__restrict__ D2, const T *__restrict__ D3,
                                                               const T *__restrict__ va, double *__restrict__ out)
{
    const long long stride = (long long)gridDim.x * S3_THREADS;
    for (long long i = (long long)blockIdx.x * S3_THREADS + threadIdx.x; i < F; i += stride) {
        const double a = va[i];
        out[F + i] += (double)D1[i] * a;
        out[2 * F + i] += (double)D2[i] * a;
        out[3 * F + i] += (double)D3[i] * a;
    }
}

template <typename T>
__global__ void __launch_bounds__(S3_THREADS) s3_axpy_kernel(long long n, T *__restrict__ Y, const T *__restrict__ X,
                                                             T a)
{
    const long long stride = (long long)gridDim.x * S3_THREADS;
    for (long long i = (long long)blockIdx.x * S3_THREADS + threadIdx.x; i < n; i += stride) Y[i] = Y[i] + a * X[i];
}

// ---------------------------------------------------------------------------------------------
static unsigned s3_grid(long long n)
{
    const long long g = (n + S3_THREADS - 1) / S3_THREADS;
    return (unsigned)(g < 152LL * 16 ? g : 152LL * 16);
}

template <typename T>
cudaError_t launch_s3_stage_in(long long n6, const T *A, const T *SCR, T *X, T beta, long long np, const T *PV,
                               const T *SPV, T *PSI, cudaStream_t st)
{
    s3_stage_in<T><<<s3_grid(n6 + np), S3_THREADS, 0, st>>>(n6, A, SCR, X, beta, np, PV, SPV, PSI);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_s3_div(const S3Args &a, const S3Bg<T> &bg, const T *D1, const T *D2, T *D3, const T *XIZ,
                          const T *PSIVZ, T *SPSIVZ, T *PP, T *RHO, cudaStream_t st)
{
    const long long n = (long long)a.nb * a.nxy * a.nz;
    s3_div_kernel<T><<<s3_grid(n), S3_THREADS, 0, st>>>(a, bg, D1, D2, D3, XIZ, PSIVZ, SPSIVZ, PP, RHO);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_s3_adv(const S3Args &a, const T *D1, const T *D2, const T *D3, const T *V0X, const T *V0Y,
                          const T *V0Z, T *OUT, cudaStream_t st)
{
    const long long n = (long long)a.nb * a.nxy * a.nz;
    s3_adv_kernel<T><<<s3_grid(n), S3_THREADS, 0, st>>>(a, D1, D2, D3, V0X, V0Y, V0Z, OUT);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_s3_rhs(const S3Args &a, const S3Bg<T> &bg, const T *X, T *SCR, const T *GX, const T *GY,
                          const T *GZ, const T *PSIP, T *SPSIP, const T *RHO, const T *PAT, T amp, const T *ADJ,
                          int k_obs, cudaStream_t st)
{
    const long long n = (long long)a.nb * a.nxy * a.nz;
    s3_rhs_kernel<T><<<s3_grid(n), S3_THREADS, 0, st>>>(a, bg, X, SCR, GX, GY, GZ, PSIP, SPSIP, RHO, PAT, amp, ADJ,
                                                        k_obs);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_s3_adjsrc(long long lvl, long long nxy, const double *rows, int nrows, int i0, const S3Lagr &w,
                             double scale, T *ADJ, cudaStream_t st)
{
    s3_adjsrc_kernel<T><<<s3_grid(lvl), S3_THREADS, 0, st>>>(lvl, nxy, rows, nrows, i0, w, scale, ADJ);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_s3_record(long long F, const T *D1, const T *D2, const T *D3, const T *A, const T *SCR, T *snap,
                             cudaStream_t st)
{
    s3_record_kernel<T><<<s3_grid(F), S3_THREADS, 0, st>>>(F, D1, D2, D3, A, SCR, snap);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_s3_kacc_div(long long F, const T *D1, const T *D2, const T *D3, const T *snap, double *out,
                               cudaStream_t st)
{
    s3_kacc_div_kernel<T><<<s3_grid(F), S3_THREADS, 0, st>>>(F, D1, D2, D3, snap, out);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_s3_kacc_v(long long F, const T *D1, const T *D2, const T *D3, const T *va, double *out,
                             cudaStream_t st)
{
    s3_kacc_v_kernel<T><<<s3_grid(F), S3_THREADS, 0, st>>>(F, D1, D2, D3, va, out);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_s3_end(const S3Args &a, T *A, const T *SCR, T dt, int filter, T *PV, const T *SPV,
                          cudaStream_t st)
{
    const long long cols = 6LL * a.nb * a.nxy;
    s3_end_kernel<T><<<(unsigned)((cols + S3_THREADS - 1) / S3_THREADS), S3_THREADS, 0, st>>>(a, A, SCR, dt, filter);
    const long long np = 2LL * a.nb * a.nxy * (a.npmlbot + a.npmltop);
    if (np > 0) s3_axpy_kernel<T><<<s3_grid(np), S3_THREADS, 0, st>>>(np, PV, SPV, dt);
    return cudaGetLastError();
}

#define S3_INST(T)                                                                                                    \
    template cudaError_t launch_ddy<T>(const T *, T *, int, int, int, T, const T *, const T *, const T *,            \
                                       cudaStream_t);                                                                \
    template cudaError_t launch_s3_stage_in<T>(long long, const T *, const T *, T *, T, long long, const T *,        \
                                               const T *, T *, cudaStream_t);                                        \
    template cudaError_t launch_s3_div<T>(const S3Args &, const S3Bg<T> &, const T *, const T *, T *, const T *,     \
                                          const T *, T *, T *, T *, cudaStream_t);                                   \
    template cudaError_t launch_s3_adv<T>(const S3Args &, const T *, const T *, const T *, const T *, const T *,     \
                                          const T *, T *, cudaStream_t);                                             \
    template cudaError_t launch_s3_rhs<T>(const S3Args &, const S3Bg<T> &, const T *, T *, const T *, const T *,     \
                                          const T *, const T *, T *, const T *, const T *, T, const T *, int,        \
                                          cudaStream_t);                                                             \
    template cudaError_t launch_s3_adjsrc<T>(long long, long long, const double *, int, int, const S3Lagr &, double, \
                                             T *, cudaStream_t);                                                     \
    template cudaError_t launch_s3_record<T>(long long, const T *, const T *, const T *, const T *, const T *, T *,  \
                                             cudaStream_t);                                                          \
    template cudaError_t launch_s3_kacc_div<T>(long long, const T *, const T *, const T *, const T *, double *,      \
                                               cudaStream_t);                                                        \
    template cudaError_t launch_s3_kacc_v<T>(long long, const T *, const T *, const T *, const T *, double *,        \
                                             cudaStream_t);                                                          \
    template cudaError_t launch_s3_end<T>(const S3Args &, T *, const T *, T, int, T *, const T *, cudaStream_t);
S3_INST(float)
S3_INST(double)
#undef S3_INST

}  // namespace sparc
