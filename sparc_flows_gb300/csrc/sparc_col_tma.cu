// sparc_col_tma.cu -- column pass of an RK stage with TMA-staged inputs.
//
// Same arithmetic as col_stage_kernel (sparc_col.cu, physics2d.f90:943-1094), different data
// movement: one elected thread issues 2-D bulk tensor copies of the nine per-solve input tiles
// of the block ([nz][8] columns each: xi_z, v_x, v_z of the state, three RHS-ring tiles, and
// the row pass's dxi_x/dx and x-advection terms) onto one mbarrier, so every input of the stage
// is in flight at once and no global load sits on a dependency chain.  The phases then update
// the staged tiles in place (xi_z -> xi_z of stage s, v_x -> v_x of stage s, the RHS tile of
// stage s-2 -> pressure, ...), so nine tiles are the whole shared-memory footprint.
#include "sparc_common.cuh"
#include "sparc_tma.cuh"

namespace sparc {

constexpr int TMA_CW = 8;       // columns per block (8 floats = one 32-byte sector per row)
constexpr int TMA_LMAX = 16;    // rows per z-chunk (same chunking as the classic pass)
constexpr int TMA_NTILE = 9;
constexpr uint32_t TMA_WAIT_ITERS = 1u << 24;

template <typename T>
__global__ void __launch_bounds__(TMA_CW * 20, (sizeof(T) == 4 ? 2 : 1))
    col_stage_tma_kernel(const __grid_constant__ ColMaps maps, StepArgs<T> a)
{
    constexpr int CW = TMA_CW, LMAX = TMA_LMAX;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);
    const int nz = a.nz, nx = a.nx, nch = a.nch, boxr = a.boxr;
    const size_t TBe = (size_t)2 * boxr * CW;  // elements per staged tile
    // tiles start on a 128-byte boundary (each tile is a multiple of 128 bytes long)
    unsigned char *tiles = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 8 + 127) & ~uintptr_t(127));
    T *XZ = reinterpret_cast<T *>(tiles);
    T *VX = XZ + TBe, *VZ = VX + TBe, *PS = VZ + TBe, *SX1 = PS + TBe, *SZ1 = SX1 + TBe;
    T *DXs = SZ1 + TBe, *FXXs = DXs + TBe, *FXZs = FXXs + TBe;
    T *YB = FXZs + TBe;  // 4 x [2 nch][CW]
    T *yb0 = YB, *yb1 = YB + 2 * nch * CW, *yb2 = YB + 4 * nch * CW, *yb3 = YB + 6 * nch * CW;

    const int c = threadIdx.x % CW, j = threadIdx.x / CW;
    const int x0 = blockIdx.x * CW, x = x0 + c;
    const int b = blockIdx.y;
    const int k0 = j * a.L;
    const int n = min(a.L, nz - k0);
    const size_t F = (size_t)nz * nx;
    const int s = a.stage;
    const T bs = a.bs, bsm1 = a.bsm1;
    const int time = *a.d_time;

    // ---- stage every input tile with TMA
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t boxb = (uint32_t)boxr * CW * sizeof(T);
        // tiles: XZ VX VZ DX always; PS (s>=3); SX1 SZ1 (s>=2); FXX FXZ (flows)
        const uint32_t ntiles = 4 + (s >= 3 ? 1 : 0) + (s >= 2 ? 2 : 0) + (a.flows ? 2 : 0);
        mbar_arrive_expect_tx(bar, ntiles * 2 * boxb);
        auto load = [&](T *dst, const CUtensorMap *m, int row0) {
            tma_load_2d(dst, m, x0, row0, bar);
            tma_load_2d(dst + (size_t)boxr * CW, m, x0, row0 + boxr, bar);
        };
        load(XZ, &maps.A, (b * 4 + F_XIZ) * nz);
        load(VX, &maps.A, (b * 4 + F_VX) * nz);
        load(VZ, &maps.A, (b * 4 + F_VZ) * nz);
        load(DXs, &maps.DX, b * nz);
        if (s >= 3) load(PS, &maps.SV, ((a.slot_sm2 * a.nb + b) * 2 + 1) * nz);
        if (s >= 2) {
            load(SX1, &maps.SV, ((a.slot_sm1 * a.nb + b) * 2 + 0) * nz);
            load(SZ1, &maps.SV, ((a.slot_sm1 * a.nb + b) * 2 + 1) * nz);
        }
        if (a.flows) {
            load(FXXs, &maps.FXX, b * nz);
            load(FXZs, &maps.FXZ, b * nz);
        }
    }
    const bool ok = mbar_wait_bounded(bar, 0, TMA_WAIT_ITERS);
    if (__syncthreads_or(!ok)) {
        // give up on this block: record the time-out, let the copies land, leave
        if (threadIdx.x == 0) atomicExch(a.d_err, SPARC_DEV_ERR_TMA_TIMEOUT);
        mbar_wait_bounded(bar, 0, TMA_WAIT_ITERS);
        __syncthreads();
        return;
    }

    // ---- A: xi_z of stage s, in place (scr xi_z = v_z of stage s-1 with the RHS boundary zeros)
    for (int m = 0; m < n; m++) {
        const int k = k0 + m, q = k * CW + c;
        T v = XZ[q];
        if (s >= 2) {
            T t = VZ[q];
            if (s >= 3) t += bsm1 * PS[q];
            if (k == 0 || x == 0 || x == nx - 1) t = T(0);
            v += bs * t;
        }
        XZ[q] = v;
    }
    __syncthreads();
    // ---- B: local solve of d xi_z/dz (ibc 3, top value -dxi_x/dx * unstretch)
    T y[LMAX], y2[LMAX], rg[LMAX];
    const T preset3 = -__ldg(a.TOPDX + (size_t)b * nx + x) * a.unstretch_top;
    {
        const T last = zlocal<T, LMAX>(a.z3, XZ, CW, c, k0, n, nz, preset3, y);
        yb0[(2 * j) * CW + c] = y[0];
        yb0[(2 * j + 1) * CW + c] = last;
    }
    __syncthreads();
    // ---- C: vertical PML, divergence, pressure (into PS), v_x of stage s (in place)
    {
        T xl, xr;
        zcouple(a.z3, yb0, CW, c, j, nch, xl, xr);
#pragma unroll
        for (int m = 0; m < LMAX; m++) {
            if (m < n) {
                const int k = k0 + m, q = k * CW + c;
                const size_t g = (size_t)k * nx + x;
                T dzz = zcorrect(a.z3, y[m], k, xl, xr) * __ldg(a.stretch + k);
                const int pi = pml_row(a, k);
                T fd = T(1);
                if (pi >= 0) {
                    const size_t qz = ((size_t)b * 2 * a.nzpml + pi) * nx + x;
                    const size_t qb = (size_t)b * a.bgz + (size_t)pi * nx + x;
                    T ps = __ldg(a.PZ + qz);
                    if (s >= 2) ps += bs * __ldg(a.SPZ + (size_t)a.slot_sm1 * a.nb * 2 * a.nzpml * nx + qz);
                    a.SPZ[(size_t)a.slot_s * a.nb * 2 * a.nzpml * nx + qz] =
                        __ldg(a.az + qb) * dzz + __ldg(a.bz + qb) * ps;
                    dzz += ps;
                    fd = __ldg(a.fdz + qb);
                }
                const T xiz = XZ[q];
                const T div = DXs[q] + dzz;
                const T c2r = a.c2d ? __ldg(a.c2rho0 + (size_t)b * a.bg2 + g) : __ldg(a.c2rho0 + k);
                const T p = -c2r * div - __ldg(a.gp0 + k) * fd * xiz;
                const T rho = -__ldg(a.rho0 + k) * div - __ldg(a.gr0 + k) * fd * xiz;
                rg[m] = rho * __ldg(a.g + k);
                PS[q] = p;
                a.P[(size_t)b * F + g] = p;
                if (s >= 2) VX[q] += bs * SX1[q];
            }
        }
    }
    __syncthreads();
    // ---- D: local solves of dp/dz (ibc 2, bottom value 0) and dv_x/dz (ibc 1)
    {
        const T last = zlocal<T, LMAX>(a.z2, PS, CW, c, k0, n, nz, T(0), y);
        yb1[(2 * j) * CW + c] = y[0];
        yb1[(2 * j + 1) * CW + c] = last;
    }
    if (a.flows) {
        const T last = zlocal<T, LMAX>(a.z1, VX, CW, c, k0, n, nz, T(0), y2);
        yb2[(2 * j) * CW + c] = y2[0];
        yb2[(2 * j + 1) * CW + c] = last;
    }
    __syncthreads();
    // ---- E: gradient of p and RHS v_z without advection; z-advection of v_x; v_z of stage s
    {
        T xl, xr, xl2 = T(0), xr2 = T(0);
        zcouple(a.z2, yb1, CW, c, j, nch, xl, xr);
        if (a.flows) zcouple(a.z1, yb2, CW, c, j, nch, xl2, xr2);
#pragma unroll
        for (int m = 0; m < LMAX; m++) {
            if (m < n) {
                const int k = k0 + m, q = k * CW + c;
                const size_t g = (size_t)k * nx + x;
                T gpz = zcorrect(a.z2, y[m], k, xl, xr) * __ldg(a.stretch + k);
                const int pi = pml_row(a, k);
                if (pi >= 0) {
                    const size_t qz = (((size_t)b * 2 + 1) * a.nzpml + pi) * nx + x;
                    const size_t qb = (size_t)b * a.bgz + (size_t)pi * nx + x;
                    T ps = __ldg(a.PZ + qz);
                    if (s >= 2) ps += bs * __ldg(a.SPZ + (size_t)a.slot_sm1 * a.nb * 2 * a.nzpml * nx + qz);
                    a.SPZ[(size_t)a.slot_s * a.nb * 2 * a.nzpml * nx + qz] =
                        __ldg(a.az + qb) * gpz + __ldg(a.bz + qb) * ps;
                    gpz += ps;
                }
                rg[m] = -__ldg(a.rhoinv + k) * (gpz + rg[m]);
                T rv = T(0);
                if (a.flows) {
                    const T dvxdz = zcorrect(a.z1, y2[m], k, xl2, xr2) * __ldg(a.stretch + k);
                    rv = FXXs[q] - T(2) * a.fsign * __ldg(a.v0z + (size_t)b * a.bg2 + g) * dvxdz;
                }
                a.RVXP[(size_t)b * F + g] = rv;
                if (s >= 2) VZ[q] += bs * SZ1[q];
            }
        }
    }
    __syncthreads();
    // ---- F: local solve of dv_z/dz
    if (a.flows) {
        const T last = zlocal<T, LMAX>(a.z1, VZ, CW, c, k0, n, nz, T(0), y2);
        yb3[(2 * j) * CW + c] = y2[0];
        yb3[(2 * j + 1) * CW + c] = last;
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
            const int k = k0 + m, q = k * CW + c;
            const size_t g = (size_t)k * nx + x;
            T r = rg[m];
            if (k == a.k_inj) r += forcing;
            if (a.flows) {
                const T dvzdz = zcorrect(a.z1, y2[m], k, xl2, xr2) * __ldg(a.stretch + k);
                r += FXZs[q] - T(2) * a.fsign * __ldg(a.v0z + (size_t)b * a.bg2 + g) * dvzdz;
            }
            if (k == 0 || x == 0 || x == nx - 1) r = T(0);
            svz[g] = r;
        }
    }
}

template <typename T>
size_t col_tma_smem_bytes(int nz, int nch, int boxr)
{
    return 256 + (size_t)TMA_NTILE * 2 * boxr * TMA_CW * sizeof(T) + (size_t)8 * nch * TMA_CW * sizeof(T);
}

template <typename T>
cudaError_t launch_col_stage_tma(const ColMaps &maps, const StepArgs<T> &a, cudaStream_t st)
{
    if (a.nx % TMA_CW || a.L > TMA_LMAX || a.nch > 20 || 2 * a.boxr < a.nz) return cudaErrorInvalidValue;
    const size_t smem = col_tma_smem_bytes<T>(a.nz, a.nch, a.boxr);
    auto k = col_stage_tma_kernel<T>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(a.nx / TMA_CW, a.nb);
    k<<<grid, TMA_CW * a.nch, smem, st>>>(maps, a);
    return cudaGetLastError();
}

template size_t col_tma_smem_bytes<float>(int, int, int);
template size_t col_tma_smem_bytes<double>(int, int, int);
template cudaError_t launch_col_stage_tma<float>(const ColMaps &, const StepArgs<float> &, cudaStream_t);
template cudaError_t launch_col_stage_tma<double>(const ColMaps &, const StepArgs<double> &, cudaStream_t);

// End of step with TMA-staged tiles: a += deltat scr and FILTER_VARS_2D (physics2d.f90:509-556),
// pmlvars += deltat scrpml, seismogram and partial-state records (driver.f90:386-417).
template <typename T>
__device__ __forceinline__ T filt11_s(const T *B, int k, int c)
{
    constexpr int CW = TMA_CW;
    const T c0 = T(0.75390625), h1 = T(0.5 * 0.41015625), h2 = T(0.5 * -0.234375), h3 = T(0.5 * 0.087890625),
            h4 = T(0.5 * -0.01953125), h5 = T(0.5 * 0.001953125);
    return c0 * B[k * CW + c] + h1 * (B[(k - 1) * CW + c] + B[(k + 1) * CW + c]) +
           h2 * (B[(k - 2) * CW + c] + B[(k + 2) * CW + c]) + h3 * (B[(k - 3) * CW + c] + B[(k + 3) * CW + c]) +
           h4 * (B[(k - 4) * CW + c] + B[(k + 4) * CW + c]) + h5 * (B[(k - 5) * CW + c] + B[(k + 5) * CW + c]);
}

template <typename T>
__global__ void __launch_bounds__(TMA_CW * 20, (sizeof(T) == 4 ? 2 : 1))
    end_step_tma_kernel(const __grid_constant__ ColMaps maps, StepArgs<T> a)
{
    constexpr int CW = TMA_CW;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);
    const int nz = a.nz, nx = a.nx, boxr = a.boxr;
    const size_t TBe = (size_t)2 * boxr * CW;
    unsigned char *tiles = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 8 + 127) & ~uintptr_t(127));
    T *ST = reinterpret_cast<T *>(tiles);  // 4 state tiles: xi_x, xi_z, v_x, v_z
    T *R4x = ST + 4 * TBe, *R4z = R4x + TBe, *R5x = R4z + TBe, *R5z = R5x + TBe;
    const int c = threadIdx.x % CW, j = threadIdx.x / CW;
    const int x0 = blockIdx.x * CW, x = x0 + c;
    const int b = blockIdx.y;
    const int k0 = j * a.L;
    const int n = min(a.L, nz - k0);
    const size_t F = (size_t)nz * nx;
    const int time = *a.d_time;
    const int rec = (a.steps_out > 0) ? time / a.steps_out - a.rec0 : 0;  // slot in the record window
    const bool record = a.steps_out > 0 && time % a.steps_out == 0 && rec >= 0 && rec < a.nrec_cap && time >= 0;
    const bool xf = a.filt_xall || ((x >= a.nh - 1) && (x <= nx - a.nh));
    T *snap = record && a.snaps ? a.snaps + ((size_t)b * a.nrec_cap + rec) * 6 * F : nullptr;

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t boxb = (uint32_t)boxr * CW * sizeof(T);
        mbar_arrive_expect_tx(bar, 8u * 2u * boxb);
        auto load = [&](T *dst, const CUtensorMap *m, int row0) {
            tma_load_2d(dst, m, x0, row0, bar);
            tma_load_2d(dst + (size_t)boxr * CW, m, x0, row0 + boxr, bar);
        };
        for (int f = 0; f < 4; f++) load(ST + f * TBe, &maps.A, (b * 4 + f) * nz);
        load(R4x, &maps.SV, ((a.slot_sm1 * a.nb + b) * 2 + 0) * nz);
        load(R4z, &maps.SV, ((a.slot_sm1 * a.nb + b) * 2 + 1) * nz);
        load(R5x, &maps.SV, ((a.slot_s * a.nb + b) * 2 + 0) * nz);
        load(R5z, &maps.SV, ((a.slot_s * a.nb + b) * 2 + 1) * nz);
    }
    const bool ok = mbar_wait_bounded(bar, 0, TMA_WAIT_ITERS);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicExch(a.d_err, SPARC_DEV_ERR_TMA_TIMEOUT);
        mbar_wait_bounded(bar, 0, TMA_WAIT_ITERS);
        __syncthreads();
        return;
    }
    // a + deltat scr for the four fields of the thread's own rows, in place
    for (int m = 0; m < n; m++) {
        const int k = k0 + m, q = k * CW + c;
        const bool bc = (k == 0 || x == 0 || x == nx - 1);
        const T vx = ST[2 * TBe + q], vz = ST[3 * TBe + q];
        const T sxix = bc ? T(0) : vx + a.bs * R4x[q];  // scr xi = v of stage 5, RHS zeros
        const T sxiz = bc ? T(0) : vz + a.bs * R4z[q];
        ST[0 * TBe + q] += a.dt * sxix;
        ST[1 * TBe + q] += a.dt * sxiz;
        ST[2 * TBe + q] = vx + a.dt * R5x[q];
        ST[3 * TBe + q] = vz + a.dt * R5z[q];
    }
    __syncthreads();
    for (int f = 0; f < 4; f++) {
        const T *B = ST + f * TBe;
        T *Ag = a.A + ((size_t)b * 4 + f) * F;
        for (int m = 0; m < n; m++) {
            const int k = k0 + m;
            const size_t g = (size_t)k * nx + x;
            T out = B[k * CW + c];
            if (xf && k >= a.filt_k0 && k <= nz - 2) {
                if (k >= 5 && k <= nz - 6) out = filt11_s(B, k, c);
                else out = T(0.5) * (B[(k + 1) * CW + c] + B[(k - 1) * CW + c]);
            }
            Ag[g] = out;
            if (snap) snap[(size_t)f * F + g] = out;
            if (record && f == F_VZ && k == a.k_obs && a.seis) a.seis[((size_t)b * a.nrec_cap + rec) * nx + x] = out;
        }
    }
    for (int m = 0; m < n; m++) {
        const int k = k0 + m;
        const size_t g = (size_t)k * nx + x;
        const int pi = pml_row(a, k);
        if (pi >= 0) {
            for (int cc = 0; cc < 2; cc++) {
                const size_t qz = (((size_t)b * 2 + cc) * a.nzpml + pi) * nx + x;
                a.PZ[qz] += a.dt * a.SPZ[(size_t)a.slot_s * a.nb * 2 * a.nzpml * nx + qz];
            }
        }
        if (snap) {
            snap[4 * F + g] = R5x[k * CW + c];
            snap[5 * F + g] = R5z[k * CW + c];
        }
    }
}

template <typename T>
size_t end_tma_smem_bytes(int boxr)
{
    return 256 + (size_t)8 * 2 * boxr * TMA_CW * sizeof(T);
}

template <typename T>
cudaError_t launch_end_step_tma(const ColMaps &maps, const StepArgs<T> &a, cudaStream_t st)
{
    if (a.nx % TMA_CW || a.L > TMA_LMAX || a.nch > 20 || 2 * a.boxr < a.nz || a.ALO) return cudaErrorInvalidValue;
    const size_t smem = end_tma_smem_bytes<T>(a.boxr);
    auto k = end_step_tma_kernel<T>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(a.nx / TMA_CW, a.nb);
    k<<<grid, TMA_CW * a.nch, smem, st>>>(maps, a);
    return cudaGetLastError();
}

template cudaError_t launch_end_step_tma<float>(const ColMaps &, const StepArgs<float> &, cudaStream_t);
template cudaError_t launch_end_step_tma<double>(const ColMaps &, const StepArgs<double> &, cudaStream_t);

}  // namespace sparc
