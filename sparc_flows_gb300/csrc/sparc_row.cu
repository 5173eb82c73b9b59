// sparc_row.cu -- row (x-direction) passes of the RK stage: spectral x-derivatives
// (derivatives.f90:28-58) with the horizontal PML (physics2d.f90:970-986, 1003-1020).
//
// One warp owns one x-row of one solve.  Two real rows are differentiated by one complex
// FFT (real part + i * imaginary part), the derivative operator mapping real rows to real
// rows.  Stage s of the RK step needs, along x:
//   d/dx of p from stage s-1   -> completes RHS v_x of stage s-1 (-rhoinv * dp/dx);
//   d/dx of xi_x at stage s    -> divergence input of stage s (plus the top-row value that
//                                 the column pass needs for its ibc=3 boundary);
//   d/dx of v_x, v_z at stage s -> advection terms -2 v0x d/dx (physics2d.f90:1065-1079).
#include "sparc_fft512.cuh"

namespace sparc {

constexpr int ROW_WPB = 4;  // rows (warps) per block

// Per-row state of a row pass and its three per-column steps, shared by the Stockham kernel and
// the register-FFT kernel.  MODE 0: stage 1 (no pressure yet), MODE 1: stages 2..5, MODE 2:
// closing pass after stage 5.
template <typename T>
struct RowCtx {
    int b, k, nx, nh, nhx;
    size_t F, ro;
    const T *Ab;
    T bs, bsm1, rhoinv_k;
    T *PXb;
    const T *axk, *bxk;
    __device__ RowCtx(const StepArgs<T> &a, int row, int N)
    {
        b = row / a.nz;
        k = row - b * a.nz;
        nx = N;
        nh = a.nh;
        nhx = a.nhx;
        F = (size_t)a.nz * nx;
        ro = (size_t)k * nx;
        Ab = a.A + (size_t)b * 4 * F;
        bs = a.bs;
        bsm1 = a.bsm1;
        rhoinv_k = __ldg(a.rhoinv + k);
        PXb = a.PX + (size_t)b * 2 * a.nz * nhx;
        axk = a.ax + (size_t)b * a.bgx + (size_t)k * nhx;
        bxk = a.bx + (size_t)b * a.bgx + (size_t)k * nhx;
    }
};

// Inputs of the first FFT at column x: (p_{s-1}, xi_x at stage s) or (p_5, 0).
template <typename T, int MODE>
__device__ __forceinline__ void row_load(const StepArgs<T> &a, const RowCtx<T> &r, int x, T &p, T &xis)
{
    const int b = r.b, k = r.k;
    const size_t F = r.F, ro = r.ro;
    p = T(0);
    xis = T(0);
    if (MODE != 0) p = __ldg(a.P + (size_t)b * F + ro + x);
    if (MODE == 0) {
        xis = __ldg(r.Ab + F_XIX * F + ro + x);
    } else if (MODE == 1) {
        T avx = __ldg(r.Ab + F_VX * F + ro + x);
        T s = (a.stage == 2) ? avx : avx + r.bsm1 * __ldg(svp(a, a.slot_sm2, b, 0) + ro + x);
        if (k == 0 || x == 0 || x == r.nx - 1) s = T(0);  // RHS boundary zeros (physics2d.f90:1083-1093)
        xis = __ldg(r.Ab + F_XIX * F + ro + x) + r.bs * s;
    }
}

// From gpx = dp/dx and dxx = dxi_x/dx at column x: x-PML, RHS v_x of stage s-1, dxi_x/dx for the
// column pass; the inputs (v_x, v_z at stage s) of the second FFT (MODE != 2).
template <typename T, int MODE>
__device__ __forceinline__ void row_mid(const StepArgs<T> &a, const RowCtx<T> &r, int x, T gpx, T dxx, T &vxs, T &vzs)
{
    const int b = r.b, k = r.k, nx = r.nx, nh = r.nh, nhx = r.nhx;
    const size_t F = r.F, ro = r.ro;
    const bool pml = (x < nh) || (x >= nx - nh);
    const int ai = (x < nh) ? x : x - (nx - nh) + nh;
    if (MODE != 2 && k == a.nz - 1) a.TOPDX[(size_t)b * nx + x] = dxx;
    if (pml) {
        const T axv = __ldg(r.axk + ai), bxv = __ldg(r.bxk + ai);
        if (MODE != 0) {  // psi_gradp_x of stage s-1
            const size_t q = ((size_t)1 * a.nz + k) * nhx + ai;
            T ps = r.PXb[q];
            if (a.stage >= 3) ps += r.bsm1 * a.SPX[((size_t)a.slot_sm2 * a.nb + b) * 2 * a.nz * nhx + q];
            gpx += ps;
            a.SPX[((size_t)a.slot_sm1 * a.nb + b) * 2 * a.nz * nhx + q] = axv * gpx + bxv * ps;
        }
        if (MODE != 2) {  // psi_vx of stage s
            const size_t q = ((size_t)0 * a.nz + k) * nhx + ai;
            T ps = r.PXb[q];
            if (MODE == 1) ps += r.bs * a.SPX[((size_t)a.slot_sm1 * a.nb + b) * 2 * a.nz * nhx + q];
            dxx += ps;
            a.SPX[((size_t)a.slot_s * a.nb + b) * 2 * a.nz * nhx + q] = axv * dxx + bxv * ps;
        }
    }
    T svx = T(0);
    if (MODE != 0) {
        svx = __ldg(a.RVXP + (size_t)b * F + ro + x) - r.rhoinv_k * gpx;
        if (k == 0 || x == 0 || x == nx - 1) svx = T(0);
        svp(a, a.slot_sm1, b, 0)[ro + x] = svx;
    }
    vxs = T(0);
    vzs = T(0);
    if (MODE != 2) {
        a.DX[(size_t)b * F + ro + x] = dxx;
        vxs = __ldg(r.Ab + F_VX * F + ro + x);
        vzs = __ldg(r.Ab + F_VZ * F + ro + x);
        if (MODE == 1) {
            vxs += r.bs * svx;
            vzs += r.bs * __ldg(svp(a, a.slot_sm1, b, 1) + ro + x);
        }
    } else if (pml) {
        // closing pass: pmlvarsx += deltat * scrpmlx (step.f90:112-115)
        for (int c = 0; c < 2; c++) {
            const size_t q = ((size_t)c * a.nz + k) * nhx + ai;
            r.PXb[q] += a.dt * a.SPX[((size_t)a.slot_sm1 * a.nb + b) * 2 * a.nz * nhx + q];
        }
    }
}

// x-advection terms -2 v0x d/dx of v_x, v_z at column x.
template <typename T>
__device__ __forceinline__ void row_out(const StepArgs<T> &a, const RowCtx<T> &r, int x, T dvx, T dvz)
{
    const T w = T(-2) * a.fsign * __ldg(a.v0x + (size_t)r.b * a.bg2 + r.ro + x);
    a.FXX[(size_t)r.b * r.F + r.ro + x] = w * dvx;
    a.FXZ[(size_t)r.b * r.F + r.ro + x] = w * dvz;
}

template <typename T, int N, int MODE>
__global__ void __launch_bounds__(ROW_WPB *WARP) row_stage_kernel(StepArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sm = reinterpret_cast<T *>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (MODE == 0 && blockIdx.x == 0 && threadIdx.x == 0) *a.d_time += 1;  // new step begins
    const int row = blockIdx.x * ROW_WPB + warp;
    if (row >= a.nb * a.nz) return;
    T *xr = sm + warp * 4 * N, *xi = xr + N, *yr = xi + N, *yi = yr + N;
    const RowCtx<T> r(a, row, N);

    T mr = T(0), mi = T(0);
    for (int x = lane; x < N; x += WARP) {
        T p, xis;
        row_load<T, MODE>(a, r, x, p, xis);
        xr[x] = p;
        xi[x] = xis;
        mr = fmax(mr, fabs(p));
        mi = fmax(mi, fabs(xis));
    }
    T sr, si, isr, isi;
    warp_row_scale(mr, sr, isr);
    warp_row_scale(mi, si, isi);
    __syncwarp();
    T *o1r, *o1i;
    fft_deriv<T, N>(xr, xi, yr, yi, a.twr, a.twi, a.kap, a.stretchx, lane, o1r, o1i, sr, si);
    __syncwarp();

    T mr2 = T(0), mi2 = T(0);
    for (int x = lane; x < N; x += WARP) {
        T vxs, vzs;
        row_mid<T, MODE>(a, r, x, o1r[x] * isr, o1i[x] * isi, vxs, vzs);
        if (MODE != 2) {
            o1r[x] = vxs;
            o1i[x] = vzs;
            mr2 = fmax(mr2, fabs(vxs));
            mi2 = fmax(mi2, fabs(vzs));
        }
    }
    if (MODE == 2 || !a.flows) return;
    T sr2, si2, isr2, isi2;
    warp_row_scale(mr2, sr2, isr2);
    warp_row_scale(mi2, si2, isi2);
    __syncwarp();
    T *gr = (o1r == xr) ? yr : xr, *gi = (o1r == xr) ? yi : xi;
    T *o2r, *o2i;
    fft_deriv<T, N>(o1r, o1i, gr, gi, a.twr, a.twi, a.kap, a.stretchx, lane, o2r, o2i, sr2, si2);
    __syncwarp();
    for (int x = lane; x < N; x += WARP) row_out(a, r, x, o2r[x] * isr2, o2i[x] * isi2);
}

// row_mid without global stores, for the register-FFT pass: the loads and arithmetic of column x;
// what row_mid stores is returned (svx: RHS v_x of stage s-1, dxo: dxi_x/dx) or, for the x-PML
// columns, left in the warp scratch P ([3][nhx]: psi_vx RHS or, closing pass, the new psi_vx;
// psi_gradp_x RHS; closing pass, the new psi_gradp_x).  The stores follow in row_mid_store.
template <int MODE>
__device__ __forceinline__ void row_mid_load(const StepArgs<float> &a, const RowCtx<float> &r, int x, float gpx,
                                             float dxx, float *P, float &svx, float &dxo, float &vxs, float &vzs)
{
    const int b = r.b, k = r.k, nx = r.nx, nh = r.nh, nhx = r.nhx;
    const size_t F = r.F, ro = r.ro;
    const bool pml = (x < nh) || (x >= nx - nh);
    const int ai = (x < nh) ? x : x - (nx - nh) + nh;
    if (pml) {
        const float axv = __ldg(r.axk + ai), bxv = __ldg(r.bxk + ai);
        float ngp = 0.f;
        if (MODE != 0) {  // psi_gradp_x of stage s-1
            const size_t q = ((size_t)1 * a.nz + k) * nhx + ai;
            float ps = r.PXb[q];
            if (a.stage >= 3) ps += r.bsm1 * a.SPX[((size_t)a.slot_sm2 * a.nb + b) * 2 * a.nz * nhx + q];
            gpx += ps;
            ngp = axv * gpx + bxv * ps;
            P[nhx + ai] = ngp;
        }
        if (MODE != 2) {  // psi_vx of stage s
            const size_t q = ((size_t)0 * a.nz + k) * nhx + ai;
            float ps = r.PXb[q];
            if (MODE == 1) ps += r.bs * a.SPX[((size_t)a.slot_sm1 * a.nb + b) * 2 * a.nz * nhx + q];
            dxx += ps;
            P[ai] = axv * dxx + bxv * ps;
        } else {  // closing pass: pmlvarsx += deltat * scrpmlx (step.f90:112-115)
            const size_t q0 = ((size_t)0 * a.nz + k) * nhx + ai, q1 = ((size_t)1 * a.nz + k) * nhx + ai;
            P[ai] = r.PXb[q0] + a.dt * a.SPX[((size_t)a.slot_sm1 * a.nb + b) * 2 * a.nz * nhx + q0];
            P[2 * nhx + ai] = r.PXb[q1] + a.dt * ngp;
        }
    }
    svx = 0.f;
    if (MODE != 0) {
        svx = __ldg(a.RVXP + (size_t)b * F + ro + x) - r.rhoinv_k * gpx;
        if (k == 0 || x == 0 || x == nx - 1) svx = 0.f;
    }
    dxo = dxx;
    vxs = 0.f;
    vzs = 0.f;
    if (MODE != 2) {
        vxs = __ldg(r.Ab + F_VX * F + ro + x);
        vzs = __ldg(r.Ab + F_VZ * F + ro + x);
        if (MODE == 1) {
            vxs += r.bs * svx;
            vzs += r.bs * __ldg(svp(a, a.slot_sm1, b, 1) + ro + x);
        }
    }
}

// The x-PML stores of row_mid_load from the warp scratch P (lanes over the PML columns).
template <int MODE>
__device__ __forceinline__ void row_mid_store_pml(const StepArgs<float> &a, const RowCtx<float> &r, const float *P,
                                                  int lane)
{
    const int b = r.b, k = r.k, nhx = r.nhx;
    for (int ai = lane; ai < nhx; ai += WARP) {
        const size_t q0 = ((size_t)0 * a.nz + k) * nhx + ai, q1 = ((size_t)1 * a.nz + k) * nhx + ai;
        if (MODE != 0) a.SPX[((size_t)a.slot_sm1 * a.nb + b) * 2 * a.nz * nhx + q1] = P[nhx + ai];
        if (MODE != 2) {
            a.SPX[((size_t)a.slot_s * a.nb + b) * 2 * a.nz * nhx + q0] = P[ai];
        } else {
            r.PXb[q0] = P[ai];
            r.PXb[q1] = P[2 * nhx + ai];
        }
    }
}

// FP32 rows of 512 columns: the same row pass with the register-resident FFT (sparc_fft512.cuh);
// register n2 of a lane holds column lane + 32 n2.  Each part loads everything it needs before it
// stores anything, so no load waits behind a store of the row it may alias.
constexpr uint32_t STAGE_WAIT_ITERS = 1u << 21;  // polls of 128 ns: about 0.3 s

// Stage overlap: wait (bounded) until every column tile of the solves of this block's rows is
// done.  Thread 0 polls with acquire loads; the barrier passes what it saw to the block.  Returns
// false to every thread on a time-out, with the device error flag set (and at once once that
// flag is set).
__device__ __forceinline__ bool stage_wait(const StepArgs<float> &a, int row0, int nrows)
{
    bool ok = true;
    if (threadIdx.x == 0) {
        // once any device error is flagged (a wait that gave up, a column block that left early)
        // the waits of the rest fail at once
        if (*(volatile int *)a.d_err != 0) ok = false;
        const int last = min(row0 + nrows, a.nb * a.nz) - 1;
        const int *cnt = a.tile_cnt + (size_t)(a.stage - 2) * a.nb;
        for (int b = row0 / a.nz; ok && b <= last / a.nz; b++) {
            uint32_t it = 0;
            for (;;) {
                int v;
                asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(cnt + b) : "memory");
                if (v >= a.tiles_per_solve) break;
                if (++it > STAGE_WAIT_ITERS) {
                    ok = false;
                    break;
                }
                __nanosleep(128);
            }
        }
        if (!ok) atomicExch(a.d_err, SPARC_DEV_ERR_STAGE_WAIT);
    }
    return !__syncthreads_or(!ok);
}

template <int MODE>
__global__ void __launch_bounds__(ROW_WPB *WARP, 4) row_stage_reg512_kernel(StepArgs<float> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (MODE != 0 && a.tile_cnt && !stage_wait(a, blockIdx.x * ROW_WPB, ROW_WPB)) return;
    if (MODE == 0 && blockIdx.x == 0 && threadIdx.x == 0) *a.d_time += 1;  // new step begins
    const int row = blockIdx.x * ROW_WPB + warp;
    if (row >= a.nb * a.nz) return;
    float *S = reinterpret_cast<float *>(smem_raw) + warp * FFT512_SCRATCH;
    const RowCtx<float> r(a, row, 512);

    float re[16], im[16];
    float mr = 0.f, mi = 0.f;
#pragma unroll
    for (int n2 = 0; n2 < 16; n2++) {
        row_load<float, MODE>(a, r, lane + 32 * n2, re[n2], im[n2]);
        mr = fmaxf(mr, fabsf(re[n2]));
        mi = fmaxf(mi, fabsf(im[n2]));
    }
    float sr, si, isr, isi;
    warp_row_scale(mr, sr, isr);
    warp_row_scale(mi, si, isi);
    fft512_deriv(re, im, S, a.twr, a.twi, a.kap, a.stretchx, lane, sr, si);

    float mr2 = 0.f, mi2 = 0.f;
    float svx[16], dxo[16];
    __syncwarp();  // the transform's last reads of S are done before S holds the x-PML values
#pragma unroll
    for (int n2 = 0; n2 < 16; n2++) {
        float vxs, vzs;
        row_mid_load<MODE>(a, r, lane + 32 * n2, re[n2] * isr, im[n2] * isi, S, svx[n2], dxo[n2], vxs, vzs);
        re[n2] = vxs;
        im[n2] = vzs;
        mr2 = fmaxf(mr2, fabsf(vxs));
        mi2 = fmaxf(mi2, fabsf(vzs));
    }
    __syncwarp();
    row_mid_store_pml<MODE>(a, r, S, lane);
    {
        const size_t F = r.F, ro = r.ro;
#pragma unroll
        for (int n2 = 0; n2 < 16; n2++) {
            const int x = lane + 32 * n2;
            if (MODE != 0) svp(a, a.slot_sm1, r.b, 0)[ro + x] = svx[n2];
            if (MODE != 2) {
                a.DX[(size_t)r.b * F + ro + x] = dxo[n2];
                if (r.k == a.nz - 1) a.TOPDX[(size_t)r.b * 512 + x] = dxo[n2];
            }
        }
    }
    if (MODE == 2 || !a.flows) return;
    __syncwarp();  // the x-PML values are read before the next transform reuses S
    float sr2, si2, isr2, isi2;
    warp_row_scale(mr2, sr2, isr2);
    warp_row_scale(mi2, si2, isi2);
    fft512_deriv(re, im, S, a.twr, a.twi, a.kap, a.stretchx, lane, sr2, si2);
    float wv[16];  // -2 v0x of the row, loaded before the advection terms are stored
#pragma unroll
    for (int n2 = 0; n2 < 16; n2++) wv[n2] = -2.f * a.fsign * __ldg(a.v0x + (size_t)r.b * a.bg2 + r.ro + lane + 32 * n2);
#pragma unroll
    for (int n2 = 0; n2 < 16; n2++) {
        const size_t q = (size_t)r.b * r.F + r.ro + lane + 32 * n2;
        a.FXX[q] = wv[n2] * (re[n2] * isr2);
        a.FXZ[q] = wv[n2] * (im[n2] * isi2);
    }
}

// Generic spectral x-derivative of nrows rows (two rows per warp).
template <typename T, int N>
__global__ void __launch_bounds__(ROW_WPB *WARP) ddx_kernel(const T *__restrict__ var, T *__restrict__ dvar,
                                                              int nrows, T stretchx, const T *twr, const T *twi,
                                                              const T *kap)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sm = reinterpret_cast<T *>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r0 = 2 * (blockIdx.x * ROW_WPB + warp);
    if (r0 >= nrows) return;
    const bool two = r0 + 1 < nrows;
    T *xr = sm + warp * 4 * N, *xi = xr + N, *yr = xi + N, *yi = yr + N;
    T mr = T(0), mi = T(0);
    for (int x = lane; x < N; x += WARP) {
        xr[x] = var[(size_t)r0 * N + x];
        xi[x] = two ? var[(size_t)(r0 + 1) * N + x] : T(0);
        mr = fmax(mr, fabs(xr[x]));
        mi = fmax(mi, fabs(xi[x]));
    }
    T sr, si, isr, isi;
    warp_row_scale(mr, sr, isr);
    warp_row_scale(mi, si, isi);
    __syncwarp();
    T *orr, *oi;
    fft_deriv<T, N>(xr, xi, yr, yi, twr, twi, kap, stretchx, lane, orr, oi, sr, si);
    __syncwarp();
    for (int x = lane; x < N; x += WARP) {
        dvar[(size_t)r0 * N + x] = orr[x] * isr;
        if (two) dvar[(size_t)(r0 + 1) * N + x] = oi[x] * isi;
    }
}

#define SPARC_FFT_SIZES(X) X(64) X(128) X(192) X(256) X(384) X(512) X(768) X(1024)

bool fft_size_supported(int n)
{
#define CASE(n_) if (n == n_) return true;
    SPARC_FFT_SIZES(CASE)
#undef CASE
    return false;
}

template <int MODE>
static void row_reg512_launch(const StepArgs<float> &a, int grid, cudaStream_t st)
{
    const size_t smem = (size_t)ROW_WPB * FFT512_SCRATCH * sizeof(float);
    if (MODE != 0 && a.tile_cnt) {  // a programmatic dependent of the column pass before it
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(ROW_WPB * WARP);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        cudaLaunchKernelEx(&cfg, row_stage_reg512_kernel<MODE>, a);
        return;
    }
    row_stage_reg512_kernel<MODE><<<grid, ROW_WPB * WARP, smem, st>>>(a);
}

template <typename T, int N>
static cudaError_t row_stage_n(const StepArgs<T> &a, cudaStream_t st)
{
    if constexpr (sizeof(T) == 4 && N == 512) {
        const int grid = (a.nb * a.nz + ROW_WPB - 1) / ROW_WPB;
        if (a.stage == 1) row_reg512_launch<0>(a, grid, st);
        else if (a.stage <= 5) row_reg512_launch<1>(a, grid, st);
        else row_reg512_launch<2>(a, grid, st);
        return cudaGetLastError();
    }
    const int rows = a.nb * a.nz;
    const int grid = (rows + ROW_WPB - 1) / ROW_WPB;
    const size_t smem = (size_t)ROW_WPB * 4 * N * sizeof(T);
    if (a.stage == 1) {
        auto k = row_stage_kernel<T, N, 0>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k<<<grid, ROW_WPB * WARP, smem, st>>>(a);
    } else if (a.stage <= 5) {
        auto k = row_stage_kernel<T, N, 1>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k<<<grid, ROW_WPB * WARP, smem, st>>>(a);
    } else {
        auto k = row_stage_kernel<T, N, 2>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k<<<grid, ROW_WPB * WARP, smem, st>>>(a);
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_row_stage(const StepArgs<T> &a, cudaStream_t st)
{
#define CASE(n_) if (a.nx == n_) return row_stage_n<T, n_>(a, st);
    SPARC_FFT_SIZES(CASE)
#undef CASE
    return cudaErrorInvalidValue;
}

template <typename T, int N>
static cudaError_t ddx_n(const T *var, T *dvar, int nrows, T stretchx, const T *twr, const T *twi, const T *kap,
                         cudaStream_t st)
{
    const int pairs = (nrows + 1) / 2;
    const int grid = (pairs + ROW_WPB - 1) / ROW_WPB;
    const size_t smem = (size_t)ROW_WPB * 4 * N * sizeof(T);
    auto k = ddx_kernel<T, N>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k<<<grid, ROW_WPB * WARP, smem, st>>>(var, dvar, nrows, stretchx, twr, twi, kap);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_ddx(const T *var, T *dvar, int nrows, int nx, T stretchx, const T *twr, const T *twi,
                       const T *kap, cudaStream_t st)
{
    if (nrows <= 0) return cudaSuccess;
#define CASE(n_) if (nx == n_) return ddx_n<T, n_>(var, dvar, nrows, stretchx, twr, twi, kap, st);
    SPARC_FFT_SIZES(CASE)
#undef CASE
    return cudaErrorInvalidValue;
}

// Kernel integral, x-derivatives of one record pair: d/dx of forward xi_x, v_x, v_z and of the
// adjoint v_x (compute_div / compute_del, kernels.f90:843-887).
template <typename T, int N>
__global__ void __launch_bounds__(ROW_WPB *WARP) kacc_row_kernel(KAccArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sm = reinterpret_cast<T *>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = blockIdx.x * ROW_WPB + warp;
    if (row >= a.nb * a.nz) return;
    T *xr = sm + warp * 4 * N, *xi = xr + N, *yr = xi + N, *yi = yr + N;
    const int b = row / a.nz, k = row - b * a.nz;
    const size_t F = (size_t)a.nz * N, ro = (size_t)k * N;
    const T *f = a.fsn + a.fbase + (size_t)b * a.fstride;
    const T *av = a.adj + (size_t)b * a.astride;
    T *w = a.work + (size_t)b * 4 * F;
    // forward xi_x with adjoint v_x, then forward v_x with v_z: the forward and adjoint fields
    // carry unrelated normalisations, so each row is scaled before it shares an FFT
    T mr = T(0), mi = T(0);
    for (int x = lane; x < N; x += WARP) {
        xr[x] = f[0 * F + ro + x];
        xi[x] = av[ro + x];
        mr = fmax(mr, fabs(xr[x]));
        mi = fmax(mi, fabs(xi[x]));
    }
    T sr, si, isr, isi;
    warp_row_scale(mr, sr, isr);
    warp_row_scale(mi, si, isi);
    __syncwarp();
    T *o1r, *o1i;
    fft_deriv<T, N>(xr, xi, yr, yi, a.twr, a.twi, a.kap, a.stretchx, lane, o1r, o1i, sr, si);
    __syncwarp();
    T mr2 = T(0), mi2 = T(0);
    for (int x = lane; x < N; x += WARP) {
        w[0 * F + ro + x] = o1r[x] * isr;
        w[1 * F + ro + x] = o1i[x] * isi;
        o1r[x] = f[2 * F + ro + x];
        o1i[x] = f[3 * F + ro + x];
        mr2 = fmax(mr2, fabs(o1r[x]));
        mi2 = fmax(mi2, fabs(o1i[x]));
    }
    T sr2, si2, isr2, isi2;
    warp_row_scale(mr2, sr2, isr2);
    warp_row_scale(mi2, si2, isi2);
    __syncwarp();
    T *gr = (o1r == xr) ? yr : xr, *gi = (o1r == xr) ? yi : xi;
    T *o2r, *o2i;
    fft_deriv<T, N>(o1r, o1i, gr, gi, a.twr, a.twi, a.kap, a.stretchx, lane, o2r, o2i, sr2, si2);
    __syncwarp();
    for (int x = lane; x < N; x += WARP) {
        w[2 * F + ro + x] = o2r[x] * isr2;
        w[3 * F + ro + x] = o2i[x] * isi2;
    }
}

template <typename T, int N>
static cudaError_t kacc_row_n(const KAccArgs<T> &a, cudaStream_t st)
{
    const int rows = a.nb * a.nz;
    const int grid = (rows + ROW_WPB - 1) / ROW_WPB;
    const size_t smem = (size_t)ROW_WPB * 4 * N * sizeof(T);
    auto k = kacc_row_kernel<T, N>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k<<<grid, ROW_WPB * WARP, smem, st>>>(a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_kacc_row(const KAccArgs<T> &a, cudaStream_t st)
{
#define CASE(n_) if (a.nx == n_) return kacc_row_n<T, n_>(a, st);
    SPARC_FFT_SIZES(CASE)
#undef CASE
    return cudaErrorInvalidValue;
}
template cudaError_t launch_kacc_row<float>(const KAccArgs<float> &, cudaStream_t);
template cudaError_t launch_kacc_row<double>(const KAccArgs<double> &, cudaStream_t);

template cudaError_t launch_row_stage<float>(const StepArgs<float> &, cudaStream_t);
template cudaError_t launch_row_stage<double>(const StepArgs<double> &, cudaStream_t);
template cudaError_t launch_ddx<float>(const float *, float *, int, int, float, const float *, const float *,
                                       const float *, cudaStream_t);
template cudaError_t launch_ddx<double>(const double *, double *, int, int, double, const double *,
                                        const double *, const double *, cudaStream_t);

}  // namespace sparc
