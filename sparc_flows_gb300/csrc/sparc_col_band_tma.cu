// sparc_col_band_tma.cu -- column pass of an RK stage (FP32 plans): geometric-band compact
// derivative (sparc_band.cuh) with every per-point input staged by TMA.
//
// Same physics as col_stage_kernel (sparc_col.cu, physics2d.f90:943-1094).  A block owns 8
// adjacent x-columns (one 32-byte sector per row) of one solve over the full depth.  One thread
// issues 2-D bulk tensor copies of the input tiles ([2 boxr][8] each, boxr >= nz/2) of all
// phases at block start, each phase's tiles completing on their own mbarrier, so the block's
// loads are all in flight at once and no load sits on a dependency chain; two buffers are
// refilled by TMA as soon as the phase that read them has passed a barrier.  Tile roles:
//   0  xi_z -> xi_z of stage s (field of d/dz)   then  rhs(v_z) ring tile of stage s-1
//   1  v_z  -> v_z of stage s (field of d/dz)
//   2  rhs(v_z) of stage s-2                     then  right-hand sides A
//   3  dxi_x/dx -> pressure (field of d/dz)
//   4  c2rho0 (2-D background)                   then  right-hand sides B
//   5  v_x  -> v_x of stage s (field of d/dz)
//   6  rhs(v_x) of stage s-1                     then  x-advection of v_z (FXZ)
//   7  x-advection of v_x (FXX)
//   8  v0z
// Every mbarrier wait is bounded; on time-out the block records SPARC_DEV_ERR_TMA_TIMEOUT,
// waits (bounded) for the copies it issued and leaves.  With 8 columns and R odd, the four row
// groups of a warp fall on disjoint shared-memory banks.
#include "sparc_band.cuh"
#include "sparc_tma.cuh"

namespace sparc {

constexpr int BT_CW = 8;
constexpr int BT_NBUF = 9, BT_NBAR = 5;
constexpr uint32_t BT_WAIT_ITERS = 1u << 24;

// End of a phase: every thread arrives, and barrier bi's tiles have landed; false (for the whole
// block) if the bounded wait gave up.
__device__ __forceinline__ bool bt_phase(uint64_t *bar, int bi)
{
    const bool ok = (bi < 0) || mbar_wait_bounded(bar + bi, 0, BT_WAIT_ITERS);
    return !__syncthreads_or(!ok);
}

// Time-out exit: record the error, wait (bounded) for every armed barrier, leave together.
__device__ __forceinline__ void bt_abort(uint64_t *bar, int armed, int *d_err)
{
    if (threadIdx.x == 0) atomicExch(d_err, SPARC_DEV_ERR_TMA_TIMEOUT);
    for (int i = 0; i < armed; i++) mbar_wait_bounded(bar + i, 0, BT_WAIT_ITERS);
    __syncthreads();
}

template <int R>
__global__ void __launch_bounds__(BT_CW * 32, 2)
    col_band_tma_kernel(const __grid_constant__ ColMaps maps, StepArgs<float> a, BandDev bd)
{
    constexpr int CW = BT_CW;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);
    const int nz = a.nz, nx = a.nx, boxr = a.boxr;
    const size_t TE = (size_t)2 * boxr * CW;  // floats per tile (a multiple of 128 bytes)
    float *tiles = reinterpret_cast<float *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + BT_NBAR * sizeof(uint64_t) + 127) & ~uintptr_t(127));
    float *B0 = tiles, *B1 = B0 + TE, *B2 = B1 + TE, *B3 = B2 + TE, *B4 = B3 + TE, *B5 = B4 + TE, *B6 = B5 + TE,
          *B7 = B6 + TE, *B8 = B7 + TE;
    const int G = blockDim.x / CW;
    const int ncar = 2 * G * CW + BandCarry<CW, R>::floats_fixed();
    float *carb = tiles + BT_NBUF * TE;
    const BandCarry<CW, R> C0(carb, G), C1(carb + ncar, G);
    float *KPB = carb + 2 * ncar;
    float *Kst = KPB, *Kri = KPB + nz, *Kr0 = KPB + 2 * nz, *Kgp = KPB + 3 * nz, *Kgr = KPB + 4 * nz, *Kg = KPB + 5 * nz,
          *Kc2 = KPB + 6 * nz;
    for (int k = threadIdx.x; k < nz; k += blockDim.x) {  // depth profiles
        Kst[k] = __ldg(a.stretch + k);
        Kri[k] = __ldg(a.rhoinv + k);
        Kr0[k] = __ldg(a.rho0 + k);
        Kgp[k] = __ldg(a.gp0 + k);
        Kgr[k] = __ldg(a.gr0 + k);
        Kg[k] = __ldg(a.g + k);
        Kc2[k] = a.c2d ? 0.f : __ldg(a.c2rho0 + k);
    }
    float *RA = B2, *RB = B4;

    const int c = threadIdx.x % CW, g = threadIdx.x / CW;
    const int x0 = blockIdx.x * CW, x = x0 + c;
    const int b = blockIdx.y;
    const int k0 = g * R;
    const int n = min(R, nz - k0);
    const size_t F = (size_t)nz * nx;
    const int s = a.stage;
    const float bs = a.bs, bsm1 = a.bsm1;
    const int time = *a.d_time;
    const int bgrow = a.bg2 ? b * nz : 0;  // first row of this solve's 2-D background
    const uint32_t tileb = (uint32_t)(2 * boxr * CW * sizeof(float));

    auto load = [&](float *dst, const CUtensorMap *m, int row0, uint64_t *br) {
        tma_load_2d(dst, m, x0, row0, br);
        tma_load_2d(dst + (size_t)boxr * CW, m, x0, row0 + boxr, br);
    };
    const int sv1 = (a.slot_sm1 * a.nb + b) * 2, sv2 = (a.slot_sm2 * a.nb + b) * 2;
    if (threadIdx.x == 0) {
        for (int i = 0; i < BT_NBAR; i++) mbar_init(bar + i, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // phase 1: xi_z, v_z, rhs(v_z) of stage s-2
        mbar_arrive_expect_tx(bar + 0, tileb * (2 + (s >= 3 ? 1 : 0)));
        load(B0, &maps.A, (b * 4 + F_XIZ) * nz, bar + 0);
        load(B1, &maps.A, (b * 4 + F_VZ) * nz, bar + 0);
        if (s >= 3) load(B2, &maps.SV, (sv2 + 1) * nz, bar + 0);
        // phase 3: dxi_x/dx, c2rho0, v_x, rhs(v_x) of stage s-1
        mbar_arrive_expect_tx(bar + 1, tileb * (2 + (a.c2d ? 1 : 0) + (s >= 2 ? 1 : 0)));
        load(B3, &maps.DX, b * nz, bar + 1);
        if (a.c2d) load(B4, &maps.C2R, bgrow, bar + 1);
        load(B5, &maps.A, (b * 4 + F_VX) * nz, bar + 1);
        if (s >= 2) load(B6, &maps.SV, (sv1 + 0) * nz, bar + 1);
        // phase 5: FXX, v0z
        mbar_arrive_expect_tx(bar + 2, tileb * (a.flows ? 2 : 0));
        if (a.flows) {
            load(B7, &maps.FXX, b * nz, bar + 2);
            load(B8, &maps.V0Z, bgrow, bar + 2);
        }
    }
    const float preset3 = -__ldg(a.TOPDX + (size_t)b * nx + x) * a.unstretch_top;
    if (!bt_phase(bar, 0)) { bt_abort(bar, 3, a.d_err); return; }

    // ---- 1: xi_z at stage s, in place (scr xi_z = v_z of stage s-1 with the RHS boundary zeros)
    float xz[R];
#pragma unroll
    for (int m = 0; m < R; m++) {
        xz[m] = 0.f;
        if (m < n) {
            const int k = k0 + m, q = k * CW + c;
            float v = B0[q];
            if (s >= 2) {
                float t = B1[q];
                if (s >= 3) t += bsm1 * B2[q];
                if (k == 0 || x == 0 || x == nx - 1) t = 0.f;
                v += bs * t;
            }
            xz[m] = v;
            B0[q] = v;
        }
    }
    __syncthreads();
    // ---- 2: right-hand side of d xi_z/dz (ibc 3, top value -dxi_x/dx * unstretch)
    {
        float rr[R];
        band_rhs<CW, R>(a.z3, B0, RA, c, k0, n, nz, preset3, rr);
        band_publish<CW, R>(bd, bd.uv[2], C0, c, g, k0, n, nz, rr);
    }
    if (!bt_phase(bar, 1)) { bt_abort(bar, 3, a.d_err); return; }
    if (threadIdx.x == 0) {  // tile 0 is free: rhs(v_z) of stage s-1 for phase 5
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(bar + 3, tileb * (s >= 2 ? 1 : 0));
        if (s >= 2) load(B0, &maps.SV, (sv1 + 1) * nz, bar + 3);
    }
    // ---- 3: d xi_z/dz, vertical PML, divergence, pressure (tile 3); v_x of stage s (tile 5)
    {
        float d[R];
        band_eval<CW, R>(bd, bd.uv[2], C0, c, g, G, k0, n, nz, RA, d);
#pragma unroll
        for (int m = 0; m < R; m++) {
            if (m < n) {
                const int k = k0 + m, q = k * CW + c;
                const size_t gq = (size_t)k * nx + x;
                float dzz = d[m] * Kst[k];
                const int pi = pml_row(a, k);
                float fd = 1.f;
                if (pi >= 0) {
                    const size_t qz = ((size_t)b * 2 * a.nzpml + pi) * nx + x;  // psi_vz
                    const size_t qb = (size_t)b * a.bgz + (size_t)pi * nx + x;
                    float ps = __ldg(a.PZ + qz);
                    if (s >= 2) ps += bs * __ldg(a.SPZ + (size_t)a.slot_sm1 * a.nb * 2 * a.nzpml * nx + qz);
                    a.SPZ[(size_t)a.slot_s * a.nb * 2 * a.nzpml * nx + qz] =
                        __ldg(a.az + qb) * dzz + __ldg(a.bz + qb) * ps;
                    dzz += ps;
                    fd = __ldg(a.fdz + qb);
                }
                const float div = B3[q] + dzz;
                const float c2r = a.c2d ? B4[q] : Kc2[k];
                const float gp = Kgp[k] * fd, gr = Kgr[k] * fd;
                const float p = -c2r * div - gp * xz[m];
                const float rho = -Kr0[k] * div - gr * xz[m];
                xz[m] = rho * Kg[k];
                B3[q] = p;
                a.P[(size_t)b * F + gq] = p;
                float vx = B5[q];
                if (s >= 2) vx += bs * B6[q];
                B5[q] = vx;
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // tile 6 is free: x-advection of v_z for phase 7
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(bar + 4, tileb * (a.flows ? 1 : 0));
        if (a.flows) load(B6, &maps.FXZ, b * nz, bar + 4);
    }
    // ---- 4: right-hand sides of dp/dz (ibc 2, bottom value 0) and dv_x/dz (ibc 1)
    {
        float rr[R];
        band_rhs<CW, R>(a.z2, B3, RA, c, k0, n, nz, 0.f, rr);
        band_publish<CW, R, false>(bd, bd.uv[1], C0, c, g, k0, n, nz, rr);
    }
    if (a.flows) {
        float rr[R];
        band_rhs<CW, R>(a.z1, B5, RB, c, k0, n, nz, 0.f, rr);
        band_publish<CW, R, false>(bd, bd.uv[0], C1, c, g, k0, n, nz, rr);
    }
    if (!bt_phase(bar, 2) || !bt_phase(bar, 3)) { bt_abort(bar, 5, a.d_err); return; }
    // ---- 5: gradient of p, RHS v_z without advection; advection of v_x along z; v_z of stage s
    {
        float d[R];
        band_eval<CW, R, 1>(bd, bd.uv[1], C0, c, g, G, k0, n, nz, RA, d);
#pragma unroll
        for (int m = 0; m < R; m++) {
            if (m < n) {
                const int k = k0 + m;
                float gpz = d[m] * Kst[k];
                const int pi = pml_row(a, k);
                if (pi >= 0) {
                    const size_t qz = (((size_t)b * 2 + 1) * a.nzpml + pi) * nx + x;  // psi_p
                    const size_t qb = (size_t)b * a.bgz + (size_t)pi * nx + x;
                    float ps = __ldg(a.PZ + qz);
                    if (s >= 2) ps += bs * __ldg(a.SPZ + (size_t)a.slot_sm1 * a.nb * 2 * a.nzpml * nx + qz);
                    a.SPZ[(size_t)a.slot_s * a.nb * 2 * a.nzpml * nx + qz] =
                        __ldg(a.az + qb) * gpz + __ldg(a.bz + qb) * ps;
                    gpz += ps;
                }
                xz[m] = -Kri[k] * (gpz + xz[m]);
            }
        }
        if (a.flows) band_eval<CW, R, 0>(bd, bd.uv[0], C1, c, g, G, k0, n, nz, RB, d);
#pragma unroll
        for (int m = 0; m < R; m++) {
            if (m < n) {
                const int k = k0 + m, q = k * CW + c;
                float rv = 0.f;
                if (a.flows) rv = B7[q] - 2.f * a.fsign * B8[q] * (d[m] * Kst[k]);
                a.RVXP[(size_t)b * F + (size_t)k * nx + x] = rv;
                float vz = B1[q];
                if (s >= 2) vz += bs * B0[q];
                B1[q] = vz;
            }
        }
    }
    __syncthreads();
    // ---- 6: right-hand side of dv_z/dz (ibc 1)
    if (a.flows) {
        float rr[R];
        band_rhs<CW, R>(a.z1, B1, RA, c, k0, n, nz, 0.f, rr);
        band_publish<CW, R, false>(bd, bd.uv[0], C0, c, g, k0, n, nz, rr);
    }
    if (!bt_phase(bar, 4)) { bt_abort(bar, 5, a.d_err); return; }
    // ---- 7: finish RHS v_z (advection, source, boundary zeros)
    float d[R];
    if (a.flows) band_eval<CW, R, 0>(bd, bd.uv[0], C0, c, g, G, k0, n, nz, RA, d);
    float forcing = 0.f;
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
        forcing = (float)f * __ldg(a.inj_scale + (size_t)b * nx + x);
    }
    float *svz = svp(a, a.slot_s, b, 1);
#pragma unroll
    for (int m = 0; m < R; m++) {
        if (m < n) {
            const int k = k0 + m, q = k * CW + c;
            float r = xz[m];
            if (k == a.k_inj) r += forcing;
            if (a.flows) r += B6[q] - 2.f * a.fsign * B8[q] * (d[m] * Kst[k]);
            if (k == 0 || x == 0 || x == nx - 1) r = 0.f;
            svz[(size_t)k * nx + x] = r;
        }
    }
}

int col_band_tma_rows(int nz)
{
    if (nz < 2 * BAND_KC + 2 * BAND_W) return 0;
    for (int R : {9, 11, 13})  // odd: the four row groups of a warp use disjoint banks
        if ((nz + R - 1) / R <= 32) return R;
    return 0;
}

template <int R>
static size_t band_tma_smem(int nz, int boxr)
{
    const int G = (nz + R - 1) / R;
    const size_t ncar = (size_t)2 * G * BT_CW + BandCarry<BT_CW, R>::floats_fixed();
    return 128 + 128 + ((size_t)BT_NBUF * 2 * boxr * BT_CW + 2 * ncar + (size_t)7 * nz) * sizeof(float);
}

size_t col_band_tma_smem_bytes(int nz, int R, int boxr)
{
    switch (R) {
        case 9: return band_tma_smem<9>(nz, boxr);
        case 11: return band_tma_smem<11>(nz, boxr);
        case 13: return band_tma_smem<13>(nz, boxr);
        default: return ~(size_t)0;
    }
}

template <int R>
cudaError_t launch_col_stage_band_tma(const ColMaps &maps, const StepArgs<float> &a, const BandDev &bd, cudaStream_t st)
{
    const int G = (a.nz + R - 1) / R;
    if (G > 32 || a.nx % BT_CW != 0 || 2 * a.boxr < a.nz) return cudaErrorInvalidValue;
    const size_t smem = band_tma_smem<R>(a.nz, a.boxr);
    cudaError_t e =
        cudaFuncSetAttribute(col_band_tma_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(a.nx / BT_CW, a.nb);
    col_band_tma_kernel<R><<<grid, G * BT_CW, smem, st>>>(maps, a, bd);
    return cudaGetLastError();
}

template cudaError_t launch_col_stage_band_tma<9>(const ColMaps &, const StepArgs<float> &, const BandDev &, cudaStream_t);
template cudaError_t launch_col_stage_band_tma<11>(const ColMaps &, const StepArgs<float> &, const BandDev &, cudaStream_t);
template cudaError_t launch_col_stage_band_tma<13>(const ColMaps &, const StepArgs<float> &, const BandDev &, cudaStream_t);

}  // namespace sparc
