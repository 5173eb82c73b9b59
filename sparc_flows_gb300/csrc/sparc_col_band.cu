// sparc_col_band.cu -- column pass of an RK stage with the geometric-band compact derivative
// (FP32 plans), direct global loads.
//
// Same physics as col_stage_kernel (sparc_col.cu, physics2d.f90:943-1094); every z-derivative
// is evaluated by the geometric band of sparc_band.cuh instead of a tridiagonal solve.  A block
// owns CW adjacent x-columns (32, 16 or 8) of one solve over the full depth.  A warp reads 32/CW
// rows that are R apart; with R odd for CW < 32 they fall on disjoint banks.  Shared memory:
// two field columns F[nz][CW], two right-hand-side columns [nz][CW], the carries of two
// derivatives and seven depth profiles.
//
// On the specialised grids (TMA1) the first phase's three input tiles (xi_z and v_z of the state,
// the RHS of v_z two stages back) are staged by 2-D bulk tensor copies into the two RHS tiles and
// the second field tile, which are idle until phase 2: one thread issues them at kernel start,
// and the block stages its PML rows and depth profiles while they are in flight.  Once phase 1
// has read them, the same thread stages phase 3's dxi_x/dx and v_x tiles into the second RHS
// tile and the second field tile (free until phases 4 and 3), in flight during phase 2.  (The
// inputs of phases 5 and 7 are L2-prefetched instead: staging them too gained nothing.)
#include "sparc_band.cuh"
#include "sparc_tma.cuh"

namespace sparc {

constexpr uint32_t BAND_TMA_WAIT_ITERS = 1u << 24;
constexpr int BAND_SMEM_PAD = 16;  // the mbarrier after the PML rows (8 bytes, 8-byte aligned)

// Every thread waits (bounded) for the mbarrier phase of parity par, then par flips.  On a
// time-out anywhere in the block: the error flag is set, the copies are waited for again
// (bounded) and false is returned to every thread, which then leave the kernel.
__device__ __forceinline__ bool band_tma_wait(uint64_t *bar, uint32_t &par, int *d_err)
{
    const bool ok = mbar_wait_bounded(bar, par, BAND_TMA_WAIT_ITERS);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicExch(d_err, SPARC_DEV_ERR_TMA_TIMEOUT);
        mbar_wait_bounded(bar, par, BAND_TMA_WAIT_ITERS);
        __syncthreads();
        return false;
    }
    par ^= 1u;
    return true;
}

// One [nz][32] tile (two boxes of nz/2 rows) from rows row0 .. row0 + nz - 1 of map at x0.
template <int NZ>
__device__ __forceinline__ void band_tma_tile(float *dst, const CUtensorMap *map, int x0, int row0, uint64_t *bar)
{
    tma_load_2d(dst, map, x0, row0, bar);
    tma_load_2d(dst + (NZ / 2) * 32, map, x0, row0 + NZ / 2, bar);
}

// NX, NZ: the grid as compile-time constants (0: taken from the arguments).  With them every
// global and shared-memory offset of the unrolled row loops is an immediate, and with NZ a
// multiple of R every thread group is full; the generic instantiation serves other grids.
// TMA1 (CW = 32, even NZ with NZ/2 <= 256): the inputs of phases 1 and 3 staged by TMA through
// the maps m.
template <int CW, int R, int NX, int NZ, bool TMA1>
__global__ void __launch_bounds__(CW *band_maxg<CW>(), band_minb<CW>())
    col_band_kernel(StepArgs<float> a, BandDev bd, const __grid_constant__ ColMaps32 m)
{
    static_assert(!TMA1 || (CW == 32 && NZ > 0 && NZ % 2 == 0 && NZ / 2 <= 256), "TMA1 geometry");
    // tiles of nz x 32 floats are nz * 128 bytes long: with a 128-byte aligned base every tile and
    // half tile is a valid TMA destination
    extern __shared__ __align__(128) float smb[];
    const int nz = NZ ? NZ : a.nz, nx = NX ? NX : a.nx;
    const int G = blockDim.x / CW;
    const int ncar = 2 * G * CW + BandCarry<CW, R>::floats_fixed();
    float *FA = smb;
    float *FB = FA + (size_t)nz * CW;
    float *RA = FB + (size_t)nz * CW;  // right-hand sides
    float *RB = RA + (size_t)nz * CW;
    const BandCarry<CW, R> C0(RB + (size_t)nz * CW, G), C1(RB + (size_t)nz * CW + ncar, G);
    float *KPB = RB + (size_t)nz * CW + 2 * ncar;
    float *Kst = KPB, *Kri = KPB + nz, *Kr0 = KPB + 2 * nz, *Kgp = KPB + 3 * nz, *Kgr = KPB + 4 * nz, *Kg = KPB + 5 * nz,
          *Kc2 = KPB + 6 * nz;
    // vertical-PML inputs of this block's PML rows [5][nzpml][CW]: stage inputs of psi_vz and psi_p
    // (replaced by their new RHS once used), az, bz, fdz
    const int nzp = a.nzpml;
    float *PS = KPB + 7 * nz;
    // TMA1: the mbarrier, on the first 8-byte boundary after the PML rows
    uint64_t *bar = reinterpret_cast<uint64_t *>(smb + ((PS - smb + 5 * nzp * CW + 1) & ~1));
    uint32_t tma_par = 0;  // parity of the mbarrier phase awaited next
    const int s = a.stage;
    const int b = blockIdx.y;
    // stage overlap: every block has started once all have passed this point, so the row pass
    // launched as this grid's dependent takes only SMs that no block of this grid still needs
    if (a.tile_cnt) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if constexpr (TMA1) {
        if ((smem_u32(smb) & 127u) != 0) {  // uniform over the block: no copy is issued
            if (threadIdx.x == 0) atomicExch(a.d_err, SPARC_DEV_ERR_TMA_ALIGN);
            return;
        }
        // xi_z -> RA, v_z -> RB (s >= 2), RHS of v_z at stage s-2 -> FB (s >= 3), two boxes each
        if (threadIdx.x == 0) {
            mbar_init(bar, 1);
            fence_mbar_init();
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const uint32_t nt = 1 + (s >= 2 ? 1 : 0) + (s >= 3 ? 1 : 0);
            mbar_arrive_expect_tx(bar, nt * (uint32_t)NZ * CW * sizeof(float));
            const int x0 = blockIdx.x * CW;
            band_tma_tile<NZ>(RA, &m.A, x0, (b * 4 + F_XIZ) * NZ, bar);
            if (s >= 2) band_tma_tile<NZ>(RB, &m.A, x0, (b * 4 + F_VZ) * NZ, bar);
            if (s >= 3) band_tma_tile<NZ>(FB, &m.SV, x0, ((a.slot_sm2 * a.nb + b) * 2 + 1) * NZ, bar);
        }
    }
    for (int k = threadIdx.x; k < nz; k += blockDim.x) {  // depth profiles
        Kst[k] = __ldg(a.stretch + k);
        Kri[k] = __ldg(a.rhoinv + k);
        Kr0[k] = __ldg(a.rho0 + k);
        Kgp[k] = __ldg(a.gp0 + k);
        Kgr[k] = __ldg(a.gr0 + k);
        Kg[k] = __ldg(a.g + k);
        Kc2[k] = a.c2d ? 0.f : __ldg(a.c2rho0 + k);
    }
    const int c = threadIdx.x % CW, g = threadIdx.x / CW;
    const int x = blockIdx.x * CW + c;
    const int k0 = g * R;
    const int n = (NZ && NZ % R == 0) ? R : min(R, nz - k0);
    const size_t F = (size_t)nz * nx;
    const float *Ab = a.A + (size_t)b * 4 * F;
    const float bs = a.bs, bsm1 = a.bsm1;
    const int time = *a.d_time;
    const bool xbc = (x == 0 || x == nx - 1);
    // does this thread group hold vertical-PML rows (uniform over the group: a warp for CW = 32)
    const bool pml_group = k0 < a.npmlbot || k0 + n > nz - a.npmltop;
    const size_t spz_slot = (size_t)a.nb * 2 * nzp * nx;  // one slot of the PML RHS ring

    // Global stores wait until the loads of their phase are issued (every phase below loads,
    // computes into registers or shared memory, and stores last), so that the loads of one row
    // never queue behind a possibly aliasing store of the previous row.

    // ---- 0: PML inputs of the block's PML rows into shared memory, loads shared by all threads
    // (the PML thread groups alone would each load seven values per row and hold every other
    // group at the first barrier)
    for (int i = threadIdx.x; i < nzp * CW; i += blockDim.x) {
        const int pi = i / CW, cc = i - pi * CW;
        const int xx = blockIdx.x * CW + cc;
        const size_t qz = ((size_t)b * 2 * nzp + pi) * nx + xx;  // psi_vz; psi_p at + nzp * nx
        const size_t qb = (size_t)b * a.bgz + (size_t)pi * nx + xx;
        float p0 = __ldg(a.PZ + qz), p1 = __ldg(a.PZ + qz + (size_t)nzp * nx);
        if (s >= 2) {
            p0 += bs * __ldg(a.SPZ + a.slot_sm1 * spz_slot + qz);
            p1 += bs * __ldg(a.SPZ + a.slot_sm1 * spz_slot + qz + (size_t)nzp * nx);
        }
        PS[(0 * nzp + pi) * CW + cc] = p0;
        PS[(1 * nzp + pi) * CW + cc] = p1;
        PS[(2 * nzp + pi) * CW + cc] = __ldg(a.az + qb);
        PS[(3 * nzp + pi) * CW + cc] = __ldg(a.bz + qb);
        PS[(4 * nzp + pi) * CW + cc] = __ldg(a.fdz + qb);
    }

    // ---- 1: xi_z at stage s (scr xi_z = v_z of stage s-1 with the RHS boundary zeros)
    if constexpr (TMA1) {
        if (!band_tma_wait(bar, tma_par, a.d_err)) return;
    }
    float xz[R];
#pragma unroll
    for (int m = 0; m < R; m++) {
        xz[m] = 0.f;
        if (m < n) {
            const int k = k0 + m;
            float v;
            if constexpr (TMA1) {
                v = RA[k * CW + c];
                if (s >= 2) {
                    const float avz = RB[k * CW + c];
                    float t = (s == 2) ? avz : avz + bsm1 * FB[k * CW + c];
                    if (k == 0 || xbc) t = 0.f;
                    v += bs * t;
                }
            } else {
                const size_t q = (size_t)k * nx + x;
                v = __ldg(Ab + F_XIZ * F + q);
                if (s >= 2) {
                    const float avz = __ldg(Ab + F_VZ * F + q);
                    float t = (s == 2) ? avz : avz + bsm1 * __ldg(svp(a, a.slot_sm2, b, 1) + q);
                    if (k == 0 || xbc) t = 0.f;
                    v += bs * t;
                }
            }
            xz[m] = v;
            FA[k * CW + c] = v;
        }
    }
    __syncthreads();
    if constexpr (TMA1) {
        // phase 3's tiles: dxi_x/dx -> RB, v_x of the state -> FB: phase 1's generic-proxy reads of both tiles are
        // ordered before the copies by the barrier above and the proxy fence
        if (threadIdx.x == 0) {
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(bar, 2u * NZ * CW * sizeof(float));
            const int x0 = blockIdx.x * CW;
            band_tma_tile<NZ>(RB, &m.DX, x0, b * NZ, bar);
            band_tma_tile<NZ>(FB, &m.A, x0, (b * 4 + F_VX) * NZ, bar);
        }
    }
    // L2 prefetch of phase 3's per-point inputs of this thread group's rows (one 128-byte line
    // per array and row, spread over the lanes, no registers held), issued once phase 1's own
    // loads have been served so that they do not compete with them
    if constexpr (CW == 32) {
        const size_t ob = (size_t)k0 * nx + (size_t)blockIdx.x * CW;
        for (int i = c; i < 4 * R; i += CW) {
            const int ai = i / R, m = i - ai * R;
            if (m >= n) continue;
            const float *p;
            switch (ai) {
                case 0: p = TMA1 ? nullptr : a.DX + (size_t)b * F; break;
                case 1: p = TMA1 ? nullptr : Ab + F_VX * F; break;
                case 2: p = s >= 2 ? svp(a, a.slot_sm1, b, 0) : nullptr; break;
                case 3: p = a.c2d ? a.c2rho0 + (size_t)b * a.bg2 : nullptr; break;
                default: p = nullptr; break;
            }
            if (p) asm volatile("prefetch.global.L2 [%0];" ::"l"(p + ob + (size_t)m * nx) : "memory");
        }
    }
    // ---- 2: right-hand side of d xi_z/dz (ibc 3, top value -dxi_x/dx * unstretch)
    {
        float ra[R];
        const float preset3 = -__ldg(a.TOPDX + (size_t)b * nx + x) * a.unstretch_top;
        band_rhs<CW, R>(a.z3, FA, RA, c, k0, n, nz, preset3, ra);
        band_publish<CW, R>(bd, bd.uv[2], C0, c, g, k0, n, nz, ra);
    }
    __syncthreads();
    // ... and of phases 5 and 7's inputs, issued as phase 3 starts
    if constexpr (CW == 32) {
        const size_t ob = (size_t)k0 * nx + (size_t)blockIdx.x * CW;
        for (int i = c; i < 4 * R; i += CW) {
            const int ai = i / R, m = i - ai * R;
            if (m >= n) continue;
            const float *p;
            switch (ai) {
                case 0: p = a.flows ? a.FXX + (size_t)b * F : nullptr; break;
                case 1: p = s >= 2 ? svp(a, a.slot_sm1, b, 1) : nullptr; break;
                case 2: p = a.flows ? a.FXZ + (size_t)b * F : nullptr; break;
                case 3: p = a.flows ? a.v0z + (size_t)b * a.bg2 : nullptr; break;
                default: p = nullptr; break;
            }
            if (p) asm volatile("prefetch.global.L2 [%0];" ::"l"(p + ob + (size_t)m * nx) : "memory");
        }
    }
    // ---- 3: d xi_z/dz, vertical PML, divergence, pressure (kept in FA); v_x of stage s
    {
        float d[R];
        band_eval<CW, R>(bd, bd.uv[2], C0, c, g, G, k0, n, nz, RA, d);
        if constexpr (TMA1) {
            if (!band_tma_wait(bar, tma_par, a.d_err)) return;
        }
#pragma unroll
        for (int m = 0; m < R; m++) {
            if (m < n) {
                const int k = k0 + m;
                const size_t q = (size_t)k * nx + x;
                float dzz = d[m] * Kst[k];
                const int pi = pml_group ? pml_row(a, k) : -1;
                float fd = 1.f;
                if (pi >= 0) {
                    const float ps = PS[(0 * nzp + pi) * CW + c];
                    PS[(0 * nzp + pi) * CW + c] = PS[(2 * nzp + pi) * CW + c] * dzz + PS[(3 * nzp + pi) * CW + c] * ps;
                    dzz += ps;
                    fd = PS[(4 * nzp + pi) * CW + c];
                }
                const float div = (TMA1 ? RB[k * CW + c] : __ldg(a.DX + (size_t)b * F + q)) + dzz;
                const float c2r = a.c2d ? __ldg(a.c2rho0 + (size_t)b * a.bg2 + q) : Kc2[k];
                const float gp = Kgp[k] * fd, gr = Kgr[k] * fd;
                const float p = -c2r * div - gp * xz[m];
                const float rho = -Kr0[k] * div - gr * xz[m];
                xz[m] = rho * Kg[k];
                FA[k * CW + c] = p;
                float vx = TMA1 ? FB[k * CW + c] : __ldg(Ab + F_VX * F + q);
                if (s >= 2) vx += bs * __ldg(svp(a, a.slot_sm1, b, 0) + q);
                FB[k * CW + c] = vx;
            }
        }
    }
    __syncthreads();
    // ---- 4: right-hand sides of dp/dz (ibc 2, bottom value 0) and dv_x/dz (ibc 1); p to HBM
    {
        float rr[R];
        band_rhs<CW, R>(a.z2, FA, RA, c, k0, n, nz, 0.f, rr);
        band_publish<CW, R, false>(bd, bd.uv[1], C0, c, g, k0, n, nz, rr);
    }
    if (a.flows) {
        float rr[R];
        band_rhs<CW, R>(a.z1, FB, RB, c, k0, n, nz, 0.f, rr);
        band_publish<CW, R, false>(bd, bd.uv[0], C1, c, g, k0, n, nz, rr);
    }
#pragma unroll
    for (int m = 0; m < R; m++)
        if (m < n) a.P[(size_t)b * F + (size_t)(k0 + m) * nx + x] = FA[(k0 + m) * CW + c];
    for (int i = threadIdx.x; i < nzp * CW; i += blockDim.x) {  // new RHS of psi_vz (phase 3)
        const int pi = i / CW, cc = i - pi * CW;
        a.SPZ[a.slot_s * spz_slot + ((size_t)b * 2 * nzp + pi) * nx + blockIdx.x * CW + cc] = PS[(0 * nzp + pi) * CW + cc];
    }
    __syncthreads();
    // ---- 5: gradient of p, RHS v_z without advection; advection of v_x along z (partial RHS
    // v_x kept in FB); v_z of stage s
    {
        float d[R];
        band_eval<CW, R, 1>(bd, bd.uv[1], C0, c, g, G, k0, n, nz, RA, d);
#pragma unroll
        for (int m = 0; m < R; m++) {
            if (m < n) {
                const int k = k0 + m;
                float gpz = d[m] * Kst[k];
                const int pi = pml_group ? pml_row(a, k) : -1;
                if (pi >= 0) {
                    const float ps = PS[(1 * nzp + pi) * CW + c];
                    PS[(1 * nzp + pi) * CW + c] = PS[(2 * nzp + pi) * CW + c] * gpz + PS[(3 * nzp + pi) * CW + c] * ps;
                    gpz += ps;
                }
                xz[m] = -Kri[k] * (gpz + xz[m]);
            }
        }
        if (a.flows) band_eval<CW, R, 0>(bd, bd.uv[0], C1, c, g, G, k0, n, nz, RB, d);
#pragma unroll
        for (int m = 0; m < R; m++) {
            if (m < n) {
                const int k = k0 + m;
                const size_t q = (size_t)k * nx + x;
                float rv = 0.f;
                if (a.flows) {
                    const float dvxdz = d[m] * Kst[k];
                    rv = __ldg(a.FXX + (size_t)b * F + q) -
                         2.f * a.fsign * __ldg(a.v0z + (size_t)b * a.bg2 + q) * dvxdz;
                    float vz = __ldg(Ab + F_VZ * F + q);
                    if (s >= 2) vz += bs * __ldg(svp(a, a.slot_sm1, b, 1) + q);
                    FA[k * CW + c] = vz;
                }
                FB[k * CW + c] = rv;
            }
        }
    }
    __syncthreads();
    // ---- 6: right-hand side of dv_z/dz (ibc 1)
    if (a.flows) {
        float rr[R];
        band_rhs<CW, R>(a.z1, FA, RA, c, k0, n, nz, 0.f, rr);
        band_publish<CW, R, false>(bd, bd.uv[0], C0, c, g, k0, n, nz, rr);
        __syncthreads();
    }
    // ---- 7: finish RHS v_z (advection, source, boundary zeros); this stage's stores
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
#pragma unroll
    for (int m = 0; m < R; m++) {
        if (m < n) {
            const int k = k0 + m;
            const size_t q = (size_t)k * nx + x;
            float r = xz[m];
            if (k == a.k_inj) r += forcing;
            if (a.flows) {
                const float dvzdz = d[m] * Kst[k];
                r += __ldg(a.FXZ + (size_t)b * F + q) - 2.f * a.fsign * __ldg(a.v0z + (size_t)b * a.bg2 + q) * dvzdz;
            }
            if (k == 0 || xbc) r = 0.f;
            xz[m] = r;
        }
    }
    float *svz = svp(a, a.slot_s, b, 1);
#pragma unroll
    for (int m = 0; m < R; m++) {
        if (m < n) {
            const int k = k0 + m;
            const size_t q = (size_t)k * nx + x;
            svz[q] = xz[m];
            a.RVXP[(size_t)b * F + q] = FB[k * CW + c];
        }
    }
    for (int i = threadIdx.x; i < nzp * CW; i += blockDim.x) {  // new RHS of psi_p (phase 5)
        const int pi = i / CW, cc = i - pi * CW;
        a.SPZ[a.slot_s * spz_slot + ((size_t)b * 2 * nzp + pi + nzp) * nx + blockIdx.x * CW + cc] =
            PS[(1 * nzp + pi) * CW + cc];
    }
    if (a.tile_cnt) {  // this tile of solve b is done: its stores, then the count (release)
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(a.tile_cnt + (size_t)(s - 1) * a.nb + b, 1);
        }
    }
}

int col_band_rows(int nz, int cw)
{
    if (nz < 2 * BAND_KC + 2 * BAND_W) return 0;
    if (cw == 32) {
        for (int R : {8, 10, 12})
            if ((nz + R - 1) / R <= 32) return R;
    } else if (cw == 16 || cw == 8) {
        for (int R : {9, 11, 13})  // odd: the 32/CW row groups of a warp use disjoint banks
            if ((nz + R - 1) / R <= 28) return R;
    }
    return 0;
}

template <int CW, int R>
static size_t band_smem(int nz, int nzpml)
{
    const int G = (nz + R - 1) / R;
    return ((size_t)4 * nz * CW + 2 * ((size_t)2 * G * CW + BandCarry<CW, R>::floats_fixed()) + (size_t)7 * nz +
            (size_t)5 * nzpml * CW) * sizeof(float) + BAND_SMEM_PAD;
}

size_t col_band_smem_bytes(int nz, int nzpml, int R, int cw)
{
    switch (cw * 100 + R) {
        case 3208: return band_smem<32, 8>(nz, nzpml);
        case 3210: return band_smem<32, 10>(nz, nzpml);
        case 3212: return band_smem<32, 12>(nz, nzpml);
        case 1609: return band_smem<16, 9>(nz, nzpml);
        case 1611: return band_smem<16, 11>(nz, nzpml);
        case 1613: return band_smem<16, 13>(nz, nzpml);
        case 809: return band_smem<8, 9>(nz, nzpml);
        case 811: return band_smem<8, 11>(nz, nzpml);
        case 813: return band_smem<8, 13>(nz, nzpml);
        default: return ~(size_t)0;
    }
}

template <int CW, int R, int NX, int NZ, bool TMA1>
static cudaError_t launch_band(const StepArgs<float> &a, const BandDev &bd, const ColMaps32 &m, cudaStream_t st)
{
    const int G = (a.nz + R - 1) / R;
    if (G > band_maxg<CW>() || a.nx % CW != 0 || R * G - a.nz >= R) return cudaErrorInvalidValue;
    if ((NX && a.nx != NX) || (NZ && a.nz != NZ)) return cudaErrorInvalidValue;
    const size_t smem = band_smem<CW, R>(a.nz, a.nzpml);
    auto kern = col_band_kernel<CW, R, NX, NZ, TMA1>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(a.nx / CW, a.nb);
    kern<<<grid, G * CW, smem, st>>>(a, bd, m);
    return cudaGetLastError();
}

// Grids with a compiled specialisation: nz = 300 (the reference's params.i depth) with the
// 32-column, 10-row geometry and nx = 128, 256, 384, 512, 1024.
bool col_band_specialised(int nx, int nz, int cw, int R)
{
    return cw == 32 && R == 10 && nz == 300 && (nx == 128 || nx == 256 || nx == 384 || nx == 512 || nx == 1024);
}

template <int CW, int R, int NX, int NZ>
static cudaError_t launch_band_sp(const StepArgs<float> &a, const BandDev &bd, const ColMaps32 *m32, cudaStream_t st)
{
    if (m32) return launch_band<CW, R, NX, NZ, true>(a, bd, *m32, st);
    return launch_band<CW, R, NX, NZ, false>(a, bd, ColMaps32{}, st);
}

template <int CW, int R>
cudaError_t launch_col_stage_band(const StepArgs<float> &a, const BandDev &bd, const ColMaps32 *m32, cudaStream_t st)
{
    if constexpr (CW == 32 && R == 10) {
        if (a.nz == 300) {
            switch (a.nx) {
                case 128: return launch_band_sp<32, 10, 128, 300>(a, bd, m32, st);
                case 256: return launch_band_sp<32, 10, 256, 300>(a, bd, m32, st);
                case 384: return launch_band_sp<32, 10, 384, 300>(a, bd, m32, st);
                case 512: return launch_band_sp<32, 10, 512, 300>(a, bd, m32, st);
                case 1024: return launch_band_sp<32, 10, 1024, 300>(a, bd, m32, st);
                default: break;
            }
        }
    }
    return launch_band<CW, R, 0, 0, false>(a, bd, ColMaps32{}, st);
}

#define SPARC_BAND_INST(cw, r)                                                                                    \
    template cudaError_t launch_col_stage_band<cw, r>(const StepArgs<float> &, const BandDev &, const ColMaps32 *, \
                                                      cudaStream_t);
SPARC_BAND_INST(32, 8)
SPARC_BAND_INST(32, 10)
SPARC_BAND_INST(32, 12)
SPARC_BAND_INST(16, 9)
SPARC_BAND_INST(16, 11)
SPARC_BAND_INST(16, 13)
SPARC_BAND_INST(8, 9)
SPARC_BAND_INST(8, 11)
SPARC_BAND_INST(8, 13)
#undef SPARC_BAND_INST

}  // namespace sparc
