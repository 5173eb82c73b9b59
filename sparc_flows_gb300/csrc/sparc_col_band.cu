// sparc_col_band.cu -- column pass of an RK stage with the banded compact derivative (FP32).
//
// Same physics as col_stage_kernel (sparc_col.cu, physics2d.f90:943-1094); the tridiagonal
// solve of every z-derivative (dbyd2.f:8-235, mtridag.f:96-112) is replaced by its banded
// inverse, which has no serial dependence along z:
//   1. rhs[k] is formed exactly as dbyd2 forms it (c1/c2 differences, boundary closures, the
//      caller-set row) and stored in a zero-padded shared-memory column;
//   2. x[k] = sum_{|d|<=20} t[|d|] rhs[k+d] + rank-2 corner corrections (BandDev).
// The band truncation is 5e-10 of t[0], far below FP32 rounding; FP64 plans keep the exact
// partitioned solve.
//
// A block owns CW adjacent x-columns (32, 16 or 8) of one solve over the full depth; thread
// group g (CW threads, one per column) holds rows [g R, g R + R).  A warp therefore reads 32/CW
// rows that are R apart; with R odd for CW < 32 they fall on disjoint banks, so shared memory
// is conflict-free.  Narrow blocks let 2 (CW 16) or 4 (CW 8) blocks share an SM, so one block's
// barrier and load waits overlap another's band sums.  The band coefficients are kernel
// parameters addressed with compile-time offsets.  Shared memory: two field columns
// F[nz][CW] and two padded right-hand-side columns [G R + 40][CW].
#include "sparc_common.cuh"

namespace sparc {

template <int CW>
constexpr int band_maxg() { return CW == 32 ? 32 : 28; }  // thread groups per block
template <int CW>
constexpr int band_minb() { return CW == 32 ? 1 : (CW == 16 ? 2 : 4); }  // resident blocks per SM

// x[r] = sum_d t[|d|] rhs[k0 + r + d] for r < R (rhs rows outside 0..nz-1 read as zero).
template <int CW, int R>
__device__ __forceinline__ void band_sum(const BandDev &bd, const float *Rp, int c, int k0, float (&x)[R])
{
#pragma unroll
    for (int r = 0; r < R; r++) x[r] = 0.f;
#pragma unroll
    for (int i = -BAND_W; i < R + BAND_W; i++) {
        const float v = Rp[(k0 + i) * CW + c];
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int d = i - r;
            if (d >= -BAND_W && d <= BAND_W) x[r] = fmaf(bd.t[d < 0 ? -d : d], v, x[r]);
        }
    }
}

// Corner corrections of the rows [k0, k0 + n) that lie within BAND_KC of either end.
template <int CW, int R>
__device__ __forceinline__ void band_corners(const float *__restrict__ uv, const float *Rp, int c, int k0, int n,
                                             int nz, float (&x)[R])
{
    constexpr int KC = BAND_KC, Q = BAND_Q;
    if (k0 < KC) {
        const float *Ub = uv, *Vb = uv + KC * Q;
        float s[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) s[q] = 0.f;
#pragma unroll 4
        for (int j = 0; j < KC; j++) {
            const float v = Rp[j * CW + c];
#pragma unroll
            for (int q = 0; q < Q; q++) s[q] = fmaf(__ldg(Vb + q * KC + j), v, s[q]);
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int k = k0 + r;
            if (r < n && k < KC)
#pragma unroll
                for (int q = 0; q < Q; q++) x[r] = fmaf(__ldg(Ub + k * Q + q), s[q], x[r]);
        }
    }
    const int o = nz - KC;
    if (k0 + n > o) {
        const float *Ut = uv + 2 * KC * Q, *Vt = uv + 3 * KC * Q;
        float s[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) s[q] = 0.f;
#pragma unroll 4
        for (int j = 0; j < KC; j++) {
            const float v = Rp[(o + j) * CW + c];
#pragma unroll
            for (int q = 0; q < Q; q++) s[q] = fmaf(__ldg(Vt + q * KC + j), v, s[q]);
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int k = k0 + r - o;
            if (r < n && k >= 0)
#pragma unroll
                for (int q = 0; q < Q; q++) x[r] = fmaf(__ldg(Ut + k * Q + q), s[q], x[r]);
        }
    }
}

// Right-hand side of the rows [k0, k0 + n) of field column Fc into the padded column Rp.
template <int CW, int R>
__device__ __forceinline__ void band_rhs(const ZTab<float> &tb, const float *Fc, float *Rp, int c, int k0, int n,
                                         int nz, float preset)
{
#pragma unroll
    for (int m = 0; m < R; m++)
        if (m < n) Rp[(k0 + m) * CW + c] = zrhs(tb, Fc, CW, c, k0 + m, nz, preset);
}

template <int CW, int R>
__device__ __forceinline__ void band_deriv(const BandDev &bd, int which, const float *Rp, int c, int k0, int n,
                                           int nz, float (&x)[R])
{
    band_sum<CW, R>(bd, Rp, c, k0, x);
    band_corners<CW, R>(bd.uv[which], Rp, c, k0, n, nz, x);
}

template <int CW, int R>
__global__ void __launch_bounds__(CW *band_maxg<CW>(), band_minb<CW>()) col_band_kernel(StepArgs<float> a, BandDev bd)
{
    extern __shared__ __align__(16) float smb[];
    const int nz = a.nz, nx = a.nx;
    const int G = blockDim.x / CW;
    const int NPR = G * R + 2 * BAND_W;
    float *FA = smb;
    float *FB = FA + (size_t)nz * CW;
    float *RA = FB + (size_t)nz * CW + BAND_W * CW;  // row 0 of a padded column
    float *RB = RA + (size_t)NPR * CW;
    const int c = threadIdx.x % CW, g = threadIdx.x / CW;
    const int x = blockIdx.x * CW + c;
    const int b = blockIdx.y;
    const int k0 = g * R;
    const int n = min(R, nz - k0);
    const size_t F = (size_t)nz * nx;
    const float *Ab = a.A + (size_t)b * 4 * F;
    const int s = a.stage;
    const float bs = a.bs, bsm1 = a.bsm1;
    const int time = *a.d_time;

    // zero rows [-W, 0) and [nz, G R + W) of both right-hand-side columns
    {
        const int npad = BAND_W + (G * R + BAND_W - nz);
        for (int i = threadIdx.x; i < npad * CW; i += blockDim.x) {
            const int rr = i / CW, cc = i % CW;
            const int k = rr < BAND_W ? rr - BAND_W : nz + (rr - BAND_W);
            RA[k * CW + cc] = 0.f;
            RB[k * CW + cc] = 0.f;
        }
    }
    // ---- 1: xi_z at stage s (scr xi_z = v_z of stage s-1 with the RHS boundary zeros)
    float xz[R];
#pragma unroll
    for (int m = 0; m < R; m++) {
        if (m < n) {
            const int k = k0 + m;
            const size_t q = (size_t)k * nx + x;
            float v = __ldg(Ab + F_XIZ * F + q);
            if (s >= 2) {
                const float avz = __ldg(Ab + F_VZ * F + q);
                float t = (s == 2) ? avz : avz + bsm1 * __ldg(svp(a, a.slot_sm2, b, 1) + q);
                if (k == 0 || x == 0 || x == nx - 1) t = 0.f;
                v += bs * t;
            }
            xz[m] = v;
            FA[k * CW + c] = v;
        }
    }
    __syncthreads();
    // ---- 2: right-hand side of d xi_z/dz (ibc 3, top value -dxi_x/dx * unstretch)
    const float preset3 = -__ldg(a.TOPDX + (size_t)b * nx + x) * a.unstretch_top;
    band_rhs<CW, R>(a.z3, FA, RA, c, k0, n, nz, preset3);
    __syncthreads();
    // ---- 3: d xi_z/dz, vertical PML, divergence, pressure; v_x of stage s
    {
        float d[R];
        band_deriv<CW, R>(bd, 2, RA, c, k0, n, nz, d);
#pragma unroll
        for (int m = 0; m < R; m++) {
            if (m < n) {
                const int k = k0 + m;
                const size_t q = (size_t)k * nx + x;
                float dzz = d[m] * __ldg(a.stretch + k);
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
                const float div = __ldg(a.DX + (size_t)b * F + q) + dzz;
                const float c2r = a.c2d ? __ldg(a.c2rho0 + (size_t)b * a.bg2 + q) : __ldg(a.c2rho0 + k);
                const float gp = __ldg(a.gp0 + k) * fd, gr = __ldg(a.gr0 + k) * fd;
                const float p = -c2r * div - gp * xz[m];
                const float rho = -__ldg(a.rho0 + k) * div - gr * xz[m];
                xz[m] = rho * __ldg(a.g + k);
                FA[k * CW + c] = p;
                a.P[(size_t)b * F + q] = p;
                float vx = __ldg(Ab + F_VX * F + q);
                if (s >= 2) vx += bs * __ldg(svp(a, a.slot_sm1, b, 0) + q);
                FB[k * CW + c] = vx;
            }
        }
    }
    __syncthreads();
    // ---- 4: right-hand sides of dp/dz (ibc 2, bottom value 0) and dv_x/dz (ibc 1)
    band_rhs<CW, R>(a.z2, FA, RA, c, k0, n, nz, 0.f);
    if (a.flows) band_rhs<CW, R>(a.z1, FB, RB, c, k0, n, nz, 0.f);
    __syncthreads();
    // ---- 5: gradient of p, RHS v_z without advection; advection of v_x along z; v_z of stage s
    {
        float d[R];
        band_deriv<CW, R>(bd, 1, RA, c, k0, n, nz, d);
#pragma unroll
        for (int m = 0; m < R; m++) {
            if (m < n) {
                const int k = k0 + m;
                float gpz = d[m] * __ldg(a.stretch + k);
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
                xz[m] = -__ldg(a.rhoinv + k) * (gpz + xz[m]);
            }
        }
        if (a.flows) band_deriv<CW, R>(bd, 0, RB, c, k0, n, nz, d);
#pragma unroll
        for (int m = 0; m < R; m++) {
            if (m < n) {
                const int k = k0 + m;
                const size_t q = (size_t)k * nx + x;
                float rv = 0.f;
                if (a.flows) {
                    const float dvxdz = d[m] * __ldg(a.stretch + k);
                    rv = __ldg(a.FXX + (size_t)b * F + q) -
                         2.f * a.fsign * __ldg(a.v0z + (size_t)b * a.bg2 + q) * dvxdz;
                }
                a.RVXP[(size_t)b * F + q] = rv;
                float vz = __ldg(Ab + F_VZ * F + q);
                if (s >= 2) vz += bs * __ldg(svp(a, a.slot_sm1, b, 1) + q);
                FA[k * CW + c] = vz;
            }
        }
    }
    __syncthreads();
    // ---- 6: right-hand side of dv_z/dz (ibc 1)
    if (a.flows) {
        band_rhs<CW, R>(a.z1, FA, RA, c, k0, n, nz, 0.f);
        __syncthreads();
    }
    // ---- 7: finish RHS v_z (advection, source, boundary zeros)
    float d[R];
    if (a.flows) band_deriv<CW, R>(bd, 0, RA, c, k0, n, nz, d);
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
            const int k = k0 + m;
            const size_t q = (size_t)k * nx + x;
            float r = xz[m];
            if (k == a.k_inj) r += forcing;
            if (a.flows) {
                const float dvzdz = d[m] * __ldg(a.stretch + k);
                r += __ldg(a.FXZ + (size_t)b * F + q) - 2.f * a.fsign * __ldg(a.v0z + (size_t)b * a.bg2 + q) * dvzdz;
            }
            if (k == 0 || x == 0 || x == nx - 1) r = 0.f;
            svz[q] = r;
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

size_t col_band_smem_bytes(int nz, int R, int cw)
{
    const int G = (nz + R - 1) / R;
    return ((size_t)2 * nz + 2 * ((size_t)G * R + 2 * BAND_W)) * cw * sizeof(float);
}

template <int CW, int R>
cudaError_t launch_col_stage_band(const StepArgs<float> &a, const BandDev &bd, cudaStream_t st)
{
    const int G = (a.nz + R - 1) / R;
    if (G > band_maxg<CW>() || a.nx % CW != 0) return cudaErrorInvalidValue;
    const size_t smem = col_band_smem_bytes(a.nz, R, CW);
    cudaError_t e =
        cudaFuncSetAttribute(col_band_kernel<CW, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(a.nx / CW, a.nb);
    col_band_kernel<CW, R><<<grid, G * CW, smem, st>>>(a, bd);
    return cudaGetLastError();
}

#define SPARC_BAND_INST(cw, r) \
    template cudaError_t launch_col_stage_band<cw, r>(const StepArgs<float> &, const BandDev &, cudaStream_t);
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
