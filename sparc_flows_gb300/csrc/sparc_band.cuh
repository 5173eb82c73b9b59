// sparc_band.cuh -- geometric-band evaluation of the compact z-derivative (FP32 column passes).
//
//   x[k] = t0 (rhs[k] + sum_{d>=1} r^d (rhs[k-d] + rhs[k+d])) + rank-2 corner corrections,
// the inverse of the infinite Toeplitz operator (1/3, 1, 1/3) (r = -0.382) plus the exact
// correction near both ends (BandDev); rhs is formed exactly as dbyd2 forms it (dbyd2.f:8-235).
// Thread group g (CW threads, one per column) holds rows [g R, g R + R) of a column block in
// shared memory ([k][CW] layout).  The two geometric sums are running sums over the group's
// own rows, L[m+1] = r (rhs[m] + L[m]) and U[m-1] = r (rhs[m] + U[m]) (stable: |r| < 1), seeded
// by carries of the three neighbouring groups on each side, exchanged through shared memory
// (terms beyond three groups are below r^27 = 5e-12).
#pragma once
#include "sparc_common.cuh"

namespace sparc {

template <int CW>
constexpr int band_maxg() { return CW == 32 ? 32 : 28; }  // thread groups per block
template <int CW>
constexpr int band_minb() { return CW == 32 ? 1 : (CW == 16 ? 2 : 4); }  // resident blocks per SM
template <int R>
constexpr int band_gb() { return (BAND_KC + R - 1) / R; }  // groups that can touch the bottom corner
template <int R>
constexpr int band_gt() { return (BAND_KC + R - 1) / R + 1; }  // ... the top corner

// Shared carries of one derivative: CL, CU [G][CW], corner partial products PB [GB][Q][CW],
// PT [GT][Q][CW], and the top-block Thomas workspace YT [GT][KC][CW].
template <int CW, int R>
struct BandCarry {
    float *CL, *CU, *PB, *PT;
    float *YT;  // top-block Thomas workspace [GT][KC][CW] (each thread its own column)
    __device__ BandCarry(float *base, int G)
    {
        CL = base;
        CU = CL + G * CW;
        PB = CU + G * CW;
        PT = PB + band_gb<R>() * BAND_Q * CW;
        YT = PT + band_gt<R>() * BAND_Q * CW;
    }
    static __host__ __device__ constexpr int floats_fixed()
    {
        return (band_gb<R>() + band_gt<R>()) * BAND_Q * CW + band_gt<R>() * BAND_KC * CW;
    }
};

// Right-hand sides of dbyd2 for the rows [k0, k0 + n) of field column Fc (rows beyond n: 0),
// also stored to the column Rc for band_eval.
template <int CW, int R>
__device__ __forceinline__ void band_rhs(const ZTab<float> &tb, const float *Fc, float *Rc, int c, int k0, int n,
                                         int nz, float preset, float (&rhs)[R])
{
    float w[R + 4];  // rows k0-2 .. k0+R+1
    if (k0 >= 2 && k0 + R + 2 <= nz) {  // every row of the group interior (uniform over the group)
#pragma unroll
        for (int i = 0; i < R + 4; i++) w[i] = Fc[(k0 - 2 + i) * CW + c];
#pragma unroll
        for (int m = 0; m < R; m++) {
            const float v = tb.c1 * (w[m + 3] - w[m + 1]) + tb.c2 * (w[m + 4] - w[m]);
            Rc[(k0 + m) * CW + c] = v;
            rhs[m] = v;
        }
        return;
    }
#pragma unroll
    for (int i = 0; i < R + 4; i++) {
        const int k = k0 - 2 + i;
        w[i] = (k >= 0 && k < nz) ? Fc[k * CW + c] : 0.f;
    }
#pragma unroll
    for (int m = 0; m < R; m++) {
        const int k = k0 + m;
        float v = 0.f;
        if (m < n) {
            if (k >= 2 && k <= nz - 3)
                v = tb.c1 * (w[m + 3] - w[m + 1]) + tb.c2 * (w[m + 4] - w[m]);
            else
                v = zrhs(tb, Fc, CW, c, k, nz, preset);  // boundary closures, caller-set row
            Rc[k * CW + c] = v;
        }
        rhs[m] = v;
    }
}

// Carries of the group's right-hand sides and its partial products with the corner factors
// (TOPC: also the top corner's; not needed where the top block is solved directly, ibc 1 and 2).
template <int CW, int R, bool TOPC = true>
__device__ __forceinline__ void band_publish(const BandDev &bd, const float *__restrict__ uv, const BandCarry<CW, R> &cb,
                                             int c, int g, int k0, int n, int nz, const float (&rhs)[R])
{
    constexpr int KC = BAND_KC, Q = BAND_Q;
    const float r = bd.r;
    float cl = 0.f, cu = 0.f;
#pragma unroll
    for (int m = 0; m < R; m++)
        if (m < n) cl = r * (cl + rhs[m]);
#pragma unroll
    for (int m = R - 1; m >= 0; m--)
        if (m < n) cu = r * (cu + rhs[m]);
    cb.CL[g * CW + c] = cl;
    cb.CU[g * CW + c] = cu;
    if (k0 < KC) {
        const float *Vb = uv + KC * Q;
#pragma unroll
        for (int q = 0; q < Q; q++) {
            float p = 0.f;
#pragma unroll
            for (int m = 0; m < R; m++)
                if (m < n && k0 + m < KC) p = fmaf(__ldg(Vb + q * KC + k0 + m), rhs[m], p);
            cb.PB[(g * Q + q) * CW + c] = p;
        }
    }
    const int o = nz - KC, gt0 = o / R;
    if (TOPC && g >= gt0) {
        const float *Vt = uv + 3 * KC * Q;
#pragma unroll
        for (int q = 0; q < Q; q++) {
            float p = 0.f;
#pragma unroll
            for (int m = 0; m < R; m++)
                if (m < n && k0 + m >= o) p = fmaf(__ldg(Vt + q * KC + (k0 + m - o)), rhs[m], p);
            cb.PT[((g - gt0) * Q + q) * CW + c] = p;
        }
    }
}

// Top block of one column by the direct tridiagonal solve (for ibc 1 and 2 the boundary row of
// T is not diagonally dominant and T^{-1} reaches 19 there, which a product with T^{-1} carries
// into FP32 rounding): x at row o-1 (outside the corner block) from the band sums over 27 rows
// on either side, then the Thomas sweeps over rows o .. nz-1 into y[0 .. KC) (stride CW).  Rc
// and y never overlap (right-hand-side tile, workspace): with the restrict qualifiers the loads
// of Rc are issued ahead of the stores to y instead of waiting behind each of them on the
// sweep's dependency chain.
template <int CW, int THT>
__device__ __forceinline__ void band_thomas(const BandDev &bd, const float *__restrict__ Rc, float *__restrict__ y,
                                            int c, int nz)
{
    constexpr int KC = BAND_KC;
    const int o = nz - KC;
    const float *th = bd.th[THT];
    const int m0 = o - 1;
    float lo = 0.f, up = 0.f;
#pragma unroll
    for (int d = 27; d >= 1; d--)
        if (m0 - d >= 0) lo = fmaf(bd.rpow[d], Rc[(m0 - d) * CW + c], lo);
#pragma unroll
    for (int d = KC; d >= 1; d--) up = fmaf(bd.rpow[d], Rc[(m0 + d) * CW + c], up);
    const float xm0 = bd.t0 * (Rc[m0 * CW + c] + lo + up);
    float prev = 0.f;
#pragma unroll
    for (int m = 0; m < KC; m++) {
        float v = Rc[(o + m) * CW + c];
        if (m == 0) v = fmaf(-th[3 * KC], xm0, v);
        v = v * th[m];
        if (m > 0) v = fmaf(-th[KC + m], prev, v);
        y[m * CW] = v;
        prev = v;
    }
#pragma unroll
    for (int m = KC - 2; m >= 0; m--) {
        prev = fmaf(-th[2 * KC + m + 1], prev, y[m * CW]);
        y[m * CW] = prev;
    }
}

// x[m] = (T^{-1} rhs)[k0 + m] for m < n, from the group's own right-hand sides (column Rc) and
// the carries.  THT = 0, 1: the top block by the direct solve with the Thomas factors of ibc 1, 2
// (-1: by the corner factors).
template <int CW, int R, int THT = -1>
__device__ __forceinline__ void band_eval(const BandDev &bd, const float *__restrict__ uv, const BandCarry<CW, R> &cb,
                                          int c, int g, int G, int k0, int n, int nz, const float *Rc, float (&x)[R])
{
    constexpr int KC = BAND_KC, Q = BAND_Q;
    float rhs[R];
#pragma unroll
    for (int m = 0; m < R; m++) rhs[m] = (m < n) ? Rc[(k0 + m) * CW + c] : 0.f;
    const float r = bd.r, rR = bd.rpow[R], r2R = bd.rpow[2 * R];
    float l = 0.f, u = 0.f;  // sum_{d>=1} r^d rhs below the first row / above the last row
    if (g >= 1) l = cb.CL[(g - 1) * CW + c];
    if (g >= 2) l = fmaf(rR, cb.CL[(g - 2) * CW + c], l);
    if (g >= 3) l = fmaf(r2R, cb.CL[(g - 3) * CW + c], l);
    if (g + 1 < G) u = cb.CU[(g + 1) * CW + c];
    if (g + 2 < G) u = fmaf(rR, cb.CU[(g + 2) * CW + c], u);
    if (g + 3 < G) u = fmaf(r2R, cb.CU[(g + 3) * CW + c], u);
#pragma unroll
    for (int m = R - 1; m >= 0; m--) {
        if (m < n) {
            x[m] = rhs[m] + u;
            u = r * (rhs[m] + u);
        } else {
            x[m] = 0.f;
        }
    }
#pragma unroll
    for (int m = 0; m < R; m++) {
        x[m] = bd.t0 * (x[m] + l);
        l = r * (rhs[m] + l);
    }
    if (k0 < KC) {
        float s[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) {
            s[q] = 0.f;
#pragma unroll
            for (int gg = 0; gg < band_gb<R>(); gg++)
                if (gg * R < KC) s[q] += cb.PB[(gg * Q + q) * CW + c];
        }
        const float *Ub = uv;
#pragma unroll
        for (int m = 0; m < R; m++) {
            const int k = k0 + m;
            if (m < n && k < KC)
#pragma unroll
                for (int q = 0; q < Q; q++) x[m] = fmaf(__ldg(Ub + k * Q + q), s[q], x[m]);
        }
    }
    const int o = nz - KC, gt0 = o / R;
    if (THT >= 0 && k0 + n > o) {
        float *y = cb.YT + (size_t)(g - gt0) * KC * CW + c;  // this group's column of the scratch
        band_thomas<CW, THT < 0 ? 0 : THT>(bd, Rc, y, c, nz);
#pragma unroll
        for (int r = 0; r < R; r++)
            if (r < n && k0 + r >= o) x[r] = y[(k0 + r - o) * CW];
    } else if (k0 + n > o) {
        float s[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) {
            s[q] = 0.f;
            for (int gg = gt0; gg < G; gg++) s[q] += cb.PT[((gg - gt0) * Q + q) * CW + c];
        }
        const float *Ut = uv + 2 * KC * Q;
#pragma unroll
        for (int m = 0; m < R; m++) {
            const int k = k0 + m - o;
            if (m < n && k >= 0)
#pragma unroll
                for (int q = 0; q < Q; q++) x[m] = fmaf(__ldg(Ut + k * Q + q), s[q], x[m]);
        }
    }
}

}  // namespace sparc
