// sparc_end.cu -- end of an RK step (step.f90:100-119, FILTER_VARS_2D physics2d.f90:509-556,
// records driver.f90:386-417), streamed through 32-column tiles.
//
// A block owns one (solve, component) pair -- (xi_x, v_x) or (xi_z, v_z), which are coupled
// because the RHS of xi is v -- over 32 adjacent x-columns and the full depth.  Its 16 warps take
// rows w, w + 16, ...; lane = column, so every global access of a warp is one 128-byte row
// segment.  Step 1: u_xi = xi + dt (v + bs rhs_v(s-1)) (zero on the RHS boundary rows/columns),
// u_v = v + dt rhs_v(s), into shared memory [nz][32] (no bank conflicts), together with the
// vertical-PML update of one psi component and the acceleration record.  Step 2, after one
// barrier: FILTER_VARS_2D of both fields from shared memory, the state written in place, the
// partial-state and seismogram records.  Rows are independent within a step, so each thread
// keeps several rows of loads in flight.
#include "sparc_common.cuh"

namespace sparc {

constexpr int END_CW = 32, END_WARPS = 16;

// The 11-point filter, operation order of FILTER_VARS_2D (physics2d.f90:517-522, the neighbour
// weights already halved).
template <typename T>
__device__ __forceinline__ T end_filt11(const T *B, int k, int c)
{
    const T c0 = T(0.75390625), h1 = T(0.5 * 0.41015625), h2 = T(0.5 * -0.234375), h3 = T(0.5 * 0.087890625),
            h4 = T(0.5 * -0.01953125), h5 = T(0.5 * 0.001953125);
    constexpr int W = END_CW;
    return c0 * B[k * W + c] + h1 * (B[(k - 1) * W + c] + B[(k + 1) * W + c]) +
           h2 * (B[(k - 2) * W + c] + B[(k + 2) * W + c]) + h3 * (B[(k - 3) * W + c] + B[(k + 3) * W + c]) +
           h4 * (B[(k - 4) * W + c] + B[(k + 4) * W + c]) + h5 * (B[(k - 5) * W + c] + B[(k + 5) * W + c]);
}

template <typename T>
__global__ void __launch_bounds__(END_CW *END_WARPS) end_step_stream_kernel(StepArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem_e[];
    T *Uxi = reinterpret_cast<T *>(smem_e);
    const int nz = a.nz, nx = a.nx;
    T *Uv = Uxi + (size_t)nz * END_CW;
    const int c = threadIdx.x % END_CW, w = threadIdx.x / END_CW;
    const int x = blockIdx.x * END_CW + c;
    const int p = blockIdx.y & 1, b = blockIdx.y >> 1;  // component (0: x, 1: z), solve
    const size_t F = (size_t)nz * nx;
    const int time = *a.d_time;
    const int rec = (a.steps_out > 0) ? time / a.steps_out - a.rec0 : 0;  // slot in the record window
    const bool record = a.steps_out > 0 && time % a.steps_out == 0 && rec >= 0 && rec < a.nrec_cap && time >= 0;
    T *snap = record && a.snaps ? a.snaps + ((size_t)b * a.nrec_cap + rec) * 6 * F : nullptr;
    const T *Axi = a.A + ((size_t)b * 4 + p) * F, *Av = a.A + ((size_t)b * 4 + 2 + p) * F;
    const T *R4 = svp(a, a.slot_sm1, b, p), *R5 = svp(a, a.slot_s, b, p);
    const T dt = a.dt, bs = a.bs;
    const bool xbc = (x == 0 || x == nx - 1);

    // ---- 0: psi component p of the vertical PML, pmlvars += deltat * scrpml (step.f90:112-115):
    // the thread's PML rows (w, w + 16, ... within the bottom and top layers), all loads first
    {
        constexpr int MP = 4;  // PML rows per batch and thread (the PML arrays hold both layers)
        const size_t ring = (size_t)a.slot_s * a.nb * 2 * a.nzpml * nx;
        for (int base = w; base < a.nzpml; base += MP * END_WARPS) {
            T pv[MP];
            size_t qv[MP];
            int np = 0;
#pragma unroll
            for (int i = 0; i < MP; i++) {
                const int pi = base + i * END_WARPS;
                if (pi < a.nzpml) {
                    const size_t qz = (((size_t)b * 2 + p) * a.nzpml + pi) * nx + x;
                    qv[i] = qz;
                    pv[i] = a.PZ[qz] + dt * a.SPZ[ring + qz];
                    np = i + 1;
                }
            }
#pragma unroll
            for (int i = 0; i < MP; i++)
                if (i < np) a.PZ[qv[i]] = pv[i];
        }
    }
    // ---- 1: updated fields into shared memory; acc record
#pragma unroll 4
    for (int k = w; k < nz; k += END_WARPS) {
        const size_t g = (size_t)k * nx + x;
        const T xi = __ldg(Axi + g), v = __ldg(Av + g), r4 = __ldg(R4 + g), r5 = __ldg(R5 + g);
        const T sxi = (k == 0 || xbc) ? T(0) : v + bs * r4;  // scr xi = v of stage 5, RHS zeros
        Uxi[k * END_CW + c] = xi + dt * sxi;
        Uv[k * END_CW + c] = v + dt * r5;
        if (snap) snap[(size_t)(4 + p) * F + g] = r5;
    }
    __syncthreads();
    // ---- 2: FILTER_VARS_2D, state in place, records
    const bool xf = a.filt_xall || ((x >= a.nh - 1) && (x <= nx - a.nh));
    T *Gxi = a.A + ((size_t)b * 4 + p) * F, *Gv = a.A + ((size_t)b * 4 + 2 + p) * F;
#pragma unroll 2
    for (int k = w; k < nz; k += END_WARPS) {
        const size_t g = (size_t)k * nx + x;
        T oxi = Uxi[k * END_CW + c], ov = Uv[k * END_CW + c];
        if (xf && k >= a.filt_k0 && k <= nz - 2) {
            if (k >= 5 && k <= nz - 6) {
                oxi = end_filt11(Uxi, k, c);
                ov = end_filt11(Uv, k, c);
            } else {
                oxi = T(0.5) * (Uxi[(k + 1) * END_CW + c] + Uxi[(k - 1) * END_CW + c]);
                ov = T(0.5) * (Uv[(k + 1) * END_CW + c] + Uv[(k - 1) * END_CW + c]);
            }
        }
        Gxi[g] = oxi;
        Gv[g] = ov;
        if (snap) {
            snap[(size_t)p * F + g] = oxi;
            snap[(size_t)(2 + p) * F + g] = ov;
        }
        if (record && p == 1 && k == a.k_obs && a.seis) a.seis[((size_t)b * a.nrec_cap + rec) * nx + x] = ov;
    }
}

// ---- compensated variant (FP32 plans with low parts ALO): the state is carried as hi + lo
// (~48 significant bits), a + deltat scr and FILTER_VARS_2D are evaluated in double-float
// arithmetic (Knuth's TwoSum, FMA-exact products), so the 3600-step accumulation does not round
// the state to FP32 every step.

__device__ __forceinline__ void ef_two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void ef_add(float &hi, float &lo, float bh, float bl)  // (hi, lo) += (bh, bl)
{
    float s, e;
    ef_two_sum(hi, bh, s, e);
    e += lo + bl;
    hi = s + e;
    lo = e - (hi - s);
}

// h (x + y) for double-float x, y and an exactly representable h, added to (hi, lo).
__device__ __forceinline__ void ef_axpy2(float &hi, float &lo, float h, float xh, float xl, float yh, float yl)
{
    float s, e;
    ef_two_sum(xh, yh, s, e);
    e += xl + yl;
    const float p = h * s;
    const float pe = fmaf(h, s, -p) + h * e;
    ef_add(hi, lo, p, pe);
}

// The (xi, v) pair of one component in one block (xi's update reads the old v, which the same
// block overwrites only after its barrier), 16 columns wide so that hi and lo of both fields
// ([nz][16] each) leave room for two blocks per SM; thread (c, r) = column c, rows r, r + 32, ...
constexpr int ENDC_CW = 16, ENDC_ROWS = 32;

__device__ __forceinline__ void ef_filt11c(const float *H, const float *L, int k, int c, float &hi, float &lo)
{
    constexpr int W = ENDC_CW;
    const float c0 = 0.75390625f, hs[5] = {0.205078125f, -0.1171875f, 0.0439453125f, -0.009765625f, 0.0009765625f};
    hi = c0 * H[k * W + c];
    lo = fmaf(c0, H[k * W + c], -hi) + c0 * L[k * W + c];
#pragma unroll
    for (int j = 1; j <= 5; j++)
        ef_axpy2(hi, lo, hs[j - 1], H[(k - j) * W + c], L[(k - j) * W + c], H[(k + j) * W + c], L[(k + j) * W + c]);
}

__device__ __forceinline__ void ef_out(const float *H, const float *L, int k, int c, int nz, bool filt, float &hi,
                                       float &lo)
{
    constexpr int W = ENDC_CW;
    hi = H[k * W + c];
    lo = L[k * W + c];
    if (filt) {
        if (k >= 5 && k <= nz - 6) {
            ef_filt11c(H, L, k, c, hi, lo);
        } else {
            float h = 0.f, l = 0.f;
            ef_axpy2(h, l, 0.5f, H[(k + 1) * W + c], L[(k + 1) * W + c], H[(k - 1) * W + c], L[(k - 1) * W + c]);
            hi = h;
            lo = l;
        }
    }
}

__global__ void __launch_bounds__(ENDC_CW *ENDC_ROWS) end_step_comp_kernel(StepArgs<float> a)
{
    extern __shared__ __align__(16) unsigned char smem_e[];
    const int nz = a.nz, nx = a.nx;
    float *Hxi = reinterpret_cast<float *>(smem_e), *Lxi = Hxi + (size_t)nz * ENDC_CW;
    float *Hv = Lxi + (size_t)nz * ENDC_CW, *Lv = Hv + (size_t)nz * ENDC_CW;
    const int c = threadIdx.x % ENDC_CW, r0 = threadIdx.x / ENDC_CW;
    const int x = blockIdx.x * ENDC_CW + c;
    const int p = blockIdx.y & 1, b = blockIdx.y >> 1;  // component (0: x, 1: z), solve
    const size_t F = (size_t)nz * nx;
    const int time = *a.d_time;
    const int rec = (a.steps_out > 0) ? time / a.steps_out - a.rec0 : 0;  // slot in the record window
    const bool record = a.steps_out > 0 && time % a.steps_out == 0 && rec >= 0 && rec < a.nrec_cap && time >= 0;
    float *snap = record && a.snaps ? a.snaps + ((size_t)b * a.nrec_cap + rec) * 6 * F : nullptr;
    float *Axi = a.A + ((size_t)b * 4 + p) * F, *Av = a.A + ((size_t)b * 4 + 2 + p) * F;
    float *Lxig = a.ALO + ((size_t)b * 4 + p) * F, *Lvg = a.ALO + ((size_t)b * 4 + 2 + p) * F;
    const float *R4 = svp(a, a.slot_sm1, b, p), *R5 = svp(a, a.slot_s, b, p);
    const float dt = a.dt, bs = a.bs;
    const bool xbc = (x == 0 || x == nx - 1);

#pragma unroll 2
    for (int k = r0; k < nz; k += ENDC_ROWS) {
        const size_t g = (size_t)k * nx + x;
        const float v = __ldg(Av + g), r4 = __ldg(R4 + g), r5 = __ldg(R5 + g);
        const float sxi = (k == 0 || xbc) ? 0.f : v + bs * r4;  // scr xi = v of stage 5, RHS zeros
        float hx = __ldg(Axi + g), lx = __ldg(Lxig + g), hv = v, lv = __ldg(Lvg + g);
        float d = dt * sxi;
        ef_add(hx, lx, d, fmaf(dt, sxi, -d));
        d = dt * r5;
        ef_add(hv, lv, d, fmaf(dt, r5, -d));
        Hxi[k * ENDC_CW + c] = hx;
        Lxi[k * ENDC_CW + c] = lx;
        Hv[k * ENDC_CW + c] = hv;
        Lv[k * ENDC_CW + c] = lv;
        if (snap) snap[(size_t)(4 + p) * F + g] = r5;
        const int pi = pml_row(a, k);
        if (pi >= 0) {  // pmlvars += deltat * scrpml (step.f90:112-115), component p
            const size_t qz = (((size_t)b * 2 + p) * a.nzpml + pi) * nx + x;
            a.PZ[qz] += dt * a.SPZ[(size_t)a.slot_s * a.nb * 2 * a.nzpml * nx + qz];
        }
    }
    __syncthreads();
    const bool xf = a.filt_xall || ((x >= a.nh - 1) && (x <= nx - a.nh));
    for (int k = r0; k < nz; k += ENDC_ROWS) {
        const size_t g = (size_t)k * nx + x;
        const bool filt = xf && k >= a.filt_k0 && k <= nz - 2;
        float hx, lx, hv, lv;
        ef_out(Hxi, Lxi, k, c, nz, filt, hx, lx);
        ef_out(Hv, Lv, k, c, nz, filt, hv, lv);
        Axi[g] = hx;
        Lxig[g] = lx;
        Av[g] = hv;
        Lvg[g] = lv;
        if (snap) {
            snap[(size_t)p * F + g] = hx;
            snap[(size_t)(2 + p) * F + g] = hv;
        }
        if (record && p == 1 && k == a.k_obs && a.seis) a.seis[((size_t)b * a.nrec_cap + rec) * nx + x] = hv;
    }
}

cudaError_t launch_end_step_comp(const StepArgs<float> &a, cudaStream_t st)
{
    if (a.nx % ENDC_CW || !a.ALO) return cudaErrorInvalidValue;
    const size_t smem = (size_t)4 * a.nz * ENDC_CW * sizeof(float);
    cudaError_t e =
        cudaFuncSetAttribute(end_step_comp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(a.nx / ENDC_CW, 2 * a.nb);
    end_step_comp_kernel<<<grid, ENDC_CW * ENDC_ROWS, smem, st>>>(a);
    return cudaGetLastError();
}

template <typename T>
size_t end_stream_smem_bytes(int nz)
{
    return (size_t)2 * nz * END_CW * sizeof(T);
}

template <typename T>
cudaError_t launch_end_step_stream(const StepArgs<T> &a, cudaStream_t st)
{
    if (a.nx % END_CW || a.ALO) return cudaErrorInvalidValue;
    const size_t smem = end_stream_smem_bytes<T>(a.nz);
    cudaError_t e = cudaFuncSetAttribute(end_step_stream_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(a.nx / END_CW, 2 * a.nb);
    end_step_stream_kernel<T><<<grid, END_CW * END_WARPS, smem, st>>>(a);
    return cudaGetLastError();
}

template size_t end_stream_smem_bytes<float>(int);
template size_t end_stream_smem_bytes<double>(int);
template cudaError_t launch_end_step_stream<float>(const StepArgs<float> &, cudaStream_t);
template cudaError_t launch_end_step_stream<double>(const StepArgs<double> &, cudaStream_t);

}  // namespace sparc
