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
    const int rec = (a.steps_out > 0) ? time / a.steps_out : 0;
    const bool record = a.steps_out > 0 && time % a.steps_out == 0 && rec < a.nrec_cap && time >= 0;
    T *snap = record && a.snaps ? a.snaps + ((size_t)b * a.nrec_cap + rec) * 6 * F : nullptr;
    const T *Axi = a.A + ((size_t)b * 4 + p) * F, *Av = a.A + ((size_t)b * 4 + 2 + p) * F;
    const T *R4 = svp(a, a.slot_sm1, b, p), *R5 = svp(a, a.slot_s, b, p);
    const T dt = a.dt, bs = a.bs;
    const bool xbc = (x == 0 || x == nx - 1);

    // ---- 1: updated fields into shared memory; psi component p of the vertical PML; acc record
#pragma unroll 4
    for (int k = w; k < nz; k += END_WARPS) {
        const size_t g = (size_t)k * nx + x;
        const T xi = __ldg(Axi + g), v = __ldg(Av + g), r4 = __ldg(R4 + g), r5 = __ldg(R5 + g);
        const T sxi = (k == 0 || xbc) ? T(0) : v + bs * r4;  // scr xi = v of stage 5, RHS zeros
        Uxi[k * END_CW + c] = xi + dt * sxi;
        Uv[k * END_CW + c] = v + dt * r5;
        if (snap) snap[(size_t)(4 + p) * F + g] = r5;
        const int pi = pml_row(a, k);
        if (pi >= 0) {  // pmlvars += deltat * scrpml (step.f90:112-115)
            const size_t qz = (((size_t)b * 2 + p) * a.nzpml + pi) * nx + x;
            a.PZ[qz] += dt * a.SPZ[(size_t)a.slot_s * a.nb * 2 * a.nzpml * nx + qz];
        }
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
