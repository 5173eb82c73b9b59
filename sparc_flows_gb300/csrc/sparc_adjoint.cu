// sparc_adjoint.cu -- dense column operators for the discrete adjoint of the option-17 step.
//
// Every z-operator of the step acts on each x-column separately and linearly: the compact
// derivative dbyd2 with its boundary closures (dbyd2.f:8-235) times the stretch factor
// (derivatives.f90:10-24), and FILTER_VARS_2D's z filter (physics2d.f90:509-583).  The discrete
// adjoint needs their transposes, closures included; held as dense nz x nz FP64 matrices (built
// once per plan by applying the device operator to the columns of the identity), a transpose is
// a matrix-vector product per column with the transposed matrix.  FP64 throughout.
#include <cuda_runtime.h>

#include <string>

#include "sparc_gb300.h"

namespace sparc {
int report_error(int code, const std::string &msg);
}

namespace {

constexpr int CM_X = 32;  // columns per block (one warp per output row: W[k][m] is broadcast)
constexpr int CM_Y = 8;   // output rows per block

// out[b][k][j] (+)= sum_m W[k][m] in[b][m][j] for columns i0 <= j <= i1; other columns copy in.
__global__ void __launch_bounds__(CM_X *CM_Y) colmat_kernel(const double *__restrict__ W, int nz,
                                                           const double *__restrict__ in, double *__restrict__ out,
                                                           int nx, int i0, int i1, int accumulate)
{
    const int j = blockIdx.x * CM_X + threadIdx.x;
    const int k = blockIdx.y * CM_Y + threadIdx.y;
    if (j >= nx || k >= nz) return;
    const size_t plane = (size_t)nz * nx;
    const double *ib = in + (size_t)blockIdx.z * plane;
    double v;
    if (j >= i0 && j <= i1) {
        const double *w = W + (size_t)k * nz;
        double s0 = 0.0, s1 = 0.0;
        int m = 0;
        for (; m + 1 < nz; m += 2) {
            s0 = fma(__ldg(w + m), __ldg(ib + (size_t)m * nx + j), s0);
            s1 = fma(__ldg(w + m + 1), __ldg(ib + (size_t)(m + 1) * nx + j), s1);
        }
        if (m < nz) s0 = fma(__ldg(w + m), __ldg(ib + (size_t)m * nx + j), s0);
        v = s0 + s1;
    } else {
        v = __ldg(ib + (size_t)k * nx + j);
    }
    double *o = out + (size_t)blockIdx.z * plane + (size_t)k * nx + j;
    *o = accumulate ? *o + v : v;
}

}  // namespace

extern "C" int sparc_colmat_apply(const double *W, int nz, const double *in, double *out, int nb, int nx, int i0,
                                  int i1, int accumulate, void *stream)
{
    if (!W || !in || !out || nz < 1 || nb < 1 || nx < 1 || in == out)
        return sparc::report_error(SPARC_ERR_ARG, "sparc_colmat_apply: null, empty or aliased argument");
    if (nb > 65535 || (nz + CM_Y - 1) / CM_Y > 65535)
        return sparc::report_error(SPARC_ERR_SIZE, "sparc_colmat_apply: grid too large");
    dim3 grid((nx + CM_X - 1) / CM_X, (nz + CM_Y - 1) / CM_Y, nb);
    colmat_kernel<<<grid, dim3(CM_X, CM_Y), 0, (cudaStream_t)stream>>>(W, nz, in, out, nx, i0, i1, accumulate);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? SPARC_OK
                            : sparc::report_error(SPARC_ERR_CUDA, std::string("sparc_colmat_apply: ") + cudaGetErrorString(e));
}
