// sparc_noalloc.cu -- kernel-integral accumulation that allocates no device memory.
//
// sparc_kernels_accumulate needs a work buffer for the x-derivatives of one record pair
// (nbatch x 4 fields x nz x nx of the plan precision) and allocates it with cudaMalloc on
// first use.  Some callers cannot allow that: an embedding host whose allocator owns every
// device allocation, or a run whose device-memory budget is fixed before it starts, must not
// see the library call cudaMalloc in the middle of a run.  sparc_kernels_accumulate_static serves them: its scratch is the
// file-scope device array below, fixed in size and held by every GPU that loads the library
// until the process exits.
#include <cstdio>
#include <mutex>
#include <string>

#include "sparc_common.cuh"
#include "sparc_gb300.h"

namespace sparc {

// 8 MiB: one solve of up to nz*nx = 524,288 points in FP32 (262,144 in FP64), or a batch
// whose nbatch*4*nz*nx values fit.
constexpr size_t STATIC_SCRATCH_BYTES = size_t(8) << 20;
static __device__ __align__(256) unsigned char g_static_scratch[STATIC_SCRATCH_BYTES];

namespace {
constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
void *g_scratch_addr[MAX_DEVICES] = {};

// Device address of g_static_scratch on the current device (looked up once per device index
// and kept for the life of the process: a context reset after the first call is unsupported).
cudaError_t scratch_address(void **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}
}  // namespace

// Accumulates one record pair through the same kernels as sparc_kernels_accumulate, with the
// work buffer placed in the static array.
template <typename T>
int kernels_accumulate_static_impl(const KAccArgs<T> &proto, cudaStream_t st, std::string &err)
{
    const size_t need = (size_t)proto.nb * 4 * proto.nz * proto.nx * sizeof(T);
    if (need > STATIC_SCRATCH_BYTES) {
        err = "sparc_kernels_accumulate_static: nbatch*4*nz*nx*sizeof(T) = " + std::to_string(need) +
              " bytes exceeds the 8 MiB static scratch";
        return SPARC_ERR_SIZE;
    }
    void *scratch = nullptr;
    cudaError_t e = scratch_address(&scratch);
    if (e != cudaSuccess) {
        err = std::string("sparc_kernels_accumulate_static: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
        return SPARC_ERR_CUDA;
    }
    KAccArgs<T> k = proto;
    k.work = (T *)scratch;  // fully written by the row pass before the column pass reads it
    e = launch_kacc<T>(k, st);
    if (e != cudaSuccess) {
        err = std::string("sparc_kernels_accumulate_static: ") + cudaGetErrorString(e);
        return SPARC_ERR_CUDA;
    }
    return SPARC_OK;
}

template int kernels_accumulate_static_impl<float>(const KAccArgs<float> &, cudaStream_t, std::string &);
template int kernels_accumulate_static_impl<double>(const KAccArgs<double> &, cudaStream_t, std::string &);

}  // namespace sparc
