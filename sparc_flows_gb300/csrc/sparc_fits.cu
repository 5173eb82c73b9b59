// sparc_fits.cu -- FITS payloads encoded and decoded on the device.
//
// The reference's kernel stage reads, and its forward and adjoint runs write, one FITS file per
// field and record (the partial states, all_modules.f90:750-784, kernels.f90:221-280): big-endian
// IEEE doubles (BITPIX -64, all_modules.f90:296-378).  Converting the device's FP32 / FP64
// little-endian fields to that byte order (and back) runs here, one thread per value, so the
// host only moves finished payloads between pinned memory and the files.
#include <cstdint>
#include <string>

#include "sparc_common.cuh"
#include "sparc_gb300.h"

namespace sparc {
int report_error(int code, const std::string &msg);
}
using namespace sparc;

namespace {

constexpr int FITS_THREADS = 256;

__device__ __forceinline__ uint64_t bswap64(uint64_t v)
{
    const uint32_t lo = (uint32_t)v, hi = (uint32_t)(v >> 32);
    return ((uint64_t)__byte_perm(lo, 0, 0x0123) << 32) | (uint64_t)__byte_perm(hi, 0, 0x0123);
}
__device__ __forceinline__ uint32_t bswap32(uint32_t v) { return __byte_perm(v, 0, 0x0123); }

template <typename S>
__global__ void __launch_bounds__(FITS_THREADS) fits_encode_kernel(const S *__restrict__ src, long long n, int bitpix,
                                                                   void *__restrict__ dst)
{
    const long long stride = (long long)gridDim.x * FITS_THREADS;
    for (long long i = (long long)blockIdx.x * FITS_THREADS + threadIdx.x; i < n; i += stride) {
        if (bitpix == -64) {
            const double v = (double)src[i];
            static_cast<uint64_t *>(dst)[i] = bswap64((uint64_t)__double_as_longlong(v));
        } else {
            const float v = (float)src[i];
            static_cast<uint32_t *>(dst)[i] = bswap32(__float_as_uint(v));
        }
    }
}

template <typename D>
__global__ void __launch_bounds__(FITS_THREADS) fits_decode_kernel(const void *__restrict__ src, long long n, int bitpix,
                                                                   D *__restrict__ dst)
{
    const long long stride = (long long)gridDim.x * FITS_THREADS;
    for (long long i = (long long)blockIdx.x * FITS_THREADS + threadIdx.x; i < n; i += stride) {
        if (bitpix == -64) dst[i] = (D)__longlong_as_double((long long)bswap64(static_cast<const uint64_t *>(src)[i]));
        else dst[i] = (D)__uint_as_float(bswap32(static_cast<const uint32_t *>(src)[i]));
    }
}

unsigned fits_grid(long long n)
{
    const long long g = (n + FITS_THREADS - 1) / FITS_THREADS;
    return (unsigned)(g < 152LL * 16 ? (g > 0 ? g : 1) : 152LL * 16);
}

}  // namespace

extern "C" {

int sparc_fits_encode(const void *src, int precision, long long n, int bitpix, void *dst, void *stream)
{
    if (!src || !dst || n < 0 || (precision != 32 && precision != 64) || (bitpix != -64 && bitpix != -32))
        return report_error(SPARC_ERR_ARG, "sparc_fits_encode: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (precision == 32) fits_encode_kernel<float><<<fits_grid(n), FITS_THREADS, 0, st>>>((const float *)src, n, bitpix, dst);
    else fits_encode_kernel<double><<<fits_grid(n), FITS_THREADS, 0, st>>>((const double *)src, n, bitpix, dst);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? SPARC_OK : report_error(SPARC_ERR_CUDA, std::string("sparc_fits_encode: ") + cudaGetErrorString(e));
}

int sparc_fits_decode(const void *src, int bitpix, long long n, void *dst, int precision, void *stream)
{
    if (!src || !dst || n < 0 || (precision != 32 && precision != 64) || (bitpix != -64 && bitpix != -32))
        return report_error(SPARC_ERR_ARG, "sparc_fits_decode: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (precision == 32) fits_decode_kernel<float><<<fits_grid(n), FITS_THREADS, 0, st>>>(src, n, bitpix, (float *)dst);
    else fits_decode_kernel<double><<<fits_grid(n), FITS_THREADS, 0, st>>>(src, n, bitpix, (double *)dst);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? SPARC_OK : report_error(SPARC_ERR_CUDA, std::string("sparc_fits_decode: ") + cudaGetErrorString(e));
}

}  // extern "C"
