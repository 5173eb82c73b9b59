// sparc_fft512.cuh -- register-resident spectral derivative of 512-point complex rows, one warp
// per row (FP32 row passes of 512-column grids).
//
// n = n1 + 32 n2 (n1 = lane, n2 = register), k = k2 + 16 k1:
//   X[k2 + 16 k1] = sum_{n1} W32^{n1 k1} W512^{n1 k2} sum_{n2} W16^{n2 k2} x[n1 + 32 n2].
// Each lane does a 16-point DFT of its registers, multiplies by W512^{n1 k2}, and one padded
// shared-memory transpose gives lane pair (2 q, 2 q + 1) the even / odd n1 entries of column
// k2 = q; a 16-point DFT in each lane and one radix-2 exchange with the partner (shuffles)
// complete the 32-point DFT over n1.  Lane (q, e) then holds X[q + 16 j + 256 e], j = 0..15.
// After the multiplication by i kap[k] the inverse runs the same steps backwards and leaves
// the derivative in the input layout (register n2 <-> column lane + 32 n2).  Per transform one
// transpose (16 x 34-word rows: conflict-free both ways) instead of three Stockham passes.
#pragma once
#include "sparc_common.cuh"

namespace sparc {

// cos(2 pi j / 32), j = 0..8 (quarter wave)
__host__ __device__ constexpr double q32(int j)
{
    constexpr double c[9] = {1.0,
                             0.98078528040323044912618223613424,
                             0.92387953251128675612818318939679,
                             0.83146961230254523707878837761791,
                             0.70710678118654752440084436210485,
                             0.55557023301960222474283081394853,
                             0.38268343236508977172845998403040,
                             0.19509032201612826784828486847702,
                             0.0};
    return c[j];
}
// cos / sin of 2 pi j / 32 for j = 0..31
__host__ __device__ constexpr double c32(int j)
{
    j &= 31;
    return j <= 8 ? q32(j) : j <= 16 ? -q32(16 - j) : j <= 24 ? -q32(j - 16) : q32(32 - j);
}
__host__ __device__ constexpr double s32(int j) { return c32(j - 8); }

// In-register 16-point DFT (forward: W = exp(-2 pi i / 16); inverse: conjugate), natural order.
template <bool INV>
__device__ __forceinline__ void dft16(float (&re)[16], float (&im)[16])
{
    float ur[16], ui[16];
#pragma unroll
    for (int b = 0; b < 4; b++) {
        float xr[4] = {re[b], re[4 + b], re[8 + b], re[12 + b]};
        float xi[4] = {im[b], im[4 + b], im[8 + b], im[12 + b]};
        butterfly<float, 4>(xr, xi, INV);
#pragma unroll
        for (int kp = 0; kp < 4; kp++) {
            const float wr = (float)c32(2 * b * kp), wi = INV ? (float)s32(2 * b * kp) : -(float)s32(2 * b * kp);
            if (b * kp == 0) {
                ur[b * 4 + kp] = xr[kp];
                ui[b * 4 + kp] = xi[kp];
            } else {
                ur[b * 4 + kp] = xr[kp] * wr - xi[kp] * wi;
                ui[b * 4 + kp] = xr[kp] * wi + xi[kp] * wr;
            }
        }
    }
#pragma unroll
    for (int kp = 0; kp < 4; kp++) {
        float yr[4] = {ur[kp], ur[4 + kp], ur[8 + kp], ur[12 + kp]};
        float yi[4] = {ui[kp], ui[4 + kp], ui[8 + kp], ui[12 + kp]};
        butterfly<float, 4>(yr, yi, INV);
#pragma unroll
        for (int kk = 0; kk < 4; kk++) {
            re[kp + 4 * kk] = yr[kk];
            im[kp + 4 * kk] = yi[kk];
        }
    }
}

constexpr int FFT512_LD = 34;                    // padded row of the transpose buffer
constexpr int FFT512_SCRATCH = 2 * 16 * FFT512_LD;  // floats per warp

// Derivative of the complex row held as (re[n2], im[n2]) = x[lane + 32 n2] (inputs scaled by
// sr, si first); result in place, same layout.  twr/twi: W512^t; kap: i-multiplier with the
// 1/512 normalisation and the zero Nyquist bin; S: FFT512_SCRATCH floats of warp scratch.
__device__ __forceinline__ void fft512_deriv(float (&re)[16], float (&im)[16], float *S, const float *__restrict__ twr,
                                             const float *__restrict__ twi, const float *__restrict__ kap,
                                             float scale, int lane, float sr, float si)
{
    float *Sr = S, *Si = S + 16 * FFT512_LD;
    const int q = lane >> 1, e = lane & 1;
#pragma unroll
    for (int n2 = 0; n2 < 16; n2++) {
        re[n2] *= sr;
        im[n2] *= si;
    }
    // ---- forward
    dft16<false>(re, im);
#pragma unroll
    for (int k2 = 1; k2 < 16; k2++) {
        const int t = lane * k2;  // < 512
        const float wr = __ldg(twr + t), wi = __ldg(twi + t);
        const float a = re[k2], b = im[k2];
        re[k2] = a * wr - b * wi;
        im[k2] = a * wi + b * wr;
    }
    __syncwarp();
#pragma unroll
    for (int k2 = 0; k2 < 16; k2++) {
        Sr[k2 * FFT512_LD + lane] = re[k2];
        Si[k2 * FFT512_LD + lane] = im[k2];
    }
    __syncwarp();
#pragma unroll
    for (int m = 0; m < 16; m++) {
        re[m] = Sr[q * FFT512_LD + 2 * m + e];
        im[m] = Si[q * FFT512_LD + 2 * m + e];
    }
    dft16<false>(re, im);
    if (e) {  // odd half times W32^j
#pragma unroll
        for (int j = 1; j < 16; j++) {
            const float wr = (float)c32(j), wi = -(float)s32(j);
            const float a = re[j], b = im[j];
            re[j] = a * wr - b * wi;
            im[j] = a * wi + b * wr;
        }
    }
#pragma unroll
    for (int j = 0; j < 16; j++) {  // lane e = 0: E + O W; lane e = 1: E - O W
        const float pr = __shfl_xor_sync(0xffffffffu, re[j], 1), pi = __shfl_xor_sync(0xffffffffu, im[j], 1);
        re[j] = e ? pr - re[j] : re[j] + pr;
        im[j] = e ? pi - im[j] : im[j] + pi;
    }
    // ---- times i kap[k] scale, k = q + 16 j + 256 e
#pragma unroll
    for (int j = 0; j < 16; j++) {
        const float kk = __ldg(kap + q + 16 * j + 256 * e) * scale;
        const float a = re[j], b = im[j];
        re[j] = -kk * b;
        im[j] = kk * a;
    }
    // ---- inverse
#pragma unroll
    for (int j = 0; j < 16; j++) {  // lane e = 0: lo + hi; lane e = 1: (lo - hi) W32^-j
        const float pr = __shfl_xor_sync(0xffffffffu, re[j], 1), pi = __shfl_xor_sync(0xffffffffu, im[j], 1);
        re[j] = e ? pr - re[j] : re[j] + pr;
        im[j] = e ? pi - im[j] : im[j] + pi;
    }
    if (e) {
#pragma unroll
        for (int j = 1; j < 16; j++) {
            const float wr = (float)c32(j), wi = (float)s32(j);
            const float a = re[j], b = im[j];
            re[j] = a * wr - b * wi;
            im[j] = a * wi + b * wr;
        }
    }
    dft16<true>(re, im);
    __syncwarp();
#pragma unroll
    for (int m = 0; m < 16; m++) {
        Sr[q * FFT512_LD + 2 * m + e] = re[m];
        Si[q * FFT512_LD + 2 * m + e] = im[m];
    }
    __syncwarp();
#pragma unroll
    for (int k2 = 0; k2 < 16; k2++) {
        re[k2] = Sr[k2 * FFT512_LD + lane];
        im[k2] = Si[k2 * FFT512_LD + lane];
    }
#pragma unroll
    for (int k2 = 1; k2 < 16; k2++) {
        const int t = lane * k2;
        const float wr = __ldg(twr + t), wi = -__ldg(twi + t);
        const float a = re[k2], b = im[k2];
        re[k2] = a * wr - b * wi;
        im[k2] = a * wi + b * wr;
    }
    dft16<true>(re, im);
}

}  // namespace sparc
