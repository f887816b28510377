/* The runner's verification step on the device (HPC-Dwarfs/RabbitCT
 * src/rabbitRunner.c:320-384): every voxel is converted to Hounsfield units,
 * HU = floor(hus0 * v + hus1 + 0.5) for v > 0 else 0, clamped to 4095, and
 * compared with a uint16 reference volume: mean squared error, maximum
 * absolute error, PSNR = 10 log10(4095^2 / MSE) and an 11-bin histogram of
 * |error| (bins 0-1, ..., 9-10, >= 10).  With convertInPlace the HU values
 * replace the volume, as the runner does before writing -o.  Avoids copying a
 * 4 GiB volume to the host just to check it.
 *
 * One grid-stride pass: per-thread FP64 partial sums, block reduction in
 * shared memory, one FP64 atomic per block; the maximum through an integer
 * atomicMax on the (non-negative) float's bits; histogram per block in shared
 * memory.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <cuda_runtime.h>

#include "lolaCuda.h"
#include "lolacuda_internal.h"

namespace {

struct VerifyOut {
  double sumSq;
  unsigned int maxAbsBits;
  unsigned int pad;
  unsigned long long hist[11];
};

__global__ void __launch_bounds__(256) verifyKernel(float *vol, const uint16_t *ref, size_t n,
    float s0, float s1, int convert, VerifyOut *out)
{
  __shared__ double partial[256];
  __shared__ unsigned int hist[11];
  if (threadIdx.x < 11)
    hist[threadIdx.x] = 0;
  __syncthreads();
  double acc = 0.0;
  float mx = 0.0f;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float v = vol[i];
    /* US_ROUND(hus0 * v + hus1) with a rounding after each operation */
    float hu = (v > 0.0f) ? floorf(__fadd_rn(__fadd_rn(__fmul_rn(s0, v), s1), 0.5f)) : 0.0f;
    if (hu > 4095.0f)
      hu = 4095.0f;
    const float err = hu - (float)ref[i];
    const float a = fabsf(err);
    acc += (double)(err * err);
    mx = fmaxf(mx, a);
    unsigned int bin = (unsigned int)floorf(a);
    if (bin > 10u)
      bin = 10u;
    atomicAdd(&hist[bin], 1u);
    if (convert)
      vol[i] = hu;
  }
  partial[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      partial[threadIdx.x] += partial[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    atomicAdd(&out->sumSq, partial[0]);
  atomicMax(&out->maxAbsBits, __float_as_uint(mx));
  if (threadIdx.x < 11 && hist[threadIdx.x])
    atomicAdd(&out->hist[threadIdx.x], (unsigned long long)hist[threadIdx.x]);
}

} /* namespace */

extern "C" int lolaCudaVerifyVolume(float *d_volume, size_t voxels, const uint16_t *h_reference,
    const float *hus, int convertInPlace, void *stream, LolaCudaQuality *q)
{
  if (d_volume == nullptr || h_reference == nullptr || hus == nullptr || q == nullptr)
    return lolaSetError("verify: null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  uint16_t *d_ref = nullptr;
  VerifyOut *d_out = nullptr;
  VerifyOut h;
  cudaError_t e = cudaMalloc(&d_ref, voxels * sizeof(uint16_t));
  if (e == cudaSuccess)
    e = cudaMalloc(&d_out, sizeof(VerifyOut));
  if (e == cudaSuccess)
    e = cudaMemsetAsync(d_out, 0, sizeof(VerifyOut), st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_ref, h_reference, voxels * sizeof(uint16_t), cudaMemcpyHostToDevice,
        st);
  if (e == cudaSuccess) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    (void)cudaGetLastError();  /* report this launch's error, not an earlier one */
    verifyKernel<<<sms * 8, 256, 0, st>>>(d_volume, d_ref, voxels, hus[0], hus[1],
        convertInPlace, d_out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&h, d_out, sizeof(VerifyOut), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(st);
  cudaFree(d_ref);
  cudaFree(d_out);
  if (e != cudaSuccess)
    return lolaSetError("verify: %s", cudaGetErrorString(e));
  q->mse = h.sumSq / (double)voxels;
  q->rmse = sqrt(q->mse);
  float mx;
  memcpy(&mx, &h.maxAbsBits, sizeof(mx));
  q->maxAbs = (double)mx;
  q->psnr = q->mse > 1e-8 ? 10.0 * log10(4095.0 * 4095.0 / q->mse) : INFINITY;
  for (int i = 0; i < 11; ++i)
    q->histogram[i] = h.hist[i];
  return 1;
}

extern "C" int lolaCudaPlanVerify(LolaCudaPlan *plan, const uint16_t *h_reference,
    const float *hus, int convertInPlace, LolaCudaQuality *q)
{
  if (plan == nullptr)
    return lolaSetError("verify: null plan");
  if (!lolaCudaPlanSynchronize(plan))
    return 0;
  const size_t n = lolaPlanVoxels(plan);
  return lolaCudaVerifyVolume(lolaCudaPlanVolume(plan), n, h_reference, hus, convertInPlace,
      lolaCudaPlanStream(plan), q);
}
