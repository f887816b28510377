/* Roofline probes: the two throughputs that bound the backprojection pass.
 *
 *  issue   independent FP32 FMA chains, the SM's FP32 instruction issue rate
 *          (thread-instructions / s).  The pass kernel is a chain of FP32 and
 *          integer ops per voxel update, so issue rate / (instructions per
 *          update) bounds its update rate.
 *  gather  the pass kernel's local 2D gather pattern with trivial arithmetic:
 *          each warp reads, for 32 lanes at detector columns spaced 1.25 px
 *          apart, the 2x2 taps of a stored projection, in the kernel's storage
 *          layouts (4 x 4 B, 4 x 2 B, 1 x 16 B or 1 x 8 B per update, or one
 *          texel fetch).  Each thread issues four independent fetches per
 *          step, two detector rows apart (as a thread's voxels along z
 *          project), so the rate is that of the pipes and not of one fetch's
 *          latency.  Returns updates / s the gather path alone sustains:
 *          lolaCudaProbeGatherRate at random positions of a full-size,
 *          L2-resident projection (no reuse in L1), lolaCudaProbeGatherPeak
 *          inside a small image that every SM keeps in L1 — the rate of the
 *          gather pipes themselves for this lane spacing.
 *  texture rows  8-lane texture requests whose texels lie in 1, 2, 4 or 8
 *          detector rows (lolaCudaProbeTextureRows): the texture data stage
 *          takes one wavefront per row a request touches, which is why the
 *          pass kernel gives each warp quarter a compact 4 x 2 voxel patch.
 * They run on every SM with enough warps to saturate it and are timed with
 * CUDA events on the default stream.
 */
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "lolaCuda.h"
#include "lolacuda_internal.h"

namespace {

__global__ void __launch_bounds__(256) issueProbe(float *out, int iters, float a, float b)
{
  float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f;
  float x4 = x0 + 4.f, x5 = x0 + 5.f, x6 = x0 + 6.f, x7 = x0 + 7.f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      x0 = fmaf(x0, a, b);
      x1 = fmaf(x1, a, b);
      x2 = fmaf(x2, a, b);
      x3 = fmaf(x3, a, b);
      x4 = fmaf(x4, a, b);
      x5 = fmaf(x5, a, b);
      x6 = fmaf(x6, a, b);
      x7 = fmaf(x7, a, b);
    }
  }
  const float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 1234.5f)
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

/* kind: 0 = 4 x FP32 taps, 1 = 4 x 16-bit taps, 2 = 1 x 16 B quad, 3 = 1 x 8 B quad,
 * 4 = one 4-texel texture gather (tld4), 5 = one point fetch of an RGBA texel,
 * 6 = one fetch of an RGBA texel by integer index from a linear texture */
template <int KIND>
__global__ void __launch_bounds__(256) gatherProbe(const void *img, int pitch, int rows,
    int iters, float *out, cudaTextureObject_t tex)
{
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  /* bases in the first (pitch - 64) x (rows - 8) pixels: the lanes' columns
     (up to 38 px right) and the four fetches' rows (up to 7 rows down, with
     the lower taps) stay inside the image */
  const uint32_t span = (uint32_t)(pitch - 64) * (uint32_t)(rows - 8);
  uint32_t state = 2654435761u * (uint32_t)(warp + 1);
  float acc = 0.0f;
  for (int i = 0; i < iters; ++i) {
    state = state * 1664525u + 1013904223u;
    const uint32_t base = (state >> 8) % span + ((uint32_t)lane * 5u >> 2);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const uint32_t idx = base + (uint32_t)(2 * r * pitch);
      if (KIND == 0) {
        const float *f = static_cast<const float *>(img) + idx;
        acc += __ldg(f) + __ldg(f + 1) + __ldg(f + pitch) + __ldg(f + pitch + 1);
      } else if (KIND == 1) {
        const unsigned short *h = static_cast<const unsigned short *>(img) + idx;
        acc += __uint_as_float(((uint32_t)__ldg(h) << 16) | __ldg(h + 1)) +
               __uint_as_float(((uint32_t)__ldg(h + pitch) << 16) | __ldg(h + pitch + 1));
      } else if (KIND == 2) {
        const float4 q = __ldg(static_cast<const float4 *>(img) + idx);
        acc += (q.x + q.y) + (q.z + q.w);
      } else if (KIND == 3) {
        const uint2 q = __ldg(static_cast<const uint2 *>(img) + idx);
        acc += __uint_as_float(q.x) + __uint_as_float(q.y);
      } else if (KIND == 4) {
        const float cx = (float)(idx % (uint32_t)pitch) + 1.0f;
        const float cy = (float)(idx / (uint32_t)pitch) + 1.0f;
        const float4 g = tex2Dgather<float4>(tex, cx, cy, 0);
        acc += (g.x + g.y) + (g.z + g.w);
      } else if (KIND == 5) {
        const float cx = (float)(idx % (uint32_t)pitch) + 0.5f;
        const float cy = (float)(idx / (uint32_t)pitch) + 0.5f;
        const float4 g = tex2D<float4>(tex, cx, cy);
        acc += (g.x + g.y) + (g.z + g.w);
      } else {
        const float4 g = tex1Dfetch<float4>(tex, (int)idx);
        acc += (g.x + g.y) + (g.z + g.w);
      }
    }
  }
  if (acc == 1234.5f)
    out[0] = acc;
}

/* 8-lane texture requests whose eight texels lie in `rows` detector rows
 * (1, 2, 4 or 8): lanes 1.25 px apart within a row, each 8-lane quarter of
 * the warp 10 px right of the previous one, four independent fetches per
 * step (8 rows apart), in an L1-resident RGBA16F linear texture of
 * 128 x 48 texels. */
__global__ void __launch_bounds__(256) textureRowsProbe(int rows, int iters, float *out,
    cudaTextureObject_t tex)
{
  const int lane = threadIdx.x & 31, q = lane >> 3, j = lane & 7;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int perRow = 8 / rows;
  uint32_t state = 2654435761u * (uint32_t)(warp + 1);
  float acc = 0.0f;
  for (int i = 0; i < iters; ++i) {
    state = state * 1664525u + 1013904223u;
    const int bc = (int)((state >> 8) & 31u), br = (int)((state >> 16) & 7u);
    /* columns <= 31 + 30 + 8, rows <= 7 + 7 + 24: inside the 128 x 48 image */
    const int col = bc + q * 10 + ((j % perRow) * 5) / 4;
    const int row = br + j / perRow;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const float4 g = tex1Dfetch<float4>(tex, (row + 8 * r) * 128 + col);
      acc += (g.x + g.y) + (g.z + g.w);
    }
  }
  if (acc == 1234.5f)
    out[0] = acc;
}

int smCount()
{
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

} /* namespace */

/* Thread-level FP32 FMA instructions per second. */
extern "C" double lolaCudaProbeIssueRate(void)
{
  const int sms = smCount();
  const int blocks = sms * 8, threads = 256, iters = 4096;
  float *out = nullptr;
  if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(float)) != cudaSuccess)
    return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  issueProbe<<<blocks, threads>>>(out, 64, 0.999f, 1e-3f);
  cudaEventRecord(e0);
  issueProbe<<<blocks, threads>>>(out, iters, 0.999f, 1e-3f);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess || ms <= 0.0f)
    return -1.0;
  const double fmas = (double)blocks * threads * iters * 64.0;
  return fmas / (ms * 1e-3);
}

/* Voxel updates per second the gather alone sustains, for a storage layout
 * (LOLA_STORE_*) over a width x height detector padded like the pass kernel. */
static double probeKind(int kind, int elem, int channels, int width, int height);
static double probeStorage(int storage, int width, int height);

extern "C" double lolaCudaProbeGatherRate(int storage, int width, int height)
{
  return probeStorage(storage, width, height);
}

/* The same fetches inside a 112 x 24 image (43 KB of FP32 quads) that stays
 * in every SM's L1: the gather pipes' own rate.  (gatherProbe draws bases in
 * the first (pitch - 64) x (rows - 8) pixels, so with 64 + 48 columns and
 * 8 + 16 rows every fetch stays inside the image.) */
extern "C" double lolaCudaProbeGatherPeak(int storage)
{
  return probeStorage(storage, -112, -24);
}

static double probeStorage(int storage, int width, int height)
{
  if (storage == LOLA_STORE_F16QX || storage == LOLA_STORE_F32QX) {
    /* the two pipes run in parallel on their shares of the voxels */
    const int elem = storage == LOLA_STORE_F16QX ? 8 : 16;
    /* the pass kernel's texture share (PassTexMask in bp_kernels.cuh) */
    const unsigned mask = storage == LOLA_STORE_F16QX
                              ? LOLA_F16QX_TEX_MASK
                              : (LOLA_F32QX_COLS ? LOLA_F32QX_COLS_TEX_MASK : LOLA_MIXED_TEX_MASK);
    const double lsu = (mask & 0xFFFFu) == 0xFFFFu
                           ? 1.0
                           : probeKind(elem == 8 ? 3 : 2, elem, 1, width, height);
    const double tex = probeKind(LOLA_MIXED_TEX_LINEAR ? 6 : 5, elem, 4, width, height);
    const double ft = __builtin_popcount(mask & 0xFFFFu) / 16.0;
    if (lsu <= 0.0 || tex <= 0.0)
      return -1.0;
    if (ft <= 0.0)
      return lsu;
    if (ft >= 1.0)
      return tex;
    const double a = lsu / (1.0 - ft), b = tex / ft;
    return a < b ? a : b;
  }
  int kind, elem;
  switch (storage) {
  case LOLA_STORE_F32: kind = 0; elem = 4; break;
  case LOLA_STORE_F16:
  case LOLA_STORE_BF16: kind = 1; elem = 2; break;
  case LOLA_STORE_F32Q: kind = 2; elem = 16; break;
  case LOLA_STORE_F16Q:
  case LOLA_STORE_BF16Q: kind = 3; elem = 8; break;
  case LOLA_STORE_TEX32: kind = 4; elem = 4; break;
  case LOLA_STORE_TEX16: kind = 4; elem = 2; break;
  default: return -1.0;
  }
  return probeKind(kind, elem, 1, width, height);
}

/* width, height < 0: an unpadded |width| x |height| image (L1 resident) */
static double probeKind(int kind, int elem, int channels, int width, int height)
{
  const int pitch = width < 0 ? -width : (width + 128 + 31) & ~31;
  const int rows = height < 0 ? -height : height + 128;
  const size_t bytes = (size_t)pitch * rows * elem;
  void *img = nullptr;
  float *out = nullptr;
  if (cudaMalloc(&img, bytes) != cudaSuccess)
    return -1.0;
  if (cudaMalloc(&out, sizeof(float)) != cudaSuccess) {
    cudaFree(img);
    return -1.0;
  }
  cudaMemset(img, 0, bytes);
  cudaTextureObject_t tex = 0;
  if (kind >= 4) {
    cudaResourceDesc rd = {};
    const int bits = 8 * elem / channels;
    const cudaChannelFormatDesc texel = cudaCreateChannelDesc(bits, channels > 1 ? bits : 0,
        channels > 1 ? bits : 0, channels > 1 ? bits : 0, cudaChannelFormatKindFloat);
    if (kind == 6) {
      rd.resType = cudaResourceTypeLinear;
      rd.res.linear.devPtr = img;
      rd.res.linear.desc = texel;
      rd.res.linear.sizeInBytes = bytes;
    } else {
      rd.resType = cudaResourceTypePitch2D;
      rd.res.pitch2D.devPtr = img;
      rd.res.pitch2D.desc = texel;
      rd.res.pitch2D.width = (size_t)pitch;
      rd.res.pitch2D.height = (size_t)rows;
      rd.res.pitch2D.pitchInBytes = (size_t)pitch * elem;
    }
    cudaTextureDesc td = {};
    td.addressMode[0] = td.addressMode[1] = cudaAddressModeBorder;
    td.filterMode = cudaFilterModePoint;
    td.readMode = cudaReadModeElementType;
    if (cudaCreateTextureObject(&tex, &rd, &td, nullptr) != cudaSuccess) {
      cudaFree(img);
      cudaFree(out);
      return -1.0;
    }
  }
  const int sms = smCount();
  const int blocks = sms * 8, threads = 256, iters = 512;  /* 4 fetches per iteration */
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto launch = [&](int it) {
    switch (kind) {
    case 0: gatherProbe<0><<<blocks, threads>>>(img, pitch, rows, it, out, tex); break;
    case 1: gatherProbe<1><<<blocks, threads>>>(img, pitch, rows, it, out, tex); break;
    case 2: gatherProbe<2><<<blocks, threads>>>(img, pitch, rows, it, out, tex); break;
    case 3: gatherProbe<3><<<blocks, threads>>>(img, pitch, rows, it, out, tex); break;
    case 4: gatherProbe<4><<<blocks, threads>>>(img, pitch, rows, it, out, tex); break;
    case 5: gatherProbe<5><<<blocks, threads>>>(img, pitch, rows, it, out, tex); break;
    default: gatherProbe<6><<<blocks, threads>>>(img, pitch, rows, it, out, tex); break;
    }
  };
  launch(16);
  cudaEventRecord(e0);
  launch(iters);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (tex)
    cudaDestroyTextureObject(tex);
  cudaFree(img);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess || ms <= 0.0f)
    return -1.0;
  return (double)blocks * threads * iters * 4.0 / (ms * 1e-3);
}

/* Lane fetches per second of 8-lane texture requests spanning `rows`
 * detector rows (1, 2, 4 or 8): the texture data stage takes one wavefront
 * per row (or 128-byte window) that a request touches. */
extern "C" double lolaCudaProbeTextureRows(int rows)
{
  if (rows != 1 && rows != 2 && rows != 4 && rows != 8)
    return -1.0;
  const int width = 128, height = 48, elem = 8;
  const size_t bytes = (size_t)width * height * elem;
  void *img = nullptr;
  float *out = nullptr;
  if (cudaMalloc(&img, bytes) != cudaSuccess)
    return -1.0;
  if (cudaMalloc(&out, sizeof(float)) != cudaSuccess) {
    cudaFree(img);
    return -1.0;
  }
  cudaMemset(img, 0, bytes);
  cudaResourceDesc rd = {};
  rd.resType = cudaResourceTypeLinear;
  rd.res.linear.devPtr = img;
  rd.res.linear.desc = cudaCreateChannelDesc(16, 16, 16, 16, cudaChannelFormatKindFloat);
  rd.res.linear.sizeInBytes = bytes;
  cudaTextureDesc td = {};
  td.filterMode = cudaFilterModePoint;
  td.readMode = cudaReadModeElementType;
  cudaTextureObject_t tex = 0;
  if (cudaCreateTextureObject(&tex, &rd, &td, nullptr) != cudaSuccess) {
    cudaFree(img);
    cudaFree(out);
    return -1.0;
  }
  const int blocks = smCount() * 8, threads = 256, iters = 256;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  textureRowsProbe<<<blocks, threads>>>(rows, 16, out, tex);
  cudaEventRecord(e0);
  textureRowsProbe<<<blocks, threads>>>(rows, iters, out, tex);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaDestroyTextureObject(tex);
  cudaFree(img);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess || ms <= 0.0f)
    return -1.0;
  return (double)blocks * threads * iters * 4.0 / (ms * 1e-3);
}

extern "C" int lolaCudaDeviceInfo(int *smCountOut, int *clockKHz, char *name, int nameLen)
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess)
    return 0;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess)
    return 0;
  if (smCountOut)
    *smCountOut = prop.multiProcessorCount;
  if (clockKHz) {
    int c = 0;
    cudaDeviceGetAttribute(&c, cudaDevAttrClockRate, dev);
    *clockKHz = c;
  }
  if (name && nameLen > 0) {
    int i = 0;
    for (; i < nameLen - 1 && prop.name[i]; i++)
      name[i] = prop.name[i];
    name[i] = 0;
  }
  return 1;
}

extern "C" void *lolaCudaHostAlloc(size_t bytes)
{
  void *p = nullptr;
  if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess)
    return nullptr;
  return p;
}

extern "C" int lolaCudaHostFree(void *p)
{
  return cudaFreeHost(p) == cudaSuccess;
}
