/* Batched reconstructions of uneven sizes (volume edge, detector, projection
 * count) in one persistent launch per wave.
 *
 * A wave is projections [wave*b, wave*b + b) of every job.  batchPackKernel
 * stores all of them (each job's own padded layout) into one ring; then the
 * persistent batchPassKernel, one CTA per resident slot of the GPU, pulls
 * work items — (job, tile) pairs, numbered job by job — from an atomic
 * counter until the wave is done, so small and large jobs balance across the
 * SMs without one launch per job.  A work item is exactly a passKernel tile
 * (32 x 8 x 8 voxels in registers across the wave's projections).  The host
 * captures the whole sequence of waves into a CUDA graph once and replays it.
 */
#pragma once

#include "bp_kernels.cuh"

namespace lola {

template <int S>
__global__ void __launch_bounds__(256) batchPackKernel(const LolaBatchWave w)
{
  const int pair = blockIdx.z;
  const int j = pair / w.b, slot = pair - j * w.b;
  const LolaBatchJob &J = w.jobs[j];
  const int view = w.wave * w.b + slot;
  if (view >= J.nproj)
    return;
  const int pu = blockIdx.x * 32 + threadIdx.x;
  const int pv = blockIdx.y * 8 + threadIdx.y;
  if (pu >= J.pitch || pv >= J.rows)
    return;
  const float *img = J.images + (size_t)view * J.width * J.height;
  const int u = pu - J.margin, v = pv - J.margin;
  auto px = [&](int uu, int vv) -> float {
    return (uu >= 0 && uu < J.width && vv >= 0 && vv < J.height)
               ? __ldg(img + (size_t)vv * J.width + uu)
               : 0.0f;
  };
  const size_t o = (size_t)slot * J.slotElems + (size_t)pv * J.pitch + pu;
  if constexpr (Layout<S>::kQuad)
    Layout<S>::store(J.ring, o, px(u, v), px(u + 1, v), px(u, v + 1), px(u + 1, v + 1));
  else
    Layout<S>::store(J.ring, o, px(u, v), 0.f, 0.f, 0.f);
}

template <int S, bool KAHAN>
__global__ void __launch_bounds__(256, 6) batchPassKernel(const LolaBatchWave w)
{
  constexpr int VPT = 8, ROWS = 8;
  __shared__ TileProj sp[LOLA_MAX_BATCH];
  __shared__ long long itemS;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const float fi = (float)threadIdx.x, fj = (float)threadIdx.y;
  for (;;) {
    if (tid == 0)
      itemS = atomicAdd(w.counter, 1);
    __syncthreads();
    const long long item = itemS;
    __syncthreads(); /* every thread holds the item before tid 0 takes the next */
    if (item >= w.totalItems)
      break;
    /* job of the item: last j with tilePrefix[j] <= item */
    int lo = 0, hi = w.njobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (w.tilePrefix[mid] <= item)
        lo = mid;
      else
        hi = mid - 1;
    }
    const LolaBatchJob &J = w.jobs[lo];
    const int count = min(w.b, J.nproj - w.wave * w.b);
    if (count <= 0)
      continue;
    long long t = item - w.tilePrefix[lo];
    const int tx = (int)(t % J.tilesX);
    t /= J.tilesX;
    const int ty = (int)(t % J.tilesY);
    const int tz = (int)(t / J.tilesY);
    const int N = J.N;
    const int x0 = tx * 32, y0 = ty * ROWS, z0 = tz * VPT;

    TileGeom g;
    g.N = N;
    g.zEnd = N;
    g.voxelSize = J.voxelSize;
    g.originIndex = J.originIndex;
    g.width = J.width;
    g.height = J.height;
    g.margin = J.margin;
    setupTileGeom<ROWS, VPT>(w.proj + (size_t)lo * w.b, count, g, sp, tid, 32 * ROWS, x0, y0, z0);

    PassArgs a;
    a.ring = J.ring;
    a.slotBytes = J.slotBytes;
    a.volume = J.volume;
    a.tileCounters = nullptr;
    a.width = J.width;
    a.height = J.height;
    a.margin = J.margin;
    a.pitch = J.pitch;
    a.rows = J.rows;

    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    const bool inXY = (x < N) && (y < N);
    const size_t slice = (size_t)N * (size_t)N;
    float *vcol = J.volume + ((size_t)z0 * N + (size_t)(inXY ? y : 0)) * (size_t)N +
                  (inXY ? x : 0);
    float acc[VPT], comp[VPT];
#pragma unroll
    for (int k = 0; k < VPT; ++k) {
      acc[k] = (inXY && z0 + k < N) ? vcol[k * slice] : 0.0f;
      comp[k] = 0.0f;
    }
    for (int p = 0; p < count; ++p) {
      const int mode = sp[p].mode;
      if (mode == MODE_SKIP)
        continue;
      const TileProj tp = sp[p];
      const void *img = J.ring + (size_t)tp.slot * J.slotBytes;
      const unsigned long long tex =
          (Layout<S>::kTex || Layout<S>::kMixed) ? J.tex[tp.slot] : 0ull;
      if (mode == MODE_FAST)
        applyProjection<S, VPT, KAHAN, false>(tp, img, tex, a, fi, fj, acc, comp);
      else
        applyProjection<S, VPT, KAHAN, true>(tp, img, tex, a, fi, fj, acc, comp);
    }
#pragma unroll
    for (int k = 0; k < VPT; ++k)
      if (inXY && z0 + k < N)
        vcol[k * slice] = KAHAN ? (acc[k] - comp[k]) : acc[k];
    __syncthreads(); /* sp[] is rewritten by the next item's setup */
  }
}

template <int S>
int launchBatchPack(const LolaBatchWave *w, cudaStream_t stream)
{
  const dim3 block(32, 8);
  const dim3 grid((w->maxPitch + 31) / 32, (w->maxRows + 7) / 8, w->njobs * w->b);
  batchPackKernel<S><<<grid, block, 0, stream>>>(*w);
  return (int)cudaGetLastError();
}

template <int S>
int launchBatchPass(const LolaBatchWave *w, int blocks, cudaStream_t stream)
{
  const dim3 block(32, 8);
  if (w->accumulation == LOLA_ACCUM_KAHAN)
    batchPassKernel<S, true><<<blocks, block, 0, stream>>>(*w);
  else
    batchPassKernel<S, false><<<blocks, block, 0, stream>>>(*w);
  return (int)cudaGetLastError();
}

template <int S>
int batchOccupancy(int accumulation, int *blocks)
{
  cudaError_t e = accumulation == LOLA_ACCUM_KAHAN
                      ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                            blocks, batchPassKernel<S, true>, 256, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                            blocks, batchPassKernel<S, false>, 256, 0);
  return (int)e;
}

} /* namespace lola */
