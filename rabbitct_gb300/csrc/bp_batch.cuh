/* Batched reconstructions of uneven sizes (volume edge, detector, projection
 * count) in one persistent launch per wave.
 *
 * A wave is projections [wave*b, wave*b + b) of every job.  batchPackKernel
 * stores all of them (each job's own padded layout) into one ring; then the
 * persistent batchPassKernel, one CTA per resident slot of the GPU, pulls
 * work items — (job, tile) pairs, numbered job by job — from an atomic
 * counter until the wave is done, so small and large jobs balance across the
 * SMs without one launch per job.  A work item is exactly a passKernel tile
 * of LOLA_BATCH_ROWS warps and LOLA_BATCH_VPT voxels per thread (8 x 16 x 16
 * voxels, in registers across the wave's projections).  The host
 * captures the whole sequence of waves into a CUDA graph once and replays it.
 */
#pragma once

#include "bp_kernels.cuh"

namespace lola {

/* The stored-image geometry the per-projection updates read (the fields of
 * PassArgs they use), held in registers for the current job. */
struct ImageGeom {
  int width, height, margin, pitch, rows;
};

/* The image geometry of batchParamPassKernel: ImageGeom plus the texel index
   of the projection's slot within its job's one texture. */
struct SlotGeom {
  int width, height, margin, pitch, rows;
  uint32_t texBase;
};

template <> __device__ __forceinline__ uint32_t texIndexBase<SlotGeom>(const SlotGeom &a)
{
  return a.texBase;
}

/* Stores one wave: block (pair, r) packs rows r, r + LOLA_BATCH_PACK_ROWS, ...
   of the stored image of pair = (job, slot), 256 columns at a time, so that
   the grid covers each job's own image and no more (a grid over the largest
   image for every pair left most blocks of the small detectors idle). */
#define LOLA_BATCH_PACK_ROWS 64
template <int S>
__global__ void __launch_bounds__(256) batchPackKernel(const __grid_constant__ LolaBatchWave w)
{
  const int pair = blockIdx.x;
  const int j = pair / w.b, slot = pair - j * w.b;
  const LolaBatchJob &J = w.jobs[j];
  const int view = w.wave * w.b + slot;
  if (view >= J.nproj)
    return;
  const float *img = J.images + (size_t)view * J.width * J.height;
  auto px = [&](int uu, int vv) -> float {
    return (uu >= 0 && uu < J.width && vv >= 0 && vv < J.height)
               ? __ldg(img + (size_t)vv * J.width + uu)
               : 0.0f;
  };
  for (int pv = blockIdx.y; pv < J.rows; pv += LOLA_BATCH_PACK_ROWS) {
    const int v = pv - J.margin;
    for (int pu = threadIdx.x; pu < J.pitch; pu += 256) {
      const int u = pu - J.margin;
      const size_t o = (size_t)slot * J.slotElems + (size_t)pv * J.pitch + pu;
      if constexpr (Layout<S>::kQuad)
        Layout<S>::store(J.ring, o, px(u, v), px(u + 1, v), px(u, v + 1), px(u + 1, v + 1));
      else
        Layout<S>::store(J.ring, o, px(u, v), 0.f, 0.f, 0.f);
    }
  }
}

/* Resident blocks per SM for the batched pass; its per-job geometry lives in
 * registers rather than the constant bank, so it needs more of them than
 * passKernel (a build-time tuning knob). */
/* 1: the batched pass takes the paired path on positive fast tiles like
   passKernel (a build-time switch for comparisons) */
#ifndef LOLA_BATCH_PAIRED
#define LOLA_BATCH_PAIRED 1
#endif

/* Mixed layouts in the batched pass fetch every quad through loads.  The
   texture object of a work item's projection comes from device memory (the
   wave's per-job handle table), not from the kernel parameters as in
   passKernel, and a texture fetch through such a handle kept f16qx's
   per-item state far beyond its registers (6 KB of spills).  Same values
   either way: the FP16 point fetch widens exactly. */
#ifndef LOLA_BATCH_TEX_MASK
#define LOLA_BATCH_TEX_MASK 0u
#endif

/* resident blocks of LOLA_BATCH_ROWS warps per SM: passKernel's occupancy
   for a load path (36 warps for FP32 layouts, 28 for 16-bit ones) */
#ifndef LOLA_BATCH_MIN_BLOCKS
#define LOLA_BATCH_MIN_BLOCKS(S)                                                            \
  ((MinBlocks<S, LOLA_BATCH_VPT, LOLA_BATCH_ROWS>::kWide32 ? 36 : 28) / LOLA_BATCH_ROWS)
#endif

template <int S, bool KAHAN>
__global__ void __launch_bounds__(32 * LOLA_BATCH_ROWS, LOLA_BATCH_MIN_BLOCKS(S))
    batchPassKernel(const LolaBatchWave w)
{
  constexpr int VPT = LOLA_BATCH_VPT, ROWS = LOLA_BATCH_ROWS;
  constexpr int TX = LOLA_WARP_X, TY = 32 * ROWS / TX;
  __shared__ TileProj sp[LOLA_BATCH_MAX_WAVE];
  /* the current work item: its job's descriptor and tile, shared by the
     block so the per-voxel loop keeps only what passKernel keeps */
  __shared__ LolaBatchJob J;
  __shared__ int itemJob, itemCount, itemX0, itemY0, itemZ0, itemDone;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  int tx, ty;
  laneVoxel<TX, LaneGroups<S>::kValue>(threadIdx.x, threadIdx.y, tx, ty);
  const float fi = (float)tx, fj = (float)ty;
  for (;;) {
    if (tid == 0) {
      const long long item = atomicAdd(w.counter, 1);
      itemDone = item >= w.totalItems;
      if (!itemDone) {
        /* job of the item: last j with tilePrefix[j] <= item */
        int lo = 0, hi = w.njobs - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (w.tilePrefix[mid] <= item)
            lo = mid;
          else
            hi = mid - 1;
        }
        J = w.jobs[lo];
        long long t = item - w.tilePrefix[lo];
        itemJob = lo;
        itemCount = min(w.b, J.nproj - w.wave * w.b);
        itemX0 = (int)(t % J.tilesX) * TX;
        t /= J.tilesX;
        itemY0 = (int)(t % J.tilesY) * TY;
        itemZ0 = (int)(t / J.tilesY) * VPT;
      }
    }
    __syncthreads();
    if (itemDone)
      break;
    const int count = itemCount;
    if (count > 0) {
      const int x0 = itemX0, y0 = itemY0, z0 = itemZ0;
      TileGeom g;
      g.N = J.N;
      g.zEnd = J.N;
      g.voxelSize = J.voxelSize;
      g.originIndex = J.originIndex;
      g.width = J.width;
      g.height = J.height;
      g.margin = J.margin;
      setupTileGeom<ROWS, VPT, TX>(w.proj + (size_t)itemJob * w.b, count, g, sp, tid, 32 * ROWS,
          x0, y0, z0);
      const int N = J.N;
      const int x = x0 + tx, y = y0 + ty;
      const bool inXY = (x < N) && (y < N);
      const size_t slice = (size_t)N * (size_t)N;
      float2 acc[VPT / 2], comp[VPT / 2];
      {
        const float *vcol = J.volume + ((size_t)z0 * N + (size_t)(inXY ? y : 0)) * (size_t)N +
                            (inXY ? x : 0);
#pragma unroll
        for (int k = 0; k < VPT; ++k) {
          voxel(acc, k) = (inXY && z0 + k < N) ? vcol[k * slice] : 0.0f;
          voxel(comp, k) = 0.0f;
        }
      }
      /* read through a volatile view: re-read per projection from shared
         memory instead of pinned in registers across the loop */
      const volatile LolaBatchJob *Jv = &J;
      for (int p = 0; p < count; ++p) {
        const int mode = sp[p].mode;
        if (mode == MODE_SKIP)
          continue;
        const TileProj tp = sp[p];
        ImageGeom a;
        a.width = Jv->width;
        a.height = Jv->height;
        a.margin = Jv->margin;
        a.pitch = Jv->pitch;
        a.rows = Jv->rows;
        const void *img = Jv->ring + (size_t)tp.slot * Jv->slotBytes;
        const unsigned long long tex =
            (Layout<S>::kTex || Layout<S>::kMixed) ? Jv->tex[tp.slot] : 0ull;
        if (mode == MODE_FAST && tp.pos && LOLA_PAIRED && LOLA_BATCH_PAIRED)
          applyPairs<S, VPT, KAHAN, ImageGeom, LOLA_BATCH_TEX_MASK>(tp, img, tex, a, fi, fj,
              acc, comp);
        else if (mode == MODE_FAST)
          applyProjection<S, VPT, KAHAN, false, ImageGeom, LOLA_BATCH_TEX_MASK>(tp, img, tex, a,
              fi, fj, acc, comp);
        else
          applyProjection<S, VPT, KAHAN, true, ImageGeom, LOLA_BATCH_TEX_MASK>(tp, img, tex, a,
              fi, fj, acc, comp);
      }
      float *vcol = J.volume + ((size_t)z0 * N + (size_t)(inXY ? y : 0)) * (size_t)N +
                    (inXY ? x : 0);
#pragma unroll
      for (int k = 0; k < VPT; ++k)
        if (inXY && z0 + k < N)
          vcol[k * slice] = KAHAN ? (voxel(acc, k) - voxel(comp, k)) : voxel(acc, k);
    }
    __syncthreads(); /* J, sp[] and the item fields are rewritten next */
  }
}

/* The persistent pass from the wave's kernel parameters (LolaBatchWave.pj,
   up to LOLA_BATCH_PARAM_JOBS jobs): the work item's job, tile and
   geometry are uniform values of the parameter space, as in passKernel, so
   f16qx fetches every quad through its job's one linear texture (at the
   slot's texel offset) like passKernel does; no job descriptor is copied to
   shared memory. */
template <int S> struct ParamTexMask {
  static constexpr unsigned kValue = S == LOLA_STORE_F16QX ? LOLA_F16QX_TEX_MASK : 0u;
};

template <int S, bool KAHAN>
__global__ void __launch_bounds__(32 * LOLA_BATCH_ROWS,
    (MinBlocks<S, LOLA_BATCH_VPT, LOLA_BATCH_ROWS>::kValue))
    batchParamPassKernel(const __grid_constant__ LolaBatchWave w)
{
  constexpr int VPT = LOLA_BATCH_VPT, ROWS = LOLA_BATCH_ROWS;
  constexpr int TX = LOLA_WARP_X, TY = 32 * ROWS / TX;
  constexpr unsigned TEXMASK = ParamTexMask<S>::kValue;
  __shared__ TileProj sp[LOLA_BATCH_MAX_WAVE];
  __shared__ long long sItem;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  int tx, ty;
  laneVoxel<TX, LaneGroups<S>::kValue>(threadIdx.x, threadIdx.y, tx, ty);
  const float fi = (float)tx, fj = (float)ty;
  for (;;) {
    if (tid == 0)
      sItem = atomicAdd(w.counter, 1);
    __syncthreads();
    const long long item = sItem;
    if (item >= w.totalItems)
      break;
    /* job of the item: the last j with pj[j].firstItem <= item */
    int lo = 0, hi = w.njobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (w.pj[mid].firstItem <= item)
        lo = mid;
      else
        hi = mid - 1;
    }
    const LolaBatchParamJob &J = w.pj[lo];
    const int count = min(w.b, J.count);
    if (count > 0) {
      long long t = item - J.firstItem;
      const int x0 = (int)(t % J.tilesX) * TX;
      t /= J.tilesX;
      const int y0 = (int)(t % J.tilesY) * TY;
      const int z0 = (int)(t / J.tilesY) * VPT;
      TileGeom g;
      g.N = J.N;
      g.zEnd = J.N;
      g.voxelSize = J.voxelSize;
      g.originIndex = J.originIndex;
      g.width = J.width;
      g.height = J.height;
      g.margin = LOLA_MARGIN;
      setupTileGeom<ROWS, VPT, TX>(w.proj + (size_t)lo * w.b, count, g, sp, tid, 32 * ROWS, x0,
          y0, z0);
      const int N = J.N;
      const int x = x0 + tx, y = y0 + ty;
      const bool inXY = (x < N) && (y < N);
      const size_t slice = (size_t)N * (size_t)N;
      float2 acc[VPT / 2], comp[VPT / 2];
      {
        const float *vcol = J.volume + ((size_t)z0 * N + (size_t)(inXY ? y : 0)) * (size_t)N +
                            (inXY ? x : 0);
#pragma unroll
        for (int k = 0; k < VPT; ++k) {
          voxel(acc, k) = (inXY && z0 + k < N) ? vcol[k * slice] : 0.0f;
          voxel(comp, k) = 0.0f;
        }
      }
      for (int p = 0; p < count; ++p) {
        const int mode = sp[p].mode;
        if (mode == MODE_SKIP)
          continue;
        const TileProj tp = sp[p];
        SlotGeom a;
        a.width = J.width;
        a.height = J.height;
        a.margin = LOLA_MARGIN;
        a.pitch = J.pitch;
        a.rows = J.rows;
        a.texBase = (uint32_t)tp.slot * J.slotElems;
        const void *img = J.ring + (size_t)tp.slot * J.slotBytes;
        const unsigned long long tex = J.tex;
        if (mode == MODE_FAST && tp.pos && LOLA_PAIRED && LOLA_BATCH_PAIRED)
          applyPairs<S, VPT, KAHAN, SlotGeom, TEXMASK>(tp, img, tex, a, fi, fj, acc, comp);
        else if (mode == MODE_FAST)
          applyProjection<S, VPT, KAHAN, false, SlotGeom, TEXMASK>(tp, img, tex, a, fi, fj,
              acc, comp);
        else
          applyProjection<S, VPT, KAHAN, true, SlotGeom, TEXMASK>(tp, img, tex, a, fi, fj,
              acc, comp);
      }
      float *vcol = J.volume + ((size_t)z0 * N + (size_t)(inXY ? y : 0)) * (size_t)N +
                    (inXY ? x : 0);
#pragma unroll
      for (int k = 0; k < VPT; ++k)
        if (inXY && z0 + k < N)
          vcol[k * slice] = KAHAN ? (voxel(acc, k) - voxel(comp, k)) : voxel(acc, k);
    }
    __syncthreads(); /* sp[] and sItem are rewritten next */
  }
}

template <int S>
int launchBatchPack(const LolaBatchWave *w, cudaStream_t stream)
{
  const dim3 block(256);
  const dim3 grid(w->njobs * w->b, LOLA_BATCH_PACK_ROWS);
  (void)cudaGetLastError();  /* report this launch's error, not an earlier one */
  batchPackKernel<S><<<grid, block, 0, stream>>>(*w);
  return (int)cudaGetLastError();
}

template <int S>
int launchBatchPass(const LolaBatchWave *w, int blocks, cudaStream_t stream)
{
  const dim3 block(32, LOLA_BATCH_ROWS);
  (void)cudaGetLastError();  /* report this launch's error, not an earlier one */
  const bool kahan = w->accumulation == LOLA_ACCUM_KAHAN;
  if (w->paramJobs) {
    if (kahan)
      batchParamPassKernel<S, true><<<blocks, block, 0, stream>>>(*w);
    else
      batchParamPassKernel<S, false><<<blocks, block, 0, stream>>>(*w);
  } else {
    if (kahan)
      batchPassKernel<S, true><<<blocks, block, 0, stream>>>(*w);
    else
      batchPassKernel<S, false><<<blocks, block, 0, stream>>>(*w);
  }
  return (int)cudaGetLastError();
}

template <int S>
int batchOccupancy(int accumulation, int paramJobs, int *blocks)
{
  const int threads = 32 * LOLA_BATCH_ROWS;
  if (paramJobs)
    return (int)(accumulation == LOLA_ACCUM_KAHAN
                     ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks,
                           batchParamPassKernel<S, true>, threads, 0)
                     : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks,
                           batchParamPassKernel<S, false>, threads, 0));
  cudaError_t e = accumulation == LOLA_ACCUM_KAHAN
                      ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                            blocks, batchPassKernel<S, true>, 32 * LOLA_BATCH_ROWS, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                            blocks, batchPassKernel<S, false>, 32 * LOLA_BATCH_ROWS, 0);
  return (int)e;
}

} /* namespace lola */
