/* TMA-staged backprojection pass for sm_103a.
 *
 * Same method and tile mapping as passKernel (bp_kernels.cuh); what changes is
 * where the taps come from.  For every (tile, projection) whose footprint fits
 * the staging box, one elected producer thread copies that box of the stored
 * projection from L2/HBM into shared memory with a 3D tensor copy
 * (cp.async.bulk.tensor, completion on an mbarrier), two stages deep, while
 * the consumer warps gather the previous projection's taps from shared
 * memory.  The L2 round trip of every first touch, which dominated the
 * load-path kernel's stalls, leaves the critical path.
 *
 * Block: ROWS consumer warps (the passKernel tile of 32 ROWS x VPT voxels, in registers
 * across the pass) plus one producer warp.  Barriers per stage s:
 *   full[s]   1 arrival (producer, with the box's byte count), completed by
 *             the tensor copy;
 *   empty[s]  ROWS arrivals (one per consumer warp when done with the stage).
 * The k-th staged projection of the pass uses stage k % LOLA_STAGES in phase
 * k / LOLA_STAGES.
 * Tiles that are skipped, clamped or too large for the box keep using the
 * global path of passKernel inside the same launch.
 *
 * Every wait is bounded by a clock budget; on expiry the thread records an
 * error code in PassStage::errorFlag (read by the host after the pass),
 * abandons staged work and returns normally.
 */
#pragma once

#include <cuda.h>

#include "bp_kernels.cuh"

namespace lola {

enum { MODE_STAGED = 3 };

struct StageArgs {
  int boxW, boxH;        /* staging box, pixels */
  int align;             /* box origin alignment, pixels (16 B) */
  int elemsPerPixel;     /* tensor-map elements per stored pixel */
  int stageBytes;        /* bytes per stage buffer (128 B multiple) */
  int boxBytes;          /* bytes one tensor copy delivers */
  int *errorFlag;
};

/* Clock budget of every mbarrier wait: about 1 s at 2 GHz. */
#ifndef LOLA_STAGE_WAIT_CYCLES
#define LOLA_STAGE_WAIT_CYCLES 2000000000ll
#endif
constexpr long long kWaitLimitCycles = LOLA_STAGE_WAIT_CYCLES;

/* 1: the producer issues the tensor copies.  0 is for the wait-timeout test
   build only (tests/test_gpu_stage_timeout.py, with a short
   LOLA_STAGE_WAIT_CYCLES): the producer issues neither the copies nor their
   byte counts, so no copy is ever in flight, every stage's full barrier stays
   incomplete and each consumer warp's bounded wait runs out, records its
   error code and abandons the staged work. */
#ifndef LOLA_STAGE_ISSUE_COPIES
#define LOLA_STAGE_ISSUE_COPIES 1
#endif

__device__ __forceinline__ uint32_t smemAddr(const void *p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbarInit(uint32_t bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbarExpectTx(uint32_t bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbarArrive(uint32_t bar)
{
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbarTryWait(uint32_t bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile("{\n\t.reg .pred p;\n\t"
               "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
               "selp.u32 %0, 1, 0, p;\n\t}"
               : "=r"(ok)
               : "r"(bar), "r"(parity)
               : "memory");
  return ok != 0;
}

/* Waits for the phase of `bar` with the given parity; false after the budget. */
__device__ __forceinline__ bool mbarWait(uint32_t bar, uint32_t parity)
{
  if (mbarTryWait(bar, parity))
    return true;
  const long long t0 = clock64();
  while (!mbarTryWait(bar, parity))
    if (clock64() - t0 > kWaitLimitCycles)
      return false;
  return true;
}

__device__ __forceinline__ void tmaLoad3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z,
    uint32_t bar)
{
  asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
               " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
               "l"(map), "r"(x), "r"(y), "r"(z), "r"(bar)
               : "memory");
}

/* ---- taps from a staged box (row-major, boxW pixels per row) ---------------- */

template <int S> struct SharedTaps;

template <> struct SharedTaps<LOLA_STORE_F32> {
  static constexpr bool kQuad = false;
  static constexpr bool kDiff = false;
  __device__ static __forceinline__ void fetch(const unsigned char *b, uint32_t i, int w,
      float &p00, float &p10, float &p01, float &p11)
  {
    const float *f = reinterpret_cast<const float *>(b) + i;
    p00 = f[0];
    p10 = f[1];
    p01 = f[w];
    p11 = f[w + 1];
  }
};

template <> struct SharedTaps<LOLA_STORE_F16> {
  static constexpr bool kQuad = false;
  static constexpr bool kDiff = false;
  __device__ static __forceinline__ void fetch(const unsigned char *b, uint32_t i, int w,
      float &p00, float &p10, float &p01, float &p11)
  {
    const __half *h = reinterpret_cast<const __half *>(b) + i;
    p00 = __half2float(h[0]);
    p10 = __half2float(h[1]);
    p01 = __half2float(h[w]);
    p11 = __half2float(h[w + 1]);
  }
};

template <> struct SharedTaps<LOLA_STORE_BF16> {
  static constexpr bool kQuad = false;
  static constexpr bool kDiff = false;
  __device__ static __forceinline__ void fetch(const unsigned char *b, uint32_t i, int w,
      float &p00, float &p10, float &p01, float &p11)
  {
    const unsigned short *h = reinterpret_cast<const unsigned short *>(b) + i;
    p00 = __uint_as_float((uint32_t)h[0] << 16);
    p10 = __uint_as_float((uint32_t)h[1] << 16);
    p01 = __uint_as_float((uint32_t)h[w] << 16);
    p11 = __uint_as_float((uint32_t)h[w + 1] << 16);
  }
};

/* FP32 quads in the order Layout<S> stores them */
template <bool COLS> struct SharedQuadF32 {
  static constexpr bool kQuad = true;
  static constexpr bool kDiff = false;
  __device__ static __forceinline__ void fetch(const unsigned char *b, uint32_t i, int,
      float &p00, float &p10, float &p01, float &p11)
  {
    const float4 q = reinterpret_cast<const float4 *>(b)[i];
    p00 = q.x;
    p10 = COLS ? q.z : q.y;
    p01 = COLS ? q.y : q.z;
    p11 = q.w;
  }
};

template <> struct SharedTaps<LOLA_STORE_F32Q>
    : SharedQuadF32<Layout<LOLA_STORE_F32Q>::kCols> {};

/* FP16 quads in the order Layout<S> stores them */
template <bool COLS> struct SharedQuadF16 {
  static constexpr bool kQuad = true;
  static constexpr bool kDiff = LOLA_QUAD_TERMS;  /* as stored by Layout<S> */
  __device__ static __forceinline__ void fetch(const unsigned char *b, uint32_t i, int,
      float &p00, float &p10, float &p01, float &p11)
  {
    const uint2 q = reinterpret_cast<const uint2 *>(b)[i];
    const float2 lo = __half22float2(*reinterpret_cast<const __half2 *>(&q.x));
    const float2 hi = __half22float2(*reinterpret_cast<const __half2 *>(&q.y));
    p00 = lo.x;
    p10 = COLS ? hi.x : lo.y;
    p01 = COLS ? lo.y : hi.x;
    p11 = hi.y;
  }
};

template <> struct SharedTaps<LOLA_STORE_F16Q> : SharedQuadF16<Layout<LOLA_STORE_F16Q>::kCols> {};

template <> struct SharedTaps<LOLA_STORE_BF16Q> {
  static constexpr bool kQuad = true;
  static constexpr bool kDiff = LOLA_QUAD_TERMS;  /* as stored by Layout<S> */
  __device__ static __forceinline__ void fetch(const unsigned char *b, uint32_t i, int,
      float &p00, float &p10, float &p01, float &p11)
  {
    const uint2 q = reinterpret_cast<const uint2 *>(b)[i];
    p00 = bf16LoToFloat(q.x);
    p10 = bf16HiToFloat(q.x);
    p01 = bf16LoToFloat(q.y);
    p11 = bf16HiToFloat(q.y);
  }
};

template <> struct SharedTaps<LOLA_STORE_F16QX>
    : SharedQuadF16<Layout<LOLA_STORE_F16QX>::kCols> {};
template <> struct SharedTaps<LOLA_STORE_F32QX>
    : SharedQuadF32<Layout<LOLA_STORE_F32QX>::kCols> {};

/* Applies one staged projection to the thread's VPT voxels (unclamped: only
 * tiles on the fast path are staged). */
template <int S, int VPT, bool KAHAN>
__device__ __forceinline__ void applyStaged(const TileProj &tp, const unsigned char *box,
    const StageArgs &g, float fi, float fj, float2 (&acc)[VPT / 2], float2 (&comp)[VPT / 2])
{
  const float bw = (float)g.boxW;
  const uint32_t maxIdx = SharedTaps<S>::kQuad ? (uint32_t)(g.boxW * g.boxH - 1)
                                               : (uint32_t)(g.boxW * g.boxH - g.boxW - 2);
  const float ut = fmaf(fj, tp.su[1], fmaf(fi, tp.su[0], tp.u0));
  const float vt = fmaf(fj, tp.sv[1], fmaf(fi, tp.sv[0], tp.v0));
  const float wt = fmaf(fj, tp.sw[1], fmaf(fi, tp.sw[0], tp.w0));
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    const float kf = (float)k;
    const float w = fmaf(kf, tp.sw[2], wt);
    const float u = fmaf(kf, tp.su[2], ut);
    const float v = fmaf(kf, tp.sv[2], vt);
    const float r = rcpApprox(w);
    const float ix = fmaf(u, r, tp.cu);
    const float iy = fmaf(v, r, tp.cv);
    const float tx = truncf(ix);
    const float ty = truncf(iy);
    const float ax = ix - tx;
    const float ay = iy - ty;
    /* box-local index of pixel (tx, ty), formed as 2^23 + index in FP32 */
    uint32_t idx = __float_as_uint(fmaf(ty, bw, tx + tp.sbias)) - 0x4B000000u;
    idx = min(idx, maxIdx);  /* stays inside the stage buffer whatever the input */
    float p00, p10, p01, p11;
    SharedTaps<S>::fetch(box, idx, g.boxW, p00, p10, p01, p11);
    const float val = bilinear<SharedTaps<S>::kDiff>(ax, ay, p00, p10, p01, p11);
    const float term = val * (r * r);
    float &ak = voxel(acc, k);
    if (KAHAN) {
      float &ck = voxel(comp, k);
      const float y = term - ck;
      const float s = ak + y;
      ck = (s - ak) - y;
      ak = s;
    } else {
      ak += term;
    }
  }
}

/* The paired update (pairedUpdate) on a staged box: the same arithmetic as
 * applyPairs on the ring, so both gather paths give identical results. */
template <int S, int VPT, bool KAHAN>
__device__ __forceinline__ void applyStagedPairs(const TileProj &tp, const unsigned char *box,
    const StageArgs &g, float fi, float fj, float2 (&acc)[VPT / 2], float2 (&comp)[VPT / 2])
{
  const uint32_t maxIdx = SharedTaps<S>::kQuad ? (uint32_t)(g.boxW * g.boxH - 1)
                                               : (uint32_t)(g.boxW * g.boxH - g.boxW - 2);
  const int boxW = g.boxW;
  auto fetch = [&](int, float idxf, float, float, float &p00, float &p10, float &p01,
                   float &p11) {
    uint32_t idx = __float_as_uint(idxf) - 0x4B000000u;
    idx = min(idx, maxIdx);  /* stays inside the stage buffer whatever the input */
    SharedTaps<S>::fetch(box, idx, boxW, p00, p10, p01, p11);
  };
  /* 2^23 + box-local index of pixel (cu, cv), which lies in the box (the tile
     origin's own pixel is inside its footprint) */
  const float kxc = fmaf(tp.cv + tp.syo, (float)g.boxW, tp.sxm + tp.cu);
  pairedUpdate<VPT, KAHAN, SharedTaps<S>::kDiff, 0u>(tp, fi, fj, kxc, (float)g.boxW, fetch,
      acc, comp);
}

#ifndef LOLA_STAGED_MIN_BLOCKS
#define LOLA_STAGED_MIN_BLOCKS 4
#endif

template <int S, int VPT, int ROWS, bool KAHAN>
__global__ void __launch_bounds__(32 * (ROWS + 1), LOLA_STAGED_MIN_BLOCKS)
    stagedPassKernel(const PassArgs a, const LolaPassParams P, const StageArgs g,
        const __grid_constant__ CUtensorMap tmap)
{
  extern __shared__ __align__(128) unsigned char stageMem[];
  __shared__ TileProj sp[LOLA_MAX_BATCH];
  constexpr int NS = LOLA_STAGES;
  __shared__ __align__(8) unsigned long long bars[2 * NS]; /* full[NS], empty[NS] */
  const int N = P.N;
  const int count = P.count;
  constexpr int TX = LOLA_WARP_X, TY = 32 * ROWS / TX;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = P.zBegin + blockIdx.z * VPT;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const uint32_t full0 = smemAddr(&bars[0]);
  const uint32_t empty0 = smemAddr(&bars[NS]);

  if (tid == 0) {
    for (int s = 0; s < NS; ++s) {
      mbarInit(full0 + 8 * s, 1);
      mbarInit(empty0 + 8 * s, ROWS);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  setupTile<ROWS, VPT, TX>(P, a, sp, tid, 32 * (ROWS + 1), x0, y0, z0);

  /* which fast-path projections fit the box: numbered in pass order */
  if (tid == 0) {
    int k = 0;
    for (int p = 0; p < count; ++p) {
      TileProj &t = sp[p];
      t.seq = -1;
      if (t.mode != MODE_FAST)
        continue;
      /* taps lie in [floor(f0), floor(f1) + 3): truncation is floor, or floor + 1
         for negative coordinates, and the second tap is one further */
      const int xlo = (int)floorf(t.fx0) + a.margin, xhi = (int)floorf(t.fx1) + 3 + a.margin;
      const int ylo = (int)floorf(t.fy0) + a.margin, yhi = (int)floorf(t.fy1) + 3 + a.margin;
      const int bx = xlo & ~(g.align - 1);
      if (xhi - bx > g.boxW || yhi - ylo > g.boxH)
        continue;
      t.mode = MODE_STAGED;
      t.seq = k++;
      t.bx = bx;
      t.by = ylo;
      t.sbias = 8388608.0f + (float)((a.margin - bx) + (a.margin - ylo) * g.boxW);
      t.sxm = 8388608.0f + (float)(a.margin - bx);
      t.syo = (float)(a.margin - ylo);
    }
  }
  __syncthreads();

  if (a.tileCounters != nullptr && tid == 0) {
    unsigned long long n[5] = { 0, 0, 0, 0, 0 };
    for (int p = 0; p < count; ++p) {
      const int m = sp[p].mode;
      n[0] += (m == MODE_SKIP);
      n[1] += (m == MODE_FAST);
      n[2] += (m == MODE_SLOW);
      n[3] += (m == MODE_STAGED);
      n[4] += ((m == MODE_FAST || m == MODE_STAGED) && sp[p].pos && LOLA_PAIRED);
    }
    const unsigned copy =
        (blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)) % LOLA_COUNTER_SPREAD;
    unsigned long long *counters = a.tileCounters + copy * LOLA_TILE_COUNTERS;
    atomicAdd(counters + 0, n[0]);
    atomicAdd(counters + 1, n[1] + n[3]);
    atomicAdd(counters + 2, n[2]);
    atomicAdd(counters + 3, n[3]);
    atomicAdd(counters + 4, n[4]);
  }

  if (threadIdx.y == ROWS) {
    /* producer warp: one elected lane issues the tensor copies in pass order */
    if (threadIdx.x == 0) {
      for (int p = 0; p < count; ++p) {
        const TileProj &t = sp[p];
        if (t.mode != MODE_STAGED)
          continue;
        const int k = t.seq, s = k % NS;
        if (k >= NS && !mbarWait(empty0 + 8 * s, (uint32_t)((k / NS - 1) & 1))) {
          atomicExch(g.errorFlag, 1);
          break;
        }
        if (LOLA_STAGE_ISSUE_COPIES) {
          mbarExpectTx(full0 + 8 * s, (uint32_t)g.boxBytes);
          tmaLoad3d(smemAddr(stageMem + s * g.stageBytes), &tmap, t.bx * g.elemsPerPixel, t.by,
              t.slot, full0 + 8 * s);
        }
      }
    }
    return;
  }

  /* consumer warps */
  const int tx = threadIdx.x % TX, ty = threadIdx.y * (32 / TX) + threadIdx.x / TX;
  const int x = x0 + tx, y = y0 + ty;
  const bool inXY = (x < N) && (y < N);
  const size_t slice = (size_t)N * (size_t)N;
  /* the plan holds only the slab z in [zBegin, zEnd) */
  float *vcol = a.volume + ((size_t)(z0 - P.zBegin) * N + (size_t)(inXY ? y : 0)) * (size_t)N +
                (inXY ? x : 0);
  float2 acc[VPT / 2], comp[VPT / 2];
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    voxel(acc, k) = (inXY && z0 + k < P.zEnd) ? vcol[k * slice] : 0.0f;
    voxel(comp, k) = 0.0f;
  }
  const float fi = (float)tx, fj = (float)ty;
  bool abandoned = false;
  for (int p = 0; p < count; ++p) {
    const int mode = sp[p].mode;
    if (mode == MODE_SKIP)
      continue;
    const TileProj tp = sp[p];
    if (mode == MODE_STAGED) {
      const int s = tp.seq % NS;
      if (!abandoned && !mbarWait(full0 + 8 * s, (uint32_t)((tp.seq / NS) & 1))) {
        atomicExch(g.errorFlag, 2);
        abandoned = true;
      }
      if (!abandoned && tp.pos && LOLA_PAIRED)
        applyStagedPairs<S, VPT, KAHAN>(tp, stageMem + s * g.stageBytes, g, fi, fj, acc,
            comp);
      else if (!abandoned)
        applyStaged<S, VPT, KAHAN>(tp, stageMem + s * g.stageBytes, g, fi, fj, acc, comp);
      __syncwarp();
      if (threadIdx.x == 0)
        mbarArrive(empty0 + 8 * s);
      continue;
    }
    const void *img = static_cast<const char *>(a.ring) + (size_t)tp.slot * a.slotBytes;
    const unsigned long long tex =
        (Layout<S>::kTex || Layout<S>::kMixed) ? a.tex[tp.slot] : 0ull;
    if (mode == MODE_FAST && tp.pos && LOLA_PAIRED)
      applyPairs<S, VPT, KAHAN>(tp, img, tex, a, fi, fj, acc, comp);
    else if (mode == MODE_FAST)
      applyProjection<S, VPT, KAHAN, false>(tp, img, tex, a, fi, fj, acc, comp);
    else
      applyProjection<S, VPT, KAHAN, true>(tp, img, tex, a, fi, fj, acc, comp);
  }
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    if (inXY && z0 + k < P.zEnd)
      vcol[k * slice] = KAHAN ? (voxel(acc, k) - voxel(comp, k)) : voxel(acc, k);
  }
}

template <int S, int VPT, int ROWS, bool KAHAN>
int launchStagedShape(const PassArgs &a, const LolaPassParams *P, const StageArgs &g,
    const CUtensorMap &map, cudaStream_t stream)
{
  const int N = P->N;
  const dim3 block(32, ROWS + 1);
  const int nz = P->zEnd - P->zBegin;
  constexpr int TX = LOLA_WARP_X, TY = 32 * ROWS / TX;
  const dim3 grid((N + TX - 1) / TX, (N + TY - 1) / TY, (nz + VPT - 1) / VPT);
  const size_t smem = (size_t)LOLA_STAGES * (size_t)g.stageBytes;
  auto kernel = stagedPassKernel<S, VPT, ROWS, KAHAN>;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
      (int)smem);
  if (e != cudaSuccess)
    return (int)e;
  (void)cudaGetLastError();  /* report this launch's error, not an earlier one */
  kernel<<<grid, block, smem, stream>>>(a, *P, g, map);
  return (int)cudaGetLastError();
}

template <int S, bool KAHAN>
int launchStagedAccum(const PassArgs &a, const LolaPassParams *P, const StageArgs &g,
    const CUtensorMap &map, cudaStream_t stream)
{
  if (P->voxelsPerThread == 8 && P->rowsPerBlock == 8)
    return launchStagedShape<S, 8, 8, KAHAN>(a, P, g, map, stream);
  if (P->voxelsPerThread == 8 && P->rowsPerBlock == 4)
    return launchStagedShape<S, 8, 4, KAHAN>(a, P, g, map, stream);
  return (int)cudaErrorInvalidConfiguration;
}

template <int S>
int launchStaged(const LolaStoreDesc *st, const LolaPassParams *P, const LolaStageDesc *sd,
    const void *ring, float *volume, unsigned long long *counters, cudaStream_t stream)
{
  if constexpr (Layout<S>::kTex) {
    return (int)cudaErrorNotSupported;
  } else {
    PassArgs a;
    fillPassArgs(a, st, ring, volume, counters);
    StageArgs g;
    g.boxW = sd->boxW;
    g.boxH = sd->boxH;
    g.align = sd->align;
    g.elemsPerPixel = sd->elemsPerPixel;
    g.stageBytes = sd->stageBytes;
    g.boxBytes = sd->boxBytes;
    g.errorFlag = sd->d_error;
    const CUtensorMap &map = sd->tensorMap;
    if (P->accumulation == LOLA_ACCUM_KAHAN)
      return launchStagedAccum<S, true>(a, P, g, map, stream);
    return launchStagedAccum<S, false>(a, P, g, map, stream);
  }
}

} /* namespace lola */
