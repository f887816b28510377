/* LolaCUDA kernels: projection packing and volume-tile-stationary
 * backprojection for sm_103a.
 *
 * Method (identical to LolaBunny, HPC-Dwarfs/RabbitCT src/LolaBunny.c:44-75):
 * for every voxel (i, j, k) at world position O + (i, j, k) * voxelSize and
 * every projection with matrix a (3x4, column-major):
 *     w = a2 x + a5 y + a8 z + a11,  u = (a0 x + a3 y + a6 z + a9) / w,
 *     v = (a1 x + a4 y + a7 z + a10) / w
 *     vol += 1/w^2 * bilinear(image, u, v)
 * where bilinear() truncates toward zero ((int)u, so the weight is negative
 * for u in (-2, 0)) and reads 0 outside the detector (src/LolaBunny.c:11-30).
 *
 * GB300 mapping:
 *  - A CTA of ROWS warps owns a tile of 32 ROWS x VPT voxels: each warp an
 *    LOLA_WARP_X x (32 / LOLA_WARP_X) patch of the xy plane (8 x 4 by default,
 *    a compact detector footprint; for the texture-fetched FP16 quads and the
 *    FP32 quads each 8-lane quarter a 4 x 2 part of it, laneVoxel), each
 *    thread VPT voxels along z.  Each
 *    thread keeps its VPT voxels (one xy column, consecutive z) in registers for a
 *    whole pass of up to LOLA_MAX_BATCH projections, so the volume crosses HBM
 *    once per pass instead of once per projection.
 *  - Per (tile, projection) the tile origin is projected in FP64 (the only
 *    FP64 work: 11 DFMA).  The homogeneous coordinates are re-centred on an
 *    FP32 pixel offset c, u' = u - c w, so the FP32 values stepped per voxel
 *    are small and ix = c + u'/w keeps the precision of ix itself.
 *  - The 8 tile corners give the tile's detector footprint (the projection of
 *    a box with w > 0 lies in the convex hull of its corners).  A tile whose
 *    footprint misses the detector is skipped for that projection (LolaBunny
 *    adds exact zeros there); one inside the zero margin runs without clamps;
 *    any other runs the clamped path, which is exact for every voxel.
 *  - Projections are stored zero-padded by LOLA_MARGIN pixels and stay L2
 *    resident; taps are gathered through the read-only L1 path.  The quad
 *    layouts store each pixel's 2x2 neighbourhood together, so one 16 B (FP32)
 *    or 8 B (FP16/BF16) load fetches all four taps.
 *  - Floor/index arithmetic avoids the conversion pipe: the stored index is
 *    formed in FP32 (exact below 2^24) and read from the float's mantissa
 *    after adding 2^23.
 */
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "lolacuda_internal.h"

namespace lola {

enum { MODE_SKIP = 0, MODE_FAST = 1, MODE_SLOW = 2 };

/* 1: positive fast tiles take the packed two-voxel path (applyPairs); 0: every
   tile the one-voxel path (a build-time switch for comparisons) */
#ifndef LOLA_PAIRED
#define LOLA_PAIRED 1
#endif

/* 1: the per-tile setup reads the pass's projections from their device copy
   (LolaPassParams.projDevice) where the host provides one */
#ifndef LOLA_PROJ_DEVICE
#define LOLA_PROJ_DEVICE 1
#endif

/* Per (tile, projection) setup kept in shared memory for the whole pass. */
/* 16-byte aligned so that a thread can read its fields from shared memory
   four at a time (FP32 quads 1298 vs 1261 GUPS at N=1024 on GB300; storing
   the paired path's constant pairs here as well measured 2-3 % slower) */
#ifndef LOLA_TILEPROJ_ALIGN
#define LOLA_TILEPROJ_ALIGN 16
#endif
struct __align__(LOLA_TILEPROJ_ALIGN) TileProj {
  float u0, v0, w0;   /* re-centred homogeneous coordinates at the tile origin */
  float cu, cv;       /* pixel offsets: ix = cu + u'/w, iy = cv + v'/w */
  float su[3], sv[3], sw[3]; /* per-axis steps (x, y, z) of u', v', w */
  int mode;
  int pos;            /* MODE_FAST with non-negative detector coordinates only */
  int slot;
  float fx0, fx1, fy0, fy1;  /* footprint of the tile on the detector (pixels) */
  /* shared-memory staging (staged pass only) */
  int seq;                   /* index among the staged projections of the pass */
  int bx, by;                /* box origin in the padded image */
  float sbias;               /* 2^23 + box-local index of detector pixel (0, 0) */
  float sxm, syo;            /* 2^23 + box-local column of detector column 0; box-local
                                row of detector row 0 */
};

__device__ __forceinline__ float rcpApprox(float x)
{
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float bf16LoToFloat(uint32_t x) { return __uint_as_float(x << 16); }
__device__ __forceinline__ float bf16HiToFloat(uint32_t x) { return __uint_as_float(x & 0xffff0000u); }

/* ---- bilinear interpolation ------------------------------------------------- */

/* 1: the 16-bit quad layouts store bilinear terms (below); 0: the four taps
   (a build-time switch for comparisons) */
#ifndef LOLA_QUAD_TERMS
#define LOLA_QUAD_TERMS 1
#endif

/* The 16-bit quad layouts store each pixel's bilinear terms instead of its four
 * taps: p00, p10 - p00, p01 - p00 and p11 - p01 - p10 + p00 (formed in FP32,
 * then rounded), so that
 *     bilinear = p00 + ax (p10 - p00) + ay ((p01 - p00) + ax (p11 - p01 - p10 + p00))
 * takes three FMAs instead of six operations.  It is LolaBunny's product form
 * (src/LolaBunny.c:24-29) regrouped; the 16-bit rounding falls on the terms
 * instead of the taps. */
__device__ __forceinline__ float4 bilinearTerms(float p00, float p10, float p01, float p11)
{
  const float d10 = p10 - p00;
  return make_float4(p00, d10, p01 - p00, (p11 - p01) - d10);
}

/* Bilinear value from the four fetched terms: taps (p00, p10, p01, p11), or,
 * for DIFF layouts, the terms of bilinearTerms. */
template <bool DIFF>
__device__ __forceinline__ float bilinear(float ax, float ay, float q0, float q1, float q2,
    float q3)
{
  if (DIFF) {
    const float b = fmaf(ax, q1, q0);
    const float c = fmaf(ax, q3, q2);
    return fmaf(ay, c, b);
  }
  const float b = fmaf(ax, q1 - q0, q0);
  const float t = fmaf(ax, q3 - q2, q2);
  return fmaf(ay, t - b, b);
}

/* ---- tap fetch per storage layout ------------------------------------------ */

template <int S> struct Layout;

template <> struct Layout<LOLA_STORE_F32> {
  static constexpr bool kTex = false;
  static constexpr bool kMixed = false;
  static constexpr bool kCols = false;
  typedef float Elem;
  static constexpr bool kQuad = false;
  static constexpr bool kDiff = false;
  __device__ static __forceinline__ void fetch(const void *img, uint32_t idx, int pitch,
      float &p00, float &p10, float &p01, float &p11)
  {
    const float *f = static_cast<const float *>(img) + idx;
    p00 = __ldg(f);
    p10 = __ldg(f + 1);
    p01 = __ldg(f + pitch);
    p11 = __ldg(f + pitch + 1);
  }
  __device__ static __forceinline__ void store(void *dst, size_t o, float a, float, float, float)
  {
    static_cast<float *>(dst)[o] = a;
  }
};

template <> struct Layout<LOLA_STORE_F16> {
  static constexpr bool kTex = false;
  static constexpr bool kMixed = false;
  static constexpr bool kCols = false;
  typedef __half Elem;
  static constexpr bool kQuad = false;
  static constexpr bool kDiff = false;
  __device__ static __forceinline__ void fetch(const void *img, uint32_t idx, int pitch,
      float &p00, float &p10, float &p01, float &p11)
  {
    const __half *h = static_cast<const __half *>(img) + idx;
    p00 = __half2float(__ldg(h));
    p10 = __half2float(__ldg(h + 1));
    p01 = __half2float(__ldg(h + pitch));
    p11 = __half2float(__ldg(h + pitch + 1));
  }
  __device__ static __forceinline__ void store(void *dst, size_t o, float a, float, float, float)
  {
    static_cast<__half *>(dst)[o] = __float2half_rn(a);
  }
};

template <> struct Layout<LOLA_STORE_BF16> {
  static constexpr bool kTex = false;
  static constexpr bool kMixed = false;
  static constexpr bool kCols = false;
  typedef __nv_bfloat16 Elem;
  static constexpr bool kQuad = false;
  static constexpr bool kDiff = false;
  __device__ static __forceinline__ void fetch(const void *img, uint32_t idx, int pitch,
      float &p00, float &p10, float &p01, float &p11)
  {
    const unsigned short *h = static_cast<const unsigned short *>(img) + idx;
    p00 = __uint_as_float((uint32_t)__ldg(h) << 16);
    p10 = __uint_as_float((uint32_t)__ldg(h + 1) << 16);
    p01 = __uint_as_float((uint32_t)__ldg(h + pitch) << 16);
    p11 = __uint_as_float((uint32_t)__ldg(h + pitch + 1) << 16);
  }
  __device__ static __forceinline__ void store(void *dst, size_t o, float a, float, float, float)
  {
    static_cast<__nv_bfloat16 *>(dst)[o] = __float2bfloat16_rn(a);
  }
};

/* 1: FP32 quads are stored column by column, (p00, p01, p10, p11), so that a
   quad load lands as the two column pairs the paired path interpolates in
   x with one packed FMA each (f32q 1352 vs 1294 GUPS at N=1024 on GB300);
   0: row by row, (p00, p10, p01, p11).  The mixed layout f32qx has its own
   switch, LOLA_F32QX_COLS. */
#ifndef LOLA_F32Q_COLS
#define LOLA_F32Q_COLS 1
#endif

template <bool COLS> struct QuadF32Layout {
  static constexpr bool kTex = false;
  static constexpr bool kMixed = false;
  static constexpr bool kCols = COLS;
  typedef float4 Elem;
  static constexpr bool kQuad = true;
  static constexpr bool kDiff = false;
  __device__ static __forceinline__ void fetch(const void *img, uint32_t idx, int,
      float &p00, float &p10, float &p01, float &p11)
  {
    const float4 q = __ldg(static_cast<const float4 *>(img) + idx);
    p00 = q.x;
    p10 = kCols ? q.z : q.y;
    p01 = kCols ? q.y : q.z;
    p11 = q.w;
  }
  /* the stored components in their stored order */
  __device__ static __forceinline__ void fetchRaw(const void *img, uint32_t idx, int,
      float &q0, float &q1, float &q2, float &q3)
  {
    const float4 q = __ldg(static_cast<const float4 *>(img) + idx);
    q0 = q.x;
    q1 = q.y;
    q2 = q.z;
    q3 = q.w;
  }
  /* taps p00, p10, p01, p11 */
  __device__ static __forceinline__ void store(void *dst, size_t o, float a, float b, float c,
      float d)
  {
    static_cast<float4 *>(dst)[o] = kCols ? make_float4(a, c, b, d) : make_float4(a, b, c, d);
  }
};

template <> struct Layout<LOLA_STORE_F32Q> : QuadF32Layout<LOLA_F32Q_COLS> {};

/* FP16 quads: four halves per pixel, the taps or (LOLA_QUAD_TERMS) the
 * bilinear terms, in the slots (00, 10, 01, 11), or with COLS in the order
 * (00, 01, 10, 11).  fetch returns them by slot name. */
template <bool COLS> struct QuadF16Layout {
  static constexpr bool kTex = false;
  static constexpr bool kMixed = false;
  static constexpr bool kCols = COLS;
  typedef uint2 Elem;
  static constexpr bool kQuad = true;
  static constexpr bool kDiff = LOLA_QUAD_TERMS;
  __device__ static __forceinline__ void fetch(const void *img, uint32_t idx, int,
      float &p00, float &p10, float &p01, float &p11)
  {
    const uint2 q = __ldg(static_cast<const uint2 *>(img) + idx);
    __half2 lo, hi;
    lo = *reinterpret_cast<const __half2 *>(&q.x);
    hi = *reinterpret_cast<const __half2 *>(&q.y);
    const float2 a = __half22float2(lo);
    const float2 b = __half22float2(hi);
    p00 = a.x;
    p10 = COLS ? b.x : a.y;
    p01 = COLS ? a.y : b.x;
    p11 = b.y;
  }
  __device__ static __forceinline__ void store(void *dst, size_t o, float a, float b, float c,
      float d)
  {
    const float4 t = LOLA_QUAD_TERMS ? bilinearTerms(a, b, c, d) : make_float4(a, b, c, d);
    const __half2 lo = COLS ? __floats2half2_rn(t.x, t.z) : __floats2half2_rn(t.x, t.y);
    const __half2 hi = COLS ? __floats2half2_rn(t.y, t.w) : __floats2half2_rn(t.z, t.w);
    uint2 q;
    q.x = *reinterpret_cast<const uint32_t *>(&lo);
    q.y = *reinterpret_cast<const uint32_t *>(&hi);
    static_cast<uint2 *>(dst)[o] = q;
  }
};

template <> struct Layout<LOLA_STORE_F16Q> : QuadF16Layout<false> {};

template <> struct Layout<LOLA_STORE_BF16Q> {
  static constexpr bool kTex = false;
  static constexpr bool kMixed = false;
  static constexpr bool kCols = false;
  typedef uint2 Elem;
  static constexpr bool kQuad = true;
  static constexpr bool kDiff = LOLA_QUAD_TERMS;
  __device__ static __forceinline__ void fetch(const void *img, uint32_t idx, int,
      float &p00, float &p10, float &p01, float &p11)
  {
    const uint2 q = __ldg(static_cast<const uint2 *>(img) + idx);
    p00 = bf16LoToFloat(q.x);
    p10 = bf16HiToFloat(q.x);
    p01 = bf16LoToFloat(q.y);
    p11 = bf16HiToFloat(q.y);
  }
  __device__ static __forceinline__ void store(void *dst, size_t o, float a, float b, float c,
      float d)
  {
    const float4 t = LOLA_QUAD_TERMS ? bilinearTerms(a, b, c, d) : make_float4(a, b, c, d);
    const __nv_bfloat162 lo = __floats2bfloat162_rn(t.x, t.y);
    const __nv_bfloat162 hi = __floats2bfloat162_rn(t.z, t.w);
    uint2 q;
    q.x = *reinterpret_cast<const uint32_t *>(&lo);
    q.y = *reinterpret_cast<const uint32_t *>(&hi);
    static_cast<uint2 *>(dst)[o] = q;
  }
};


/* Texture layouts: the stored image is a 2D texture with border addressing;
 * tld4 (tex2Dgather) returns the 2x2 texels that bilinear filtering at
 * (c_x, c_y) would use, texels floor(c - 0.5) and floor(c - 0.5) + 1, as
 * exact values (no filtering; FP16 is widened exactly).  Component order is
 * (i, j+1), (i+1, j+1), (i+1, j), (i, j). */
template <> struct Layout<LOLA_STORE_TEX32> {
  static constexpr bool kTex = true;
  static constexpr bool kMixed = false;
  static constexpr bool kCols = false;
  typedef float Elem;
  static constexpr bool kQuad = false;
  static constexpr bool kDiff = false;
  __device__ static __forceinline__ void store(void *dst, size_t o, float a, float, float, float)
  {
    static_cast<float *>(dst)[o] = a;
  }
};

template <> struct Layout<LOLA_STORE_TEX16> {
  static constexpr bool kTex = true;
  static constexpr bool kMixed = false;
  static constexpr bool kCols = false;
  typedef __half Elem;
  static constexpr bool kQuad = false;
  static constexpr bool kDiff = false;
  __device__ static __forceinline__ void store(void *dst, size_t o, float a, float, float, float)
  {
    static_cast<__half *>(dst)[o] = __float2half_rn(a);
  }
};

__device__ __forceinline__ void texTaps(unsigned long long tex, float cx, float cy, float &p00,
    float &p10, float &p01, float &p11)
{
  const float4 g = tex2Dgather<float4>((cudaTextureObject_t)tex, cx, cy, 0);
  p00 = g.w;
  p10 = g.z;
  p01 = g.x;
  p11 = g.y;
}


/* Mixed layouts: the 2x2 quads of the F16Q / F32Q layouts, also bound as an
 * RGBA texture (one texel = one quad).  Voxels whose bit is set in
 * LOLA_MIXED_TEX_MASK (lolacuda_internal.h) fetch their quad through the
 * texture unit (a point fetch, widened to FP32 there), the others through the
 * load path, so both gather pipes work in parallel. */

template <> struct Layout<LOLA_STORE_F16QX> : QuadF16Layout<LOLA_F16QX_COLS> {
  static constexpr bool kMixed = true;
};

template <> struct Layout<LOLA_STORE_F32QX> : QuadF32Layout<LOLA_F32QX_COLS> {
  static constexpr bool kMixed = true;
};

/* One texel of a mixed layout's quad texture: the taps (p00, p10, p01, p11)
   by name (COLS: the texel holds them column by column), or with RAW the
   texel's components in their stored order. */
template <bool COLS, bool RAW = false>
__device__ __forceinline__ void texQuad(unsigned long long tex, float cx, float cy, float &p00,
    float &p10, float &p01, float &p11)
{
  const float4 q = tex2D<float4>((cudaTextureObject_t)tex, cx, cy);
  p00 = q.x;
  p10 = (COLS && !RAW) ? q.z : q.y;
  p01 = (COLS && !RAW) ? q.y : q.z;
  p11 = q.w;
}

/* One texel of a mixed layout's quad texture by its integer pixel index in
   the ring slot (LOLA_MIXED_TEX_LINEAR: a linear texture over the slot), in
   the order texQuad gives. */
template <bool COLS, bool RAW = false>
__device__ __forceinline__ void texQuadLinear(unsigned long long tex, uint32_t idx, float &p00,
    float &p10, float &p01, float &p11)
{
  const float4 q = tex1Dfetch<float4>((cudaTextureObject_t)tex, (int)idx);
  p00 = q.x;
  p10 = (COLS && !RAW) ? q.z : q.y;
  p01 = (COLS && !RAW) ? q.y : q.z;
  p11 = q.w;
}

/* Texel index of a projection's first stored pixel within its linear
   texture: 0 where each ring slot has a texture of its own (the pass kernel's
   geometry), the slot's offset where one texture spans a job's slots (the
   batched pass's SlotGeom, bp_batch.cuh). */
template <class A> __device__ __forceinline__ uint32_t texIndexBase(const A &) { return 0u; }

/* ---- packing: FP32 detector image -> zero-padded stored layout ------------- */

struct PackArgs {
  const float *src;
  size_t srcStride;   /* floats between consecutive source images */
  void *ring;
  size_t slotElems;
  int slot0;
  int width, height, margin, pitch, rows;
  unsigned long long surf[LOLA_MAX_BATCH];  /* per ring slot, or 0 (LolaStoreDesc) */
};

/* Copies a stored pixel into a texture layout's CUDA array as well. */
template <class E>
__device__ __forceinline__ void surfStore(unsigned long long surf, E e, int x, int y)
{
  surf2Dwrite(e, (cudaSurfaceObject_t)surf, x * (int)sizeof(E), y);
}
__device__ __forceinline__ void surfStore(unsigned long long surf, __half e, int x, int y)
{
  surf2Dwrite(__half_as_ushort(e), (cudaSurfaceObject_t)surf, x * 2, y);
}

template <int S>
__global__ void __launch_bounds__(256) packKernel(const PackArgs a)
{
  const int pu = blockIdx.x * 32 + threadIdx.x;
  const int pv = blockIdx.y * 8 + threadIdx.y;
  const int p = blockIdx.z;
  if (pu >= a.pitch || pv >= a.rows)
    return;
  const float *img = a.src + (size_t)p * a.srcStride;
  const int u = pu - a.margin, v = pv - a.margin;
  auto px = [&](int uu, int vv) -> float {
    return (uu >= 0 && uu < a.width && vv >= 0 && vv < a.height)
               ? __ldg(img + (size_t)vv * a.width + uu)
               : 0.0f;
  };
  const size_t o = (size_t)(a.slot0 + p) * a.slotElems + (size_t)pv * a.pitch + pu;
  if constexpr (Layout<S>::kQuad)
    Layout<S>::store(a.ring, o, px(u, v), px(u + 1, v), px(u, v + 1), px(u + 1, v + 1));
  else
    Layout<S>::store(a.ring, o, px(u, v), 0.f, 0.f, 0.f);
  if constexpr (Layout<S>::kTex || Layout<S>::kMixed) {
    const unsigned long long surf = a.surf[a.slot0 + p];
    if (surf)  /* the same element, read back from this thread's own store */
      surfStore(surf, static_cast<const typename Layout<S>::Elem *>(a.ring)[o], pu, pv);
  }
}

/* ---- backprojection pass ---------------------------------------------------- */

struct PassArgs {
  const void *ring;
  size_t slotBytes;
  float *volume;
  unsigned long long *tileCounters;  /* LOLA_COUNTER_SPREAD x LOLA_TILE_COUNTERS, or null */
  int width, height, margin, pitch, rows;
  unsigned long long tex[LOLA_MAX_BATCH];  /* texture layouts: object per ring slot */
};

/* Voxel k of a thread's column in accumulators held as pairs (k, k+1) =
 * (.x, .y); k is a compile-time constant after unrolling. */
__device__ __forceinline__ float &voxel(float2 *v, int k)
{
  return (k & 1) ? v[k >> 1].y : v[k >> 1].x;
}

/* Applies one projection to the thread's VPT voxels, one voxel at a time. */
/* A (PassArgs, or the batched pass's ImageGeom) supplies width, height,
 * margin, pitch and rows of the stored image.  TEXMASK: the voxels a mixed
 * layout fetches through the texture unit (the values are the same either
 * way: the FP16 point fetch widens exactly). */
template <int S, int VPT, bool KAHAN, bool CLAMP, class A,
    unsigned TEXMASK = LOLA_MIXED_TEX_MASK>
__device__ __forceinline__ void applyProjection(const TileProj &tp, const void *img,
    unsigned long long tex, const A &a, float fi, float fj, float2 (&acc)[VPT / 2],
    float2 (&comp)[VPT / 2])
{
  const float pitchF = (float)a.pitch;
  /* index = (ty + M) * pitch + (tx + M), formed as 2^23 + index in FP32 */
  const float biasF = 8388608.0f + (float)(a.margin * a.pitch + a.margin);
  const uint32_t maxIdx = Layout<S>::kQuad ? (uint32_t)(a.pitch * a.rows - 1)
                                           : (uint32_t)(a.pitch * a.rows - a.pitch - 2);
  const float wLim = (float)(a.width + 1);
  const float hLim = (float)(a.height + 1);

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
    float ix = fmaf(u, r, tp.cu);
    float iy = fmaf(v, r, tp.cv);
    if (CLAMP) {
      /* outside [-2, W+1] every tap is in the zero margin, as in LolaBunny */
      ix = fminf(fmaxf(ix, -2.0f), wLim);
      iy = fminf(fmaxf(iy, -2.0f), hLim);
    }
    const float tx = truncf(ix);  /* (int)x of src/LolaBunny.c:21 */
    const float ty = truncf(iy);
    const float ax = ix - tx;
    const float ay = iy - ty;
    float p00, p10, p01, p11;
    if constexpr (Layout<S>::kTex) {
      /* texel (tx, ty) of the detector sits at (tx + M, ty + M) of the padded
         texture; gathering at that + 1 selects it as the lower-left tap */
      const float off = (float)a.margin + 1.0f;
      texTaps(tex, tx + off, ty + off, p00, p10, p01, p11);
    } else if (Layout<S>::kMixed && ((TEXMASK >> k) & 1u)) {
      if (LOLA_MIXED_TEX_LINEAR) {
        /* the texel at the load path's index; any index past the slot reads 0 */
        const uint32_t idx = __float_as_uint(fmaf(ty, pitchF, tx + biasF)) - 0x4B000000u;
        texQuadLinear<Layout<S>::kCols>(tex, idx + texIndexBase(a), p00, p10, p01, p11);
      } else {
        /* point fetch of texel (tx + M, ty + M): any coordinate inside it works */
        const float off = (float)a.margin + 0.5f;
        texQuad<Layout<S>::kCols>(tex, tx + off, ty + off, p00, p10, p01, p11);
      }
    } else {
      uint32_t idx = __float_as_uint(fmaf(ty, pitchF, tx + biasF)) - 0x4B000000u;
      idx = min(idx, maxIdx);  /* memory-safety net; never active on valid input */
      Layout<S>::fetch(img, idx, a.pitch, p00, p10, p01, p11);
    }
    const float val = bilinear<Layout<S>::kDiff>(ax, ay, p00, p10, p01, p11);
    float term = val * (r * r);
    if (CLAMP)
      term = (val == 0.0f) ? 0.0f : term;  /* w = 0 would give 0 * inf */
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

/* Applies one projection to the thread's VPT voxels two at a time: voxels
 * (k, k+1) go through every FP32 operation together as one packed f32x2
 * instruction (sm_100 family), half the issue slots of the scalar code, with
 * the same operations per voxel except two: w, u and v step by two voxels from
 * the first pair, and the floor comes from a round-down add.  Only for tiles
 * with tp.pos (footprint inside the zero margin, coordinates >= 0), where C
 * truncation is floor: floor(ix) is read from ix + 2^23 rounded down (the FMA
 * pipe) instead of a float-to-integer conversion (the slower XU pipe), and the
 * stored index is formed from the same sums.
 *
 * The tile's pixel offsets (cu, cv) are integers, so floor(ix) = cu + floor(q)
 * with q = u'/w small (and of either sign): its fraction is exact and more
 * precise than one taken of ix itself.  kxc = 2^23 + the stored index of pixel
 * (cu, cv) in the image read (an integer); xm = kxc + floor(q) is the
 * round-down sum q + kxc, exact because it lies in [2^23, 2^24) (it is 2^23 +
 * the index of pixel (floor(ix), cv), and every such index of a paired tile is
 * >= 0).  Likewise ym = 2^23 + cv + floor(qv) from qv + 2^23 + cv (floor(iy)
 * >= 0), and the stored index of the voxel's pixel is
 * xm + floor(qv) * rowPitch.
 * fetch(k, idxf, nqx, nqy, p00, p10, p01, p11) reads voxel k's taps given
 * idxf = 2^23 + its pixel index, and nqx = cu - floor(ix), nqy = cv - floor(iy)
 * (integers).  Voxel pairs whose bits are both set in COLSMASK get their taps
 * (or terms) column by column, (00, 01, 10, 11), and each voxel is
 * interpolated in x with one packed FMA over its two column pairs (the same
 * roundings as the pairwise form below). */
template <int VPT, bool KAHAN, bool DIFF, unsigned COLSMASK, class Fetch>
__device__ __forceinline__ void pairedUpdate(const TileProj &tp, float fi, float fj, float kxc,
    float rowPitch, Fetch fetch, float2 (&acc)[VPT / 2], float2 (&comp)[VPT / 2])
{
  const float magic = 8388608.0f;  /* 2^23 */
  const float2 KX = make_float2(kxc, kxc);
  const float2 KY = make_float2(magic + tp.cv, magic + tp.cv);
  const float2 npitch = make_float2(-rowPitch, -rowPitch);
  const float2 neg1 = make_float2(-1.0f, -1.0f);

  const float ut = fmaf(fj, tp.su[1], fmaf(fi, tp.su[0], tp.u0));
  const float vt = fmaf(fj, tp.sv[1], fmaf(fi, tp.sv[0], tp.v0));
  const float wt = fmaf(fj, tp.sw[1], fmaf(fi, tp.sw[0], tp.w0));
  /* w, u and v step by two voxels from the first pair: one packed add per
     coordinate and pair (two scalar FMAs from the pair's own k measured 6 %
     slower for the issue slots they take) */
  float2 U = make_float2(ut, ut + tp.su[2]);
  float2 V = make_float2(vt, vt + tp.sv[2]);
  float2 W = make_float2(wt, wt + tp.sw[2]);
  const float2 dU = make_float2(2.0f * tp.su[2], 2.0f * tp.su[2]);
  const float2 dV = make_float2(2.0f * tp.sv[2], 2.0f * tp.sv[2]);
  const float2 dW = make_float2(2.0f * tp.sw[2], 2.0f * tp.sw[2]);
#pragma unroll
  for (int j = 0; j < VPT / 2; ++j) {
    if (j > 0) {
      U = __fadd2_rn(U, dU);
      V = __fadd2_rn(V, dV);
      W = __fadd2_rn(W, dW);
    }
    const float2 R = make_float2(rcpApprox(W.x), rcpApprox(W.y));
    const float2 Q = __fmul2_rn(U, R);    /* ix - cu */
    const float2 QV = __fmul2_rn(V, R);   /* iy - cv */
    const float2 XM = __fadd2_rd(Q, KX);  /* kxc + floor(q), exact */
    const float2 YM = __fadd2_rd(QV, KY); /* 2^23 + cv + floor(qv), exact */
    const float2 TX = __ffma2_rn(XM, neg1, KX);  /* -floor(q), exact */
    const float2 TY = __ffma2_rn(YM, neg1, KY);  /* -floor(qv) */
    const float2 AX = __fadd2_rn(Q, TX);  /* ix - floor(ix), exact */
    const float2 AY = __fadd2_rn(QV, TY);
    const float2 IDX = __ffma2_rn(TY, npitch, XM);  /* 2^23 + pixel index */
    float2 VAL;
    if (((COLSMASK >> (2 * j)) & 3u) == 3u) {
      float val[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float q0, q1, q2, q3;
        fetch(2 * j + h, h ? IDX.y : IDX.x, h ? TX.y : TX.x, h ? TY.y : TY.x, q0, q1, q2, q3);
        const float2 c0 = make_float2(q0, q1), c1 = make_float2(q2, q3);
        const float ax = h ? AX.y : AX.x, ay = h ? AY.y : AY.x;
        if (DIFF) {
          /* terms (t0, t2), (t1, t3): the rows' x interpolants (b, c) */
          const float2 bc = __ffma2_rn(make_float2(ax, ax), c1, c0);
          val[h] = fmaf(ay, bc.y, bc.x);
        } else {
          /* (p10 - p00, p11 - p01), then the rows' x interpolants (b, t) */
          const float2 bt = __ffma2_rn(make_float2(ax, ax), __ffma2_rn(c0, neg1, c1), c0);
          val[h] = fmaf(ay, fmaf(bt.x, -1.0f, bt.y), bt.x);
        }
      }
      VAL = make_float2(val[0], val[1]);
    } else {
      /* pairwise: the two voxels' taps (or terms) packed slot by slot */
      float p00[2], p10[2], p01[2], p11[2];
#pragma unroll
      for (int h = 0; h < 2; ++h)
        fetch(2 * j + h, h ? IDX.y : IDX.x, h ? TX.y : TX.x, h ? TY.y : TY.x, p00[h], p10[h],
            p01[h], p11[h]);
      const float2 P00 = make_float2(p00[0], p00[1]), P10 = make_float2(p10[0], p10[1]);
      const float2 P01 = make_float2(p01[0], p01[1]), P11 = make_float2(p11[0], p11[1]);
      if (DIFF) {  /* terms: p00, p10 - p00, p01 - p00, p11 - p01 - p10 + p00 */
        const float2 B = __ffma2_rn(AX, P10, P00);
        const float2 C = __ffma2_rn(AX, P11, P01);
        VAL = __ffma2_rn(AY, C, B);
      } else {
        const float2 B = __ffma2_rn(AX, __ffma2_rn(P00, neg1, P10), P00);
        const float2 T = __ffma2_rn(AX, __ffma2_rn(P01, neg1, P11), P01);
        VAL = __ffma2_rn(AY, __ffma2_rn(B, neg1, T), B);
      }
    }
    const float2 RR = __fmul2_rn(R, R);
    if (KAHAN) {
      const float2 term = __fmul2_rn(VAL, RR);
      const float2 y = __ffma2_rn(comp[j], neg1, term);
      const float2 s = __fadd2_rn(acc[j], y);
      comp[j] = __ffma2_rn(y, neg1, __ffma2_rn(acc[j], neg1, s));
      acc[j] = s;
    } else {
      acc[j] = __ffma2_rn(VAL, RR, acc[j]);
    }
  }
}

/* Texture mask of a mixed layout in the pass kernel. */
template <int S> struct PassTexMask {
  static constexpr unsigned kValue = S == LOLA_STORE_F16QX ? LOLA_F16QX_TEX_MASK
                                     : !Layout<S>::kCols   ? LOLA_MIXED_TEX_MASK
                                                           : LOLA_F32QX_COLS_TEX_MASK;
};

/* The paired update on the stored ring (loads, texture or both).  Voxels
 * whose fetch delivers column pairs (every voxel of a column-ordered load
 * layout; the texture voxels of a column-ordered mixed layout) are
 * interpolated per voxel; the rest pairwise. */
template <int S, int VPT, bool KAHAN, class A, unsigned TEXMASK = LOLA_MIXED_TEX_MASK>
__device__ __forceinline__ void applyPairs(const TileProj &tp, const void *img,
    unsigned long long tex, const A &a, float fi, float fj, float2 (&acc)[VPT / 2],
    float2 (&comp)[VPT / 2])
{
  const uint32_t maxIdx = Layout<S>::kQuad ? (uint32_t)(a.pitch * a.rows - 1)
                                           : (uint32_t)(a.pitch * a.rows - a.pitch - 2);
  const int pitch = a.pitch;
  const float margin = (float)a.margin;
  /* 2^23 + stored index of pixel (cu, cv): (cv + M) * pitch + (cu + M) */
  const float kxc = fmaf(tp.cv, (float)a.pitch,
      8388608.0f + (float)(a.margin * a.pitch + a.margin) + tp.cu);
  /* texture coordinate of pixel (cu, cv): +1 selects it as the lower-left tap
     of a tld4 gather, +0.5 is the centre of its texel for a point fetch; the
     voxel's coordinate is that minus (cu - floor(ix)), exact (integers and
     halves) */
  const float toff = margin + (Layout<S>::kTex ? 1.0f : 0.5f);
  const float tcx = tp.cu + toff, tcy = tp.cv + toff;
  /* voxels whose fetch returns the stored components in stored order: all
     of a column-ordered load layout; of a mixed one, the texture voxels of
     pairs read wholly through the texture */
  constexpr unsigned kTexPairs = TEXMASK & (TEXMASK >> 1) & 0x55555555u;
  constexpr unsigned COLSMASK = !Layout<S>::kCols ? 0u
                                : Layout<S>::kMixed ? (kTexPairs | (kTexPairs << 1))
                                                    : 0xffffffffu;
  auto fetch = [&](int k, float idxf, float nqx, float nqy, float &p00, float &p10, float &p01,
                   float &p11) {
    if constexpr (Layout<S>::kTex) {
      texTaps(tex, tcx - nqx, tcy - nqy, p00, p10, p01, p11);
    } else {
      if (Layout<S>::kMixed && ((TEXMASK >> k) & 1u)) {
        if (LOLA_MIXED_TEX_LINEAR) {
          /* an index past the slot reads 0: no clamp needed for memory safety */
          const uint32_t idx = __float_as_uint(idxf) - 0x4B000000u + texIndexBase(a);
          if ((COLSMASK >> k) & 1u)
            texQuadLinear<Layout<S>::kCols, true>(tex, idx, p00, p10, p01, p11);
          else
            texQuadLinear<Layout<S>::kCols>(tex, idx, p00, p10, p01, p11);
        } else if ((COLSMASK >> k) & 1u) {
          texQuad<Layout<S>::kCols, true>(tex, tcx - nqx, tcy - nqy, p00, p10, p01, p11);
        } else {
          texQuad<Layout<S>::kCols>(tex, tcx - nqx, tcy - nqy, p00, p10, p01, p11);
        }
      } else {
        uint32_t idx = __float_as_uint(idxf) - 0x4B000000u;
        idx = min(idx, maxIdx);  /* memory-safety net; never active on valid input */
        if constexpr (Layout<S>::kCols && !Layout<S>::kMixed)
          Layout<S>::fetchRaw(img, idx, pitch, p00, p10, p01, p11);
        else
          Layout<S>::fetch(img, idx, pitch, p00, p10, p01, p11);
      }
    }
  };
  pairedUpdate<VPT, KAHAN, Layout<S>::kDiff, COLSMASK>(tp, fi, fj, kxc, (float)a.pitch, fetch,
      acc, comp);
}

/* Lane -> voxel within a warp's TX x (32 / TX) patch of the xy plane.  The
 * texture unit (and the L1 for quad loads) serves a warp's fetch in 8-lane
 * quarters, one data-stage wavefront for each detector row (or 128-byte
 * window) that a quarter's eight texels touch.  The voxels of one quarter
 * project to the same detector row unless their depths along the ray
 * differ (the magnification then moves them up to about a pixel per 8
 * voxels at the detector's top and bottom), so GROUPS gives each quarter a
 * 4 x 2 patch instead of a row of 8 voxels: its depth spread is
 * 3|sin a| + |cos a| voxels instead of 7|sin a| (a: the angle between the
 * ray and the y axis), and it straddles a row boundary about half as often
 * (f16qx: 1.63 -> 1.47 wavefronts per quarter at N=640, 1775 -> 1868 GUPS
 * at N=1024, bit-identical volumes; lolaStorePitch's row skew then takes it
 * to 1.19).  Without GROUPS the warp's lanes run along x row by row. */
#ifndef LOLA_LANE_GROUPS
#define LOLA_LANE_GROUPS -1  /* -1: per storage (LaneGroups); 0: never; 1: always */
#endif
template <int S> struct LaneGroups {
  /* measured at N=1024 on GB300 (the other layouts within +-0.8 % either
     way, so they keep rows of 8): f16qx +5 %, f32q +2.6 % */
  static constexpr bool kValue =
      LOLA_LANE_GROUPS < 0 ? (S == LOLA_STORE_F16QX || S == LOLA_STORE_F32Q)
                           : LOLA_LANE_GROUPS != 0;
};

template <int TX, bool GROUPS>
__device__ __forceinline__ void laneVoxel(int lane, int warp, int &tx, int &ty)
{
  if (GROUPS && TX == 8) {
    const int q = lane >> 3, j = lane & 7;  /* quarter, lane in the quarter */
    tx = (q & 1) * 4 + (j & 3);
    ty = warp * 4 + (q >> 1) * 2 + (j >> 2);
  } else {
    tx = lane % TX;
    ty = warp * (32 / TX) + lane / TX;
  }
}

/* Per-(tile, projection) setup shared by the pass kernels: the FP64 tile
 * origin (phase A, one thread per projection) and the footprint and mode from
 * the 8 tile corners (phase B, 8 lanes per projection).  Ends with the block
 * synchronised and sp[0 .. count) complete.  nthreads is a multiple of 32. */
/* 1: the setup's divisions (the offsets cu, cv and the footprint corners)
   use the fast approximate division: cu and cv may be any nearby integers,
   and the footprint carries half a pixel of slack against rounding */
#ifndef LOLA_SETUP_FASTDIV
#define LOLA_SETUP_FASTDIV 1
#endif
__device__ __forceinline__ float setupDiv(float a, float b)
{
#if LOLA_SETUP_FASTDIV
  return __fdividef(a, b);
#else
  return a / b;
#endif
}

/* Geometry of one volume and its stored projections, as setupTile needs it. */
struct TileGeom {
  int N;          /* volume edge */
  int zEnd;       /* end of the slab held */
  float voxelSize, originIndex;
  int width, height, margin;
};

template <int ROWS, int VPT, int TX = 32>
__device__ __forceinline__ void setupTileGeom(const LolaPassProj *proj, int count,
    const TileGeom &g, TileProj *sp, int tid, int nthreads, int x0, int y0, int z0)
{
  const int N = g.N;
  /* -- setup A: FP64 projection of the tile origin, one thread per view -- */
  if (tid < count) {
    const LolaPassProj &pp = proj[tid];
    const double *m = pp.a;
    const double vs = (double)g.voxelSize, o = (double)g.originIndex;
    const double X = o + (double)x0 * vs, Y = o + (double)y0 * vs, Z = o + (double)z0 * vs;
    const double U = m[0] * X + m[3] * Y + m[6] * Z + m[9];
    const double V = m[1] * X + m[4] * Y + m[7] * Z + m[10];
    const double Wd = m[2] * X + m[5] * Y + m[8] * Z + m[11];
    /* integer pixel offsets: floor(ix) = cu + floor(u'/w) on the paired path.
       They are kept within one detector size of the padded image: where the
       tile origin lies near the source plane (w ~ 0) its projection is huge,
       and so would be the cancellation in u' = u - cu w for the tile's other
       voxels.  Tiles that project inside (every fast tile) are unaffected. */
    const float Wf = (float)g.width, Hf = (float)g.height, Mf = (float)g.margin;
    float cu = rintf(setupDiv((float)U, (float)Wd));
    float cv = rintf(setupDiv((float)V, (float)Wd));
    cu = isfinite(cu) ? fminf(fmaxf(cu, -(Wf + Mf)), 2.0f * Wf + Mf) : 0.0f;
    cv = isfinite(cv) ? fminf(fmaxf(cv, -(Hf + Mf)), 2.0f * Hf + Mf) : 0.0f;
    TileProj tp;
    tp.cu = cu;
    tp.cv = cv;
    tp.u0 = (float)(U - (double)tp.cu * Wd);
    tp.v0 = (float)(V - (double)tp.cv * Wd);
    tp.w0 = (float)Wd;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      tp.sw[ax] = pp.step[ax][2];
      tp.su[ax] = fmaf(-tp.cu, pp.step[ax][2], pp.step[ax][0]);
      tp.sv[ax] = fmaf(-tp.cv, pp.step[ax][2], pp.step[ax][1]);
    }
    tp.mode = MODE_SLOW;
    tp.pos = 0;
    tp.slot = pp.slot;
    sp[tid] = tp;
  }
  __syncthreads();

  /* -- setup B: footprint of the tile from its 8 corners, 8 lanes per view -- */
  /* tile: TX x (32 ROWS / TX) x VPT voxels */
  const int ex = min(TX, N - x0) - 1, ey = min(32 * ROWS / TX, N - y0) - 1;
  const int ez = min(VPT, g.zEnd - z0) - 1;
  for (int base = 0; base < 8 * count; base += nthreads) {
    const int t = base + tid;
    const bool active = t < 8 * count;
    const int p = active ? (t >> 3) : 0;
    const int c = t & 7;
    const TileProj &tp = sp[p];
    const float ox = (c & 1) ? (float)ex : 0.0f;
    const float oy = (c & 2) ? (float)ey : 0.0f;
    const float oz = (c & 4) ? (float)ez : 0.0f;
    const float u = tp.u0 + ox * tp.su[0] + oy * tp.su[1] + oz * tp.su[2];
    const float v = tp.v0 + ox * tp.sv[0] + oy * tp.sv[1] + oz * tp.sv[2];
    const float w = tp.w0 + ox * tp.sw[0] + oy * tp.sw[1] + oz * tp.sw[2];
    const float ix = tp.cu + setupDiv(u, w), iy = tp.cv + setupDiv(v, w);
    int ok = (w > 0.0f) && isfinite(ix) && isfinite(iy);
    float mnx = ix, mxx = ix, mny = iy, mxy = iy;
#pragma unroll
    for (int s = 1; s < 8; s <<= 1) {
      mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, s));
      mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, s));
      mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, s));
      mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, s));
      ok &= __shfl_xor_sync(0xffffffffu, ok, s);
    }
    if (active && c == 0) {
      const float slack = 0.5f;
      const float W = (float)g.width, H = (float)g.height, M = (float)g.margin;
      int mode;
      if (!ok)
        mode = MODE_SLOW;
      else if (mxx + slack <= -2.0f || mnx - slack >= W || mxy + slack <= -2.0f ||
               mny - slack >= H)
        mode = MODE_SKIP;
      else if (mnx - slack >= 1.0f - M && mxx + slack <= W + M - 3.0f &&
               mny - slack >= 1.0f - M && mxy + slack <= H + M - 3.0f)
        mode = MODE_FAST;
      else
        mode = MODE_SLOW;
      sp[p].mode = mode;
      /* C truncation equals floor where every coordinate is >= 0 */
      sp[p].pos = (mode == MODE_FAST) && mnx - slack >= 0.0f && mny - slack >= 0.0f;
      sp[p].fx0 = mnx - slack;
      sp[p].fx1 = mxx + slack;
      sp[p].fy0 = mny - slack;
      sp[p].fy1 = mxy + slack;
    }
  }
  __syncthreads();

}

template <int ROWS, int VPT, int TX = 32>
__device__ __forceinline__ void setupTile(const LolaPassParams &P, const PassArgs &a,
    TileProj *sp, int tid, int nthreads, int x0, int y0, int z0)
{
  TileGeom g;
  g.N = P.N;
  g.zEnd = P.zEnd;
  g.voxelSize = P.voxelSize;
  g.originIndex = P.originIndex;
  g.width = a.width;
  g.height = a.height;
  g.margin = a.margin;
#if LOLA_PROJ_DEVICE
  const LolaPassProj *proj = P.projDevice != nullptr ? P.projDevice : P.proj;
#else
  const LolaPassProj *proj = P.proj;
#endif
  setupTileGeom<ROWS, VPT, TX>(proj, P.count, g, sp, tid, nthreads, x0, y0, z0);
}

/* Resident blocks per SM requested from the register allocator.  The pass is
 * bound by the latency of its gathers, so occupancy pays up to the point where
 * registers spill.  Measured on GB300 at N=1024 (496 projections, 1248x960):
 *  - 8 voxels per thread: 40 warps per SM (48 registers; the paired path at
 *    48 warps spilled and ran 5-13 % slower, 36 warps 1-5 % slower);
 *  - 16 voxels per thread: 28 warps for the layouts that widen 16-bit taps
 *    (72 registers: f16qx 1337 GUPS vs 1286 at 32 warps and 1309 at 36) and
 *    36 warps for FP32 ones (56 registers: f32 1151 GUPS vs 1115 at 32 and
 *    1108 at 40).
 * LOLA_MIN_BLOCKS overrides it at build time (0 = the compiler's choice). */
template <int S, int VPT, int ROWS> struct MinBlocks {
  static constexpr bool kWide32 = S == LOLA_STORE_F32 || S == LOLA_STORE_F32Q ||
                                  S == LOLA_STORE_TEX32 || S == LOLA_STORE_F32QX;
  /* f16qx with every voxel by texture widens nothing itself: 32 warps (64
     registers) measured 1781 vs 1767 GUPS at 28 and 1668 at 24 */
  static constexpr bool kAllTex = S == LOLA_STORE_F16QX && LOLA_F16QX_TEX_MASK == 0xFFFFu;
  static constexpr int kWarps = (VPT <= 8) ? 40 : (kWide32 ? 36 : (kAllTex ? 32 : 28));
  static constexpr int kValue = kWarps / ROWS;
};
#ifdef LOLA_MIN_BLOCKS
#define LOLA_PASS_MIN_BLOCKS(S, VPT, ROWS) LOLA_MIN_BLOCKS
#else
#define LOLA_PASS_MIN_BLOCKS(S, VPT, ROWS) (MinBlocks<S, VPT, ROWS>::kValue)
#endif

template <int S, int VPT, int ROWS, bool KAHAN, unsigned TEXMASK = PassTexMask<S>::kValue>
__global__ void __launch_bounds__(32 * ROWS, LOLA_PASS_MIN_BLOCKS(S, VPT, ROWS))
    passKernel(const PassArgs a, const LolaPassParams P)
{
  /* the per-projection setup of the tile: P.count entries (dynamic shared
     memory, so that a short pass reserves only what it uses) */
  extern __shared__ __align__(16) unsigned char passShared[];
  TileProj *sp = reinterpret_cast<TileProj *>(passShared);
  const int N = P.N;
  /* a warp covers TX x (32 / TX) voxels of the xy plane */
  constexpr int TX = LOLA_WARP_X, TY = 32 * ROWS / TX;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = P.zBegin + blockIdx.z * VPT;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const int count = P.count;

  /* the thread's voxel column.  The plan holds only the slab z in
     [zBegin, zEnd); the column address is formed again for the store rather
     than kept live across the pass.  For the FP32 layouts the column's loads
     are issued before the setup, so that their latency overlaps the setup's
     (f32 +1.3 %, f32q +0.9 % at N=1024 on GB300); for the 16-bit layouts,
     whose registers are fuller, after it (f16qx 1 % faster that way) */
  int tx, ty;
  laneVoxel<TX, LaneGroups<S>::kValue>(threadIdx.x, threadIdx.y, tx, ty);
  const int x = x0 + tx, y = y0 + ty;
  const bool inXY = (x < N) && (y < N);
  const size_t slice = (size_t)N * (size_t)N;
  auto column = [&]() {
    return a.volume + ((size_t)(z0 - P.zBegin) * N + (size_t)(inXY ? y : 0)) * (size_t)N +
           (inXY ? x : 0);
  };
  float2 acc[VPT / 2], comp[VPT / 2];
  auto loadColumn = [&]() {
    const float *vcol = column();
#pragma unroll
    for (int k = 0; k < VPT; ++k) {
      voxel(acc, k) = (inXY && z0 + k < P.zEnd) ? vcol[k * slice] : 0.0f;
      voxel(comp, k) = 0.0f;
    }
  };
  constexpr bool kLoadsFirst = MinBlocks<S, VPT, ROWS>::kWide32;
  if (kLoadsFirst)
    loadColumn();

  setupTile<ROWS, VPT, TX>(P, a, sp, tid, 32 * ROWS, x0, y0, z0);
  if (!kLoadsFirst)
    loadColumn();

  if (a.tileCounters != nullptr && tid == 0) {
    const unsigned copy =
        (blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)) % LOLA_COUNTER_SPREAD;
    unsigned long long *counters = a.tileCounters + copy * LOLA_TILE_COUNTERS;
    unsigned long long nSkip = 0, nFast = 0, nSlow = 0, nPaired = 0;
    for (int p = 0; p < count; ++p) {
      const int m = sp[p].mode;
      nSkip += (m == MODE_SKIP);
      nFast += (m == MODE_FAST);
      nSlow += (m == MODE_SLOW);
      nPaired += (m == MODE_FAST && sp[p].pos && LOLA_PAIRED);
    }
    atomicAdd(counters + 0, nSkip);
    atomicAdd(counters + 1, nFast);
    atomicAdd(counters + 2, nSlow);
    atomicAdd(counters + 4, nPaired);
  }

  const float fi = (float)tx, fj = (float)ty;
  for (int p = 0; p < count; ++p) {
    const int mode = sp[p].mode;
    if (mode == MODE_SKIP)
      continue;
    const TileProj tp = sp[p];
    const void *img = static_cast<const char *>(a.ring) + (size_t)tp.slot * a.slotBytes;
    const unsigned long long tex =
        (Layout<S>::kTex || Layout<S>::kMixed) ? a.tex[tp.slot] : 0ull;
    constexpr unsigned kMask = TEXMASK;
    if (mode == MODE_FAST && tp.pos && LOLA_PAIRED)
      applyPairs<S, VPT, KAHAN, PassArgs, kMask>(tp, img, tex, a, fi, fj, acc, comp);
    else if (mode == MODE_FAST)
      applyProjection<S, VPT, KAHAN, false, PassArgs, kMask>(tp, img, tex, a, fi, fj, acc, comp);
    else
      applyProjection<S, VPT, KAHAN, true, PassArgs, kMask>(tp, img, tex, a, fi, fj, acc, comp);
  }
  float *vcol = column();
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    if (inXY && z0 + k < P.zEnd)
      vcol[k * slice] = KAHAN ? (voxel(acc, k) - voxel(comp, k)) : voxel(acc, k);
  }
}

/* ---- host-side launch helpers (instantiated per storage layout) ------------- */

template <int S>
int launchPack(const LolaStoreDesc *st, const float *src, size_t srcStride, void *ring, int slot0,
    int count, cudaStream_t stream)
{
  PackArgs a;
  a.src = src;
  a.srcStride = srcStride;
  a.ring = ring;
  a.slotElems = st->slotElems;
  a.slot0 = slot0;
  a.width = st->width;
  a.height = st->height;
  a.margin = st->margin;
  a.pitch = st->pitch;
  a.rows = st->rows;
  for (int i = 0; i < LOLA_MAX_BATCH; ++i)
    a.surf[i] = st->surfObjects[i];
  const dim3 block(32, 8);
  const dim3 grid((st->pitch + 31) / 32, (st->rows + 7) / 8, count);
  (void)cudaGetLastError();  /* report this launch's error, not an earlier one */
  packKernel<S><<<grid, block, 0, stream>>>(a);
  return (int)cudaGetLastError();
}

template <int S, int VPT, int ROWS, bool KAHAN>
int launchPassShape(const PassArgs &a, const LolaPassParams *P, cudaStream_t stream)
{
  const int N = P->N;
  const dim3 block(32, ROWS);
  const int nz = P->zEnd - P->zBegin;
  constexpr int TX = LOLA_WARP_X, TY = 32 * ROWS / TX;
  const dim3 grid((N + TX - 1) / TX, (N + TY - 1) / TY, (nz + VPT - 1) / VPT);
  const size_t smem = (size_t)P->count * sizeof(TileProj);
  (void)cudaGetLastError();
  passKernel<S, VPT, ROWS, KAHAN><<<grid, block, smem, stream>>>(a, *P);
  return (int)cudaGetLastError();
}

template <int S, bool KAHAN>
int launchPassAccum(const PassArgs &a, const LolaPassParams *P, cudaStream_t stream)
{
  const int vpt = P->voxelsPerThread, rows = P->rowsPerBlock;
  if (vpt == 8 && rows == 8) return launchPassShape<S, 8, 8, KAHAN>(a, P, stream);
  if (vpt == 8 && rows == 4) return launchPassShape<S, 8, 4, KAHAN>(a, P, stream);
  if (vpt == 16 && rows == 8) return launchPassShape<S, 16, 8, KAHAN>(a, P, stream);
  if (vpt == 16 && rows == 4) return launchPassShape<S, 16, 4, KAHAN>(a, P, stream);
  if (vpt == 4 && rows == 8) return launchPassShape<S, 4, 8, KAHAN>(a, P, stream);
  return (int)cudaErrorInvalidConfiguration;
}

inline void fillPassArgs(PassArgs &a, const LolaStoreDesc *st, const void *ring, float *volume,
    unsigned long long *counters)
{
  a.ring = ring;
  a.slotBytes = st->slotElems * (size_t)st->elemBytes;
  a.volume = volume;
  a.tileCounters = counters;
  a.width = st->width;
  a.height = st->height;
  a.margin = st->margin;
  a.pitch = st->pitch;
  a.rows = st->rows;
  for (int i = 0; i < LOLA_MAX_BATCH; ++i)
    a.tex[i] = st->texObjects[i];
}

template <int S>
int launchPass(const LolaStoreDesc *st, const LolaPassParams *P, const void *ring, float *volume,
    unsigned long long *counters, cudaStream_t stream)
{
  PassArgs a;
  fillPassArgs(a, st, ring, volume, counters);
  if (P->accumulation == LOLA_ACCUM_KAHAN)
    return launchPassAccum<S, true>(a, P, stream);
  return launchPassAccum<S, false>(a, P, stream);
}

} /* namespace lola */

#define LOLA_INSTANTIATE_STORAGE(S, NAME)                                                  \
  extern "C" int lolaLaunchPack_##NAME(const LolaStoreDesc *st, const float *src,          \
      size_t srcStride, void *ring, int slot0, int count, void *stream)                    \
  {                                                                                        \
    return lola::launchPack<S>(st, src, srcStride, ring, slot0, count,                     \
        static_cast<cudaStream_t>(stream));                                                \
  }                                                                                        \
  extern "C" int lolaLaunchPass_##NAME(const LolaStoreDesc *st, const LolaPassParams *P,   \
      const LolaStageDesc *sd, const void *ring, float *volume,                            \
      unsigned long long *counters, void *stream)                                          \
  {                                                                                        \
    if (sd != nullptr)                                                                     \
      return lola::launchStaged<S>(st, P, sd, ring, volume, counters,                      \
          static_cast<cudaStream_t>(stream));                                              \
    return lola::launchPass<S>(st, P, ring, volume, counters,                              \
        static_cast<cudaStream_t>(stream));                                                \
  }                                                                                        \
  extern "C" int lolaLaunchBatchPack_##NAME(const LolaBatchWave *w, void *stream)          \
  {                                                                                        \
    return lola::launchBatchPack<S>(w, static_cast<cudaStream_t>(stream));                 \
  }                                                                                        \
  extern "C" int lolaLaunchBatchPass_##NAME(const LolaBatchWave *w, int blocks,            \
      void *stream)                                                                        \
  {                                                                                        \
    return lola::launchBatchPass<S>(w, blocks, static_cast<cudaStream_t>(stream));         \
  }                                                                                        \
  extern "C" int lolaBatchOccupancy_##NAME(int accumulation, int paramJobs, int *blocks)   \
  {                                                                                        \
    return lola::batchOccupancy<S>(accumulation, paramJobs, blocks);                       \
  }
