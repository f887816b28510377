/* Internal interface between the C host code (lolacuda_host.c,
 * lolacuda_file.c, lolacuda_result.c) and the CUDA side (bp_*.cu kernels,
 * lolacuda_dispatch.cu launchers, lolacuda_batch.cu, lolacuda_verify.cu).
 * Plain C types only. */
#ifndef LOLACUDA_INTERNAL_H
#define LOLACUDA_INTERNAL_H

#include <stddef.h>
#include <stdint.h>

#include <cuda.h>

#include "lolaCuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Zero margin around every stored projection, in pixels.  Taps outside the
 * detector read these zeros, which is LolaBunny's pN() = 0 outside the image
 * (src/LolaBunny.c:11-17).  A (tile, projection) pair whose footprint lies
 * inside the margin runs without coordinate clamps. */
#define LOLA_MARGIN 64

/* Row pitch, in pixels, of a stored projection of the given width: the
 * padded width rounded up to 32 pixels (row starts 64-byte aligned for every
 * element size, as texture fetches from pitched memory need), and for the
 * layouts read by pixel index (loads, or a linear texture) 64 bytes more, so
 * that consecutive rows start 64 bytes apart modulo the L1's 128-byte bank
 * width: the texels of a warp quarter that straddle two detector rows then
 * meet fewer bank conflicts (N=1024 on GB300: f16qx +0.6 %, f32 +1.0 %, f32q
 * unchanged).  The volume does not depend on the pitch. */
static inline int lolaStorePitch(int width, int storage, int elemBytes)
{
  const int pitch = (width + 2 * LOLA_MARGIN + 31) & ~31;
  if (storage == LOLA_STORE_TEX32 || storage == LOLA_STORE_TEX16 || elemBytes <= 0)
    return pitch;
  return pitch + 64 / elemBytes;
}

/* Stored (padded) projection layout on the device. */
typedef struct {
  int32_t storage;      /* LOLA_STORE_* */
  int32_t elemBytes;    /* bytes per stored pixel (quad layouts: 4 taps) */
  int32_t margin;       /* LOLA_MARGIN */
  int32_t pitch;        /* padded width, pixels */
  int32_t rows;         /* padded height, pixels */
  int32_t width;        /* detector width */
  int32_t height;       /* detector height */
  int32_t reserved;
  size_t slotElems;     /* pixels per ring slot (>= pitch * rows, 256 B multiple) */
  /* texture layouts: one texture object per ring slot (cudaTextureObject_t) */
  unsigned long long texObjects[LOLA_MAX_BATCH];
  /* texture layouts read from CUDA arrays: the surface object (cudaSurfaceObject_t)
     the pack kernel writes each slot's array through; 0 = textures read the
     linear ring */
  unsigned long long surfObjects[LOLA_MAX_BATCH];
} LolaStoreDesc;

/* 1: the plan's texture layouts read CUDA arrays (the GPU's block-linear 2D
   layout) written by the pack kernel through surfaces; 0: pitch-linear
   textures over the ring.  Measured on GB300 at N=1024 the arrays gain
   nothing (tex16 +0.5 %, tex32 0, f16qx -2.5 % for its second copy): the
   footprints are small enough for the texture cache either way. */
#ifndef LOLA_TEX_ARRAYS
#define LOLA_TEX_ARRAYS 0
#endif

/* One projection of a kernel pass: the FP64 matrix and its FP32 voxel steps. */
typedef struct {
  double a[12];         /* column-major 3x4, a[col*3 + row] */
  float step[3][3];     /* step[axis][comp]: (float)(a[axis*3 + comp] * voxelSize) */
  int32_t slot;         /* ring slot holding the stored image */
  int32_t reserved[3];
} LolaPassProj;

typedef struct {
  int32_t N;
  int32_t count;        /* projections in this pass, 1..LOLA_MAX_BATCH */
  int32_t zBegin;       /* slab of the volume held by this pass: z in [zBegin, zEnd) */
  int32_t zEnd;
  float voxelSize;
  float originIndex;
  int32_t accumulation; /* LOLA_ACCUM_* */
  int32_t voxelsPerThread;
  int32_t rowsPerBlock;
  int32_t countTiles;   /* accumulate fast/slow/skipped tile counters */
  /* device copy of proj[0 .. count), or null.  The per-tile setup reads each
     projection from one lane; from the kernel parameters those reads differ
     per lane and the constant cache serves them one address at a time, from
     global memory they are ordinary cached loads */
  const LolaPassProj *projDevice;
  LolaPassProj proj[LOLA_MAX_BATCH];
} LolaPassParams;

/* Voxels along x covered by one warp of a pass kernel: a warp holds an
 * LOLA_WARP_X x (32 / LOLA_WARP_X) patch of the tile's xy plane, and a tile of
 * R warps spans LOLA_WARP_X x (32 R / LOLA_WARP_X) x voxels-per-thread voxels.
 * A compact patch keeps a warp's detector footprint compact: measured on
 * GB300 at N=1024, 8 x 4 beat 32 x 1 by 6-8 % for the four-tap layouts (f32
 * 1214 vs 1127 GUPS), 2 % for tex16, and was within 1 % for the quad layouts
 * (f16qx with column-ordered quads: 16 x 2 warps 1516 vs 1514 GUPS). */
#ifndef LOLA_WARP_X
#define LOLA_WARP_X 8
#endif

/* Per-plan tile counters of the pass kernels: (tile, projection) pairs
 * skipped, fast (staged included), slow, staged, and fast on the paired path. */
#define LOLA_TILE_COUNTERS 5
/* Copies of the counters the pass kernels spread their atomic adds over
 * (block index modulo this): one set per plan would have every block's adds
 * meet at four addresses.  The host sums the copies. */
#define LOLA_COUNTER_SPREAD 64

/* Mixed layouts: voxels (bit k of a thread's column) that fetch through the
 * texture unit.  Row-ordered quads (f32qx, and f16qx with LOLA_F16QX_COLS 0):
 * with the paired path (one load and one texture voxel per pair) 4 of every
 * 8 measured best on GB300: +2.5 % over 2 of 8, 4 % over 1 of 8 or none, 2 %
 * over whole pairs through the texture unit. */
#ifndef LOLA_MIXED_TEX_MASK
#define LOLA_MIXED_TEX_MASK 0xAAAAu
#endif

/* 1: f16qx stores its quads column by column.  A texel then lands as the two
 * column pairs that one packed FMA interpolates in x, so voxel pairs read
 * wholly through the texture unit need no register moves. */
#ifndef LOLA_F16QX_COLS
#define LOLA_F16QX_COLS 1
#endif
/* f16qx: the voxels (bit k of a thread's column) that fetch through the
 * texture unit; the others load.  With linear textures (LOLA_MIXED_TEX_LINEAR)
 * every voxel by texture measured fastest on GB300 at N=1024 (f16qx GUPS,
 * batch 16, 16 x 4 tiles, one box): 0xFFFF 1757-1767, 0xBBBB 1675,
 * 0xBFBF 1672, 0xEEEE 1658, 0xFBFB 1633, 0xABAB 1619-1625 — and 2D textures
 * at float coordinates with 0xABAB, the earlier default, 1544.  At N=512 all
 * by texture 1438 against 1297 for the earlier default. */
#ifndef LOLA_F16QX_TEX_MASK
#define LOLA_F16QX_TEX_MASK 0xFFFFu
#endif

/* 1: the mixed layouts' texture voxels fetch their quad with tex1Dfetch from
 * a linear texture over the ring slot, by the same integer pixel index the
 * load path forms: no float texture coordinates (two FADDs per voxel fewer)
 * and an index past the slot reads zero.  0: tex2D point fetch from a
 * pitch-linear 2D texture at float coordinates.  Measured on GB300 at
 * N=1024 with the mask 0xABAB: f16qx 1625 vs 1544 GUPS. */
#ifndef LOLA_MIXED_TEX_LINEAR
#define LOLA_MIXED_TEX_LINEAR 1
#endif

/* 1: f32qx stores its quads column by column and the pass kernel uses
 * LOLA_F32QX_COLS_TEX_MASK; 0: row order and LOLA_MIXED_TEX_MASK.  Measured
 * on GB300 at N=1024, batch 32 (GUPS): row order 1196; column order with
 * 0x2A2A 1231, 0x0303 1174, 0xABAB 1112, 0x2323 1081; all below f32q (1441),
 * whose loads alone are faster than any share of 16-byte texels. */
#ifndef LOLA_F32QX_COLS
#define LOLA_F32QX_COLS 0
#endif
#ifndef LOLA_F32QX_COLS_TEX_MASK
#define LOLA_F32QX_COLS_TEX_MASK 0xABABu
#endif

/* Stage buffers of the staged pass (a build-time tuning knob). */
#ifndef LOLA_STAGES
#define LOLA_STAGES 3
#endif

/* z-chunks of a volume transfer overlapped with a pass (upload before the
   first pass, download after the last one) */
#define LOLA_XFER_CHUNKS 8
/* volumes smaller than this move in one piece */
#define LOLA_XFER_MIN_CHUNK_BYTES (32u << 20)

/* Shared-memory staging of one pass (bp_staged.cuh): the tensor map over the
 * stored ring and the staging box. */
typedef struct {
  CUtensorMap tensorMap;  /* 3D: {pixel elements, rows, slots} */
  int32_t boxW, boxH;     /* staging box, pixels */
  int32_t align;          /* box origin alignment, pixels */
  int32_t elemsPerPixel;  /* tensor elements per stored pixel */
  int32_t stageBytes;     /* one stage buffer, 128 B multiple */
  int32_t boxBytes;       /* bytes one tensor copy delivers */
  int *d_error;           /* device flag set on a wait timeout */
} LolaStageDesc;

/* Projections per wave of a batched reconstruction (its kernels keep the
 * wave's per-projection setup in a static shared array of this size). */
#define LOLA_BATCH_MAX_WAVE 32

/* Work item of the persistent batched pass (bp_batch.cuh): a passKernel tile
 * of LOLA_BATCH_ROWS warps, LOLA_WARP_X x (32 LOLA_BATCH_ROWS / LOLA_WARP_X) x
 * LOLA_BATCH_VPT voxels (the default pass tile, 8 x 16 x 16). */
#define LOLA_BATCH_VPT 16
#define LOLA_BATCH_ROWS 4

/* One reconstruction of a batch (bp_batch.cuh), as the device sees it. */
typedef struct {
  float *volume;                    /* N^3 FP32 */
  const float *images;              /* nproj x height x width FP32 */
  unsigned char *ring;              /* this job's `b` stored slots */
  const unsigned long long *tex;    /* device array of b texture objects, or null */
  size_t slotBytes;
  size_t slotElems;
  int32_t N, width, height, margin, pitch, rows;
  float voxelSize, originIndex;
  int32_t tilesX, tilesY, tilesZ, nproj;
} LolaBatchJob;

/* A job as the persistent pass reads it from its wave's kernel parameters
 * (LolaBatchWave.pj): every per-item value uniform, as passKernel's are. */
typedef struct {
  float *volume;                    /* N^3 FP32 */
  const unsigned char *ring;        /* this job's `b` stored slots */
  unsigned long long tex;           /* f16qx: one linear texture over the slots, else 0 */
  long long firstItem;              /* the job's first work item in this wave */
  size_t slotBytes;
  uint32_t slotElems;
  int32_t count;                    /* projections of this wave (<= 0: none) */
  int32_t N, width, height, pitch, rows, tilesX, tilesY;
  float voxelSize, originIndex;
} LolaBatchParamJob;

/* Jobs a wave carries in its kernel parameters; batches of more jobs run the
 * persistent pass from the device job table instead. */
#define LOLA_BATCH_PARAM_JOBS 128

/* One wave of a batch: projections [wave*b, wave*b + b) of every job. */
typedef struct {
  const LolaBatchJob *jobs;         /* device, njobs */
  const long long *tilePrefix;      /* device, njobs + 1: first work item of each job */
  const LolaPassProj *proj;         /* device, njobs x b: this wave's projections */
  int *counter;                     /* device: this wave's work-item counter */
  long long totalItems;
  int32_t njobs, b, wave, maxPitch, maxRows, accumulation, storage;
  int32_t paramJobs;                /* 1: pj[0 .. njobs) holds the jobs */
  LolaBatchParamJob pj[LOLA_BATCH_PARAM_JOBS];
} LolaBatchWave;

/* Kernel launchers (lolacuda_dispatch.cu).  Return 0 on success or a
 * cudaError_t value. */
int lolaLaunchPack(const LolaStoreDesc *store, const float *d_src, size_t srcStride,
    void *d_ring, int slot0, int count, void *stream);

/* stage = NULL: load-path pass; otherwise the TMA-staged pass. */
int lolaLaunchBackproject(const LolaStoreDesc *store, const LolaPassParams *params,
    const LolaStageDesc *stage, const void *d_ring, float *d_volume,
    unsigned long long *d_tileCounters, void *stream);

/* Voxels of a plan's volume (N^3). */
size_t lolaPlanVoxels(const LolaCudaPlan *plan);
const LolaCudaGeometry *lolaPlanGeometry(const LolaCudaPlan *p);
/* Projections the plan's next host-staged pass takes with `left` projections
   of the scan still to stage (0 = unknown), and the most any pass takes. */
int lolaPlanPassCapacity(const LolaCudaPlan *p, int left);
int lolaPlanRingSlots(const LolaCudaPlan *p);

/* Sets the thread's lolaCudaLastError() message; returns 0. */
int lolaSetError(const char *fmt, ...);

/* Batched waves: pack every job's slots, then one persistent pass. */
int lolaLaunchBatchPack(const LolaBatchWave *wave, void *stream);
int lolaLaunchBatchPass(const LolaBatchWave *wave, int blocks, void *stream);
/* Resident blocks per SM of the batched pass for a storage layout. */
int lolaBatchPassOccupancy(int storage, int accumulation, int paramJobs, int *blocksPerSM);

/* 1 if the (voxelsPerThread, rowsPerBlock) pair has a compiled kernel. */
int lolaKernelShapeSupported(int voxelsPerThread, int rowsPerBlock);

#ifdef __cplusplus
}
#endif

#endif /* LOLACUDA_INTERNAL_H */
