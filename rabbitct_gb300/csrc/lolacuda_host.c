/* LolaCUDA host code (C99): the RabbitCT module API, configuration and the
 * plan API declared in include/lolaCuda.h.
 *
 * Data layout in device memory (one plan):
 *   volume   N^3 FP32, x fastest, identical to the runner's volumeData so the
 *            final copy is one contiguous transfer (src/rabbitRunner.c:192)
 *   ring     `batch` stored projections, each zero-padded by LOLA_MARGIN
 *            pixels in the configured storage layout
 *   stage    `batch` raw FP32 detector images, landing zone of host uploads
 *   counters 3 x u64 (tile statistics)
 *
 * Module state follows the reference modules: one static instance per
 * process (the reference modules keep their padding and line ranges in file
 * statics too, e.g. src/LolaOPT.c:18-21).
 */
#define _POSIX_C_SOURCE 200809L
#include <ctype.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <math.h>

#include <cuda.h>
#include <cuda_runtime_api.h>

#include "lolaCuda.h"
#include "lolacuda_internal.h"

/* ---- errors ---------------------------------------------------------------- */

static __thread char gLastError[512];

static int setError(const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(gLastError, sizeof(gLastError), fmt, ap);
  va_end(ap);
  return 0;
}

const char *lolaCudaLastError(void)
{
  return gLastError;
}

int lolaSetError(const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(gLastError, sizeof(gLastError), fmt, ap);
  va_end(ap);
  return 0;
}

/* A failed call's error is also taken out of the runtime's last-error slot
   (for the non-sticky ones, such as a failed allocation), so that a later
   launch check does not report it again. */
#define CUDA_TRY(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      (void)cudaGetLastError();                                                          \
      return setError("%s:%d: %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
    }                                                                                    \
  } while (0)

#define LAUNCH_TRY(call)                                                                 \
  do {                                                                                   \
    int e_ = (call);                                                                     \
    if (e_ != 0)                                                                         \
      return setError("%s:%d: kernel launch failed: %s", __FILE__, __LINE__,             \
          cudaGetErrorString((cudaError_t)e_));                                          \
  } while (0)

/* ---- configuration ---------------------------------------------------------- */

static int storageFromName(const char *s)
{
  static const char *names[] = { "f32", "f16", "bf16", "f32q", "f16q", "bf16q", "tex32",
    "tex16", "f16qx", "f32qx" };
  for (int i = 0; i < 10; i++) {
    const char *a = names[i], *b = s;
    while (*a && *b && tolower((unsigned char)*b) == *a) {
      a++;
      b++;
    }
    if (*a == 0 && *b == 0)
      return i;
  }
  return -1;
}

static int envInt(const char *name, int dflt)
{
  const char *v = getenv(name);
  if (v == NULL || *v == 0)
    return dflt;
  return atoi(v);
}

void lolaCudaDefaultConfig(LolaCudaConfig *c)
{
  memset(c, 0, sizeof(*c));
  /* FP32 2x2 quads: the exact FP32 taps of plain FP32 storage and identical
     results, one 16-byte load per update instead of four 4-byte loads
     (1282 vs 1132 GUPS at N=1024 on GB300) */
  c->storage = LOLA_STORE_F32Q;
  c->accumulation = LOLA_ACCUM_PLAIN;
  c->batch = 16;
  /* 16 x 4 tiles: the fastest shape measured for FP32 and FP16 storage at
     N=1024 on GB300 (f32 1151, f16qx 1337 GUPS vs 1026 and 1224 for 8x8 tiles) */
  c->voxelsPerThread = 16;
  c->rowsPerBlock = 4;
  c->syncEachCall = 1;
  c->exitOnError = 1;
  c->collectStats = 0;
  c->device = 0;
  const char *s = getenv("LOLACUDA_STORAGE");
  if (s != NULL && storageFromName(s) >= 0)
    c->storage = storageFromName(s);
  const char *acc = getenv("LOLACUDA_ACCUM");
  if (acc != NULL && strcmp(acc, "kahan") == 0)
    c->accumulation = LOLA_ACCUM_KAHAN;
  c->batch = envInt("LOLACUDA_BATCH", c->batch);
  c->voxelsPerThread = envInt("LOLACUDA_VPT", c->voxelsPerThread);
  c->rowsPerBlock = envInt("LOLACUDA_ROWS", c->rowsPerBlock);
  c->syncEachCall = envInt("LOLACUDA_SYNC", c->syncEachCall);
  c->exitOnError = envInt("LOLACUDA_EXIT", c->exitOnError);
  c->staging = envInt("LOLACUDA_STAGING", 0);
  c->batchMode = envInt("LOLACUDA_BATCH_MODE", LOLA_BATCH_BRANCHES);
  c->batchBranches = envInt("LOLACUDA_BATCH_BRANCHES", 16);
  /* per-class shape tuning measured no better than the default 16 x 4 tiles on
     the 64-job uneven workload (912 vs 921 GUPS), so it is opt-in */
  c->batchTune = envInt("LOLACUDA_BATCH_TUNE", 0);
  c->edgeBatch = envInt("LOLACUDA_EDGE_BATCH", 0);
}

static int validateConfig(const LolaCudaConfig *c)
{
  if (c->storage < LOLA_STORE_F32 || c->storage > LOLA_STORE_F32QX)
    return setError("invalid storage %d", c->storage);
  if (c->accumulation != LOLA_ACCUM_PLAIN && c->accumulation != LOLA_ACCUM_KAHAN)
    return setError("invalid accumulation %d", c->accumulation);
  if (c->batch < 1 || c->batch > LOLA_MAX_BATCH)
    return setError("batch %d outside 1..%d", c->batch, LOLA_MAX_BATCH);
  if (c->edgeBatch != 0 && (c->edgeBatch < c->batch || c->edgeBatch > LOLA_MAX_BATCH))
    return setError("edge batch %d outside %d..%d (or 0)", c->edgeBatch, c->batch,
        LOLA_MAX_BATCH);
  if (!lolaKernelShapeSupported(c->voxelsPerThread, c->rowsPerBlock))
    return setError("no kernel for %d voxels per thread x %d rows per block",
        c->voxelsPerThread, c->rowsPerBlock);
  return 1;
}

static LolaCudaConfig gConfig;
static int gConfigSet = 0;

int lolaCudaSetConfig(const LolaCudaConfig *c)
{
  if (c == NULL)
    return setError("null config");
  if (!validateConfig(c))
    return 0;
  gConfig = *c;
  gConfigSet = 1;
  return 1;
}

int lolaCudaGetConfig(LolaCudaConfig *c)
{
  if (!gConfigSet) {
    lolaCudaDefaultConfig(&gConfig);
    gConfigSet = 1;
  }
  *c = gConfig;
  return 1;
}

/* ---- plan --------------------------------------------------------------------- */

typedef struct {
  cudaEvent_t start, stop;
} EventPair;

struct LolaCudaPlan {
  LolaCudaGeometry geom;
  LolaCudaConfig cfg;
  LolaStoreDesc store;
  int device;
  cudaStream_t stream;      /* packing + passes */
  cudaStream_t copyStream;  /* host uploads into the stage */
  cudaEvent_t stageFree;    /* stage consumed by the last pack */
  cudaEvent_t stageReady;   /* uploads of the pending batch done */
  cudaEvent_t timerStart, timerStop;
  float *d_volume;
  void *d_ring;
  cudaArray_t texArrays[LOLA_MAX_BATCH];  /* texture layouts with LOLA_TEX_ARRAYS */
  float *d_stage;
  unsigned long long *d_counters;
  LolaPassProj *d_proj;   /* device copy of the current pass's projections */
  int *d_error;           /* staged-pass wait timeouts */
  int stagedLaunched;     /* a staged pass ran since the last error check */
  LolaStageDesc stageDesc; /* tensor map of the ring for the current box */
  int stageBoxW, stageBoxH;
  size_t imageElems;
  /* volume transfers overlapped with a pass: an asynchronous upload lands in
     z-chunks and the next pass starts on each chunk as it arrives; a
     streamed-out pass copies each chunk to the host once it is finished */
  cudaStream_t xferStream;
  cudaEvent_t upChunk[LOLA_XFER_CHUNKS], outChunk[LOLA_XFER_CHUNKS];
  cudaEvent_t xferDone, streamMark;
  int uploadChunks;  /* chunks of an asynchronous upload the next pass waits for */
  const float *uploadSrc;  /* host volume of an asynchronous upload not yet issued */
  int xferPending;   /* transfers the plan stream is not yet ordered after */
  float *streamOut;  /* host target for the volume after the next pass */
  float *outValid;   /* host copy streamed out after the last pass, if any */
  /* host-staged batch (module API / BackprojectHost) */
  int pending;
  int passCap;    /* projections the pass being staged takes before it launches */
  int ringSlots;  /* stage and ring slots: the larger of batch and the edge batch */
  int scanLeft;   /* projections of the scan not yet staged, this one included
                     (0 = unknown); set by the module API before each stage */
  double pendingMats[LOLA_MAX_BATCH][12];
  /* statistics */
  LolaCudaStats stats;
  EventPair *events;
  int nEvents, capEvents;
};

static int elemBytesOf(int storage)
{
  switch (storage) {
  case LOLA_STORE_F32: return 4;
  case LOLA_STORE_F16: return 2;
  case LOLA_STORE_BF16: return 2;
  case LOLA_STORE_F32Q: return 16;
  case LOLA_STORE_F16Q: return 8;
  case LOLA_STORE_BF16Q: return 8;
  case LOLA_STORE_TEX32: return 4;
  case LOLA_STORE_TEX16: return 2;
  case LOLA_STORE_F16QX: return 8;
  case LOLA_STORE_F32QX: return 16;
  default: return 0;
  }
}

/* Layouts read (also) through the texture unit, and their texel format:
 * 1 channel for the gather layouts, 4 (one 2x2 quad per texel) for the
 * mixed ones. */
static int isTexture(int storage)
{
  return storage == LOLA_STORE_TEX32 || storage == LOLA_STORE_TEX16 ||
         storage == LOLA_STORE_F16QX || storage == LOLA_STORE_F32QX;
}

static int texChannels(int storage)
{
  return (storage == LOLA_STORE_F16QX || storage == LOLA_STORE_F32QX) ? 4 : 1;
}

static int planRelease(LolaCudaPlan *p)
{
  if (p == NULL)
    return 1;
  cudaSetDevice(p->device);
  if (p->stream)
    cudaStreamSynchronize(p->stream);
  if (p->copyStream)
    cudaStreamSynchronize(p->copyStream);
  if (p->xferStream)
    cudaStreamSynchronize(p->xferStream);
  for (int i = 0; i < p->nEvents; i++) {
    cudaEventDestroy(p->events[i].start);
    cudaEventDestroy(p->events[i].stop);
  }
  free(p->events);
  for (int i = 0; i < LOLA_MAX_BATCH; i++) {
    if (p->store.texObjects[i])
      cudaDestroyTextureObject((cudaTextureObject_t)p->store.texObjects[i]);
    if (p->store.surfObjects[i])
      cudaDestroySurfaceObject((cudaSurfaceObject_t)p->store.surfObjects[i]);
    if (p->texArrays[i])
      cudaFreeArray(p->texArrays[i]);
  }
  cudaFree(p->d_volume);
  cudaFree(p->d_ring);
  cudaFree(p->d_stage);
  cudaFree(p->d_counters);
  cudaFree(p->d_proj);
  cudaFree(p->d_error);
  if (p->stageFree)
    cudaEventDestroy(p->stageFree);
  if (p->stageReady)
    cudaEventDestroy(p->stageReady);
  if (p->timerStart)
    cudaEventDestroy(p->timerStart);
  if (p->timerStop)
    cudaEventDestroy(p->timerStop);
  if (p->stream)
    cudaStreamDestroy(p->stream);
  if (p->copyStream)
    cudaStreamDestroy(p->copyStream);
  for (int i = 0; i < LOLA_XFER_CHUNKS; i++) {
    if (p->upChunk[i])
      cudaEventDestroy(p->upChunk[i]);
    if (p->outChunk[i])
      cudaEventDestroy(p->outChunk[i]);
  }
  if (p->xferDone)
    cudaEventDestroy(p->xferDone);
  if (p->streamMark)
    cudaEventDestroy(p->streamMark);
  if (p->xferStream)
    cudaStreamDestroy(p->xferStream);
  free(p);
  return 1;
}

int lolaCudaPlanDestroy(LolaCudaPlan *p)
{
  return planRelease(p);
}

static int planInit(LolaCudaPlan *p)
{
  const LolaCudaGeometry *g = &p->geom;
  CUDA_TRY(cudaSetDevice(p->device));
  CUDA_TRY(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
  CUDA_TRY(cudaStreamCreateWithFlags(&p->copyStream, cudaStreamNonBlocking));
  CUDA_TRY(cudaEventCreateWithFlags(&p->stageFree, cudaEventDisableTiming));
  CUDA_TRY(cudaEventCreateWithFlags(&p->stageReady, cudaEventDisableTiming));
  CUDA_TRY(cudaEventCreate(&p->timerStart));
  CUDA_TRY(cudaEventCreate(&p->timerStop));
  CUDA_TRY(cudaStreamCreateWithFlags(&p->xferStream, cudaStreamNonBlocking));
  for (int i = 0; i < LOLA_XFER_CHUNKS; i++) {
    CUDA_TRY(cudaEventCreateWithFlags(&p->upChunk[i], cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&p->outChunk[i], cudaEventDisableTiming));
  }
  CUDA_TRY(cudaEventCreateWithFlags(&p->xferDone, cudaEventDisableTiming));
  CUDA_TRY(cudaEventCreateWithFlags(&p->streamMark, cudaEventDisableTiming));

  LolaStoreDesc *s = &p->store;
  s->storage = p->cfg.storage;
  s->elemBytes = elemBytesOf(s->storage);
  s->margin = LOLA_MARGIN;
  s->width = g->imageWidth;
  s->height = g->imageHeight;
  s->pitch = lolaStorePitch(g->imageWidth, s->storage, s->elemBytes);
  s->rows = g->imageHeight + 2 * LOLA_MARGIN;
  /* index arithmetic in the kernel is exact below 2^23 pixels */
  if ((long long)s->pitch * s->rows >= (1LL << 23) - 2 * (long long)s->pitch)
    return setError("detector %dx%d too large (padded image must stay below 2^23 pixels)",
        g->imageWidth, g->imageHeight);
  const size_t px = (size_t)s->pitch * (size_t)s->rows;
  s->slotElems = (px + 255) & ~(size_t)255;  /* slot bases 512 B aligned */
  p->imageElems = (size_t)g->imageWidth * (size_t)g->imageHeight;

  p->ringSlots = p->cfg.edgeBatch > p->cfg.batch ? p->cfg.edgeBatch
      : p->cfg.edgeBatch == 0 ? 2 * p->cfg.batch : p->cfg.batch;
  if (p->ringSlots > LOLA_MAX_BATCH)
    p->ringSlots = LOLA_MAX_BATCH;
  const size_t nvox = lolaPlanVoxels(p);
  CUDA_TRY(cudaMalloc((void **)&p->d_volume, nvox * sizeof(float)));
  CUDA_TRY(cudaMemsetAsync(p->d_volume, 0, nvox * sizeof(float), p->stream));
  CUDA_TRY(cudaMalloc(&p->d_ring, (size_t)p->ringSlots * s->slotElems * s->elemBytes));
  CUDA_TRY(cudaMemsetAsync(p->d_ring, 0, (size_t)p->ringSlots * s->slotElems * s->elemBytes,
      p->stream));
  if (isTexture(s->storage)) {
    for (int i = 0; i < p->ringSlots; i++) {
      struct cudaResourceDesc rd;
      memset(&rd, 0, sizeof(rd));
      const int ch = texChannels(s->storage);
      const int bits = 8 * s->elemBytes / ch;
      const struct cudaChannelFormatDesc texel = cudaCreateChannelDesc(bits,
          ch > 1 ? bits : 0, ch > 1 ? bits : 0, ch > 1 ? bits : 0, cudaChannelFormatKindFloat);
      void *slotBase = (char *)p->d_ring + (size_t)i * s->slotElems * s->elemBytes;
      if (LOLA_MIXED_TEX_LINEAR && ch == 4) {
        /* mixed layouts: quads fetched by their integer index in the slot */
        rd.resType = cudaResourceTypeLinear;
        rd.res.linear.devPtr = slotBase;
        rd.res.linear.desc = texel;
        rd.res.linear.sizeInBytes = s->slotElems * (size_t)s->elemBytes;
      } else {
        rd.resType = cudaResourceTypePitch2D;
        rd.res.pitch2D.devPtr = slotBase;
        rd.res.pitch2D.desc = texel;
        rd.res.pitch2D.width = (size_t)s->pitch;
        rd.res.pitch2D.height = (size_t)s->rows;
        rd.res.pitch2D.pitchInBytes = (size_t)s->pitch * s->elemBytes;
      }
      if (LOLA_TEX_ARRAYS && rd.resType == cudaResourceTypePitch2D) {
        /* a CUDA array per slot (block-linear), written through a surface */
        const struct cudaChannelFormatDesc cd = rd.res.pitch2D.desc;
        CUDA_TRY(cudaMallocArray(&p->texArrays[i], &cd, (size_t)s->pitch, (size_t)s->rows,
            cudaArraySurfaceLoadStore));
        memset(&rd, 0, sizeof(rd));
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = p->texArrays[i];
        cudaSurfaceObject_t sf = 0;
        CUDA_TRY(cudaCreateSurfaceObject(&sf, &rd));
        s->surfObjects[i] = (unsigned long long)sf;
      }
      struct cudaTextureDesc td;
      memset(&td, 0, sizeof(td));
      td.addressMode[0] = cudaAddressModeBorder;
      td.addressMode[1] = cudaAddressModeBorder;
      td.filterMode = cudaFilterModePoint;
      td.readMode = cudaReadModeElementType;
      td.normalizedCoords = 0;
      cudaTextureObject_t t = 0;
      CUDA_TRY(cudaCreateTextureObject(&t, &rd, &td, NULL));
      s->texObjects[i] = (unsigned long long)t;
    }
  }
  CUDA_TRY(cudaMalloc((void **)&p->d_stage,
      (size_t)p->ringSlots * p->imageElems * sizeof(float)));
  CUDA_TRY(cudaMalloc((void **)&p->d_counters,
      LOLA_COUNTER_SPREAD * LOLA_TILE_COUNTERS * sizeof(unsigned long long)));
  CUDA_TRY(cudaMalloc((void **)&p->d_proj, LOLA_MAX_BATCH * sizeof(LolaPassProj)));
  CUDA_TRY(cudaMemsetAsync(p->d_counters, 0,
      LOLA_COUNTER_SPREAD * LOLA_TILE_COUNTERS * sizeof(unsigned long long),
      p->stream));
  CUDA_TRY(cudaMalloc((void **)&p->d_error, sizeof(int)));
  CUDA_TRY(cudaMemsetAsync(p->d_error, 0, sizeof(int), p->stream));
  CUDA_TRY(cudaEventRecord(p->stageFree, p->stream));
  CUDA_TRY(cudaStreamSynchronize(p->stream));
  return 1;
}

int lolaCudaPlanCreate(const LolaCudaGeometry *g, const LolaCudaConfig *cfg, LolaCudaPlan **out)
{
  if (out == NULL || g == NULL)
    return setError("null argument");
  *out = NULL;
  LolaCudaConfig c;
  if (cfg != NULL)
    c = *cfg;
  else
    lolaCudaDefaultConfig(&c);
  if (!validateConfig(&c))
    return 0;
  if (g->problemSize <= 0 || g->imageWidth <= 0 || g->imageHeight <= 0)
    return setError("invalid geometry N=%d W=%d H=%d", g->problemSize, g->imageWidth,
        g->imageHeight);
  if (g->problemSize > 2048)
    return setError("problem size %d above the supported 2048", g->problemSize);
  if (!(g->voxelSize > 0.0f))
    return setError("voxel size must be positive");
  LolaCudaPlan *p = (LolaCudaPlan *)calloc(1, sizeof(LolaCudaPlan));
  if (p == NULL)
    return setError("out of host memory");
  p->geom = *g;
  if (p->geom.sliceCount == 0 && p->geom.sliceBegin == 0)
    p->geom.sliceCount = g->problemSize;
  if (p->geom.sliceBegin < 0 || p->geom.sliceCount <= 0 ||
      p->geom.sliceBegin + p->geom.sliceCount > g->problemSize) {
    free(p);
    return setError("slab [%d, %d) outside the %d slices", g->sliceBegin,
        g->sliceBegin + g->sliceCount, g->problemSize);
  }
  p->cfg = c;
  p->device = c.device;
  if (!planInit(p)) {
    char msg[512];
    snprintf(msg, sizeof(msg), "%s", gLastError);
    planRelease(p);
    return setError("%s", msg);
  }
  *out = p;
  return 1;
}

static void xferChunkRange(const LolaCudaPlan *p, int c, int k, int *zb, int *ze);

/* Issues an asynchronous volume upload that lolaCudaPlanUploadVolumeAsync
 * deferred: its z-chunk copies on the transfer stream after the plan stream's
 * work so far, each chunk's landing recorded for the pass that waits for it.
 * Deferred to the first pass that needs the volume (or any other use of it),
 * so that pass's projections, copied by the calls before it, do not queue
 * behind the whole volume on the host link: in the module API the first pass
 * then starts on chunk 0 about 3 ms after its projections are in, instead of
 * after the entire 4 GiB upload (24 ms at N=1024). */
static int issueUpload(LolaCudaPlan *p)
{
  if (p->uploadSrc == NULL)
    return 1;
  const float *h = p->uploadSrc;
  p->uploadSrc = NULL;
  cudaStream_t us = p->xferStream;
  /* the upload overwrites what earlier work on the plan stream produces */
  CUDA_TRY(cudaEventRecord(p->streamMark, p->stream));
  CUDA_TRY(cudaStreamWaitEvent(us, p->streamMark, 0));
  const int k = p->uploadChunks;
  const size_t slice = (size_t)p->geom.problemSize * (size_t)p->geom.problemSize;
  for (int c = 0; c < k; c++) {
    int zb, ze;
    xferChunkRange(p, c, k, &zb, &ze);
    if (ze > zb)
      CUDA_TRY(cudaMemcpyAsync(p->d_volume + (size_t)zb * slice, h + (size_t)zb * slice,
          (size_t)(ze - zb) * slice * sizeof(float), cudaMemcpyHostToDevice, us));
    CUDA_TRY(cudaEventRecord(p->upChunk[c], us));
  }
  CUDA_TRY(cudaEventRecord(p->xferDone, us));
  p->xferPending = 1;
  return 1;
}

/* Orders the plan stream after every volume transfer, issuing a deferred
   upload first. */
static int joinTransfers(LolaCudaPlan *p)
{
  if (!issueUpload(p))
    return 0;
  if (p->xferPending) {
    CUDA_TRY(cudaStreamWaitEvent(p->stream, p->xferDone, 0));
    p->xferPending = 0;
  }
  p->uploadChunks = 0;
  return 1;
}

float *lolaCudaPlanVolume(LolaCudaPlan *p)
{
  if (p == NULL)
    return NULL;
  cudaSetDevice(p->device);
  joinTransfers(p);
  return p->d_volume;
}

void *lolaCudaPlanStream(LolaCudaPlan *p)
{
  return p ? (void *)p->stream : NULL;
}

size_t lolaPlanVoxels(const LolaCudaPlan *p)
{
  const size_t n = (size_t)p->geom.problemSize;
  return n * n * (size_t)p->geom.sliceCount;
}

const LolaCudaGeometry *lolaPlanGeometry(const LolaCudaPlan *p)
{
  return &p->geom;
}

static size_t volumeBytes(const LolaCudaPlan *p)
{
  return lolaPlanVoxels(p) * sizeof(float);
}

/* Number of z-chunks a volume transfer is split into; chunk boundaries fall
   on tile boundaries (multiples of voxelsPerThread from the slab start), so a
   pass launched chunk by chunk computes exactly the tiles of a whole pass. */
static int xferChunks(const LolaCudaPlan *p)
{
  const int vpt = p->cfg.voxelsPerThread;
  const int tiles = (p->geom.sliceCount + vpt - 1) / vpt;
  size_t k = volumeBytes(p) / LOLA_XFER_MIN_CHUNK_BYTES;
  if (k > LOLA_XFER_CHUNKS)
    k = LOLA_XFER_CHUNKS;
  if (k > (size_t)tiles)
    k = (size_t)tiles;
  return k < 1 ? 1 : (int)k;
}

/* Slices [*zb, *ze) of chunk c of k, relative to the slab start. */
static void xferChunkRange(const LolaCudaPlan *p, int c, int k, int *zb, int *ze)
{
  const int vpt = p->cfg.voxelsPerThread;
  const int nz = p->geom.sliceCount;
  const int tiles = (nz + vpt - 1) / vpt;
  *zb = (int)((long long)tiles * c / k) * vpt;
  const int e = (int)((long long)tiles * (c + 1) / k) * vpt;
  *ze = e > nz ? nz : e;
}

int lolaCudaSlab(int N, int rank, int ranks, int align, int32_t *begin, int32_t *count)
{
  if (N <= 0 || ranks <= 0 || rank < 0 || rank >= ranks || align <= 0 || begin == NULL ||
      count == NULL)
    return setError("slab: invalid arguments");
  const int units = (N + align - 1) / align;
  const int b = (int)((long long)units * rank / ranks) * align;
  int e = (int)((long long)units * (rank + 1) / ranks) * align;
  e = e > N ? N : e;
  *begin = b;
  *count = e > b ? e - b : 0;
  return 1;
}

int lolaCudaPlanZeroVolume(LolaCudaPlan *p)
{
  if (p == NULL)
    return setError("null plan");
  CUDA_TRY(cudaSetDevice(p->device));
  if (!joinTransfers(p))
    return 0;
  CUDA_TRY(cudaMemsetAsync(p->d_volume, 0, volumeBytes(p), p->stream));
  p->outValid = NULL;
  return 1;
}

int lolaCudaPlanUploadVolume(LolaCudaPlan *p, const float *h)
{
  if (p == NULL || h == NULL)
    return setError("null argument");
  CUDA_TRY(cudaSetDevice(p->device));
  if (!joinTransfers(p))
    return 0;
  CUDA_TRY(cudaMemcpyAsync(p->d_volume, h, volumeBytes(p), cudaMemcpyHostToDevice, p->stream));
  CUDA_TRY(cudaStreamSynchronize(p->stream));
  p->outValid = NULL;
  return 1;
}

int lolaCudaPlanUploadVolumeAsync(LolaCudaPlan *p, const float *h)
{
  if (p == NULL || h == NULL)
    return setError("null argument");
  CUDA_TRY(cudaSetDevice(p->device));
  /* a previous upload not yet issued is overwritten by this one anyway */
  p->uploadSrc = h;
  p->uploadChunks = xferChunks(p);
  p->outValid = NULL;
  /* from page-locked memory the copies wait for the next pass; from pageable
     memory the driver stages them through its own buffers and holds this
     thread until it has read the volume, so they are issued here, where the
     module API's prepare pays for them, as before */
  struct cudaPointerAttributes attr;
  const int pinned = cudaPointerGetAttributes(&attr, h) == cudaSuccess &&
                     attr.type == cudaMemoryTypeHost;
  cudaGetLastError(); /* an unknown pointer is not an error here */
  if (!pinned)
    return issueUpload(p);
  return 1;
}

int lolaCudaPlanStreamVolumeOut(LolaCudaPlan *p, float *h)
{
  if (p == NULL || h == NULL)
    return setError("null argument");
  p->streamOut = h;
  return 1;
}

int lolaCudaPlanDownloadVolume(LolaCudaPlan *p, float *h)
{
  if (p == NULL || h == NULL)
    return setError("null argument");
  CUDA_TRY(cudaSetDevice(p->device));
  if (!joinTransfers(p))
    return 0;
  CUDA_TRY(cudaMemcpyAsync(h, p->d_volume, volumeBytes(p), cudaMemcpyDeviceToHost, p->stream));
  CUDA_TRY(cudaStreamSynchronize(p->stream));
  return 1;
}

/* FP32 voxel steps of one view: step[axis][comp] = a[axis*3 + comp] * voxelSize */
static void fillPassProj(LolaPassProj *pp, const double *m, float voxelSize, int slot)
{
  memcpy(pp->a, m, 12 * sizeof(double));
  for (int ax = 0; ax < 3; ax++)
    for (int c = 0; c < 3; c++)
      pp->step[ax][c] = (float)(m[ax * 3 + c] * (double)voxelSize);
  pp->slot = slot;
}

static int pushEvent(LolaCudaPlan *p, EventPair **out)
{
  if (p->nEvents == p->capEvents) {
    const int cap = p->capEvents ? 2 * p->capEvents : 64;
    EventPair *e = (EventPair *)realloc(p->events, (size_t)cap * sizeof(EventPair));
    if (e == NULL)
      return setError("out of host memory");
    p->events = e;
    p->capEvents = cap;
  }
  EventPair *e = &p->events[p->nEvents];
  CUDA_TRY(cudaEventCreate(&e->start));
  CUDA_TRY(cudaEventCreate(&e->stop));
  p->nEvents++;
  *out = e;
  return 1;
}


/* ---- shared-memory staging ------------------------------------------------------
 * The staged pass copies, per (tile, projection), the box of the stored
 * projection that the tile's taps fall in.  The box is sized per pass from
 * the footprints of 27 sample tiles (corners, edge midpoints and centre of the
 * tile grid) under the pass's matrices; tiles whose footprint exceeds it use
 * the load path inside the same launch. */

typedef CUresult (*TensorMapEncodeFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
    const cuuint64_t *, const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
    CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static TensorMapEncodeFn tensorMapEncoder(void)
{
  static TensorMapEncodeFn fn = NULL;
  static int tried = 0;
  if (!tried) {
    tried = 1;
    void *f = NULL;
    enum cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
            &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (TensorMapEncodeFn)f;
  }
  return fn;
}

/* Tensor-map element type, elements per stored pixel and bytes per pixel. */
static int stageFormat(int storage, CUtensorMapDataType *dt, int *epp, int *pix)
{
  switch (storage) {
  case LOLA_STORE_F32: *dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT32; *epp = 1; *pix = 4; return 1;
  case LOLA_STORE_F16:
  case LOLA_STORE_BF16: *dt = CU_TENSOR_MAP_DATA_TYPE_UINT16; *epp = 1; *pix = 2; return 1;
  case LOLA_STORE_F32Q:
  case LOLA_STORE_F32QX: *dt = CU_TENSOR_MAP_DATA_TYPE_UINT64; *epp = 2; *pix = 16; return 1;
  case LOLA_STORE_F16Q:
  case LOLA_STORE_F16QX:
  case LOLA_STORE_BF16Q: *dt = CU_TENSOR_MAP_DATA_TYPE_UINT64; *epp = 1; *pix = 8; return 1;
  default: return 0;
  }
}

/* per stage; LOLA_STAGES of them share about 72 KB per block */
#define LOLA_STAGE_MAX_BYTES (72 * 1024 / LOLA_STAGES)

/* Box (pixels) that holds the taps of the sampled tiles; 0 if nothing fits. */
static void sampleFootprint(const LolaCudaPlan *p, const double *mats, int count, int *needW,
    int *needH)
{
  const int N = p->geom.problemSize;
  const int TX = 32, TY = p->cfg.rowsPerBlock, TZ = p->cfg.voxelsPerThread;
  const int nt[3] = { (N + TX - 1) / TX, (N + TY - 1) / TY, (N + TZ - 1) / TZ };
  const int te[3] = { TX, TY, TZ };
  const double vs = (double)p->geom.voxelSize, o = (double)p->geom.originIndex;
  const double W = p->geom.imageWidth, H = p->geom.imageHeight;
  int mw = 0, mh = 0;
  for (int q = 0; q < count; q++) {
    const double *a = mats + 12 * (size_t)q;
    for (int t = 0; t < 27; t++) {
      int org[3], ext[3];
      int tt = t;
      for (int d = 0; d < 3; d++) {
        const int sel = tt % 3;
        tt /= 3;
        const int ti = sel == 0 ? 0 : (sel == 1 ? nt[d] / 2 : nt[d] - 1);
        org[d] = ti * te[d];
        ext[d] = (org[d] + te[d] <= N ? te[d] : N - org[d]) - 1;
      }
      double mnu = 1e30, mxu = -1e30, mnv = 1e30, mxv = -1e30;
      int bad = 0;
      for (int c = 0; c < 8; c++) {
        const double X = o + (double)(org[0] + ((c & 1) ? ext[0] : 0)) * vs;
        const double Y = o + (double)(org[1] + ((c & 2) ? ext[1] : 0)) * vs;
        const double Z = o + (double)(org[2] + ((c & 4) ? ext[2] : 0)) * vs;
        const double w = a[2] * X + a[5] * Y + a[8] * Z + a[11];
        if (!(w > 0.0)) {
          bad = 1;
          break;
        }
        const double u = (a[0] * X + a[3] * Y + a[6] * Z + a[9]) / w;
        const double v = (a[1] * X + a[4] * Y + a[7] * Z + a[10]) / w;
        mnu = u < mnu ? u : mnu;
        mxu = u > mxu ? u : mxu;
        mnv = v < mnv ? v : mnv;
        mxv = v > mxv ? v : mxv;
      }
      if (bad || mxu <= -2.0 || mnu >= W || mxv <= -2.0 || mnv >= H)
        continue;
      const int w = (int)(floor(mxu + 0.5) - floor(mnu - 0.5)) + 3;
      const int h = (int)(floor(mxv + 0.5) - floor(mnv - 0.5)) + 3;
      mw = w > mw ? w : mw;
      mh = h > mh ? h : mh;
    }
  }
  *needW = mw;
  *needH = mh;
}

/* Fills p->stageDesc for this pass; returns 1 if the pass should be staged. */
static int prepareStage(LolaCudaPlan *p, const double *mats, int count)
{
  if (!p->cfg.staging)
    return 0;
  /* staged kernels are compiled for 8 voxels per thread and 4 or 8 rows */
  if (p->cfg.voxelsPerThread != 8 || (p->cfg.rowsPerBlock != 8 && p->cfg.rowsPerBlock != 4))
    return 0;
  CUtensorMapDataType dt;
  int epp, pix;
  if (!stageFormat(p->store.storage, &dt, &epp, &pix))
    return 0;
  TensorMapEncodeFn encode = tensorMapEncoder();
  if (encode == NULL)
    return 0;
  int needW, needH;
  sampleFootprint(p, mats, count, &needW, &needH);
  if (needW <= 0 || needH <= 0)
    return 0;
  const int align = pix >= 16 ? 1 : 16 / pix;
  /* 10 % headroom over the sampled maximum, plus the alignment slack */
  int bw = ((needW + needW / 10 + 2 * align - 1) / align) * align;
  int bh = needH + needH / 10 + 1;
  const int maxW = (256 / epp / align) * align;
  if (bw > maxW)
    bw = maxW;
  if (bh > 256)
    bh = 256;
  while ((long)bw * bh * pix > LOLA_STAGE_MAX_BYTES && bh > 8)
    bh--;
  /* a box smaller than the sampled footprints would send most tiles down the
     load path anyway: stage only when the sampled tiles fit */
  if (bw < needW + align - 1 || bh < needH)
    return 0;
  if (bw != p->stageBoxW || bh != p->stageBoxH) {
    const LolaStoreDesc *st = &p->store;
    cuuint64_t dims[3] = { (cuuint64_t)st->pitch * epp, (cuuint64_t)st->rows,
      (cuuint64_t)p->ringSlots };
    cuuint64_t strides[2] = { (cuuint64_t)st->pitch * pix, (cuuint64_t)st->slotElems * pix };
    cuuint32_t box[3] = { (cuuint32_t)(bw * epp), (cuuint32_t)bh, 1 };
    cuuint32_t estr[3] = { 1, 1, 1 };
    CUresult r = encode(&p->stageDesc.tensorMap, dt, 3, p->d_ring, dims, strides, box, estr,
        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
      return 0;
    p->stageBoxW = bw;
    p->stageBoxH = bh;
  }
  LolaStageDesc *sd = &p->stageDesc;
  sd->boxW = bw;
  sd->boxH = bh;
  sd->align = align;
  sd->elemsPerPixel = epp;
  sd->boxBytes = bw * bh * pix;
  sd->stageBytes = (sd->boxBytes + 127) & ~127;
  sd->d_error = p->d_error;
  return 1;
}

/* Reports (and clears) a wait timeout recorded by a staged pass. */
static int checkStageError(LolaCudaPlan *p)
{
  if (!p->stagedLaunched)
    return 1;
  p->stagedLaunched = 0;
  int e = 0;
  CUDA_TRY(cudaMemcpy(&e, p->d_error, sizeof(int), cudaMemcpyDeviceToHost));
  if (e != 0) {
    CUDA_TRY(cudaMemset(p->d_error, 0, sizeof(int)));
    return setError("staged pass: a shared-memory stage wait timed out (code %d)", e);
  }
  return 1;
}

/* One backprojection pass over ring slots [0, count) with the given matrices. */
static int launchPass(LolaCudaPlan *p, const double *mats, int count)
{
  LolaPassParams P;
  memset(&P, 0, sizeof(P));
  P.N = p->geom.problemSize;
  P.count = count;
  P.zBegin = p->geom.sliceBegin;
  P.zEnd = p->geom.sliceBegin + p->geom.sliceCount;
  P.voxelSize = p->geom.voxelSize;
  P.originIndex = p->geom.originIndex;
  P.accumulation = p->cfg.accumulation;
  P.voxelsPerThread = p->cfg.voxelsPerThread;
  P.rowsPerBlock = p->cfg.rowsPerBlock;
  P.countTiles = p->cfg.collectStats;
  for (int i = 0; i < count; i++)
    fillPassProj(&P.proj[i], mats + 12 * (size_t)i, p->geom.voxelSize, i);
  /* stream-ordered: the copy lands after the previous pass has read it */
  CUDA_TRY(cudaMemcpyAsync(p->d_proj, P.proj, (size_t)count * sizeof(LolaPassProj),
      cudaMemcpyHostToDevice, p->stream));
  P.projDevice = p->d_proj;
  EventPair *ev = NULL;
  if (p->cfg.collectStats) {
    if (!pushEvent(p, &ev))
      return 0;
    CUDA_TRY(cudaEventRecord(ev->start, p->stream));
  }
  const int staged = prepareStage(p, mats, count);
  const LolaStageDesc *sd = staged ? &p->stageDesc : NULL;
  unsigned long long *counters = p->cfg.collectStats ? p->d_counters : NULL;
  const int up = p->uploadChunks > 0, out = p->streamOut != NULL;
  if (!up && !out) {
    if (!joinTransfers(p))
      return 0;
    LAUNCH_TRY(lolaLaunchBackproject(&p->store, &P, sd, p->d_ring, p->d_volume, counters,
        p->stream));
    p->outValid = NULL;
  } else {
    /* chunk by chunk: each starts once its slices have landed and/or is
       copied out as soon as it is done; tiles are those of a whole pass */
    if (up && !issueUpload(p))
      return 0;
    if (!up && !joinTransfers(p))
      return 0;
    const int k = up ? p->uploadChunks : xferChunks(p);
    const size_t slice = (size_t)P.N * (size_t)P.N;
    for (int c = 0; c < k; c++) {
      int zb, ze;
      xferChunkRange(p, c, k, &zb, &ze);
      if (up)
        CUDA_TRY(cudaStreamWaitEvent(p->stream, p->upChunk[c], 0));
      if (ze <= zb)
        continue;
      LolaPassParams Pc = P;
      Pc.zBegin = P.zBegin + zb;
      Pc.zEnd = P.zBegin + ze;
      LAUNCH_TRY(lolaLaunchBackproject(&p->store, &Pc, sd, p->d_ring,
          p->d_volume + (size_t)zb * slice, counters, p->stream));
      p->stats.chunkLaunches++;
      if (out) {
        CUDA_TRY(cudaEventRecord(p->outChunk[c], p->stream));
        CUDA_TRY(cudaStreamWaitEvent(p->xferStream, p->outChunk[c], 0));
        CUDA_TRY(cudaMemcpyAsync(p->streamOut + (size_t)zb * slice,
            p->d_volume + (size_t)zb * slice, (size_t)(ze - zb) * slice * sizeof(float),
            cudaMemcpyDeviceToHost, p->xferStream));
      }
    }
    p->stats.overlappedPasses++;
    /* the plan stream has waited for every uploaded chunk */
    p->uploadChunks = 0;
    p->xferPending = 0;
    p->outValid = NULL;
    if (out) {
      CUDA_TRY(cudaEventRecord(p->xferDone, p->xferStream));
      p->xferPending = 1;
      p->outValid = p->streamOut;
      p->streamOut = NULL;
    }
  }
  if (staged) {
    p->stagedLaunched = 1;
    p->stats.stagedPasses++;
  }
  if (ev != NULL)
    CUDA_TRY(cudaEventRecord(ev->stop, p->stream));
  p->stats.passes++;
  p->stats.projections += count;
  return 1;
}

int lolaCudaPlanBackprojectDevice(LolaCudaPlan *p, const float *d_images, size_t imageStride,
    const double *h_mats, int count)
{
  if (p == NULL)
    return setError("null plan");
  if (count < 0)
    return setError("negative projection count");
  if (count == 0)
    return 1;  /* nothing to read: the pointers may be null */
  if (d_images == NULL || h_mats == NULL)
    return setError("null argument");
  if (p->pending != 0)
    return setError("host-staged projections pending; synchronize the plan first");
  CUDA_TRY(cudaSetDevice(p->device));
  /* a pending stream-out request belongs to the call's last pass */
  float *out = p->streamOut;
  p->streamOut = NULL;
  for (int done = 0; done < count;) {
    const int n = (count - done < p->cfg.batch) ? count - done : p->cfg.batch;
    LAUNCH_TRY(lolaLaunchPack(&p->store, d_images + (size_t)done * imageStride, imageStride,
        p->d_ring, 0, n, p->stream));
    p->stats.packs++;
    if (done + n == count)
      p->streamOut = out;
    if (!launchPass(p, h_mats + 12 * (size_t)done, n))
      return 0;
    done += n;
  }
  return 1;
}

/* Packs and backprojects the host-staged batch. */
static int flushPending(LolaCudaPlan *p)
{
  if (p->pending == 0)
    return 1;
  CUDA_TRY(cudaEventRecord(p->stageReady, p->copyStream));
  CUDA_TRY(cudaStreamWaitEvent(p->stream, p->stageReady, 0));
  LAUNCH_TRY(lolaLaunchPack(&p->store, p->d_stage, p->imageElems, p->d_ring, 0, p->pending,
      p->stream));
  p->stats.packs++;
  CUDA_TRY(cudaEventRecord(p->stageFree, p->stream));
  const int n = p->pending;
  p->pending = 0;
  return launchPass(p, &p->pendingMats[0][0], n);
}

/* Projections the next host-staged pass takes.  Edge passes take the edge
 * batch: the first pass after an asynchronous upload (it starts on each
 * z-chunk as the chunk lands, so more projections per chunk hide more of the
 * upload) and the last pass of a scan of known length (it streams each chunk
 * out as it finishes, likewise).  The pass before the last one is shortened
 * where needed so that the last one is full.  With the edge batch equal to
 * the batch every pass takes the batch, the last one what is left. */
static int passCapacity(const LolaCudaPlan *p, int left)
{
  int cap = p->uploadChunks > 0 ? p->ringSlots : p->cfg.batch;
  if (left > 0 && p->ringSlots > p->cfg.batch) {
    if (left <= p->ringSlots)
      cap = left;
    else if (cap > left - p->ringSlots)
      cap = left - p->ringSlots;
  }
  return cap;
}

int lolaPlanPassCapacity(const LolaCudaPlan *p, int left)
{
  return passCapacity(p, left);
}

int lolaPlanRingSlots(const LolaCudaPlan *p)
{
  return p->ringSlots;
}

/* Stages one host projection; flushes when the pass is complete. */
static int stageHost(LolaCudaPlan *p, const float *image, const double *matrix, int *flushed)
{
  if (p->pending == 0) {
    CUDA_TRY(cudaStreamWaitEvent(p->copyStream, p->stageFree, 0));
    p->passCap = passCapacity(p, p->scanLeft);
  }
  CUDA_TRY(cudaMemcpyAsync(p->d_stage + (size_t)p->pending * p->imageElems, image,
      p->imageElems * sizeof(float), cudaMemcpyHostToDevice, p->copyStream));
  memcpy(p->pendingMats[p->pending], matrix, 12 * sizeof(double));
  p->pending++;
  if (p->pending >= p->passCap) {
    if (!flushPending(p))
      return 0;
    *flushed = 1;
  }
  return 1;
}

int lolaCudaPlanBackprojectHost(LolaCudaPlan *p, const float *h_images, size_t imageStride,
    const double *h_mats, int count)
{
  if (p == NULL)
    return setError("null plan");
  if (count < 0)
    return setError("negative projection count");
  if (count > 0 && (h_images == NULL || h_mats == NULL))
    return setError("null argument");
  CUDA_TRY(cudaSetDevice(p->device));
  int flushed = 0;
  /* a pending stream-out request belongs to this call's last pass, the end
     of its scan: that pass takes the edge batch, and the call's earlier
     passes leave the request alone */
  float *out = p->streamOut;
  p->streamOut = NULL;
  for (int i = 0; i < count; i++) {
    p->scanLeft = out != NULL ? count - i : 0;
    if (i == count - 1)
      p->streamOut = out;
    if (!stageHost(p, h_images + (size_t)i * imageStride, h_mats + 12 * (size_t)i, &flushed)) {
      p->scanLeft = 0;
      return 0;
    }
  }
  p->scanLeft = 0;
  if (count == 0)
    p->streamOut = out;
  if (!flushPending(p))
    return 0;
  CUDA_TRY(cudaStreamSynchronize(p->copyStream));
  return 1;
}

static int collectEvents(LolaCudaPlan *p)
{
  for (int i = 0; i < p->nEvents; i++) {
    float ms = 0.0f;
    CUDA_TRY(cudaEventSynchronize(p->events[i].stop));
    CUDA_TRY(cudaEventElapsedTime(&ms, p->events[i].start, p->events[i].stop));
    p->stats.passMs += ms;
    cudaEventDestroy(p->events[i].start);
    cudaEventDestroy(p->events[i].stop);
  }
  p->nEvents = 0;
  return 1;
}

int lolaCudaPlanSynchronize(LolaCudaPlan *p)
{
  if (p == NULL)
    return setError("null plan");
  CUDA_TRY(cudaSetDevice(p->device));
  if (!flushPending(p))
    return 0;
  if (!issueUpload(p))
    return 0;
  if (p->streamOut != NULL) {
    /* no pass consumed the stream-out request: copy the volume as it is */
    if (!joinTransfers(p))
      return 0;
    CUDA_TRY(cudaMemcpyAsync(p->streamOut, p->d_volume, volumeBytes(p), cudaMemcpyDeviceToHost,
        p->stream));
    p->outValid = p->streamOut;
    p->streamOut = NULL;
  }
  CUDA_TRY(cudaStreamSynchronize(p->copyStream));
  CUDA_TRY(cudaStreamSynchronize(p->xferStream));
  CUDA_TRY(cudaStreamSynchronize(p->stream));
  p->xferPending = 0;
  p->uploadChunks = 0;
  return checkStageError(p);
}

int lolaCudaPlanTimerStart(LolaCudaPlan *p)
{
  if (p == NULL)
    return setError("null plan");
  CUDA_TRY(cudaSetDevice(p->device));
  CUDA_TRY(cudaEventRecord(p->timerStart, p->stream));
  return 1;
}

int lolaCudaPlanTimerStop(LolaCudaPlan *p, double *ms)
{
  if (p == NULL || ms == NULL)
    return setError("null argument");
  CUDA_TRY(cudaSetDevice(p->device));
  CUDA_TRY(cudaEventRecord(p->timerStop, p->stream));
  CUDA_TRY(cudaEventSynchronize(p->timerStop));
  float f = 0.0f;
  CUDA_TRY(cudaEventElapsedTime(&f, p->timerStart, p->timerStop));
  *ms = (double)f;
  return 1;
}

int lolaCudaPlanGetStats(LolaCudaPlan *p, LolaCudaStats *out)
{
  if (p == NULL || out == NULL)
    return setError("null argument");
  if (!lolaCudaPlanSynchronize(p))
    return 0;
  if (!collectEvents(p))
    return 0;
  unsigned long long all[LOLA_COUNTER_SPREAD * LOLA_TILE_COUNTERS];
  CUDA_TRY(cudaMemcpy(all, p->d_counters, sizeof(all), cudaMemcpyDeviceToHost));
  unsigned long long c[LOLA_TILE_COUNTERS] = { 0, 0, 0, 0, 0 };
  for (int i = 0; i < LOLA_COUNTER_SPREAD * LOLA_TILE_COUNTERS; i++)
    c[i % LOLA_TILE_COUNTERS] += all[i];
  p->stats.tilePassesSkipped = (int64_t)c[0];
  p->stats.tilePassesFast = (int64_t)c[1];
  p->stats.tilePassesSlow = (int64_t)c[2];
  p->stats.tilePassesStaged = (int64_t)c[3];
  p->stats.tilePassesPaired = (int64_t)c[4];
  *out = p->stats;
  return 1;
}

int lolaCudaPlanResetStats(LolaCudaPlan *p)
{
  if (p == NULL)
    return setError("null plan");
  if (!lolaCudaPlanSynchronize(p) || !collectEvents(p))
    return 0;
  memset(&p->stats, 0, sizeof(p->stats));
  CUDA_TRY(cudaMemset(p->d_counters, 0,
      LOLA_COUNTER_SPREAD * LOLA_TILE_COUNTERS * sizeof(unsigned long long)));
  return 1;
}

/* ---- autotuning ------------------------------------------------------------------ */

int lolaCudaAutotune(const LolaCudaGeometry *g, const float *d_images, size_t imageStride,
    const double *h_mats, int count, LolaCudaConfig *cfg, LolaCudaTuneReport *report)
{
  if (g == NULL || d_images == NULL || h_mats == NULL || cfg == NULL || count <= 0)
    return setError("autotune: invalid arguments");
  static const int shapes[][2] = { { 8, 8 }, { 8, 4 }, { 16, 4 }, { 16, 8 }, { 4, 8 } };
  static const int batches[] = { 8, 16, 32, 64 };
  LolaCudaTuneReport local;
  LolaCudaTuneReport *r = report ? report : &local;
  memset(r, 0, sizeof(*r));
  r->best = -1;
  double bestMs = 1e300;
  LolaCudaConfig best = *cfg;
  for (int si = 0; si < 5; si++)
    for (int bi = 0; bi < 3; bi++)
      for (int staging = 0; staging <= 1; staging++) {
        /* staging exists for 8 voxels per thread only */
        if (staging && shapes[si][0] != 8)
          continue;
        if (r->candidates >= LOLA_TUNE_MAX_CANDIDATES)
          break;
        LolaCudaConfig c = *cfg;
        c.voxelsPerThread = shapes[si][0];
        c.rowsPerBlock = shapes[si][1];
        c.batch = batches[bi] < count ? batches[bi] : count;
        c.staging = staging;
        c.collectStats = 0;
        LolaCudaTuneCandidate *t = &r->tried[r->candidates++];
        t->voxelsPerThread = c.voxelsPerThread;
        t->rowsPerBlock = c.rowsPerBlock;
        t->batch = c.batch;
        t->staging = staging;
        t->ms = -1.0;
        LolaCudaPlan *p = NULL;
        if (!lolaCudaPlanCreate(g, &c, &p))
          continue;
        double ms = -1.0;
        /* one warm-up, then the timed run */
        if (lolaCudaPlanBackprojectDevice(p, d_images, imageStride, h_mats, count) &&
            lolaCudaPlanSynchronize(p) && lolaCudaPlanTimerStart(p) &&
            lolaCudaPlanBackprojectDevice(p, d_images, imageStride, h_mats, count))
          lolaCudaPlanTimerStop(p, &ms);
        planRelease(p);
        t->ms = ms;
        if (ms > 0.0 && ms < bestMs) {
          bestMs = ms;
          best = c;
          r->best = r->candidates - 1;
        }
      }
  if (r->best < 0)
    return setError("autotune: no candidate ran");
  best.collectStats = cfg->collectStats;
  *cfg = best;
  return 1;
}

/* ---- device helpers ------------------------------------------------------------ */

void *lolaCudaDeviceAlloc(size_t bytes)
{
  void *d = NULL;
  cudaError_t e = cudaMalloc(&d, bytes);
  if (e != cudaSuccess) {
    setError("cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    return NULL;
  }
  return d;
}

int lolaCudaDeviceFree(void *d)
{
  CUDA_TRY(cudaFree(d));
  return 1;
}

int lolaCudaCopyToDevice(void *d, const void *h, size_t bytes)
{
  CUDA_TRY(cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice));
  return 1;
}

int lolaCudaCopyToHost(void *h, const void *d, size_t bytes)
{
  CUDA_TRY(cudaMemcpy(h, d, bytes, cudaMemcpyDeviceToHost));
  return 1;
}

int lolaCudaDeviceSynchronize(void)
{
  CUDA_TRY(cudaDeviceSynchronize());
  return 1;
}

/* ---- RabbitCT module API ------------------------------------------------------- */

static LolaCudaPlan *gPlan = NULL;
static uint32_t gTotalProjections = 0; /* known with -a (src/rabbitRunner.c:209-210) */
static int gVolumePinned = 0;          /* volumeData is page-locked host memory */

static int moduleFail(const char *where)
{
  LolaCudaConfig c;
  lolaCudaGetConfig(&c);
  fprintf(stderr, "LolaCUDA %s: %s\n", where, gLastError);
  fflush(stderr);
  if (c.exitOnError)
    exit(EXIT_FAILURE);
  return 0;
}

int lolaCudaPrepare(RabbitCtGlobalData *d)
{
  LolaCudaConfig c;
  lolaCudaGetConfig(&c);
  if (d == NULL) {
    setError("null global data");
    return moduleFail("prepare");
  }
  if (gPlan != NULL) {
    planRelease(gPlan);
    gPlan = NULL;
  }
  LolaCudaGeometry g;
  g.problemSize = (int32_t)d->problemSize;
  g.imageWidth = (int32_t)d->imageWidth;
  g.imageHeight = (int32_t)d->imageHeight;
  g.voxelSize = d->voxelSize;
  g.originIndex = d->O_Index;
  g.sliceBegin = 0;
  g.sliceCount = 0;
  if (d->volumeData == NULL) {
    setError("volumeData is null");
    return moduleFail("prepare");
  }
  if (!lolaCudaPlanCreate(&g, &c, &gPlan))
    return moduleFail("prepare");
  /* the module accumulates into whatever the caller's volume holds, like
     LolaBunny's `+=` (src/LolaBunny.c:68); the upload is issued with the
     first pass, after the projections it reads, and that pass starts on each
     z-chunk as it lands (the runner leaves volumeData alone until finish) */
  if (!lolaCudaPlanUploadVolumeAsync(gPlan, d->volumeData))
    return moduleFail("prepare");
  gTotalProjections = d->numberOfProjections;
  struct cudaPointerAttributes attr;
  gVolumePinned = cudaPointerGetAttributes(&attr, d->volumeData) == cudaSuccess &&
                  attr.type == cudaMemoryTypeHost;
  cudaGetLastError(); /* an unknown pointer is not an error here */
  return 1;
}

int lolaCudaBackprojection(RabbitCtGlobalData *d)
{
  if (gPlan == NULL) {
    setError("backprojection called before prepare");
    return moduleFail("backprojection");
  }
  if (d == NULL || (d->numberOfProjections > 0 && d->projectionBuffer == NULL)) {
    setError("no projection buffer");
    return moduleFail("backprojection");
  }
  if ((int32_t)d->imageWidth != gPlan->geom.imageWidth ||
      (int32_t)d->imageHeight != gPlan->geom.imageHeight ||
      (int32_t)d->problemSize != gPlan->geom.problemSize) {
    setError("geometry changed between prepare and backprojection");
    return moduleFail("backprojection");
  }
  LolaCudaPlan *p = gPlan;
  if (cudaSetDevice(p->device) != cudaSuccess) {
    setError("cudaSetDevice failed");
    return moduleFail("backprojection");
  }
  int flushed = 0, closesScan = 0;
  for (uint32_t i = 0; i < d->numberOfProjections; i++) {
    const Projection *pr = &d->projectionBuffer[i];
    if (pr->image == NULL || pr->matrix == NULL) {
      setError("projection %u has no image or matrix", i);
      return moduleFail("backprojection");
    }
    const int last = gTotalProjections > 0 && pr->id >= (int)gTotalProjections;
    p->scanLeft = gTotalProjections > 0 && pr->id >= 1 && pr->id <= (int)gTotalProjections
        ? (int)gTotalProjections - pr->id + 1 : 0;
    /* the scan's last pass copies the volume out chunk by chunk as it
       finishes them, overlapping the download with the pass's tail; only
       into page-locked memory, where the copies do not hold up this (timed)
       call — a pageable volume is copied in the untimed finish as before */
    if (last && gVolumePinned && !lolaCudaPlanStreamVolumeOut(p, d->volumeData))
      return moduleFail("backprojection");
    if (!stageHost(p, pr->image, pr->matrix, &flushed))
      return moduleFail("backprojection");
    /* the last view of the scan closes the pass, so no work is left for the
       untimed finish (src/rabbitRunner.c:287) */
    if (last && p->pending > 0) {
      if (!flushPending(p))
        return moduleFail("backprojection");
      flushed = 1;
    }
    closesScan |= last;
  }
  /* the runner reuses its buffers after we return (src/rabbitRunner.c:275-278) */
  if (cudaStreamSynchronize(p->copyStream) != cudaSuccess) {
    setError("upload failed: %s", cudaGetErrorString(cudaGetLastError()));
    return moduleFail("backprojection");
  }
  /* the call that closes the scan waits for every pass even without
     syncEachCall: the runner's timer around the calls then covers all of the
     backprojection work, whatever the earlier calls left running */
  if (flushed && (p->cfg.syncEachCall || closesScan)) {
    cudaError_t e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) {
      setError("pass failed: %s", cudaGetErrorString(e));
      return moduleFail("backprojection");
    }
    if (!checkStageError(p))
      return moduleFail("backprojection");
  }
  return 1;
}

int lolaCudaFinish(RabbitCtGlobalData *d)
{
  if (gPlan == NULL) {
    setError("finish called before prepare");
    return moduleFail("finish");
  }
  if (d == NULL || d->volumeData == NULL) {
    setError("volumeData is null");
    return moduleFail("finish");
  }
  LolaCudaPlan *p = gPlan;
  /* without the scan length (no -a) the last call cannot know it is the last,
     so its pass runs here, outside the runner's timer: say so */
  if (p->pending > 0 && gTotalProjections == 0) {
    fprintf(stderr, "LolaCUDA finish: the last %d projection(s) were backprojected in finish, "
                    "outside the timed calls (run with -a to close the scan in its last call)\n",
        p->pending);
    fflush(stderr);
  }
  /* unless the last pass already streamed the volume out, the closing pass
     (or, with none pending, a plain copy) delivers it */
  if ((p->pending > 0 || p->outValid != d->volumeData) &&
      !lolaCudaPlanStreamVolumeOut(p, d->volumeData))
    return moduleFail("finish");
  if (!lolaCudaPlanSynchronize(p))
    return moduleFail("finish");
  if (p->outValid != d->volumeData && !lolaCudaPlanDownloadVolume(p, d->volumeData))
    return moduleFail("finish");
  planRelease(gPlan);
  gPlan = NULL;
  gTotalProjections = 0;
  return 1;
}
