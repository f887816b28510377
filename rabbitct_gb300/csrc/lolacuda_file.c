/* Reconstruction straight from a RabbitCT .rct file, and the runner's module
 * loop over projections already in host memory (C99).
 *
 * File format (reference src/ctFileReader_types.h:11-15, src/ctFileReader.c:
 * 47-61): a 20-byte header {u32 width, u32 height, u32 count, f32 hus[2]},
 * then per projection 12 FP64 matrix values followed by width*height FP32
 * pixels.  The reference runner reads one record at a time between timed
 * module calls (src/rabbitRunner.c:275-279).  Here chunks of `batch` records
 * are read into two page-locked buffers in turn: while the GPU uploads and
 * backprojects chunk k (asynchronously, lolaCudaPlanBackprojectHost returns
 * once the upload is done), the host reads chunk k+1 from disk.
 */
#define _POSIX_C_SOURCE 200809L
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <cuda_runtime_api.h>

#include "lolaCuda.h"
#include "lolacuda_internal.h"

static double nowSeconds(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

typedef struct {
  uint32_t width, height, count;
  float hus[2];
} RctHeader;

int lolaCudaReadRctHeader(const char *path, uint32_t *width, uint32_t *height, uint32_t *count,
    float *hus)
{
  FILE *f = fopen(path, "rb");
  if (f == NULL)
    return lolaSetError("cannot open %s", path);
  unsigned char raw[20];
  const size_t got = fread(raw, 1, sizeof(raw), f);
  fclose(f);
  if (got != sizeof(raw))
    return lolaSetError("%s: no RabbitCT header", path);
  RctHeader h;
  memcpy(&h.width, raw, 4);
  memcpy(&h.height, raw + 4, 4);
  memcpy(&h.count, raw + 8, 4);
  memcpy(h.hus, raw + 12, 8);
  if (width)
    *width = h.width;
  if (height)
    *height = h.height;
  if (count)
    *count = h.count;
  if (hus) {
    hus[0] = h.hus[0];
    hus[1] = h.hus[1];
  }
  return 1;
}

int lolaCudaReconstructFile(const char *path, int problemSize, float voxelSize, float originIndex,
    const LolaCudaConfig *config, float *h_volume, LolaCudaFileReport *report)
{
  if (path == NULL || h_volume == NULL)
    return lolaSetError("reconstruct file: null argument");
  const double t0 = nowSeconds();
  uint32_t W, H, count;
  float hus[2];
  if (!lolaCudaReadRctHeader(path, &W, &H, &count, hus))
    return 0;
  if (W == 0 || H == 0 || count == 0)
    return lolaSetError("%s: empty scan", path);
  LolaCudaConfig c;
  if (config != NULL)
    c = *config;
  else
    lolaCudaDefaultConfig(&c);
  LolaCudaGeometry g;
  memset(&g, 0, sizeof(g));
  g.problemSize = problemSize;
  g.imageWidth = (int32_t)W;
  g.imageHeight = (int32_t)H;
  g.voxelSize = voxelSize;
  g.originIndex = originIndex;
  LolaCudaPlan *plan = NULL;
  if (!lolaCudaPlanCreate(&g, &c, &plan))
    return 0;

  /* chunks are the plan's passes: the edge batch first and last (they
     overlap the volume transfers), the batch in between */
  const int chunk = lolaPlanRingSlots(plan);
  const size_t img = (size_t)W * H;
  float *pinned[2] = { NULL, NULL };
  double *mats = (double *)malloc((size_t)2 * chunk * 12 * sizeof(double));
  FILE *f = fopen(path, "rb");
  int ok = 1;
  double readSeconds = 0.0;
  if (mats == NULL || f == NULL) {
    ok = lolaSetError("reconstruct file: cannot open %s or allocate", path);
    goto done;
  }
  for (int i = 0; i < 2; ++i)
    if (cudaHostAlloc((void **)&pinned[i], (size_t)chunk * img * sizeof(float),
            cudaHostAllocDefault) != cudaSuccess) {
      ok = lolaSetError("reconstruct file: pinned allocation failed");
      goto done;
    }
  if (fseek(f, 20, SEEK_SET) != 0) {
    ok = lolaSetError("%s: seek failed", path);
    goto done;
  }
  /* the first pass overlaps the volume upload, the last one its download */
  if (!lolaCudaPlanUploadVolumeAsync(plan, h_volume)) {
    ok = 0;
    goto done;
  }
  for (uint32_t consumed = 0, k = 0; consumed < count; ++k) {
    const uint32_t left = count - consumed;
    int n = lolaPlanPassCapacity(plan, left > (uint32_t)INT32_MAX ? 0 : (int)left);
    if ((uint32_t)n > left)
      n = (int)left;
    float *buf = pinned[k & 1];
    double *m = mats + (size_t)(k & 1) * chunk * 12;
    const double r0 = nowSeconds();
    for (int i = 0; i < n; ++i) {
      if (fread(m + 12 * (size_t)i, sizeof(double), 12, f) != 12 ||
          fread(buf + (size_t)i * img, sizeof(float), img, f) != img) {
        ok = lolaSetError("%s: truncated at projection %u", path, consumed + (uint32_t)i + 1);
        goto done;
      }
    }
    readSeconds += nowSeconds() - r0;
    if (consumed + (uint32_t)n == count && !lolaCudaPlanStreamVolumeOut(plan, h_volume)) {
      ok = 0;
      goto done;
    }
    /* returns once the chunk is on the device; its pass runs on while the
       next chunk is read into the other buffer */
    if (!lolaCudaPlanBackprojectHost(plan, buf, img, m, n)) {
      ok = 0;
      goto done;
    }
    consumed += (uint32_t)n;
  }
  if (!lolaCudaPlanSynchronize(plan))
    ok = 0;
done:
  if (f != NULL)
    fclose(f);
  /* no page-locked buffer is released while a copy from it may be pending */
  if (plan != NULL)
    lolaCudaPlanSynchronize(plan);
  for (int i = 0; i < 2; ++i)
    if (pinned[i] != NULL)
      cudaFreeHost(pinned[i]);
  free(mats);
  if (plan != NULL)
    lolaCudaPlanDestroy(plan);
  if (ok && report != NULL) {
    report->seconds = nowSeconds() - t0;
    report->readSeconds = readSeconds;
    report->projections = count;
    report->gups = (double)problemSize * problemSize * problemSize * count / report->seconds /
                   1e9;
    report->hus[0] = hus[0];
    report->hus[1] = hus[1];
  }
  return ok;
}

int lolaCudaRunScan(RabbitCtGlobalData *data, const float *h_images, size_t imageStride,
    const double *h_matrices, int count, int callBatch, LolaCudaScanTiming *timing)
{
  if (data == NULL || (count > 0 && (h_images == NULL || h_matrices == NULL)))
    return lolaSetError("run scan: null argument");
  if (count < 0 || callBatch < 1)
    return lolaSetError("run scan: count %d, call batch %d", count, callBatch);
  Projection *projs = (Projection *)malloc((size_t)callBatch * sizeof(Projection));
  if (projs == NULL)
    return lolaSetError("out of host memory");
  Projection *savedBuffer = data->projectionBuffer;
  const uint32_t savedCount = data->numberOfProjections;
  double calls = 0.0;
  const double t0 = nowSeconds();
  int ok = lolaCudaPrepare(data);
  const double t1 = nowSeconds();
  for (int done = 0; ok && done < count;) {
    const int n = (count - done < callBatch) ? count - done : callBatch;
    for (int i = 0; i < n; ++i) {
      projs[i].id = done + i + 1;
      projs[i].matrix = (double *)(h_matrices + 12 * (size_t)(done + i));
      projs[i].image = (float *)(h_images + imageStride * (size_t)(done + i));
    }
    data->projectionBuffer = projs;
    data->numberOfProjections = (uint32_t)n;
    const double c0 = nowSeconds();
    ok = lolaCudaBackprojection(data);
    calls += nowSeconds() - c0;
    done += n;
  }
  const double t2 = nowSeconds();
  ok = lolaCudaFinish(data) && ok;
  const double t3 = nowSeconds();
  data->projectionBuffer = savedBuffer;
  data->numberOfProjections = savedCount;
  free(projs);
  if (ok && timing != NULL) {
    timing->prepareSeconds = t1 - t0;
    timing->callSeconds = calls;
    timing->finishSeconds = t3 - t2;
    timing->totalSeconds = t3 - t0;
  }
  return ok;
}
