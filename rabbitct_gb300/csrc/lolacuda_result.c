/* The reference runner's optional outputs, written from a plan's device volume
 * (C99).
 *
 *  - PGM slice (-p, reference src/rabbitRunner.c:289-315): slice N/2-1 of the
 *    FP32 volume in Hounsfield units, 16-bit big-endian, maxval 4095.
 *  - result.rctd (-c, src/rabbitRunner.c:317-412): magic 591984, problem
 *    size, image count, one uint64 time in microseconds per image (the mean),
 *    slice N/2-1 in HU as FP32, MSE and maximum absolute error (FP64), the
 *    11-bin error histogram (uint32), magic 489195.
 *
 * Only the slice leaves the device; the metrics come from the device
 * verification pass.  HU = floor(hus0 * v + hus1 + 0.5) for v > 0 else 0,
 * clamped to 4095, rounded after each operation (this file is compiled with
 * floating-point contraction off).
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "lolaCuda.h"
#include "lolacuda_internal.h"

static float toHu(float v, const float *hus)
{
  if (!(v > 0.0f))
    return 0.0f;
  float t = hus[0] * v;
  t = t + hus[1];
  t = t + 0.5f;
  const float h = floorf(t);
  return h > 4095.0f ? 4095.0f : h;
}

/* Copies slice z (absolute index) of the plan's volume to the host. */
static float *downloadSlice(LolaCudaPlan *plan, int z)
{
  const LolaCudaGeometry *g = lolaPlanGeometry(plan);
  if (z < g->sliceBegin || z >= g->sliceBegin + g->sliceCount) {
    lolaSetError("slice %d is not held by the plan (slab %d..%d)", z, g->sliceBegin,
        g->sliceBegin + g->sliceCount - 1);
    return NULL;
  }
  if (!lolaCudaPlanSynchronize(plan))
    return NULL;
  const size_t area = (size_t)g->problemSize * (size_t)g->problemSize;
  float *h = (float *)malloc(area * sizeof(float));
  if (h == NULL) {
    lolaSetError("out of host memory");
    return NULL;
  }
  cudaStream_t st = (cudaStream_t)lolaCudaPlanStream(plan);
  const float *d = lolaCudaPlanVolume(plan) + (size_t)(z - g->sliceBegin) * area;
  cudaError_t e = cudaMemcpyAsync(h, d, area * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    free(h);
    lolaSetError("slice download: %s", cudaGetErrorString(e));
    return NULL;
  }
  return h;
}

int lolaCudaPlanWriteSlicePgm(LolaCudaPlan *plan, const char *path, const float *hus)
{
  if (plan == NULL || path == NULL || hus == NULL)
    return lolaSetError("write pgm: null argument");
  const int n = lolaPlanGeometry(plan)->problemSize;
  float *slice = downloadSlice(plan, n / 2 - 1);
  if (slice == NULL)
    return 0;
  const size_t area = (size_t)n * (size_t)n;
  unsigned char *row = (unsigned char *)malloc(area * 2);
  FILE *f = row ? fopen(path, "wb") : NULL;
  int ok = f != NULL;
  if (ok) {
    for (size_t i = 0; i < area; ++i) {
      /* through int32 like the reference's float -> uint16 conversion on
         x86 (a negative HU wraps instead of saturating) */
      const uint16_t v = (uint16_t)(int32_t)toHu(slice[i], hus);
      row[2 * i] = (unsigned char)(v >> 8);
      row[2 * i + 1] = (unsigned char)(v & 0xff);
    }
    ok = fprintf(f, "P5\n%d %d\n4095\n", n, n) > 0 && fwrite(row, 2, area, f) == area;
    ok = (fclose(f) == 0) && ok;
  }
  free(row);
  free(slice);
  return ok ? 1 : lolaSetError("write pgm: cannot write %s", path);
}

int lolaCudaPlanWriteResult(LolaCudaPlan *plan, const char *path, const uint16_t *h_reference,
    const float *hus, uint32_t numberOfImages, uint64_t totalMicroseconds,
    LolaCudaQuality *quality)
{
  if (plan == NULL || path == NULL || h_reference == NULL || hus == NULL)
    return lolaSetError("write result: null argument");
  const LolaCudaGeometry *g = lolaPlanGeometry(plan);
  const int n = g->problemSize;
  if (g->sliceBegin != 0 || g->sliceCount != n)
    return lolaSetError("write result: the plan must hold the whole volume");
  if (numberOfImages == 0)
    return lolaSetError("write result: no images");
  LolaCudaQuality q;
  /* the runner converts the volume to HU in place while it checks it */
  if (!lolaCudaPlanVerify(plan, h_reference, hus, 1, &q))
    return 0;
  float *slice = downloadSlice(plan, n / 2 - 1);
  if (slice == NULL)
    return 0;
  const size_t area = (size_t)n * (size_t)n;
  const int32_t magic = 591984, magicEnd = 489195, size = n;
  const uint64_t mean = totalMicroseconds / numberOfImages;
  uint32_t hist[11];
  for (int i = 0; i < 11; ++i)
    hist[i] = (uint32_t)q.histogram[i];
  FILE *f = fopen(path, "wb");
  int ok = f != NULL;
  if (ok) {
    ok = fwrite(&magic, 4, 1, f) == 1 && fwrite(&size, 4, 1, f) == 1 &&
         fwrite(&numberOfImages, 4, 1, f) == 1;
    for (uint32_t i = 0; ok && i < numberOfImages; ++i)
      ok = fwrite(&mean, 8, 1, f) == 1;
    ok = ok && fwrite(slice, sizeof(float), area, f) == area && fwrite(&q.mse, 8, 1, f) == 1 &&
         fwrite(&q.maxAbs, 8, 1, f) == 1 && fwrite(hist, 4, 11, f) == 11 &&
         fwrite(&magicEnd, 4, 1, f) == 1;
    ok = (fclose(f) == 0) && ok;
  }
  free(slice);
  if (!ok)
    return lolaSetError("write result: cannot write %s", path);
  if (quality != NULL)
    *quality = q;
  return 1;
}
