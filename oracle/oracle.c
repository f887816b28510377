/* ORACLE — test infrastructure only.
 *
 * CPU restatements of RabbitCT's backprojection (HPC-Dwarfs/RabbitCT), used
 * as the checker for the CUDA path and as the timed CPU baseline.  Only the
 * tests, the smoke check and the benchmark's CPU-baseline arm may load this
 * library; the product never links or calls it.
 *
 * Pinning: the restatements are checked against the reference's own
 * LolaBunny / LolaOPT / computeLineRanges built from its unmodified sources
 * (oracle/ref.mk -> oracle/_ref/libref.so) and against golden fixtures made
 * from that build (tests/golden/make_golden.py).  The reference ships no test
 * vectors of its own.
 *
 * Functions and the reference lines they follow:
 *   oracleBunnyF64        src/LolaBunny.c:11-30 (pN, pHatN), :44-75 (loops),
 *                         with the accumulation kept in FP64 (error baseline)
 *   oracleBunnyF32        the same, accumulating (float)(1/w^2 * pHatN) into
 *                         an FP32 volume exactly as src/LolaBunny.c:68 does
 *   oracleShadow          src/analyseGeometry.c:50-93
 *   oracleLineRanges      src/analyseGeometry.c:229-275 (scan + alignment);
 *                         `signedHit` = 0 keeps the reference's unsigned
 *                         comparison (iix = -1 counts as a miss), 1 uses the
 *                         signed test that matches LolaBunny's support
 *   (the LolaOPT port used as the timed CPU baseline is in oracle_opt.c)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- LolaBunny, FP64 --------------------------------------------------- */

static inline double tapN(const float *img, int W, int H, int i, int j)
{
  /* pN: zero outside [0,W) x [0,H)  (src/LolaBunny.c:11-17) */
  if (i >= 0 && i < W && j >= 0 && j < H)
    return (double)img[(size_t)j * (size_t)W + (size_t)i];
  return 0.0;
}

static inline double hatN(const float *img, int W, int H, double x, double y)
{
  /* pHatN: C truncation toward zero, product-form bilinear weights
     (src/LolaBunny.c:19-30) */
  const int i = (int)x;
  const int j = (int)y;
  const double alpha = x - (double)i;
  const double beta = y - (double)j;
  return (1.0 - alpha) * (1.0 - beta) * tapN(img, W, H, i, j) +
         alpha * (1.0 - beta) * tapN(img, W, H, i + 1, j) +
         (1.0 - alpha) * beta * tapN(img, W, H, i, j + 1) +
         alpha * beta * tapN(img, W, H, i + 1, j + 1);
}

/* contribution of one view to voxel (i, j, k) in FP64, as LolaBunny forms it */
static inline double bunnyTerm(const double *a, const float *img, int W, int H,
    double x, double y, double z)
{
  const double w = a[2] * x + a[5] * y + a[8] * z + a[11];
  const double u = (a[0] * x + a[3] * y + a[6] * z + a[9]) / w;
  const double v = (a[1] * x + a[4] * y + a[7] * z + a[10]) / w;
  return 1.0 / (w * w) * hatN(img, W, H, u, v);
}

/* vol (N^3 doubles, x fastest) += sum over views, summed in FP64.
 * Views are applied in order 0..nproj-1 to every voxel, like the reference. */
void oracleBunnyF64(int N, float voxelSize, float originIndex, int W, int H, int nproj,
    const double *mats, const float *images, double *vol)
{
  const size_t img = (size_t)W * (size_t)H;
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < N; k++) {
    const double z = (double)originIndex + (double)k * (double)voxelSize;
    for (int j = 0; j < N; j++) {
      const double y = (double)originIndex + (double)j * (double)voxelSize;
      double *line = vol + ((size_t)k * N + j) * (size_t)N;
      for (int i = 0; i < N; i++) {
        const double x = (double)originIndex + (double)i * (double)voxelSize;
        double acc = line[i];
        for (int p = 0; p < nproj; p++)
          acc += bunnyTerm(mats + 12 * (size_t)p, images + img * p, W, H, x, y, z);
        line[i] = acc;
      }
    }
  }
}

/* vol (N^3 floats) += (float)(term) per view, exactly LolaBunny's update. */
void oracleBunnyF32(int N, float voxelSize, float originIndex, int W, int H, int nproj,
    const double *mats, const float *images, float *vol)
{
  const size_t img = (size_t)W * (size_t)H;
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < N; k++) {
    const double z = (double)originIndex + (double)k * (double)voxelSize;
    for (int j = 0; j < N; j++) {
      const double y = (double)originIndex + (double)j * (double)voxelSize;
      float *line = vol + ((size_t)k * N + j) * (size_t)N;
      for (int i = 0; i < N; i++) {
        const double x = (double)originIndex + (double)i * (double)voxelSize;
        float acc = line[i];
        for (int p = 0; p < nproj; p++)
          acc += (float)bunnyTerm(mats + 12 * (size_t)p, images + img * p, W, H, x, y, z);
        line[i] = acc;
      }
    }
  }
}

/* LolaBunny at selected voxels only (flattened indices k*N*N + j*N + i), for
 * error statistics of full-size volumes.  fp32Accumulate = 0 sums in FP64;
 * 1 accumulates (float)(term) per view in FP32 like src/LolaBunny.c:68.
 * out[q] starts from zero. */
void oracleBunnyPoints(int N, float voxelSize, float originIndex, int W, int H, int nproj,
    const double *mats, const float *images, int npts, const int64_t *index, int fp32Accumulate,
    double *out)
{
  const size_t img = (size_t)W * (size_t)H;
  const int64_t NN = (int64_t)N * N;
#pragma omp parallel for schedule(dynamic, 16)
  for (int q = 0; q < npts; q++) {
    const int64_t id = index[q];
    const int k = (int)(id / NN), j = (int)((id / N) % N), i = (int)(id % N);
    const double x = (double)originIndex + (double)i * (double)voxelSize;
    const double y = (double)originIndex + (double)j * (double)voxelSize;
    const double z = (double)originIndex + (double)k * (double)voxelSize;
    double acc = 0.0;
    float acc32 = 0.0f;
    for (int p = 0; p < nproj; p++) {
      const double t = bunnyTerm(mats + 12 * (size_t)p, images + img * p, W, H, x, y, z);
      acc += t;
      acc32 += (float)t;
    }
    out[q] = fp32Accumulate ? (double)acc32 : acc;
  }
}

/* ---- geometry analysis ---------------------------------------------------- */

/* shadow[4] = {Umin, Umax, Vmin, Vmax} of the 8 volume corners over all views */
void oracleShadow(int N, float voxelSize, float originIndex, int W, int H, int nproj,
    const double *mats, int *shadow)
{
  double minU = W + 1, minV = H + 1, maxU = -2, maxV = -2;
  for (int p = 0; p < nproj; p++) {
    const double *a = mats + 12 * (size_t)p;
    for (int c = 0; c < 8; c++) {
      const double x = originIndex + (double)((c & 1) ? N - 1 : 0) * voxelSize;
      const double y = originIndex + (double)((c & 2) ? N - 1 : 0) * voxelSize;
      const double z = originIndex + (double)((c & 4) ? N - 1 : 0) * voxelSize;
      const double w = a[2] * x + a[5] * y + a[8] * z + a[11];
      const double u = (a[0] * x + a[3] * y + a[6] * z + a[9]) / w;
      const double v = (a[1] * x + a[4] * y + a[7] * z + a[10]) / w;
      if (u < minU) minU = u;
      if (v < minV) minV = v;
      if (u > maxU) maxU = u;
      if (v > maxV) maxV = v;
    }
  }
  shadow[0] = (int)floor(minU);
  shadow[1] = (int)ceil(maxU);
  shadow[2] = (int)floor(minV);
  shadow[3] = (int)ceil(maxV);
}

/* Hit test of one voxel.  The reference compares the signed truncated pixel
 * index with `unsigned isx - 1` (src/analyseGeometry.c:105-106,235), so a
 * negative index converts to a huge unsigned value and counts as a miss;
 * signedHit = 1 keeps iix = -1 / iiy = -1, where LolaBunny still reads the
 * pixel at index 0 with a negative weight. */
static inline int voxelHits(const double *a, double x, double y, double z, int W, int H,
    int signedHit)
{
  const double w = a[2] * x + a[5] * y + a[8] * z + a[11];
  const double u = (a[0] * x + a[3] * y + a[6] * z + a[9]) / w;
  const double v = (a[1] * x + a[4] * y + a[7] * z + a[10]) / w;
  const int iix = (int)u, iiy = (int)v;
  if (signedHit)
    return !((iix + 1 < 0) || (iix > W - 1) || (iiy + 1 < 0) || (iiy > H - 1));
  const unsigned isx = (unsigned)W, isy = (unsigned)H;
  return !((iix + 1 < 0) || ((unsigned)iix > isx - 1) || (iiy + 1 < 0) ||
           ((unsigned)iiy > isy - 1));
}

/* ranges: nproj * N * N pairs of int16 {start, stop}, row index z*N + y.
 * Same scan order and alignment widening as the reference (start rounded down,
 * stop rounded up to a multiple of vectorSize; an all-miss row is {0, 0}). */
void oracleLineRanges(int N, float voxelSize, float originIndex, int W, int H, int nproj,
    const double *mats, int vectorSize, int signedHit, int16_t *ranges)
{
  /* the reference steps wz / wy as float accumulators (wz += mm); the same
     sequence is precomputed so rows can be scanned in parallel */
  float *wseq = (float *)malloc((size_t)N * sizeof(float));
  float acc = originIndex;
  for (int i = 0; i < N; i++, acc += voxelSize)
    wseq[i] = acc;
#pragma omp parallel for schedule(dynamic, 4) collapse(2)
  for (int p = 0; p < nproj; p++) {
    for (int z = 0; z < N; z++) {
      const double *a = mats + 12 * (size_t)p;
      const float wz = wseq[z];
      for (int y = 0; y < N; y++) {
        const float wy = wseq[y];
        int xstart = -1, xstop = -1;
        for (int x = 0; x < N; x++) {
          const float wx = x * voxelSize + originIndex;
          if (voxelHits(a, wx, wy, wz, W, H, signedHit)) {
            xstart = x;
            break;
          }
        }
        int16_t *r = ranges + 2 * ((size_t)p * N * N + (size_t)z * N + y);
        if (xstart == -1) {
          r[0] = 0;
          r[1] = 0;
          continue;
        }
        for (int x = N - 1; x >= 0; --x) {
          const float wx = x * voxelSize + originIndex;
          if (voxelHits(a, wx, wy, wz, W, H, signedHit)) {
            xstop = x + 1;
            break;
          }
        }
        int align;
        if ((align = xstop % vectorSize))
          xstop += vectorSize - align;
        if ((align = xstart % vectorSize))
          xstart -= align;
        r[0] = (int16_t)xstart;
        r[1] = (int16_t)xstop;
      }
    }
  }
  free(wseq);
}

/* Number of threads OpenMP would use (1 without OpenMP). */
int oracleThreads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
