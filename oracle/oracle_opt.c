/* ORACLE — test infrastructure only (see oracle.c for the rules).
 *
 * Port of LolaOPT's backprojection (HPC-Dwarfs/RabbitCT src/LolaOPT.c), the
 * reference's plain-C FP32 CPU method.  It is the CPU baseline that the
 * benchmark times on the host cores.  Compiled like the reference compiles
 * its modules (-O3 -ffast-math, OpenMP), without -march=native so that the
 * same source builds on x86_64 and aarch64 hosts.
 *
 *   oracleOptPadding      src/LolaOPT.c:64-73 (pad sizes from the shadow)
 *   oracleOptBackproject  src/LolaOPT.c:91-179 (padded image, FP32 row loop)
 */
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- LolaOPT port: the timed CPU baseline -------------------------------- */

/* pad[4] = {left, right, bottom, top} from the shadow, as src/LolaOPT.c:65-68
 * forms them (abs() of the shadow bounds).  Returns the padded width. */
int oracleOptPadding(const int *shadow, int W, int H, int *pad)
{
  pad[0] = abs(shadow[0]);
  pad[1] = abs(shadow[1]) - W;
  pad[2] = abs(shadow[2]);
  pad[3] = abs(shadow[3]) - H;
  return pad[0] + W + pad[1];
}

/* One call of LolaOPT's backprojection for `nproj` views whose global ids
 * (1-based) are ids[p]; ranges from oracleLineRanges over all views, padded
 * images prepared by the caller: padded[p] points to view p's zero-padded
 * buffer and `startOffset` / `lineOffset` follow src/LolaOPT.c:71-73.
 * FP32 arithmetic with the row invariants formed in FP64 and cast
 * (src/LolaOPT.c:140-142), incremental wx (:160), lerp-form bilinear
 * (:167-169). */
void oracleOptBackproject(int N, float voxelSize, float originIndex, int nproj,
    const int *ids, const double *mats, const float *const *padded, int startOffset,
    int lineOffset, const int16_t *ranges, float *vol)
{
  const int l = N;
  const float mm = voxelSize, o = originIndex;
  for (int p = 0; p < nproj; ++p) {
    const double *a = mats + 12 * (size_t)p;
    const float *img = padded[p] + startOffset;
    const int16_t *R = ranges + 2 * (size_t)(ids[p] - 1) * l * l;
#pragma omp parallel for schedule(dynamic, 16) collapse(2)
    for (int z = 0; z < l; ++z) {
      for (int y = 0; y < l; ++y) {
        const int start = R[2 * (z * l + y)];
        const int stop = R[2 * (z * l + y) + 1];
        if (stop - start == 0)
          continue;
        const float wz = z * mm + o;
        const float wy = y * mm + o;
        float wx = start * mm + o;
        float *line = vol + (size_t)z * l * l + (size_t)y * l;
        const float t0 = (float)(a[3] * wy + a[6] * wz + a[9]);
        const float t1 = (float)(a[4] * wy + a[7] * wz + a[10]);
        const float t2 = (float)(a[5] * wy + a[8] * wz + a[11]);
        for (int x = start; x < stop; ++x) {
          const float u = (float)(t0 + wx * a[0]);
          const float v = (float)(t1 + wx * a[1]);
          const float w = (float)(t2 + wx * a[2]);
          const float rcpW = 1.0f / w;
          const float rcp2W = rcpW * rcpW;
          const float ix = u * rcpW, iy = v * rcpW;
          const int iix = (int)ix, iiy = (int)iy;
          const float sx = ix - iix, sy = iy - iiy;
          wx += mm;
          const float *q = img + (ptrdiff_t)iiy * lineOffset + iix;
          const float b = (1 - sx) * q[0] + sx * q[1];
          const float t = (1 - sx) * q[lineOffset] + sx * q[lineOffset + 1];
          line[x] += ((1 - sy) * b + sy * t) * rcp2W;
        }
      }
    }
  }
}

