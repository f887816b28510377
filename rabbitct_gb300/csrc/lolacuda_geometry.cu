/* Geometry analysis on the device: the x-line clipping table of the
 * reference's computeLineRanges (HPC-Dwarfs/RabbitCT
 * src/analyseGeometry.c:102-298) and the projection shadow
 * (computeShadowOfProjection, src/analyseGeometry.c:50-93).
 *
 * computeLineRanges scans every (view, z, y) row from both ends in FP64 until
 * a voxel "hits" the detector — O(N) evaluations per empty row, minutes at
 * N=1024 — and caches the 2 GB result in a file keyed only on N and the
 * vector width.  Here one thread handles one row:
 *   1. solve, in FP64, the interval of world x where the hit test holds: u and
 *      v are ratios of linear functions of x (w > 0), so each bound on u or v
 *      is a half-line in x and the hit set is an interval;
 *   2. decide the first and last hit exactly with the reference's own test
 *      (same float wx = x*mm + O, float-accumulated wy and wz, FP64
 *      projection, C truncation, the reference's unsigned comparison unless
 *      signedHit) in a window of +-2 voxels around each analytic bound;
 *   3. rows where the analysis does not apply (w not positive along the row)
 *      are scanned in full, exactly as the reference does.
 * The same alignment widening to a multiple of the vector width follows
 * (src/analyseGeometry.c:270-275).  Output is identical to the reference's.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime.h>

#include "lolaCuda.h"
#include "lolacuda_internal.h"

namespace {

struct RowArgs {
  const double *mats;   /* views x 12 */
  const float *wseq;    /* N floats: the reference's float-accumulated O + k*mm */
  int16_t *out;         /* views x N*N x 2 */
  int N, W, H, views, vectorSize, signedHit;
  float mm, o;
};

/* a0*x + a1*y + a2*z + a3 with C's left-to-right evaluation and a rounding
 * after every operation (no contraction), as the reference's FP64 expressions */
__device__ __forceinline__ double affine(double a0, double x, double a1, double y, double a2,
    double z, double a3)
{
  return __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(a0, x), __dmul_rn(a1, y)), __dmul_rn(a2, z)),
      a3);
}

__device__ __forceinline__ bool hits(const double *a, float wx, float wy, float wz, int W, int H,
    int signedHit)
{
  const double x = wx, y = wy, z = wz;
  const double w = affine(a[2], x, a[5], y, a[8], z, a[11]);
  const double u = __ddiv_rn(affine(a[0], x, a[3], y, a[6], z, a[9]), w);
  const double v = __ddiv_rn(affine(a[1], x, a[4], y, a[7], z, a[10]), w);
  const int iix = __double2int_rz(u), iiy = __double2int_rz(v);
  if (signedHit)
    return !((iix + 1 < 0) || (iix > W - 1) || (iiy + 1 < 0) || (iiy > H - 1));
  /* the reference compares with `unsigned isx - 1`: negative indices miss */
  return !((iix + 1 < 0) || ((unsigned)iix > (unsigned)W - 1u) || (iiy + 1 < 0) ||
           ((unsigned)iiy > (unsigned)H - 1u));
}

/* Intersects [lo, hi] with {x : p*x + q > 0}. */
__device__ __forceinline__ void cut(double p, double q, double &lo, double &hi)
{
  if (p > 0.0)
    lo = fmax(lo, -q / p);
  else if (p < 0.0)
    hi = fmin(hi, -q / p);
  else if (!(q > 0.0))
    hi = -INFINITY;
}

__global__ void __launch_bounds__(256) lineRangeKernel(const RowArgs r)
{
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  const int z = blockIdx.y;
  const int view = blockIdx.z;
  if (y >= r.N)
    return;
  const double *a = r.mats + 12 * (size_t)view;
  const float wy = r.wseq[y], wz = r.wseq[z];
  const int N = r.N;
  const float mm = r.mm, o = r.o;
  /* wx = x * mm + O in float, two roundings (src/analyseGeometry.c:231,257) */
  auto wxOf = [&](int x) { return __fadd_rn(__fmul_rn((float)x, mm), o); };

  int xstart = -1, xstop = -1;
  /* row terms of u, v, w as functions of world x */
  const double Y = wy, Z = wz;
  const double cu = a[3] * Y + a[6] * Z + a[9];
  const double cv = a[4] * Y + a[7] * Z + a[10];
  const double cw = a[5] * Y + a[8] * Z + a[11];
  const double x0 = wxOf(0), x1 = wxOf(N - 1);
  const bool wPositive = (a[2] * x0 + cw > 0.0) && (a[2] * x1 + cw > 0.0);
  if (wPositive) {
    /* hit  <=>  lo_u < u < hi_u  and  lo_v < v < hi_v  (truncation toward
       zero: trunc(u) in [first, last] <=> u in (first - 1, last + 1)) */
    const double firstU = r.signedHit ? -1.0 : 0.0, lastU = (double)(r.W - 1);
    const double firstV = r.signedHit ? -1.0 : 0.0, lastV = (double)(r.H - 1);
    double lo = -INFINITY, hi = INFINITY;
    cut(a[0] - (firstU - 1.0) * a[2], cu - (firstU - 1.0) * cw, lo, hi);
    cut((lastU + 1.0) * a[2] - a[0], (lastU + 1.0) * cw - cu, lo, hi);
    cut(a[1] - (firstV - 1.0) * a[2], cv - (firstV - 1.0) * cw, lo, hi);
    cut((lastV + 1.0) * a[2] - a[1], (lastV + 1.0) * cw - cv, lo, hi);
    /* voxel-index window of the analytic interval, widened by 2 voxels: FP64
       rounding can move the test's outcome only at the interval's ends */
    const double il = fmin(fmax((lo - (double)o) / (double)mm, -4.0), (double)N + 3.0);
    const double ih = fmin(fmax((hi - (double)o) / (double)mm, -4.0), (double)N + 3.0);
    int xl = (int)floor(il) - 2, xh = (int)ceil(ih) + 2;
    if (!(lo <= hi + 1e-3 * (double)mm))
      xh = xl - 1; /* empty by more than rounding can bridge */
    xl = max(xl, 0);
    xh = min(xh, N - 1);
    for (int x = xl; x <= xh; ++x)
      if (hits(a, wxOf(x), wy, wz, r.W, r.H, r.signedHit)) {
        xstart = x;
        break;
      }
    if (xstart >= 0)
      for (int x = xh; x >= xstart; --x)
        if (hits(a, wxOf(x), wy, wz, r.W, r.H, r.signedHit)) {
          xstop = x + 1;
          break;
        }
  } else {
    /* the reference's own scan (src/analyseGeometry.c:229-268) */
    for (int x = 0; x < N; ++x)
      if (hits(a, wxOf(x), wy, wz, r.W, r.H, r.signedHit)) {
        xstart = x;
        break;
      }
    if (xstart >= 0)
      for (int x = N - 1; x >= 0; --x)
        if (hits(a, wxOf(x), wy, wz, r.W, r.H, r.signedHit)) {
          xstop = x + 1;
          break;
        }
  }
  int16_t *o2 = r.out + 2 * ((size_t)view * N * N + (size_t)z * N + y);
  if (xstart < 0) {
    o2[0] = 0;
    o2[1] = 0;
    return;
  }
  const int vsz = r.vectorSize;
  int align;
  if ((align = xstop % vsz))
    xstop += vsz - align;
  if ((align = xstart % vsz))
    xstart -= align;
  o2[0] = (int16_t)xstart;
  o2[1] = (int16_t)xstop;
}

} /* namespace */

/* Device version of computeLineRanges over data->numberOfProjections views of
 * data->globalGeometry; range[view] receives N*N {start, stop} int16 pairs
 * (row z*N + y), the reference's LineRangeType table. */
extern "C" int lolaCudaComputeLineRanges(const RabbitCtGlobalData *data, int16_t **range,
    int vectorSize, int signedHit)
{
  if (data == nullptr || range == nullptr || data->globalGeometry == nullptr)
    return lolaSetError("line ranges: null argument");
  const int N = (int)data->problemSize, views = (int)data->numberOfProjections;
  if (N <= 0 || N > 32767 || views <= 0 || vectorSize <= 0)
    return lolaSetError("line ranges: invalid N=%d views=%d vector size=%d", N, views,
        vectorSize);
  for (int v = 0; v < views; ++v)
    if (range[v] == nullptr)
      return lolaSetError("line ranges: range[%d] is null", v);
  /* the reference accumulates wz and wy in float: wz += mm from O_Index */
  float *wseq = (float *)malloc((size_t)N * sizeof(float));
  if (wseq == nullptr)
    return lolaSetError("line ranges: out of host memory");
  float acc = data->O_Index;
  for (int i = 0; i < N; ++i, acc += data->voxelSize)
    wseq[i] = acc;
  const size_t rowsPerView = (size_t)N * N;
  /* bounded device footprint: views in chunks of ~256 MB of output */
  int chunk = (int)((256u << 20) / (rowsPerView * 4));
  chunk = chunk < 1 ? 1 : (chunk > views ? views : chunk);
  double *d_mats = nullptr;
  float *d_wseq = nullptr;
  int16_t *d_out = nullptr;
  int ok = 1;
  cudaError_t e = cudaMalloc(&d_mats, (size_t)views * 12 * sizeof(double));
  if (e == cudaSuccess)
    e = cudaMalloc(&d_wseq, (size_t)N * sizeof(float));
  if (e == cudaSuccess)
    e = cudaMalloc(&d_out, (size_t)chunk * rowsPerView * 2 * sizeof(int16_t));
  if (e == cudaSuccess)
    e = cudaMemcpy(d_mats, data->globalGeometry, (size_t)views * 12 * sizeof(double),
        cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(d_wseq, wseq, (size_t)N * sizeof(float), cudaMemcpyHostToDevice);
  for (int v0 = 0; e == cudaSuccess && v0 < views; v0 += chunk) {
    const int nv = (views - v0 < chunk) ? views - v0 : chunk;
    RowArgs r;
    r.mats = d_mats + 12 * (size_t)v0;
    r.wseq = d_wseq;
    r.out = d_out;
    r.N = N;
    r.W = (int)data->imageWidth;
    r.H = (int)data->imageHeight;
    r.views = nv;
    r.vectorSize = vectorSize;
    r.signedHit = signedHit;
    r.mm = data->voxelSize;
    r.o = data->O_Index;
    const dim3 grid((N + 255) / 256, N, nv);
    (void)cudaGetLastError();  /* report this launch's error, not an earlier one */
    lineRangeKernel<<<grid, 256>>>(r);
    e = cudaGetLastError();
    for (int v = 0; e == cudaSuccess && v < nv; ++v)
      e = cudaMemcpy(range[v0 + v], d_out + 2 * (size_t)v * rowsPerView,
          rowsPerView * 2 * sizeof(int16_t), cudaMemcpyDeviceToHost);
  }
  if (e != cudaSuccess)
    ok = lolaSetError("line ranges: %s", cudaGetErrorString(e));
  cudaFree(d_mats);
  cudaFree(d_wseq);
  cudaFree(d_out);
  free(wseq);
  return ok;
}

/* computeShadowOfProjection (src/analyseGeometry.c:50-93): floor/ceil of the
 * u/v bounding box of the 8 volume corners over all views; shadow = {Umin,
 * Umax, Vmin, Vmax}.  8 x views FP64 projections: computed on the host. */
extern "C" int lolaCudaComputeShadow(const RabbitCtGlobalData *data, int *shadow)
{
  if (data == nullptr || shadow == nullptr || data->globalGeometry == nullptr)
    return lolaSetError("shadow: null argument");
  const int N = (int)data->problemSize;
  const double rL = data->voxelSize, oL = data->O_Index;
  double minU = data->imageWidth + 1.0, minV = data->imageHeight + 1.0;
  double maxU = -2.0, maxV = -2.0;
  for (uint32_t view = 0; view < data->numberOfProjections; ++view) {
    const double *a = data->globalGeometry + 12 * (size_t)view;
    for (int c = 0; c < 8; ++c) {
      const double x = oL + (double)((c & 1) ? N - 1 : 0) * rL;
      const double y = oL + (double)((c & 2) ? N - 1 : 0) * rL;
      const double z = oL + (double)((c & 4) ? N - 1 : 0) * rL;
      const double w = a[2] * x + a[5] * y + a[8] * z + a[11];
      const double u = (a[0] * x + a[3] * y + a[6] * z + a[9]) / w;
      const double v = (a[1] * x + a[4] * y + a[7] * z + a[10]) / w;
      minU = u < minU ? u : minU;
      minV = v < minV ? v : minV;
      maxU = u > maxU ? u : maxU;
      maxV = v > maxV ? v : maxV;
    }
  }
  shadow[0] = (int)floor(minU);
  shadow[1] = (int)ceil(maxU);
  shadow[2] = (int)floor(minV);
  shadow[3] = (int)ceil(maxV);
  return 1;
}
