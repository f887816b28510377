/* Seeded synthetic C-arm scans in RabbitCT's data model.
 *
 * The RabbitCT rabbit dataset (496 projections of 1248x960 float32, one 3x4
 * FP64 projection matrix each; reference README.md:100-107) cannot be shipped
 * here, so every workload is synthesised with the same shapes and formats:
 *
 *   - geometry: circular scan about the volume z axis, source at distance SOD
 *     from the isocentre, flat detector at SID, square pixels of `pitch` mm,
 *     principal point at the detector centre plus a seeded jitter.  Each view
 *     is P = K [R | -R S] stored column-major, a[col*3+row], which is the
 *     layout LolaBunny reads (src/LolaBunny.c:64-66: w = a2 x + a5 y + a8 z +
 *     a11).  w is the depth of the point along the principal ray in mm.
 *   - values: analytic line integrals through seeded random ellipsoids plus
 *     per-pixel Gaussian noise from a counter-based generator, so the images
 *     do not depend on thread count or scheduling.
 *
 * Pixel (i, j) is sampled at detector coordinate (u, v) = (i, j), matching
 * LolaBunny's pN(image, i, j) = image[j*W + i] (src/LolaBunny.c:11-17).
 *
 * Everything here is plain C99 + OpenMP; results are identical on x86_64 and
 * aarch64 up to libm's last-ulp behaviour in sqrt/log/cos (the noise draw).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define RCT_SYNTH_MAX_ELLIPSOIDS 64

typedef struct {
  int32_t nproj;
  int32_t width;
  int32_t height;
  int32_t reserved;
  double sod;        /* source-isocentre distance, mm */
  double sid;        /* source-detector distance, mm */
  double pitch;      /* detector pixel pitch, mm */
  double arcDeg;     /* angular range covered by the views */
  double startDeg;   /* angle of view 0 */
  double ppJitter;   /* principal point jitter, +-px (uniform) */
  uint64_t seed;
} RctScanGeometry;

typedef struct {
  double center[3];
  double axes[3];    /* semi-axes, mm */
  double rot[9];     /* row-major rotation, body -> world */
  double density;    /* per cm of path */
} RctEllipsoid;

/* ---- counter-based random numbers (splitmix64 finaliser) ---------------- */

static inline uint64_t mix64(uint64_t z)
{
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

/* uniform in (0, 1), never 0 */
static inline double unit01(uint64_t key)
{
  return ((double)(mix64(key) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

static inline uint64_t key3(uint64_t seed, uint64_t a, uint64_t b)
{
  return mix64(seed ^ mix64(a * 0x100000001B3ULL + 0x51ED27ULL) ^ mix64(b + 0xC0FFEEULL));
}

/* ---- geometry ------------------------------------------------------------ */

void rctSynthMatrices(const RctScanGeometry *g, double *mats)
{
  const double f  = g->sid / g->pitch;
  const double cx = 0.5 * (double)(g->width - 1);
  const double cy = 0.5 * (double)(g->height - 1);
  const double deg = 3.14159265358979323846 / 180.0;

  for (int p = 0; p < g->nproj; p++) {
    const double th = (g->startDeg + g->arcDeg * (double)p / (double)g->nproj) * deg;
    const double c = cos(th), s = sin(th);
    const double cu = cx + g->ppJitter * (2.0 * unit01(key3(g->seed, 11, (uint64_t)p)) - 1.0);
    const double cv = cy + g->ppJitter * (2.0 * unit01(key3(g->seed, 12, (uint64_t)p)) - 1.0);
    /* camera axes: u along the orbit tangent, v along -z, w towards the
       isocentre; right-handed, w = depth */
    const double eu[3] = { -s, c, 0.0 };
    const double ev[3] = { 0.0, 0.0, -1.0 };
    const double ew[3] = { -c, -s, 0.0 };
    /* translation -R S with S = sod (c, s, 0) is (0, 0, sod) */
    double P[3][4];
    for (int k = 0; k < 3; k++) {
      P[0][k] = f * eu[k] + cu * ew[k];
      P[1][k] = f * ev[k] + cv * ew[k];
      P[2][k] = ew[k];
    }
    P[0][3] = cu * g->sod;
    P[1][3] = cv * g->sod;
    P[2][3] = g->sod;
    double *a = mats + 12 * (size_t)p;
    for (int col = 0; col < 4; col++)
      for (int row = 0; row < 3; row++)
        a[col * 3 + row] = P[row][col];
  }
}

/* ---- phantom ------------------------------------------------------------- */

/* Seeded random ellipsoids inside a ball of radius `radius` mm. */
int rctSynthPhantom(uint64_t seed, int count, double radius, RctEllipsoid *out)
{
  if (count < 0 || count > RCT_SYNTH_MAX_ELLIPSOIDS)
    return 0;
  for (int e = 0; e < count; e++) {
    double r[16];
    for (int k = 0; k < 16; k++)
      r[k] = unit01(key3(seed, 100 + (uint64_t)e, (uint64_t)k));
    /* centre: uniform direction, radius^(1/3) for a uniform ball, kept in the
       inner half so most of each body is inside the field of view */
    const double zc = 2.0 * r[0] - 1.0;
    const double ph = 2.0 * 3.14159265358979323846 * r[1];
    const double rc = 0.5 * radius * cbrt(r[2]);
    const double sc = sqrt(1.0 - zc * zc);
    out[e].center[0] = rc * sc * cos(ph);
    out[e].center[1] = rc * sc * sin(ph);
    out[e].center[2] = rc * zc;
    for (int k = 0; k < 3; k++)
      out[e].axes[k] = radius * (0.08 + 0.30 * r[3 + k]);
    /* rotation from a uniform random unit quaternion (Shoemake) */
    const double u1 = r[6], u2 = r[7], u3 = r[8];
    const double tw = 2.0 * 3.14159265358979323846;
    const double qx = sqrt(1 - u1) * sin(tw * u2), qy = sqrt(1 - u1) * cos(tw * u2);
    const double qz = sqrt(u1) * sin(tw * u3), qw = sqrt(u1) * cos(tw * u3);
    double *R = out[e].rot;
    R[0] = 1 - 2 * (qy * qy + qz * qz);
    R[1] = 2 * (qx * qy - qz * qw);
    R[2] = 2 * (qx * qz + qy * qw);
    R[3] = 2 * (qx * qy + qz * qw);
    R[4] = 1 - 2 * (qx * qx + qz * qz);
    R[5] = 2 * (qy * qz - qx * qw);
    R[6] = 2 * (qx * qz - qy * qw);
    R[7] = 2 * (qy * qz + qx * qw);
    R[8] = 1 - 2 * (qx * qx + qy * qy);
    out[e].density = 0.1 + 0.9 * r[9];
  }
  return count;
}

/* ---- projections --------------------------------------------------------- */

/* Source position and inverse-camera mapping of one view. */
typedef struct {
  double src[3];
  double eu[3], ev[3], ew[3];
  double f, cu, cv;
} ViewFrame;

static void viewFrame(const RctScanGeometry *g, int p, ViewFrame *v)
{
  const double deg = 3.14159265358979323846 / 180.0;
  const double th = (g->startDeg + g->arcDeg * (double)p / (double)g->nproj) * deg;
  const double c = cos(th), s = sin(th);
  v->src[0] = g->sod * c;
  v->src[1] = g->sod * s;
  v->src[2] = 0.0;
  v->eu[0] = -s; v->eu[1] = c;  v->eu[2] = 0.0;
  v->ev[0] = 0;  v->ev[1] = 0;  v->ev[2] = -1.0;
  v->ew[0] = -c; v->ew[1] = -s; v->ew[2] = 0.0;
  v->f  = g->sid / g->pitch;
  v->cu = 0.5 * (double)(g->width - 1) +
          g->ppJitter * (2.0 * unit01(key3(g->seed, 11, (uint64_t)p)) - 1.0);
  v->cv = 0.5 * (double)(g->height - 1) +
          g->ppJitter * (2.0 * unit01(key3(g->seed, 12, (uint64_t)p)) - 1.0);
}

/* images: nproj * height * width float32, row-major per view (image[j*W+i]).
 * Pixel = sum over ellipsoids of density * chord_mm / 10 + N(0, noiseSigma). */
void rctSynthProjections(const RctScanGeometry *g, const RctEllipsoid *ell, int nell,
    double noiseSigma, uint64_t noiseSeed, float *images)
{
  const int W = g->width, H = g->height;
  /* per-ellipsoid world->unit-sphere linear map M = diag(1/axes) R^T */
  double M[RCT_SYNTH_MAX_ELLIPSOIDS][9];
  for (int e = 0; e < nell; e++)
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++)
        M[e][r * 3 + c] = ell[e].rot[c * 3 + r] / ell[e].axes[r];

#pragma omp parallel for schedule(dynamic, 4) collapse(2)
  for (int p = 0; p < g->nproj; p++) {
    for (int j = 0; j < H; j++) {
      ViewFrame vf;
      viewFrame(g, p, &vf);
      double o[RCT_SYNTH_MAX_ELLIPSOIDS][3], C[RCT_SYNTH_MAX_ELLIPSOIDS];
      for (int e = 0; e < nell; e++) {
        double d[3];
        for (int k = 0; k < 3; k++)
          d[k] = vf.src[k] - ell[e].center[k];
        for (int r = 0; r < 3; r++)
          o[e][r] = M[e][r * 3] * d[0] + M[e][r * 3 + 1] * d[1] + M[e][r * 3 + 2] * d[2];
        C[e] = o[e][0] * o[e][0] + o[e][1] * o[e][1] + o[e][2] * o[e][2] - 1.0;
      }
      float *row = images + ((size_t)p * H + j) * (size_t)W;
      const double dv = ((double)j - vf.cv) / vf.f;
      for (int i = 0; i < W; i++) {
        const double du = ((double)i - vf.cu) / vf.f;
        double dir[3];
        for (int k = 0; k < 3; k++)
          dir[k] = du * vf.eu[k] + dv * vf.ev[k] + vf.ew[k];
        const double inv = 1.0 / sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
        for (int k = 0; k < 3; k++)
          dir[k] *= inv;
        double acc = 0.0;
        for (int e = 0; e < nell; e++) {
          const double *m = M[e];
          const double d0 = m[0] * dir[0] + m[1] * dir[1] + m[2] * dir[2];
          const double d1 = m[3] * dir[0] + m[4] * dir[1] + m[5] * dir[2];
          const double d2 = m[6] * dir[0] + m[7] * dir[1] + m[8] * dir[2];
          const double A = d0 * d0 + d1 * d1 + d2 * d2;
          const double B = o[e][0] * d0 + o[e][1] * d1 + o[e][2] * d2;
          const double disc = B * B - A * C[e];
          if (disc > 0.0)
            acc += ell[e].density * 0.1 * (2.0 * sqrt(disc) / A);
        }
        if (noiseSigma > 0.0) {
          const uint64_t pix = (uint64_t)j * (uint64_t)W + (uint64_t)i;
          const double u1 = unit01(key3(noiseSeed, (uint64_t)p, 2 * pix));
          const double u2 = unit01(key3(noiseSeed, (uint64_t)p, 2 * pix + 1));
          acc += noiseSigma * sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
        }
        row[i] = (float)acc;
      }
    }
  }
}
