/* ORACLE — test infrastructure only (see oracle.c for the rules).
 *
 * Restatement of LolaASM (HPC-Dwarfs/RabbitCT src/LolaASM.c:84-211 with its
 * SIMD row kernel fastrabbit, src/fastRabbitNEON.S:36-203 and
 * src/fastRabbitAVX.S), the reference's fastest CPU method, in portable C:
 * GCC vector types of 4 floats, which compile to NEON on aarch64 and SSE on
 * x86_64 (no intrinsics, no assembly, no -march=native).  It is the CPU
 * baseline that the benchmark times on the host cores beside the LolaOPT
 * port, because the reference's own build cannot run on the GPU host.
 *
 *   oracleAsmPadding      src/LolaASM.c:45-63 (pads from the shadow, each
 *                         rounded up to the vector width)
 *   oracleAsmBackproject  src/LolaASM.c:84-211: z over threads, y blocked by
 *                         8, all views of the call inside the y block, one
 *                         row kernel per (view, row)
 *   rowKernel             fastrabbit: per group of 4 voxels along x,
 *                         u, v, w = tmp + a * wx; reciprocal refined by
 *                         Newton-Raphson; truncation through an integer
 *                         conversion; the four tap offsets formed in FP32
 *                         (iiy * width + iix, +1, +width) and truncated;
 *                         scalar gathers; lerp-form bilinear (1 - s) a + s b;
 *                         vol += val / w^2; wx += 4 mm.  Like the assembly
 *                         loop it runs at least once per row (a count of 0
 *                         still processes one group) and steps by the vector
 *                         width until count is used up.
 *
 * The reciprocal: the reference refines a hardware estimate (frecpe + two
 * Newton-Raphson steps on NEON, rcpps + one on x86).  There is no portable
 * estimate instruction, so this restatement starts from the classic
 * integer-subtraction initial guess for 1/w (bits(r0) = 0x7EF311C3 -
 * bits(w), exact in sign and within 12 % for positive normal w) and takes
 * three Newton-Raphson steps r <- r (2 - w r), which reach FP32 precision.
 * Results agree with the reference's LolaASM within a few ulp per voxel
 * (tests/test_oracle_golden.py pins them against its build); like the
 * reference, the compiler's FMA contraction makes them differ by ulps
 * between hosts.
 */
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef float v4f __attribute__((vector_size(16)));
typedef int32_t v4i __attribute__((vector_size(16)));

#define ASM_BLOCKING 8 /* BLOCKING_FACTOR of src/LolaASM.c:84 */

static inline v4f splat(float x) { return (v4f){ x, x, x, x }; }

static inline v4f loadu(const float *p)
{
  v4f v;
  memcpy(&v, p, sizeof(v));
  return v;
}

static inline void storeu(float *p, v4f v) { memcpy(p, &v, sizeof(v)); }

/* 1/w by Newton-Raphson from the integer initial guess (see the header). */
static inline v4f reciprocal(v4f w)
{
  v4i bits;
  memcpy(&bits, &w, sizeof(bits));
  bits = (v4i){ 0x7EF311C3, 0x7EF311C3, 0x7EF311C3, 0x7EF311C3 } - bits;
  v4f r;
  memcpy(&r, &bits, sizeof(r));
  const v4f two = splat(2.0f);
  r = r * (two - w * r);
  r = r * (two - w * r);
  r = r * (two - w * r);
  return r;
}

/* The row kernel: `count` voxels of one row from vol, starting at x = wx. */
static void rowKernel(const float a0, const float a1, const float a2, const float *img,
    const float t0, const float t1, const float t2, float *vol, float wx0, float mm,
    float width, int count, int vecsize)
{
  const v4f A0 = splat(a0), A1 = splat(a1), A2 = splat(a2);
  const v4f T0 = splat(t0), T1 = splat(t1), T2 = splat(t2);
  const v4f W = splat(width), one = splat(1.0f), step = splat(4.0f * mm);
  v4f wx = (v4f){ wx0, wx0 + mm, wx0 + 2.0f * mm, wx0 + 3.0f * mm };
  /* one assembly iteration covers `vecsize` voxels: vecsize / 4 groups */
  do {
    for (int g = 0; g < vecsize; g += 4) {
      const v4f u = T0 + A0 * wx;
      const v4f v = T1 + A1 * wx;
      const v4f w = T2 + A2 * wx;
      const v4f r = reciprocal(w);
      const v4f ix = u * r, iy = v * r;
      const v4f r2 = r * r;
      const v4i iix = __builtin_convertvector(ix, v4i);  /* truncation */
      const v4i iiy = __builtin_convertvector(iy, v4i);
      const v4f fx = __builtin_convertvector(iix, v4f);
      const v4f fy = __builtin_convertvector(iiy, v4f);
      const v4f sx = ix - fx, sy = iy - fy;
      const v4f obl = fy * W + fx;       /* offsets of the four taps, in FP32 */
      const v4f otl = obl + W;
      const v4f obr = obl + one;
      const v4f otr = otl + one;
      const v4i ibl = __builtin_convertvector(obl, v4i);
      const v4i itl = __builtin_convertvector(otl, v4i);
      const v4i ibr = __builtin_convertvector(obr, v4i);
      const v4i itr = __builtin_convertvector(otr, v4i);
      v4f bl, tl, br, tr;
      for (int l = 0; l < 4; ++l) {
        bl[l] = img[ibl[l]];
        tl[l] = img[itl[l]];
        br[l] = img[ibr[l]];
        tr[l] = img[itr[l]];
      }
      const v4f ox = one - sx, oy = one - sy;
      const v4f vb = bl * ox + br * sx;
      const v4f vt = tl * ox + tr * sx;
      const v4f val = vb * oy + vt * sy;
      storeu(vol, loadu(vol) + val * r2);
      vol += 4;
      wx = wx + step;
    }
    count -= vecsize;
  } while (count > 0);
}

/* pad[4] = {left, right, bottom, top} from the shadow as src/LolaASM.c:45-63
 * forms them, each rounded up to a multiple of vecsize.  Returns the padded
 * width; *rows receives the padded height. */
int oracleAsmPadding(const int *shadow, int W, int H, int vecsize, int *pad, int *rows)
{
  pad[0] = abs(shadow[0]);
  pad[1] = abs(shadow[1]) - W;
  pad[2] = abs(shadow[2]);
  pad[3] = abs(shadow[3]) - H;
  for (int i = 0; i < 4; ++i) {
    const int r = pad[i] % vecsize;
    if (r)
      pad[i] += vecsize - r;
  }
  *rows = pad[2] + H + pad[3];
  return pad[0] + W + pad[1];
}

/* One call of LolaASM's backprojection for `nproj` views (global 1-based ids
 * ids[p], matrices mats[p*12..]) whose zero-padded images the caller
 * prepared (padded[p]; startOffset / lineOffset as src/LolaASM.c:60-62);
 * ranges from oracleLineRanges over all views with vector size `vecsize`
 * (4 or 8, a multiple of this restatement's 4-float vectors). */
void oracleAsmBackproject(int N, float voxelSize, float originIndex, int nproj,
    const int *ids, const double *mats, const float *const *padded, int startOffset,
    int lineOffset, const int16_t *ranges, int vecsize, float *vol)
{
  const int l = N;
  const float mm = voxelSize, o = originIndex;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < l; ++z) {
    const float wz = z * mm + o;
    for (int y = 0; y < l; y += ASM_BLOCKING) {
      for (int p = 0; p < nproj; ++p) {
        const double *a = mats + 12 * (size_t)p;
        const float *img = padded[p] + startOffset;
        const int16_t *R = ranges + 2 * (size_t)(ids[p] - 1) * l * l;
        for (int yh = 0; yh < ASM_BLOCKING && y + yh < l; ++yh) {
          const int yn = y + yh;
          const int start = R[2 * (z * l + yn)];
          const int count = R[2 * (z * l + yn) + 1] - start;
          if (start < 0)
            continue;
          const float wy = yn * mm + o;
          const float wx = start * mm + o;
          /* the row invariants in FP64, cast (src/LolaASM.c:152-154) */
          const float t0 = (float)(a[3] * wy + a[6] * wz + a[9]);
          const float t1 = (float)(a[4] * wy + a[7] * wz + a[10]);
          const float t2 = (float)(a[5] * wy + a[8] * wz + a[11]);
          rowKernel((float)a[0], (float)a[1], (float)a[2], img, t0, t1, t2,
              vol + (size_t)z * l * l + (size_t)yn * l + start, wx, mm, (float)lineOffset,
              count, vecsize);
        }
      }
    }
  }
}
