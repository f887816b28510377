/* Backprojection without device allocation.
 *
 * Some callers cannot allocate device memory while they run: an acquisition
 * loop that reserves all of its device memory at start-up and must not stall
 * on cudaMalloc / cudaFree (both can synchronise the whole device), or a host
 * framework that owns the device memory pool and forbids libraries from
 * allocating behind its back.  lolaCudaBackprojectNoAlloc serves them: the
 * caller passes the volume and the projections, already in device memory, and
 * the scratch the operation needs — the ring of packed, zero-padded
 * projections that the pass kernel gathers from, and each pass's projection
 * records — are the fixed arrays below, part of the library's device image.
 *
 * Limits and sharing:
 *  - the scratch is LOLA_NOALLOC_SCRATCH_BYTES (32 MiB) on every GPU that
 *    loads the library, held until the process exits;
 *  - one packed projection must fit in it; as many as fit, up to the
 *    configured batch, share a pass.  At 1248x960 (1376x1088 padded): FP32
 *    taps 6.0 MB (5 per pass), FP16/BF16 taps 3.0 MB (10), FP16/BF16 quads
 *    12 MB (2), FP32 quads 24 MB (1: the library's default storage, so a
 *    call with config NULL runs one pass per projection);
 *  - the storages read by loads only: f32, f16, bf16, f32q, f16q, bf16q.
 *    f16qx and f32qx run as f16q and f32q (the same values, read by loads
 *    only); tex32 and tex16 are rejected (they need texture objects);
 *  - every call uses the same array.  The pack kernel rewrites every element
 *    of each ring slot, zero margin included, before a pass reads it, so no
 *    state carries over from the previous call; but two calls whose work
 *    overlaps on the GPU (different streams, or different host threads on one
 *    device) race on the array and must be serialised by the caller.
 *  - the device addresses of the arrays are looked up once per CUDA context
 *    (normally once per device, the device's primary context), on the first
 *    call made with it current; make that first call before any stream
 *    capture begins.  A context destroyed and recreated at the same handle
 *    (cudaDeviceReset) keeps the stale addresses: do not reset the device
 *    between calls.
 */
#include <mutex>

#include <cuda_runtime.h>

#include "lolaCuda.h"
#include "lolacuda_internal.h"

static __device__ __align__(256) unsigned char gNoAllocScratch[LOLA_NOALLOC_SCRATCH_BYTES];
/* the current pass's projections, where the per-tile setup reads them (from
   the kernel parameters one lane per projection reads divergent addresses,
   which the constant cache serves one at a time) */
static __device__ LolaPassProj gNoAllocProj[LOLA_MAX_BATCH];

/* Copies a pass's projections from its parameters into gNoAllocProj: a
   kernel, so that the call stays free of host copies and capturable. */
__global__ void __launch_bounds__(128) noAllocProjKernel(const __grid_constant__ LolaPassParams P,
    LolaPassProj *dst)
{
  const int words = P.count * (int)(sizeof(LolaPassProj) / sizeof(uint32_t));
  const uint32_t *src = reinterpret_cast<const uint32_t *>(P.proj);
  uint32_t *d = reinterpret_cast<uint32_t *>(dst);
  for (int i = threadIdx.x; i < words; i += blockDim.x)
    d[i] = src[i];
}

namespace {

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);

/* cuCtxGetCurrent through the runtime's driver entry points (no -lcuda). */
CtxGetCurrentFn ctxGetCurrent()
{
  static CtxGetCurrentFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetCurrentFn>(f);
  }
  return fn;
}

/* One entry per (device, context) the entry point ran in. */
struct ScratchAddr {
  int device;
  CUcontext ctx;
  void *ring;
  LolaPassProj *proj;
};
constexpr int kMaxContexts = 64;
ScratchAddr gAddr[kMaxContexts];
int gAddrCount = 0;
std::mutex gScratchMutex;

CUcontext currentContext()
{
  CUcontext ctx = nullptr;
  CtxGetCurrentFn get = ctxGetCurrent();
  if (get == nullptr || get(&ctx) != CUDA_SUCCESS)
    return nullptr;
  return ctx;
}

/* Address pair cached for (device, ctx); the mutex is held. */
const ScratchAddr *findAddress(int device, CUcontext ctx)
{
  for (int i = 0; i < gAddrCount; i++)
    if (gAddr[i].device == device && gAddr[i].ctx == ctx)
      return &gAddr[i];
  return nullptr;
}

/* Device addresses of gNoAllocScratch and gNoAllocProj in the current context
 * of `device`.  The symbols' names in host code are only host-side handles,
 * so the addresses must come from the runtime (cudaGetSymbolAddress), once
 * per context.  A thread with no context bound yet (ctx null) gets the
 * device's primary context bound by that lookup, and then finds the entry
 * another thread made for it. */
int scratchAddress(int device, void **out, LolaPassProj **proj)
{
  std::lock_guard<std::mutex> lock(gScratchMutex);
  CUcontext ctx = currentContext();
  const ScratchAddr *a = ctx != nullptr ? findAddress(device, ctx) : nullptr;
  if (a == nullptr) {
    void *p = nullptr, *q = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, gNoAllocScratch);
    if (e == cudaSuccess)
      e = cudaGetSymbolAddress(&q, gNoAllocProj);
    if (e != cudaSuccess)
      return lolaSetError("cudaGetSymbolAddress(no-alloc scratch): %s", cudaGetErrorString(e));
    ctx = currentContext();
    a = findAddress(device, ctx);
    if (a == nullptr) {
      if (gAddrCount == kMaxContexts)
        return lolaSetError("no-alloc entry point used in more than %d contexts", kMaxContexts);
      ScratchAddr &n = gAddr[gAddrCount++];
      n.device = device;
      n.ctx = ctx;
      n.ring = p;
      n.proj = static_cast<LolaPassProj *>(q);
      a = &n;
    }
  }
  *out = a->ring;
  *proj = a->proj;
  return 1;
}

int elemBytes(int storage)
{
  switch (storage) {
  case LOLA_STORE_F32: return 4;
  case LOLA_STORE_F16:
  case LOLA_STORE_BF16: return 2;
  case LOLA_STORE_F32Q: return 16;
  case LOLA_STORE_F16Q:
  case LOLA_STORE_BF16Q: return 8;
  default: return 0;
  }
}

} /* namespace */

extern "C" int lolaCudaBackprojectNoAlloc(const LolaCudaGeometry *g, const LolaCudaConfig *config,
    float *d_volume, const float *d_images, size_t imageStride, const double *h_matrices,
    int count, void *stream)
{
  if (g == nullptr)
    return lolaSetError("null geometry");
  LolaCudaConfig c;
  if (config != nullptr)
    c = *config;
  else
    lolaCudaDefaultConfig(&c);
  if (count < 0)
    return lolaSetError("negative projection count");
  if (g->problemSize <= 0 || g->problemSize > 2048 || g->imageWidth <= 0 || g->imageHeight <= 0)
    return lolaSetError("invalid geometry N=%d W=%d H=%d", g->problemSize, g->imageWidth,
        g->imageHeight);
  if (!(g->voxelSize > 0.0f))
    return lolaSetError("voxel size must be positive");
  /* the mixed layouts' values are their load-only layouts' (bit for bit); the
     texture layouts need texture objects, which this entry point does not make */
  if (c.storage == LOLA_STORE_F16QX)
    c.storage = LOLA_STORE_F16Q;
  else if (c.storage == LOLA_STORE_F32QX)
    c.storage = LOLA_STORE_F32Q;
  if (c.storage == LOLA_STORE_TEX32 || c.storage == LOLA_STORE_TEX16)
    return lolaSetError("storage %s needs texture objects; the no-allocation entry point "
                        "reads f32, f16, bf16, f32q, f16q, bf16q (f16qx, f32qx as f16q, f32q)",
        c.storage == LOLA_STORE_TEX32 ? "tex32" : "tex16");
  const int eb = elemBytes(c.storage);
  if (eb == 0)
    return lolaSetError("invalid storage %d", c.storage);
  if (c.accumulation != LOLA_ACCUM_PLAIN && c.accumulation != LOLA_ACCUM_KAHAN)
    return lolaSetError("invalid accumulation %d", c.accumulation);
  if (!lolaKernelShapeSupported(c.voxelsPerThread, c.rowsPerBlock))
    return lolaSetError("no kernel for %d voxels per thread x %d rows per block",
        c.voxelsPerThread, c.rowsPerBlock);
  /* z-slab of the volume held in d_volume (N x N x sliceCount), as for a plan:
     0 / 0 is the whole volume */
  int zBegin = g->sliceBegin, zCount = g->sliceCount;
  if (zBegin == 0 && zCount == 0)
    zCount = g->problemSize;
  if (zBegin < 0 || zCount <= 0 || zBegin + zCount > g->problemSize)
    return lolaSetError("slab [%d, %d) outside the %d slices", g->sliceBegin,
        g->sliceBegin + g->sliceCount, g->problemSize);
  if (count == 0)
    return 1;
  if (d_volume == nullptr || d_images == nullptr || h_matrices == nullptr)
    return lolaSetError("null argument");

  LolaStoreDesc st;
  memset(&st, 0, sizeof(st));  /* no texture objects or surfaces */
  st.storage = c.storage;
  st.elemBytes = eb;
  st.margin = LOLA_MARGIN;
  st.width = g->imageWidth;
  st.height = g->imageHeight;
  /* the plan's layout: its pitch, slots 256 pixels apart */
  st.pitch = lolaStorePitch(g->imageWidth, st.storage, eb);
  st.rows = g->imageHeight + 2 * LOLA_MARGIN;
  st.reserved = 0;
  if ((long long)st.pitch * st.rows >= (1LL << 23) - 2 * (long long)st.pitch)
    return lolaSetError("detector %dx%d too large (padded image must stay below 2^23 pixels)",
        g->imageWidth, g->imageHeight);
  st.slotElems = ((size_t)st.pitch * (size_t)st.rows + 255) & ~(size_t)255;
  const size_t slotBytes = st.slotElems * (size_t)eb;
  if (slotBytes > LOLA_NOALLOC_SCRATCH_BYTES)
    return lolaSetError("one packed %dx%d projection needs %zu bytes; the no-allocation "
                        "entry point has %u bytes of scratch (use FP16/BF16 or plain "
                        "storage, or the plan API)",
        g->imageWidth, g->imageHeight, slotBytes, (unsigned)LOLA_NOALLOC_SCRATCH_BYTES);
  int perPass = (int)(LOLA_NOALLOC_SCRATCH_BYTES / slotBytes);
  if (perPass > LOLA_MAX_BATCH)
    perPass = LOLA_MAX_BATCH;
  if (c.batch >= 1 && perPass > c.batch)
    perPass = c.batch;

  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess)
    return lolaSetError("cudaGetDevice: %s", cudaGetErrorString(e));
  void *ring = nullptr;
  LolaPassProj *projScratch = nullptr;
  if (!scratchAddress(device, &ring, &projScratch))
    return 0;

  LolaPassParams P;
  memset(&P, 0, sizeof(P));  /* no tile counters; every field set below or zero */
  for (int done = 0; done < count;) {
    const int n = (count - done < perPass) ? count - done : perPass;
    int rc = lolaLaunchPack(&st, d_images + (size_t)done * imageStride, imageStride, ring, 0, n,
        stream);
    if (rc != 0)
      return lolaSetError("pack launch failed: %s", cudaGetErrorString((cudaError_t)rc));
    P.N = g->problemSize;
    P.count = n;
    P.zBegin = zBegin;
    P.zEnd = zBegin + zCount;
    P.voxelSize = g->voxelSize;
    P.originIndex = g->originIndex;
    P.accumulation = c.accumulation;
    P.voxelsPerThread = c.voxelsPerThread;
    P.rowsPerBlock = c.rowsPerBlock;
    P.countTiles = 0;
    P.projDevice = projScratch;
    for (int i = 0; i < n; i++) {
      const double *m = h_matrices + 12 * (size_t)(done + i);
      LolaPassProj &pp = P.proj[i];
      for (int k = 0; k < 12; k++)
        pp.a[k] = m[k];
      for (int ax = 0; ax < 3; ax++)
        for (int comp = 0; comp < 3; comp++)
          pp.step[ax][comp] = (float)(m[ax * 3 + comp] * (double)g->voxelSize);
      pp.slot = i;
      pp.reserved[0] = pp.reserved[1] = pp.reserved[2] = 0;
    }
    (void)cudaGetLastError();
    noAllocProjKernel<<<1, 128, 0, static_cast<cudaStream_t>(stream)>>>(P, projScratch);
    rc = (int)cudaGetLastError();
    if (rc != 0)
      return lolaSetError("projection copy launch failed: %s", cudaGetErrorString((cudaError_t)rc));
    rc = lolaLaunchBackproject(&st, &P, nullptr, ring, d_volume, nullptr, stream);
    if (rc != 0)
      return lolaSetError("pass launch failed: %s", cudaGetErrorString((cudaError_t)rc));
    done += n;
  }
  return 1;
}
