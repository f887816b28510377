/* Dispatch from the C host code to the per-layout kernel launchers. */
#include <cuda_runtime.h>

#include "lolacuda_internal.h"

#define LOLA_DECLARE(NAME)                                                                 \
  extern "C" int lolaLaunchPack_##NAME(const LolaStoreDesc *, const float *, size_t,       \
      void *, int, int, void *);                                                           \
  extern "C" int lolaLaunchPass_##NAME(const LolaStoreDesc *, const LolaPassParams *,      \
      const LolaStageDesc *, const void *, float *, unsigned long long *, void *);         \
  extern "C" int lolaLaunchBatchPack_##NAME(const LolaBatchWave *, void *);                \
  extern "C" int lolaLaunchBatchPass_##NAME(const LolaBatchWave *, int, void *);           \
  extern "C" int lolaBatchOccupancy_##NAME(int, int, int *);

LOLA_DECLARE(F32)
LOLA_DECLARE(F16)
LOLA_DECLARE(BF16)
LOLA_DECLARE(F32Q)
LOLA_DECLARE(F16Q)
LOLA_DECLARE(BF16Q)
LOLA_DECLARE(TEX32)
LOLA_DECLARE(TEX16)
LOLA_DECLARE(F16QX)
LOLA_DECLARE(F32QX)

static_assert(sizeof(LolaPassParams) < 32000, "pass parameters exceed the kernel parameter limit");

extern "C" int lolaLaunchPack(const LolaStoreDesc *st, const float *d_src, size_t srcStride,
    void *d_ring, int slot0, int count, void *stream)
{
  if (count <= 0)
    return 0;
  switch (st->storage) {
  case LOLA_STORE_F32: return lolaLaunchPack_F32(st, d_src, srcStride, d_ring, slot0, count, stream);
  case LOLA_STORE_F16: return lolaLaunchPack_F16(st, d_src, srcStride, d_ring, slot0, count, stream);
  case LOLA_STORE_BF16: return lolaLaunchPack_BF16(st, d_src, srcStride, d_ring, slot0, count, stream);
  case LOLA_STORE_F32Q: return lolaLaunchPack_F32Q(st, d_src, srcStride, d_ring, slot0, count, stream);
  case LOLA_STORE_F16Q: return lolaLaunchPack_F16Q(st, d_src, srcStride, d_ring, slot0, count, stream);
  case LOLA_STORE_BF16Q: return lolaLaunchPack_BF16Q(st, d_src, srcStride, d_ring, slot0, count, stream);
  case LOLA_STORE_TEX32: return lolaLaunchPack_TEX32(st, d_src, srcStride, d_ring, slot0, count, stream);
  case LOLA_STORE_TEX16: return lolaLaunchPack_TEX16(st, d_src, srcStride, d_ring, slot0, count, stream);
  case LOLA_STORE_F16QX: return lolaLaunchPack_F16QX(st, d_src, srcStride, d_ring, slot0, count, stream);
  case LOLA_STORE_F32QX: return lolaLaunchPack_F32QX(st, d_src, srcStride, d_ring, slot0, count, stream);
  default: return (int)cudaErrorInvalidValue;
  }
}

extern "C" int lolaLaunchBackproject(const LolaStoreDesc *st, const LolaPassParams *P,
    const LolaStageDesc *sd, const void *d_ring, float *d_volume,
    unsigned long long *d_tileCounters, void *stream)
{
  if (P->count <= 0)
    return 0;
  if (P->count > LOLA_MAX_BATCH)
    return (int)cudaErrorInvalidValue;
  switch (st->storage) {
  case LOLA_STORE_F32: return lolaLaunchPass_F32(st, P, sd, d_ring, d_volume, d_tileCounters, stream);
  case LOLA_STORE_F16: return lolaLaunchPass_F16(st, P, sd, d_ring, d_volume, d_tileCounters, stream);
  case LOLA_STORE_BF16: return lolaLaunchPass_BF16(st, P, sd, d_ring, d_volume, d_tileCounters, stream);
  case LOLA_STORE_F32Q: return lolaLaunchPass_F32Q(st, P, sd, d_ring, d_volume, d_tileCounters, stream);
  case LOLA_STORE_F16Q: return lolaLaunchPass_F16Q(st, P, sd, d_ring, d_volume, d_tileCounters, stream);
  case LOLA_STORE_BF16Q: return lolaLaunchPass_BF16Q(st, P, sd, d_ring, d_volume, d_tileCounters, stream);
  case LOLA_STORE_TEX32: return lolaLaunchPass_TEX32(st, P, sd, d_ring, d_volume, d_tileCounters, stream);
  case LOLA_STORE_TEX16: return lolaLaunchPass_TEX16(st, P, sd, d_ring, d_volume, d_tileCounters, stream);
  case LOLA_STORE_F16QX: return lolaLaunchPass_F16QX(st, P, sd, d_ring, d_volume, d_tileCounters, stream);
  case LOLA_STORE_F32QX: return lolaLaunchPass_F32QX(st, P, sd, d_ring, d_volume, d_tileCounters, stream);
  default: return (int)cudaErrorInvalidValue;
  }
}

extern "C" int lolaKernelShapeSupported(int voxelsPerThread, int rowsPerBlock)
{
  return (voxelsPerThread == 8 && (rowsPerBlock == 8 || rowsPerBlock == 4)) ||
         (voxelsPerThread == 16 && (rowsPerBlock == 8 || rowsPerBlock == 4)) ||
         (voxelsPerThread == 4 && rowsPerBlock == 8);
}

#define LOLA_BATCH_CASES(CALL)                                                             \
  switch (storage) {                                                                       \
  case LOLA_STORE_F32: return CALL(F32);                                                   \
  case LOLA_STORE_F16: return CALL(F16);                                                   \
  case LOLA_STORE_BF16: return CALL(BF16);                                                 \
  case LOLA_STORE_F32Q: return CALL(F32Q);                                                 \
  case LOLA_STORE_F16Q: return CALL(F16Q);                                                 \
  case LOLA_STORE_BF16Q: return CALL(BF16Q);                                               \
  case LOLA_STORE_TEX32: return CALL(TEX32);                                               \
  case LOLA_STORE_TEX16: return CALL(TEX16);                                               \
  case LOLA_STORE_F16QX: return CALL(F16QX);                                               \
  case LOLA_STORE_F32QX: return CALL(F32QX);                                               \
  default: return (int)cudaErrorInvalidValue;                                              \
  }

extern "C" int lolaLaunchBatchPack(const LolaBatchWave *w, void *stream)
{
  const int storage = w->storage;
#define PACK_CALL(NAME) lolaLaunchBatchPack_##NAME(w, stream)
  LOLA_BATCH_CASES(PACK_CALL)
#undef PACK_CALL
}

extern "C" int lolaLaunchBatchPass(const LolaBatchWave *w, int blocks, void *stream)
{
  const int storage = w->storage;
#define PASS_CALL(NAME) lolaLaunchBatchPass_##NAME(w, blocks, stream)
  LOLA_BATCH_CASES(PASS_CALL)
#undef PASS_CALL
}

extern "C" int lolaBatchPassOccupancy(int storage, int accumulation, int paramJobs, int *blocks)
{
#define OCC_CALL(NAME) lolaBatchOccupancy_##NAME(accumulation, paramJobs, blocks)
  LOLA_BATCH_CASES(OCC_CALL)
#undef OCC_CALL
}
