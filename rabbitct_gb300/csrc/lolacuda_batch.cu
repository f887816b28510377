/* Batched reconstructions: many volumes of uneven size, detector and
 * projection count, reconstructed together (host side of bp_batch.cuh).
 *
 * lolaCudaBatchCreate lays out one projection ring holding `b` stored slots
 * per job and captures the whole run into a CUDA graph; lolaCudaBatchRun
 * replays the graph on the batch's stream.  Two schedules:
 *  - branches (default): each job's pack and pass launches (the plan kernels,
 *    with a tile shape timed per (N, detector) class when batchTune is set)
 *    go to one of K parallel graph branches, largest jobs first;
 *  - persistent: per-wave projection parameters and work lists (prefix sums
 *    of the tiles of the jobs that still have projections in that wave), then
 *    a counter reset and, per wave, one pack launch and one persistent pass
 *    launch (bp_batch.cuh).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include <cuda_runtime.h>

#include "lolaCuda.h"
#include "lolacuda_internal.h"

struct LolaCudaBatch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<cudaStream_t> branches;
  std::vector<cudaEvent_t> events;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  LolaCudaConfig cfg;
  int njobs = 0, b = 0, waves = 0, blocks = 0, launches = 0;
  double updates = 0.0;
  size_t ringBytes = 0;
  unsigned char *d_ring = nullptr;
  LolaBatchJob *d_jobs = nullptr;
  long long *d_prefix = nullptr;
  LolaPassProj *d_proj = nullptr;
  int *d_counters = nullptr;
  unsigned long long *d_tex = nullptr;
  std::vector<cudaTextureObject_t> textures;
};

namespace {

int pixelBytes(int storage)
{
  switch (storage) {
  case LOLA_STORE_F32: case LOLA_STORE_TEX32: return 4;
  case LOLA_STORE_F16: case LOLA_STORE_BF16: case LOLA_STORE_TEX16: return 2;
  case LOLA_STORE_F32Q: case LOLA_STORE_F32QX: return 16;
  case LOLA_STORE_F16Q: case LOLA_STORE_BF16Q: case LOLA_STORE_F16QX: return 8;
  default: return 0;
  }
}

int textureChannels(int storage)
{
  switch (storage) {
  case LOLA_STORE_TEX32: case LOLA_STORE_TEX16: return 1;
  case LOLA_STORE_F16QX: case LOLA_STORE_F32QX: return 4;
  default: return 0;
  }
}

void release(LolaCudaBatch *bt)
{
  if (bt == nullptr)
    return;
  cudaSetDevice(bt->device);
  if (bt->stream)
    cudaStreamSynchronize(bt->stream);
  if (bt->exec)
    cudaGraphExecDestroy(bt->exec);
  if (bt->graph)
    cudaGraphDestroy(bt->graph);
  for (cudaTextureObject_t t : bt->textures)
    cudaDestroyTextureObject(t);
  cudaFree(bt->d_ring);
  cudaFree(bt->d_jobs);
  cudaFree(bt->d_prefix);
  cudaFree(bt->d_proj);
  cudaFree(bt->d_counters);
  cudaFree(bt->d_tex);
  for (cudaStream_t b : bt->branches)
    cudaStreamDestroy(b);
  for (cudaEvent_t e : bt->events)
    cudaEventDestroy(e);
  if (bt->stream)
    cudaStreamDestroy(bt->stream);
  delete bt;
}

#define BT_TRY(call)                                                                      \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      (void)cudaGetLastError();                                                           \
      lolaSetError("batch: %s: %s", #call, cudaGetErrorString(e_));                       \
      return 0;                                                                           \
    }                                                                                     \
  } while (0)


/* LOLA_BATCH_BRANCHES: each job's waves (pack, pass) chained in one of K
 * parallel branches of the captured graph; jobs assigned largest first to the
 * least loaded branch. */
/* Tile shape per job: the configured one, or with batchTune the fastest of
 * the compiled shapes, timed once per distinct (N, detector) class on that
 * class's first projections with a scratch plan. */
int chooseShapes(LolaCudaBatch *bt, const LolaCudaJob *jobs, const std::vector<LolaBatchJob> &hj,
    std::vector<int> &vpt, std::vector<int> &rows)
{
  const int nj = bt->njobs;
  vpt.assign(nj, bt->cfg.voxelsPerThread);
  rows.assign(nj, bt->cfg.rowsPerBlock);
  if (!bt->cfg.batchTune)
    return 1;
  static const int shapes[][2] = { { 8, 8 }, { 8, 4 }, { 16, 4 }, { 16, 8 }, { 4, 8 } };
  std::vector<int> done(nj, 0);
  for (int j = 0; j < nj; ++j) {
    if (done[j] || hj[j].nproj <= 0)
      continue;
    const int count = hj[j].nproj < 2 * bt->b ? hj[j].nproj : 2 * bt->b;
    double bestMs = 1e300;
    int bv = bt->cfg.voxelsPerThread, br = bt->cfg.rowsPerBlock;
    for (const auto &sh : shapes) {
      LolaCudaConfig c = bt->cfg;
      c.voxelsPerThread = sh[0];
      c.rowsPerBlock = sh[1];
      c.staging = 0;
      c.collectStats = 0;
      LolaCudaGeometry g = jobs[j].geometry;
      g.sliceBegin = g.sliceCount = 0;
      LolaCudaPlan *p = nullptr;
      if (!lolaCudaPlanCreate(&g, &c, &p))
        continue;
      double ms = -1.0;
      const size_t img = (size_t)hj[j].width * hj[j].height;
      if (lolaCudaPlanBackprojectDevice(p, hj[j].images, img, jobs[j].h_matrices, count) &&
          lolaCudaPlanSynchronize(p) && lolaCudaPlanTimerStart(p) &&
          lolaCudaPlanBackprojectDevice(p, hj[j].images, img, jobs[j].h_matrices, count))
        lolaCudaPlanTimerStop(p, &ms);
      lolaCudaPlanDestroy(p);
      if (ms > 0.0 && ms < bestMs) {
        bestMs = ms;
        bv = sh[0];
        br = sh[1];
      }
    }
    for (int k = j; k < nj; ++k)
      if (!done[k] && hj[k].N == hj[j].N && hj[k].width == hj[j].width &&
          hj[k].height == hj[j].height) {
        vpt[k] = bv;
        rows[k] = br;
        done[k] = 1;
      }
  }
  return 1;
}

/* 1: the branch passes read their projections from the batch's device table */
#ifndef LOLA_BATCH_PROJ_DEVICE
#define LOLA_BATCH_PROJ_DEVICE 1
#endif

int captureBranches(LolaCudaBatch *bt, const LolaCudaJob *jobs,
    const std::vector<LolaBatchJob> &hj, const std::vector<unsigned long long> &tex)
{
  const int nj = bt->njobs, b = bt->b;
  std::vector<int> vpt, rows;
  if (!chooseShapes(bt, jobs, hj, vpt, rows))
    return 0;
  int K = bt->cfg.batchBranches > 0 ? bt->cfg.batchBranches : 16;
  K = K > nj ? nj : K;
  std::vector<int> order(nj);
  for (int j = 0; j < nj; ++j)
    order[j] = j;
  auto work = [&](int j) { return (double)hj[j].N * hj[j].N * hj[j].N * hj[j].nproj; };
  std::sort(order.begin(), order.end(), [&](int a, int c) { return work(a) > work(c); });
  std::vector<std::vector<int>> lanes(K);
  std::vector<double> load(K, 0.0);
  for (int j : order) {
    int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    lanes[k].push_back(j);
    load[k] += work(j);
  }
  bt->branches.resize(K);
  bt->events.resize(K + 1);
  for (int k = 0; k < K; ++k)
    BT_TRY(cudaStreamCreateWithFlags(&bt->branches[k], cudaStreamNonBlocking));
  for (int k = 0; k <= K; ++k)
    BT_TRY(cudaEventCreateWithFlags(&bt->events[k], cudaEventDisableTiming));

  /* every job's projections in device memory, job after job, each with the
     ring slot its wave packs it into: the passes' per-tile setup reads them
     there (kernel-parameter reads from one lane per projection would be
     served one address at a time) */
  std::vector<size_t> first(nj + 1, 0);
  for (int j = 0; j < nj; ++j)
    first[j + 1] = first[j] + (size_t)(hj[j].nproj > 0 ? hj[j].nproj : 0);
  if (first[nj] > 0) {
    std::vector<LolaPassProj> all(first[nj]);
    memset(all.data(), 0, all.size() * sizeof(LolaPassProj));
    for (int j = 0; j < nj; ++j)
      for (int k = 0; k < hj[j].nproj; ++k) {
        const double *m = jobs[j].h_matrices + 12 * (size_t)k;
        LolaPassProj &pp = all[first[j] + k];
        memcpy(pp.a, m, 12 * sizeof(double));
        for (int ax = 0; ax < 3; ++ax)
          for (int c = 0; c < 3; ++c)
            pp.step[ax][c] = (float)(m[ax * 3 + c] * (double)hj[j].voxelSize);
        pp.slot = k % b;
      }
    BT_TRY(cudaMalloc(&bt->d_proj, all.size() * sizeof(LolaPassProj)));
    BT_TRY(cudaMemcpy(bt->d_proj, all.data(), all.size() * sizeof(LolaPassProj),
        cudaMemcpyHostToDevice));
  }

  BT_TRY(cudaStreamBeginCapture(bt->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaEventRecord(bt->events[K], bt->stream);
  int rc = 0;
  for (int k = 0; k < K && e == cudaSuccess && rc == 0; ++k) {
    cudaStream_t st = bt->branches[k];
    e = cudaStreamWaitEvent(st, bt->events[K], 0);
    for (int j : lanes[k]) {
      const LolaBatchJob &J = hj[j];
      LolaStoreDesc sd;
      memset(&sd, 0, sizeof(sd));
      sd.storage = bt->cfg.storage;
      sd.elemBytes = (int32_t)(J.slotBytes / J.slotElems);
      sd.margin = J.margin;
      sd.pitch = J.pitch;
      sd.rows = J.rows;
      sd.width = J.width;
      sd.height = J.height;
      sd.slotElems = J.slotElems;
      for (int s = 0; s < b && !tex.empty(); ++s)
        sd.texObjects[s] = tex[(size_t)j * b + s];
      const size_t img = (size_t)J.width * J.height;
      for (int w0 = 0; w0 < J.nproj && e == cudaSuccess && rc == 0; w0 += b) {
        const int n = J.nproj - w0 < b ? J.nproj - w0 : b;
        rc = lolaLaunchPack(&sd, J.images + (size_t)w0 * img, img, J.ring, 0, n, st);
        if (rc != 0)
          break;
        LolaPassParams P;
        memset(&P, 0, sizeof(P));
        P.N = J.N;
        P.count = n;
        P.zBegin = 0;
        P.zEnd = J.N;
        P.voxelSize = J.voxelSize;
        P.originIndex = J.originIndex;
        P.accumulation = bt->cfg.accumulation;
        P.voxelsPerThread = vpt[j];
        P.rowsPerBlock = rows[j];
        for (int i = 0; i < n; ++i) {
          const double *m = jobs[j].h_matrices + 12 * (size_t)(w0 + i);
          memcpy(P.proj[i].a, m, 12 * sizeof(double));
          for (int ax = 0; ax < 3; ++ax)
            for (int c = 0; c < 3; ++c)
              P.proj[i].step[ax][c] = (float)(m[ax * 3 + c] * (double)J.voxelSize);
          P.proj[i].slot = i;
        }
        P.projDevice = LOLA_BATCH_PROJ_DEVICE ? bt->d_proj + first[j] + w0 : nullptr;
        rc = lolaLaunchBackproject(&sd, &P, nullptr, J.ring, J.volume, nullptr, st);
        bt->launches += 2;
      }
    }
    if (e == cudaSuccess)
      e = cudaEventRecord(bt->events[k], st);
    if (e == cudaSuccess)
      e = cudaStreamWaitEvent(bt->stream, bt->events[k], 0);
  }
  cudaError_t ce = cudaStreamEndCapture(bt->stream, &bt->graph);
  if (e != cudaSuccess || rc != 0 || ce != cudaSuccess)
    return lolaSetError("batch: capture failed: %s / %s / %s", cudaGetErrorString(e),
        cudaGetErrorString((cudaError_t)rc), cudaGetErrorString(ce));
  BT_TRY(cudaGraphInstantiate(&bt->exec, bt->graph, 0));
  bt->blocks = 0;
  return 1;
}

int build(LolaCudaBatch *bt, const LolaCudaJob *jobs)
{
  const int nj = bt->njobs, b = bt->b, storage = bt->cfg.storage;
  const int pix = pixelBytes(storage);
  BT_TRY(cudaSetDevice(bt->device));
  BT_TRY(cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking));

  /* per-job stored layouts and the shared ring */
  std::vector<LolaBatchJob> hj(nj);
  std::vector<size_t> ringOffset(nj);
  int maxPitch = 0, maxRows = 0;
  size_t ring = 0;
  for (int j = 0; j < nj; ++j) {
    const LolaCudaGeometry &g = jobs[j].geometry;
    LolaBatchJob &J = hj[j];
    memset(&J, 0, sizeof(J));
    J.N = g.problemSize;
    J.width = g.imageWidth;
    J.height = g.imageHeight;
    J.margin = LOLA_MARGIN;
    J.pitch = lolaStorePitch(g.imageWidth, storage, pix);
    J.rows = g.imageHeight + 2 * LOLA_MARGIN;
    if ((long long)J.pitch * J.rows >= (1LL << 23) - 2 * (long long)J.pitch)
      return lolaSetError("batch: job %d detector %dx%d too large", j, g.imageWidth,
          g.imageHeight);
    J.slotElems = ((size_t)J.pitch * J.rows + 255) & ~(size_t)255;
    J.slotBytes = J.slotElems * pix;
    J.voxelSize = g.voxelSize;
    J.originIndex = g.originIndex;
    /* the persistent pass's work items (LOLA_BATCH_VPT, LOLA_BATCH_ROWS) */
    {
      const int ty = 32 * LOLA_BATCH_ROWS / LOLA_WARP_X;
      J.tilesX = (J.N + LOLA_WARP_X - 1) / LOLA_WARP_X;
      J.tilesY = (J.N + ty - 1) / ty;
      J.tilesZ = (J.N + LOLA_BATCH_VPT - 1) / LOLA_BATCH_VPT;
    }
    J.nproj = jobs[j].projections;
    J.volume = jobs[j].d_volume;
    J.images = jobs[j].d_images;
    ringOffset[j] = ring;
    ring += (size_t)b * J.slotBytes;
    maxPitch = J.pitch > maxPitch ? J.pitch : maxPitch;
    maxRows = J.rows > maxRows ? J.rows : maxRows;
    bt->updates += (double)J.N * J.N * J.N * J.nproj;
    const int w = (J.nproj + b - 1) / b;
    bt->waves = w > bt->waves ? w : bt->waves;
  }
  bt->ringBytes = ring;
  BT_TRY(cudaMalloc(&bt->d_ring, ring));
  BT_TRY(cudaMemset(bt->d_ring, 0, ring));

  const int ch = textureChannels(storage);
  std::vector<unsigned long long> texHandles;
  if (ch > 0) {
    texHandles.resize((size_t)nj * b);
    for (int j = 0; j < nj; ++j)
      for (int s = 0; s < b; ++s) {
        cudaResourceDesc rd;
        memset(&rd, 0, sizeof(rd));
        unsigned char *slotBase = bt->d_ring + ringOffset[j] + (size_t)s * hj[j].slotBytes;
        const int bits = 8 * pix / ch;
        const cudaChannelFormatDesc texel = cudaCreateChannelDesc(bits, ch > 1 ? bits : 0,
            ch > 1 ? bits : 0, ch > 1 ? bits : 0, cudaChannelFormatKindFloat);
        if (LOLA_MIXED_TEX_LINEAR && ch == 4) {
          /* mixed layouts: quads fetched by their integer index in the slot */
          rd.resType = cudaResourceTypeLinear;
          rd.res.linear.devPtr = slotBase;
          rd.res.linear.desc = texel;
          rd.res.linear.sizeInBytes = hj[j].slotBytes;
        } else {
          rd.resType = cudaResourceTypePitch2D;
          rd.res.pitch2D.devPtr = slotBase;
          rd.res.pitch2D.desc = texel;
          rd.res.pitch2D.width = (size_t)hj[j].pitch;
          rd.res.pitch2D.height = (size_t)hj[j].rows;
          rd.res.pitch2D.pitchInBytes = (size_t)hj[j].pitch * pix;
        }
        cudaTextureDesc td;
        memset(&td, 0, sizeof(td));
        td.addressMode[0] = cudaAddressModeBorder;
        td.addressMode[1] = cudaAddressModeBorder;
        td.filterMode = cudaFilterModePoint;
        td.readMode = cudaReadModeElementType;
        cudaTextureObject_t t = 0;
        BT_TRY(cudaCreateTextureObject(&t, &rd, &td, nullptr));
        bt->textures.push_back(t);
        texHandles[(size_t)j * b + s] = (unsigned long long)t;
      }
    BT_TRY(cudaMalloc(&bt->d_tex, texHandles.size() * sizeof(unsigned long long)));
    BT_TRY(cudaMemcpy(bt->d_tex, texHandles.data(),
        texHandles.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice));
  }
  for (int j = 0; j < nj; ++j) {
    hj[j].ring = bt->d_ring + ringOffset[j];
    hj[j].tex = ch > 0 ? bt->d_tex + (size_t)j * b : nullptr;
  }
  BT_TRY(cudaMalloc(&bt->d_jobs, (size_t)nj * sizeof(LolaBatchJob)));
  BT_TRY(cudaMemcpy(bt->d_jobs, hj.data(), (size_t)nj * sizeof(LolaBatchJob),
      cudaMemcpyHostToDevice));

  if (bt->cfg.batchMode == LOLA_BATCH_BRANCHES)
    return captureBranches(bt, jobs, hj, texHandles);

  /* per wave: work lists over the jobs still active and their projections */
  const int W = bt->waves;
  std::vector<long long> prefix((size_t)W * (nj + 1));
  std::vector<LolaPassProj> proj((size_t)W * nj * b);
  memset(proj.data(), 0, proj.size() * sizeof(LolaPassProj));
  std::vector<long long> totals(W);
  for (int w = 0; w < W; ++w) {
    long long acc = 0;
    for (int j = 0; j < nj; ++j) {
      prefix[(size_t)w * (nj + 1) + j] = acc;
      const int count = hj[j].nproj - w * b;
      if (count > 0)
        acc += (long long)hj[j].tilesX * hj[j].tilesY * hj[j].tilesZ;
      for (int s = 0; s < b && s < count; ++s) {
        const double *m = jobs[j].h_matrices + 12 * (size_t)(w * b + s);
        LolaPassProj &pp = proj[((size_t)w * nj + j) * b + s];
        memcpy(pp.a, m, 12 * sizeof(double));
        for (int ax = 0; ax < 3; ++ax)
          for (int c = 0; c < 3; ++c)
            pp.step[ax][c] = (float)(m[ax * 3 + c] * (double)hj[j].voxelSize);
        pp.slot = s;
      }
    }
    prefix[(size_t)w * (nj + 1) + nj] = acc;
    totals[w] = acc;
  }
  BT_TRY(cudaMalloc(&bt->d_prefix, prefix.size() * sizeof(long long)));
  BT_TRY(cudaMemcpy(bt->d_prefix, prefix.data(), prefix.size() * sizeof(long long),
      cudaMemcpyHostToDevice));
  BT_TRY(cudaMalloc(&bt->d_proj, proj.size() * sizeof(LolaPassProj)));
  BT_TRY(cudaMemcpy(bt->d_proj, proj.data(), proj.size() * sizeof(LolaPassProj),
      cudaMemcpyHostToDevice));
  BT_TRY(cudaMalloc(&bt->d_counters, (size_t)W * sizeof(int)));

  /* persistent grid: every resident slot of the GPU */
  int sms = 0, perSM = 0;
  BT_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, bt->device));
  /* the jobs in each wave's kernel parameters (batchParamPassKernel) when they
     fit there, for the layouts read by loads or, f16qx, through one linear
     texture over each job's slots */
  int paramJobs = nj <= LOLA_BATCH_PARAM_JOBS && ch != 1;
  std::vector<unsigned long long> jobTex(nj, 0ull);
  if (paramJobs && storage == LOLA_STORE_F16QX) {
    int maxLinear = 0;
    BT_TRY(cudaDeviceGetAttribute(&maxLinear, cudaDevAttrMaxTexture1DLinearWidth, bt->device));
    for (int j = 0; j < nj; ++j)
      if ((double)b * (double)hj[j].slotElems > (double)maxLinear ||
          (double)b * (double)hj[j].slotElems >= 4294967296.0)
        paramJobs = 0;
    for (int j = 0; paramJobs && j < nj; ++j) {
      cudaResourceDesc rd;
      memset(&rd, 0, sizeof(rd));
      rd.resType = cudaResourceTypeLinear;
      rd.res.linear.devPtr = bt->d_ring + ringOffset[j];
      rd.res.linear.desc = cudaCreateChannelDesc(16, 16, 16, 16, cudaChannelFormatKindFloat);
      rd.res.linear.sizeInBytes = (size_t)b * hj[j].slotBytes;
      cudaTextureDesc td;
      memset(&td, 0, sizeof(td));
      td.addressMode[0] = cudaAddressModeBorder;
      td.filterMode = cudaFilterModePoint;
      td.readMode = cudaReadModeElementType;
      cudaTextureObject_t t = 0;
      BT_TRY(cudaCreateTextureObject(&t, &rd, &td, nullptr));
      bt->textures.push_back(t);
      jobTex[j] = (unsigned long long)t;
    }
  }
  int rc = lolaBatchPassOccupancy(storage, bt->cfg.accumulation, paramJobs, &perSM);
  if (rc != 0 || perSM <= 0)
    return lolaSetError("batch: occupancy query failed (%d)", rc);
  bt->blocks = sms * perSM;

  /* capture the run */
  BT_TRY(cudaStreamBeginCapture(bt->stream, cudaStreamCaptureModeThreadLocal));
  int launchRc = 0;
  cudaError_t me = cudaMemsetAsync(bt->d_counters, 0, (size_t)W * sizeof(int), bt->stream);
  for (int w = 0; w < W && me == cudaSuccess && launchRc == 0; ++w) {
    LolaBatchWave wa;
    memset(&wa, 0, sizeof(wa));
    wa.paramJobs = paramJobs;
    for (int j = 0; paramJobs && j < nj; ++j) {
      const LolaBatchJob &J = hj[j];
      LolaBatchParamJob &q = wa.pj[j];
      q.volume = J.volume;
      q.ring = J.ring;
      q.tex = jobTex[j];
      q.firstItem = prefix[(size_t)w * (nj + 1) + j];
      q.slotBytes = J.slotBytes;
      q.slotElems = (uint32_t)J.slotElems;
      q.count = J.nproj - w * b;
      q.N = J.N;
      q.width = J.width;
      q.height = J.height;
      q.pitch = J.pitch;
      q.rows = J.rows;
      q.tilesX = J.tilesX;
      q.tilesY = J.tilesY;
      q.voxelSize = J.voxelSize;
      q.originIndex = J.originIndex;
    }
    wa.jobs = bt->d_jobs;
    wa.tilePrefix = bt->d_prefix + (size_t)w * (nj + 1);
    wa.proj = bt->d_proj + (size_t)w * nj * b;
    wa.counter = bt->d_counters + w;
    wa.totalItems = totals[w];
    wa.njobs = nj;
    wa.b = b;
    wa.wave = w;
    wa.maxPitch = maxPitch;
    wa.maxRows = maxRows;
    wa.accumulation = bt->cfg.accumulation;
    wa.storage = storage;
    launchRc = lolaLaunchBatchPack(&wa, bt->stream);
    if (launchRc == 0)
      launchRc = lolaLaunchBatchPass(&wa, bt->blocks, bt->stream);
    bt->launches += 2;
  }
  cudaError_t ce = cudaStreamEndCapture(bt->stream, &bt->graph);
  if (me != cudaSuccess || launchRc != 0 || ce != cudaSuccess)
    return lolaSetError("batch: capture failed: %s / %s / %s", cudaGetErrorString(me),
        cudaGetErrorString((cudaError_t)launchRc), cudaGetErrorString(ce));
  BT_TRY(cudaGraphInstantiate(&bt->exec, bt->graph, 0));
  return 1;
}

} /* namespace */

extern "C" int lolaCudaBatchCreate(const LolaCudaJob *jobs, int njobs,
    const LolaCudaConfig *config, LolaCudaBatch **out)
{
  if (out == nullptr || jobs == nullptr || njobs <= 0)
    return lolaSetError("batch: no jobs");
  *out = nullptr;
  LolaCudaBatch *bt = new LolaCudaBatch();
  if (config != nullptr)
    bt->cfg = *config;
  else
    lolaCudaDefaultConfig(&bt->cfg);
  bt->device = bt->cfg.device;
  bt->njobs = njobs;
  bt->b = bt->cfg.batch;
  if (bt->b < 1 || bt->b > LOLA_BATCH_MAX_WAVE || pixelBytes(bt->cfg.storage) == 0 ||
      (bt->cfg.accumulation != LOLA_ACCUM_PLAIN && bt->cfg.accumulation != LOLA_ACCUM_KAHAN)) {
    delete bt;
    return lolaSetError("batch: invalid configuration");
  }
  for (int j = 0; j < njobs; ++j) {
    const LolaCudaGeometry &g = jobs[j].geometry;
    if (g.problemSize <= 0 || g.problemSize > 2048 || g.imageWidth <= 0 ||
        g.imageHeight <= 0 || !(g.voxelSize > 0.0f) || jobs[j].projections < 0 ||
        (jobs[j].projections > 0 && (jobs[j].d_images == nullptr ||
                                     jobs[j].h_matrices == nullptr)) ||
        jobs[j].d_volume == nullptr) {
      delete bt;
      return lolaSetError("batch: job %d is invalid", j);
    }
  }
  if (!build(bt, jobs)) {
    char msg[512];
    strncpy(msg, lolaCudaLastError(), sizeof(msg) - 1);
    msg[sizeof(msg) - 1] = 0;
    release(bt);
    return lolaSetError("%s", msg);
  }
  *out = bt;
  return 1;
}

extern "C" int lolaCudaBatchRun(LolaCudaBatch *bt)
{
  if (bt == nullptr)
    return lolaSetError("batch: null");
  BT_TRY(cudaSetDevice(bt->device));
  BT_TRY(cudaGraphLaunch(bt->exec, bt->stream));
  return 1;
}

extern "C" int lolaCudaBatchSynchronize(LolaCudaBatch *bt)
{
  if (bt == nullptr)
    return lolaSetError("batch: null");
  BT_TRY(cudaSetDevice(bt->device));
  BT_TRY(cudaStreamSynchronize(bt->stream));
  return 1;
}

extern "C" void *lolaCudaBatchStream(LolaCudaBatch *bt)
{
  return bt ? (void *)bt->stream : nullptr;
}

extern "C" int lolaCudaBatchGetInfo(LolaCudaBatch *bt, LolaCudaBatchInfo *info)
{
  if (bt == nullptr || info == nullptr)
    return lolaSetError("batch: null argument");
  info->jobs = bt->njobs;
  info->waves = bt->waves;
  info->blocks = bt->blocks;
  info->launchesPerRun = bt->launches;
  info->voxelUpdates = bt->updates;
  info->ringBytes = bt->ringBytes;
  return 1;
}

extern "C" int lolaCudaBatchDestroy(LolaCudaBatch *bt)
{
  release(bt);
  return 1;
}
