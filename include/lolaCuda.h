/* LolaCUDA — GB300 (sm_103a) cone-beam backprojection module for RabbitCT.
 *
 * C ABI of liblolacuda.so.  Three groups of entry points:
 *
 *  1. The RabbitCT module API.  lolaCudaPrepare / lolaCudaBackprojection /
 *     lolaCudaFinish have exactly the signatures of the reference's module
 *     function-pointer types (HPC-Dwarfs/RabbitCT src/moduleLoader_types.h:10-12)
 *     and are registered as one more row of the static algorithm table
 *     (src/algorithmRegistry.c:39-48), so the stock rabbitRunner drives them
 *     like LolaBunny / LolaOPT / LolaASM.
 *
 *  2. Configuration (no counterpart in the reference, whose modules are
 *     configured at compile time): storage type of the projections, the
 *     accumulation mode, the number of projections staged per kernel pass and
 *     the error convention.
 *
 *  3. The plan API: the same kernels driven on device-resident data, for
 *     callers that keep projections in HBM (the benchmark, batched
 *     reconstructions, tests).  All pointers named d_* are device pointers.
 *
 * Return convention: 1 = success, 0 = failure (message in lolaCudaLastError()),
 * like the reference modules' `return 1`.  By default the three module entry
 * points print the error and exit(EXIT_FAILURE) on failure, which is the
 * reference convention (src/error.h:21-31) and necessary because rabbitRunner
 * ignores the return codes (src/rabbitRunner.c:225,279,287).
 */
#ifndef LOLACUDA_H
#define LOLACUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- RabbitCT data contract --------------------------------------------
 * Layout-identical to the reference's src/rabbitCt.h:9-27.  The include guard
 * of that header is honoured in both directions so the two headers can be
 * included together in a registry translation unit. */
#ifndef RABBITRUNNER_TYPES_H
#define RABBITRUNNER_TYPES_H
typedef struct {
  int id;          /* 1-based global projection index */
  double *matrix;  /* 12 doubles, 3x4 column-major: a[col*3 + row] */
  float *image;    /* imageWidth * imageHeight floats, image[j*W + i] */
} Projection;

typedef struct {
  uint32_t problemSize;          /* N: volume is N^3 voxels */
  uint32_t imageWidth;
  uint32_t imageHeight;
  float voxelSize;               /* mm */
  float O_Index;                 /* world coordinate of voxel index 0 */
  float *volumeData;             /* N^3 floats, x fastest, host */
  uint32_t numberOfProjections;  /* total at prepare with -a, else 0; per call: batch size */
  double *globalGeometry;        /* numberOfProjections * 12 doubles (with -a) */
  Projection *projectionBuffer;
  char *clipFilename;
} RabbitCtGlobalData;
#endif

/* ---- 1. Module API --------------------------------------------------------
 * Replaces FncPrepareAlgorithmType (src/moduleLoader_types.h:10).  Called once
 * (src/rabbitRunner.c:222-232).  Allocates the device volume and the
 * projection ring and starts the upload of the caller's volumeData as the
 * starting volume; the first pass overlaps that upload chunk by chunk, so
 * volumeData must not change before finish (the runner does not touch it). */
int lolaCudaPrepare(RabbitCtGlobalData *data);

/* Replaces FncAlgorithmIterationType (src/moduleLoader_types.h:11).  Called
 * once per batch of data->numberOfProjections projections
 * (src/rabbitRunner.c:279).  The projections' images and matrices are copied
 * before it returns (the runner overwrites them, src/rabbitRunner.c:275-278).
 * Projections are staged until `batch` are buffered or the last global id is
 * reached, then backprojected; with syncEachCall (default) the call returns
 * only after that work finished, so the runner's timer covers it. */
int lolaCudaBackprojection(RabbitCtGlobalData *data);

/* Replaces FncFinishAlgorithmType (src/moduleLoader_types.h:12).  Flushes any
 * staged projections, completes the copy of the volume to data->volumeData
 * (which the scan's last pass starts chunk by chunk when the scan length is
 * known) and frees all device resources (src/rabbitRunner.c:287). */
int lolaCudaFinish(RabbitCtGlobalData *data);

/* ---- 2. Configuration ------------------------------------------------------ */
#define LOLA_MAX_BATCH 64

enum {
  LOLA_STORE_F32 = 0,   /* 4 FP32 taps per update */
  LOLA_STORE_F16 = 1,   /* 4 FP16 taps */
  LOLA_STORE_BF16 = 2,  /* 4 BF16 taps */
  LOLA_STORE_F32Q = 3,  /* FP32, 2x2 neighbourhood packed per pixel: 1 x 16 B load */
  LOLA_STORE_F16Q = 4,  /* FP16, packed 2x2: 1 x 8 B load */
  LOLA_STORE_BF16Q = 5, /* BF16, packed 2x2: 1 x 8 B load */
  LOLA_STORE_TEX32 = 6, /* FP32 texture: one 4-texel gather (tld4) per update */
  LOLA_STORE_TEX16 = 7, /* FP16 texture: one 4-texel gather, widened by the texture unit */
  LOLA_STORE_F16QX = 8, /* FP16 2x2 quads read both by loads and as an RGBA16F texture:
                           each thread's voxels alternate between the two paths */
  LOLA_STORE_F32QX = 9  /* FP32 2x2 quads, loads + RGBA32F texture */
};

enum {
  LOLA_ACCUM_PLAIN = 0, /* vol += term, FP32 */
  LOLA_ACCUM_KAHAN = 1  /* compensated FP32 summation over each kernel pass */
};

typedef struct {
  int32_t storage;       /* LOLA_STORE_* */
  int32_t accumulation;  /* LOLA_ACCUM_* */
  int32_t batch;         /* projections per kernel pass, 1..LOLA_MAX_BATCH */
  int32_t voxelsPerThread; /* voxels per thread along z: 4, 8 or 16 (0 = default) */
  int32_t rowsPerBlock;  /* warps (y rows) per block: 4 or 8 (0 = default) */
  int32_t syncEachCall;  /* module API: wait for the pass before returning */
  int32_t exitOnError;   /* module API: print + exit(EXIT_FAILURE) on error */
  int32_t collectStats;  /* record CUDA events around every backprojection pass */
  int32_t device;        /* CUDA device ordinal */
  int32_t staging;       /* 1: stage each tile's projection footprint in shared
                            memory with tensor copies where it fits; 0: gather
                            through the load / texture path (default: measured
                            faster on GB300 at N=1024) */
  int32_t batchMode;     /* batched reconstructions: LOLA_BATCH_* */
  int32_t batchBranches; /* LOLA_BATCH_BRANCHES: concurrent graph branches (0 = 16) */
  int32_t batchTune;     /* LOLA_BATCH_BRANCHES: time the tile shapes once per distinct
                            (N, detector) class at create and use the fastest for
                            its jobs (1), or use voxelsPerThread x rowsPerBlock (0,
                            the default) */
  int32_t edgeBatch;     /* projections in the edge passes of a scan, 0 = twice batch,
                            at most LOLA_MAX_BATCH; batch..LOLA_MAX_BATCH otherwise.
                            The first pass after an asynchronous volume upload and,
                            where the module API knows the scan length (-a), its
                            last pass take this many: the volume transfers they
                            overlap (one z-chunk at a time) then hide behind more
                            compute.  Set it to batch for uniform passes. */
  int32_t reserved[2];
} LolaCudaConfig;

enum {
  LOLA_BATCH_BRANCHES = 0,  /* per-job pass launches in parallel graph branches */
  LOLA_BATCH_PERSISTENT = 1 /* one persistent pass launch per wave over all jobs */
};

/* Defaults: FP32 quad storage (LOLA_STORE_F32Q: the same results as LOLA_STORE_F32,
 * faster), plain accumulation, batch 16, 16 voxels per thread,
 * 4 rows per block, syncEachCall 1, exitOnError 1, no stats, device 0,
 * staging 0, edge passes of twice batch (32).
 * Environment overrides read by lolaCudaDefaultConfig: LOLACUDA_STORAGE
 * (f32|f16|bf16|f32q|f16q|bf16q|tex32|tex16|f16qx|f32qx), LOLACUDA_ACCUM (plain|kahan),
 * LOLACUDA_BATCH, LOLACUDA_VPT, LOLACUDA_ROWS, LOLACUDA_SYNC, LOLACUDA_EXIT,
 * LOLACUDA_STAGING, LOLACUDA_EDGE_BATCH. */
void lolaCudaDefaultConfig(LolaCudaConfig *config);

/* Configuration used by the next lolaCudaPrepare (module API). */
int lolaCudaSetConfig(const LolaCudaConfig *config);
int lolaCudaGetConfig(LolaCudaConfig *config);

/* Last error message of this thread ("" if none). */
const char *lolaCudaLastError(void);

/* ---- 3. Plan API ------------------------------------------------------------ */
typedef struct {
  int32_t problemSize;   /* N */
  int32_t imageWidth;
  int32_t imageHeight;
  float voxelSize;
  float originIndex;     /* O_Index */
  /* z-slab held by the plan: slices [sliceBegin, sliceBegin + sliceCount) of
     the N^3 volume (sliceCount 0 = the whole volume).  Slabs let several GPUs
     share one volume with no exchange: each backprojects every projection
     into its own slab.  Slabs starting at multiples of the tile depth
     (voxelsPerThread) give bit-identical voxels to an unsharded plan. */
  int32_t sliceBegin;
  int32_t sliceCount;
} LolaCudaGeometry;

typedef struct {
  int64_t passes;        /* backprojection kernel launches since the last reset */
  int64_t packs;         /* projection-conversion kernel launches */
  int64_t projections;   /* projections backprojected */
  double passMs;         /* summed CUDA-event time of the passes (collectStats) */
  int64_t tilePassesFast;  /* (tile, projection) pairs on the unclamped path */
  int64_t tilePassesSlow;  /* ... on the clamped border path */
  int64_t tilePassesSkipped; /* ... whose footprint misses the detector */
  int64_t tilePassesStaged;  /* fast-path pairs served from shared-memory staging */
  int64_t stagedPasses;      /* passes launched with staging */
  int64_t overlappedPasses;  /* passes run in z-chunks to overlap a volume transfer */
  int64_t chunkLaunches;     /* kernel launches of those passes */
  int64_t tilePassesPaired;  /* fast-path pairs run two voxels per packed instruction */
} LolaCudaStats;

typedef struct LolaCudaPlan LolaCudaPlan;

/* Allocates the device volume (zeroed) and the projection ring. */
int lolaCudaPlanCreate(const LolaCudaGeometry *geometry, const LolaCudaConfig *config,
    LolaCudaPlan **plan);
int lolaCudaPlanDestroy(LolaCudaPlan *plan);

/* Device pointer of the plan's FP32 volume, N x N x sliceCount, x fastest.
 * Work the caller then puts on the plan's stream is ordered after the plan's
 * volume transfers. */
float *lolaCudaPlanVolume(LolaCudaPlan *plan);
/* cudaStream_t the plan launches on. */
void *lolaCudaPlanStream(LolaCudaPlan *plan);

int lolaCudaPlanZeroVolume(LolaCudaPlan *plan);
/* Synchronous copies of the whole volume. */
int lolaCudaPlanUploadVolume(LolaCudaPlan *plan, const float *h_volume);
int lolaCudaPlanDownloadVolume(LolaCudaPlan *plan, float *h_volume);
/* Uploads h_volume asynchronously in z-chunks on the plan's transfer stream;
 * the next pass starts on each chunk as soon as it has landed.  From
 * page-locked memory the call returns at once and the copies are issued with
 * that pass, after the projections it reads (or by any other operation on
 * the volume or lolaCudaPlanSynchronize, whichever comes first); from
 * pageable memory they are issued before the call returns (the driver holds
 * the thread until it has read the volume).  h_volume must stay unchanged
 * until lolaCudaPlanSynchronize.  The next host-staged pass takes up to the
 * edge batch of projections (LolaCudaConfig.edgeBatch). */
int lolaCudaPlanUploadVolumeAsync(LolaCudaPlan *plan, const float *h_volume);
/* Asks for the volume in h_volume after the last pass of the next
 * backprojection call (lolaCudaPlanBackprojectHost / Device): that pass runs
 * in z-chunks and each chunk is copied out as soon as it is finished, so the
 * download overlaps the pass.  If no pass runs first, lolaCudaPlanSynchronize
 * copies the volume as it is.  The copy is complete when
 * lolaCudaPlanSynchronize returns.  Results are identical to a whole pass
 * followed by lolaCudaPlanDownloadVolume. */
int lolaCudaPlanStreamVolumeOut(LolaCudaPlan *plan, float *h_volume);

/* Backprojects `count` FP32 projections that are already in device memory
 * (d_images[p * imageStride + j * W + i]) with host matrices
 * h_matrices[p * 12 + ...], in passes of `batch`.  Asynchronous on the plan's
 * stream; the matrices are consumed before the call returns. */
int lolaCudaPlanBackprojectDevice(LolaCudaPlan *plan, const float *d_images,
    size_t imageStride, const double *h_matrices, int count);

/* Same from host images (h_images[p * imageStride + ...]); the images are
 * copied to the device before the call returns.  Each call closes its last
 * pass.  Passes take `batch` projections, except the edge passes: the first
 * after lolaCudaPlanUploadVolumeAsync and, in a call made after
 * lolaCudaPlanStreamVolumeOut, the last (the pass before it is shortened so
 * that it is full), which take up to the edge batch. */
int lolaCudaPlanBackprojectHost(LolaCudaPlan *plan, const float *h_images,
    size_t imageStride, const double *h_matrices, int count);

int lolaCudaPlanSynchronize(LolaCudaPlan *plan);

/* CUDA-event timer on the plan's stream: Start records an event, Stop records
 * one, waits for it and returns the elapsed milliseconds in *ms. */
int lolaCudaPlanTimerStart(LolaCudaPlan *plan);
int lolaCudaPlanTimerStop(LolaCudaPlan *plan, double *ms);
int lolaCudaPlanGetStats(LolaCudaPlan *plan, LolaCudaStats *stats);
int lolaCudaPlanResetStats(LolaCudaPlan *plan);

/* ---- Batched reconstructions ---------------------------------------------------
 * No counterpart in the reference, whose runner drives one reconstruction per
 * process.  Many volumes of uneven size, detector and projection count are
 * reconstructed together, the whole run captured into a CUDA graph at create
 * and replayed by each run.  Two schedules (config batchMode):
 * LOLA_BATCH_BRANCHES (default) runs each job's pack and pass launches in one
 * of batchBranches parallel graph branches, with tile shapes timed per
 * (N, detector) class when batchTune is set; LOLA_BATCH_PERSISTENT runs, per
 * wave of `batch` projections of every job, one pack launch and one
 * persistent pass launch whose blocks pull (job, tile) work items from a
 * counter.  All jobs share the config's storage, accumulation and batch (at
 * most 32 projections per wave here); FP32 arithmetic throughout. */
typedef struct {
  LolaCudaGeometry geometry;   /* whole volume: slice fields must be 0 */
  int32_t projections;
  int32_t reserved;
  const float *d_images;       /* projections x imageHeight x imageWidth FP32, device */
  const double *h_matrices;    /* projections x 12, host; copied at create */
  float *d_volume;             /* N^3 FP32, device, caller-owned; accumulated into */
} LolaCudaJob;

typedef struct {
  int32_t jobs;
  int32_t waves;
  int32_t blocks;              /* persistent blocks per pass launch */
  int32_t launchesPerRun;
  double voxelUpdates;         /* sum over jobs of N^3 x projections */
  size_t ringBytes;
} LolaCudaBatchInfo;

typedef struct LolaCudaBatch LolaCudaBatch;

int lolaCudaBatchCreate(const LolaCudaJob *jobs, int njobs, const LolaCudaConfig *config,
    LolaCudaBatch **batch);
/* Replays the captured run on the batch's stream (asynchronous). */
int lolaCudaBatchRun(LolaCudaBatch *batch);
int lolaCudaBatchSynchronize(LolaCudaBatch *batch);
void *lolaCudaBatchStream(LolaCudaBatch *batch);
int lolaCudaBatchGetInfo(LolaCudaBatch *batch, LolaCudaBatchInfo *info);
int lolaCudaBatchDestroy(LolaCudaBatch *batch);

/* ---- Verification on the device ------------------------------------------------
 * The runner's -c check (src/rabbitRunner.c:320-384) without copying the
 * volume to the host: HU = floor(hus[0] * v + hus[1] + 0.5) for v > 0 else 0,
 * clamped to 4095, against a uint16 HU reference volume (host memory, N^3).
 * With convertInPlace the HU values replace the volume, as the runner does
 * before it writes -o. */
typedef struct {
  double mse;              /* HU^2 */
  double rmse;             /* HU */
  double maxAbs;           /* HU */
  double psnr;             /* dB, 10 log10(4095^2 / mse); inf when mse <= 1e-8 */
  uint64_t histogram[11];  /* |error| in [0,1), [1,2), ..., [9,10), >= 10 */
} LolaCudaQuality;

int lolaCudaVerifyVolume(float *d_volume, size_t voxels, const uint16_t *h_reference,
    const float *hus, int convertInPlace, void *stream, LolaCudaQuality *quality);
int lolaCudaPlanVerify(LolaCudaPlan *plan, const uint16_t *h_reference, const float *hus,
    int convertInPlace, LolaCudaQuality *quality);

/* The runner's optional outputs from the plan's volume, copying only slice
 * N/2-1 to the host.  lolaCudaPlanWriteSlicePgm replaces the -p writer
 * (src/rabbitRunner.c:289-315): the slice in HU as a 16-bit big-endian PGM;
 * call it before lolaCudaPlanWriteResult, which converts the volume to HU.
 * lolaCudaPlanWriteResult replaces the -c result.rctd writer
 * (src/rabbitRunner.c:317-412): verifies on the device (converting in place,
 * as the runner does), then writes the file with totalMicroseconds /
 * numberOfImages as every image's time.  It needs a whole-volume plan. */
int lolaCudaPlanWriteSlicePgm(LolaCudaPlan *plan, const char *path, const float *hus);
int lolaCudaPlanWriteResult(LolaCudaPlan *plan, const char *path, const uint16_t *h_reference,
    const float *hus, uint32_t numberOfImages, uint64_t totalMicroseconds,
    LolaCudaQuality *quality);

/* ---- Geometry analysis on the device ----------------------------------------
 * Replaces computeLineRanges (src/analyseGeometry.c:102-298) for the
 * reference's clipping modules: range[view] (view < data->numberOfProjections,
 * from data->globalGeometry) receives N*N {start, stop} int16 pairs for rows
 * z*N + y, identical to the reference's table for the same vectorSize
 * (VECTORSIZE there).  signedHit = 0 keeps the reference's hit test (its
 * unsigned comparison counts pixel index -1 as a miss); 1 keeps every voxel
 * LolaBunny reads a non-zero tap for.  No cache file is read or written. */
int lolaCudaComputeLineRanges(const RabbitCtGlobalData *data, int16_t **range, int vectorSize,
    int signedHit);
/* computeShadowOfProjection (src/analyseGeometry.c:50-93): shadow[4] =
 * {Umin, Umax, Vmin, Vmax}. */
int lolaCudaComputeShadow(const RabbitCtGlobalData *data, int *shadow);

/* Slab of `rank` among `ranks` for an N^3 volume: near-equal counts, starts at
 * multiples of `align` (the tile depth) so voxels match an unsharded plan. */
int lolaCudaSlab(int problemSize, int rank, int ranks, int align, int32_t *sliceBegin,
    int32_t *sliceCount);

/* ---- Backprojection without device allocation ------------------------------
 * No counterpart in the reference (its modules are CPU code).  For callers
 * that cannot allocate device memory while they run — an acquisition loop
 * that reserves its device memory at start-up and must not stall on
 * cudaMalloc/cudaFree (which can synchronise the device), or a host framework
 * that owns the device memory pool.  Same result, bit for bit, as
 * lolaCudaPlanBackprojectDevice with the same batch into a caller-owned
 * volume: d_volume (N x N x sliceCount FP32, x fastest; the geometry's slab
 * fields as for a plan, 0 / 0 = the whole N^3 volume) += the `count` FP32
 * projections at d_images[p * imageStride + j * W + i] with host matrices
 * h_matrices[p * 12 + ...].  Enqueued on `stream` (a cudaStream_t of the
 * current device, NULL = its default stream); the caller synchronises.  Runs
 * on the calling thread's current device: config->device is not used.
 * `config` may be NULL (defaults); its batch is capped by what fits in the
 * scratch.  Storages: f32, f16, bf16, f32q, f16q, bf16q; f16qx and f32qx run
 * as f16q and f32q (the same values, by loads only); tex32 and tex16 are
 * rejected.  Projections per pass at 1248x960: f32 5, f16/bf16 10,
 * f16q/bf16q 2, f32q 1 (the default storage).
 * Calls no cudaMalloc, cudaFree or other allocating routine: the packed
 * projections live in a fixed LOLA_NOALLOC_SCRATCH_BYTES device array, and
 * each pass's projection records (LOLA_MAX_BATCH x 152 bytes) in a second,
 * both held by every GPU loading this library until exit; a one-block kernel
 * per pass fills the second from its launch parameters.  A packed projection
 * larger than the first array is rejected with an error.  All calls share the
 * arrays, so calls whose work overlaps on the GPU race and must be serialised.
 * The arrays' device addresses are looked up on the first call in each CUDA
 * context (each device's primary context, normally): make that call before
 * any stream capture begins, and do not reset the device between calls. */
#define LOLA_NOALLOC_SCRATCH_BYTES (32u << 20)
int lolaCudaBackprojectNoAlloc(const LolaCudaGeometry *geometry, const LolaCudaConfig *config,
    float *d_volume, const float *d_images, size_t imageStride, const double *h_matrices,
    int count, void *stream);

/* ---- Reconstruction from a .rct file ---------------------------------------
 * The input path of the reference runner (src/ctFileReader.c:47-61,
 * src/rabbitRunner.c:267-287) without the runner: the projection records of
 * a .rct file are read in chunks of `batch` into two page-locked buffers in
 * turn, so disk reads overlap uploads and passes.  h_volume (N^3, host) is
 * the starting volume and receives the result. */
typedef struct {
  double seconds;       /* wall time of the whole call */
  double readSeconds;   /* time spent reading the file */
  int64_t projections;
  double gups;          /* N^3 x projections / seconds */
  float hus[2];         /* the file's HU scaling factors */
} LolaCudaFileReport;

int lolaCudaReadRctHeader(const char *path, uint32_t *width, uint32_t *height, uint32_t *count,
    float *hus);
int lolaCudaReconstructFile(const char *path, int problemSize, float voxelSize,
    float originIndex, const LolaCudaConfig *config, float *h_volume,
    LolaCudaFileReport *report);

/* The runner's module loop (src/rabbitRunner.c:222-287) over projections that
 * are already in host memory, in C: prepare, one lolaCudaBackprojection call
 * per callBatch projections (each Projection pointing into h_images and
 * h_matrices, ids 1..count), finish.  data holds the geometry, volumeData and
 * (optionally, like -a) globalGeometry with numberOfProjections = count; its
 * projectionBuffer and numberOfProjections are used during the calls and
 * restored.  Wall-clock times of the three phases (CLOCK_MONOTONIC), like the
 * runner's timer around its calls.  No counterpart in the reference, whose
 * runner reads each projection from the file between calls. */
typedef struct {
  double prepareSeconds;
  double callSeconds;   /* summed over the backprojection calls (the runner's Total) */
  double finishSeconds;
  double totalSeconds;  /* prepare through finish */
} LolaCudaScanTiming;

int lolaCudaRunScan(RabbitCtGlobalData *data, const float *h_images, size_t imageStride,
    const double *h_matrices, int count, int callBatch, LolaCudaScanTiming *timing);

/* ---- Autotuning --------------------------------------------------------------
 * No counterpart in the reference (compile-time VECTORSIZE / BLOCKING_FACTOR).
 * Times candidate execution parameters — tile shape (voxels per thread x rows
 * per block), projections per pass and shared-memory staging — on the
 * caller's own geometry and projections (count of them, device-resident,
 * FP32) and writes the fastest into *config.  Storage and accumulation are
 * taken from *config unchanged, so the result keeps its accuracy.  Each
 * candidate is timed with CUDA events after a warm-up, on a scratch plan. */
typedef struct {
  int32_t voxelsPerThread, rowsPerBlock, batch, staging;
  double ms;                 /* time for the count projections; < 0: not run */
} LolaCudaTuneCandidate;

#define LOLA_TUNE_MAX_CANDIDATES 64

typedef struct {
  int32_t candidates;
  int32_t best;
  LolaCudaTuneCandidate tried[LOLA_TUNE_MAX_CANDIDATES];
} LolaCudaTuneReport;

int lolaCudaAutotune(const LolaCudaGeometry *geometry, const float *d_images, size_t imageStride,
    const double *h_matrices, int count, LolaCudaConfig *config, LolaCudaTuneReport *report);

/* Small device-memory helpers so hosts without a CUDA binding (ctypes, cgo)
 * can stage device-resident inputs. */
void *lolaCudaDeviceAlloc(size_t bytes);
int lolaCudaDeviceFree(void *d_ptr);
int lolaCudaCopyToDevice(void *d_dst, const void *h_src, size_t bytes);
int lolaCudaCopyToHost(void *h_dst, const void *d_src, size_t bytes);
int lolaCudaDeviceSynchronize(void);

/* Page-locked host memory (cudaHostAlloc), so callers' projection and volume
 * buffers can be DMA'd at full link speed. */
void *lolaCudaHostAlloc(size_t bytes);
int lolaCudaHostFree(void *h_ptr);

/* ---- Measurement helpers (used by the benchmark's roofline) ----------------
 * FP32 FMA issue rate of the current device, thread-instructions per second. */
double lolaCudaProbeIssueRate(void);
/* Voxel updates per second that the pass kernel's 2x2 gather pattern alone
 * sustains for a storage layout over a padded width x height detector, at
 * random positions (L2-resident, no reuse in L1): lanes 1.25 px apart, four
 * independent fetches per thread and step, two rows apart. */
double lolaCudaProbeGatherRate(int storage, int width, int height);
/* The same fetches inside an image small enough to stay in every SM's L1:
 * the rate of the gather pipes themselves for this lane spacing. */
double lolaCudaProbeGatherPeak(int storage);
/* Lane fetches per second of 8-lane texture requests (RGBA16F texels by
 * index, L1-resident) whose eight texels lie in `rows` detector rows (1, 2, 4
 * or 8; -1 for another value): what a request that straddles rows costs. */
double lolaCudaProbeTextureRows(int rows);
/* SM count, SM clock (kHz) and name of the current device. */
int lolaCudaDeviceInfo(int *smCount, int *clockKHz, char *name, int nameLen);

#ifdef __cplusplus
}
#endif

#endif /* LOLACUDA_H */
