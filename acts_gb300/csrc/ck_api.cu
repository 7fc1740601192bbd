// ck_api.cu — implementation of the C ABI declared in include/cudakalman.h.
//
// A ck_handle owns the resident detector (surface table, field map), the
// grow-only device buffers of the batch pipeline, the scratch records of the
// tracks in flight and the tuned launch shape. One handle serves one stream;
// concurrent callers on the same handle are serialised by its mutex.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <mutex>
#include <string>
#include <vector>

#include "ck_api_internal.h"
#include "ck_launch.h"

using namespace ck;

namespace ck {

thread_local std::string g_lastError;

ck_status fail(ck_status s, const std::string& msg) {
  g_lastError = msg;
  return s;
}

ck_status cudaFail(cudaError_t e, const char* what) {
  return fail(e == cudaErrorMemoryAllocation ? CK_ERR_OUT_OF_MEMORY : CK_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

cudaError_t DevBuf::ensure(size_t bytes) {
  if (bytes <= cap) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  size_t want = bytes + bytes / 4 + 256;
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    p = nullptr;
    return e;
  }
  cap = want;
  return cudaSuccess;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
}

MatConst makeMatConst() {
  // Interactions.cpp:23-31 constants, evaluated with the reference's
  // long-double unit literals (Units.hpp:181-187)
  auto MeV = [](long double x) { return (double)(1e-3 * x); };
  auto eV = [](long double x) { return (double)(1e-9 * x); };
  MatConst c;
  c.Me = (float)MeV(0.5109989461L);
  c.K = (float)(MeV(30.7075L) * 1.0);
  c.plasmaScale = (float)eV(28.816L);
  c.invCm3 = static_cast<float>(1 / (10.0 * 10.0 * 10.0));
  c.highland = MeV(13.6L);
  c.rossi = MeV(17.5L);
  c.log10f = (float)std::log((double)10.0f);
  c.pad = 0.0f;
  return c;
}

DevSurface toDevSurface(const ck_surface& s) {
  DevSurface d;
  std::memset(&d, 0, sizeof(d));
  for (int i = 0; i < 9; ++i) d.R[i] = s.rotation[i];
  for (int i = 0; i < 3; ++i) d.c[i] = s.center[i];
  d.radius = s.radius;
  d.type = s.type;
  d.flags = s.flags;
  d.matI = s.mat_mean_excitation;
  d.matNe = s.mat_molar_electron_rho;
  // MaterialSlab(material, thickness) (MaterialSlab.hpp:119-128)
  const float eps = 2 * std::numeric_limits<float>::epsilon();
  d.thickness = s.mat_thickness;
  d.tX0 = (eps < s.mat_x0) ? (s.mat_thickness / s.mat_x0) : 0.0f;
  d.tL0 = (eps < s.mat_l0) ? (s.mat_thickness / s.mat_l0) : 0.0f;
  d.split = s.split_factor;
  d.vacuum = (s.mat_ar > 0.0f) ? 0 : 1;
  for (int i = 0; i < 9; ++i) d.Rf[i] = (float)s.rotation[i];
  for (int i = 0; i < 3; ++i) d.cf[i] = (float)s.center[i];
  d.radiusf = (float)s.radius;
  return d;
}

DevOptions toDevOptions(const ck_options& o) {
  DevOptions d;
  d.stepTolerance = o.step_tolerance;
  d.stepSizeCutOff = o.step_size_cutoff;
  d.initialStepSize = o.initial_step_size;
  d.maxStepSize = o.max_step_size;
  d.pathLimit = o.path_limit;
  d.loopFraction = o.loop_fraction;
  d.surfaceTolerance = o.surface_tolerance;
  d.nearLimit = o.near_limit;
  d.outlierChi2Cut = o.outlier_chi2_cut;
  d.maxRkTrials = o.max_rk_step_trials;
  d.maxSteps = o.max_steps;
  d.maxTargetSkipping = o.max_target_skipping;
  d.loopProtection = o.loop_protection;
  d.multipleScattering = o.multiple_scattering;
  d.energyLoss = o.energy_loss;
  d.joseph = o.use_joseph;
  d.useOutlierCut = std::isinf(o.outlier_chi2_cut) ? 0 : 1;
  d.earlyTermination = o.early_termination;
  d.smoother = o.smoother;
  d.freeToBoundCorrection = o.free_to_bound_correction;
  d.reverseFiltering = o.reverse_filtering;
  d.reverseCovScaling = o.reverse_filtering_cov_scaling;
  d.reverseMomThreshold = o.reverse_filtering_mom_threshold;
  return d;
}

ck_status validateOptions(const ck_options* o) {
  if (!o) return fail(CK_ERR_INVALID_ARGUMENT, "options is NULL");
  if (o->reference_surface < -1)
    return fail(CK_ERR_INVALID_ARGUMENT, "reference_surface must be -1 or a surface index");
  if (o->reference_strategy < CK_EXTRAPOLATE_FIRST ||
      o->reference_strategy > CK_EXTRAPOLATE_FIRST_OR_LAST)
    return fail(CK_ERR_INVALID_ARGUMENT, "unknown reference_strategy");
  if (o->precision < 0 || o->precision >= CK_NUM_PRECISIONS)
    return fail(CK_ERR_INVALID_ARGUMENT, "unknown precision");
  if (o->smoother != CK_SMOOTHER_GAIN_MATRIX && o->smoother != CK_SMOOTHER_MBF)
    return fail(CK_ERR_INVALID_ARGUMENT, "unknown smoother");
  if (!(o->step_tolerance > 0) || !(o->initial_step_size > 0))
    return fail(CK_ERR_INVALID_ARGUMENT, "step tolerance and initial step size must be > 0");
  if (o->max_steps == 0) return fail(CK_ERR_INVALID_ARGUMENT, "max_steps must be > 0");
  return CK_OK;
}

}  // namespace ck

// ------------------------------------------------------------ queue kernels
// The work queue: the tracks ordered by sequence length, longest first, by a
// stable counting sort (tracks of equal length keep their input order, so
// neighbouring queue positions hold neighbouring tracks and the smoother's
// output writes coalesce). Three launches: per-block histograms, one scan
// over (length bin, block) in descending length order, rank-preserving
// scatter.
namespace {

constexpr int kBins = 64;

__device__ __forceinline__ int lengthBin(const int32_t* __restrict__ off, int t) {
  int len = off[t + 1] - off[t];
  return len < 0 ? 0 : (len >= kBins ? kBins - 1 : len);
}

// counts[bin * nb + block]
__global__ void __launch_bounds__(kSortBlock) queueBlockHist(const int32_t* __restrict__ off,
                                                             int n, int32_t* counts, int nb) {
  __shared__ int32_t h[kBins];
  for (int i = threadIdx.x; i < kBins; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const int t = blockIdx.x * kSortBlock + threadIdx.x;
  if (t < n) atomicAdd(&h[lengthBin(off, t)], 1);
  __syncthreads();
  for (int i = threadIdx.x; i < kBins; i += blockDim.x) counts[i * nb + blockIdx.x] = h[i];
}

// exclusive scan of the counts in the order (bin 63 .. 0) x (block 0 .. nb-1),
// one block of kSortBlock threads, each over a contiguous chunk
__global__ void __launch_bounds__(kSortBlock) queueScanCounts(int32_t* counts, int nb) {
  __shared__ int32_t part[kSortBlock];
  const long long total = (long long)kBins * nb;
  const long long chunk = (total + kSortBlock - 1) / kSortBlock;
  const long long lo = threadIdx.x * chunk < total ? threadIdx.x * chunk : total;
  const long long hi = lo + chunk < total ? lo + chunk : total;
  // entry j of the scan order is counts[(kBins - 1 - j / nb) * nb + j % nb]
  auto at = [&](long long j) -> int32_t& {
    return counts[(kBins - 1 - (int)(j / nb)) * (long long)nb + (int)(j % nb)];
  };
  int32_t sum = 0;
  for (long long j = lo; j < hi; ++j) sum += at(j);
  part[threadIdx.x] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    int32_t acc = 0;
    for (int i = 0; i < kSortBlock; ++i) {
      const int32_t c = part[i];
      part[i] = acc;
      acc += c;
    }
  }
  __syncthreads();
  int32_t acc = part[threadIdx.x];
  for (long long j = lo; j < hi; ++j) {
    const int32_t c = at(j);
    at(j) = acc;
    acc += c;
  }
}

__global__ void __launch_bounds__(kSortBlock) queueScatterStable(const int32_t* __restrict__ off,
                                                                 int n,
                                                                 const int32_t* __restrict__ counts,
                                                                 int nb, int32_t* perm) {
  constexpr int kWarps = kSortBlock / 32;
  __shared__ int32_t wc[kWarps][kBins];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kWarps * kBins; i += blockDim.x) wc[i / kBins][i % kBins] = 0;
  __syncthreads();
  const int t = blockIdx.x * kSortBlock + threadIdx.x;
  const int bin = t < n ? lengthBin(off, t) : -1;
  const unsigned same = __match_any_sync(0xffffffffu, bin);
  const int rank = __popc(same & ((1u << lane) - 1u));
  if (bin >= 0 && rank == 0) wc[warp][bin] = __popc(same);
  __syncthreads();
  // exclusive prefix over the warps, per bin
  for (int b = threadIdx.x; b < kBins; b += blockDim.x) {
    int32_t acc = 0;
    for (int w = 0; w < kWarps; ++w) {
      const int32_t c = wc[w][b];
      wc[w][b] = acc;
      acc += c;
    }
  }
  __syncthreads();
  if (bin >= 0) perm[counts[bin * nb + blockIdx.x] + wc[warp][bin] + rank] = t;
}

}  // namespace

// --------------------------------------------------------------- helpers
namespace ck {

size_t compBytes(int n, int maxStates, int C, size_t elem) {
  return (size_t)n * (size_t)maxStates * (size_t)C * elem;
}

void loadTuneCache(ck_handle* h) {
  if (h->cachePath.empty()) return;
  std::ifstream f(h->cachePath);
  int p, v, tpb, bps, spr, stg;
  while (f >> p >> v >> tpb >> bps >> spr >> stg) {
    if (p < 0 || p >= CK_NUM_PRECISIONS || !validLaunch(v, tpb) || bps <= 0 || spr < 1 ||
        spr > 64)
      continue;
    h->tune[p] = {v, tpb, bps, spr, 1, 0, stg ? 1 : 0};
  }
}

void saveTuneCache(ck_handle* h) {
  if (h->cachePath.empty()) return;
  std::ofstream f(h->cachePath);
  for (int p = 0; p < CK_NUM_PRECISIONS; ++p)
    if (h->tune[p].tuned)
      f << p << " " << h->tune[p].variant << " " << h->tune[p].tpb << " " << h->tune[p].bps << " "
        << h->tune[p].spr << " " << h->tune[p].staged << "\n";
}

cudaError_t launchFit(const FitParams& fp, int precision, const Tune& tn, int grid,
                      cudaStream_t st) {
  switch (precision) {
    case CK_PRECISION_MIXED: return launchFitMixed(fp, tn.variant, grid, tn.tpb, st);
    default: return launchFitFP64(fp, tn.variant, grid, tn.tpb, st);
  }
}

int gridBlocksFor(ck_handle* h, const Tune& tn) {
  return tn.grid > 0 ? tn.grid : h->smCount * tn.bps;
}

size_t recordStateBytes(int precision) {
  return precision == CK_PRECISION_MIXED ? sizeof(RecState<float>) : sizeof(RecState<double>);
}

size_t recordBytesPerTrack(int maxStates, int precision) {
  return (size_t)maxStates * recordStateBytes(precision) + 2 * sizeof(int32_t);
}

ck_status validateReference(const ck_handle* h, const ck_options* o) {
  if (o->reference_surface < 0) return CK_OK;
  if (o->reference_surface >= h->nSurfaces)
    return fail(CK_ERR_INVALID_ARGUMENT, "reference_surface outside the surface table");
  if (h->hostSurfaces[o->reference_surface].type != CK_SURFACE_LINE)
    return fail(CK_ERR_UNSUPPORTED, "the reference surface must be a line (perigee) surface");
  return CK_OK;
}

// Allocates (grow-only) the scratch of a batch pipeline: the track-state
// records of n tracks, the queue permutation, the tips and the tail-smoothing
// marks. Never called while a stream is being captured.
ck_status preparePipeline(ck_handle* h, FitContext& c, int n, int maxStates, int precision,
                          bool extrapolate) {
  (void)h;
  cudaError_t e;
  if (extrapolate && (e = c.ext.ensure((size_t)n * 2 * sizeof(ExtStart) + 16)))
    return cudaFail(e, "extrapolation scratch");
  if ((e = c.rec.ensure(compBytes(n, maxStates, 1, recordStateBytes(precision)))) ||
      (e = c.perm.ensure((size_t)n * sizeof(int32_t) + 16)) ||
      (e = c.tip.ensure((size_t)n * sizeof(int32_t) + 16)) ||
      (e = c.sortCounts.ensure(sortCountsBytes(n))) ||
      (e = c.smoothed.ensure((size_t)n + 16)) ||
      (e = c.ticket.ensure(2 * sizeof(int32_t))))
    return cudaFail(e, "scratch allocation");
  return CK_OK;
}

// Records the whole batch pipeline (inputs already on the device, scratch
// prepared) on `st`: queue reset, queue ordering, forward-filter kernel,
// smoother kernel.
ck_status enqueuePipeline(ck_handle* h, FitContext& c, const ck_options& opt,
                          const ck_batch_in& din, const ck_batch_out& dout, const Tune& tn,
                          cudaStream_t st, bool timed, int gridBlocks, const cudaEvent_t* timing) {
  const cudaEvent_t ev0 = timing ? timing[0] : h->ev0, evMid = timing ? timing[1] : h->evMid,
                    ev1 = timing ? timing[2] : h->ev1;
  const int n = din.n_tracks;
  const int grid = gridBlocks;
  const int maxStates = dout.max_states;
  cudaError_t e;
  int32_t* dTicket = (int32_t*)c.ticket.p;
  int launches = 0;
  h->lastChunks = 0;
  cudaMemsetAsync(dTicket, 0, 2 * sizeof(int32_t), st);  // queue and tail-smoothing tickets
  if (n > 0) cudaMemsetAsync(c.tip.p, 0xff, sizeof(int32_t) * (size_t)n, st);
  const int32_t* perm = nullptr;
  if (h->sortQueue && n > 0) {
    const int nb = sortBlocks(n);
    int32_t* counts = (int32_t*)c.sortCounts.p;
    queueBlockHist<<<nb, kSortBlock, 0, st>>>(din.seq_offsets, n, counts, nb);
    queueScanCounts<<<1, kSortBlock, 0, st>>>(counts, nb);
    queueScatterStable<<<nb, kSortBlock, 0, st>>>(din.seq_offsets, n, counts, nb,
                                                  (int32_t*)c.perm.p);
    launches += 3;
    perm = (const int32_t*)c.perm.p;
  }
  FitParams fp;
  std::memset(&fp, 0, sizeof(fp));
  fp.n_tracks = n;
  fp.n_queue = n;
  fp.seq_off = din.seq_offsets;
  fp.seq_surf = din.seq_surfaces;
  fp.meas_off = din.meas_offsets;
  fp.meas_surf = din.meas_surfaces;
  fp.meas_val = din.meas_values;
  fp.meas_cov = din.meas_cov;
  fp.meas_sub = din.meas_subspace;
  fp.start_params = din.start_params;
  fp.start_cov = din.start_cov;
  fp.start_frames = din.start_frames;
  fp.particle = din.particle;
  fp.pdg = din.particle_pdg;
  fp.perm = perm;
  fp.ticket = dTicket;
  fp.rec = c.rec.p;
  fp.tip = (int32_t*)c.tip.p;
  // the free-to-bound correction's kernel: 256 slots, one block per SM
  const bool f2b = opt.free_to_bound_correction != 0;
  const int fitGrid = f2b ? h->smCount : grid;
  const int fitTpb = f2b ? 256 : tn.tpb;
  {
    const long long warps = (long long)fitGrid * (fitTpb / 32);
    const long long per = warps > 0 ? (n + warps - 1) / warps : 32;
    fp.lanes_per_warp = (int)std::min<long long>(32, std::max<long long>(1, per));
  }
  fp.max_states = maxStates;
  fp.out = dout;
  fp.surfaces = h->dSurfaces;
  fp.trig = h->dTrig;
  fp.steps_per_round = tn.spr > 0 ? tn.spr : 1;
  fp.smooth_staged = tn.staged;
  fp.n_surfaces = h->nSurfaces;
  fp.field = h->field;
  fp.mc = h->mc;
  fp.opt = toDevOptions(opt);
  fp.ref_surface = opt.reference_surface;
  fp.ref_strategy = opt.reference_strategy;
  fp.ext = needsExtStart(opt) ? (ExtStart*)c.ext.p : nullptr;
  // smoothing in the forward filter's tail: the compaction kernels (variants
  // 3 and 4, and the free-to-bound correction's), without reverse filtering
  if (h->tailSmoothing && n > 0 && c.smoothed.p && c.smoothed.cap >= (size_t)n &&
      c.ticket.cap >= 2 * sizeof(int32_t) && !anyReverse(opt) &&
      (f2b || tn.variant == 3 || tn.variant == 4)) {
    cudaMemsetAsync(c.smoothed.p, 0, (size_t)n, st);
    fp.smoothed = (uint8_t*)c.smoothed.p;
    fp.smooth_ticket = dTicket + 1;
  }
  {
    // the extrapolation's propagator options: the reference's defaults
    // (KalmanFitter.hpp:960-961 constructs them without the fit's options)
    ck_options d;
    ck_options_default(&d);
    fp.extOpt = toDevOptions(d);
  }
  // inside a stream capture the timing events become event-record nodes of
  // the graph (cudaEventRecordExternal), so they time every replay
  unsigned recFlags = cudaEventRecordDefault;
  if (timed) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive)
      recFlags = cudaEventRecordExternal;
    cudaEventRecordWithFlags(ev0, st, recFlags);
  }
  if (n > 0) {
    e = launchFit(fp, opt.precision, tn, fitGrid, st);
    if (e != cudaSuccess) return cudaFail(e, "fit kernel launch");
    ++launches;
    if (timed) cudaEventRecordWithFlags(evMid, st, recFlags);
    if (anyReverse(opt)) {
      // the reversed pass: the 256-slot compaction kernel, one block per SM,
      // over the same queue (the tracks the reverse-filtering logic selects)
      FitParams rp = fp;
      const long long warps = (long long)h->smCount * (256 / 32);
      rp.lanes_per_warp = (int)std::min<long long>(32, std::max<long long>(1, (n + warps - 1) / warps));
      cudaMemsetAsync(dTicket, 0, sizeof(int32_t), st);
      e = launchReverse(rp, opt.precision, h->smCount, st);
      if (e != cudaSuccess) return cudaFail(e, "reversed filter kernel launch");
      ++launches;
      e = launchReverseOutput(fp, opt.precision, st);
      if (e != cudaSuccess) return cudaFail(e, "reverse filtering output kernel launch");
      ++launches;
    }
    if (!opt.reverse_filtering) {
      e = launchSmooth(fp, opt.precision, st);
      if (e != cudaSuccess) return cudaFail(e, "smoother kernel launch");
      ++launches;
    }
    if (opt.reference_surface >= 0) {
      e = launchExtrapolate(fp, opt.precision, st);
      if (e != cudaSuccess) return cudaFail(e, "extrapolation kernel launch");
      ++launches;
    }
  }
  if (timed) cudaEventRecordWithFlags(ev1, st, recFlags);
  h->lastLaunches = launches;
  h->lastTimed = timed;
  return CK_OK;
}

struct OutArrays {
  void* host[kOutArrays];
  void* dev[kOutArrays];
  size_t bytes[kOutArrays];
  int count = 0;
};

}  // namespace ck

// ------------------------------------------------------------------ C ABI
extern "C" {

void ck_options_default(ck_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->step_tolerance = 1e-4;
  o->step_size_cutoff = 0.0;
  o->initial_step_size = 10000.0;
  o->max_step_size = std::numeric_limits<double>::max();
  o->max_rk_step_trials = 10000;
  o->max_steps = 1000;
  o->max_target_skipping = 100;
  o->loop_protection = 1;
  o->path_limit = std::numeric_limits<double>::max();
  o->loop_fraction = 0.5;
  o->surface_tolerance = 1e-4;
  o->near_limit = -0.1;
  o->multiple_scattering = 1;
  o->energy_loss = 1;
  o->use_joseph = 0;
  o->precision = CK_PRECISION_FP64;
  o->outlier_chi2_cut = std::numeric_limits<double>::infinity();
  o->reverse_filtering = 0;
  o->free_to_bound_correction = 0;
  o->reference_surface = -1;
  o->early_termination = 0;
  o->smoother = CK_SMOOTHER_GAIN_MATRIX;
  o->reference_strategy = CK_EXTRAPOLATE_FIRST_OR_LAST;
  o->reverse_filtering_cov_scaling = 100.0;
  o->reverse_filtering_mom_threshold = 0.0;
}

int32_t ck_api_version(void) { return CK_API_VERSION; }

const char* ck_status_string(ck_status s) {
  switch (s) {
    case CK_OK:
      return "ok";
    case CK_ERR_INVALID_ARGUMENT:
      return "invalid argument";
    case CK_ERR_CUDA:
      return "CUDA error";
    case CK_ERR_NO_DEVICE:
      return "no CUDA device";
    case CK_ERR_OUT_OF_MEMORY:
      return "out of device memory";
    case CK_ERR_UNSUPPORTED:
      return "unsupported feature";
    case CK_ERR_BUDGET:
      return "request exceeds the memory budget";
    case CK_ERR_TIMEOUT:
      return "timeout";
    case CK_ERR_NOT_READY:
      return "not ready";
    case CK_ERR_SCRATCH_LIMIT:
      return "request exceeds the fixed scratch capacity";
  }
  return "unknown status";
}

const char* ck_last_error(void) { return g_lastError.c_str(); }

// sizes of the ABI structs, for binding checks
void ck_abi_struct_sizes(int64_t* out, int32_t n) {
  const int64_t s[] = {(int64_t)sizeof(ck_surface),   (int64_t)sizeof(ck_field),
                       (int64_t)sizeof(ck_options),   (int64_t)sizeof(ck_config),
                       (int64_t)sizeof(ck_batch_in),  (int64_t)sizeof(ck_batch_out),
                       (int64_t)sizeof(ck_server_config), (int64_t)sizeof(ck_propagate_in),
                       (int64_t)sizeof(ck_propagate_out), (int64_t)sizeof(ck_ckf_options),
                       (int64_t)sizeof(ck_ckf_in),        (int64_t)sizeof(ck_ckf_out)};
  for (int i = 0; i < n && i < (int)(sizeof(s) / sizeof(s[0])); ++i) out[i] = s[i];
}

ck_status ck_create(const ck_config* cfg, ck_handle** out) {
  if (!cfg || !out) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return fail(CK_ERR_NO_DEVICE, "no CUDA device visible");
  if (cfg->device < 0 || cfg->device >= ndev) return fail(CK_ERR_INVALID_ARGUMENT, "bad device");
  if (cfg->n_surfaces < 0 || (cfg->n_surfaces > 0 && !cfg->surfaces))
    return fail(CK_ERR_INVALID_ARGUMENT, "bad surface table");
  for (int i = 0; i < cfg->n_surfaces; ++i) {
    const ck_surface& s = cfg->surfaces[i];
    if (s.type != CK_SURFACE_PLANE && s.type != CK_SURFACE_CYLINDER && s.type != CK_SURFACE_LINE)
      return fail(CK_ERR_UNSUPPORTED, "surface " + std::to_string(i) + ": unsupported type");
    if (s.type == CK_SURFACE_CYLINDER && !(s.radius > 0))
      return fail(CK_ERR_INVALID_ARGUMENT, "surface " + std::to_string(i) + ": radius <= 0");
  }
  const ck_field& f = cfg->field;
  if (f.kind != CK_FIELD_CONSTANT && f.kind != CK_FIELD_GRID_XYZ)
    return fail(CK_ERR_UNSUPPORTED, "unsupported field kind");
  if (f.kind == CK_FIELD_GRID_XYZ) {
    for (int i = 0; i < 3; ++i)
      if (f.n[i] < 2 || !(f.max[i] > f.min[i]))
        return fail(CK_ERR_INVALID_ARGUMENT, "bad field grid axes");
    if (!f.values_tesla) return fail(CK_ERR_INVALID_ARGUMENT, "field values missing");
  }
  if ((e = cudaSetDevice(cfg->device)) != cudaSuccess) return cudaFail(e, "cudaSetDevice");
  if ((e = configureFitKernels()) != cudaSuccess) return cudaFail(e, "kernel set-up");
  ck_handle* h = new ck_handle();
  h->device = cfg->device;
  cudaDeviceGetAttribute(&h->smCount, cudaDevAttrMultiProcessorCount, cfg->device);
  if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreate(&h->ev0)) != cudaSuccess ||
      (e = cudaEventCreate(&h->ev1)) != cudaSuccess ||
      (e = cudaEventCreate(&h->evMid)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&h->lastCall, cudaEventDisableTiming)) != cudaSuccess) {
    delete h;
    return cudaFail(e, "stream/event creation");
  }
  h->nSurfaces = cfg->n_surfaces;
  h->hostSurfaces.assign(cfg->surfaces, cfg->surfaces + cfg->n_surfaces);
  std::vector<DevSurface> ds;
  for (int i = 0; i < cfg->n_surfaces; ++i) ds.push_back(toDevSurface(cfg->surfaces[i]));
  if (!ds.empty()) {
    if ((e = cudaMalloc(&h->dSurfaces, ds.size() * sizeof(DevSurface))) != cudaSuccess ||
        (e = cudaMemcpy(h->dSurfaces, ds.data(), ds.size() * sizeof(DevSurface),
                        cudaMemcpyHostToDevice)) != cudaSuccess) {
      ck_destroy(h);
      return cudaFail(e, "surface upload");
    }
  }
  {
    // (cos, sin) of the reference angles k * kTrigStep, evaluated in long
    // double for the angle exactly as the kernels form it in double
    std::vector<double2> tab(kTrigEntries);
    for (int k = -64; k <= 64; ++k) {
      const long double a = (long double)((double)k * kTrigStep);
      tab[k + 64] = make_double2((double)std::cos(a), (double)std::sin(a));
    }
    if ((e = cudaMalloc(&h->dTrig, sizeof(double2) * kTrigEntries)) != cudaSuccess ||
        (e = cudaMemcpy(h->dTrig, tab.data(), sizeof(double2) * kTrigEntries,
                        cudaMemcpyHostToDevice)) != cudaSuccess) {
      ck_destroy(h);
      return cudaFail(e, "table upload");
    }
  }
  std::memset(&h->field, 0, sizeof(h->field));
  h->field.kind = f.kind;
  for (int i = 0; i < 3; ++i) h->field.b[i] = f.constant_tesla[i] * 0.000299792458;
  h->hostField = f;
  if (f.kind == CK_FIELD_GRID_XYZ) {
    size_t nn = (size_t)f.n[0] * f.n[1] * f.n[2];
    std::vector<float4> nodes(nn);
    for (size_t i = 0; i < nn; ++i)
      nodes[i] = make_float4(f.values_tesla[3 * i], f.values_tesla[3 * i + 1],
                             f.values_tesla[3 * i + 2], 0.0f);
    if ((e = cudaMalloc(&h->dNodes, nn * sizeof(float4))) != cudaSuccess ||
        (e = cudaMemcpy(h->dNodes, nodes.data(), nn * sizeof(float4), cudaMemcpyHostToDevice)) !=
            cudaSuccess) {
      ck_destroy(h);
      return cudaFail(e, "field upload");
    }
    for (int i = 0; i < 3; ++i) {
      // fieldMapXYZ axis: n bins over [min, max + step) (Helpers.hpp:289-310)
      h->field.n[i] = f.n[i];
      double xmin = f.min[i], xmax = f.max[i];
      double step = (xmax - xmin) / static_cast<double>(f.n[i] - 1);
      xmax += step;
      h->field.mn[i] = xmin;
      h->field.width[i] = (xmax - xmin) / static_cast<double>(f.n[i]);
      h->field.upper[i] = xmin + static_cast<double>(f.n[i] - 1) * h->field.width[i];
    }
    h->field.nodes = h->dNodes;
  }
  for (int i = 0; i < 3; ++i) {
    h->field.bf[i] = (float)h->field.b[i];
    h->field.mnf[i] = (float)h->field.mn[i];
    h->field.widthf[i] = (float)h->field.width[i];
    h->field.upperf[i] = (float)h->field.upper[i];
  }
  h->mc = makeMatConst();
  h->useGraph = cfg->use_graph;
  h->sortQueue = true;
  if (cfg->autotune_cache) h->cachePath = cfg->autotune_cache;
  for (int p = 0; p < CK_NUM_PRECISIONS; ++p) {
    // default: the block-compaction kernel with 256 slots per block, unless
    // the configuration asks for a thread count
    const bool fixedTpb = cfg->threads_per_block > 0;
    h->tune[p].variant = fixedTpb ? 0 : kDefaultVariant;
    h->tune[p].tpb = fixedTpb ? std::min(cfg->threads_per_block, kFitMaxBlock)
                              : variantBlock(kDefaultVariant);
    h->tune[p].bps = cfg->blocks_per_sm > 0 ? cfg->blocks_per_sm : 0;
    h->tune[p].spr = kDefaultStepsPerRound[p];
    h->tune[p].tuned = 0;
    h->tune[p].staged = kDefaultSmootherStaged;
  }
  loadTuneCache(h);
  for (int p = 0; p < CK_NUM_PRECISIONS; ++p) {
    if (h->tune[p].bps <= 0) {
      // default: as many resident blocks as the register budget allows
      h->tune[p].bps = ck::occupancyBlocks(p, h->tune[p].variant, h->tune[p].tpb);
      if (h->tune[p].bps <= 0) h->tune[p].bps = 1;
    }
  }
  *out = h;
  return CK_OK;
}

ck_status ck_destroy(ck_handle* h) {
  if (!h) return CK_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->graphExec) cudaGraphExecDestroy(h->graphExec);
  for (auto& b : h->inBufs) b.release();
  for (auto& b : h->outBufs) b.release();
  for (auto& set : h->chunkIn)
    for (auto& b : set) b.release();
  for (cudaEvent_t ev : h->inFree)
    if (ev) cudaEventDestroy(ev);
  h->ctx.release();
  h->unitBuf.release();
  if (h->dSurfaces) cudaFree(h->dSurfaces);
  if (h->dTrig) cudaFree(h->dTrig);
  if (h->dNodes) cudaFree(h->dNodes);
  if (h->dGenSurfaces) cudaFree(h->dGenSurfaces);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->evMid) cudaEventDestroy(h->evMid);
  if (h->lastCall) cudaEventDestroy(h->lastCall);
  for (cudaEvent_t ev : h->chunkTiming) cudaEventDestroy(ev);
  for (cudaEvent_t ev : h->chunkSync) cudaEventDestroy(ev);
  if (h->copyIn) cudaStreamDestroy(h->copyIn);
  if (h->copyOut) cudaStreamDestroy(h->copyOut);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return CK_OK;
}

namespace {

// Host batches of at least two chunks are pipelined: the inputs of chunk c+1
// travel on one copy stream while chunk c is fitted on the caller's stream
// and the outputs of chunk c-1 travel back on a second copy stream, so the
// transfers hide behind the kernels. The device inputs alternate between two
// sets from call to call, so that a call's first inputs travel while the
// previous call's last chunk is still being fitted. A chunk is a view of the full device
// input arrays (the CSR offsets are absolute: the chunk shifts only its
// offset and per-track arrays by its first track); its outputs fill their own
// block of the device output buffers (SoA over the chunk's tracks) and reach
// the caller's layout with one 2D copy per array (rows: states x components).
// (a fit launch carries a few ms of work that does not shrink with the batch
// — measured on GB300, barrel tracks, mixed: 8 ms for 125k tracks, 30 ms for
// 1M — so chunks stay large: a 1M-track host batch runs as two)
constexpr int kDefaultChunkTracks = 500000;

int chunkTracksOf(const ck_handle* h) {
  return h->chunkTracks == 0 ? kDefaultChunkTracks : h->chunkTracks;
}

ck_status ensureChunkResources(ck_handle* h, int chunks) {
  cudaError_t e;
  if (!h->copyIn && (e = cudaStreamCreateWithFlags(&h->copyIn, cudaStreamNonBlocking)) != cudaSuccess)
    return cudaFail(e, "copy stream");
  if (!h->copyOut && (e = cudaStreamCreateWithFlags(&h->copyOut, cudaStreamNonBlocking)) != cudaSuccess)
    return cudaFail(e, "copy stream");
  while ((int)h->chunkTiming.size() < 3 * chunks) {
    cudaEvent_t ev;
    if ((e = cudaEventCreate(&ev)) != cudaSuccess) return cudaFail(e, "chunk event");
    h->chunkTiming.push_back(ev);
  }
  while ((int)h->chunkSync.size() < 2 * chunks + 2) {
    cudaEvent_t ev;
    if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess)
      return cudaFail(e, "chunk event");
    h->chunkSync.push_back(ev);
  }
  for (cudaEvent_t& ev : h->inFree)
    if (!ev && (e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess)
      return cudaFail(e, "chunk event");
  return CK_OK;
}

// Chunk boundaries of a host batch: equal chunks, but a shorter last one.
// Every chunk's fit launch pays the same floor (its longest track), so the
// split does not change the kernel time; the copy of the last chunk's
// outputs is the one transfer that no fit hides (the first chunk's inputs
// travel while the previous call's last chunk runs), so the last chunk is
// the small one.
constexpr double kLastChunkWeight = 0.43;

std::vector<int> chunkBounds(int n, int chunks) {
  std::vector<int> b(chunks + 1);
  const double wsum = (chunks - 1) + kLastChunkWeight;
  for (int c = 0; c < chunks; ++c) b[c] = (int)((double)n * c / wsum);
  b[chunks] = n;
  return b;
}

}  // namespace

// The chunked host path (both sides in host memory, n >= 2 chunks); the
// options and arrays are validated by the caller.
static ck_status fitBatchHostChunked(ck_handle* h, const ck_options& opt, const ck_batch_in& in,
                                     const ck_batch_out& out, cudaStream_t st) {
  const int n = in.n_tracks;
  const int chunkTracks = chunkTracksOf(h);
  const int chunks = (n + chunkTracks - 1) / chunkTracks;
  const std::vector<int> bounds = chunkBounds(n, chunks);
  int per = 0;  // the largest chunk
  for (int c = 0; c < chunks; ++c) per = std::max(per, bounds[c + 1] - bounds[c]);
  const int ms = out.max_states;
  const Tune tn = h->tune[opt.precision];
  ck_status s = ensureChunkResources(h, chunks);
  if (s != CK_OK) return s;
  const int set = h->inSet;
  h->inSet ^= 1;
  DevBuf* inBufs = h->chunkIn[set];
  cudaError_t e;
  const int32_t* so = in.seq_offsets;
  const int32_t* mo = in.meas_offsets;
  // ---- device input arrays (full size) and what one track / one CSR entry holds
  struct In {
    const void* src;
    int kind;  // 0 offsets (n + 1), 1 per sequence entry, 2 per measurement, 3 per track
    size_t elem;
    const void** dst;
  } ins[] = {
      {in.seq_offsets, 0, 4, nullptr},       {in.seq_surfaces, 1, 4, nullptr},
      {in.meas_offsets, 0, 4, nullptr},      {in.meas_surfaces, 2, 4, nullptr},
      {in.meas_values, 2, 16, nullptr},      {in.meas_cov, 2, 32, nullptr},
      {in.start_params, 3, 48, nullptr},     {in.start_cov, 3, 288, nullptr},
      {in.start_frames, 3, 96, nullptr},     {in.particle, 3, 8, nullptr},
      {in.particle_pdg, 3, 4, nullptr},      {in.meas_subspace, 2, 4, nullptr},
  };
  static_assert(sizeof(ins) / sizeof(ins[0]) == kInputArrays, "input arrays");
  const size_t nSeq = (size_t)so[n], nMeas = (size_t)mo[n];
  auto total = [&](int kind) -> size_t {
    return kind == 0 ? (size_t)n + 1 : kind == 1 ? nSeq : kind == 2 ? nMeas : (size_t)n;
  };
  for (int i = 0; i < kInputArrays; ++i) {
    if (!ins[i].src) {
      if (i >= 10) continue;
      return fail(CK_ERR_INVALID_ARGUMENT, "input array missing");
    }
    if ((e = inBufs[i].ensure(total(ins[i].kind) * ins[i].elem)) != cudaSuccess)
      return cudaFail(e, "input buffer");
  }
  // ---- device output buffers: per track, per state (rows ms x C) or per
  // track component (rows C)
  const int cc = covComponents(out);
  struct Out {
    void* host;
    int rows;  // copy rows of one track column
    size_t elem;
  } outs[] = {
      {out.status, 1, 4},       {out.n_states, 1, 4},           {out.n_measurements, 1, 4},
      {out.n_holes, 1, 4},      {out.n_outliers, 1, 4},         {out.ndf, 1, 4},
      {out.chi2_sum, 1, 8},     {out.state_surface, ms, 4},     {out.state_flags, ms, 4},
      {out.state_path_length, ms, 8}, {out.state_chi2, ms, 8},  {out.predicted, 6 * ms, 8},
      {out.predicted_cov, cc * ms, 8}, {out.filtered, 6 * ms, 8}, {out.filtered_cov, cc * ms, 8},
      {out.smoothed, 6 * ms, 8}, {out.smoothed_cov, cc * ms, 8}, {out.jacobian, 36 * ms, 8},
      {out.track_params, 6, 8}, {out.track_cov, 36, 8},
  };
  static_assert(sizeof(outs) / sizeof(outs[0]) == kOutArrays, "output arrays");
  for (int i = 0; i < kOutArrays; ++i)
    if (outs[i].host && (e = h->outBufs[i].ensure((size_t)n * outs[i].rows * outs[i].elem)) !=
                            cudaSuccess)
      return cudaFail(e, "output buffer");
  if ((s = preparePipeline(h, h->ctx, per, ms, opt.precision, needsExtStart(opt))) != CK_OK)
    return s;
  cudaEvent_t* sync = h->chunkSync.data();
  cudaEvent_t evStart = sync[2 * chunks], evDone = sync[2 * chunks + 1];
  cudaEventRecord(evStart, st);
  // (the inputs wait only for the kernels of the call before last, which
  // read this input set; the outputs for everything before this call)
  cudaStreamWaitEvent(h->copyIn, h->inFree[set], 0);
  cudaStreamWaitEvent(h->copyOut, evStart, 0);
  size_t h2d = 0, d2h = 0;
  int launches = 0;
  for (int c = 0; c < chunks; ++c) {
    const int t0 = bounds[c], t1 = bounds[c + 1], nc = t1 - t0;
    // inputs of this chunk
    for (int i = 0; i < kInputArrays; ++i) {
      if (!ins[i].src) continue;
      size_t a, b;
      switch (ins[i].kind) {
        case 0: a = t0, b = t1 + 1; break;
        case 1: a = so[t0], b = so[t1]; break;
        case 2: a = mo[t0], b = mo[t1]; break;
        default: a = t0, b = t1; break;
      }
      const size_t bytes = (b - a) * ins[i].elem;
      if (bytes &&
          (e = cudaMemcpyAsync((char*)inBufs[i].p + a * ins[i].elem,
                               (const char*)ins[i].src + a * ins[i].elem, bytes,
                               cudaMemcpyHostToDevice, h->copyIn)) != cudaSuccess)
        return cudaFail(e, "input copy");
      h2d += bytes;
    }
    cudaEventRecord(sync[2 * c], h->copyIn);
    // the chunk's views
    ck_batch_in din = in;
    din.memory = CK_MEM_DEVICE;
    din.n_tracks = nc;
    const void** dins[] = {(const void**)&din.seq_offsets, (const void**)&din.seq_surfaces,
                           (const void**)&din.meas_offsets, (const void**)&din.meas_surfaces,
                           (const void**)&din.meas_values, (const void**)&din.meas_cov,
                           (const void**)&din.start_params, (const void**)&din.start_cov,
                           (const void**)&din.start_frames, (const void**)&din.particle,
                           (const void**)&din.particle_pdg, (const void**)&din.meas_subspace};
    for (int i = 0; i < kInputArrays; ++i) {
      if (!ins[i].src) {
        *dins[i] = nullptr;
        continue;
      }
      const size_t shift = (ins[i].kind == 0 || ins[i].kind == 3) ? (size_t)t0 * ins[i].elem : 0;
      *dins[i] = (const char*)inBufs[i].p + shift;
    }
    ck_batch_out dout = out;
    dout.memory = CK_MEM_DEVICE;
    void** douts[] = {(void**)&dout.status, (void**)&dout.n_states, (void**)&dout.n_measurements,
                      (void**)&dout.n_holes, (void**)&dout.n_outliers, (void**)&dout.ndf,
                      (void**)&dout.chi2_sum, (void**)&dout.state_surface,
                      (void**)&dout.state_flags, (void**)&dout.state_path_length,
                      (void**)&dout.state_chi2, (void**)&dout.predicted,
                      (void**)&dout.predicted_cov, (void**)&dout.filtered,
                      (void**)&dout.filtered_cov, (void**)&dout.smoothed,
                      (void**)&dout.smoothed_cov, (void**)&dout.jacobian,
                      (void**)&dout.track_params, (void**)&dout.track_cov};
    for (int i = 0; i < kOutArrays; ++i)
      if (outs[i].host)
        *douts[i] = (char*)h->outBufs[i].p + (size_t)t0 * outs[i].rows * outs[i].elem;
    // the fit of this chunk, timed with its own events
    cudaStreamWaitEvent(st, sync[2 * c], 0);
    s = enqueuePipeline(h, h->ctx, opt, din, dout, tn, st, true, gridBlocksFor(h, tn),
                        h->chunkTiming.data() + 3 * c);
    if (s != CK_OK) return s;
    launches += h->lastLaunches;
    cudaEventRecord(sync[2 * c + 1], st);
    // its outputs, into the caller's layout
    cudaStreamWaitEvent(h->copyOut, sync[2 * c + 1], 0);
    for (int i = 0; i < kOutArrays; ++i) {
      if (!outs[i].host) continue;
      const size_t w = (size_t)nc * outs[i].elem;
      char* dst = (char*)outs[i].host + (size_t)t0 * outs[i].elem;
      const char* src = (const char*)*douts[i];
      if ((e = cudaMemcpy2DAsync(dst, (size_t)n * outs[i].elem, src, w, w, outs[i].rows,
                                 cudaMemcpyDeviceToHost, h->copyOut)) != cudaSuccess)
        return cudaFail(e, "output copy");
      d2h += w * outs[i].rows;
    }
  }
  // this input set is free once the last chunk's kernels have run
  cudaEventRecord(h->inFree[set], st);
  cudaEventRecord(evDone, h->copyOut);
  cudaStreamWaitEvent(st, evDone, 0);
  h->lastLaunches = launches;
  h->lastChunks = chunks;
  h->lastTimed = true;
  h->lastH2D = h2d;
  h->lastD2H = d2h;
  if ((e = cudaGetLastError()) != cudaSuccess) return cudaFail(e, "batch pipeline");
  return CK_OK;
}

ck_status ck_fit_batch(ck_handle* h, const ck_options* opt, const ck_batch_in* in,
                       ck_batch_out* out, void* stream) {
  if (!h || !in || !out) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  ck_status vs = validateOptions(opt);
  if (vs != CK_OK) return vs;
  if ((vs = validateReference(h, opt)) != CK_OK) return vs;
  if (in->n_tracks < 0) return fail(CK_ERR_INVALID_ARGUMENT, "n_tracks < 0");
  if (out->max_states <= 0) return fail(CK_ERR_INVALID_ARGUMENT, "max_states <= 0");
  if (!out->status) return fail(CK_ERR_INVALID_ARGUMENT, "status array is required");
  const bool needsCov[4] = {out->predicted != nullptr, out->filtered != nullptr,
                            out->smoothed != nullptr, false};
  if ((needsCov[0] && !out->predicted_cov) || (needsCov[1] && !out->filtered_cov) ||
      (needsCov[2] && !out->smoothed_cov))
    return fail(CK_ERR_INVALID_ARGUMENT, "parameter arrays need their covariance arrays");
  std::lock_guard<std::mutex> lock(h->mu);
  cudaSetDevice(h->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
  const int n = in->n_tracks;
  const Tune tn = h->tune[opt->precision];
  cudaError_t e;
  // calls of one handle run on the device in call order, whatever their
  // streams: they share the staging buffers and the scratch
  if (h->lastCallStream && h->lastCallStream != st) cudaStreamWaitEvent(st, h->lastCall, 0);
  auto done = [&](ck_status s) {
    if (s == CK_OK) {
      cudaEventRecord(h->lastCall, st);
      h->lastCallStream = st;
    }
    return s;
  };

  // ---- inputs
  ck_batch_in din = *in;
  if (in->memory == CK_MEM_HOST && n > 0) {
    if (!in->seq_offsets || !in->meas_offsets)
      return fail(CK_ERR_INVALID_ARGUMENT, "offsets missing");
    // (the kernels read the CSR rows [off[t], off[t + 1]) of the copied
    // arrays, and chunk boundaries cut them: the offsets must be a
    // non-decreasing partition)
    if (in->seq_offsets[0] < 0 || in->meas_offsets[0] < 0)
      return fail(CK_ERR_INVALID_ARGUMENT, "negative CSR offset");
    for (int t = 0; t < n; ++t)
      if (in->seq_offsets[t + 1] < in->seq_offsets[t] || in->meas_offsets[t + 1] < in->meas_offsets[t])
        return fail(CK_ERR_INVALID_ARGUMENT, "decreasing CSR offsets");
    const int nSeq = in->seq_offsets[n], nMeas = in->meas_offsets[n];
    if (out->memory == CK_MEM_HOST && chunkTracksOf(h) > 0 && n >= 2 * chunkTracksOf(h))
      return done(fitBatchHostChunked(h, *opt, *in, *out, st));
    struct Item {
      const void* src;
      size_t bytes;
      const void** dst;
    } items[] = {
        {in->seq_offsets, sizeof(int32_t) * (n + 1), (const void**)&din.seq_offsets},
        {in->seq_surfaces, sizeof(int32_t) * nSeq, (const void**)&din.seq_surfaces},
        {in->meas_offsets, sizeof(int32_t) * (n + 1), (const void**)&din.meas_offsets},
        {in->meas_surfaces, sizeof(int32_t) * nMeas, (const void**)&din.meas_surfaces},
        {in->meas_values, sizeof(double) * 2 * nMeas, (const void**)&din.meas_values},
        {in->meas_cov, sizeof(double) * 4 * nMeas, (const void**)&din.meas_cov},
        {in->start_params, sizeof(double) * 6 * n, (const void**)&din.start_params},
        {in->start_cov, sizeof(double) * 36 * n, (const void**)&din.start_cov},
        {in->start_frames, sizeof(double) * 12 * n, (const void**)&din.start_frames},
        {in->particle, sizeof(float) * 2 * n, (const void**)&din.particle},
        {in->particle_pdg, sizeof(int32_t) * n, (const void**)&din.particle_pdg},
        {in->meas_subspace, sizeof(int32_t) * nMeas, (const void**)&din.meas_subspace},
    };
    size_t h2d = 0;
    for (int i = 0; i < kInputArrays; ++i) {
      if (!items[i].src) {
        if (i >= 10) {  // optional arrays
          *items[i].dst = nullptr;
          continue;
        }
        return fail(CK_ERR_INVALID_ARGUMENT, "input array missing");
      }
      if ((e = h->inBufs[i].ensure(items[i].bytes)) != cudaSuccess)
        return cudaFail(e, "input buffer");
      if (items[i].bytes &&
          (e = cudaMemcpyAsync(h->inBufs[i].p, items[i].src, items[i].bytes,
                               cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cudaFail(e, "input copy");
      *items[i].dst = h->inBufs[i].p;
      h2d += items[i].bytes;
    }
    din.memory = CK_MEM_DEVICE;
    h->lastH2D = h2d;
  } else {
    h->lastH2D = 0;
  }

  // ---- outputs
  ck_batch_out dout = *out;
  OutArrays oa;
  if (out->memory == CK_MEM_HOST && n > 0) {
    const int ms = out->max_states;
    struct Item {
      void** field;
      size_t bytes;
    } items[] = {
        {(void**)&dout.status, sizeof(int32_t) * n},
        {(void**)&dout.n_states, sizeof(int32_t) * n},
        {(void**)&dout.n_measurements, sizeof(int32_t) * n},
        {(void**)&dout.n_holes, sizeof(int32_t) * n},
        {(void**)&dout.n_outliers, sizeof(int32_t) * n},
        {(void**)&dout.ndf, sizeof(int32_t) * n},
        {(void**)&dout.chi2_sum, sizeof(double) * n},
        {(void**)&dout.state_surface, compBytes(n, ms, 1, 4)},
        {(void**)&dout.state_flags, compBytes(n, ms, 1, 4)},
        {(void**)&dout.state_path_length, compBytes(n, ms, 1, 8)},
        {(void**)&dout.state_chi2, compBytes(n, ms, 1, 8)},
        {(void**)&dout.predicted, compBytes(n, ms, 6, 8)},
        {(void**)&dout.predicted_cov, compBytes(n, ms, covComponents(*out), 8)},
        {(void**)&dout.filtered, compBytes(n, ms, 6, 8)},
        {(void**)&dout.filtered_cov, compBytes(n, ms, covComponents(*out), 8)},
        {(void**)&dout.smoothed, compBytes(n, ms, 6, 8)},
        {(void**)&dout.smoothed_cov, compBytes(n, ms, covComponents(*out), 8)},
        {(void**)&dout.jacobian, compBytes(n, ms, 36, 8)},
        {(void**)&dout.track_params, sizeof(double) * 6 * (size_t)n},
        {(void**)&dout.track_cov, sizeof(double) * 36 * (size_t)n},
    };
    for (int i = 0; i < kOutArrays; ++i) {
      void* hostPtr = *items[i].field;
      if (!hostPtr) continue;
      if ((e = h->outBufs[i].ensure(items[i].bytes)) != cudaSuccess)
        return cudaFail(e, "output buffer");
      *items[i].field = h->outBufs[i].p;
      oa.host[oa.count] = hostPtr;
      oa.dev[oa.count] = h->outBufs[i].p;
      oa.bytes[oa.count] = items[i].bytes;
      ++oa.count;
    }
    dout.memory = CK_MEM_DEVICE;
  }

  // ---- pipeline (graph-captured for device-resident batches)
  const int gridBlocks = gridBlocksFor(h, tn);
  ck_status s = preparePipeline(h, h->ctx, n, out->max_states, opt->precision,
                                needsExtStart(*opt));
  if (s != CK_OK) return s;
  const bool deviceOnly = in->memory == CK_MEM_DEVICE && out->memory == CK_MEM_DEVICE;
  if (deviceOnly && h->useGraph && n > 0) {
    GraphKey key;
    key.in = *in;
    key.out = *out;
    key.opt = *opt;
    key.tune = tn;
    key.stream = st;
    key.scratch[0] = h->ctx.rec.p;
    key.scratch[1] = h->ctx.sortCounts.p;
    key.scratch[2] = h->ctx.ext.p;
    key.scratch[3] = h->ctx.perm.p;
    key.scratch[4] = h->ctx.ticket.p;
    key.scratch[5] = h->ctx.tip.p;
    key.scratch[6] = h->ctx.smoothed.p;
    key.sort = h->sortQueue;
    key.tailSmoothing = h->tailSmoothing;
    if (!h->graphExec || std::memcmp(&key, &h->graphKey, sizeof(key)) != 0) {
      if (h->graphExec) {
        cudaGraphExecDestroy(h->graphExec);
        h->graphExec = nullptr;
      }
      cudaGraph_t g;
      if ((e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return cudaFail(e, "graph capture begin");
      s = enqueuePipeline(h, h->ctx, *opt, din, dout, tn, st, true, gridBlocks);
      e = cudaStreamEndCapture(st, &g);
      if (s != CK_OK) return s;
      if (e != cudaSuccess) return cudaFail(e, "graph capture end");
      e = cudaGraphInstantiate(&h->graphExec, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return cudaFail(e, "graph instantiate");
      h->graphKey = key;
      h->graphLaunches = h->lastLaunches;
    }
    if ((e = cudaGraphLaunch(h->graphExec, st)) != cudaSuccess) return cudaFail(e, "graph launch");
    h->lastLaunches = h->graphLaunches;
    h->lastTimed = true;
  } else {
    s = enqueuePipeline(h, h->ctx, *opt, din, dout, tn, st, true, gridBlocks);
    if (s != CK_OK) return s;
  }
  size_t d2h = 0;
  for (int i = 0; i < oa.count; ++i) {
    if ((e = cudaMemcpyAsync(oa.host[i], oa.dev[i], oa.bytes[i], cudaMemcpyDeviceToHost, st)) !=
        cudaSuccess)
      return cudaFail(e, "output copy");
    d2h += oa.bytes[i];
  }
  h->lastD2H = d2h;
  if ((e = cudaGetLastError()) != cudaSuccess) return cudaFail(e, "batch pipeline");
  return done(CK_OK);
}

ck_status ck_sync(ck_handle* h) {
  if (!h) return fail(CK_ERR_INVALID_ARGUMENT, "NULL handle");
  cudaSetDevice(h->device);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cudaFail(e, "stream synchronize");
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cudaFail(e, "device synchronize");
  return CK_OK;
}

ck_status ck_last_kernel_ms(ck_handle* h, double* ms) {
  if (!h || !ms) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!h->lastTimed) return fail(CK_ERR_NOT_READY, "no timed batch");
  cudaSetDevice(h->device);
  if (h->lastChunks > 0) {
    double a = 0, b = 0;
    ck_status s = ck_last_kernel_split_ms(h, &a, &b);
    *ms = a + b;
    return s;
  }
  cudaError_t e = cudaEventSynchronize(h->ev1);
  if (e != cudaSuccess) return cudaFail(e, "event synchronize");
  float f = 0;
  e = cudaEventElapsedTime(&f, h->ev0, h->ev1);
  if (e != cudaSuccess) return cudaFail(e, "event elapsed");
  *ms = f;
  return CK_OK;
}

ck_status ck_last_kernel_split_ms(ck_handle* h, double* filter_ms, double* smoother_ms) {
  if (!h || !filter_ms || !smoother_ms) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!h->lastTimed) return fail(CK_ERR_NOT_READY, "no timed batch");
  cudaSetDevice(h->device);
  if (h->lastChunks > 0) {
    // a chunked host batch: the sum over its chunks
    double fa = 0, fb = 0;
    for (int c = 0; c < h->lastChunks; ++c) {
      float a = 0, b = 0;
      cudaError_t e = cudaEventSynchronize(h->chunkTiming[3 * c + 2]);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&a, h->chunkTiming[3 * c], h->chunkTiming[3 * c + 1]);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&b, h->chunkTiming[3 * c + 1], h->chunkTiming[3 * c + 2]);
      if (e != cudaSuccess) return cudaFail(e, "event elapsed");
      fa += a;
      fb += b;
    }
    *filter_ms = fa;
    *smoother_ms = fb;
    return CK_OK;
  }
  cudaError_t e = cudaEventSynchronize(h->ev1);
  if (e != cudaSuccess) return cudaFail(e, "event synchronize");
  float a = 0, b = 0;
  if ((e = cudaEventElapsedTime(&a, h->ev0, h->evMid)) != cudaSuccess ||
      (e = cudaEventElapsedTime(&b, h->evMid, h->ev1)) != cudaSuccess)
    return cudaFail(e, "event elapsed");
  *filter_ms = a;
  *smoother_ms = b;
  return CK_OK;
}

ck_status ck_last_launch_count(ck_handle* h, int32_t* n) {
  if (!h || !n) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  *n = h->lastLaunches;
  return CK_OK;
}

ck_status ck_last_transfer_bytes(ck_handle* h, int64_t* h2d, int64_t* d2h) {
  if (!h || !h2d || !d2h) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  *h2d = (int64_t)h->lastH2D;
  *d2h = (int64_t)h->lastD2H;
  return CK_OK;
}

ck_status ck_get_launch_config(ck_handle* h, int32_t precision, int32_t* tpb, int32_t* bps) {
  if (!h || !tpb || !bps || precision < 0 || precision >= CK_NUM_PRECISIONS)
    return fail(CK_ERR_INVALID_ARGUMENT, "bad argument");
  *tpb = h->tune[precision].tpb;
  *bps = h->tune[precision].bps;
  return CK_OK;
}

ck_status ck_get_launch_variant(ck_handle* h, int32_t precision, int32_t* variant,
                                int32_t* steps_per_round) {
  if (!h || !variant || !steps_per_round || precision < 0 || precision >= CK_NUM_PRECISIONS)
    return fail(CK_ERR_INVALID_ARGUMENT, "bad argument");
  *variant = h->tune[precision].variant;
  *steps_per_round = h->tune[precision].spr;
  return CK_OK;
}

ck_status ck_set_launch_config(ck_handle* h, int32_t precision, int32_t variant, int32_t tpb,
                               int32_t bps) {
  if (!h || precision < 0 || precision >= CK_NUM_PRECISIONS || !validLaunch(variant, tpb) ||
      bps <= 0)
    return fail(CK_ERR_INVALID_ARGUMENT, "bad launch configuration");
  std::lock_guard<std::mutex> lock(h->mu);
  int maxB = occupancyBlocks(precision, variant, tpb);
  if (bps > maxB) return fail(CK_ERR_INVALID_ARGUMENT, "more blocks per SM than fit");
  h->tune[precision] = {variant, tpb, bps, h->tune[precision].spr, 1, h->tune[precision].grid,
                        h->tune[precision].staged};
  return CK_OK;
}

ck_status ck_set_smoother_staging(ck_handle* h, int32_t precision, int32_t enable) {
  if (!h || precision < 0 || precision >= CK_NUM_PRECISIONS)
    return fail(CK_ERR_INVALID_ARGUMENT, "bad precision");
  std::lock_guard<std::mutex> lock(h->mu);
  h->tune[precision].staged = enable ? 1 : 0;
  return CK_OK;
}

ck_status ck_set_grid_blocks(ck_handle* h, int32_t precision, int32_t blocks) {
  if (!h || precision < 0 || precision >= CK_NUM_PRECISIONS || blocks < 0)
    return fail(CK_ERR_INVALID_ARGUMENT, "bad precision, or negative block count");
  std::lock_guard<std::mutex> lock(h->mu);
  h->tune[precision].grid = blocks;
  return CK_OK;
}

ck_status ck_set_host_chunk_tracks(ck_handle* h, int32_t tracks) {
  if (!h) return fail(CK_ERR_INVALID_ARGUMENT, "NULL handle");
  std::lock_guard<std::mutex> lock(h->mu);
  h->chunkTracks = tracks;
  return CK_OK;
}

ck_status ck_set_steps_per_round(ck_handle* h, int32_t precision, int32_t steps) {
  if (!h || precision < 0 || precision >= CK_NUM_PRECISIONS || steps < 1 || steps > 64)
    return fail(CK_ERR_INVALID_ARGUMENT, "bad precision, or steps per round outside [1, 64]");
  std::lock_guard<std::mutex> lock(h->mu);
  h->tune[precision].spr = steps;
  if (h->graphExec) {
    cudaGraphExecDestroy(h->graphExec);
    h->graphExec = nullptr;
  }
  return CK_OK;
}

ck_status ck_set_tail_smoothing(ck_handle* h, int32_t enable) {
  if (!h) return fail(CK_ERR_INVALID_ARGUMENT, "NULL handle");
  std::lock_guard<std::mutex> lock(h->mu);
  h->tailSmoothing = enable != 0;
  return CK_OK;
}

ck_status ck_sort_queue(ck_handle* h, int32_t enable) {
  if (!h) return fail(CK_ERR_INVALID_ARGUMENT, "NULL handle");
  std::lock_guard<std::mutex> lock(h->mu);
  h->sortQueue = enable != 0;
  if (h->graphExec) {
    cudaGraphExecDestroy(h->graphExec);
    h->graphExec = nullptr;
  }
  return CK_OK;
}

ck_status ck_autotune(ck_handle* h, const ck_options* opt, const ck_batch_in* in,
                      ck_batch_out* out) {
  if (!h || !in || !out) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  ck_status vs = validateOptions(opt);
  if (vs != CK_OK) return vs;
  if ((vs = validateReference(h, opt)) != CK_OK) return vs;
  if (in->memory != CK_MEM_DEVICE || out->memory != CK_MEM_DEVICE)
    return fail(CK_ERR_INVALID_ARGUMENT, "autotuning needs a device-resident batch");
  const int p = opt->precision;
  Tune best = h->tune[p];
  double bestMs = 1e30;
  std::string log;
  // candidates: every variant and block size, resident blocks per SM at the
  // maximum, 3/4 and 1/2 of it; the compaction variants at the maximum with
  // 1-4 Runge-Kutta trials per round
  std::vector<Tune> cands;
  for (int v = 0; v < kNumFitVariants; ++v)
    for (int tpb : {32, 64, 128, 256}) {
      if (!validLaunch(v, tpb)) continue;
      const int maxB = occupancyBlocks(p, v, tpb);
      if (maxB <= 0) continue;
      const int stg = h->tune[p].staged;
      if (variantBlock(v)) {
        for (int spr = 1; spr <= 4; ++spr) cands.push_back({v, tpb, maxB, spr, 1, 0, stg});
      } else {
        const int bs[3] = {maxB, std::max(1, (maxB * 3) / 4), std::max(1, maxB / 2)};
        for (int i = 0; i < 3; ++i)
          if (i == 0 || bs[i] != bs[i - 1]) cands.push_back({v, tpb, bs[i], 1, 1, 0, stg});
      }
    }
  // the best launch shape, then the same with the other smoother kernel
  // (gain-matrix smoother only)
  const size_t nShapes = cands.size();
  for (size_t ci = 0; ci <= nShapes; ++ci) {
    Tune cand;
    if (ci < nShapes) {
      cand = cands[ci];
    } else {
      if (opt->smoother != CK_SMOOTHER_GAIN_MATRIX || bestMs >= 1e30) break;
      cand = best;
      cand.staged = 1 - best.staged;
    }
    {
      std::lock_guard<std::mutex> lock(h->mu);
      h->tune[p] = cand;
    }
    double tot = 0;
    for (int rep = 0; rep < 3; ++rep) {
      ck_status s = ck_fit_batch(h, opt, in, out, nullptr);
      if (s != CK_OK) return s;
      double ms = 0;
      if ((s = ck_last_kernel_ms(h, &ms)) != CK_OK) return s;
      if (rep > 0) tot += ms;
    }
    const double ms = tot / 2;
    char buf[128];
    std::snprintf(buf, sizeof(buf), "v%d tpb%d bps%d spr%d stg%d %.3fms; ", cand.variant,
                  cand.tpb, cand.bps, cand.spr, cand.staged, ms);
    log += buf;
    if (ms < bestMs) {
      bestMs = ms;
      best = cand;
    }
  }
  {
    std::lock_guard<std::mutex> lock(h->mu);
    h->tune[p] = best;
    h->tuneLog = log;
  }
  saveTuneCache(h);
  return CK_OK;
}

const char* ck_autotune_log(ck_handle* h) { return h ? h->tuneLog.c_str() : ""; }

}  // extern "C"
