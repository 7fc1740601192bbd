// ck_api_internal.h — the handle behind the C ABI (private).
#pragma once

#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "ck_internal.h"
#include "cudakalman.h"

namespace ck {

// Grow-only device allocation.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes);
  void release();
};

// Launch shape of the fit kernel for one precision.
struct Tune {
  int variant;  // kernel variant (ck_launch.h)
  int tpb;      // threads per block
  int bps;      // resident blocks per SM (grid = SMs * bps)
  int spr;      // Runge-Kutta trials per round (compaction variants)
  int tuned;
  int grid;     // blocks of the fit kernel's grid; 0: SMs * bps
  int staged;   // smoother with warp-cooperative record staging
};

// Identity of a captured batch pipeline.
struct GraphKey {
  ck_batch_in in;
  ck_batch_out out;
  ck_options opt;
  Tune tune;
  cudaStream_t stream;
  void* scratch[7];
  bool sort;
  bool tailSmoothing;
  GraphKey() { std::memset(this, 0, sizeof(*this)); }
};

int occupancyBlocks(int precision, int variant, int tpb);

// Scratch of one batch pipeline in flight: records of the resident lanes,
// the ordered work queue and its ticket. A handle owns one; the serving loop
// owns one per stream.
struct FitContext {
  DevBuf rec, perm, ticket, tip, sortCounts;
  DevBuf ext;       // extrapolation start states (reference surface set)
  DevBuf smoothed;  // per queue position: smoothed in the forward filter's tail
  void release() {
    smoothed.release();
    ext.release();
    sortCounts.release();
    tip.release();
    rec.release();
    perm.release();
    ticket.release();
  }
};

extern thread_local std::string g_lastError;
ck_status fail(ck_status s, const std::string& msg);
ck_status cudaFail(cudaError_t e, const char* what);
ck_status validateOptions(const ck_options* o);
// the reference surface of the options against the handle's table (a line
// surface) and the strategy
ck_status validateReference(const ck_handle* h, const ck_options* o);
// the extrapolation start slots are needed for the extrapolation to the
// reference surface and for reverse filtering
inline bool anyReverse(const ck_options& o) {
  return o.reverse_filtering != 0 || o.reverse_filtering_mom_threshold > 0.0;
}
inline bool needsExtStart(const ck_options& o) { return o.reference_surface >= 0 || anyReverse(o); }
DevOptions toDevOptions(const ck_options& o);
// components per state of the covariance arrays of a ck_batch_out (21 packed,
// 36 full)
inline int covComponents(const ck_batch_out& o) {
  return (o.components & CK_OUT_PACKED_COV) ? 21 : 36;
}
MatConst makeMatConst();
DevSurface toDevSurface(const ck_surface& s);
size_t recordStateBytes(int precision);
// the work-queue sort: blocks of kSortBlock tracks, 64 length bins each
// arrays of ck_batch_in staged for host batches (particle_pdg and
// meas_subspace optional)
constexpr int kInputArrays = 12;
// arrays of ck_batch_out (status ... jacobian, track_params, track_cov)
constexpr int kOutArrays = 20;
constexpr int kSortBlock = 1024;
inline int sortBlocks(int n) { return n > 0 ? (n + kSortBlock - 1) / kSortBlock : 1; }
inline size_t sortCountsBytes(int n) { return sizeof(int32_t) * 64 * (size_t)sortBlocks(n); }
size_t recordBytesPerTrack(int maxStates, int precision);
ck_status preparePipeline(ck_handle* h, FitContext& c, int n, int maxStates, int precision,
                          bool extrapolate);
// `timing`: the (start, filter end, end) events a timed pipeline records;
// null: the handle's own
ck_status enqueuePipeline(ck_handle* h, FitContext& c, const ck_options& opt,
                          const ck_batch_in& din, const ck_batch_out& dout, const Tune& tn,
                          cudaStream_t st, bool timed, int gridBlocks,
                          const cudaEvent_t* timing = nullptr);
int gridBlocksFor(ck_handle* h, const Tune& tn);

}  // namespace ck

struct ck_handle {
  int device = 0;
  int smCount = 1;
  int lastCkfLanes = 0;  // lanes per seed of the last ck_find_tracks launch
  void* dGenSurfaces = nullptr;  // the surface table as ck_surface (ck_simulate)
  bool ckfSortSmemSet = false;   // the candidate sort kernel's shared-memory attribute
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evMid = nullptr;
  ck::DevSurface* dSurfaces = nullptr;
  double2* dTrig = nullptr;
  int nSurfaces = 0;
  std::vector<ck_surface> hostSurfaces;
  ck_field hostField{};
  ck::DevField field{};
  float4* dNodes = nullptr;
  ck::MatConst mc{};
  ck::Tune tune[CK_NUM_PRECISIONS]{};
  std::string cachePath;
  std::string tuneLog;
  int useGraph = 1;
  bool sortQueue = true;
  // smoothing in the compaction kernels' tail (ck_set_tail_smoothing)
  bool tailSmoothing = true;
  ck::DevBuf inBufs[ck::kInputArrays];
  ck::DevBuf outBufs[ck::kOutArrays];
  ck::FitContext ctx;
  ck::DevBuf unitBuf;
  int lastLaunches = 0;
  bool lastTimed = false;
  size_t lastH2D = 0, lastD2H = 0;
  cudaGraphExec_t graphExec = nullptr;
  ck::GraphKey graphKey;
  int graphLaunches = 0;
  // chunked host batches: the copy streams, one (ev0, evMid, ev1) timing
  // triplet per chunk of the last call, and the ordering events
  cudaStream_t copyIn = nullptr, copyOut = nullptr;
  std::vector<cudaEvent_t> chunkTiming;  // 3 per chunk
  std::vector<cudaEvent_t> chunkSync;    // 2 per chunk + 2
  int lastChunks = 0;
  // their device inputs, two sets used by turns: a call's inputs travel
  // while the previous call's last chunks are fitted; inFree[s] is recorded
  // after the last kernel that reads set s
  ck::DevBuf chunkIn[2][ck::kInputArrays];
  cudaEvent_t inFree[2] = {nullptr, nullptr};
  int inSet = 0;
  // the end of the last ck_fit_batch on the device, and its stream: a call
  // on another stream waits for it (calls share the staging buffers and the
  // scratch)
  cudaEvent_t lastCall = nullptr;
  cudaStream_t lastCallStream = nullptr;
  int chunkTracks = 0;  // 0: kDefaultChunkTracks; < 0: never chunk
  std::mutex mu;
};
