// ck_server.cu — continuous-batching serving loop of the fitter.
//
// Events arrive through ck_server_submit from any host thread, each with its
// own input arrays (ck_batch_in) and result arrays (ck_batch_out), both
// owned by the caller and in host (pageable or page-locked) or device
// memory. Nothing is copied at submission. One request thread runs the loop:
//   * admission: while a stream slot is free, the pending events (oldest
//     first) that fit the slot's capacity are taken together into one
//     co-batch — events of different sizes share one launch;
//   * launch: each event's inputs are copied straight from the caller's
//     arrays into the slot's device buffers (its CSR offsets shifted on the
//     device), the co-batch is fitted on the slot's stream on a share of
//     the GPU (by default the SMs divided by n_streams - 1: a co-batch
//     admitted while others run starts on free SMs at once; the fit of one
//     event is bound by the serial chain of its tracks, not by the SM count,
//     so a share costs it little) with more Runge-Kutta trials per
//     scheduling round than offline batches use; each event's results are
//     copied from the co-batch's
//     SoA arrays into the caller's arrays with one strided copy per array
//     (pageable host results go through the slot's page-locked buffer);
//   * completion: finished slots are found with CUDA events; an event's
//     latency is its submit-to-results wall time.
// Device memory: every slot holds input, output and record buffers for its
// capacity; the capacity is the largest track count for which all slots fit
// the memory budget. An event larger than a slot is rejected with
// CK_ERR_BUDGET at submission. Track state stays on the device from the
// input copy to the result copy.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "ck_api_internal.h"
#include "ck_launch.h"

using namespace ck;

namespace {

using Clock = std::chrono::steady_clock;

constexpr int kMaxEventsPerBatch = 1024;
constexpr int kPlannedSurfacesPerTrack = 20;
// Runge-Kutta trials per scheduling round of the co-batches: measured best
// for the latency of 10k-track uneven events (filter 2.7 ms at 6 against
// 3.1 ms at 3, mixed form)
constexpr int kServerStepsPerRound = 6;

struct Event {
  int64_t id = 0;
  int n = 0;
  int nSeq = 0, nMeas = 0;
  ck_batch_in in{};
  ck_batch_out out{};
  bool staged = false;  // pageable host results: through the slot's pinned buffer
  ck_status status = CK_OK;
  Clock::time_point submitted;
  double latencyMs = 0;
};

// Output components computed by the server.
struct OutSpec {
  bool sm, fi, pr, jac;
  bool packed;  // CK_OUT_PACKED_COV: covariance arrays of 21 components
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  FitContext ctx;
  DevBuf din[kInputArrays];
  size_t inPlanned[kInputArrays] = {};
  DevBuf dout[kOutArrays];
  DevBuf table;              // per-event {t0, m, seqBase, measBase} on the device
  int32_t* pinTable = nullptr;
  void* pinOut = nullptr;    // staging of pageable results
  size_t pinOutBytes = 0;
  std::vector<std::unique_ptr<Event>> events;
  int nTracks = 0, nSeq = 0, nMeas = 0;
  bool busy = false;
  bool harvesting = false;  // done on the GPU; the delivery thread copies its results
};

// element size and components per ck_batch_out array, in the order of
// outFields()
constexpr size_t kOutElem[kOutArrays] = {4, 4, 4, 4, 4, 4, 8, 4, 4, 8,
                                         8, 8, 8, 8, 8, 8, 8, 8, 8, 8};
constexpr int kOutComp[kOutArrays] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1,
                                      1, 6, 36, 6, 36, 6, 36, 36, 6, 36};
constexpr bool kPerState[kOutArrays] = {false, false, false, false, false, false, false,
                                        true,  true,  true,  true,  true,  true,  true,
                                        true,  true,  true,  true,  false, false};

void outFields(ck_batch_out& o, void** f[kOutArrays]) {
  void** a[kOutArrays] = {(void**)&o.status,          (void**)&o.n_states,
                  (void**)&o.n_measurements,  (void**)&o.n_holes,
                  (void**)&o.n_outliers,      (void**)&o.ndf,
                  (void**)&o.chi2_sum,        (void**)&o.state_surface,
                  (void**)&o.state_flags,     (void**)&o.state_path_length,
                  (void**)&o.state_chi2,      (void**)&o.predicted,
                  (void**)&o.predicted_cov,   (void**)&o.filtered,
                  (void**)&o.filtered_cov,    (void**)&o.smoothed,
                  (void**)&o.smoothed_cov,    (void**)&o.jacobian,
                  (void**)&o.track_params,    (void**)&o.track_cov};
  for (int i = 0; i < kOutArrays; ++i) f[i] = a[i];
}

// CSR offsets of a co-batch: each event's offsets were copied unshifted to
// [t0, t0 + m) (the last event's also to n); add the event's bases.
__global__ void shiftOffsets(int32_t* __restrict__ seqOff, int32_t* __restrict__ measOff,
                             const int4* __restrict__ table, int nEvents) {
  const int e = blockIdx.y;
  const int4 ev = table[e];
  const int count = ev.y + (e == nEvents - 1 ? 1 : 0);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    seqOff[ev.x + i] += ev.z;
    measOff[ev.x + i] += ev.w;
  }
}

__global__ void fillInt(int32_t* __restrict__ p, int n, int32_t v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

}  // namespace

struct ck_server {
  ck_handle* h = nullptr;
  ck_options opt{};
  ck_server_config cfg{};
  OutSpec spec{};
  int capacity = 0;  // tracks per slot
  int gridBlocks = 1;
  Tune tune{};
  std::vector<std::unique_ptr<Slot>> slots;
  std::mutex mu;
  std::condition_variable cvWork, cvDone;
  std::deque<std::unique_ptr<Event>> pending;
  std::deque<std::unique_ptr<Event>> finished;
  std::thread worker;
  // delivery of pageable host results: the slots whose staged results the
  // delivery thread de-strides (with helper threads), off the request loop
  std::thread delivery;
  std::deque<Slot*> toHarvest;
  std::condition_variable cvHarvest;
  int copyThreads = 1;
  bool stop = false;
  ck_status error = CK_OK;
  std::string errorMsg;
  int64_t submitted = 0, completed = 0, tracksDone = 0;
  size_t bytesInUse = 0;

  // device bytes per track of a slot: inputs at the planned surfaces per
  // track, outputs of the computed components, track-state records
  size_t perTrackBytes(int maxStates) const {
    const size_t k = kPlannedSurfacesPerTrack;
    const size_t in = 2 * 4 + k * 4 + k * (4 + 16 + 32 + 4) + 48 + 288 + 96 + 8 + 4;
    size_t out = 7 * 8 + (size_t)maxStates * 24;
    const size_t pc = spec.packed ? 27 : 42;
    if (spec.sm) out += (size_t)maxStates * pc * 8;
    if (spec.fi) out += (size_t)maxStates * pc * 8;
    if (spec.pr) out += (size_t)maxStates * pc * 8;
    if (spec.jac) out += (size_t)maxStates * 36 * 8;
    if (opt.reference_surface >= 0) out += 42 * 8;
    if (needsExtStart(opt)) out += 2 * sizeof(ExtStart);
    return in + out + recordBytesPerTrack(maxStates, opt.precision);
  }
  // components of output array `field` (the covariance arrays may be packed)
  int comp(int field) const {
    if (spec.packed && (field == 12 || field == 14 || field == 16)) return 21;
    return kOutComp[field];
  }
  bool computes(int field) const {
    switch (field) {
      case 11: case 12: return spec.pr;
      case 13: case 14: return spec.fi;
      case 15: case 16: return spec.sm;
      case 17: return spec.jac;
      case 18: case 19: return opt.reference_surface >= 0;
      default: return true;
    }
  }
};

namespace {

ck_status slotAlloc(ck_server* s, Slot& sl) {
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming)) != cudaSuccess)
    return cudaFail(e, "server stream");
  const size_t cap = (size_t)s->capacity;
  const size_t k = kPlannedSurfacesPerTrack;
  const int ms = s->cfg.max_states;
  const size_t inBytes[kInputArrays] = {4 * (cap + 1), 4 * cap * k, 4 * (cap + 1), 4 * cap * k,
                                        16 * cap * k,  32 * cap * k, 48 * cap,  288 * cap,
                                        96 * cap,      8 * cap,      4 * cap,   4 * cap * k};
  for (int i = 0; i < kInputArrays; ++i) {
    if ((e = sl.din[i].ensure(inBytes[i])) != cudaSuccess) return cudaFail(e, "server input");
    sl.inPlanned[i] = inBytes[i];
  }
  const size_t S = cap * (size_t)ms;
  size_t pout = 0;
  for (int i = 0; i < kOutArrays; ++i) {
    if (!s->computes(i)) continue;
    const size_t bytes = kOutElem[i] * s->comp(i) * (kPerState[i] ? S : cap);
    if ((e = sl.dout[i].ensure(bytes)) != cudaSuccess) return cudaFail(e, "server output");
    pout += (bytes + 255) & ~(size_t)255;
  }
  if ((e = sl.table.ensure(sizeof(int4) * kMaxEventsPerBatch)) != cudaSuccess)
    return cudaFail(e, "server table");
  if ((e = cudaMallocHost((void**)&sl.pinTable, sizeof(int4) * kMaxEventsPerBatch)) !=
          cudaSuccess ||
      (e = cudaMallocHost(&sl.pinOut, pout)) != cudaSuccess)
    return cudaFail(e, "server pinned buffers");
  sl.pinOutBytes = pout;
  return preparePipeline(s->h, sl.ctx, s->capacity, ms, s->opt.precision,
                         needsExtStart(s->opt));
}

// Offsets of the staged result arrays in the slot's pinned buffer.
void stagedBases(ck_server* s, Slot& sl, size_t base[kOutArrays]) {
  const size_t n = (size_t)sl.nTracks, S = n * (size_t)s->cfg.max_states;
  size_t off = 0;
  for (int i = 0; i < kOutArrays; ++i) {
    base[i] = off;
    if (!s->computes(i)) continue;
    off += (kOutElem[i] * s->comp(i) * (kPerState[i] ? S : n) + 255) & ~(size_t)255;
  }
}

// Copies the co-batch's inputs, launches the fit and the result copies on the
// slot's stream.
ck_status launchSlot(ck_server* s, Slot& sl) {
  const int n = sl.nTracks;
  const int nEv = (int)sl.events.size();
  cudaError_t e;
  // ---- inputs, straight from the callers' arrays
  int t0 = 0, seqBase = 0, measBase = 0, maxM = 1;
  for (int i = 0; i < nEv; ++i) {
    Event& ev = *sl.events[i];
    const ck_batch_in& in = ev.in;
    const int m = ev.n;
    sl.pinTable[4 * i + 0] = t0;
    sl.pinTable[4 * i + 1] = m;
    sl.pinTable[4 * i + 2] = seqBase;
    sl.pinTable[4 * i + 3] = measBase;
    maxM = std::max(maxM, m + 1);
    const bool last = (i == nEv - 1);
    struct Item {
      int buf;
      const void* src;
      size_t dstOff, bytes;
    } items[] = {
        {0, in.seq_offsets, 4 * (size_t)t0, 4 * (size_t)(m + (last ? 1 : 0))},
        {1, in.seq_surfaces, 4 * (size_t)seqBase, 4 * (size_t)ev.nSeq},
        {2, in.meas_offsets, 4 * (size_t)t0, 4 * (size_t)(m + (last ? 1 : 0))},
        {3, in.meas_surfaces, 4 * (size_t)measBase, 4 * (size_t)ev.nMeas},
        {4, in.meas_values, 16 * (size_t)measBase, 16 * (size_t)ev.nMeas},
        {5, in.meas_cov, 32 * (size_t)measBase, 32 * (size_t)ev.nMeas},
        {6, in.start_params, 48 * (size_t)t0, 48 * (size_t)m},
        {7, in.start_cov, 288 * (size_t)t0, 288 * (size_t)m},
        {8, in.start_frames, 96 * (size_t)t0, 96 * (size_t)m},
        {9, in.particle, 8 * (size_t)t0, 8 * (size_t)m},
        {10, in.particle_pdg, 4 * (size_t)t0, 4 * (size_t)m},
        {11, in.meas_subspace, 4 * (size_t)measBase, 4 * (size_t)ev.nMeas},
    };
    for (const Item& it : items) {
      if (!it.bytes) continue;
      if (it.dstOff + it.bytes > sl.inPlanned[it.buf])
        return fail(CK_ERR_BUDGET, "co-batch exceeds slot buffers");
      char* dst = (char*)sl.din[it.buf].p + it.dstOff;
      if (it.buf == 10 && !it.src) {
        fillInt<<<(m + 255) / 256, 256, 0, sl.stream>>>((int32_t*)dst, m, 211);
        continue;
      }
      if (it.buf == 11 && !it.src) {  // 2D source links
        const int nm = ev.nMeas;
        fillInt<<<(nm + 255) / 256, 256, 0, sl.stream>>>((int32_t*)dst, nm, CK_MEAS_LOC01);
        continue;
      }
      if ((e = cudaMemcpyAsync(dst, it.src, it.bytes, cudaMemcpyDefault, sl.stream)) !=
          cudaSuccess)
        return cudaFail(e, "server input copy");
    }
    t0 += m;
    seqBase += ev.nSeq;
    measBase += ev.nMeas;
  }
  if ((e = cudaMemcpyAsync(sl.table.p, sl.pinTable, sizeof(int4) * nEv, cudaMemcpyHostToDevice,
                           sl.stream)) != cudaSuccess)
    return cudaFail(e, "server table copy");
  {
    dim3 grid((unsigned)std::min(64, (maxM + 255) / 256), (unsigned)nEv);
    shiftOffsets<<<grid, 256, 0, sl.stream>>>((int32_t*)sl.din[0].p, (int32_t*)sl.din[2].p,
                                              (const int4*)sl.table.p, nEv);
    if ((e = cudaGetLastError()) != cudaSuccess) return cudaFail(e, "offset shift");
  }
  ck_batch_in din{};
  din.n_tracks = n;
  din.memory = CK_MEM_DEVICE;
  din.seq_offsets = (const int32_t*)sl.din[0].p;
  din.seq_surfaces = (const int32_t*)sl.din[1].p;
  din.meas_offsets = (const int32_t*)sl.din[2].p;
  din.meas_surfaces = (const int32_t*)sl.din[3].p;
  din.meas_values = (const double*)sl.din[4].p;
  din.meas_cov = (const double*)sl.din[5].p;
  din.start_params = (const double*)sl.din[6].p;
  din.start_cov = (const double*)sl.din[7].p;
  din.start_frames = (const double*)sl.din[8].p;
  din.particle = (const float*)sl.din[9].p;
  din.particle_pdg = (const int32_t*)sl.din[10].p;
  din.meas_subspace = (const int32_t*)sl.din[11].p;
  ck_batch_out dout{};
  dout.max_states = s->cfg.max_states;
  dout.components = s->cfg.components;
  dout.memory = CK_MEM_DEVICE;
  void** f[kOutArrays];
  outFields(dout, f);
  for (int i = 0; i < kOutArrays; ++i) *f[i] = sl.dout[i].cap ? sl.dout[i].p : nullptr;
  ck_status st;
  {
    std::lock_guard<std::mutex> lock(s->h->mu);
    cudaSetDevice(s->h->device);
    st = enqueuePipeline(s->h, sl.ctx, s->opt, din, dout, s->tune, sl.stream, false,
                         s->gridBlocks);
  }
  if (st != CK_OK) return st;
  // ---- results
  const int ms = s->cfg.max_states;
  bool anyStaged = false;
  t0 = 0;
  for (auto& evp : sl.events) {
    Event& ev = *evp;
    const int m = ev.n;
    if (ev.staged) {
      anyStaged = true;
    } else {
      ck_batch_out o = ev.out;
      void** g[kOutArrays];
      outFields(o, g);
      for (int i = 0; i < kOutArrays; ++i) {
        if (!*g[i] || !sl.dout[i].cap) continue;
        const size_t el = kOutElem[i];
        const char* src = (const char*)sl.dout[i].p + el * t0;
        // rows of the SoA array: components (x states)
        const size_t rows = (kPerState[i] ? (size_t)ms : 1) * (size_t)s->comp(i);
        if (rows == 1)
          e = cudaMemcpyAsync(*g[i], src, el * m, cudaMemcpyDefault, sl.stream);
        else
          e = cudaMemcpy2DAsync(*g[i], el * m, src, el * n, el * m, rows, cudaMemcpyDefault,
                                sl.stream);
        if (e != cudaSuccess) return cudaFail(e, "server result copy");
      }
    }
    t0 += m;
  }
  if (anyStaged) {
    size_t base[kOutArrays];
    stagedBases(s, sl, base);
    const size_t S = (size_t)n * ms;
    for (int i = 0; i < kOutArrays; ++i) {
      if (!sl.dout[i].cap) continue;
      const size_t bytes = kOutElem[i] * s->comp(i) * (kPerState[i] ? S : (size_t)n);
      if ((e = cudaMemcpyAsync((char*)sl.pinOut + base[i], sl.dout[i].p, bytes,
                               cudaMemcpyDeviceToHost, sl.stream)) != cudaSuccess)
        return cudaFail(e, "server staged copy");
    }
  }
  if ((e = cudaEventRecord(sl.done, sl.stream)) != cudaSuccess) return cudaFail(e, "event");
  return CK_OK;
}

// Completes a finished slot: host copies of the staged events' results
// (the rows of every staged array, split over the server's copy threads:
// de-striding into pageable memory is bound by page faults and memory
// bandwidth, which several cores share out).
void harvestSlot(ck_server* s, Slot& sl) {
  const int n = sl.nTracks, ms = s->cfg.max_states;
  size_t base[kOutArrays];
  stagedBases(s, sl, base);
  struct Row {
    char* dst;
    const char* src;
    size_t bytes;
  };
  std::vector<Row> rows;
  size_t total = 0;
  int t0 = 0;
  for (auto& evp : sl.events) {
    Event& ev = *evp;
    const int m = ev.n;
    if (ev.staged) {
      ck_batch_out o = ev.out;
      void** g[kOutArrays];
      outFields(o, g);
      for (int i = 0; i < kOutArrays; ++i) {
        if (!*g[i] || !sl.dout[i].cap) continue;
        const size_t el = kOutElem[i];
        const char* src = (const char*)sl.pinOut + base[i] + el * t0;
        char* dst = (char*)*g[i];
        const int nr = (kPerState[i] ? ms : 1) * s->comp(i);
        for (int r = 0; r < nr; ++r)
          rows.push_back({dst + el * m * (size_t)r, src + el * n * (size_t)r, el * m});
        total += el * m * (size_t)nr;
      }
    }
    t0 += m;
  }
  // one thread per 4 MB, at most the server's copy threads
  const int nt = (int)std::max<size_t>(1, std::min<size_t>(s->copyThreads, total >> 22));
  auto work = [&](int k) {
    for (size_t r = k; r < rows.size(); r += nt) std::memcpy(rows[r].dst, rows[r].src, rows[r].bytes);
  };
  std::vector<std::thread> helpers;
  for (int k = 1; k < nt; ++k) helpers.emplace_back(work, k);
  work(0);
  for (auto& h : helpers) h.join();
  const auto now = Clock::now();
  for (auto& evp : sl.events)
    evp->latencyMs = std::chrono::duration<double, std::milli>(now - evp->submitted).count();
}

void finishSlot(ck_server* s, Slot& sl, ck_status st) {
  for (auto& ev : sl.events) {
    if (st != CK_OK) {
      ev->status = st;
      ev->latencyMs =
          std::chrono::duration<double, std::milli>(Clock::now() - ev->submitted).count();
    }
    s->tracksDone += ev->n;
    ++s->completed;
    s->finished.push_back(std::move(ev));
  }
  sl.events.clear();
  s->bytesInUse -= (size_t)sl.nTracks * s->perTrackBytes(s->cfg.max_states);
  sl.nTracks = sl.nSeq = sl.nMeas = 0;
  sl.busy = false;
  s->cvDone.notify_all();
}

// The delivery thread: de-strides the staged (pageable) results of finished
// slots, so that the request loop keeps admitting and launching meanwhile;
// the slot is free again once its results are in place.
void deliveryLoop(ck_server* s) {
  std::unique_lock<std::mutex> lock(s->mu);
  while (true) {
    s->cvHarvest.wait(lock, [&] { return s->stop || !s->toHarvest.empty(); });
    if (s->toHarvest.empty()) break;  // stopping, nothing left
    Slot* sl = s->toHarvest.front();
    s->toHarvest.pop_front();
    lock.unlock();
    harvestSlot(s, *sl);
    lock.lock();
    sl->harvesting = false;
    finishSlot(s, *sl, CK_OK);
    s->cvWork.notify_one();
  }
}

void workerLoop(ck_server* s) {
  cudaSetDevice(s->h->device);
  const size_t planned = (size_t)kPlannedSurfacesPerTrack * (size_t)s->capacity;
  std::unique_lock<std::mutex> lock(s->mu);
  while (true) {
    // completion of in-flight slots
    for (auto& slp : s->slots) {
      Slot& sl = *slp;
      if (!sl.busy || sl.harvesting) continue;
      cudaError_t q = cudaEventQuery(sl.done);
      if (q == cudaErrorNotReady) continue;
      ck_status st = CK_OK;
      if (q != cudaSuccess) {
        st = cudaFail(q, "server batch");
        s->error = st;
        s->errorMsg = g_lastError;
      } else {
        bool staged = false;
        for (auto& ev : sl.events) staged |= ev->staged;
        if (staged) {
          // pageable results: the delivery thread copies them
          sl.harvesting = true;
          s->toHarvest.push_back(&sl);
          s->cvHarvest.notify_one();
          continue;
        }
        const auto now = Clock::now();
        for (auto& ev : sl.events)
          ev->latencyMs = std::chrono::duration<double, std::milli>(now - ev->submitted).count();
      }
      finishSlot(s, sl, st);
    }
    // admission into free slots: co-batch the oldest pending events
    for (auto& slp : s->slots) {
      Slot& sl = *slp;
      if (sl.busy || s->pending.empty()) continue;
      int n = 0;
      size_t nSeq = 0, nMeas = 0;
      while (!s->pending.empty() && (int)sl.events.size() < kMaxEventsPerBatch) {
        const Event& ev = *s->pending.front();
        if (n + ev.n > s->capacity || nSeq + ev.nSeq > planned || nMeas + ev.nMeas > planned)
          break;
        n += ev.n;
        nSeq += ev.nSeq;
        nMeas += ev.nMeas;
        sl.events.push_back(std::move(s->pending.front()));
        s->pending.pop_front();
      }
      if (sl.events.empty()) continue;
      sl.nTracks = n;
      sl.nSeq = (int)nSeq;
      sl.nMeas = (int)nMeas;
      sl.busy = true;
      s->bytesInUse += (size_t)n * s->perTrackBytes(s->cfg.max_states);
      lock.unlock();
      ck_status st = launchSlot(s, sl);
      lock.lock();
      if (st != CK_OK) {
        s->error = st;
        s->errorMsg = g_lastError;
        cudaStreamSynchronize(sl.stream);
        finishSlot(s, sl, st);
      }
    }
    bool anyBusy = false, anyGpu = false;
    for (auto& slp : s->slots) {
      anyBusy |= slp->busy;
      anyGpu |= slp->busy && !slp->harvesting;
    }
    if (s->stop && !anyBusy && s->pending.empty()) break;
    if (anyGpu) {
      // poll in-flight work at a short interval
      s->cvWork.wait_for(lock, std::chrono::microseconds(50));
    } else if (anyBusy) {
      // slots in delivery: the delivery thread notifies when one frees
      s->cvWork.wait_for(lock, std::chrono::milliseconds(1));
    } else {
      s->cvWork.wait(lock, [&] { return s->stop || !s->pending.empty(); });
    }
  }
}

ck_status readCount(const int32_t* offsets, int n, int memory, int* out) {
  if (memory == CK_MEM_HOST) {
    *out = offsets[n];
    return CK_OK;
  }
  cudaError_t e = cudaMemcpy(out, offsets + n, sizeof(int32_t), cudaMemcpyDefault);
  return e == cudaSuccess ? CK_OK : cudaFail(e, "event size");
}

}  // namespace

extern "C" {

ck_status ck_server_create(ck_handle* h, const ck_options* opt, const ck_server_config* cfg,
                           ck_server** out) {
  if (!h || !cfg || !out) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  ck_status vs = validateOptions(opt);
  if (vs != CK_OK) return vs;
  if ((vs = validateReference(h, opt)) != CK_OK) return vs;
  if (cfg->n_streams < 1 || cfg->n_streams > 16 || cfg->max_states < 1 ||
      cfg->memory_budget_bytes <= 0 || cfg->max_batch_tracks < 1 || cfg->grid_blocks < 0 ||
      cfg->steps_per_round < 0 || cfg->steps_per_round > 64)
    return fail(CK_ERR_INVALID_ARGUMENT, "bad server configuration");
  *out = nullptr;
  auto s = std::make_unique<ck_server>();
  s->h = h;
  s->opt = *opt;
  s->cfg = *cfg;
  s->spec = {(cfg->components & CK_OUT_SMOOTHED) != 0, (cfg->components & CK_OUT_FILTERED) != 0,
             (cfg->components & CK_OUT_PREDICTED) != 0, (cfg->components & CK_OUT_JACOBIAN) != 0,
             (cfg->components & CK_OUT_PACKED_COV) != 0};
  s->tune = h->tune[opt->precision];
  s->tune.spr = cfg->steps_per_round > 0 ? cfg->steps_per_round : kServerStepsPerRound;
  s->tune.grid = 0;
  const int whole = std::max(1, gridBlocksFor(h, s->tune));
  s->gridBlocks = cfg->grid_blocks > 0
                      ? cfg->grid_blocks
                      : (cfg->n_streams > 1 ? (whole + cfg->n_streams - 2) / (cfg->n_streams - 1)
                                            : whole);
  const size_t perTrack = s->perTrackBytes(cfg->max_states);
  int64_t cap = cfg->memory_budget_bytes / (int64_t)(perTrack * cfg->n_streams);
  cap = std::min<int64_t>(cap, cfg->max_batch_tracks);
  if (cap < 1) return fail(CK_ERR_BUDGET, "budget too small for one track per stream");
  s->capacity = (int)cap;
  cudaSetDevice(h->device);
  for (int i = 0; i < cfg->n_streams; ++i) {
    s->slots.push_back(std::make_unique<Slot>());
    ck_status st = slotAlloc(s.get(), *s->slots.back());
    if (st != CK_OK) {
      ck_server_destroy(s.release());
      return st;
    }
  }
  s->copyThreads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  s->worker = std::thread(workerLoop, s.get());
  s->delivery = std::thread(deliveryLoop, s.get());
  *out = s.release();
  return CK_OK;
}

ck_status ck_server_submit(ck_server* s, int64_t event_id, const ck_batch_in* in,
                           const ck_batch_out* results) {
  if (!s || !in || !results || in->n_tracks < 0)
    return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument or negative track count");
  const int n = in->n_tracks;
  if (n > s->capacity) return fail(CK_ERR_BUDGET, "event larger than a stream's capacity");
  if (results->max_states != s->cfg.max_states)
    return fail(CK_ERR_INVALID_ARGUMENT, "results.max_states differs from the server's");
  if (!results->status) return fail(CK_ERR_INVALID_ARGUMENT, "status array is required");
  {
    ck_batch_out o = *results;
    void** g[kOutArrays];
    outFields(o, g);
    for (int i = 0; i < kOutArrays; ++i)
      if (*g[i] && !s->computes(i))
        return fail(CK_ERR_INVALID_ARGUMENT, "results ask for a component the server omits");
  }
  if (n > 0 && (!in->seq_offsets || !in->seq_surfaces || !in->meas_offsets ||
                !in->meas_surfaces || !in->meas_values || !in->meas_cov || !in->start_params ||
                !in->start_cov || !in->start_frames || !in->particle))
    return fail(CK_ERR_INVALID_ARGUMENT, "input array missing");
  auto ev = std::make_unique<Event>();
  ev->id = event_id;
  ev->n = n;
  ev->in = *in;
  ev->out = *results;
  if (n > 0) {
    if (in->memory == CK_MEM_HOST && (in->seq_offsets[0] != 0 || in->meas_offsets[0] != 0))
      return fail(CK_ERR_INVALID_ARGUMENT, "CSR offsets must start at 0");
    ck_status st;
    if ((st = readCount(in->seq_offsets, n, in->memory, &ev->nSeq)) != CK_OK ||
        (st = readCount(in->meas_offsets, n, in->memory, &ev->nMeas)) != CK_OK)
      return st;
  }
  const size_t planned = (size_t)kPlannedSurfacesPerTrack * (size_t)s->capacity;
  if (ev->nSeq < 0 || ev->nMeas < 0 || (size_t)ev->nSeq > planned || (size_t)ev->nMeas > planned)
    return fail(CK_ERR_BUDGET, "event exceeds the planned surfaces of a stream");
  if (results->memory == CK_MEM_HOST) {
    cudaPointerAttributes a{};
    ev->staged = cudaPointerGetAttributes(&a, results->status) != cudaSuccess ||
                 a.type == cudaMemoryTypeUnregistered;
    cudaGetLastError();
  }
  ev->submitted = Clock::now();
  {
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) return fail(CK_ERR_INVALID_ARGUMENT, "server stopping");
    ++s->submitted;
    if (n == 0) {
      ++s->completed;
      s->finished.push_back(std::move(ev));
      s->cvDone.notify_all();
      return CK_OK;
    }
    s->pending.push_back(std::move(ev));
  }
  s->cvWork.notify_one();
  return CK_OK;
}

ck_status ck_server_poll(ck_server* s, int64_t* event_id, double* latency_ms,
                         int32_t timeout_ms) {
  if (!s || !event_id) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  std::unique_ptr<Event> ev;
  {
    std::unique_lock<std::mutex> lock(s->mu);
    if (s->finished.empty() && timeout_ms > 0)
      s->cvDone.wait_for(lock, std::chrono::milliseconds(timeout_ms),
                         [&] { return !s->finished.empty(); });
    if (s->finished.empty()) return fail(CK_ERR_NOT_READY, "no finished event");
    ev = std::move(s->finished.front());
    s->finished.pop_front();
  }
  *event_id = ev->id;
  if (latency_ms) *latency_ms = ev->latencyMs;
  if (ev->status != CK_OK) return fail(ev->status, "the event's batch failed");
  return CK_OK;
}

ck_status ck_server_stats(ck_server* s, int64_t* submitted, int64_t* completed, int64_t* tracks,
                          int64_t* bytes_in_use) {
  if (!s) return fail(CK_ERR_INVALID_ARGUMENT, "NULL server");
  std::lock_guard<std::mutex> lock(s->mu);
  if (submitted) *submitted = s->submitted;
  if (completed) *completed = s->completed;
  if (tracks) *tracks = s->tracksDone;
  if (bytes_in_use) *bytes_in_use = (int64_t)s->bytesInUse;
  if (s->error != CK_OK) {
    g_lastError = s->errorMsg;
    return s->error;
  }
  return CK_OK;
}

int32_t ck_server_capacity(ck_server* s) { return s ? s->capacity : 0; }

ck_status ck_server_destroy(ck_server* s) {
  if (!s) return CK_OK;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
  }
  s->cvWork.notify_all();
  if (s->worker.joinable()) s->worker.join();
  s->cvHarvest.notify_all();
  if (s->delivery.joinable()) s->delivery.join();
  cudaSetDevice(s->h->device);
  for (auto& slp : s->slots) {
    Slot& sl = *slp;
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    for (auto& b : sl.din) b.release();
    for (auto& b : sl.dout) b.release();
    sl.table.release();
    sl.ctx.release();
    if (sl.pinTable) cudaFreeHost(sl.pinTable);
    if (sl.pinOut) cudaFreeHost(sl.pinOut);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  delete s;
  return CK_OK;
}

}  // extern "C"
