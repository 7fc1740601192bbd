// ck_server.cu — continuous-batching serving loop of the fitter.
//
// Events (one ck_batch_in each) arrive through ck_server_submit from any
// host thread; their inputs are copied and queued. One request thread runs
// the loop:
//   * admission: while a stream slot is free, the pending events (oldest
//     first) that fit the slot's track capacity are taken together into one
//     co-batch — events of different sizes share a launch;
//   * launch: the co-batch's inputs are staged through the slot's pinned
//     buffer, copied to the slot's device buffers and fitted on the slot's
//     stream with a share of the GPU (grid = resident blocks / streams), so
//     batches on different streams overlap on the device;
//   * completion: finished slots are detected with CUDA events, their
//     results copied back and split per event, each event's latency is its
//     submit-to-completion wall time.
// Device memory: every slot holds input, output and scratch buffers for its
// capacity; the capacity is the largest track count for which all slots fit
// the memory budget. An event larger than a slot's capacity is rejected with
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
#include <type_traits>
#include <vector>

#include "ck_api_internal.h"
#include "ck_launch.h"

using namespace ck;

namespace {

using Clock = std::chrono::steady_clock;

struct Event {
  int64_t id = 0;
  int n = 0;
  std::vector<int32_t> seqOff, seq, measOff, measSurf, pdg;
  std::vector<double> measVal, measCov, sp, sc, frames;
  std::vector<float> part;
  Clock::time_point submitted;
  // results (host)
  std::vector<int32_t> status, nStates, nMeas, nHoles, nOut, ndf, surf;
  std::vector<uint32_t> flags;
  std::vector<double> chi2, path, schi2, sm, smc, fi, fic, pr, prc, jac;
  double latencyMs = 0;
};

// Output components carried per event.
struct OutSpec {
  bool sm, fi, pr, jac;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  FitContext ctx;
  DevBuf din[11];
  size_t inPlanned[11] = {};
  DevBuf dout[18];
  void* pinIn = nullptr;
  size_t pinInBytes = 0;
  void* pinOut = nullptr;
  size_t pinOutBytes = 0;
  std::vector<std::unique_ptr<Event>> events;
  int nTracks = 0;
  bool busy = false;
};

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
  bool stop = false;
  ck_status error = CK_OK;
  std::string errorMsg;
  int64_t submitted = 0, completed = 0, tracksDone = 0;
  size_t bytesInUse = 0;

  size_t perTrackBytes(int maxStates) const {
    // inputs: offsets, 20 sequence surfaces, 20 measurements, start pars
    const size_t in = 2 * 4 + 20 * 4 + 20 * (4 + 16 + 32) + 48 + 288 + 96 + 8 + 4;
    size_t out = 7 * 8 + (size_t)maxStates * 24;
    if (spec.sm) out += (size_t)maxStates * 42 * 8;
    if (spec.fi) out += (size_t)maxStates * 42 * 8;
    if (spec.pr) out += (size_t)maxStates * 42 * 8;
    if (spec.jac) out += (size_t)maxStates * 36 * 8;
    return in + out + recordBytesPerTrack(maxStates, opt.precision);
  }
};

namespace {

ck_status slotAlloc(ck_server* s, Slot& sl) {
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming)) != cudaSuccess)
    return cudaFail(e, "server stream");
  const size_t cap = (size_t)s->capacity;
  const int ms = s->cfg.max_states;
  const size_t inBytes[11] = {4 * (cap + 1), 4 * cap * 20, 4 * (cap + 1), 4 * cap * 20,
                              16 * cap * 20, 32 * cap * 20, 48 * cap, 288 * cap,
                              96 * cap, 8 * cap, 4 * cap};
  size_t pin = 0;
  for (int i = 0; i < 11; ++i) {
    if ((e = sl.din[i].ensure(inBytes[i])) != cudaSuccess) return cudaFail(e, "server input");
    sl.inPlanned[i] = inBytes[i];
    pin += (inBytes[i] + 255) & ~(size_t)255;
  }
  const size_t S = cap * (size_t)ms;
  const size_t outBytes[18] = {4 * cap, 4 * cap, 4 * cap, 4 * cap, 4 * cap, 4 * cap, 8 * cap,
                               4 * S, 4 * S, 8 * S, 8 * S,
                               s->spec.pr ? 48 * S : 0, s->spec.pr ? 288 * S : 0,
                               s->spec.fi ? 48 * S : 0, s->spec.fi ? 288 * S : 0,
                               s->spec.sm ? 48 * S : 0, s->spec.sm ? 288 * S : 0,
                               s->spec.jac ? 288 * S : 0};
  size_t pout = 0;
  for (int i = 0; i < 18; ++i) {
    if (outBytes[i] == 0) continue;
    if ((e = sl.dout[i].ensure(outBytes[i])) != cudaSuccess) return cudaFail(e, "server output");
    pout += (outBytes[i] + 255) & ~(size_t)255;
  }
  if ((e = cudaMallocHost(&sl.pinIn, pin)) != cudaSuccess ||
      (e = cudaMallocHost(&sl.pinOut, pout)) != cudaSuccess)
    return cudaFail(e, "server pinned buffers");
  sl.pinInBytes = pin;
  sl.pinOutBytes = pout;
  ck_status st = preparePipeline(s->h, sl.ctx, s->capacity, ms, s->opt.precision);
  return st;
}

// Concatenates the slot's events into its pinned buffer and launches the
// copies and the fit on the slot's stream.
ck_status launchSlot(ck_server* s, Slot& sl) {
  const int n = sl.nTracks;
  // host staging: concatenate the events with shifted offsets
  std::vector<int32_t> so(1, 0), mo(1, 0), seq, msf, pdg;
  std::vector<double> mv, mc, sp, sc, fr;
  std::vector<float> pa;
  for (auto& ev : sl.events) {
    const int sBase = so.back(), mBase = mo.back();
    for (int t = 0; t < ev->n; ++t) {
      so.push_back(sBase + ev->seqOff[t + 1]);
      mo.push_back(mBase + ev->measOff[t + 1]);
    }
    seq.insert(seq.end(), ev->seq.begin(), ev->seq.end());
    msf.insert(msf.end(), ev->measSurf.begin(), ev->measSurf.end());
    mv.insert(mv.end(), ev->measVal.begin(), ev->measVal.end());
    mc.insert(mc.end(), ev->measCov.begin(), ev->measCov.end());
    sp.insert(sp.end(), ev->sp.begin(), ev->sp.end());
    sc.insert(sc.end(), ev->sc.begin(), ev->sc.end());
    fr.insert(fr.end(), ev->frames.begin(), ev->frames.end());
    pa.insert(pa.end(), ev->part.begin(), ev->part.end());
    pdg.insert(pdg.end(), ev->pdg.begin(), ev->pdg.end());
  }
  const void* srcs[11] = {so.data(), seq.data(), mo.data(), msf.data(), mv.data(), mc.data(),
                          sp.data(), sc.data(),  fr.data(), pa.data(),  pdg.data()};
  const size_t bytes[11] = {4 * so.size(), 4 * seq.size(), 4 * mo.size(), 4 * msf.size(),
                            8 * mv.size(), 8 * mc.size(),  8 * sp.size(), 8 * sc.size(),
                            8 * fr.size(), 4 * pa.size(),  4 * pdg.size()};
  // the pinned staging buffer holds exactly the planned sizes
  for (int i = 0; i < 11; ++i)
    if (bytes[i] > sl.inPlanned[i]) return fail(CK_ERR_BUDGET, "co-batch exceeds slot buffers");
  char* pin = (char*)sl.pinIn;
  size_t off = 0;
  cudaError_t e;
  for (int i = 0; i < 11; ++i) {
    std::memcpy(pin + off, srcs[i], bytes[i]);
    if (bytes[i] &&
        (e = cudaMemcpyAsync(sl.din[i].p, pin + off, bytes[i], cudaMemcpyHostToDevice,
                             sl.stream)) != cudaSuccess)
      return cudaFail(e, "server input copy");
    off += (bytes[i] + 255) & ~(size_t)255;
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
  ck_batch_out dout{};
  dout.max_states = s->cfg.max_states;
  dout.memory = CK_MEM_DEVICE;
  void** f[18] = {(void**)&dout.status,          (void**)&dout.n_states,
                  (void**)&dout.n_measurements,  (void**)&dout.n_holes,
                  (void**)&dout.n_outliers,      (void**)&dout.ndf,
                  (void**)&dout.chi2_sum,        (void**)&dout.state_surface,
                  (void**)&dout.state_flags,     (void**)&dout.state_path_length,
                  (void**)&dout.state_chi2,      (void**)&dout.predicted,
                  (void**)&dout.predicted_cov,   (void**)&dout.filtered,
                  (void**)&dout.filtered_cov,    (void**)&dout.smoothed,
                  (void**)&dout.smoothed_cov,    (void**)&dout.jacobian};
  for (int i = 0; i < 18; ++i) *f[i] = sl.dout[i].cap ? sl.dout[i].p : nullptr;
  ck_status st;
  {
    std::lock_guard<std::mutex> lock(s->h->mu);
    cudaSetDevice(s->h->device);
    st = enqueuePipeline(s->h, sl.ctx, s->opt, din, dout, s->tune, sl.stream, false,
                         s->gridBlocks);
  }
  if (st != CK_OK) return st;
  // results back to the pinned buffer
  const int ms = s->cfg.max_states;
  const size_t S = (size_t)n * ms;
  const size_t ob[18] = {4 * (size_t)n, 4 * (size_t)n, 4 * (size_t)n, 4 * (size_t)n, 4 * (size_t)n,
                         4 * (size_t)n, 8 * (size_t)n, 4 * S, 4 * S, 8 * S, 8 * S, 48 * S, 288 * S,
                         48 * S, 288 * S, 48 * S, 288 * S, 288 * S};
  char* po = (char*)sl.pinOut;
  off = 0;
  for (int i = 0; i < 18; ++i) {
    if (!sl.dout[i].cap) continue;
    if ((e = cudaMemcpyAsync(po + off, sl.dout[i].p, ob[i], cudaMemcpyDeviceToHost,
                             sl.stream)) != cudaSuccess)
      return cudaFail(e, "server output copy");
    off += (ob[i] + 255) & ~(size_t)255;
  }
  if ((e = cudaEventRecord(sl.done, sl.stream)) != cudaSuccess) return cudaFail(e, "event");
  return CK_OK;
}

// Splits a finished slot's results into its events (SoA with the co-batch's
// track count innermost -> each event's own SoA).
void harvestSlot(ck_server* s, Slot& sl) {
  const int n = sl.nTracks, ms = s->cfg.max_states;
  const size_t S = (size_t)n * ms;
  const size_t ob[18] = {4 * (size_t)n, 4 * (size_t)n, 4 * (size_t)n, 4 * (size_t)n, 4 * (size_t)n,
                         4 * (size_t)n, 8 * (size_t)n, 4 * S, 4 * S, 8 * S, 8 * S, 48 * S, 288 * S,
                         48 * S, 288 * S, 48 * S, 288 * S, 288 * S};
  const char* po = (const char*)sl.pinOut;
  const char* base[18];
  size_t off = 0;
  for (int i = 0; i < 18; ++i) {
    base[i] = nullptr;
    if (!sl.dout[i].cap) continue;
    base[i] = po + off;
    off += (ob[i] + 255) & ~(size_t)255;
  }
  const auto now = Clock::now();
  int t0 = 0;
  for (auto& ev : sl.events) {
    const int m = ev->n;
    auto per = [&](int i, auto& v) {
      using T = typename std::remove_reference<decltype(v)>::type::value_type;
      v.assign((const T*)base[i] + t0, (const T*)base[i] + t0 + m);
    };
    per(0, ev->status);
    per(1, ev->nStates);
    per(2, ev->nMeas);
    per(3, ev->nHoles);
    per(4, ev->nOut);
    per(5, ev->ndf);
    per(6, ev->chi2);
    auto soa = [&](int i, int C, auto& v) {
      using T = typename std::remove_reference<decltype(v)>::type::value_type;
      if (!base[i]) return;
      const T* src = (const T*)base[i];
      v.resize((size_t)ms * C * m);
      for (int k = 0; k < ms; ++k)
        for (int c = 0; c < C; ++c)
          std::memcpy(&v[((size_t)k * C + c) * m], src + ((size_t)k * C + c) * n + t0,
                      sizeof(T) * m);
    };
    soa(7, 1, ev->surf);
    soa(8, 1, ev->flags);
    soa(9, 1, ev->path);
    soa(10, 1, ev->schi2);
    soa(11, 6, ev->pr);
    soa(12, 36, ev->prc);
    soa(13, 6, ev->fi);
    soa(14, 36, ev->fic);
    soa(15, 6, ev->sm);
    soa(16, 36, ev->smc);
    soa(17, 36, ev->jac);
    ev->latencyMs = std::chrono::duration<double, std::milli>(now - ev->submitted).count();
    t0 += m;
  }
}

void workerLoop(ck_server* s) {
  cudaSetDevice(s->h->device);
  std::unique_lock<std::mutex> lock(s->mu);
  while (true) {
    // completion of in-flight slots
    for (auto& slp : s->slots) {
      Slot& sl = *slp;
      if (!sl.busy) continue;
      cudaError_t q = cudaEventQuery(sl.done);
      if (q == cudaErrorNotReady) continue;
      if (q != cudaSuccess) {
        s->error = cudaFail(q, "server batch");
        s->errorMsg = g_lastError;
      } else {
        harvestSlot(s, sl);
      }
      for (auto& ev : sl.events) {
        s->tracksDone += ev->n;
        ++s->completed;
        s->finished.push_back(std::move(ev));
      }
      sl.events.clear();
      s->bytesInUse -= (size_t)sl.nTracks * s->perTrackBytes(s->cfg.max_states);
      sl.nTracks = 0;
      sl.busy = false;
      s->cvDone.notify_all();
    }
    // admission into free slots: co-batch the oldest pending events
    for (auto& slp : s->slots) {
      Slot& sl = *slp;
      if (sl.busy || s->pending.empty()) continue;
      int n = 0;
      while (!s->pending.empty() && n + s->pending.front()->n <= s->capacity) {
        n += s->pending.front()->n;
        sl.events.push_back(std::move(s->pending.front()));
        s->pending.pop_front();
      }
      if (sl.events.empty()) continue;
      sl.nTracks = n;
      s->bytesInUse += (size_t)n * s->perTrackBytes(s->cfg.max_states);
      lock.unlock();
      ck_status st = launchSlot(s, sl);
      lock.lock();
      if (st != CK_OK) {
        s->error = st;
        s->errorMsg = g_lastError;
        for (auto& ev : sl.events) {
          ev->status.assign(ev->n, CK_TRACK_NOT_PROCESSED);
          ++s->completed;
          s->finished.push_back(std::move(ev));
        }
        sl.events.clear();
        s->bytesInUse -= (size_t)n * s->perTrackBytes(s->cfg.max_states);
        sl.nTracks = 0;
        s->cvDone.notify_all();
        continue;
      }
      sl.busy = true;
    }
    bool anyBusy = false;
    for (auto& slp : s->slots) anyBusy |= slp->busy;
    if (s->stop && !anyBusy && s->pending.empty()) break;
    if (anyBusy) {
      // poll in-flight work at a short interval
      s->cvWork.wait_for(lock, std::chrono::microseconds(50));
    } else {
      s->cvWork.wait(lock, [&] { return s->stop || !s->pending.empty(); });
    }
  }
}

}  // namespace

extern "C" {

ck_status ck_server_create(ck_handle* h, const ck_options* opt, const ck_server_config* cfg,
                           ck_server** out) {
  if (!h || !cfg || !out) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  ck_status vs = validateOptions(opt);
  if (vs != CK_OK) return vs;
  if (cfg->n_streams < 1 || cfg->n_streams > 16 || cfg->max_states < 1 ||
      cfg->memory_budget_bytes <= 0 || cfg->max_batch_tracks < 1)
    return fail(CK_ERR_INVALID_ARGUMENT, "bad server configuration");
  *out = nullptr;
  auto s = std::make_unique<ck_server>();
  s->h = h;
  s->opt = *opt;
  s->cfg = *cfg;
  s->spec = {(cfg->components & CK_OUT_SMOOTHED) != 0, (cfg->components & CK_OUT_FILTERED) != 0,
             (cfg->components & CK_OUT_PREDICTED) != 0, (cfg->components & CK_OUT_JACOBIAN) != 0};
  s->tune = h->tune[opt->precision];
  // each stream gets an equal share of the resident blocks
  s->gridBlocks = std::max(1, gridBlocksFor(h, s->tune) / cfg->n_streams);
  const size_t perTrack = s->perTrackBytes(cfg->max_states);
  const int64_t avail = cfg->memory_budget_bytes;
  int64_t cap = avail / (int64_t)(perTrack * cfg->n_streams);
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
  s->worker = std::thread(workerLoop, s.get());
  *out = s.release();
  return CK_OK;
}

ck_status ck_server_submit(ck_server* s, int64_t event_id, const ck_batch_in* in) {
  if (!s || !in || in->n_tracks < 0 || in->memory != CK_MEM_HOST)
    return fail(CK_ERR_INVALID_ARGUMENT, "bad event (host memory required)");
  const int n = in->n_tracks;
  if (n > s->capacity) return fail(CK_ERR_BUDGET, "event larger than a stream's capacity");
  auto ev = std::make_unique<Event>();
  ev->id = event_id;
  ev->n = n;
  const int nSeq = in->seq_offsets[n], nMeas = in->meas_offsets[n];
  if (nSeq > 20 * n || nMeas > 20 * n)
    return fail(CK_ERR_INVALID_ARGUMENT, "more than 20 surfaces per track on average");
  ev->seqOff.assign(in->seq_offsets, in->seq_offsets + n + 1);
  ev->seq.assign(in->seq_surfaces, in->seq_surfaces + nSeq);
  ev->measOff.assign(in->meas_offsets, in->meas_offsets + n + 1);
  ev->measSurf.assign(in->meas_surfaces, in->meas_surfaces + nMeas);
  ev->measVal.assign(in->meas_values, in->meas_values + 2 * (size_t)nMeas);
  ev->measCov.assign(in->meas_cov, in->meas_cov + 4 * (size_t)nMeas);
  ev->sp.assign(in->start_params, in->start_params + 6 * (size_t)n);
  ev->sc.assign(in->start_cov, in->start_cov + 36 * (size_t)n);
  ev->frames.assign(in->start_frames, in->start_frames + 12 * (size_t)n);
  ev->part.assign(in->particle, in->particle + 2 * (size_t)n);
  if (in->particle_pdg)
    ev->pdg.assign(in->particle_pdg, in->particle_pdg + n);
  else
    ev->pdg.assign(n, 211);
  ev->submitted = Clock::now();
  {
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) return fail(CK_ERR_INVALID_ARGUMENT, "server stopping");
    s->pending.push_back(std::move(ev));
    ++s->submitted;
  }
  s->cvWork.notify_one();
  return CK_OK;
}

ck_status ck_server_poll(ck_server* s, int64_t* event_id, ck_batch_out* out,
                         int32_t out_capacity_tracks, double* latency_ms, int32_t timeout_ms) {
  if (!s || !event_id) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  std::unique_ptr<Event> ev;
  {
    std::unique_lock<std::mutex> lock(s->mu);
    if (s->finished.empty() && timeout_ms > 0)
      s->cvDone.wait_for(lock, std::chrono::milliseconds(timeout_ms),
                         [&] { return !s->finished.empty(); });
    if (s->finished.empty()) return fail(CK_ERR_NOT_READY, "no finished event");
    if (out && s->finished.front()->n > out_capacity_tracks)
      return fail(CK_ERR_INVALID_ARGUMENT, "output capacity smaller than the event");
    ev = std::move(s->finished.front());
    s->finished.pop_front();
  }
  *event_id = ev->id;
  if (latency_ms) *latency_ms = ev->latencyMs;
  if (out) {
    const int m = ev->n, ms = s->cfg.max_states;
    if (out->max_states != ms) return fail(CK_ERR_INVALID_ARGUMENT, "max_states mismatch");
    auto cp = [](auto* dst, const auto& v) {
      if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(v[0]));
    };
    cp(out->status, ev->status);
    cp(out->n_states, ev->nStates);
    cp(out->n_measurements, ev->nMeas);
    cp(out->n_holes, ev->nHoles);
    cp(out->n_outliers, ev->nOut);
    cp(out->ndf, ev->ndf);
    cp(out->chi2_sum, ev->chi2);
    cp(out->state_surface, ev->surf);
    cp(out->state_flags, ev->flags);
    cp(out->state_path_length, ev->path);
    cp(out->state_chi2, ev->schi2);
    cp(out->smoothed, ev->sm);
    cp(out->smoothed_cov, ev->smc);
    cp(out->filtered, ev->fi);
    cp(out->filtered_cov, ev->fic);
    cp(out->predicted, ev->pr);
    cp(out->predicted_cov, ev->prc);
    cp(out->jacobian, ev->jac);
    (void)m;
  }
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
  cudaSetDevice(s->h->device);
  for (auto& slp : s->slots) {
    Slot& sl = *slp;
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    for (auto& b : sl.din) b.release();
    for (auto& b : sl.dout) b.release();
    sl.ctx.release();
    if (sl.pinIn) cudaFreeHost(sl.pinIn);
    if (sl.pinOut) cudaFreeHost(sl.pinOut);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  delete s;
  return CK_OK;
}

}  // extern "C"
