// ck_static.cu — ck_fit_batch_static: the batch fit of a device-resident
// batch whose pipeline scratch (track-state records, work-queue permutation,
// tips, queue ticket) lives in one statically sized device array of this
// translation unit instead of the handle's grow-only allocations.
//
// Who needs it: a caller inside a latency-critical loop that reserves all of
// its device memory when it starts and must not touch the allocator while it
// runs — for instance an online event filter. cudaMalloc and cudaFree can
// synchronise the device and stall every other stream, and the handle's
// buffers are reallocated whenever a batch is larger than any before it, so
// ck_fit_batch can allocate at an unpredictable moment. This entry point
// performs no device or host allocation of its own.
//
// Rules of use:
//   - inputs and outputs must already be in device memory;
//   - the scratch holds kStaticScratchBytes (32 MiB); a batch that needs more
//     (ck_static_scratch_bytes_for gives the exact figure for a call's
//     options) is rejected with CK_ERR_SCRATCH_LIMIT;
//   - nothing in the scratch has to start at zero: every call clears the
//     queue ticket itself and writes the length histograms, each track's tip
//     and its records before reading them;
//   - there is one array per device, shared by every handle of this library
//     on that device: calls whose work overlaps on the device (different
//     streams, or different handles, without ordering between them) race on
//     it; order them on one stream or wait between them;
//   - the first call on a device resolves the array's address
//     (cudaGetSymbolAddress), which may load this module: make the first call
//     before the caller starts capturing its stream.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "ck_api_internal.h"
#include "ck_launch.h"

using namespace ck;

namespace {

constexpr size_t kStaticScratchBytes = size_t(32) << 20;
constexpr size_t kAlign = 256;
constexpr size_t kTicketBytes = 256;  // the queue and tail-smoothing tickets
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_staticScratch[kStaticScratchBytes];

std::mutex g_symbolMutex;
void* g_symbolAddress[kMaxDevices] = {};

size_t roundUp(size_t b) { return (b + kAlign - 1) & ~(kAlign - 1); }

// Scratch layout for n tracks of up to maxStates states.
struct Layout {
  size_t rec, perm, tip, sortCounts, ticket, smoothed, ext, total;
};

// ext: the extrapolation start states (only with a reference surface)
Layout layoutFor(int n, int maxStates, int precision, bool ext) {
  const size_t ns = (size_t)n * (size_t)maxStates;
  Layout l;
  l.rec = roundUp(ns * recordStateBytes(precision));
  l.perm = roundUp((size_t)n * sizeof(int32_t));
  l.tip = roundUp((size_t)n * sizeof(int32_t));
  l.sortCounts = roundUp(sortCountsBytes(n));
  l.ticket = kTicketBytes;
  l.smoothed = roundUp((size_t)n);
  l.ext = ext ? roundUp((size_t)n * 2 * sizeof(ExtStart)) : 0;
  l.total = l.rec + l.perm + l.tip + l.sortCounts + l.ticket + l.smoothed + l.ext;
  return l;
}

// Address of the array on the current device (resolved once per device).
ck_status scratchAddress(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices)
    return fail(CK_ERR_INVALID_ARGUMENT, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_symbolMutex);
  if (!g_symbolAddress[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_staticScratch);
    if (e != cudaSuccess) return cudaFail(e, "static scratch address");
    g_symbolAddress[device] = p;
  }
  *out = static_cast<unsigned char*>(g_symbolAddress[device]);
  return CK_OK;
}

}  // namespace

extern "C" {

int64_t ck_static_scratch_bytes(int32_t n_tracks, int32_t max_states, int32_t precision) {
  if (n_tracks < 0 || max_states <= 0) return -1;
  return (int64_t)layoutFor(n_tracks, max_states, precision, false).total;
}

int64_t ck_static_scratch_bytes_for(const ck_options* opt, int32_t n_tracks, int32_t max_states) {
  if (!opt || n_tracks < 0 || max_states <= 0) return -1;
  if (validateOptions(opt) != CK_OK) return -1;
  return (int64_t)layoutFor(n_tracks, max_states, opt->precision, needsExtStart(*opt)).total;
}

int64_t ck_static_scratch_capacity(void) { return (int64_t)kStaticScratchBytes; }

ck_status ck_fit_batch_static(ck_handle* h, const ck_options* opt, const ck_batch_in* in,
                              ck_batch_out* out, void* stream) {
  if (!h || !in || !out) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  ck_status vs = validateOptions(opt);
  if (vs != CK_OK) return vs;
  if ((vs = validateReference(h, opt)) != CK_OK) return vs;
  if (in->memory != CK_MEM_DEVICE || out->memory != CK_MEM_DEVICE)
    return fail(CK_ERR_INVALID_ARGUMENT,
                "ck_fit_batch_static takes device-resident inputs and outputs only");
  if (in->n_tracks < 0) return fail(CK_ERR_INVALID_ARGUMENT, "n_tracks < 0");
  if (out->max_states <= 0) return fail(CK_ERR_INVALID_ARGUMENT, "max_states <= 0");
  if (!out->status) return fail(CK_ERR_INVALID_ARGUMENT, "status array is required");
  if ((out->predicted && !out->predicted_cov) || (out->filtered && !out->filtered_cov) ||
      (out->smoothed && !out->smoothed_cov))
    return fail(CK_ERR_INVALID_ARGUMENT, "parameter arrays need their covariance arrays");
  const int n = in->n_tracks;
  const Layout l = layoutFor(n, out->max_states, opt->precision, needsExtStart(*opt));
  if (l.total > kStaticScratchBytes)
    return fail(CK_ERR_SCRATCH_LIMIT,
                "batch needs " + std::to_string(l.total) + " bytes of scratch; the static scratch "
                "holds " + std::to_string(kStaticScratchBytes) + " (use ck_fit_batch, or split it)");
  std::lock_guard<std::mutex> lock(h->mu);
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return cudaFail(e, "set device");
  unsigned char* base = nullptr;
  ck_status s = scratchAddress(h->device, &base);
  if (s != CK_OK) return s;
  // the pipeline's scratch views into the array (never grown or freed)
  FitContext c;
  size_t off = 0;
  auto view = [&](DevBuf& b, size_t bytes) {
    b.p = base + off;
    b.cap = bytes;
    off += bytes;
  };
  view(c.rec, l.rec);
  view(c.perm, l.perm);
  view(c.tip, l.tip);
  view(c.sortCounts, l.sortCounts);
  view(c.ticket, l.ticket);
  view(c.smoothed, l.smoothed);
  if (l.ext) view(c.ext, l.ext);
  cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
  const Tune tn = h->tune[opt->precision];
  h->lastH2D = 0;
  h->lastD2H = 0;
  s = enqueuePipeline(h, c, *opt, *in, *out, tn, st, false, gridBlocksFor(h, tn));
  if (s != CK_OK) return s;
  // (launch errors of the pipeline's memsets and kernels)
  if ((e = cudaGetLastError()) != cudaSuccess) return cudaFail(e, "batch pipeline");
  return CK_OK;
}

}  // extern "C"
