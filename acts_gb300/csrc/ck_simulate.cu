// ck_simulate.cu — ck_simulate: truth simulation and digitisation of
// generated tracks on the device (the Fatras-like kick-and-smear of
// ck_simulate.h, the same source the host generator runs), through the
// handle's surface table and field, into device memory in the layout of the
// generator's ckg_out (compact CSR rows with their offsets).
//
// Three launches: one thread per track simulates it into rows of fixed
// capacity in device scratch (its header outputs go straight to `out`);
// one block scans the row lengths into the CSR offsets; one thread per
// track copies its rows to their compact place.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "ck_api_internal.h"
#include "ck_simulate.h"

using namespace ck;

namespace {

constexpr int kSimBlock = 128;
constexpr int kScanThreads = 1024;

// rows of one track at capacity positions [t * cap, t * cap + cap)
struct SimRows {
  int32_t* seq;
  int32_t* msurf;
  int32_t* msub;
  double* mval;   // 2 per measurement
  double* mcov;   // 4
  double* truth;  // 6
  uint8_t* outl;
  int32_t* nseq;  // [n] rows written (capped)
  int32_t* nmeas;
};

// the simulation's sink on the device: rows beyond the capacity are
// dropped, as the host generator truncates them
struct DeviceSink {
  const SimRows* r;
  size_t base;
  int cap, ns, nm;
  __device__ void onSurface(int sid) {
    if (ns < cap) r->seq[base + ns] = sid;
    ++ns;
  }
  __device__ void onMeasurement(int sid, int sub, const double* val, const double* cov,
                                const double* tr, bool outl) {
    if (nm < cap) {
      const size_t i = base + nm;
      r->msurf[i] = sid;
      r->msub[i] = sub;
      for (int c = 0; c < 2; ++c) r->mval[2 * i + c] = val[c];
      for (int c = 0; c < 4; ++c) r->mcov[4 * i + c] = cov[c];
      for (int c = 0; c < 6; ++c) r->truth[6 * i + c] = tr[c];
      r->outl[i] = outl ? 1 : 0;
    }
    ++nm;
  }
};

struct SimParams {
  int preset;
  uint64_t seed;
  long long first;
  int n, cap;
  const ck_surface* surf;
  int nSurf;
  cks::FieldEval F;
  SimRows rows;
  ckg_out out;  // device pointers
};

__global__ void __launch_bounds__(kSimBlock) simulateKernel(SimParams sp) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= sp.n) return;
  cks::TrackHeader hd;
  DeviceSink sink{&sp.rows, (size_t)t * sp.cap, sp.cap, 0, 0};
  cks::simulateTrack(sp.preset, sp.seed, sp.first + t, sp.surf, sp.nSurf, sp.F, hd, sink);
  sp.rows.nseq[t] = sink.ns < sp.cap ? sink.ns : sp.cap;
  sp.rows.nmeas[t] = sink.nm < sp.cap ? sink.nm : sp.cap;
  const ckg_out& o = sp.out;
  for (int c = 0; c < 6; ++c) o.start_params[6 * (size_t)t + c] = hd.startParams[c];
  for (int c = 0; c < 36; ++c) o.start_cov[36 * (size_t)t + c] = hd.startCov[c];
  for (int c = 0; c < 12; ++c) o.start_frames[12 * (size_t)t + c] = hd.frame[c];
  if (o.truth_start)
    for (int c = 0; c < 6; ++c) o.truth_start[6 * (size_t)t + c] = hd.truthStart[c];
  o.particle[2 * (size_t)t] = hd.particle[0];
  o.particle[2 * (size_t)t + 1] = hd.particle[1];
  o.particle_pdg[t] = hd.pdg;
}

// exclusive scans of the row lengths into the CSR offsets, in chunks of
// the block's size with a running carry (one block)
__global__ void __launch_bounds__(kScanThreads) scanKernel(const int32_t* __restrict__ ns,
                                                           const int32_t* __restrict__ nm, int n,
                                                           int32_t* __restrict__ seqOff,
                                                           int32_t* __restrict__ measOff) {
  __shared__ int32_t a[kScanThreads], b[kScanThreads];
  __shared__ int32_t carryA, carryB;
  const int tid = threadIdx.x;
  if (tid == 0) {
    carryA = carryB = 0;
    seqOff[0] = 0;
    measOff[0] = 0;
  }
  __syncthreads();
  for (int base = 0; base < n; base += kScanThreads) {
    const int i = base + tid;
    a[tid] = i < n ? ns[i] : 0;
    b[tid] = i < n ? nm[i] : 0;
    __syncthreads();
    // Hillis-Steele inclusive scan
    for (int d = 1; d < kScanThreads; d <<= 1) {
      const int va = tid >= d ? a[tid - d] : 0;
      const int vb = tid >= d ? b[tid - d] : 0;
      __syncthreads();
      a[tid] += va;
      b[tid] += vb;
      __syncthreads();
    }
    if (i < n) {
      seqOff[i + 1] = carryA + a[tid];
      measOff[i + 1] = carryB + b[tid];
    }
    __syncthreads();
    if (tid == kScanThreads - 1) {
      carryA += a[tid];
      carryB += b[tid];
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kSimBlock) compactKernel(SimParams sp) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= sp.n) return;
  const ckg_out& o = sp.out;
  const SimRows& r = sp.rows;
  const size_t src = (size_t)t * sp.cap;
  const int ns = r.nseq[t], nm = r.nmeas[t];
  const size_t ds = o.seq_offsets[t], dm = o.meas_offsets[t];
  for (int k = 0; k < ns; ++k) o.seq_surfaces[ds + k] = r.seq[src + k];
  for (int k = 0; k < nm; ++k) {
    const size_t i = src + k, j = dm + k;
    o.meas_surfaces[j] = r.msurf[i];
    for (int c = 0; c < 2; ++c) o.meas_values[2 * j + c] = r.mval[2 * i + c];
    for (int c = 0; c < 4; ++c) o.meas_cov[4 * j + c] = r.mcov[4 * i + c];
    if (o.truth_meas)
      for (int c = 0; c < 6; ++c) o.truth_meas[6 * j + c] = r.truth[6 * i + c];
    if (o.meas_outlier) o.meas_outlier[j] = r.outl[i];
    if (o.meas_subspace) o.meas_subspace[j] = r.msub[i];
  }
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

extern "C" ck_status ck_simulate(ck_handle* h, int32_t preset, uint64_t seed, int64_t first_track,
                                 int32_t n_tracks, ckg_out* out, void* stream) {
  if (!h || !out) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  if (n_tracks < 0 || first_track < 0) return fail(CK_ERR_INVALID_ARGUMENT, "negative count");
  const int base = cks::basePreset(preset);
  if (base != CKG_TELESCOPE && base != CKG_BARREL && base != CKG_BARREL_MIXED &&
      base != CKG_UNEVEN && base != CKG_SERVING)
    return fail(CK_ERR_INVALID_ARGUMENT, "unknown preset");
  const int cap = out->max_per_track;
  if (cap < 1) return fail(CK_ERR_INVALID_ARGUMENT, "max_per_track < 1");
  if (!out->seq_offsets || !out->seq_surfaces || !out->meas_offsets || !out->meas_surfaces ||
      !out->meas_values || !out->meas_cov || !out->start_params || !out->start_cov ||
      !out->start_frames || !out->particle || !out->particle_pdg)
    return fail(CK_ERR_INVALID_ARGUMENT, "a required output array is NULL");
  std::lock_guard<std::mutex> lock(h->mu);
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return cudaFail(e, "set device");
  cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
  // the surface table as the simulation reads it (ck_surface), once per handle
  if (!h->dGenSurfaces && h->nSurfaces > 0) {
    if ((e = cudaMalloc(&h->dGenSurfaces, sizeof(ck_surface) * h->nSurfaces)) != cudaSuccess ||
        (e = cudaMemcpy(h->dGenSurfaces, h->hostSurfaces.data(),
                        sizeof(ck_surface) * h->nSurfaces, cudaMemcpyHostToDevice)) !=
            cudaSuccess)
      return cudaFail(e, "surface table upload");
  }
  if (n_tracks == 0) {
    const int32_t zero = 0;
    cudaMemcpyAsync(out->seq_offsets, &zero, 4, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(out->meas_offsets, &zero, 4, cudaMemcpyHostToDevice, st);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cudaFail(e, "simulation");
    return CK_OK;
  }
  const size_t n = (size_t)n_tracks, rowsN = n * (size_t)cap;
  const size_t parts[] = {4 * rowsN, 4 * rowsN, 4 * rowsN, 16 * rowsN, 32 * rowsN,
                          48 * rowsN, rowsN, 4 * n, 4 * n};
  size_t total = 0;
  for (size_t b : parts) total += align256(b);
  if ((e = h->unitBuf.ensure(total)) != cudaSuccess) return cudaFail(e, "simulation scratch");
  char* p = (char*)h->unitBuf.p;
  void* ptrs[9];
  for (int i = 0; i < 9; ++i) {
    ptrs[i] = p;
    p += align256(parts[i]);
  }
  SimParams sp;
  std::memset(&sp, 0, sizeof(sp));
  sp.preset = preset;
  sp.seed = seed;
  sp.first = first_track;
  sp.n = n_tracks;
  sp.cap = cap;
  sp.surf = (const ck_surface*)h->dGenSurfaces;
  sp.nSurf = h->nSurfaces;
  const ck_field& f = h->hostField;
  sp.F.kind = f.kind;
  for (int i = 0; i < 3; ++i) sp.F.b[i] = f.constant_tesla[i];
  if (f.kind == CK_FIELD_GRID_XYZ) {
    for (int i = 0; i < 3; ++i) {
      sp.F.n[i] = f.n[i];
      sp.F.mn[i] = f.min[i];
      sp.F.step[i] = (f.max[i] - f.min[i]) / (sp.F.n[i] - 1);
    }
    sp.F.v = reinterpret_cast<const float*>(h->dNodes);  // float4 nodes
    sp.F.stride = 4;
  }
  sp.rows.seq = (int32_t*)ptrs[0];
  sp.rows.msurf = (int32_t*)ptrs[1];
  sp.rows.msub = (int32_t*)ptrs[2];
  sp.rows.mval = (double*)ptrs[3];
  sp.rows.mcov = (double*)ptrs[4];
  sp.rows.truth = (double*)ptrs[5];
  sp.rows.outl = (uint8_t*)ptrs[6];
  sp.rows.nseq = (int32_t*)ptrs[7];
  sp.rows.nmeas = (int32_t*)ptrs[8];
  sp.out = *out;
  const int grid = (int)((n + kSimBlock - 1) / kSimBlock);
  simulateKernel<<<grid, kSimBlock, 0, st>>>(sp);
  scanKernel<<<1, kScanThreads, 0, st>>>(sp.rows.nseq, sp.rows.nmeas, n_tracks, out->seq_offsets,
                                         out->meas_offsets);
  compactKernel<<<grid, kSimBlock, 0, st>>>(sp);
  if ((e = cudaGetLastError()) != cudaSuccess) return cudaFail(e, "simulation launch");
  h->lastLaunches = 3;
  return CK_OK;
}
