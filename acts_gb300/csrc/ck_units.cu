// ck_units.cu — batched unit operators of the fitter exposed through the C
// ABI: the GainMatrixUpdater, the GainMatrixSmoother, the pointwise material
// effects and the field lookup, each as its own kernel over a batch. They run
// the same device functions the fit kernel uses, so the reference's unit
// known-answer tests can be replayed on the GPU.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "ck_api_internal.h"
#include "ck_device.cuh"

using namespace ck;

namespace {

__global__ void updateKernel(int n, int joseph, const double* __restrict__ pred,
                             const double* __restrict__ predCov, const double* __restrict__ meas,
                             const double* __restrict__ measCov,
                             const int32_t* __restrict__ sub, double* filt, double* filtCov,
                             double* chi2, int32_t* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double p[6], P[21], V[4], f[6], F[21], c2 = 0.0;
  for (int k = 0; k < 6; ++k) p[k] = pred[6 * i + k];
  for (int r = 0; r < 6; ++r)
    for (int c = r; c < 6; ++c) P[sidx(r, c)] = predCov[36 * i + r * 6 + c];
  for (int k = 0; k < 4; ++k) V[k] = measCov[4 * i + k];
  const int s = sub ? sub[i] : CK_MEAS_LOC01;
  const bool ok =
      kalmanUpdateSub(p, P, s, meas[2 * i], meas[2 * i + 1], V, joseph != 0, f, F, c2);
  status[i] = ok ? CK_TRACK_OK : CK_TRACK_UPDATE_FAILED;
  if (!ok) return;
  for (int k = 0; k < 6; ++k) filt[6 * i + k] = f[k];
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) filtCov[36 * i + r * 6 + c] = F[sidx(r, c)];
  chi2[i] = c2;
}

__global__ void atan2Kernel(int n, const double* __restrict__ y, const double* __restrict__ x,
                            const double2* __restrict__ tab, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = atan2Table(y[i], x[i], tab);
}

__global__ void smoothKernel(int nTraj, int nStates, const double* __restrict__ pred,
                             const double* __restrict__ predCov, const double* __restrict__ filt,
                             const double* __restrict__ filtCov, const double* __restrict__ jac,
                             double* smth, double* smthCov, int32_t* status) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nTraj) return;
  const size_t b = (size_t)t * nStates;
  const int last = nStates - 1;
  double ps[6], Psp[21];
  for (int k = 0; k < 6; ++k) ps[k] = filt[6 * (b + last) + k];
  for (int r = 0; r < 6; ++r)
    for (int c = r; c < 6; ++c) Psp[sidx(r, c)] = filtCov[36 * (b + last) + r * 6 + c];
  for (int k = 0; k < 6; ++k) smth[6 * (b + last) + k] = ps[k];
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) smthCov[36 * (b + last) + r * 6 + c] = Psp[sidx(r, c)];
  status[t] = CK_TRACK_OK;
  for (int k = last - 1; k >= 0; --k) {
    double f[6], Pf[21], pp[6], Ppp[21], J[36], sm[6], Ps[21];
    for (int i = 0; i < 6; ++i) f[i] = filt[6 * (b + k) + i];
    for (int r = 0; r < 6; ++r)
      for (int c = r; c < 6; ++c) Pf[sidx(r, c)] = filtCov[36 * (b + k) + r * 6 + c];
    for (int i = 0; i < 6; ++i) pp[i] = pred[6 * (b + k + 1) + i];
    for (int r = 0; r < 6; ++r)
      for (int c = r; c < 6; ++c) Ppp[sidx(r, c)] = predCov[36 * (b + k + 1) + r * 6 + c];
    for (int i = 0; i < 36; ++i) J[i] = jac[36 * (b + k + 1) + i];
    if (!smoothStep(f, Pf, pp, Ppp, J, ps, Psp, sm, Ps)) {
      status[t] = CK_TRACK_SMOOTH_FAILED;
      return;
    }
    for (int i = 0; i < 6; ++i) smth[6 * (b + k) + i] = sm[i];
    for (int r = 0; r < 6; ++r)
      for (int c = 0; c < 6; ++c) smthCov[36 * (b + k) + r * 6 + c] = Ps[sidx(r, c)];
    for (int i = 0; i < 6; ++i) ps[i] = sm[i];
    for (int i = 0; i < 21; ++i) Psp[i] = Ps[i];
  }
}

// MbfSmoother on whole trajectories (FP64): state k's flags select the
// measurement visit; its Jacobian carries the lambdas to state k-1.
__global__ void mbfKernel(int nTraj, int nStates, const uint32_t* __restrict__ flags,
                          const double* __restrict__ pred, const double* __restrict__ predCov,
                          const double* __restrict__ filt, const double* __restrict__ filtCov,
                          const double* __restrict__ jac, const double* __restrict__ meas,
                          const double* __restrict__ measCov, double* smth, double* smthCov) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nTraj) return;
  const size_t b = (size_t)t * nStates;
  double L[21], l[6];
  for (int i = 0; i < 21; ++i) L[i] = 0.0;
  for (int i = 0; i < 6; ++i) l[i] = 0.0;
  for (int k = nStates - 1; k >= 0; --k) {
    const size_t s = b + k;
    double f[6], Pf[21], sm[6], Ps[21];
    for (int i = 0; i < 6; ++i) f[i] = filt[6 * s + i];
    for (int r = 0; r < 6; ++r)
      for (int c = r; c < 6; ++c) Pf[sidx(r, c)] = filtCov[36 * s + r * 6 + c];
    mbfSmoothed<double>(f, Pf, L, l, false, sm, Ps);
    for (int i = 0; i < 6; ++i) smth[6 * s + i] = sm[i];
    for (int r = 0; r < 6; ++r)
      for (int c = 0; c < 6; ++c) smthCov[36 * s + r * 6 + c] = Ps[sidx(r, c)];
    if (k == 0) break;
    const uint32_t fl = flags[s];
    if ((fl & CK_FLAG_HAS_MEASUREMENT) && !(fl & CK_FLAG_IS_OUTLIER)) {
      double p[6], Pp[21], V[4];
      for (int i = 0; i < 6; ++i) p[i] = pred[6 * s + i];
      for (int r = 0; r < 6; ++r)
        for (int c = r; c < 6; ++c) Pp[sidx(r, c)] = predCov[36 * s + r * 6 + c];
      for (int i = 0; i < 4; ++i) V[i] = measCov[4 * s + i];
      mbfMeasurement<double>(p, Pp, meas[2 * s], meas[2 * s + 1], V, L, l);
    }
    mbfTransport<double>(jac + 36 * s, L, l);
  }
}

__global__ void materialKernel(int n, MatConst mc, const DevSurface* __restrict__ surf,
                               const int32_t* __restrict__ sid, const float* __restrict__ scale,
                               const double* __restrict__ dir, const double* __restrict__ qop,
                               const float* __restrict__ mass, const float* __restrict__ absQ,
                               const int32_t* __restrict__ pdg, int ms, int el, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d[3] = {dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]};
  bool vac = false;
  MatEffects e = materialEffects<double>(mc, surf + sid[i], 1.0f, scale[i], pdg[i], mass[i],
                                         absQ[i], d, (float)qop[i], ms != 0, el != 0, vac);
  out[4 * i + 0] = e.eLoss;
  out[4 * i + 1] = e.varPhi;
  out[4 * i + 2] = e.varTheta;
  out[4 * i + 3] = e.varQoP;
}

// getField in the stepper scalar P: the positions rounded to P as the
// Runge-Kutta stages round them (FP32 in the mixed form)
template <typename P>
__global__ void fieldKernel(int n, DevField F, const double* __restrict__ pos, double* out,
                            int32_t* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const P p[3] = {toP<P>(pos[3 * i]), toP<P>(pos[3 * i + 1]), toP<P>(pos[3 * i + 2])};
  P B[3] = {0, 0, 0};
  const bool ok = getField(F, p, B);
  status[i] = ok ? 0 : CK_TRACK_FIELD_OUT_OF_BOUNDS;
  for (int c = 0; c < 3; ++c) out[3 * i + c] = ok ? (double)B[c] : 0.0;
}

// Scratch arena for one synchronous unit call.
struct Arena {
  ck_handle* h;
  size_t used = 0;
  std::vector<std::pair<size_t, size_t>> parts;
  char* base = nullptr;
  void* add(size_t bytes) {
    size_t off = (used + 255) & ~(size_t)255;
    used = off + bytes;
    parts.push_back({off, bytes});
    return (void*)off;
  }
  cudaError_t commit() {
    cudaError_t e = h->unitBuf.ensure(used);
    base = (char*)h->unitBuf.p;
    return e;
  }
  template <typename T>
  T* at(void* tag) {
    return (T*)(base + (size_t)tag);
  }
};

}  // namespace

extern "C" {

ck_status ck_gain_matrix_update(ck_handle* h, int32_t n, int32_t use_joseph,
                                const double* predicted, const double* predicted_cov,
                                const double* meas, const double* meas_cov,
                                const int32_t* subspace, double* filtered,
                                double* filtered_cov, double* chi2, int32_t* status) {
  if (!h || n < 0 || !predicted || !predicted_cov || !meas || !meas_cov || !filtered ||
      !filtered_cov || !chi2 || !status)
    return fail(CK_ERR_INVALID_ARGUMENT, "bad argument");
  if (subspace)
    for (int i = 0; i < n; ++i)
      if (subspace[i] < CK_MEAS_LOC0 || subspace[i] > CK_MEAS_LOC01)
        return fail(CK_ERR_INVALID_ARGUMENT, "unknown measurement subspace");
  if (n == 0) return CK_OK;
  std::lock_guard<std::mutex> lock(h->mu);
  cudaSetDevice(h->device);
  Arena a{h};
  void* tP = a.add(48 * n);
  void* tPC = a.add(288 * n);
  void* tM = a.add(16 * n);
  void* tMC = a.add(32 * n);
  void* tF = a.add(48 * n);
  void* tFC = a.add(288 * n);
  void* tC = a.add(8 * n);
  void* tS = a.add(4 * n);
  void* tSub = a.add(4 * n);
  cudaError_t e = a.commit();
  if (e != cudaSuccess) return cudaFail(e, "unit buffer");
  cudaStream_t st = h->stream;
  cudaMemcpyAsync(a.at<double>(tP), predicted, 48 * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tPC), predicted_cov, 288 * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tM), meas, 16 * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tMC), meas_cov, 32 * n, cudaMemcpyHostToDevice, st);
  if (subspace) cudaMemcpyAsync(a.at<int32_t>(tSub), subspace, 4 * n, cudaMemcpyHostToDevice, st);
  updateKernel<<<(n + 127) / 128, 128, 0, st>>>(
      n, use_joseph, a.at<double>(tP), a.at<double>(tPC), a.at<double>(tM), a.at<double>(tMC),
      subspace ? a.at<int32_t>(tSub) : nullptr, a.at<double>(tF), a.at<double>(tFC),
      a.at<double>(tC), a.at<int32_t>(tS));
  cudaMemcpyAsync(filtered, a.at<double>(tF), 48 * n, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(filtered_cov, a.at<double>(tFC), 288 * n, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(chi2, a.at<double>(tC), 8 * n, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(status, a.at<int32_t>(tS), 4 * n, cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cudaFail(e, "update kernel");
  h->lastLaunches = 1;
  return CK_OK;
}

ck_status ck_gain_matrix_smooth(ck_handle* h, int32_t n_traj, int32_t n_states,
                                const double* predicted, const double* predicted_cov,
                                const double* filtered, const double* filtered_cov,
                                const double* jacobian, double* smoothed, double* smoothed_cov,
                                int32_t* status) {
  if (!h || n_traj < 0 || n_states < 1 || !predicted || !predicted_cov || !filtered ||
      !filtered_cov || !jacobian || !smoothed || !smoothed_cov || !status)
    return fail(CK_ERR_INVALID_ARGUMENT, "bad argument");
  if (n_traj == 0) return CK_OK;
  std::lock_guard<std::mutex> lock(h->mu);
  cudaSetDevice(h->device);
  const size_t m = (size_t)n_traj * n_states;
  Arena a{h};
  void* tP = a.add(48 * m);
  void* tPC = a.add(288 * m);
  void* tF = a.add(48 * m);
  void* tFC = a.add(288 * m);
  void* tJ = a.add(288 * m);
  void* tS = a.add(48 * m);
  void* tSC = a.add(288 * m);
  void* tSt = a.add(4 * (size_t)n_traj);
  cudaError_t e = a.commit();
  if (e != cudaSuccess) return cudaFail(e, "unit buffer");
  cudaStream_t st = h->stream;
  cudaMemcpyAsync(a.at<double>(tP), predicted, 48 * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tPC), predicted_cov, 288 * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tF), filtered, 48 * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tFC), filtered_cov, 288 * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tJ), jacobian, 288 * m, cudaMemcpyHostToDevice, st);
  smoothKernel<<<(n_traj + 127) / 128, 128, 0, st>>>(
      n_traj, n_states, a.at<double>(tP), a.at<double>(tPC), a.at<double>(tF), a.at<double>(tFC),
      a.at<double>(tJ), a.at<double>(tS), a.at<double>(tSC), a.at<int32_t>(tSt));
  cudaMemcpyAsync(smoothed, a.at<double>(tS), 48 * m, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(smoothed_cov, a.at<double>(tSC), 288 * m, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(status, a.at<int32_t>(tSt), 4 * (size_t)n_traj, cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cudaFail(e, "smooth kernel");
  h->lastLaunches = 1;
  return CK_OK;
}

ck_status ck_mbf_smooth(ck_handle* h, int32_t n_traj, int32_t n_states, const uint32_t* flags,
                        const double* predicted, const double* predicted_cov,
                        const double* filtered, const double* filtered_cov,
                        const double* jacobian, const double* measurement,
                        const double* measurement_cov, double* smoothed, double* smoothed_cov) {
  if (!h || n_traj < 0 || n_states < 1 || !flags || !predicted || !predicted_cov || !filtered ||
      !filtered_cov || !jacobian || !measurement || !measurement_cov || !smoothed ||
      !smoothed_cov)
    return fail(CK_ERR_INVALID_ARGUMENT, "bad argument");
  if (n_traj == 0) return CK_OK;
  std::lock_guard<std::mutex> lock(h->mu);
  cudaSetDevice(h->device);
  const size_t m = (size_t)n_traj * n_states;
  Arena a{h};
  void* tFl = a.add(4 * m);
  void* tP = a.add(48 * m);
  void* tPC = a.add(288 * m);
  void* tF = a.add(48 * m);
  void* tFC = a.add(288 * m);
  void* tJ = a.add(288 * m);
  void* tM = a.add(16 * m);
  void* tMC = a.add(32 * m);
  void* tS = a.add(48 * m);
  void* tSC = a.add(288 * m);
  cudaError_t e = a.commit();
  if (e != cudaSuccess) return cudaFail(e, "unit buffer");
  cudaStream_t st = h->stream;
  cudaMemcpyAsync(a.at<uint32_t>(tFl), flags, 4 * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tP), predicted, 48 * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tPC), predicted_cov, 288 * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tF), filtered, 48 * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tFC), filtered_cov, 288 * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tJ), jacobian, 288 * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tM), measurement, 16 * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tMC), measurement_cov, 32 * m, cudaMemcpyHostToDevice, st);
  mbfKernel<<<(n_traj + 127) / 128, 128, 0, st>>>(
      n_traj, n_states, a.at<uint32_t>(tFl), a.at<double>(tP), a.at<double>(tPC),
      a.at<double>(tF), a.at<double>(tFC), a.at<double>(tJ), a.at<double>(tM),
      a.at<double>(tMC), a.at<double>(tS), a.at<double>(tSC));
  cudaMemcpyAsync(smoothed, a.at<double>(tS), 48 * m, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(smoothed_cov, a.at<double>(tSC), 288 * m, cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cudaFail(e, "mbf kernel");
  h->lastLaunches = 1;
  return CK_OK;
}

ck_status ck_material_effects(ck_handle* h, int32_t n, const int32_t* surface,
                              const float* thickness_scale, const double* direction,
                              const double* qop, const float* mass, const float* abs_q,
                              const int32_t* pdg, int32_t multiple_scattering,
                              int32_t energy_loss, double* effects) {
  if (!h || n < 0 || !surface || !thickness_scale || !direction || !qop || !mass || !abs_q ||
      !pdg || !effects)
    return fail(CK_ERR_INVALID_ARGUMENT, "bad argument");
  if (n == 0) return CK_OK;
  for (int i = 0; i < n; ++i)
    if (surface[i] < 0 || surface[i] >= h->nSurfaces)
      return fail(CK_ERR_INVALID_ARGUMENT, "surface id out of range");
  std::lock_guard<std::mutex> lock(h->mu);
  cudaSetDevice(h->device);
  Arena a{h};
  void* tSid = a.add(4 * n);
  void* tSc = a.add(4 * n);
  void* tDir = a.add(24 * n);
  void* tQ = a.add(8 * n);
  void* tM = a.add(4 * n);
  void* tA = a.add(4 * n);
  void* tPdg = a.add(4 * n);
  void* tOut = a.add(32 * n);
  cudaError_t e = a.commit();
  if (e != cudaSuccess) return cudaFail(e, "unit buffer");
  cudaStream_t st = h->stream;
  cudaMemcpyAsync(a.at<int32_t>(tSid), surface, 4 * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<float>(tSc), thickness_scale, 4 * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tDir), direction, 24 * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tQ), qop, 8 * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<float>(tM), mass, 4 * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<float>(tA), abs_q, 4 * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<int32_t>(tPdg), pdg, 4 * n, cudaMemcpyHostToDevice, st);
  materialKernel<<<(n + 127) / 128, 128, 0, st>>>(
      n, h->mc, h->dSurfaces, a.at<int32_t>(tSid), a.at<float>(tSc), a.at<double>(tDir),
      a.at<double>(tQ), a.at<float>(tM), a.at<float>(tA), a.at<int32_t>(tPdg),
      multiple_scattering, energy_loss, a.at<double>(tOut));
  cudaMemcpyAsync(effects, a.at<double>(tOut), 32 * n, cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cudaFail(e, "material kernel");
  h->lastLaunches = 1;
  return CK_OK;
}

ck_status ck_atan2_mixed(ck_handle* h, int32_t n, const double* y, const double* x,
                         double* out) {
  if (!h || n < 0 || !y || !x || !out) return fail(CK_ERR_INVALID_ARGUMENT, "bad argument");
  if (n == 0) return CK_OK;
  std::lock_guard<std::mutex> lock(h->mu);
  cudaSetDevice(h->device);
  Arena a{h};
  void* tY = a.add(8 * n);
  void* tX = a.add(8 * n);
  void* tO = a.add(8 * n);
  cudaError_t e = a.commit();
  if (e != cudaSuccess) return cudaFail(e, "unit buffer");
  cudaStream_t st = h->stream;
  cudaMemcpyAsync(a.at<double>(tY), y, 8 * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(a.at<double>(tX), x, 8 * n, cudaMemcpyHostToDevice, st);
  atan2Kernel<<<(n + 127) / 128, 128, 0, st>>>(n, a.at<double>(tY), a.at<double>(tX), h->dTrig,
                                               a.at<double>(tO));
  cudaMemcpyAsync(out, a.at<double>(tO), 8 * n, cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cudaFail(e, "atan2 kernel");
  h->lastLaunches = 1;
  return CK_OK;
}

ck_status ck_field_lookup(ck_handle* h, int32_t n, const double* pos, double* out,
                          int32_t* status) {
  return ck_field_lookup_precision(h, CK_PRECISION_FP64, n, pos, out, status);
}

ck_status ck_field_lookup_precision(ck_handle* h, int32_t precision, int32_t n, const double* pos,
                                    double* out, int32_t* status) {
  if (!h || n < 0 || !pos || !out || !status) return fail(CK_ERR_INVALID_ARGUMENT, "bad argument");
  if (precision != CK_PRECISION_FP64 && precision != CK_PRECISION_MIXED)
    return fail(CK_ERR_INVALID_ARGUMENT, "unknown precision");
  if (n == 0) return CK_OK;
  std::lock_guard<std::mutex> lock(h->mu);
  cudaSetDevice(h->device);
  Arena a{h};
  void* tP = a.add(24 * n);
  void* tO = a.add(24 * n);
  void* tS = a.add(4 * n);
  cudaError_t e = a.commit();
  if (e != cudaSuccess) return cudaFail(e, "unit buffer");
  cudaStream_t st = h->stream;
  cudaMemcpyAsync(a.at<double>(tP), pos, 24 * n, cudaMemcpyHostToDevice, st);
  if (precision == CK_PRECISION_FP64)
    fieldKernel<double><<<(n + 127) / 128, 128, 0, st>>>(n, h->field, a.at<double>(tP),
                                                         a.at<double>(tO), a.at<int32_t>(tS));
  else
    fieldKernel<float><<<(n + 127) / 128, 128, 0, st>>>(n, h->field, a.at<double>(tP),
                                                        a.at<double>(tO), a.at<int32_t>(tS));
  cudaMemcpyAsync(out, a.at<double>(tO), 24 * n, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(status, a.at<int32_t>(tS), 4 * n, cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cudaFail(e, "field kernel");
  h->lastLaunches = 1;
  return CK_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Arithmetic-pipe peak probes: independent FMA chains per thread, timed with
// CUDA events; the roofline denominators of the FP64 / FP32 fit kernels.
namespace {

template <typename T>
__global__ void fmaPeakKernel(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
  T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      x0 = fma(x0, a, b);
      x1 = fma(x1, a, b);
      x2 = fma(x2, a, b);
      x3 = fma(x3, a, b);
      x4 = fma(x4, a, b);
      x5 = fma(x5, a, b);
      x6 = fma(x6, a, b);
      x7 = fma(x7, a, b);
    }
  }
  const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == T(-1)) out[blockIdx.x] = s;  // keeps the chains alive
}

}  // namespace

extern "C" ck_status ck_fp_peak_gflops(ck_handle* h, int32_t precision, double* gflops) {
  if (!h || !gflops) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  std::lock_guard<std::mutex> lock(h->mu);
  cudaSetDevice(h->device);
  cudaError_t e = h->unitBuf.ensure(sizeof(double) * 4096);
  if (e != cudaSuccess) return cudaFail(e, "probe buffer");
  const int blocks = h->smCount * 8, threads = 256;
  const int iters = precision == CK_PRECISION_FP64 ? 64 : 2048;
  cudaStream_t st = h->stream;
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(h->ev0, st);
    if (precision == CK_PRECISION_FP64)
      fmaPeakKernel<double><<<blocks, threads, 0, st>>>((double*)h->unitBuf.p, iters, 0.999999,
                                                        1e-7);
    else
      fmaPeakKernel<float><<<blocks, threads, 0, st>>>((float*)h->unitBuf.p, iters, 0.999999f,
                                                       1e-7f);
    cudaEventRecord(h->ev1, st);
    if ((e = cudaEventSynchronize(h->ev1)) != cudaSuccess) return cudaFail(e, "probe");
    float ms = 0;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    if (rep > 0 && ms < best) best = ms;
  }
  const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
  *gflops = flops / (best * 1e-3) / 1e9;
  h->lastLaunches = 4;
  return CK_OK;
}
