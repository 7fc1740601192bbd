// ck_propagate.cu — ck_propagate: a batch of independent propagations of
// bound track parameters with the fitter's own stepper (Lane::step in its
// propagation mode), the GPU counterpart of
//   Propagator<EigenStepper<>, VoidNavigator>::propagate(start[, target], options)
//   (Core/include/Acts/Propagator/Propagator.ipp:25-260).
// One thread per propagation; every loop is bounded (max steps, max
// Runge-Kutta trials). It runs the same step, intersection and covariance
// transport code as the fit kernels, so the reference's propagation property
// tests (forward-backward closure, reaching constructed target surfaces,
// covariance transport against numerical derivatives) pin the fit's stepper.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "ck_api_internal.h"
#include "ck_fitter.cuh"

using namespace ck;

namespace {

constexpr int kPropagateBlock = 64;

template <typename P, typename CV>
__global__ void __launch_bounds__(kPropagateBlock) propagateKernel(FitParams fp) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < fp.n_tracks;
       t += gridDim.x * blockDim.x) {
    Lane<P, CV> L;
    L.startPropagation(fp, t);
    // bounded: every accepted step counts towards maxSteps, every rejected
    // trial towards maxRungeKuttaStepTrials
    while (L.phase == PH_STEP) L.template step<kStepPropagate>(fp, t);
  }
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

extern "C" ck_status ck_propagate(ck_handle* h, const ck_options* opt, const ck_propagate_in* in,
                                  ck_propagate_out* out, void* stream) {
  if (!h || !in || !out) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  ck_status vs = validateOptions(opt);
  if (vs != CK_OK) return vs;
  const int n = in->n;
  if (n < 0) return fail(CK_ERR_INVALID_ARGUMENT, "n < 0");
  if (in->memory != CK_MEM_HOST && in->memory != CK_MEM_DEVICE)
    return fail(CK_ERR_INVALID_ARGUMENT, "unknown memory kind");
  if (n == 0) return CK_OK;
  if (!in->start_params || !in->start_frames || !in->particle || !in->path_limit || !out->status ||
      !out->end_params)
    return fail(CK_ERR_INVALID_ARGUMENT, "a required array is NULL");
  const bool host = in->memory == CK_MEM_HOST;
  if (host && in->target) {
    for (int i = 0; i < n; ++i) {
      const int s = in->target[i];
      if (s >= h->nSurfaces || s < -1) return fail(CK_ERR_INVALID_ARGUMENT, "target out of range");
    }
  }
  std::lock_guard<std::mutex> lock(h->mu);
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return cudaFail(e, "set device");
  cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;

  // device views of the arrays; host batches are staged in the handle's
  // unit buffer (inputs, outputs and the fail path's tip scratch)
  struct Arr {
    const void* src;
    void* dst;
    size_t bytes;
    bool input;
  };
  const size_t nn = (size_t)n;
  Arr arrs[] = {
      {in->start_params, nullptr, 48 * nn, true},  {in->start_cov, nullptr, 288 * nn, true},
      {in->start_frames, nullptr, 96 * nn, true},  {in->particle, nullptr, 8 * nn, true},
      {in->target, nullptr, 4 * nn, true},         {in->path_limit, nullptr, 8 * nn, true},
      {out->status, nullptr, 4 * nn, false},       {out->end_params, nullptr, 48 * nn, false},
      {out->end_cov, nullptr, 288 * nn, false},    {out->jacobian, nullptr, 288 * nn, false},
      {out->end_frames, nullptr, 96 * nn, false},  {out->path_length, nullptr, 8 * nn, false},
      {out->steps, nullptr, 4 * nn, false}};
  constexpr int kArrs = sizeof(arrs) / sizeof(arrs[0]);
  size_t total = align256(4 * nn);  // tip scratch
  if (host)
    for (int i = 0; i < kArrs; ++i)
      if (arrs[i].src) total += align256(arrs[i].bytes);
  if ((e = h->unitBuf.ensure(total)) != cudaSuccess) return cudaFail(e, "propagation buffer");
  char* base = (char*)h->unitBuf.p;
  int32_t* dTip = (int32_t*)base;
  size_t off = align256(4 * nn);
  for (int i = 0; i < kArrs; ++i) {
    if (!arrs[i].src) continue;
    if (host) {
      arrs[i].dst = base + off;
      off += align256(arrs[i].bytes);
      if (arrs[i].input)
        cudaMemcpyAsync(arrs[i].dst, arrs[i].src, arrs[i].bytes, cudaMemcpyHostToDevice, st);
    } else {
      arrs[i].dst = const_cast<void*>(arrs[i].src);
    }
  }
  FitParams fp;
  std::memset(&fp, 0, sizeof(fp));
  fp.n_tracks = n;
  fp.n_queue = n;
  fp.start_params = (const double*)arrs[0].dst;
  fp.start_cov = (const double*)arrs[1].dst;
  fp.start_frames = (const double*)arrs[2].dst;
  fp.particle = (const float*)arrs[3].dst;
  fp.prop.target = (const int32_t*)arrs[4].dst;
  fp.prop.path_limit = (const double*)arrs[5].dst;
  fp.out.status = (int32_t*)arrs[6].dst;
  fp.out.track_params = (double*)arrs[7].dst;
  fp.out.track_cov = (double*)arrs[8].dst;
  fp.prop.jac = (double*)arrs[9].dst;
  fp.prop.frames = (double*)arrs[10].dst;
  fp.prop.path = (double*)arrs[11].dst;
  fp.prop.steps = (int32_t*)arrs[12].dst;
  fp.tip = dTip;
  fp.max_states = 1;
  fp.lanes_per_warp = 32;
  fp.steps_per_round = 1;
  fp.surfaces = h->dSurfaces;
  fp.n_surfaces = h->nSurfaces;
  fp.trig = h->dTrig;
  fp.field = h->field;
  fp.mc = h->mc;
  fp.opt = toDevOptions(*opt);
  fp.ref_surface = -1;
  const int grid = (n + kPropagateBlock - 1) / kPropagateBlock;
  if (opt->precision == CK_PRECISION_MIXED)
    propagateKernel<float, float><<<grid, kPropagateBlock, 0, st>>>(fp);
  else
    propagateKernel<double, double><<<grid, kPropagateBlock, 0, st>>>(fp);
  if ((e = cudaGetLastError()) != cudaSuccess) return cudaFail(e, "propagation kernel launch");
  if (host) {
    for (int i = 0; i < kArrs; ++i)
      if (arrs[i].src && !arrs[i].input)
        cudaMemcpyAsync(const_cast<void*>(arrs[i].src), arrs[i].dst, arrs[i].bytes,
                        cudaMemcpyDeviceToHost, st);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cudaFail(e, "propagation kernel");
  }
  h->lastLaunches = 1;
  return CK_OK;
}
