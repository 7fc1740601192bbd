#!/usr/bin/env python3
"""Benchmark of the CudaKalman fitter: tracks/s fitted on one GB300.

Workload (one "step" = one pass of the fit over one batch): the barrel
configuration — 10 silicon cylinders r = 32..1020 mm (0.3 mm, x/X0 = 0.32 %,
multiple scattering and Bethe energy loss on), constant 2 T field, pions with
pT log-uniform in [0.5, 100] GeV, |eta| < 1.5, vertex sigma_z = 50 mm,
measurements (r*phi, z) with sigma 20/50 um, smeared start parameters — at
1,000,000 tracks per step (the mixed-precision accuracy configuration size),
synthetic, generated by acts_gb300.generate with a fixed seed per rank.

Reported (one JSON line, rank 0):
  value     tracks/s of the mixed-precision form with inputs resident in HBM
            (device batch pipeline: queue ordering + persistent fit kernel,
            CUDA-graph replayed), timed with CUDA events on the launching
            stream, K steps after W warm-up steps, max over ranks.
  fp64      the same for the plain FP64 form.
  e2e       the mixed form through the C ABI with pinned host buffers:
            host->device copy of the inputs, the fit, device->host copy of
            the smoothed parameters and covariances inside the timed region.
  Outputs of both: per state the surface, flags, path length, chi2, the
  smoothed parameters and the smoothed covariance as its upper triangle
  (CK_OUT_PACKED_COV: the 21 distinct entries of the symmetric matrix).
  roofline  fit kernel: algorithmic FP64 flops (reference formulation,
            counted by the oracle's counting scalar on a sample) per launch /
            kernel time, against the FP64 FMA peak measured live.
  accuracy  mixed vs FP64 on the first 100k tracks of the batch.
  cpu_baseline  the oracle (CPU restatement of the reference fit) on all
            host cores over a bounded sample.

--impl reference times the CPU restatement of the reference fit (the
reference itself cannot be built here: Eigen/Boost are absent) on the
host cores over bounded samples of the same workload.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOAD = "barrel10_si_2T_pions_1M_tracks"
SEED = 20240


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    from acts_gb300 import replicas

    return replicas.env()


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if len(s) > 2 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 2 and s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for i, n in enumerate(names):
                if len(s) > 5 + i and s[5 + i].strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


def make_workload(n, rank):
    from acts_gb300 import abi, generate

    det = generate.Detector(abi.CKG_BARREL)
    from acts_gb300 import replicas

    # replicas: every rank fits its own shard (distinct seeded tracks)
    b = generate.generate(det, n, seed=replicas.rank_seed(SEED, rank), cap=12)
    return det, b


def device_batch(b, torch, dev):
    """Uploads a Batch to torch device tensors; returns (ck_batch_in, keep)."""
    from acts_gb300 import abi

    keep = {}
    bi = abi.ck_batch_in()
    bi.n_tracks = b.n
    bi.memory = abi.MEM_DEVICE
    for name, ct in (("seq_offsets", C.c_int32), ("seq_surfaces", C.c_int32),
                     ("meas_offsets", C.c_int32), ("meas_surfaces", C.c_int32),
                     ("meas_values", C.c_double), ("meas_cov", C.c_double),
                     ("start_params", C.c_double), ("start_cov", C.c_double),
                     ("start_frames", C.c_double), ("particle", C.c_float),
                     ("particle_pdg", C.c_int32)):
        t = torch.from_numpy(getattr(b, name)).to(dev)
        keep[name] = t
        setattr(bi, name, C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ct)))
    return bi, keep


def device_outputs(n, max_states, torch, dev):
    from acts_gb300 import abi

    keep = {}
    bo = abi.ck_batch_out()
    bo.max_states = max_states
    bo.components = abi.OUT_SMOOTHED | abi.OUT_PACKED_COV
    bo.memory = abi.MEM_DEVICE
    spec = {"status": (n, torch.int32, C.c_int32), "n_states": (n, torch.int32, C.c_int32),
            "n_measurements": (n, torch.int32, C.c_int32), "n_holes": (n, torch.int32, C.c_int32),
            "n_outliers": (n, torch.int32, C.c_int32), "ndf": (n, torch.int32, C.c_int32),
            "chi2_sum": (n, torch.float64, C.c_double),
            "state_surface": (n * max_states, torch.int32, C.c_int32),
            "state_flags": (n * max_states, torch.int32, C.c_uint32),
            "state_path_length": (n * max_states, torch.float64, C.c_double),
            "state_chi2": (n * max_states, torch.float64, C.c_double),
            "smoothed": (n * max_states * 6, torch.float64, C.c_double),
            "smoothed_cov": (n * max_states * 21, torch.float64, C.c_double)}
    for name, (size, dt, ct) in spec.items():
        t = torch.zeros(size, dtype=dt, device=dev)
        keep[name] = t
        setattr(bo, name, C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ct)))
    return bo, keep


def host_pinned_batch(b, torch):
    """Pinned host copies of the inputs (ck_batch_in with memory = host)."""
    from acts_gb300 import abi

    keep = {}
    bi = abi.ck_batch_in()
    bi.n_tracks = b.n
    bi.memory = abi.MEM_HOST
    for name, ct in (("seq_offsets", C.c_int32), ("seq_surfaces", C.c_int32),
                     ("meas_offsets", C.c_int32), ("meas_surfaces", C.c_int32),
                     ("meas_values", C.c_double), ("meas_cov", C.c_double),
                     ("start_params", C.c_double), ("start_cov", C.c_double),
                     ("start_frames", C.c_double), ("particle", C.c_float),
                     ("particle_pdg", C.c_int32)):
        t = torch.from_numpy(getattr(b, name)).pin_memory()
        keep[name] = t
        setattr(bi, name, C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ct)))
    return bi, keep


def host_pinned_outputs(n, max_states, torch):
    from acts_gb300 import abi

    keep = {}
    bo = abi.ck_batch_out()
    bo.max_states = max_states
    bo.components = abi.OUT_SMOOTHED | abi.OUT_PACKED_COV
    bo.memory = abi.MEM_HOST
    spec = {"status": (n, torch.int32, C.c_int32), "n_states": (n, torch.int32, C.c_int32),
            "n_measurements": (n, torch.int32, C.c_int32), "n_holes": (n, torch.int32, C.c_int32),
            "n_outliers": (n, torch.int32, C.c_int32), "ndf": (n, torch.int32, C.c_int32),
            "chi2_sum": (n, torch.float64, C.c_double),
            "state_surface": (n * max_states, torch.int32, C.c_int32),
            "state_flags": (n * max_states, torch.int32, C.c_uint32),
            "state_path_length": (n * max_states, torch.float64, C.c_double),
            "state_chi2": (n * max_states, torch.float64, C.c_double),
            "smoothed": (n * max_states * 6, torch.float64, C.c_double),
            "smoothed_cov": (n * max_states * 21, torch.float64, C.c_double)}
    for name, (size, dt, ct) in spec.items():
        t = torch.zeros(size, dtype=dt).pin_memory()
        keep[name] = t
        setattr(bo, name, C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ct)))
    return bo, keep


def accuracy_report(b, r64, rmx, n):
    """Mixed vs FP64 on tracks [0, n): relative parameter error
    |x_mixed - x_fp64| / max(|x_fp64|, sigma_fp64) over measurement states,
    pull widths against the generator truth, chi2/ndf shift."""
    from acts_gb300 import abi

    ms = r64["max_states"]
    ok = (r64["status"][:n] == 0) & (rmx["status"][:n] == 0)
    agree = float(np.mean(r64["status"][:n] == rmx["status"][:n]))
    # the bound applies to valid fits (FP64 chi2/ndf < 5); fits broken in
    # FP64 (the cylinder phi = +-pi seam) are chaotic in any precision
    good = ok & (r64["chi2_sum"][:n] < 5.0 * np.maximum(r64["ndf"][:n], 1))
    n_broken = int((ok & ~good).sum())
    ok = good
    fl = r64["state_flags"].reshape(ms, r64["N"])[:, :n].T
    sm64 = r64["smoothed"].reshape(ms, 6, r64["N"])[:, :, :n].transpose(2, 0, 1)
    smmx = rmx["smoothed"].reshape(ms, 6, rmx["N"])[:, :, :n].transpose(2, 0, 1)
    # (packed upper triangles: the diagonal entries at 0, 6, 11, 15, 18, 20)
    cv64 = r64["smoothed_cov"].reshape(ms, 21, r64["N"])[:, :, :n].transpose(2, 0, 1)
    cvmx = rmx["smoothed_cov"].reshape(ms, 21, rmx["N"])[:, :, :n].transpose(2, 0, 1)
    diag = [0, 6, 11, 15, 18, 20]
    sig64 = np.sqrt(np.abs(cv64[..., diag]))
    meas = ((fl & abi.FLAG_HAS_MEASUREMENT) != 0) & ((fl & abi.FLAG_IS_OUTLIER) == 0)
    meas &= ok[:, None]
    d = np.abs(smmx - sm64)
    d[..., 2] = np.abs((smmx[..., 2] - sm64[..., 2] + np.pi) % (2 * np.pi) - np.pi)
    # (entries beyond a track's states are zero in both fits: 0/0, not used)
    with np.errstate(invalid="ignore", divide="ignore"):
        rel = d / np.maximum(np.abs(sm64), sig64)
    relm = rel[meas]
    # pulls against truth at the measurement states (smoothed loc0, loc1, phi, theta, q/p)
    surf = r64["state_surface"].reshape(ms, r64["N"])[:, :n].T
    mo, msurf = b.meas_offsets, b.meas_surfaces
    truth = b.truth_meas.reshape(-1, 6)
    pulls64, pullsmx = [[] for _ in range(5)], [[] for _ in range(5)]
    tracks = np.nonzero(ok)[0][:20000]
    for t in tracks:
        lut = {int(msurf[m]): m for m in range(mo[t], mo[t + 1])}
        for k in range(ms):
            if not meas[t, k]:
                continue
            m = lut.get(int(surf[t, k]))
            if m is None:
                continue
            for i in range(5):
                tv = truth[m, i]
                for arr, sm, cv in ((pulls64, sm64, cv64), (pullsmx, smmx, cvmx)):
                    dd = sm[t, k, i] - tv
                    if i == 2:
                        dd = (dd + np.pi) % (2 * np.pi) - np.pi
                    arr[i].append(dd / np.sqrt(cv[t, k, diag[i]]))
    names = ["loc0", "loc1", "phi", "theta", "qop"]
    w64 = [float(np.std(np.clip(p, -10, 10))) for p in pulls64]
    wmx = [float(np.std(np.clip(p, -10, 10))) for p in pullsmx]
    c64 = float(r64["chi2_sum"][:n][ok].sum() / max(1, r64["ndf"][:n][ok].sum()))
    cmx = float(rmx["chi2_sum"][:n][ok].sum() / max(1, rmx["ndf"][:n][ok].sum()))
    return {"tracks": int(n), "status_agreement": agree, "valid_fits": int(ok.sum()),
            "excluded_broken_fits": n_broken,
            "rel_err_definition": "|x_mixed - x_fp64| / max(|x_fp64|, sigma_fp64), smoothed "
                                  "parameters at measurement states",
            "max_rel_param_err": float(relm.max()) if relm.size else None,
            "p99_rel_param_err": float(np.quantile(relm, 0.99)) if relm.size else None,
            "max_rel_err_per_param": dict(zip(["loc0", "loc1", "phi", "theta", "qop", "time"],
                                              [float("%.3g" % x) for x in relm.max(axis=0)]))
            if relm.size else None,
            "pull_width_fp64": dict(zip(names, [round(x, 4) for x in w64])),
            "pull_width_mixed": dict(zip(names, [round(x, 4) for x in wmx])),
            "max_pull_width_shift": float(max(abs(a - b2) / a for a, b2 in zip(w64, wmx))),
            "chi2ndf_fp64": c64, "chi2ndf_mixed": cmx}


# Forward-filter kernel of a precision form and variant (ck_set_launch_config),
# as ncu names its template instance
_VARIANT_KERNELS = {
    "float": {0: "fitKernel<float, float, 128, 1>", 1: "fitKernel<float, float, 128, 3>",
              2: "fitKernel<float, float, 128, 4>",
              3: "fitKernelCompact<float, float, 256, false, false>",
              4: "fitKernelCompact<float, float, 128, false, false>",
              5: "fitKernelPool<float, float, 384, 256>",
              6: "fitKernelPool<float, float, 448, 256>"},
    "double": {0: "fitKernel<double, double, 128, 1>", 1: "fitKernel<double, double, 128, 3>",
               2: "fitKernel<double, double, 128, 4>",
               3: "fitKernelCompact<double, double, 256, false, false>",
               4: "fitKernelCompact<double, double, 128, false, false>",
               5: "fitKernelPool<double, double, 320, 256>",
               6: "fitKernelPool<double, double, 256, 256>"}}
COUNTERS = os.path.join(ROOT, "profiles", "fit_kernel_counters.txt")


def kernel_counters(scalar, variant):
    """The committed ncu per-track counters of a forward-filter kernel plus
    the smoother kernel that follows it (the filter smooths most tracks in
    its tail, the smoother kernel the rest: their sum is the filter and
    smoother work of every track), when they were captured from the sources
    that run now (else None, reason)."""
    from acts_gb300 import profile_counters

    name = _VARIANT_KERNELS[scalar].get(variant)
    smoother = "smoothKernel<%s, 128>" % scalar
    if not os.path.exists(COUNTERS):
        return None, "no counters file"
    src, lines = profile_counters.parse(COUNTERS)
    if src != profile_counters.source_hash():
        return None, "counters captured from other kernel sources (%s)" % src
    pick = lambda k: next((ln for ln in lines if k and _kernel_key(k) in _kernel_key(ln["kernel"])),
                          None)
    fwd, smo = pick(name), pick(smoother)
    if fwd is None or smo is None:
        return None, "no capture of %s" % (name if fwd is None else smoother)
    both = dict(fwd)
    for k in ("fp64_flops", "fp32_flops", "dram_bytes", "conversions"):
        both[k] = fwd[k] + smo[k]
    both["filter"] = fwd
    return both, "%s + %s" % (name, smoother)


def _kernel_key(name):
    """A kernel name as ncu may print it: template booleans as 0/1, no spaces."""
    return name.replace("false", "0").replace("true", "1").replace(" ", "")


def best_of_tune_log(log):
    """The fastest entry of an autotuner log ("v3 tpb256 bps1 spr3 12.345ms; ...")."""
    best = None
    for item in log.split(";"):
        parts = item.split()
        if len(parts) >= 2 and parts[-1].endswith("ms"):
            ms = float(parts[-1][:-2])
            if best is None or ms < best[1]:
                best = (" ".join(parts[:-1]), ms)
    return None if best is None else {"config": best[0], "kernel_ms": best[1],
                                      "configs_tried": len([x for x in log.split(";") if x.strip()])}


def cpu_baseline(det, b, opt, budget_s=10.0):
    """The oracle on all host cores over a bounded sample (~budget_s)."""
    from oracle import kforacle

    cores = os.cpu_count() or 1
    probe = min(b.n, 4000)
    dt = kforacle.time_batch(det, b, opt, cores, 0, probe)
    rate = probe / max(dt, 1e-6)
    count = int(min(b.n, max(probe, rate * budget_s)))
    dt = kforacle.time_batch(det, b, opt, cores, 0, count)
    return {"value": count / dt, "unit": "tracks/s", "cores": cores, "kind": "port",
            "sample": "%d barrel tracks (first of the step batch), %.1f s on %d host threads; "
                      "oracle = C++ restatement of the reference fit (reference not buildable "
                      "here: Eigen/Boost absent)" % (count, dt, cores)}


def bench_config(n, max_states):
    """The workload description both arms print."""
    return {"workload": WORKLOAD, "tracks_per_step_per_gpu": n,
            "precision": "mixed (stepper, transport, field and the Kalman update in FP32; "
                         "parameter accumulation, smoother-gain inverse and bound-parameter "
                         "conversions in FP64)",
            "l2": "inputs ~1 GB per step > 129 MB L2 (no flush needed)",
            "max_states": max_states,
            "outputs": "smoothed parameters + covariances (packed upper triangles)"}


def reference_arm(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    from acts_gb300 import abi
    from oracle import kforacle

    # the native arm's workload; each step fits a bounded sample of it
    det, b = make_workload(args.tracks, 0)
    opt = abi.default_options()
    cores = os.cpu_count() or 1
    probe = min(b.n, 4000)
    dt = kforacle.time_batch(det, b, opt, cores, 0, probe)
    rate = probe / max(dt, 1e-6)
    per_step = int(min(b.n, max(probe, rate * 3.0)))  # ~3 s of CPU work per step
    for _ in range(max(0, args.warmup)):
        kforacle.time_batch(det, b, opt, cores, 0, min(per_step, 2000))
    times = []
    for s in range(args.steps):
        first = (s * per_step) % max(1, b.n - per_step + 1)
        times.append(kforacle.time_batch(det, b, opt, cores, first, per_step))
    tot = sum(times)
    value = per_step * args.steps / tot
    line = {"metric": "tracks/s fitted (FP64 vs mixed, same accuracy); p50/p99 event latency",
            "impl": "reference", "value": value, "unit": "tracks/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": bench_config(args.tracks, 10),
            "cpu_baseline": {"value": value, "unit": "tracks/s", "cores": cores, "kind": "port",
                             "sample": "%d of the workload's %d barrel tracks per step, on "
                                       "%d host threads (C++ restatement of the reference fit in "
                                       "FP64; the reference needs Eigen/Boost, absent here)"
                                       % (per_step, b.n, cores)},
            "e2e": {"value": value, "unit": "tracks/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def native_arm(args):
    import torch

    from acts_gb300 import abi
    from acts_gb300.fitter import CudaKalman

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = args.tracks
    ms = 10
    t0 = time.time()
    det, b = make_workload(n, rank)
    log("rank %d: generated %d tracks in %.1f s" % (rank, n, time.time() - t0))
    fit = CudaKalman.for_detector(det, device=local, use_graph=True)
    bi, keep_in = device_batch(b, torch, dev)
    bo, keep_out = device_outputs(n, ms, torch, dev)
    # a dedicated stream: the fit is launched on it and the CUDA events that
    # time it are recorded on it
    stream = torch.cuda.Stream(dev)
    sp = C.c_void_p(stream.cuda_stream)

    from acts_gb300 import replicas

    forms = {"mixed": abi.default_options(precision=abi.PRECISION_MIXED),
             "fp64": abi.default_options(precision=abi.PRECISION_FP64)}
    results = {}
    snapshots = {}
    clocks = ClockSampler(local)
    tune_log = {}
    for name, opt in forms.items():
        # the project's autotuner picks the kernel variant, threads per block
        # and resident blocks per SM on this very batch (before any timing)
        if args.autotune:
            tune_log[name] = fit.autotune(opt, bi, bo)
        for _ in range(max(3, args.warmup)):
            fit.fit_batch_raw(opt, bi, bo, sp)
        torch.cuda.synchronize(dev)
        launches_per_step = fit.last_launch_count()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        kernel_ms = []
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        with clocks if name == "mixed" else _Null():
            ev0.record(stream)
            for _ in range(args.steps):
                fit.fit_batch_raw(opt, bi, bo, sp)
            ev1.record(stream)
            torch.cuda.synchronize(dev)
        ms_total = ev0.elapsed_time(ev1)
        # kernel-only time of one more step (events recorded inside the graph)
        fit.fit_batch_raw(opt, bi, bo, sp)
        torch.cuda.synchronize(dev)
        kernel_ms.append(fit.last_kernel_ms())
        split_ms = fit.last_kernel_split_ms()
        ms_total = replicas.max_over_ranks(ms_total)
        status = keep_out["status"].cpu().numpy()
        results[name] = {"ms_per_step": ms_total / args.steps,
                         "tracks_per_s": n * world / (ms_total / args.steps / 1e3),
                         "kernel_ms": float(np.mean(kernel_ms)),
                         "filter_kernel_ms": split_ms[0], "smoother_kernel_ms": split_ms[1],
                         "launches_per_step": launches_per_step,
                         "ok_fraction": float(np.mean(status == 0)),
                         "launch_config": fit.launch_config(opt.precision),
                         "autotuned": best_of_tune_log(tune_log.get(name, ""))}
        na = min(n, 100000)
        snapshots[name] = {k: keep_out[k].cpu().numpy() for k in
                           ("status", "state_flags", "state_surface", "smoothed",
                            "smoothed_cov", "chi2_sum", "ndf")}
        snapshots[name]["N"] = n
        snapshots[name]["max_states"] = ms
        log("rank %d %s: %.3f ms/step, %.3g tracks/s, kernel %.3f ms" %
            (rank, name, results[name]["ms_per_step"], results[name]["tracks_per_s"],
             results[name]["kernel_ms"]))

    # ---- end-to-end through the C ABI with pinned host buffers
    hbi, keep_hin = host_pinned_batch(b, torch)
    hbo, keep_hout = host_pinned_outputs(n, ms, torch)
    opt = forms["mixed"]
    for _ in range(max(3, args.warmup)):
        fit.fit_batch_raw(opt, hbi, hbo, sp)
    torch.cuda.synchronize(dev)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        fit.fit_batch_raw(opt, hbi, hbo, sp)
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    e2e_ms = ev0.elapsed_time(ev1) / args.steps
    h2d, d2h = fit.last_transfer_bytes()
    e2e_launches = fit.last_launch_count()
    e2e_ms = replicas.max_over_ranks(e2e_ms)

    if rank != 0:
        fit.close()
        if world > 1:
            torch.distributed.barrier()
        return 0

    # ---- roofline of the dominant kernel of the mixed step: the forward
    # filter, which smooths most tracks in its tail (the smoother kernel
    # takes the rest), bound by the FP64 pipe. The FP64 flops and DRAM bytes
    # per track of the pair come from the committed ncu counters of the
    # kernel variant launched, valid while their source hash matches the
    # sources that run (both scale with the track count); the duration of
    # the pair is measured here.
    from oracle import kforacle

    flops = kforacle.count_flops(det, b, forms["fp64"], 0, 300)
    peak64 = fit.fp_peak_gflops(abi.PRECISION_FP64) / 1e3
    peak32 = fit.fp_peak_gflops(abi.PRECISION_MIXED) / 1e3
    fwd_mx = (results["mixed"]["filter_kernel_ms"] + results["mixed"]["smoother_kernel_ms"]) * 1e-3
    fwd_64 = (results["fp64"]["filter_kernel_ms"] + results["fp64"]["smoother_kernel_ms"]) * 1e-3
    cm, why_m = kernel_counters("float", fit.launch_variant(abi.PRECISION_MIXED)[0])
    c64, why_64 = kernel_counters("double", fit.launch_variant(abi.PRECISION_FP64)[0])
    roofline = {"bound": "fp64", "unit": "TFLOP/s", "peak": round(peak64, 4),
                "duration_ms": round(fwd_mx * 1e3, 3),
                "peak_source": "measured live: FP64 FMA loop (ck_fp_peak_gflops); "
                               "MEASURED_PEAKS.json holds no FP64 figure",
                "counters_source": "profiles/fit_kernel_counters.txt (ncu per-track counts of "
                                   "the launched kernel; source hash checked)"}
    if cm is not None:
        ach_mx = cm["fp64_flops"] * n / fwd_mx / 1e12
        roofline.update({
            "kernel": why_m + " (mixed forward filter smoothing in its tail, and the "
                              "smoother kernel for the rest)",
            "achieved": round(ach_mx, 4), "frac": round(ach_mx / peak64, 4),
            "traffic": int(cm["dram_bytes"] * n),
            "algorithmic_flops_per_track": round(cm["fp64_flops"], 1),
            "flops_definition": "FP64 flops of the mixed formulation's forward filter and "
                                "smoother per track (its FP32 work, %.1f kflop/track, runs on a "
                                "63x faster pipe), counted by ncu" % (cm["fp32_flops"] / 1e3),
            "fp64_pipe_busy_ncu": cm["fp64_pipe_busy"],
            "fp32_frac": round(cm["fp32_flops"] * n / fwd_mx / 1e12 / peak32, 4)})
    else:
        roofline.update({"kernel": "mixed forward filter", "achieved": None, "frac": None,
                         "traffic": None, "counters_missing": why_m})
    if c64 is not None:
        ach_64 = c64["fp64_flops"] * n / fwd_64 / 1e12
        roofline["fp64_form"] = {"kernel": why_64, "achieved": round(ach_64, 4),
                                 "frac": round(ach_64 / peak64, 4),
                                 "duration_ms": round(fwd_64 * 1e3, 3),
                                 "fp64_pipe_busy_ncu": c64["fp64_pipe_busy"],
                                 "traffic": int(c64["dram_bytes"] * n)}
    else:
        roofline["fp64_form"] = {"duration_ms": round(fwd_64 * 1e3, 3), "frac": None,
                                 "counters_missing": why_64}
    roofline.update({
                "reference_formulation": {
                    "flops_per_track": round(flops["flops"], 1),
                    "definition": "FP64 flops of the reference's dense formulation (8x8 "
                                  "transport, dense products), counted by the oracle's counting "
                                  "scalar over %d tracks" % flops["tracks"],
                    "equivalent_tflops_mixed": round(flops["flops"] * n /
                                                     (results["mixed"]["kernel_ms"] * 1e-3) / 1e12, 3),
                    "equivalent_tflops_fp64": round(flops["flops"] * n /
                                                    (results["fp64"]["kernel_ms"] * 1e-3) / 1e12, 3)},
                "fp32_peak_tflops": round(peak32, 3)})
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        roofline["hbm_gbs_of_measured"] = round(roofline["traffic"] / fwd_mx / 1e9 / peaks["hbm_gbs"], 5)
    except (OSError, KeyError, ValueError, ZeroDivisionError, TypeError):
        pass

    acc = accuracy_report(b, snapshots["fp64"], snapshots["mixed"], min(n, 100000))
    cpu = cpu_baseline(det, b, forms["fp64"], budget_s=10.0)
    fit.close()
    del keep_in, keep_out, keep_hin, keep_hout
    events = (batched_events_report(torch, dev, args.steps, args.warmup, args.autotune)
              if args.events else None)
    serving = serving_report(torch) if args.serving else None
    ckf = ckf_report(torch, dev, args.steps, args.warmup) if args.ckf else None
    mixed = results["mixed"]
    line = {"metric": "tracks/s fitted (FP64 vs mixed, same accuracy); p50/p99 event latency",
            "value": round(mixed["tracks_per_s"], 1), "unit": "tracks/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(mixed["ms_per_step"], 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic",
            "config": bench_config(n, ms),
            "fp64": {"value": round(results["fp64"]["tracks_per_s"], 1), "unit": "tracks/s",
                     "ms_per_step": round(results["fp64"]["ms_per_step"], 3),
                     "mixed_over_fp64": round(mixed["tracks_per_s"] /
                                              results["fp64"]["tracks_per_s"], 3)},
            "e2e": {"value": round(n * world / (e2e_ms / 1e3), 1), "unit": "tracks/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "ms_per_step": round(e2e_ms, 3), "path": "ck_fit_batch, host memory"},
            "roofline": roofline, "accuracy": acc, "cpu_baseline": cpu,
            "batched_events": events, "serving": serving, "track_finding": ckf,
            "clocks": clocks.summary(),
            "gpu_launches": int(mixed["launches_per_step"] * args.steps),
            "kernel": {"mixed": mixed, "fp64": results["fp64"]},
            "e2e_launches_per_step": e2e_launches}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()
    return 0


def _ckf_device(tf, torch, dev):
    """Device copies of a TrackFinding's arrays: (ck_ckf_in, ck_ckf_out, keep)."""
    from acts_gb300 import abi

    keep = {}
    di = tf.as_in()
    di.memory = abi.MEM_DEVICE
    for name, _ in abi.ck_ckf_in._fields_:
        v = getattr(tf, name, None)
        if isinstance(v, np.ndarray):
            t = torch.from_numpy(np.ascontiguousarray(v)).to(dev)
            keep[name] = t
            setattr(di, name, C.cast(C.c_void_p(t.data_ptr()), type(getattr(di, name))))
    do = tf.as_out()
    for name, _ in abi.ck_ckf_out._fields_:
        t = torch.from_numpy(np.ascontiguousarray(getattr(tf, name))).to(dev)
        keep["out_" + name] = t
        setattr(do, name, C.cast(C.c_void_p(t.data_ptr()), type(getattr(do, name))))
    return di, do, keep


def _ckf_time(fit, opt, ko, tf, make_host, torch, dev, steps, warmup):
    """Device-resident ms per call (CUDA events on a stream of its own) and
    host-memory ms per call (wall clock), with the host call's results."""
    stream = torch.cuda.Stream(dev)
    di, do, keep = _ckf_device(tf, torch, dev)
    torch.cuda.synchronize(dev)
    for _ in range(max(warmup, 1)):
        fit.find_tracks_raw(opt, ko, di, do, stream.cuda_stream)
    torch.cuda.synchronize(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        fit.find_tracks_raw(opt, ko, di, do, stream.cuda_stream)
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    ms = ev0.elapsed_time(ev1) / steps
    del keep
    host = make_host()
    fit.find_tracks(opt, ko, host)  # (warms the host path's staging buffer)
    t0 = time.perf_counter()
    for _ in range(steps):
        fit.find_tracks(opt, ko, host)
    return ms, (time.perf_counter() - t0) / steps * 1e3, host


def ckf_report(torch, dev, steps, warmup, n_seeds=10000, seed=95, sample_seeds=1000,
               n_events=50, event_mean=2000.0):
    """Track finding (ck_find_tracks) on the barrel workload, chi2 cut 15,
    one candidate per surface, branches ended by loop protection:
    * one event of 10,000 pions (100,000 measurements, 10,000 on each of the
      10 cylinder layers), every track's start parameters a seed with its
      surface sequence;
    * 50 events of Poisson(2,000) pions in one call (each seed sees its own
      event's measurements).
    Times the device-resident call (CUDA events on the launching stream) and
    the host-memory call (wall clock, copies included) for both forms, the
    oracle on a sample of the single event's seeds (against the whole
    event's measurements) on all host threads, and checks the FP64 results
    of that sample against it."""
    from acts_gb300 import abi, generate
    from acts_gb300.fitter import CudaKalman
    from oracle import kforacle

    det = generate.Detector(abi.CKG_BARREL)
    b = generate.generate(det, n_seeds, seed=seed)
    tf = generate.ckf_event(det, b, max_states=24, max_tracks=4)
    ko = tf.options(chi2_cut=15.0, max_branches=8)
    sizes = generate.event_sizes(seed, n_events, mean=event_mean)
    bm = generate.generate(det, int(sizes.sum()), seed=seed + 1)
    tfm = generate.ckf_events(det, bm, sizes, max_states=24, max_tracks=4)
    fit = CudaKalman.for_detector(det)
    report = {"workload": "barrel: one event of %d seeds, %d measurements (%d per layer); and %d "
                          "events of Poisson(%d) seeds (%d seeds) in one call; chi2 cut 15, 1 "
                          "candidate per surface" % (n_seeds, tf.n_meas, tf.n_meas // 10,
                                                     n_events, event_mean, tfm.n),
              "unit": "seeds/s"}
    for name in ("fp64", "mixed"):
        prec = abi.PRECISION_MIXED if name == "mixed" else abi.PRECISION_FP64
        opt = abi.default_options(precision=prec)
        ms, e2e, host = _ckf_time(fit, opt, ko, tf,
                                  lambda: generate.ckf_event(det, b, max_states=24, max_tracks=4),
                                  torch, dev, steps, warmup)
        msm, e2em, hostm = _ckf_time(fit, opt, ko, tfm,
                                     lambda: generate.ckf_events(det, bm, sizes, max_states=24,
                                                                 max_tracks=4),
                                     torch, dev, steps, warmup)
        report[name] = {"seeds_per_s": round(n_seeds / (ms / 1e3), 1), "ms": round(ms, 3),
                        "e2e_seeds_per_s": round(n_seeds / (e2e / 1e3), 1),
                        "e2e_ms": round(e2e, 3), "lanes_per_seed": fit.last_ckf_lanes(),
                        "tracks_found": int(host.n_tracks.sum()),
                        "status_ok": int((host.status == 0).sum()),
                        "events": {"seeds_per_s": round(tfm.n / (msm / 1e3), 1),
                                   "ms": round(msm, 3),
                                   "e2e_seeds_per_s": round(tfm.n / (e2em / 1e3), 1),
                                   "e2e_ms": round(e2em, 3),
                                   "tracks_found": int(hostm.n_tracks.sum()),
                                   "status_ok": int((hostm.status == 0).sum())}}
        if name == "fp64":
            gpu64 = host
    fit.close()
    # oracle on the first `sample_seeds` seeds against the whole event
    S = sample_seeds
    so = tf.seq_offsets[:S + 1]
    sub = abi.TrackFinding(so, tf.seq_surfaces[:so[-1]], tf.start_params[:S], tf.start_cov[:S],
                           tf.start_frames[:S], tf.particle[:S], tf.surf_meas_offsets,
                           tf.meas_values, tf.meas_cov, meas_subspace=tf.meas_subspace,
                           particle_pdg=tf.particle_pdg[:S], max_states=24, max_tracks=4)
    threads = kforacle.hardware_threads()
    t0 = time.perf_counter()
    kforacle.find_tracks(det.surfaces, det.field, abi.default_options(), ko, sub,
                         n_threads=threads)
    cpu_s = time.perf_counter() - t0
    report["cpu_baseline"] = {"value": round(S / cpu_s, 1), "unit": "seeds/s", "cores": threads,
                              "kind": "port", "sample": "%d seeds of the 10,000-seed event" % S}
    same = int(sum(1 for s in range(S)
                   if gpu64.status[s] == sub.status[s] and gpu64.n_tracks[s] == sub.n_tracks[s]
                   and all(gpu64.track_measurements(s, k) == sub.track_measurements(s, k)
                           for k in range(sub.n_tracks[s]))))
    report["fp64_parity_sample"] = {"seeds": S, "identical_tracks": same}
    return report


def batched_events_report(torch, dev, steps, warmup, autotune, seed=91, n_events=50,
                          mean_tracks=5000.0, max_states=20):
    """The batched uneven-events configuration: 50 events with Poisson(5,000)
    tracks each, 4-20 hits per track (holes 10 %, 5 % outliers displaced 10
    sigma, chi2 outlier cut 15), the synthetic 3D grid field map read with
    trilinear interpolation; all events as one device-resident batch fitted
    by one persistent forward-filter launch (plus queue ordering and
    smoother), CUDA-graph replayed, launch shape autotuned on this batch.
    Inputs (~250 MB) exceed the L2. Reports tracks/s per precision form."""
    from acts_gb300 import abi, generate
    from acts_gb300.fitter import CudaKalman

    det = generate.Detector(abi.CKG_UNEVEN)
    sizes = generate.event_sizes(seed, n_events, mean=mean_tracks)
    n = int(sizes.sum())
    b = generate.generate(det, n, seed=seed)
    fit = CudaKalman.for_detector(det, device=dev.index or 0, use_graph=True)
    bi, keep_in = device_batch(b, torch, dev)
    bo, keep_out = device_outputs(n, max_states, torch, dev)
    stream = torch.cuda.Stream(dev)
    sp = C.c_void_p(stream.cuda_stream)
    rep = {"workload": "%d uneven events, Poisson(%d) tracks each (%d tracks), 4-20 hits, "
                       "holes 10 %%, outliers 5 %% at 10 sigma, chi2 cut 15, 3D grid field "
                       "(151x151x301, 20 mm pitch, trilinear)" % (n_events, mean_tracks, n),
           "tracks": n, "events": n_events, "max_states": max_states}
    for name, prec in (("mixed", abi.PRECISION_MIXED), ("fp64", abi.PRECISION_FP64)):
        opt = abi.default_options(precision=prec, outlier_chi2_cut=15.0)
        tl = fit.autotune(opt, bi, bo) if autotune else ""
        for _ in range(max(3, warmup)):
            fit.fit_batch_raw(opt, bi, bo, sp)
        torch.cuda.synchronize(dev)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            fit.fit_batch_raw(opt, bi, bo, sp)
        ev1.record(stream)
        torch.cuda.synchronize(dev)
        ms = ev0.elapsed_time(ev1) / steps
        fit.fit_batch_raw(opt, bi, bo, sp)
        torch.cuda.synchronize(dev)
        split = fit.last_kernel_split_ms()
        st = keep_out["status"].cpu().numpy()
        codes, counts = np.unique(st, return_counts=True)
        rep[name] = {"tracks_per_s": round(n / (ms / 1e3), 1), "ms_per_step": round(ms, 3),
                     "filter_kernel_ms": round(split[0], 3),
                     "smoother_kernel_ms": round(split[1], 3),
                     "launch_config": fit.launch_config(prec),
                     "autotuned": best_of_tune_log(tl),
                     "statuses": {abi.TRACK_STATUS.get(int(c), str(c)): int(k)
                                  for c, k in zip(codes, counts)}}
        log("batched events %s: %.3f ms/step, %.3g tracks/s" % (name, ms, n / (ms / 1e3)))
    rep["mixed_over_fp64"] = round(rep["mixed"]["tracks_per_s"] / rep["fp64"]["tracks_per_s"], 3)
    fit.close()
    return rep


class EventPool:
    """Events of the serving configuration as slices of one pool of uneven
    tracks in page-locked host memory: event i takes `sizes[i]` consecutive
    pool tracks from a random start, with its own CSR offsets rebased to 0
    (the other arrays are pointers into the pool)."""

    PER_TRACK = (("start_params", C.c_double, 6), ("start_cov", C.c_double, 36),
                 ("start_frames", C.c_double, 12), ("particle", C.c_float, 2),
                 ("particle_pdg", C.c_int32, 1))
    PER_SEQ = (("seq_surfaces", C.c_int32, 1),)
    PER_MEAS = (("meas_surfaces", C.c_int32, 1), ("meas_values", C.c_double, 2),
                ("meas_cov", C.c_double, 4))

    def __init__(self, b, torch):
        self.b = b
        self.keep = {}
        for name, ct, k in self.PER_TRACK + self.PER_SEQ + self.PER_MEAS:
            self.keep[name] = torch.from_numpy(getattr(b, name)).pin_memory()
        self.so = np.asarray(b.seq_offsets)
        self.mo = np.asarray(b.meas_offsets)

    def event(self, start, m):
        from acts_gb300 import abi

        a, e = start, start + m
        so = np.ascontiguousarray(self.so[a:e + 1] - self.so[a], np.int32)
        mo = np.ascontiguousarray(self.mo[a:e + 1] - self.mo[a], np.int32)
        bi = abi.ck_batch_in()
        bi.n_tracks = m
        bi.memory = abi.MEM_HOST
        bi.seq_offsets = abi.ptr(so, C.c_int32)
        bi.meas_offsets = abi.ptr(mo, C.c_int32)
        for group, first in ((self.PER_TRACK, a), (self.PER_SEQ, int(self.so[a])),
                             (self.PER_MEAS, int(self.mo[a]))):
            for name, ct, k in group:
                t = self.keep[name]
                addr = t.data_ptr() + first * k * t.element_size()
                setattr(bi, name, C.cast(C.c_void_p(addr), C.POINTER(ct)))
        return bi, (so, mo)


def serving_report(torch, n_events=10000, seed=77, max_states=20, pool_tracks=400000,
                   lo=100, hi=20000):
    """The serving configuration: events with log-uniform 100-20,000 tracks
    of the uneven workload (20-cylinder barrel, 4-20 hits, holes, outliers,
    grid field), arriving as a Poisson process at an offered rate swept from
    10 % to 120 % of the measured capacity, admitted against a 40 GB device
    budget by the continuous-batching server; inputs in page-locked host
    memory, results written to device buffers (at half load also to
    page-locked and to pageable host buffers). Reports per load the
    sustained tracks/s and p50/p99 submit-to-results latency of all events
    and of the events with 8,000-12,000 tracks."""
    import threading

    from acts_gb300 import abi, generate
    from acts_gb300.fitter import CudaKalman
    from acts_gb300.results import Results, TorchResults
    from acts_gb300.serving import FitServer

    det = generate.Detector(abi.CKG_UNEVEN)
    pool = EventPool(generate.generate(det, pool_tracks, seed=seed), torch)
    sizes = generate.event_sizes(seed, n_events, -1.0, lo, hi)
    rng = np.random.default_rng(seed)
    starts = rng.integers(0, pool_tracks - hi, n_events)
    mean = float(sizes.mean())
    comps = abi.OUT_SMOOTHED | abi.OUT_PACKED_COV
    fit = CudaKalman.for_detector(det)
    report = {"workload": "%d events, log-uniform %d-%d tracks (mean %.0f) of the uneven "
                          "workload (4-20 hits, holes 10 %%, outliers 5 %%, grid field), "
                          "Poisson arrivals; inputs in page-locked host memory"
                          % (n_events, lo, hi, mean),
              "memory_budget_gb": 40, "streams": 3, "max_states": max_states,
              "launch": "each co-batch on the SMs / (streams - 1) blocks, 6 Runge-Kutta trials "
                        "per scheduling round (the server's defaults)"}

    class _Lat:
        def __init__(self):
            self.lat, self.done = {}, threading.Event()

    for name in ("mixed", "fp64"):
        prec = abi.PRECISION_MIXED if name == "mixed" else abi.PRECISION_FP64
        opt = abi.default_options(precision=prec, outlier_chi2_cut=15.0)
        srv = FitServer(fit, opt, memory_budget_bytes=40 << 30, n_streams=3,
                        max_states=max_states, max_batch_tracks=8 * hi, components=comps)

        def run(idx, rate, results_of):
            """Submits events idx (Poisson arrivals at `rate` events/s; 0:
            back to back); returns {event: latency ms} and the wall time."""
            st = _Lat()
            n_ev = len(idx)
            held = {}

            def poller():
                try:
                    while len(st.lat) < n_ev:
                        r = srv.poll(timeout_ms=200)
                        if r is not None:
                            st.lat[r[0]] = r[2]
                            held.pop(r[0], None)
                finally:
                    st.done.set()

            th = threading.Thread(target=poller, daemon=True)
            th.start()
            t0 = time.perf_counter()
            gaps = rng.exponential(1.0 / rate, n_ev) if rate else np.zeros(n_ev)
            t_next = t0
            for k, i in enumerate(idx):
                t_next += gaps[k]
                while True:
                    dt = t_next - time.perf_counter()
                    if dt <= 0:
                        break
                    time.sleep(min(dt, 0.0005))
                bi, keep = pool.event(int(starts[i]), int(sizes[i]))
                res = results_of(int(sizes[i]))
                held[int(i)] = (keep, res)
                srv.submit(int(i), _Wrap(bi), res)
            st.done.wait(600)
            return st.lat, time.perf_counter() - t0

        def stats(lat, idx, wall):
            v = np.array([lat[int(i)] for i in idx])
            m = sizes[idx]
            sel = (m >= 8000) & (m <= 12000)
            out = {"events": int(len(idx)),
                   "sustained_tracks_per_s": round(float(m.sum()) / wall, 1),
                   "p50_ms": round(float(np.percentile(v, 50)), 3),
                   "p99_ms": round(float(np.percentile(v, 99)), 3)}
            if sel.sum() >= 10:
                out["events_8k_12k"] = int(sel.sum())
                out["p50_ms_8k_12k"] = round(float(np.percentile(v[sel], 50)), 3)
                out["p99_ms_8k_12k"] = round(float(np.percentile(v[sel], 99)), 3)
            return out

        on_device = lambda m: TorchResults(m, max_states, comps, device="cuda:0")
        run(np.arange(50), 0, on_device)  # warm-up
        cap_idx = np.arange(2000 if name == "mixed" else 500)
        lat, wall = run(cap_idx, 0, on_device)
        cap_tracks = float(sizes[cap_idx].sum()) / wall
        res = {"capacity_tracks_per_s": round(cap_tracks, 1), "results": "device memory",
               "loads": []}
        if name == "mixed":
            plan = ((0.1, 2500), (0.3, n_events), (0.5, n_events), (0.8, n_events),
                    (1.0, n_events), (1.2, n_events))
        else:
            plan = ((0.1, 800), (0.5, 1000), (1.0, 1000), (1.2, 1000))
        for f, cnt in plan:
            idx = np.arange(cnt)
            rate = f * cap_tracks / mean
            lat, wall = run(idx, rate, on_device)
            entry = {"offered_fraction": f, "offered_tracks_per_s": round(rate * mean, 1)}
            entry.update(stats(lat, idx, wall))
            res["loads"].append(entry)
            log("serving %s %.1f: %s" % (name, f, entry))
        if name == "mixed":
            # results delivered to host memory at half load: page-locked
            # buffers; pageable buffers allocated per event (every page is
            # touched first by the delivery copy); pageable buffers reused
            # from a ring, as a caller that keeps its containers does
            ring = [Results(hi, max_states, comps) for _ in range(32)]
            for r in ring:
                for name_, a in vars(r).items():
                    if isinstance(a, np.ndarray):
                        a.fill(0)
            ring_pos = [0]

            def from_ring(m):
                r = ring[ring_pos[0] % len(ring)]
                ring_pos[0] += 1
                return _RingResults(r, m)

            for label, mk in (("page-locked host memory",
                               lambda m: TorchResults(m, max_states, comps, device="pinned")),
                              ("pageable host memory, new buffers per event",
                               lambda m: Results(m, max_states, comps)),
                              ("pageable host memory, reused buffers", from_ring)):
                idx = np.arange(600)
                lat, wall = run(idx, 0.5 * cap_tracks / mean, mk)
                entry = {"results": label, "offered_fraction": 0.5}
                entry.update(stats(lat, idx, wall))
                res.setdefault("host_delivery", []).append(entry)
        srv.close()
        report[name] = res
    fit.close()
    return report


class _RingResults:
    """A ck_batch_out view of m tracks over a reused host Results of larger
    capacity (the SoA arrays of m tracks laid out at the start of each
    array; the ring holds 32 events, more than are in flight at half load)."""

    def __init__(self, r, m):
        self.r, self.n = r, m

    def as_batch_out(self):
        return self.r.as_batch_out_view(self.n)


class _Wrap:
    """A ready ck_batch_in for FitServer.submit."""

    def __init__(self, bi):
        self.bi = bi
        self.n = bi.n_tracks

    def as_batch_in(self):
        return self.bi


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--tracks", type=int, default=1000000)
    ap.add_argument("--no-serving", dest="serving", action="store_false",
                    help="skip the serving-loop latency measurement")
    ap.add_argument("--no-events", dest="events", action="store_false",
                    help="skip the batched uneven-events (grid field) measurement")
    ap.add_argument("--no-ckf", dest="ckf", action="store_false",
                    help="skip the track-finding (CKF) measurement")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep the default launch configuration")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    return native_arm(args)


if __name__ == "__main__":
    sys.exit(main())
