"""Where the time of a small fit launch goes: forward-filter and smoother
kernel times of one 10,000-track event of the uneven workload against
subsets of it (its tracks of more than 100 steps, one long track, 2,000
short tracks, one short track), with the grid field map and with a constant
2 T field, both forms, with and without early termination:

    python -m acts_gb300.launch_latency            # the table
    python -m acts_gb300.launch_latency --one-track [fp64]
                                                   # one 12-state track, three
                                                   # fits (the ncu capture case)

Device-resident batches, CUDA graph capture on, median of three fits after
two warm-up fits. The tracks of more than 100 steps are those an FP64 fit
with a 100-step limit stops with StepCountLimitReached.
"""
import ctypes as C
import sys

import numpy as np

from . import abi, generate

_ARRAYS = (("seq_offsets", C.c_int32), ("seq_surfaces", C.c_int32),
           ("meas_offsets", C.c_int32), ("meas_surfaces", C.c_int32),
           ("meas_values", C.c_double), ("meas_cov", C.c_double),
           ("meas_subspace", C.c_int32), ("start_params", C.c_double),
           ("start_cov", C.c_double), ("start_frames", C.c_double),
           ("particle", C.c_float), ("particle_pdg", C.c_int32))


def device_batch(b, torch, dev):
    """The batch's arrays in device memory: (ck_batch_in, tensors to keep)."""
    keep = {}
    bi = abi.ck_batch_in()
    bi.n_tracks = b.n
    bi.memory = abi.MEM_DEVICE
    for name, ct in _ARRAYS:
        v = getattr(b, name)
        if v is None:
            continue
        t = torch.from_numpy(np.ascontiguousarray(v)).to(dev)
        keep[name] = t
        setattr(bi, name, C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ct)))
    return bi, keep


def _time(fit, opt, bi, bo, warm=2, reps=3):
    for _ in range(warm):
        fit.fit_batch_raw(opt, bi, bo)
    fit.sync()
    ts = []
    for _ in range(reps):
        fit.fit_batch_raw(opt, bi, bo)
        fit.sync()
        ts.append(fit.last_kernel_split_ms())
    return float(np.median([t[0] for t in ts])), float(np.median([t[1] for t in ts]))


def one_track(precision):
    import torch

    from .fitter import CudaKalman
    from .results import TorchResults

    det = generate.Detector(abi.CKG_UNEVEN)
    b = generate.generate(det, 64, seed=77)
    ns = np.diff(np.asarray(b.seq_offsets))
    one = b.subset([int(np.nonzero(ns == 12)[0][0])])
    dev = torch.device("cuda", 0)
    bi, keep = device_batch(one, torch, dev)
    fit = CudaKalman.for_detector(det, use_graph=False)
    opt = abi.default_options(precision=precision, outlier_chi2_cut=15.0, early_termination=1)
    out = TorchResults(1, 20, abi.OUT_SMOOTHED | abi.OUT_PACKED_COV, device=dev)
    bo = out.as_batch_out()
    for _ in range(3):
        fit.fit_batch_raw(opt, bi, bo)
        fit.sync()
        print("filter, smoother ms", fit.last_kernel_split_ms(), flush=True)
    fit.close()


def table():
    import torch

    from .fitter import CudaKalman
    from .results import TorchResults

    dev = torch.device("cuda", 0)
    det = generate.Detector(abi.CKG_UNEVEN)
    b = generate.generate(det, 10000, seed=77)
    fit = CudaKalman.for_detector(det)
    r = fit.fit_batch(b, abi.default_options(outlier_chi2_cut=15.0, max_steps=100),
                      max_states=22)
    fit.close()
    long_idx = np.nonzero(np.asarray(r.status) == abi.TRACK_STEP_COUNT_LIMIT)[0]
    rng = np.random.default_rng(1)
    short_idx = rng.choice(np.setdiff1d(np.arange(10000), long_idx), 2000, replace=False)
    print("tracks of more than 100 steps: %d of 10000" % len(long_idx), flush=True)
    fconst = abi.ck_field()
    C.memmove(C.byref(fconst), C.byref(det.field), C.sizeof(abi.ck_field))
    fconst.kind = abi.FIELD_CONSTANT
    fconst.constant_tesla[0], fconst.constant_tesla[1], fconst.constant_tesla[2] = 0.0, 0.0, 2.0
    cases = [("10k event", b), ("its long tracks", b.subset(long_idx)),
             ("1 long track", b.subset(long_idx[:1])), ("2000 short", b.subset(short_idx)),
             ("1 short track", b.subset(short_idx[:1]))]
    for fname, field in (("grid", det.field), ("const", fconst)):
        fit = CudaKalman(det.surfaces, det.n_surfaces, field, use_graph=True)
        for pname, prec in (("mixed", abi.PRECISION_MIXED), ("fp64", abi.PRECISION_FP64)):
            for et in (0, 1):
                opt = abi.default_options(precision=prec, outlier_chi2_cut=15.0,
                                          early_termination=et)
                for cname, bb in cases:
                    bi, keep = device_batch(bb, torch, dev)
                    out = TorchResults(bb.n, 20, abi.OUT_SMOOTHED | abi.OUT_PACKED_COV,
                                       device=dev)
                    f, s = _time(fit, opt, bi, out.as_batch_out())
                    print("%-5s field %-5s early_termination %d %-15s n=%5d: filter %.3f ms, "
                          "smoother %.3f ms" % (fname, pname, et, cname, bb.n, f, s), flush=True)
                    del keep, out
        fit.close()


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if "--one-track" in argv:
        one_track(abi.PRECISION_FP64 if "fp64" in argv else abi.PRECISION_MIXED)
    else:
        table()
    return 0


if __name__ == "__main__":
    sys.exit(main())
