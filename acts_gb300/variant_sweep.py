"""Times every forward-filter kernel variant, Runge-Kutta trials per round
and smoother staging on fixed workloads (device-resident batches, graph
capture on), the manual sibling of ck_autotune:

    python -m acts_gb300.variant_sweep --cases barrel,uneven,uneven10k

Prints one line per configuration with the forward-filter and smoother
kernel times (median of three fits after two warm-up fits) and the tracks/s
they imply. Results do not depend on any of the knobs swept.
"""
import argparse
import ctypes as C
import sys

import numpy as np

from . import abi, generate
from .fitter import CudaKalman

# name: (preset, tracks, max states, option overrides)
CASES = {
    "barrel": (abi.CKG_BARREL, 1000000, 10, {}),
    "uneven": (abi.CKG_UNEVEN, 250000, 20, {"outlier_chi2_cut": 15.0}),
    "uneven10k": (abi.CKG_UNEVEN, 10000, 20, {"outlier_chi2_cut": 15.0}),
}


def _device_batch(b, torch, dev):
    """The batch's arrays in device memory: (ck_batch_in, tensors to keep)."""
    keep = {}
    bi = abi.ck_batch_in()
    bi.n_tracks = b.n
    bi.memory = abi.MEM_DEVICE
    for name, ct in (("seq_offsets", C.c_int32), ("seq_surfaces", C.c_int32),
                     ("meas_offsets", C.c_int32), ("meas_surfaces", C.c_int32),
                     ("meas_values", C.c_double), ("meas_cov", C.c_double),
                     ("meas_subspace", C.c_int32), ("start_params", C.c_double),
                     ("start_cov", C.c_double), ("start_frames", C.c_double),
                     ("particle", C.c_float), ("particle_pdg", C.c_int32)):
        t = torch.from_numpy(np.ascontiguousarray(getattr(b, name))).to(dev)
        keep[name] = t
        setattr(bi, name, C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ct)))
    return bi, keep


def main(argv=None):
    import torch

    from .results import TorchResults

    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--cases", default="barrel,uneven,uneven10k")
    ap.add_argument("--variants", default="3,5,6")
    ap.add_argument("--precision", default="mixed,fp64")
    ap.add_argument("--seed", type=int, default=7)
    a = ap.parse_args(argv)
    dev = torch.device("cuda", 0)
    for name in a.cases.split(","):
        preset, n, ms, kw = CASES[name]
        det = generate.Detector(preset)
        b = generate.generate(det, n, seed=a.seed)
        fit = CudaKalman.for_detector(det, use_graph=True)
        bi, keep = _device_batch(b, torch, dev)
        out = TorchResults(n, ms, abi.OUT_SMOOTHED | abi.OUT_PACKED_COV, device=dev)
        bo = out.as_batch_out()
        try:
            for pname in a.precision.split(","):
                prec = abi.PRECISION_MIXED if pname == "mixed" else abi.PRECISION_FP64
                opt = abi.default_options(precision=prec, **kw)
                for v in (int(x) for x in a.variants.split(",")):
                    for spr in (2, 3, 4):
                        for stg in ((0, 1) if spr == 3 else (0,)):
                            fit.set_launch_config(prec, v, 256, 1)
                            fit.set_steps_per_round(prec, spr)
                            fit.set_smoother_staging(prec, stg)
                            for _ in range(2):
                                fit.fit_batch_raw(opt, bi, bo)
                            fit.sync()
                            ts = []
                            for _ in range(3):
                                fit.fit_batch_raw(opt, bi, bo)
                                fit.sync()
                                ts.append(fit.last_kernel_split_ms())
                            f = float(np.median([t[0] for t in ts]))
                            sm = float(np.median([t[1] for t in ts]))
                            print("%s %s v%d spr%d stg%d: filter %.3f ms smoother %.3f ms -> %.4g "
                                  "tracks/s" % (name, pname, v, spr, stg, f, sm,
                                                n / ((f + sm) / 1e3)), flush=True)
        finally:
            fit.close()
            del keep
    return 0


if __name__ == "__main__":
    sys.exit(main())
