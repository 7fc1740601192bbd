"""A fixed fit case for profilers (ncu launch lists and kernel captures).

    python -m acts_gb300.profile_case --preset barrel --tracks 20000 --precision fp64,mixed

Generates the preset's tracks, fits them once per requested precision
(graph capture off, so every kernel is an ordinary launch) and prints the
kernel time of each fit. Profile summaries under profiles/ name the exact
command line they were produced with.
"""
import argparse
import sys

from . import abi, generate
from .fitter import CudaKalman

PRESETS = {"telescope": abi.CKG_TELESCOPE, "barrel": abi.CKG_BARREL, "uneven": abi.CKG_UNEVEN}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--preset", default="barrel", choices=sorted(PRESETS))
    ap.add_argument("--tracks", type=int, default=20000)
    ap.add_argument("--precision", default="fp64,mixed")
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--max-states", type=int, default=0)
    ap.add_argument("--variant", type=int, default=-1,
                    help="forward-filter kernel variant (default: the handle's default)")
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--blocks-per-sm", type=int, default=0)
    ap.add_argument("--perigee", action="store_true",
                    help="extrapolate to a perigee surface at the origin")
    ap.add_argument("--reverse", action="store_true", help="reverse filtering")
    a = ap.parse_args(argv)
    preset = PRESETS[a.preset]
    det = generate.Detector(preset, perigee=a.perigee)
    b = generate.generate(det, a.tracks, seed=a.seed)
    ms = a.max_states or (10 if preset != abi.CKG_UNEVEN else 20)
    fit = CudaKalman.for_detector(det, use_graph=False)
    for name in a.precision.split(","):
        prec = abi.PRECISION_MIXED if name == "mixed" else abi.PRECISION_FP64
        if a.variant >= 0:
            fit.set_launch_config(prec, a.variant, a.threads, a.blocks_per_sm)
        opt = abi.default_options(precision=prec,
                                  outlier_chi2_cut=15.0 if preset == abi.CKG_UNEVEN else float("inf"),
                                  reference_surface=det.perigee, reverse_filtering=int(a.reverse))
        comps = abi.OUT_SMOOTHED | (abi.OUT_REFERENCE if a.perigee else 0)
        for _ in range(a.repeat):
            fit.fit_batch(b, opt, max_states=ms, components=comps)
            print("%s %s %d tracks: kernel %.3f ms" % (a.preset, name, a.tracks, fit.last_kernel_ms()))
    fit.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
