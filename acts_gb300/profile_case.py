"""A fixed fit case for profilers (ncu launch lists and kernel captures).

    python -m acts_gb300.profile_case --preset barrel --tracks 20000 --precision fp64,mixed
    python -m acts_gb300.profile_case --preset barrel --tracks 10000 --ckf

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
    ap.add_argument("--variant", default="-1",
                    help="forward-filter kernel variant(s), comma-separated, each fitted in "
                         "turn (default: the handle's default)")
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--blocks-per-sm", type=int, default=0)
    ap.add_argument("--perigee", action="store_true",
                    help="extrapolate to a perigee surface at the origin")
    ap.add_argument("--reverse", action="store_true", help="reverse filtering")
    ap.add_argument("--ckf", action="store_true",
                    help="track finding instead of the fit: the tracks as one event of seeds")
    ap.add_argument("--events", type=int, default=1,
                    help="with --ckf: split the tracks into this many events")
    a = ap.parse_args(argv)
    if a.ckf:
        return _ckf(a)
    preset = PRESETS[a.preset]
    det = generate.Detector(preset, perigee=a.perigee)
    b = generate.generate(det, a.tracks, seed=a.seed)
    ms = a.max_states or (10 if preset != abi.CKG_UNEVEN else 20)
    fit = CudaKalman.for_detector(det, use_graph=False)
    for variant in (int(v) for v in a.variant.split(",")):
        for name in a.precision.split(","):
            prec = abi.PRECISION_MIXED if name == "mixed" else abi.PRECISION_FP64
            if variant >= 0:
                tpb = a.threads or (256 if variant in (3, 5, 6) else 128)
                fit.set_launch_config(prec, variant, tpb, a.blocks_per_sm or 1)
            opt = abi.default_options(
                precision=prec,
                outlier_chi2_cut=15.0 if preset == abi.CKG_UNEVEN else float("inf"),
                reference_surface=det.perigee, reverse_filtering=int(a.reverse))
            comps = abi.OUT_SMOOTHED | (abi.OUT_REFERENCE if a.perigee else 0)
            for _ in range(a.repeat):
                fit.fit_batch(b, opt, max_states=ms, components=comps)
                print("%s %s v%d %d tracks: kernel %.3f ms"
                      % (a.preset, name, variant, a.tracks, fit.last_kernel_ms()))
    fit.close()
    return 0


def _ckf(a):
    """Track finding on the preset's tracks (chi2 cut 15, one candidate)."""
    import numpy as np

    preset = PRESETS[a.preset]
    det = generate.Detector(preset)
    b = generate.generate(det, a.tracks, seed=a.seed)
    if a.events > 1:
        sizes = np.full(a.events, a.tracks // a.events)
        sizes[-1] += a.tracks - sizes.sum()
        tf = generate.ckf_events(det, b, sizes, max_states=24, max_tracks=4)
    else:
        tf = generate.ckf_event(det, b, max_states=24, max_tracks=4)
    fit = CudaKalman.for_detector(det, use_graph=False)
    for name in a.precision.split(","):
        prec = abi.PRECISION_MIXED if name == "mixed" else abi.PRECISION_FP64
        opt = abi.default_options(precision=prec)
        ko = tf.options(chi2_cut=15.0, max_branches=8,
                        end_of_world=int(preset == abi.CKG_UNEVEN))
        for _ in range(a.repeat):
            fit.find_tracks(opt, ko, tf)
            print("%s %s track finding, %d seeds in %d events: %d tracks found"
                  % (a.preset, name, a.tracks, a.events, int(tf.n_tracks.sum())))
    fit.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
