"""Launch shapes of the serving loop's co-batches, timed on the serving
configuration (mixed form):

    python -m acts_gb300.serving_sweep [label substrings ...]

Events of log-uniform 100-20,000 tracks of the uneven workload arrive as a
Poisson process; each configuration (forward-filter variant, threads per
block, resident blocks per SM, stream slots, co-batch grid, Runge-Kutta
trials per round) is measured by saturation (2,000 events back to back),
then at 10/30/50/80 % of a fixed 11.4 M tracks/s (the default shape's
capacity), 3,000 events per load, results to device memory. Prints one JSON
line per configuration: capacity, and per load the sustained tracks/s and
the p50/p99 latency of all events and of the 8,000-12,000-track events.
Results do not depend on any of the knobs swept.
"""
import json
import sys
import threading
import time

import numpy as np

# (label, variant, threads per block, blocks per SM, streams, grid blocks,
#  trials per round); 0 = the server's automatic choice
CONFIGS = [
    ("v3 bps1 s3 auto", 3, 256, 1, 3, 0, 0),
    ("v4 bps2 s3 auto", 4, 128, 2, 3, 0, 0),
    ("v4 bps2 s3 g304", 4, 128, 2, 3, 304, 0),
    ("v4 bps2 s4 auto", 4, 128, 2, 4, 0, 0),
    ("v4 bps2 s5 auto", 4, 128, 2, 5, 0, 0),
    ("v4 bps2 s3 auto spr12", 4, 128, 2, 3, 0, 12),
    ("v3 bps1 s2 g152", 3, 256, 1, 2, 152, 0),
    ("v1 128 bps3 s4 auto", 1, 128, 3, 4, 0, 0),
    ("v2 128 bps4 s5 auto", 2, 128, 4, 5, 0, 0),
]
REFERENCE_CAPACITY = 11.4e6  # tracks/s: the offered loads are fractions of it


def main(argv=None):
    import torch

    from . import abi, generate
    from .fitter import CudaKalman
    from .results import TorchResults
    from .serving import FitServer

    sys.path.insert(0, ".")
    import bench

    argv = sys.argv[1:] if argv is None else argv
    configs = [c for c in CONFIGS if not argv or any(a in c[0] for a in argv)]
    n_events, seed, max_states, pool_tracks, lo, hi = 10000, 77, 20, 400000, 100, 20000
    det = generate.Detector(abi.CKG_UNEVEN)
    pool = bench.EventPool(generate.generate(det, pool_tracks, seed=seed), torch)
    sizes = generate.event_sizes(seed, n_events, -1.0, lo, hi)
    rng = np.random.default_rng(seed)
    starts = rng.integers(0, pool_tracks - hi, n_events)
    mean = float(sizes.mean())
    comps = abi.OUT_SMOOTHED | abi.OUT_PACKED_COV

    for label, var, tpb, bps, ns, grid, spr in configs:
        fit = CudaKalman.for_detector(det)
        fit.set_launch_config(abi.PRECISION_MIXED, var, tpb, bps)
        opt = abi.default_options(precision=abi.PRECISION_MIXED, outlier_chi2_cut=15.0)
        srv = FitServer(fit, opt, memory_budget_bytes=40 << 30, n_streams=ns,
                        max_states=max_states, max_batch_tracks=8 * hi, components=comps,
                        grid_blocks=grid, steps_per_round=spr)

        def run(idx, rate):
            lat, done, held = {}, threading.Event(), {}

            def poller():
                try:
                    while len(lat) < len(idx):
                        r = srv.poll(timeout_ms=200)
                        if r is not None:
                            lat[r[0]] = r[2]
                            held.pop(r[0], None)
                finally:
                    done.set()

            threading.Thread(target=poller, daemon=True).start()
            t0 = time.perf_counter()
            gaps = rng.exponential(1.0 / rate, len(idx)) if rate else np.zeros(len(idx))
            t_next = t0
            for k, i in enumerate(idx):
                t_next += gaps[k]
                while True:
                    dt = t_next - time.perf_counter()
                    if dt <= 0:
                        break
                    time.sleep(min(dt, 0.0005))
                bi, keep = pool.event(int(starts[i]), int(sizes[i]))
                res = TorchResults(int(sizes[i]), max_states, comps, device="cuda:0")
                held[int(i)] = (keep, res)
                srv.submit(int(i), bench._Wrap(bi), res)
            done.wait(600)
            return lat, time.perf_counter() - t0

        def stats(lat, idx, wall):
            v = np.array([lat[int(i)] for i in idx])
            m = sizes[idx]
            sel = (m >= 8000) & (m <= 12000)
            pick = lambda q, a: round(float(np.percentile(a, q)), 2)  # noqa: E731
            return {"tps": round(float(m.sum()) / wall / 1e6, 2), "p50": pick(50, v),
                    "p99": pick(99, v),
                    "p50_10k": pick(50, v[sel]) if sel.sum() > 9 else None,
                    "p99_10k": pick(99, v[sel]) if sel.sum() > 9 else None}

        run(np.arange(50), 0)
        idx = np.arange(2000)
        lat, wall = run(idx, 0)
        row = {"config": label,
               "capacity_Mtps": round(float(sizes[idx].sum()) / wall / 1e6, 2)}
        for f in (0.1, 0.3, 0.5, 0.8):
            idx = np.arange(3000)
            lat, wall = run(idx, f * REFERENCE_CAPACITY / mean)
            row["%.1f" % f] = stats(lat, idx, wall)
        print(json.dumps(row), flush=True)
        srv.close()
        fit.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
