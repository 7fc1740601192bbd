"""Per-track hardware counters of the forward-filter kernels and of the
smoother kernel, for the roofline the bench reports (the forward filter
smooths most tracks in its tail; the smoother kernel takes the rest, so the
pair's counters add up to the filter and smoother work of every track).

    python -m acts_gb300.profile_counters --csv prof.csv --tracks 200000 \
        --command "<the ncu command line>" > profiles/fit_kernel_counters.txt

reads an ncu `--csv --page raw` capture of `acts_gb300.profile_case` (the
metrics of METRICS below, forward-filter and smoother launches of known
track count) and writes one line per captured kernel with its per-track
FP64 and FP32 flops (an FMA counts 2; thread-level, predicated-on), DRAM
bytes, FP64-pipe conversions and duration, headed by the hash of the kernel
sources. bench.py uses a line only while the hash matches the sources it
runs and the line's kernel is the one it launched.
"""
import argparse
import csv
import hashlib
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
KERNEL_SOURCES = ("ck_fitter.cuh", "ck_device.cuh", "ck_internal.h", "ck_kernels_mixed.cu",
                  "ck_kernels_fp64.cu")
METRICS = ("gpu__time_duration.sum", "dram__bytes_read.sum", "dram__bytes_write.sum",
           "smsp__sass_thread_inst_executed_op_dfma_pred_on.sum",
           "smsp__sass_thread_inst_executed_op_dadd_pred_on.sum",
           "smsp__sass_thread_inst_executed_op_dmul_pred_on.sum",
           "smsp__sass_thread_inst_executed_op_ffma_pred_on.sum",
           "smsp__sass_thread_inst_executed_op_fadd_pred_on.sum",
           "smsp__sass_thread_inst_executed_op_fmul_pred_on.sum",
           "smsp__sass_thread_inst_executed_op_conversion_pred_on.sum",
           "sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active",
           "sm__warps_active.avg.pct_of_peak_sustained_active")


def source_hash():
    """16 hex digits of the SHA-256 of the forward-filter kernel sources."""
    h = hashlib.sha256()
    for name in KERNEL_SOURCES:
        with open(os.path.join(HERE, "csrc", name), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def _num(x):
    return float(str(x).replace(",", ""))


def summarise(rows, tracks):
    out = []
    for r in rows:
        name = r.get("Kernel Name") or r.get("Function Name") or ""
        if "fitKernel" not in name and "smoothKernel" not in name:
            continue
        g = lambda m: _num(r[m]) if m in r and r[m] not in ("", "n/a") else float("nan")
        fp64 = 2 * g(METRICS[3]) + g(METRICS[4]) + g(METRICS[5])
        fp32 = 2 * g(METRICS[6]) + g(METRICS[7]) + g(METRICS[8])
        dur = g(METRICS[0])
        out.append({"kernel": " ".join(name.split()),
                    "fp64_flops": fp64 / tracks, "fp32_flops": fp32 / tracks,
                    "dram_bytes": (g(METRICS[1]) + g(METRICS[2])) / tracks,
                    "conversions": g(METRICS[9]) / tracks,
                    "fp64_pipe_busy": g(METRICS[10]) / 100.0,
                    "warps_active": g(METRICS[11]) / 100.0,
                    "duration_ms": dur / 1e6 if dur > 1e5 else dur})
    return out


def read_rows(path):
    with open(path, newline="") as f:
        lines = [ln for ln in f if ln.startswith('"')]
    rd = csv.DictReader(lines)
    rows = [r for r in rd]
    # (the raw page's second row holds the units)
    return [r for r in rows if r.get("ID", "").strip().isdigit()]


def parse(path):
    """The kernel lines of a counters file: (source hash, [dict])."""
    src, out = None, []
    with open(path) as f:
        for ln in f:
            ln = ln.strip()
            if ln.startswith("source "):
                src = ln.split()[1]
            elif ln.startswith("kernel="):
                kv = {}
                head, rest = ln.split(" | ", 1)
                kv["kernel"] = head[len("kernel="):]
                for item in rest.split():
                    k, v = item.split("=")
                    kv[k] = float(v)
                out.append(kv)
    return src, out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--csv", required=True)
    ap.add_argument("--tracks", type=int, required=True)
    ap.add_argument("--command", required=True)
    a = ap.parse_args(argv)
    rows = summarise(read_rows(a.csv), a.tracks)
    print("# Forward-filter and smoother kernels: per-track counters from one ncu capture (%d tracks)"
          % a.tracks)
    print("# command: %s" % a.command)
    print("# flops count an FMA as 2 (thread-level, predicated-on lanes); dram = read + write")
    print("source %s" % source_hash())
    for r in rows:
        print("kernel=%s | fp64_flops=%.1f fp32_flops=%.1f dram_bytes=%.1f conversions=%.1f "
              "fp64_pipe_busy=%.3f warps_active=%.3f duration_ms=%.3f"
              % (r["kernel"], r["fp64_flops"], r["fp32_flops"], r["dram_bytes"],
                 r["conversions"], r["fp64_pipe_busy"], r["warps_active"], r["duration_ms"]))
    return 0


if __name__ == "__main__":
    sys.exit(main())
