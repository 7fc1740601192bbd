"""The roofline counters pipeline on the host: an ncu raw CSV of forward-
filter and smoother launches becomes per-track counters, written and parsed
back with the kernel-source hash; the bench adds the launched filter's line
and the smoother's; its variant-to-kernel table covers every variant of both
forms."""
import io
import os
import sys
from contextlib import redirect_stdout

from acts_gb300 import profile_counters as pc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _csv(tmp_path):
    cols = ["ID", "Kernel Name"] + list(pc.METRICS)
    units = ["", ""] + ["" for _ in pc.METRICS]
    vals = {"gpu__time_duration.sum": "2,000,000", "dram__bytes_read.sum": "3000000",
            "dram__bytes_write.sum": "1000000",
            "smsp__sass_thread_inst_executed_op_dfma_pred_on.sum": "1000",
            "smsp__sass_thread_inst_executed_op_dadd_pred_on.sum": "500",
            "smsp__sass_thread_inst_executed_op_dmul_pred_on.sum": "250",
            "smsp__sass_thread_inst_executed_op_ffma_pred_on.sum": "4000",
            "smsp__sass_thread_inst_executed_op_fadd_pred_on.sum": "10",
            "smsp__sass_thread_inst_executed_op_fmul_pred_on.sum": "20",
            "smsp__sass_thread_inst_executed_op_conversion_pred_on.sum": "100",
            "sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active": "55.5",
            "sm__warps_active.avg.pct_of_peak_sustained_active": "12.5"}
    q = lambda xs: ",".join('"%s"' % x for x in xs)
    rows = [q(cols), q(units),
            q(["0", "void ck::fitKernelPool<float, float, 384, 256>(ck::FitParams)"] +
              [vals[m] for m in pc.METRICS]),
            q(["1", "void ck::smoothKernel<float, 128>(ck::FitParams)"] +
              [vals[m] for m in pc.METRICS])]
    p = tmp_path / "prof.csv"
    p.write_text("==PROF== note\n" + "\n".join(rows) + "\n")
    return str(p)


def test_counters_round_trip(tmp_path):
    path = _csv(tmp_path)
    buf = io.StringIO()
    with redirect_stdout(buf):
        pc.main(["--csv", path, "--tracks", "10", "--command", "ncu ..."])
    out = tmp_path / "counters.txt"
    out.write_text(buf.getvalue())
    src, lines = pc.parse(str(out))
    assert src == pc.source_hash()
    assert len(lines) == 2  # the forward filter and the smoother
    assert "smoothKernel<float, 128>" in lines[1]["kernel"]
    ln = lines[0]
    assert "fitKernelPool<float, float, 384, 256>" in ln["kernel"]
    assert ln["fp64_flops"] == (2 * 1000 + 500 + 250) / 10
    assert ln["fp32_flops"] == (2 * 4000 + 10 + 20) / 10
    assert ln["dram_bytes"] == 4000000 / 10
    assert abs(ln["fp64_pipe_busy"] - 0.555) < 1e-12
    assert abs(ln["duration_ms"] - 2.0) < 1e-12


def test_bench_names_every_variant():
    sys.path.insert(0, ROOT)
    import bench

    with open(os.path.join(ROOT, "acts_gb300", "csrc", "ck_launch.h")) as f:
        text = f.read()
    n = int(text.split("constexpr int kNumFitVariants = ")[1].split(";")[0])
    for scalar in ("float", "double"):
        assert sorted(bench._VARIANT_KERNELS[scalar]) == list(range(n))


def test_bench_matches_ncu_kernel_names(tmp_path, monkeypatch):
    """ncu prints template booleans as 0/1: the bench finds the launched
    variant's line either way, and only while the source hash matches."""
    sys.path.insert(0, ROOT)
    import bench

    out = tmp_path / "counters.txt"
    out.write_text("source %s\n"
                   "kernel=void fitKernelCompact<float, float, 256, 0, 0>(FitParams) | "
                   "fp64_flops=8722.0 fp32_flops=33411.7 dram_bytes=6058.6 conversions=1655.8 "
                   "fp64_pipe_busy=0.574 warps_active=0.125 duration_ms=12.900\n"
                   "kernel=void smoothKernel<float, 128>(FitParams) | "
                   "fp64_flops=10.0 fp32_flops=20.0 dram_bytes=30.0 conversions=1.0 "
                   "fp64_pipe_busy=0.1 warps_active=0.1 duration_ms=0.040\n"
                   "kernel=void fitKernelCompact<double, double, 256, 0, 0>(FitParams) | "
                   "fp64_flops=43871.1 fp32_flops=2626.1 dram_bytes=10252.2 conversions=314.9 "
                   "fp64_pipe_busy=0.644 warps_active=0.125 duration_ms=41.876\n"
                   % pc.source_hash())
    monkeypatch.setattr(bench, "COUNTERS", str(out))
    ln, name = bench.kernel_counters("float", 3)
    # (the filter's line plus the smoother's)
    assert ln is not None and ln["fp64_flops"] == 8732.0 and ln["dram_bytes"] == 6088.6, name
    assert ln["fp64_pipe_busy"] == 0.574 and "smoothKernel<float, 128>" in name
    ln, why = bench.kernel_counters("double", 3)
    assert ln is None and "no capture of smoothKernel<double, 128>" in why
    out.write_text(out.read_text().replace(pc.source_hash(), "0" * 16))
    ln, why = bench.kernel_counters("float", 3)
    assert ln is None and "other kernel sources" in why
