"""Smoothing in the forward filter's tail (ck_set_tail_smoothing): blocks of
the compaction kernels whose tracks have all ended smooth finished tracks
while the last ones still propagate; the smoother kernel takes the rest.
The results equal those of the smoother kernel alone, bit for bit, in both
forms, for the RTS and MBF smoothers, with the free-to-bound correction, with
the extrapolation to a reference surface, through the device-resident (CUDA
graph) and chunked host paths, and for both compaction variants."""
import numpy as np
import pytest

from acts_gb300 import abi, generate

SCALARS = ("status", "n_states", "n_measurements", "n_holes", "n_outliers", "ndf", "chi2_sum")


def _same(a, b, ms):
    for name in a.ARRAYS:
        x, y = getattr(a, name), getattr(b, name)
        if x is None:
            assert y is None, name
            continue
        if name in SCALARS:
            np.testing.assert_array_equal(x, y, err_msg=name)
        elif name in ("track_params", "track_cov"):
            ok = b.status == 0
            np.testing.assert_array_equal(a.track(name)[ok], b.track(name)[ok], err_msg=name)
        else:
            valid = np.arange(ms)[None, :] < b.n_states[:, None]
            np.testing.assert_array_equal(a.view(name)[valid], b.view(name)[valid], err_msg=name)


CASES = [
    ("barrel_mixed", abi.CKG_BARREL, dict(precision=abi.PRECISION_MIXED), 3),
    ("barrel_fp64", abi.CKG_BARREL, dict(precision=abi.PRECISION_FP64), 3),
    ("uneven_mixed_mbf", abi.CKG_UNEVEN,
     dict(precision=abi.PRECISION_MIXED, outlier_chi2_cut=15.0, smoother=abi.SMOOTHER_MBF), 3),
    ("uneven_fp64_v4", abi.CKG_UNEVEN, dict(precision=abi.PRECISION_FP64, outlier_chi2_cut=15.0), 4),
    ("strips_mixed_f2b", abi.CKG_STRIPS,
     dict(precision=abi.PRECISION_MIXED, free_to_bound_correction=1), 3),
    ("barrel_perigee", abi.CKG_BARREL, dict(precision=abi.PRECISION_MIXED, reference="perigee"), 3),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,preset,kw,variant", CASES, ids=[c[0] for c in CASES])
def test_tail_smoothing_changes_nothing(name, preset, kw, variant):
    from acts_gb300.fitter import CudaKalman

    kw = dict(kw)
    perigee = kw.pop("reference", None) == "perigee"
    det = generate.Detector(preset, perigee=perigee)
    b = generate.generate(det, 30000, seed=71)
    if perigee:
        kw["reference_surface"] = det.perigee
    opt = abi.default_options(**kw)
    comps = abi.OUT_ALL | (abi.OUT_REFERENCE if perigee else 0)
    fit = CudaKalman.for_detector(det)
    try:
        fit.set_launch_config(kw["precision"], variant, 256 if variant == 3 else 128, 1)
        fit.set_tail_smoothing(0)
        ref = fit.fit_batch(b, opt, max_states=24, components=comps)
        fit.set_tail_smoothing(1)
        got = fit.fit_batch(b, opt, max_states=24, components=comps)
    finally:
        fit.close()
    # (the uneven workload's tracks that leave the field map fail, as the reference's)
    assert (ref.status == 0).mean() > 0.5
    _same(got, ref, 24)


@pytest.mark.gpu
def test_tail_smoothing_device_graph_and_chunked_host():
    from acts_gb300.fitter import CudaKalman
    from acts_gb300.results import TorchResults

    det = generate.Detector(abi.CKG_BARREL)
    opt = abi.default_options(precision=abi.PRECISION_MIXED)
    comps = abi.OUT_SMOOTHED | abi.OUT_PACKED_COV
    fit = CudaKalman.for_detector(det)
    try:
        dev = fit.simulate(abi.CKG_BARREL, 200000, seed=72)
        b = dev.to_host()
        fit.set_tail_smoothing(0)
        fit.set_host_chunk_tracks(-1)
        ref = fit.fit_batch(b, opt, max_states=12, components=comps)
        fit.set_tail_smoothing(1)
        fit.set_host_chunk_tracks(60000)  # four chunks
        chunked = fit.fit_batch(b, opt, max_states=12, components=comps)
        out = TorchResults(dev.n, 12, comps, device="cuda:0")
        on_dev = []
        for _ in range(2):  # capture, then replay of the CUDA graph
            fit.fit_batch_raw(opt, dev.as_batch_in(), out.as_batch_out())
            fit.sync()
            on_dev.append(out.to_host())
    finally:
        fit.close()
    _same(chunked, ref, 12)
    for r in on_dev:
        _same(r, ref, 12)
