"""CK_OUT_PACKED_COV: the per-state covariances as upper triangles (21 values)
carry exactly the values of the full 6x6 layout, for both precision forms,
on every output path — host memory (staged), device memory, chunked host
batches, the serving loop — and through the C++ facade's unfolding."""
import numpy as np
import pytest

from acts_gb300 import abi, generate
from acts_gb300.results import TorchResults

FULL = abi.OUT_ALL
PACKED = abi.OUT_ALL | abi.OUT_PACKED_COV
NAMES = ("predicted_cov", "filtered_cov", "smoothed_cov", "jacobian", "smoothed", "state_flags")


def _same(a, b, n_states, ms):
    valid = np.arange(ms)[None, :] < n_states[:, None]
    for name in NAMES:
        np.testing.assert_array_equal(a.view(name)[valid], b.view(name)[valid], err_msg=name)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED],
                         ids=["fp64", "mixed"])
def test_packed_covariances_equal_full(fitter_factory, precision):
    from conftest import batch

    fit = fitter_factory(abi.CKG_UNEVEN)
    b = batch(abi.CKG_UNEVEN, 3000, seed=41)
    opt = abi.default_options(precision=precision, outlier_chi2_cut=15.0)
    full = fit.fit_batch(b, opt, max_states=22, components=FULL)
    packed = fit.fit_batch(b, opt, max_states=22, components=PACKED)
    assert packed.smoothed_cov.size * 36 == full.smoothed_cov.size * 21
    np.testing.assert_array_equal(full.status, packed.status)
    _same(full, packed, full.n_states, 22)
    # device-resident outputs
    dev = TorchResults(b.n, 22, PACKED, device="cuda:0")
    fit.fit_batch_raw(opt, b.as_batch_in(), dev.as_batch_out())
    fit.sync()
    _same(full, dev.to_host(), full.n_states, 22)


@pytest.mark.gpu
def test_packed_covariances_chunked_host_batch():
    from acts_gb300.fitter import CudaKalman

    det = generate.Detector(abi.CKG_BARREL)
    b = generate.generate(det, 300000, seed=43)
    opt = abi.default_options(precision=abi.PRECISION_MIXED)
    comps = abi.OUT_SMOOTHED
    fit = CudaKalman.for_detector(det)
    fit.set_host_chunk_tracks(120000)  # three chunks
    try:
        full = fit.fit_batch(b, opt, max_states=10, components=comps)
        packed = fit.fit_batch(b, opt, max_states=10, components=comps | abi.OUT_PACKED_COV)
    finally:
        fit.close()
    valid = np.arange(10)[None, :] < full.n_states[:, None]
    for name in ("smoothed", "smoothed_cov"):
        np.testing.assert_array_equal(full.view(name)[valid], packed.view(name)[valid])


@pytest.mark.gpu
def test_packed_covariances_serving_loop():
    from acts_gb300.fitter import CudaKalman
    from acts_gb300.serving import FitServer

    det = generate.Detector(abi.CKG_UNEVEN)
    opt = abi.default_options(precision=abi.PRECISION_MIXED, outlier_chi2_cut=15.0)
    events = [generate.generate(det, m, seed=50 + i) for i, m in enumerate((500, 2000, 700))]
    fit = CudaKalman.for_detector(det)
    try:
        ref = [fit.fit_batch(e, opt, max_states=22, components=abi.OUT_SMOOTHED) for e in events]
        srv = FitServer(fit, opt, memory_budget_bytes=4 << 30, n_streams=2, max_states=22,
                        components=abi.OUT_SMOOTHED | abi.OUT_PACKED_COV)
        try:
            for i, e in enumerate(events):
                srv.submit(i, e)
            got = {}
            while len(got) < len(events):
                r = srv.poll(timeout_ms=5000)
                assert r is not None
                got[r[0]] = r[1]
        finally:
            srv.close()
    finally:
        fit.close()
    for i, r in enumerate(ref):
        np.testing.assert_array_equal(r.status, got[i].status)
        valid = np.arange(22)[None, :] < r.n_states[:, None]
        for name in ("smoothed", "smoothed_cov"):
            np.testing.assert_array_equal(r.view(name)[valid], got[i].view(name)[valid])
