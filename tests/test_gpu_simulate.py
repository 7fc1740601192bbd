"""ck_simulate: the generator's truth simulation and digitisation run on the
GPU (one thread per track, the host generator's source) against the host
generator with the same seed. The device evaluates its own libm and
contracts multiply-adds, so values differ in the last bits; the structure
of a track (its surfaces, measurements, subspaces, outlier flags) follows
from random draws and geometry tests and matches for all but a few tracks
whose trajectory passes within rounding of a decision (a layer edge)."""
import numpy as np
import pytest

from acts_gb300 import abi, generate
from acts_gb300.results import Results

PRESETS = [(abi.CKG_TELESCOPE, 5000), (abi.CKG_BARREL, 20000), (abi.CKG_UNEVEN, 20000),
           (abi.CKG_STRIPS, 20000)]


def _rows(b, name, width, t):
    off = b.meas_offsets if name != "seq_surfaces" else b.seq_offsets
    return np.asarray(getattr(b, name)).reshape(-1, width)[off[t]:off[t + 1]]


@pytest.mark.gpu
@pytest.mark.parametrize("preset,n", PRESETS, ids=["telescope", "barrel", "uneven", "strips"])
def test_device_generation_matches_host(preset, n):
    from acts_gb300.fitter import CudaKalman

    det = generate.Detector(preset)
    host = generate.generate(det, n, seed=61, first_track=1000)
    fit = CudaKalman.for_detector(det)
    try:
        dev = fit.simulate(preset, n, seed=61, first_track=1000).to_host()
    finally:
        fit.close()
    ns_h, ns_d = np.diff(host.seq_offsets), np.diff(dev.seq_offsets)
    nm_h, nm_d = np.diff(host.meas_offsets), np.diff(dev.meas_offsets)
    same = (ns_h == ns_d) & (nm_h == nm_d)
    for t in np.nonzero(same)[0]:
        if not (np.array_equal(_rows(host, "seq_surfaces", 1, t), _rows(dev, "seq_surfaces", 1, t))
                and np.array_equal(_rows(host, "meas_surfaces", 1, t),
                                   _rows(dev, "meas_surfaces", 1, t))
                and np.array_equal(_rows(host, "meas_outlier", 1, t),
                                   _rows(dev, "meas_outlier", 1, t))):
            same[t] = False
    print("tracks with identical structure: %d of %d" % (same.sum(), n))
    assert same.sum() >= n - max(2, n // 2000)
    np.testing.assert_array_equal(host.particle_pdg, dev.particle_pdg)
    np.testing.assert_array_equal(host.particle, dev.particle)
    # values of the identically structured tracks
    rel = lambda a, b, s: float(np.max(np.abs(a - b) / np.maximum(np.abs(b), s), initial=0.0))
    sp = rel(dev.start_params.reshape(n, 6)[same], host.start_params.reshape(n, 6)[same], 1.0)
    sc = rel(dev.start_cov.reshape(n, 36)[same], host.start_cov.reshape(n, 36)[same], 1e-300)
    fr = rel(dev.start_frames.reshape(n, 12)[same], host.start_frames.reshape(n, 12)[same], 1.0)
    idx = np.concatenate([np.arange(host.meas_offsets[t], host.meas_offsets[t + 1])
                          for t in np.nonzero(same)[0]])
    mv = rel(dev.meas_values.reshape(-1, 2)[idx], host.meas_values.reshape(-1, 2)[idx], 1.0)
    tm = rel(dev.truth_meas.reshape(-1, 6)[idx], host.truth_meas.reshape(-1, 6)[idx], 1.0)
    np.testing.assert_array_equal(dev.meas_cov.reshape(-1, 4)[idx], host.meas_cov.reshape(-1, 4)[idx])
    if preset == abi.CKG_STRIPS:
        np.testing.assert_array_equal(dev.meas_subspace[idx], host.meas_subspace[idx])
    print("max relative differences: start %.2e cov %.2e frame %.2e meas %.2e truth %.2e"
          % (sp, sc, fr, mv, tm))
    assert max(sp, sc, fr) <= 1e-12
    assert max(mv, tm) <= 1e-9


@pytest.mark.gpu
def test_device_batch_fits_in_place():
    """A device-generated batch is fitted from device memory without a host
    round trip and gives the fit of its host copy."""
    from acts_gb300.fitter import CudaKalman
    from acts_gb300.results import TorchResults

    det = generate.Detector(abi.CKG_BARREL)
    fit = CudaKalman.for_detector(det)
    try:
        dev = fit.simulate(abi.CKG_BARREL, 5000, seed=62)
        opt = abi.default_options()
        out = TorchResults(dev.n, 12, abi.OUT_SMOOTHED, device="cuda:0")
        fit.fit_batch_raw(opt, dev.as_batch_in(), out.as_batch_out())
        fit.sync()
        on_dev = out.to_host()
        host = fit.fit_batch(dev.to_host(), opt, max_states=12, components=abi.OUT_SMOOTHED)
    finally:
        fit.close()
    np.testing.assert_array_equal(on_dev.status, host.status)
    assert (host.status == 0).mean() > 0.99
    valid = np.arange(12)[None, :] < host.n_states[:, None]
    np.testing.assert_array_equal(on_dev.view("smoothed")[valid], host.view("smoothed")[valid])
