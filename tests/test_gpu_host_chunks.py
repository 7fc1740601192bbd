"""Large host-memory batches run as chunks whose transfers overlap the fits
of their neighbours (ck_fit_batch, both sides in host memory, at least two
chunks): the outputs equal those of the same tracks fitted in calls below the
chunking size, bit for bit, in the caller's SoA layout, for every output
component, with reverse filtering and with the extrapolation to a reference
surface. Host CSR offsets that are not a non-decreasing partition are
rejected."""
import numpy as np
import pytest

from acts_gb300 import abi, generate
from acts_gb300.results import Results

N = 600000


@pytest.mark.gpu
@pytest.mark.parametrize("precision,reverse", [(abi.PRECISION_MIXED, 0), (abi.PRECISION_FP64, 0),
                                               (abi.PRECISION_MIXED, 1)],
                         ids=["mixed", "fp64", "mixed_reverse_filtering"])
def test_chunked_host_batch_equals_unchunked(precision, reverse):
    from acts_gb300.fitter import CudaKalman

    det = generate.Detector(abi.CKG_BARREL, perigee=True)
    b = generate.generate(det, N, seed=31)
    opt = abi.default_options(precision=precision, reference_surface=det.perigee,
                              outlier_chi2_cut=15.0, reverse_filtering=reverse)
    comps = abi.OUT_SMOOTHED | abi.OUT_REFERENCE
    fit = CudaKalman.for_detector(det)
    fit.set_host_chunk_tracks(250000)  # three chunks
    try:
        whole = fit.fit_batch(b, opt, max_states=10, components=comps)
        assert fit.last_kernel_ms() > 0
        h2d, d2h = fit.last_transfer_bytes()
        assert h2d > 0 and d2h > 0
        halves = [np.arange(0, N // 2), np.arange(N // 2, N)]
        parts = [fit.fit_batch(b.subset(i), opt, max_states=10, components=comps) for i in halves]
    finally:
        fit.close()
    assert (whole.status == 0).mean() > 0.99
    for name in ("status", "n_states", "n_measurements", "ndf", "chi2_sum"):
        np.testing.assert_array_equal(getattr(whole, name),
                                      np.concatenate([getattr(p, name) for p in parts]))
    # (state slots past a track's n_states are not written)
    for name in ("state_flags", "state_surface", "smoothed", "smoothed_cov"):
        a = whole.view(name)
        for i, p in zip(halves, parts):
            valid = np.arange(10)[None, :] < p.n_states[:, None]
            # (reverse filtering: NaN where a state has no smoothed parameters)
            np.testing.assert_array_equal(a[i][valid], p.view(name)[valid], err_msg=name)
    # (failed fits leave their track parameters unwritten)
    for name in ("track_params", "track_cov"):
        a = whole.track(name)
        for i, p in zip(halves, parts):
            ok = p.status == 0
            np.testing.assert_array_equal(a[i][ok], p.track(name)[ok], err_msg=name)


@pytest.mark.gpu
def test_uneven_chunks_every_component():
    from acts_gb300.fitter import CudaKalman

    det = generate.Detector(abi.CKG_UNEVEN)
    n = 160000
    b = generate.generate(det, n, seed=37)
    opt = abi.default_options(precision=abi.PRECISION_MIXED, outlier_chi2_cut=15.0,
                              smoother=abi.SMOOTHER_MBF)
    comps = abi.OUT_ALL | abi.OUT_PACKED_COV
    fit = CudaKalman.for_detector(det)
    try:
        fit.set_host_chunk_tracks(-1)  # never chunk
        ref = fit.fit_batch(b, opt, max_states=24, components=comps)
        fit.set_host_chunk_tracks(23456)  # seven chunks, the last one short
        got = fit.fit_batch(b, opt, max_states=24, components=comps)
    finally:
        fit.close()
    for name in got.ARRAYS:
        a, w = getattr(got, name), getattr(ref, name)
        if w is None:
            continue
        if name in ("status", "n_states", "n_measurements", "n_holes", "n_outliers", "ndf",
                    "chi2_sum"):
            np.testing.assert_array_equal(a, w, err_msg=name)
            continue
        valid = np.arange(24)[None, :] < ref.n_states[:, None]
        np.testing.assert_array_equal(got.view(name)[valid], ref.view(name)[valid], err_msg=name)


@pytest.mark.gpu
def test_decreasing_host_offsets_rejected():
    from acts_gb300.fitter import CudaKalman, CudaKalmanError

    det = generate.Detector(abi.CKG_BARREL)
    b = generate.generate(det, 100, seed=3)
    b.seq_offsets[51] = b.seq_offsets[49]  # row 50 runs backwards
    fit = CudaKalman.for_detector(det)
    try:
        with pytest.raises(CudaKalmanError, match="decreasing CSR offsets"):
            fit.fit_batch(b, abi.default_options(), max_states=12)
    finally:
        fit.close()


@pytest.mark.gpu
def test_back_to_back_chunked_calls():
    """Chunked calls issued without synchronizing in between (the next call's
    inputs travel while the previous call's last chunk is fitted, into the
    other input set), one of them on another stream: each call's results
    equal those of the same batch fitted alone."""
    import ctypes as C

    import torch

    from acts_gb300.fitter import CudaKalman

    det = generate.Detector(abi.CKG_BARREL)
    batches = [generate.generate(det, 90000, seed=80 + i) for i in range(3)]
    opt = abi.default_options(precision=abi.PRECISION_MIXED)
    comps = abi.OUT_SMOOTHED | abi.OUT_PACKED_COV
    fit = CudaKalman.for_detector(det)
    try:
        fit.set_host_chunk_tracks(-1)
        alone = [fit.fit_batch(b, opt, max_states=12, components=comps) for b in batches]
        fit.set_host_chunk_tracks(30000)  # three chunks per call
        other = torch.cuda.Stream()
        res = [Results(b.n, 12, comps) for b in batches]
        keep = [(b.as_batch_in(), r.as_batch_out()) for b, r in zip(batches, res)]
        for k, (bi, bo) in enumerate(keep):
            sp = C.c_void_p(other.cuda_stream) if k == 1 else None
            fit.fit_batch_raw(opt, bi, bo, sp)
        fit.sync()
    finally:
        fit.close()
    for r, a in zip(res, alone):
        np.testing.assert_array_equal(r.status, a.status)
        valid = np.arange(12)[None, :] < a.n_states[:, None]
        for name in ("smoothed", "smoothed_cov", "state_surface"):
            np.testing.assert_array_equal(r.view(name)[valid], a.view(name)[valid], err_msg=name)
