"""ck_fit_batch_static (the allocation-free entry point: pipeline scratch in
one static device array) gives the results of ck_fit_batch on the same
device-resident batch, on two calls in a row, and rejects batches larger than
its array. Collected last on purpose; it also passes alone in a fresh
process."""
import ctypes as C

import numpy as np
import pytest

from acts_gb300 import abi
from conftest import batch

torch = pytest.importorskip("torch")

N_TRACKS = 3000
MAX_STATES = 10
FIELDS = {"status": (C.c_int32, 1), "n_states": (C.c_int32, 1), "n_measurements": (C.c_int32, 1),
          "n_holes": (C.c_int32, 1), "n_outliers": (C.c_int32, 1), "ndf": (C.c_int32, 1),
          "chi2_sum": (C.c_double, 1), "state_surface": (C.c_int32, MAX_STATES),
          "state_flags": (C.c_uint32, MAX_STATES), "state_path_length": (C.c_double, MAX_STATES),
          "state_chi2": (C.c_double, MAX_STATES), "smoothed": (C.c_double, 6 * MAX_STATES),
          "smoothed_cov": (C.c_double, 36 * MAX_STATES)}
TORCH = {C.c_int32: torch.int32, C.c_uint32: torch.int32, C.c_double: torch.float64}


def _device_in(b, dev):
    keep = {}
    bi = abi.ck_batch_in()
    bi.n_tracks = b.n
    bi.memory = abi.MEM_DEVICE
    for name, ct in (("seq_offsets", C.c_int32), ("seq_surfaces", C.c_int32),
                     ("meas_offsets", C.c_int32), ("meas_surfaces", C.c_int32),
                     ("meas_values", C.c_double), ("meas_cov", C.c_double),
                     ("start_params", C.c_double), ("start_cov", C.c_double),
                     ("start_frames", C.c_double), ("particle", C.c_float),
                     ("particle_pdg", C.c_int32)):
        t = torch.from_numpy(getattr(b, name)).to(dev)
        keep[name] = t
        setattr(bi, name, C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ct)))
    return bi, keep


def _device_out(n, dev):
    keep = {}
    bo = abi.ck_batch_out()
    bo.max_states = MAX_STATES
    bo.components = abi.OUT_SMOOTHED
    bo.memory = abi.MEM_DEVICE
    for name, (ct, per) in FIELDS.items():
        t = torch.full((n * per,), -7, dtype=TORCH[ct], device=dev)
        keep[name] = t
        setattr(bo, name, C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ct)))
    return bo, keep


def _host(keep):
    return {k: v.cpu().numpy() for k, v in keep.items()}


def _compare(ref, got):
    ok = ref["status"] == 0
    for name in ("status", "n_states", "n_measurements", "n_holes", "n_outliers", "ndf"):
        assert np.array_equal(ref[name], got[name]), name
    assert np.allclose(got["chi2_sum"][ok], ref["chi2_sum"][ok], rtol=1e-12, atol=0)
    # per-state arrays (SoA [(k * C + c) * n + t]) of the valid states only
    ns = ref["n_states"]
    for name, (ct, per) in FIELDS.items():
        if per == 1:
            continue
        c = per // MAX_STATES
        a = ref[name].reshape(MAX_STATES, c, N_TRACKS)
        b = got[name].reshape(MAX_STATES, c, N_TRACKS)
        valid = (np.arange(MAX_STATES)[:, None] < ns[None, :]) & ok[None, :]
        va, vb = a.transpose(0, 2, 1)[valid], b.transpose(0, 2, 1)[valid]
        if np.issubdtype(va.dtype, np.integer):
            assert np.array_equal(va, vb), name
        else:
            assert np.allclose(vb, va, rtol=1e-12, atol=1e-300), name


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_static_scratch_matches_fit_batch(fitter_factory, precision):
    fit = fitter_factory(abi.CKG_BARREL)
    dev = torch.device("cuda", 0)
    b = batch(abi.CKG_BARREL, N_TRACKS, seed=29)
    opt = abi.default_options(precision=precision)
    need = fit.static_scratch_bytes(N_TRACKS, MAX_STATES, precision)
    assert 0 < need <= fit.static_scratch_capacity()
    bi, keep_in = _device_in(b, dev)
    bo_ref, keep_ref = _device_out(N_TRACKS, dev)
    fit.fit_batch_raw(opt, bi, bo_ref)
    fit.sync()
    ref = _host(keep_ref)
    assert (ref["status"] == 0).mean() > 0.99
    for _ in range(2):  # two calls in a row on the same array
        bo, keep_out = _device_out(N_TRACKS, dev)
        fit.fit_batch_static(opt, bi, bo)
        fit.sync()
        _compare(ref, _host(keep_out))


@pytest.mark.gpu
def test_static_scratch_rejects_oversized_batch(fitter_factory):
    from acts_gb300.fitter import CudaKalmanError

    fit = fitter_factory(abi.CKG_BARREL)
    dev = torch.device("cuda", 0)
    cap = fit.static_scratch_capacity()
    n = 1
    while fit.static_scratch_bytes(n, MAX_STATES, abi.PRECISION_FP64) <= cap:
        n *= 2
    b = batch(abi.CKG_BARREL, n, seed=3)
    bi, keep_in = _device_in(b, dev)
    keep = {}
    bo = abi.ck_batch_out()
    bo.max_states = MAX_STATES
    bo.memory = abi.MEM_DEVICE
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    bo.status = C.cast(C.c_void_p(st.data_ptr()), C.POINTER(C.c_int32))
    with pytest.raises(CudaKalmanError) as e:
        fit.fit_batch_static(abi.default_options(), bi, bo)
    assert e.value.status == abi.CK_ERR_SCRATCH_LIMIT
    assert "static scratch" in str(e.value)


@pytest.mark.gpu
@pytest.mark.parametrize("reverse", [0, 1], ids=["smoother", "reverse_filtering"])
def test_static_scratch_with_reference_surface(reverse):
    """ck_fit_batch_static with extrapolation to a perigee surface (its start
    states in the static array too), or with reverse filtering towards it,
    gives ck_fit_batch's perigee parameters."""
    from acts_gb300 import generate
    from acts_gb300.fitter import CudaKalman

    det = generate.Detector(abi.CKG_BARREL, perigee=True)
    b = generate.generate(det, N_TRACKS, seed=29)
    dev = torch.device("cuda", 0)
    opt = abi.default_options(precision=abi.PRECISION_MIXED, reference_surface=det.perigee,
                              reverse_filtering=reverse)
    fit = CudaKalman.for_detector(det)
    try:
        bi, keep_in = _device_in(b, dev)
        outs = []
        for call in (fit.fit_batch_raw, fit.fit_batch_static):
            bo, keep = _device_out(N_TRACKS, dev)
            tp = torch.zeros(6 * N_TRACKS, dtype=torch.float64, device=dev)
            tc = torch.zeros(36 * N_TRACKS, dtype=torch.float64, device=dev)
            bo.track_params = C.cast(C.c_void_p(tp.data_ptr()), C.POINTER(C.c_double))
            bo.track_cov = C.cast(C.c_void_p(tc.data_ptr()), C.POINTER(C.c_double))
            call(opt, bi, bo)
            fit.sync()
            outs.append((keep["status"].cpu().numpy(), tp.cpu().numpy(), tc.cpu().numpy()))
    finally:
        fit.close()
    (s0, p0, c0), (s1, p1, c1) = outs
    assert np.array_equal(s0, s1)
    assert (s0 == 0).mean() > 0.99
    assert np.array_equal(p0, p1) and np.array_equal(c0, c1)


@pytest.mark.gpu
def test_static_scratch_allocates_nothing():
    """The entry point's promise: once its first call on the device has
    resolved the array (which may load the module), later calls take no
    device memory, even for a batch larger than any before it. Free device
    memory is read with cudaMemGetInfo around such a call; every input and
    output is allocated before the first reading."""
    from acts_gb300 import generate
    from acts_gb300.fitter import CudaKalman

    det = generate.Detector(abi.CKG_BARREL, perigee=True)
    dev = torch.device("cuda", 0)
    small, large = 200, 2 * N_TRACKS
    opt = abi.default_options(precision=abi.PRECISION_MIXED, reference_surface=det.perigee)
    fit = CudaKalman.for_detector(det)
    try:
        assert fit.static_scratch_bytes_for(opt, large, MAX_STATES) <= fit.static_scratch_capacity()
        bs, keep_s = _device_in(generate.generate(det, small, seed=5), dev)
        bl, keep_l = _device_in(generate.generate(det, large, seed=6), dev)
        os_, keep_os = _device_out(small, dev)
        ol, keep_ol = _device_out(large, dev)
        fit.fit_batch_static(opt, bs, os_)
        fit.sync()
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info(dev)
        fit.fit_batch_static(opt, bl, ol)
        fit.sync()
        free1, _ = torch.cuda.mem_get_info(dev)
        assert free1 == free0, (free0, free1)
        assert (keep_ol["status"].cpu().numpy() == 0).mean() > 0.99
    finally:
        fit.close()
