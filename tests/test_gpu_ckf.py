"""ck_find_tracks on the GPU against the track-finding restatement (oracle).

FP64 form: the same search as the oracle — statuses, found tracks, state
counts, the states' surfaces, flags, measurements and chains bit-exact;
parameters within 1e-9 of max(|x|, sigma_x), covariance entries within 1e-9
of max(|C_ij|, sqrt(C_ii C_jj)), Jacobian entries within 1e-9 of
max(|J_ij|, 1e-4 max_k |J_ik|), chi2 and path lengths within 1e-9 of
max(|x|, 1) — on the reference's CKF unit-test case, generated events on
the telescope, barrel and uneven (field map) workloads, with branching,
outliers, holes, the branch stopper, the end-of-world option, a target
surface, and the error paths (field map left, capacities, invalid input).
Mixed form: the same tracks for nearly every seed (its chi2 values differ
in the last FP32 bits, which can reorder candidates at the cut).
"""
import ctypes as C

import numpy as np
import pytest

from acts_gb300 import abi, generate
from ckf_cases import WithTarget, cubic_event
from oracle import kforacle

RTOL = 1e-9
DMAX = np.finfo(float).max
DIAG = [i * 6 - (i * (i - 1)) // 2 for i in range(6)]  # packed (i, i)


def _fitter(det):
    from acts_gb300.fitter import CudaKalman

    return CudaKalman(det.surfaces, det.n_surfaces, det.field)


def _copy(tf):
    """A fresh container with the same inputs."""
    return abi.TrackFinding(tf.seq_offsets, tf.seq_surfaces, tf.start_params, tf.start_cov,
                            tf.start_frames, tf.particle, tf.surf_meas_offsets, tf.meas_values,
                            tf.meas_cov, meas_subspace=tf.meas_subspace,
                            particle_pdg=tf.particle_pdg, max_states=tf.max_states,
                            max_tracks=tf.max_tracks)


def _run(det, tf, opt, **kw):
    """(gpu, oracle) results of the same call."""
    ko = tf.options(**kw)
    ora = _copy(tf)
    kforacle.find_tracks(det.surfaces, det.field, opt, ko, ora,
                         n_threads=kforacle.hardware_threads())
    gpu = _copy(tf)
    fit = _fitter(det)
    try:
        fit.find_tracks(opt, ko, gpu)
    finally:
        fit.close()
    return gpu, ora


def _rel(a, b, scale):
    return float(np.max(np.abs(a - b) / np.maximum(scale, 1e-300), initial=0.0))


def _vec_scale(v, cov):
    sig = np.sqrt(np.abs(cov[..., DIAG]))
    return np.maximum(np.abs(v), sig)


def _cov_scale(c):
    d = np.sqrt(np.abs(c[..., DIAG]))
    full = d[..., :, None] * d[..., None, :]
    iu = np.triu_indices(6)
    return np.maximum(np.abs(c), full[..., iu[0], iu[1]])


def compare(gpu, ora):
    """Asserts the bit-exact parts; returns the worst relative differences."""
    np.testing.assert_array_equal(gpu.status, ora.status)
    np.testing.assert_array_equal(gpu.n_tracks, ora.n_tracks)
    np.testing.assert_array_equal(gpu.n_states, ora.n_states)
    rep = {}
    T = np.arange(gpu.max_tracks)[None, :] < ora.n_tracks[:, None]
    S = np.arange(gpu.max_states)[None, :] < ora.n_states[:, None]
    for name in ("track_tip", "track_n_measurements", "track_n_holes", "track_n_outliers",
                 "track_ndf"):
        np.testing.assert_array_equal(getattr(gpu, name)[T], getattr(ora, name)[T], err_msg=name)
    for name in ("state_prev", "state_surface", "state_flags", "state_measurement"):
        np.testing.assert_array_equal(getattr(gpu, name)[S], getattr(ora, name)[S], err_msg=name)
    for name, mask in (("track_chi2", T), ("state_chi2", S), ("state_path_length", S)):
        a, b = getattr(gpu, name)[mask], getattr(ora, name)[mask]
        rep[name] = _rel(a, b, np.maximum(np.abs(b), 1.0))
    tp = T & np.isfinite(ora.track_params[..., 0])
    np.testing.assert_array_equal(np.isfinite(gpu.track_params[..., 0])[T],
                                  np.isfinite(ora.track_params[..., 0])[T])
    if tp.any():
        rep["track_params"] = _rel(gpu.track_params[tp], ora.track_params[tp],
                                   _vec_scale(ora.track_params[tp], ora.track_cov[tp]))
        rep["track_cov"] = _rel(gpu.track_cov[tp], ora.track_cov[tp], _cov_scale(ora.track_cov[tp]))
    for v, c in (("predicted", "predicted_cov"), ("filtered", "filtered_cov")):
        ov, oc = getattr(ora, v)[S], getattr(ora, c)[S]
        rep[v] = _rel(getattr(gpu, v)[S], ov, _vec_scale(ov, oc))
        rep[c] = _rel(getattr(gpu, c)[S], oc, _cov_scale(oc))
    J, Jo = gpu.jacobian[S].reshape(-1, 6, 6), ora.jacobian[S].reshape(-1, 6, 6)
    floor = 1e-4 * np.abs(Jo).max(axis=2, keepdims=True)
    rep["jacobian"] = _rel(J, Jo, np.maximum(np.abs(Jo), floor))
    return rep


def _check(gpu, ora):
    rep = compare(gpu, ora)
    print(rep)
    bad = {k: v for k, v in rep.items() if not v <= RTOL}
    assert not bad, bad
    return rep


@pytest.mark.gpu
def test_zero_field_forward_on_gpu():
    """The reference's ZeroFieldForward expectations, and the oracle's
    result, for 20 smeared copies of its three particles."""
    det, tf, truth = cubic_event(n_copies=20)
    gpu, ora = _run(det, tf, abi.default_options(), chi2_cut=DMAX, max_candidates=1,
                    target_surface=det.target)
    _check(gpu, ora)
    assert (gpu.status == 0).all() and (gpu.n_tracks == 1).all()
    for s in range(gpu.n):
        m = gpu.track_measurements(s, 0)
        assert len(m) == 6 and (truth[m] % 3 == s % 3).all()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["telescope", "barrel_branching", "barrel_stopper",
                                  "uneven_end_of_world", "uneven_leaves_map", "target_behind",
                                  "strips"])
def test_fp64_parity(case):
    opt = abi.default_options()
    if case == "telescope":
        det = generate.Detector(abi.CKG_TELESCOPE)
        tf = generate.ckf_event(det, generate.generate(det, 2000, seed=21))
        kw = dict(chi2_cut=15.0)
    elif case == "barrel_branching":
        det = generate.Detector(abi.CKG_BARREL)
        tf = generate.ckf_event(det, generate.generate(det, 1000, seed=22), max_states=128,
                                max_tracks=32)
        opt = abi.default_options(max_steps=100000)
        kw = dict(chi2_cut=300.0, max_candidates=3, chi2_cut_outlier=500.0, max_branches=32)
    elif case == "barrel_stopper":
        det = generate.Detector(abi.CKG_BARREL)
        tf = generate.ckf_event(det, generate.generate(det, 2000, seed=23))
        kw = dict(chi2_cut=2.0, chi2_cut_outlier=0.0, max_holes=0, min_measurements=3)
    elif case == "uneven_end_of_world":
        det = generate.Detector(abi.CKG_UNEVEN)
        tf = generate.ckf_event(det, generate.generate(det, 2000, seed=24))
        kw = dict(chi2_cut=15.0, end_of_world=1)
    elif case == "uneven_leaves_map":
        det = generate.Detector(abi.CKG_UNEVEN)
        tf = generate.ckf_event(det, generate.generate(det, 1000, seed=25))
        kw = dict(chi2_cut=15.0)
    elif case == "strips":
        # 1D loc0 and loc1 strips on the outer layers: windows along either axis
        det = generate.Detector(abi.CKG_STRIPS)
        tf = generate.ckf_event(det, generate.generate(det, 2000, seed=27))
        kw = dict(chi2_cut=15.0, max_candidates=2, chi2_cut_outlier=100.0, max_branches=32)
    else:
        base = generate.Detector(abi.CKG_BARREL)
        det = WithTarget(base)
        tf = generate.ckf_event(det, generate.generate(base, 500, seed=26))
        kw = dict(chi2_cut=15.0, target_surface=det.target)
    gpu, ora = _run(det, tf, opt, **kw)
    st = np.unique(ora.status, return_counts=True)
    print(case, "statuses:", dict(zip(st[0].tolist(), st[1].tolist())),
          "tracks:", int(ora.n_tracks.sum()), "states:", int(ora.n_states.sum()))
    _check(gpu, ora)
    if case == "barrel_branching":
        assert (ora.n_tracks > 1).sum() > 0.05 * ora.n
    if case == "barrel_stopper":
        assert ((ora.track_n_holes == 1) & (np.arange(ora.max_tracks) < ora.n_tracks[:, None])).any()
        assert ((ora.n_tracks == 0) & (ora.status == 0)).any()
    if case == "uneven_leaves_map":
        assert (ora.status == abi.TRACK_FIELD_OUT_OF_BOUNDS).any()


@pytest.mark.gpu
def test_mixed_finds_the_same_tracks():
    det = generate.Detector(abi.CKG_BARREL)
    tf = generate.ckf_event(det, generate.generate(det, 3000, seed=27))
    gpu, ora = _run(det, tf, abi.default_options(precision=abi.PRECISION_MIXED), chi2_cut=15.0)
    same = 0
    for s in range(gpu.n):
        if gpu.status[s] != ora.status[s] or gpu.n_tracks[s] != ora.n_tracks[s]:
            continue
        same += all(gpu.track_measurements(s, k) == ora.track_measurements(s, k)
                    for k in range(gpu.n_tracks[s]))
    assert same >= 0.995 * gpu.n, same
    T = (gpu.n_tracks == ora.n_tracks)[:, None] & (np.arange(gpu.max_tracks) < gpu.n_tracks[:, None])
    a, b = gpu.track_chi2[T], ora.track_chi2[T]
    assert np.median(np.abs(a - b) / np.maximum(b, 1.0)) < 1e-4


@pytest.mark.gpu
def test_device_memory_batch_equals_host():
    """The same call on device-resident arrays (torch tensors) gives the
    host-memory results."""
    import torch

    from acts_gb300.fitter import lib

    det = generate.Detector(abi.CKG_BARREL)
    tf = generate.ckf_event(det, generate.generate(det, 500, seed=28))
    opt = abi.default_options()
    ko = tf.options(chi2_cut=15.0)
    host = _copy(tf)
    dev = _copy(tf)
    fit = _fitter(det)
    try:
        fit.find_tracks(opt, ko, host)
        keep = {}
        di = dev.as_in()
        di.memory = abi.MEM_DEVICE
        for name, _ in abi.ck_ckf_in._fields_:
            v = getattr(dev, name, None)
            if isinstance(v, np.ndarray):
                t = torch.from_numpy(np.ascontiguousarray(v)).cuda()
                keep[name] = t
                setattr(di, name, C.cast(C.c_void_p(t.data_ptr()), type(getattr(di, name))))
        do = dev.as_out()
        outs = {}
        for name, _ in abi.ck_ckf_out._fields_:
            v = getattr(dev, name)
            t = torch.from_numpy(np.ascontiguousarray(v)).cuda()
            outs[name] = t
            setattr(do, name, C.cast(C.c_void_p(t.data_ptr()), type(getattr(do, name))))
        st = lib().ck_find_tracks(fit.handle, C.byref(opt), C.byref(ko), C.byref(di), C.byref(do),
                                  None)
        assert st == abi.CK_OK
        torch.cuda.synchronize()
        for name, t in outs.items():
            setattr(dev, name, t.cpu().numpy())
    finally:
        fit.close()
    rep = compare(dev, host)
    assert all(v == 0.0 for v in rep.values()), rep


@pytest.mark.gpu
def test_invalid_arguments_are_rejected():
    from acts_gb300.fitter import CudaKalmanError

    det, tf, _ = cubic_event()
    fit = _fitter(det)
    try:
        for kw in (dict(max_candidates=0), dict(max_candidates=17), dict(max_branches=0),
                   dict(target_surface=99)):
            with pytest.raises(CudaKalmanError):
                fit.find_tracks(abi.default_options(), tf.options(**kw), _copy(tf))
        bad = _copy(tf)
        bad.surf_meas_offsets[1] = 100  # not a partition of the measurements
        with pytest.raises(CudaKalmanError):
            fit.find_tracks(abi.default_options(), bad.options(), bad)
    finally:
        fit.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED],
                         ids=["fp64", "mixed"])
def test_lanes_per_seed_select_the_same(precision):
    """One lane per seed with the windowed search over sorted candidates,
    and 2-32 lanes splitting full scans merged by shuffles, select the same
    candidates: every integer output identical, floating-point values
    within the parity tolerance (each kernel instance contracts its
    multiply-adds its own way)."""
    det = generate.Detector(abi.CKG_BARREL)
    tf = generate.ckf_event(det, generate.generate(det, 1500, seed=29), max_states=128,
                            max_tracks=32)
    opt = abi.default_options(precision=precision, max_steps=100000)
    fit = _fitter(det)
    outs = []
    try:
        for g in (1, 2, 4, 8, 16, 32):
            r = _copy(tf)
            fit.find_tracks(opt, tf.options(chi2_cut=300.0, max_candidates=3, max_branches=32,
                                            chi2_cut_outlier=500.0, lanes_per_seed=g), r)
            assert fit.last_ckf_lanes() == g
            outs.append(r)
    finally:
        fit.close()
    assert (outs[0].n_tracks > 1).any()
    for r in outs[1:]:
        rep = compare(r, outs[0])
        assert all(v <= RTOL for v in rep.values()), rep


@pytest.mark.gpu
def test_unsorted_surface_falls_back_to_the_full_scan():
    """A surface whose measurements mix loc0 and loc1 strips cannot be
    searched along one axis: the one-lane search scans it fully, with the
    oracle's result."""
    det, tf, truth = cubic_event(n_copies=5)
    # the third layer (loc0 strips): one measurement becomes a loc1 strip
    m = int(tf.surf_meas_offsets[2])
    tf.meas_subspace[m] = abi.MEAS_LOC1
    gpu, ora = _run(det, tf, abi.default_options(), chi2_cut=DMAX, max_candidates=2,
                    target_surface=det.target, max_branches=32)
    _check(gpu, ora)


def _copy_events(tf):
    r = _copy(tf)
    r.n_events, r.seed_event = tf.n_events, tf.seed_event
    r.n_surfaces = tf.n_surfaces
    return r


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED],
                         ids=["fp64", "mixed"])
def test_events_in_one_call(precision):
    """Twenty events in one launch: the oracle's result (FP64), and for both
    forms exactly the results of one call per event."""
    det = generate.Detector(abi.CKG_UNEVEN)
    sizes = generate.event_sizes(9, 20, mean=400.0)
    b = generate.generate(det, int(sizes.sum()), seed=42)
    tf = generate.ckf_events(det, b, sizes, max_states=32, max_tracks=8)
    opt = abi.default_options(precision=precision)
    ko = tf.options(chi2_cut=15.0, max_candidates=2, end_of_world=1)
    gpu = _copy_events(tf)
    fit = _fitter(det)
    try:
        fit.find_tracks(opt, ko, gpu)
        if precision == abi.PRECISION_FP64:
            ora = _copy_events(tf)
            kforacle.find_tracks(det.surfaces, det.field, opt, ko, ora,
                                 n_threads=kforacle.hardware_threads())
            _check(gpu, ora)
        start = 0
        for m in sizes:
            if m == 0:
                continue
            one = generate.ckf_event(det, b.subset(np.arange(start, start + int(m))),
                                     max_states=32, max_tracks=8)
            fit.find_tracks(opt, ko, one)
            base = int(b.meas_offsets[start])
            for s in range(int(m)):
                got = [[int(tf.meas_index[x]) for x in gpu.track_measurements(start + s, k)]
                       for k in range(gpu.n_tracks[start + s])]
                want = [[int(one.meas_index[x]) + base for x in one.track_measurements(s, k)]
                        for k in range(one.n_tracks[s])]
                assert got == want
            # (slots beyond a seed's track count are unspecified)
            valid = np.arange(gpu.max_tracks)[None, :] < one.n_tracks[:int(m), None]
            np.testing.assert_array_equal(gpu.n_tracks[start:start + int(m)], one.n_tracks[:int(m)])
            np.testing.assert_array_equal(gpu.track_chi2[start:start + int(m)][valid],
                                          one.track_chi2[:int(m)][valid])
            start += int(m)
    finally:
        fit.close()
