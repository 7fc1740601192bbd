"""Serving loop: events of different sizes submitted while others are on the
GPU are co-batched and fitted concurrently; every event's result is the same
alone and in the mix (bit for bit: the per-track computation does not depend
on its batch), latencies are reported, oversized events are rejected."""
import time

import numpy as np
import pytest

from acts_gb300 import abi, generate
from acts_gb300.fitter import CudaKalmanError
from acts_gb300.serving import FitServer
from conftest import detector


def _events(det, sizes, seed=31):
    evs, first = [], 0
    for s in sizes:
        evs.append(generate.generate(det, int(s), seed=seed, first_track=first))
        first += int(s)
    return evs


@pytest.mark.gpu
@pytest.mark.parametrize("precision,grid_blocks,steps_per_round,preset",
                         [(abi.PRECISION_FP64, 0, 0, abi.CKG_UNEVEN),
                          (abi.PRECISION_MIXED, 0, 0, abi.CKG_UNEVEN),
                          (abi.PRECISION_MIXED, 7, 1, abi.CKG_UNEVEN),
                          (abi.PRECISION_MIXED, 0, 0, abi.CKG_STRIPS)])
def test_same_result_alone_and_in_mix(fitter_factory, precision, grid_blocks, steps_per_round,
                                      preset):
    """Also with a launch shape of the co-batches far from the default (7
    blocks, one Runge-Kutta trial per round): results do not depend on it;
    and with 1D strip measurements (per-measurement subspaces staged with
    the events)."""
    det = detector(preset)
    fit = fitter_factory(preset)
    opt = abi.default_options(precision=precision, outlier_chi2_cut=15.0)
    sizes = generate.event_sizes(5, 24, lo=100, hi=5000)
    evs = _events(det, sizes)
    srv = FitServer(fit, opt, memory_budget_bytes=4 << 30, n_streams=3, max_states=24,
                    max_batch_tracks=12000, grid_blocks=grid_blocks,
                    steps_per_round=steps_per_round)
    for i, ev in enumerate(evs):
        srv.submit(i, ev)
        if i % 5 == 4:
            time.sleep(0.002)  # later events arrive while earlier ones run
    got = {}
    t0 = time.time()
    while len(got) < len(evs) and time.time() - t0 < 120:
        r = srv.poll(timeout_ms=200)
        if r is not None:
            got[r[0]] = (r[1], r[2])
    st = srv.stats()
    srv.close()
    assert len(got) == len(evs), st
    assert st["tracks"] == int(sum(sizes))
    for i, ev in enumerate(evs):
        res, lat = got[i]
        assert lat > 0
        alone = fit.fit_batch(ev, opt, max_states=24, components=abi.OUT_SMOOTHED)
        for name in ("status", "n_states", "n_measurements", "n_holes", "n_outliers", "ndf",
                     "chi2_sum"):
            assert np.array_equal(getattr(res, name), getattr(alone, name)), (i, name)
        # per-state arrays: the states of each successful track (entries past
        # n_states are not written by the fitter)
        ok = alone.status == 0
        valid = np.arange(24)[None, :] < alone.n_states[:, None]
        valid &= ok[:, None]
        for name in ("state_flags", "state_surface", "state_chi2", "smoothed", "smoothed_cov"):
            a, b = res.view(name), alone.view(name)
            assert np.array_equal(a[valid], b[valid]), (i, name)


@pytest.mark.gpu
@pytest.mark.parametrize("where", ["cuda:0", "pinned"])
def test_results_in_device_and_pinned_buffers(fitter_factory, where):
    """Results written straight into device or page-locked buffers equal the
    results of ck_fit_batch on the same events."""
    from acts_gb300.results import TorchResults

    preset = abi.CKG_UNEVEN
    det = detector(preset)
    fit = fitter_factory(preset)
    opt = abi.default_options(precision=abi.PRECISION_MIXED, outlier_chi2_cut=15.0)
    evs = _events(det, [700, 1500, 300, 2200], seed=57)
    srv = FitServer(fit, opt, memory_budget_bytes=2 << 30, n_streams=2, max_states=24,
                    max_batch_tracks=4000)
    for i, ev in enumerate(evs):
        srv.submit(i, ev, TorchResults(ev.n, 24, abi.OUT_SMOOTHED, device=where))
    got = {}
    t0 = time.time()
    while len(got) < len(evs) and time.time() - t0 < 60:
        r = srv.poll(timeout_ms=200)
        if r is not None:
            got[r[0]] = r[1]
    srv.close()
    assert len(got) == len(evs)
    for i, ev in enumerate(evs):
        res = got[i].to_host()
        alone = fit.fit_batch(ev, opt, max_states=24, components=abi.OUT_SMOOTHED)
        assert np.array_equal(res.status, alone.status)
        assert np.array_equal(res.n_states, alone.n_states)
        ok = alone.status == 0
        valid = (np.arange(24)[None, :] < alone.n_states[:, None]) & ok[:, None]
        for name in ("state_flags", "smoothed", "smoothed_cov"):
            assert np.array_equal(res.view(name)[valid], alone.view(name)[valid]), (i, name)


@pytest.mark.gpu
def test_oversized_event_rejected(fitter_factory):
    preset = abi.CKG_BARREL
    fit = fitter_factory(preset)
    srv = FitServer(fit, abi.default_options(), memory_budget_bytes=2 << 30, n_streams=2,
                    max_states=12, max_batch_tracks=1000)
    assert srv.capacity == 1000
    big = generate.generate(detector(preset), 1200, seed=1)
    with pytest.raises(CudaKalmanError) as e:
        srv.submit(1, big)
    assert e.value.status == abi.CK_ERR_BUDGET
    small = generate.generate(detector(preset), 200, seed=1)
    srv.submit(2, small)
    r = None
    t0 = time.time()
    while r is None and time.time() - t0 < 60:
        r = srv.poll(timeout_ms=200)
    srv.close()
    assert r is not None and r[0] == 2 and (r[1].status == 0).mean() > 0.99


@pytest.mark.gpu
@pytest.mark.parametrize("reverse", [0, 1], ids=["smoother", "reverse_filtering"])
def test_serving_with_reference_surface(reverse):
    """Events fitted through the serving loop with extrapolation to a
    perigee surface (or reverse filtering towards it): every event's perigee
    parameters equal its fit alone."""
    from acts_gb300.fitter import CudaKalman

    det = generate.Detector(abi.CKG_UNEVEN, perigee=True)
    fit = CudaKalman.for_detector(det)
    comps = abi.OUT_SMOOTHED | abi.OUT_REFERENCE
    opt = abi.default_options(precision=abi.PRECISION_MIXED, outlier_chi2_cut=15.0,
                              reference_surface=det.perigee, reverse_filtering=reverse)
    sizes = generate.event_sizes(9, 10, lo=100, hi=3000)
    evs = _events(det, sizes, seed=41)
    srv = FitServer(fit, opt, memory_budget_bytes=2 << 30, n_streams=2, max_states=24,
                    max_batch_tracks=8000, components=comps)
    try:
        for i, ev in enumerate(evs):
            srv.submit(i, ev)
        got = {}
        t0 = time.time()
        while len(got) < len(evs) and time.time() - t0 < 120:
            r = srv.poll(timeout_ms=200)
            if r is not None:
                got[r[0]] = r[1]
    finally:
        srv.close()
    assert len(got) == len(evs)
    try:
        for i, ev in enumerate(evs):
            res = got[i]
            alone = fit.fit_batch(ev, opt, max_states=24, components=comps)
            assert np.array_equal(res.status, alone.status), i
            ok = alone.status == 0
            assert ok.mean() > 0.3
            for name in ("track_params", "track_cov"):
                assert np.array_equal(res.track(name)[ok], alone.track(name)[ok]), (i, name)
    finally:
        fit.close()
