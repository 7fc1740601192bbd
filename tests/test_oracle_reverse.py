"""Reverse filtering in the oracle (KalmanFitter::fit_impl with
reverseFiltering, KalmanFitter.hpp:897-945): the forward states are the
smoother's, the first measurement state's smoothed parameters come from the
reversed filter pass (a filter in their own right: pulls of unit width
against the generator truth), the last one's smoothed parameters are its
filtered ones, and no other state has smoothed parameters."""
import numpy as np
import pytest

from acts_gb300 import abi, generate
from acts_gb300.results import Results
from conftest import batch, detector
from oracle import kforacle


def _fit(det, b, max_states=24, comps=abi.OUT_ALL, **kw):
    r = Results(b.n, max_states, comps)
    kforacle.fit_batch(det, b, abi.default_options(**kw), r, n_threads=4)
    return r


def _meas_states(r, t):
    f = r.view("state_flags")[t, : r.n_states[t]]
    return np.nonzero((f & abi.FLAG_HAS_MEASUREMENT) & ~(f & abi.FLAG_IS_OUTLIER))[0]


def test_reverse_filtering_keeps_the_forward_states():
    det, b = detector(abi.CKG_BARREL), batch(abi.CKG_BARREL, 300)
    s = _fit(det, b)
    v = _fit(det, b, reverse_filtering=1)
    np.testing.assert_array_equal(v.status, s.status)
    ok = s.status == 0
    assert ok.mean() > 0.99
    for name in ("n_states", "n_measurements", "n_holes", "n_outliers", "ndf", "chi2_sum"):
        np.testing.assert_array_equal(getattr(v, name)[ok], getattr(s, name)[ok])
    for name in ("state_surface", "state_flags", "state_chi2", "state_path_length", "predicted",
                 "predicted_cov", "filtered", "filtered_cov", "jacobian"):
        for t in np.nonzero(ok)[0]:
            n = s.n_states[t]
            np.testing.assert_array_equal(v.view(name)[t, :n], s.view(name)[t, :n], err_msg=name)
    sm, smc, fi, fic = v.view("smoothed"), v.view("smoothed_cov"), v.view("filtered"), v.view("filtered_cov")
    for t in np.nonzero(ok)[0]:
        m = _meas_states(v, t)
        first, last = m[0], m[-1]
        has = ~np.isnan(sm[t, : v.n_states[t], 0])
        assert set(np.nonzero(has)[0]) == {first, last}
        assert np.isnan(smc[t, : v.n_states[t]][~has]).all()
        if first != last:
            np.testing.assert_array_equal(sm[t, last], fi[t, last])
            np.testing.assert_array_equal(smc[t, last], fic[t, last])
        # the reversed pass saw every measurement: its estimate at the first
        # state is close to the smoother's (which adds the start prior)
        d = (sm[t, first] - s.view("smoothed")[t, first])[:5]
        sig = np.sqrt(s.view("smoothed_cov")[t, first][[0, 7, 14, 21, 28]])
        assert (np.abs(d) / sig).max() < 10.0


def test_reverse_filtered_first_state_pulls():
    """The reversed pass's estimate at the first measurement state against
    the generator truth there: mean 0, width 1 (time: unmeasured, carried
    with the scaled start covariance only)."""
    det, b = detector(abi.CKG_BARREL), batch(abi.CKG_BARREL, 2000)
    r = _fit(det, b, reverse_filtering=1)
    ok = np.nonzero(r.status == 0)[0]
    assert ok.size > 0.99 * b.n
    sm, smc, ss = r.view("smoothed"), r.view("smoothed_cov"), r.view("state_surface")
    tm = b.truth_meas.reshape(-1, 6)
    P = []
    for t in ok:
        k = _meas_states(r, t)[0]
        m0, m1 = b.meas_offsets[t], b.meas_offsets[t + 1]
        mi = m0 + int(np.nonzero(b.meas_surfaces[m0:m1] == ss[t, k])[0][0])
        d = sm[t, k, :5] - tm[mi, :5]
        d[2] = (d[2] + np.pi) % (2 * np.pi) - np.pi
        P.append(d / np.sqrt(smc[t, k][[0, 7, 14, 21, 28]]))
    P = np.array(P)
    assert (np.abs(P.mean(axis=0)) < 0.1).all(), P.mean(axis=0)
    assert ((P.std(axis=0) > 0.9) & (P.std(axis=0) < 1.1)).all(), P.std(axis=0)


def test_reverse_filtering_perigee_pulls():
    """With a perigee reference surface the track parameters come from the
    reversed pass (target reached) or from the extrapolation of the first
    measurement state's reverse-filtered parameters: pulls against the
    generator truth at the vertex of mean 0, width 1."""
    det = generate.Detector(abi.CKG_BARREL, perigee=True)
    b = generate.generate(det, 2000, seed=3)
    r = _fit(det, b, comps=abi.OUT_SMOOTHED | abi.OUT_REFERENCE, reference_surface=det.perigee,
             reverse_filtering=1)
    ok = r.status == 0
    assert ok.mean() > 0.99
    tp, tc = r.track("track_params"), r.track("track_cov")
    ts = b.truth_start.reshape(-1, 6)
    truth = [np.zeros(b.n), b.start_frames.reshape(-1, 12)[:, 11], ts[:, 2], ts[:, 3], ts[:, 4]]
    for i in range(5):
        d = tp[ok, i] - truth[i][ok]
        if i == 2:
            d = (d + np.pi) % (2 * np.pi) - np.pi
        pull = d / np.sqrt(tc[ok, 7 * i])
        assert abs(pull.mean()) < 0.08, (i, pull.mean())
        assert 0.93 < pull.std() < 1.07, (i, pull.std())


def test_reverse_filtering_momentum_threshold():
    """The examples' reverse-filtering logic: exactly the tracks whose last
    measurement state's filtered momentum 1/|q/p| is at most the threshold
    are reverse-filtered; the others are the smoother's, bit for bit."""
    det, b = detector(abi.CKG_BARREL), batch(abi.CKG_BARREL, 600)
    s = _fit(det, b)
    v = _fit(det, b, reverse_filtering_mom_threshold=2.0)
    np.testing.assert_array_equal(v.status, s.status)
    n_rev = 0
    for t in np.nonzero(s.status == 0)[0]:
        m = _meas_states(s, t)
        n = s.n_states[t]
        if 1.0 / abs(s.view("filtered")[t, m[-1], 4]) <= 2.0:
            has = ~np.isnan(v.view("smoothed")[t, :n, 0])
            assert set(np.nonzero(has)[0]) == {m[0], m[-1]}
            n_rev += 1
        else:
            np.testing.assert_array_equal(v.view("smoothed")[t, :n], s.view("smoothed")[t, :n])
    assert 0.1 * s.n < n_rev < 0.5 * s.n


def test_inconsistent_track_states():
    """With a tight outlier cut the reversed pass can judge the innermost
    measurement an outlier that the forward pass accepted: its last
    measurement state is then not on the forward first measurement state's
    surface and the fit fails (KalmanFitterError::InconsistentTrackStates),
    while the same tracks fit without reverse filtering."""
    det, b = detector(abi.CKG_BARREL), batch(abi.CKG_BARREL, 1000)
    s = _fit(det, b, outlier_chi2_cut=4.0)
    v = _fit(det, b, outlier_chi2_cut=4.0, reverse_filtering=1)
    bad = v.status == abi.TRACK_INCONSISTENT_STATES
    assert bad.sum() > 0.05 * b.n
    assert (s.status[bad] == 0).all()
    assert (v.n_states[bad] == 0).all()
