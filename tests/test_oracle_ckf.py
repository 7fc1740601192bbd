"""The track-finding restatement (oracle, CPU) against the reference's own
CKF unit test and the properties of the search.

  ZeroFieldForward (CombinatorialKalmanFilterTests.cpp:329-389): three
  seeds on the cubic telescope, chi2 cut at the double maximum, one
  candidate per surface: three tracks, each with a state on all six layers
  and no measurement of another particle.
  Seeds of a generated event find their own hits (telescope, 2 T).
  The depth-first search explores the best candidate first: the first track
  of a branching search is the single-candidate search's track.
  Branch stopper, outliers, holes and capacity errors behave as specified.
"""
import numpy as np
import pytest

from acts_gb300 import abi, generate
from ckf_cases import WithTarget, cubic_event
from oracle import kforacle

DMAX = np.finfo(float).max


def _find(det, tf, opt=None, **kw):
    opt = opt or abi.default_options()
    kforacle.find_tracks(det.surfaces, det.field, opt, tf.options(**kw), tf,
                         n_threads=kforacle.hardware_threads())
    return tf


def test_zero_field_forward_finds_each_particle():
    det, tf, truth = cubic_event()
    _find(det, tf, chi2_cut=DMAX, max_candidates=1, target_surface=det.target)
    assert tf.status.tolist() == [0, 0, 0]
    assert tf.n_tracks.tolist() == [1, 1, 1]
    for s in range(3):
        states = tf.track_states(s, 0)
        assert len(states) == 6  # nTrackStates == numMeasurements
        m = tf.track_measurements(s, 0)
        assert len(m) == 6 and (truth[m] == s).all()  # no mismatched hits
        assert tf.track_n_measurements[s, 0] == 6 and tf.track_ndf[s, 0] == 2 + 2 + 1 + 1 + 1 + 1
        # the branch ended on the target plane with parameters there
        assert np.isfinite(tf.track_params[s, 0]).all()
        assert abs(tf.track_params[s, 0, 2] - [0.0, -1.0, 1.0][s] * np.pi / 180) < 0.01
    # the states chain along the sequence, filtered chi2 summing to the track's
    for s in range(3):
        st = tf.track_states(s, 0)
        assert tf.state_surface[s, st].tolist() == list(range(6))
        assert abs(tf.state_chi2[s, st].sum() - tf.track_chi2[s, 0]) < 1e-9 * max(
            1.0, tf.track_chi2[s, 0])


def test_seeds_find_their_own_hits():
    det = generate.Detector(abi.CKG_TELESCOPE)
    b = generate.generate(det, 100, seed=11)
    tf = _find(det, generate.ckf_event(det, b))
    assert (tf.status == 0).all()
    assert (tf.n_tracks == 1).all()
    # (the telescope's tracks leave one point within a few mm: near the
    # first planes some seeds take a neighbour's hit)
    own = hits = 0
    for s in range(tf.n):
        m = tf.track_measurements(s, 0)
        own += (tf.meas_track[m] == s).sum()
        hits += len(m)
    assert own >= 0.97 * hits, (own, hits)
    assert (tf.track_n_measurements[:, 0] == 10).mean() >= 0.95


def _branching(det, b, **kw):
    # (every branch runs on after its last surface up to the loop-protection
    # path limit; the step counter is shared by all branches of a seed)
    tf = generate.ckf_event(det, b, max_states=512, max_tracks=64)
    return _find(det, tf, abi.default_options(max_steps=100000), max_branches=64, **kw)


def test_best_candidate_first():
    det = generate.Detector(abi.CKG_TELESCOPE)
    b = generate.generate(det, 40, seed=12)
    one = _find(det, generate.ckf_event(det, b), abi.default_options(max_steps=100000),
                chi2_cut=100.0)
    many = _branching(det, b, chi2_cut=100.0, max_candidates=3)
    assert (many.status == 0).all()
    assert many.n_tracks.sum() > one.n_tracks.sum()  # the cut lets several through
    for s in range(one.n):
        assert one.track_measurements(s, 0) == many.track_measurements(s, 0)
        assert one.track_chi2[s, 0] == many.track_chi2[s, 0]
        a, c = one.track_states(s, 0), many.track_states(s, 0)
        np.testing.assert_array_equal(one.filtered[s, a], many.filtered[s, c])
        np.testing.assert_array_equal(one.filtered_cov[s, a], many.filtered_cov[s, c])


@pytest.mark.parametrize("preset", [abi.CKG_BARREL, abi.CKG_UNEVEN], ids=["barrel", "uneven"])
def test_branch_invariants(preset):
    det = generate.Detector(preset)
    b = generate.generate(det, 60, seed=13)
    # (on the uneven workload's field map the branches end with the
    # sequence: run on to the loop-protection limit they would leave the map)
    tf = _branching(det, b, chi2_cut=30.0, max_candidates=2, chi2_cut_outlier=200.0,
                    end_of_world=int(preset == abi.CKG_UNEVEN))
    ok = tf.status == 0
    assert ok.sum() >= 0.5 * tf.n
    seq = np.split(b.seq_surfaces, b.seq_offsets[1:-1])
    for s in np.nonzero(ok)[0]:
        ns = tf.n_states[s]
        assert (tf.state_prev[s, :ns] < np.arange(ns)).all()
        for k in range(tf.n_tracks[s]):
            st = tf.track_states(s, k)
            fl = tf.state_flags[s, st]
            meas = (fl & abi.FLAG_HAS_MEASUREMENT) != 0
            out = (fl & abi.FLAG_IS_OUTLIER) != 0
            hole = (fl & abi.FLAG_IS_HOLE) != 0
            assert tf.track_n_measurements[s, k] == (meas & ~out).sum()
            assert tf.track_n_outliers[s, k] == out.sum()
            assert tf.track_n_holes[s, k] == hole.sum()
            # surfaces in the order of the seed's sequence
            pos = [list(seq[s]).index(x) for x in tf.state_surface[s, st]]
            assert pos == sorted(pos)
            c = tf.state_chi2[s, st][meas & ~out].sum()
            assert abs(c - tf.track_chi2[s, k]) <= 1e-9 * max(1.0, c)
            # holes and outliers carry their prediction as filtered state
            for i in np.array(st)[hole | out]:
                np.testing.assert_array_equal(tf.filtered[s, i], tf.predicted[s, i])


def test_branch_stopper_holes():
    det = generate.Detector(abi.CKG_BARREL)
    b = generate.generate(det, 200, seed=14)
    # a tight cut without outliers: a hole on a third of the surfaces
    tf = _find(det, generate.ckf_event(det, b), chi2_cut=2.0, chi2_cut_outlier=0.0, max_holes=0,
               min_measurements=3)
    ok = tf.status == 0
    assert ok.sum() > 0.3 * tf.n
    stopped = 0
    for s in np.nonzero(ok)[0]:
        for k in range(tf.n_tracks[s]):
            assert tf.track_n_holes[s, k] <= 1
            if tf.track_n_holes[s, k] == 1:
                # stopped at its first hole and kept: enough measurements
                stopped += 1
                last = tf.track_states(s, k)[-1]
                assert tf.state_flags[s, last] & abi.FLAG_IS_HOLE
                assert tf.track_n_measurements[s, k] >= 3
    assert stopped > 0
    # dropped: seeds whose first hole came before three measurements
    assert ((tf.n_tracks == 0) & ok).any()


def test_outliers_and_holes_when_nothing_passes():
    det, tf, _ = cubic_event()
    _find(det, tf, chi2_cut=0.0, chi2_cut_outlier=DMAX, target_surface=det.target)
    assert (tf.status == 0).all() and (tf.n_tracks == 1).all()
    assert (tf.track_n_outliers[:, 0] == 6).all() and (tf.track_n_measurements[:, 0] == 0).all()
    det, tf, _ = cubic_event()
    _find(det, tf, chi2_cut=0.0, chi2_cut_outlier=0.0, target_surface=det.target)
    assert (tf.track_n_holes[:, 0] == 6).all()
    for s in range(3):
        st = tf.track_states(s, 0)
        assert (tf.state_measurement[s, st] == -1).all()


def test_capacity_exceeded_fails_the_seed():
    det, tf, _ = cubic_event()
    _find(det, tf, chi2_cut=DMAX, target_surface=det.target, max_states=4)
    assert (tf.status == abi.TRACK_TOO_MANY_STATES).all()
    assert (tf.n_tracks == 0).all() and (tf.n_states == 0).all()


def test_zero_field_without_target_runs_into_the_step_limit():
    """The DirectNavigator never reaches an end of world: without a field
    (no loop protection) and without a target the search only ends at the
    propagator's step limit, an error of the seed as in the reference."""
    det, tf, _ = cubic_event()
    opt = abi.default_options(max_steps=200)
    _find(det, tf, opt, chi2_cut=DMAX)
    assert (tf.status == abi.TRACK_STEP_COUNT_LIMIT).all()


@pytest.mark.parametrize("bad", ["line_in_sequence", "bad_subspace"])
def test_invalid_input(bad):
    det, tf, _ = cubic_event()
    if bad == "bad_subspace":
        tf.meas_subspace[0] = 7
    else:
        tf.seq_surfaces[0] = 99
    _find(det, tf, chi2_cut=DMAX, target_surface=det.target)
    assert tf.status[0] == abi.TRACK_INVALID_INPUT


def test_end_of_world_ends_branches_with_the_sequence():
    """On the field map the searches that run on after their last surface
    leave the map (a field error of the seed, as with the reference's
    DirectNavigator); with end_of_world the branch ends with the sequence."""
    det = generate.Detector(abi.CKG_UNEVEN)
    b = generate.generate(det, 100, seed=15)
    plain = _find(det, generate.ckf_event(det, b), chi2_cut=15.0)
    assert (plain.status == abi.TRACK_FIELD_OUT_OF_BOUNDS).mean() > 0.5
    tf = _find(det, generate.ckf_event(det, b), chi2_cut=15.0, end_of_world=1)
    assert (tf.status == 0).all() and (tf.n_tracks == 1).all()
    assert np.isnan(tf.track_params[:, 0]).all()  # no target: no parameters
    own = hits = 0
    for s in range(tf.n):
        m = tf.track_measurements(s, 0)
        own += (tf.meas_track[m] == s).sum()
        hits += len(m)
    # (the seeds' wide start covariance lets a neighbour's hit through on
    # the innermost layers now and then)
    assert own >= 0.85 * hits, (own, hits)


def test_target_cylinder_around_the_seeds_is_reached_behind():
    """The actor's SurfaceReached has an unlimited near limit: a target
    cylinder around the origin intersects behind the seed first, the step
    turns back and the branch ends there with no state (the reference's
    behaviour; a target belongs beyond the sequence or behind the seed)."""
    base = generate.Detector(abi.CKG_BARREL)
    det = WithTarget(base)
    b = generate.generate(base, 20, seed=16)
    tf = _find(det, generate.ckf_event(det, b), chi2_cut=15.0, target_surface=det.target)
    assert (tf.status == 0).all() and (tf.n_tracks == 1).all()
    assert (tf.n_states == 0).all() and (tf.track_tip[:, 0] == -1).all()
    assert np.isfinite(tf.track_params[:, 0]).all()


def test_events_are_independent():
    """Several events in one call: each seed searches only its event's
    measurements, with the result of a call per event."""
    det = generate.Detector(abi.CKG_BARREL)
    b = generate.generate(det, 600, seed=41)
    sizes = [100, 250, 0, 250]
    multi = _find(det, generate.ckf_events(det, b, sizes), chi2_cut=15.0)
    assert (multi.status == 0).all()
    start = 0
    for m in sizes:
        if m == 0:
            continue
        one = _find(det, generate.ckf_event(det, b.subset(np.arange(start, start + m))),
                    chi2_cut=15.0)
        base = int(b.meas_offsets[start])
        for s in range(m):
            got = [[int(multi.meas_index[x]) for x in multi.track_measurements(start + s, k)]
                   for k in range(multi.n_tracks[start + s])]
            want = [[int(one.meas_index[x]) + base for x in one.track_measurements(s, k)]
                    for k in range(one.n_tracks[s])]
            assert got == want
            assert multi.track_chi2[start + s, 0] == one.track_chi2[s, 0]
        start += m
