"""The examples' track-fitting layer (acts_gb300/track_fitting.py):
TrackFittingAlgorithm over an event store with makeKalmanFitterFunction's
choices. CPU: the event's batch is assembled from the measurement container,
proto tracks, initial parameters and surface sequences exactly as the
generator's own batch (empty proto tracks and pickTrack give no track;
inconsistent inputs abort). GPU: the algorithm's tracks equal a direct batch
fit with the same options and the oracle's within 1e-9."""
import numpy as np
import pytest

from acts_gb300 import abi, generate
from acts_gb300.results import Results
from acts_gb300.track_fitting import (Measurements, ProcessCode, TrackFittingAlgorithm,
                                      TrackParameters, makeKalmanFitterFunction)


def _event(b, seed=5, empty=(3,)):
    """The event store of a generated batch: one measurement container in a
    shuffled order, proto tracks of measurement indices (some emptied)."""
    rng = np.random.default_rng(seed)
    nm = int(b.meas_offsets[-1])
    order = rng.permutation(nm)          # container position of batch measurement i
    inv = np.empty(nm, np.int64)
    inv[order] = np.arange(nm)
    meas = Measurements(
        surfaces=b.meas_surfaces[inv],
        values=b.meas_values.reshape(-1, 2)[inv].ravel(),
        covariances=b.meas_cov.reshape(-1, 4)[inv].ravel(),
        subspaces=None if b.meas_subspace is None else b.meas_subspace[inv])
    protos = [list(order[b.meas_offsets[t]:b.meas_offsets[t + 1]]) for t in range(b.n)]
    for t in empty:
        protos[t] = []
    seqs = [list(b.seq_surfaces[b.seq_offsets[t]:b.seq_offsets[t + 1]]) for t in range(b.n)]
    init = TrackParameters(params=b.start_params.reshape(-1, 6),
                           covariance=b.start_cov.reshape(-1, 6, 6),
                           frames=b.start_frames.reshape(-1, 12),
                           particle=b.particle.reshape(-1, 2), pdg=b.particle_pdg)
    return {"measurements": meas, "prototracks": protos, "initialparameters": init,
            "surfacesequences": seqs}


class _Recorder:
    def __init__(self):
        self.calls = []

    def __call__(self, batch, reference_surface, max_states, components):
        self.calls.append((batch, reference_surface))
        return Results(batch.n, max_states, components)


def test_event_batch_matches_the_generated_batch():
    det = generate.Detector(abi.CKG_STRIPS)
    b = generate.generate(det, 40, seed=9)
    store = _event(b)
    rec = _Recorder()
    alg = TrackFittingAlgorithm(TrackFittingAlgorithm.Config(fit=rec, referenceSurface=-1))
    assert alg.execute(store) == ProcessCode.SUCCESS
    (got, ref_surface), = rec.calls
    keep = [t for t in range(b.n) if t != 3]
    want = b.subset(keep)
    assert ref_surface == -1 and got.n == len(keep)
    for name in ("seq_offsets", "seq_surfaces", "meas_offsets", "meas_surfaces", "meas_values",
                 "meas_cov", "meas_subspace", "start_params", "start_cov", "start_frames",
                 "particle", "particle_pdg"):
        np.testing.assert_array_equal(getattr(got, name), getattr(want, name), err_msg=name)
    np.testing.assert_array_equal(store["tracks"].proto_track_index, keep)


def test_pick_track_and_inconsistent_inputs():
    det = generate.Detector(abi.CKG_BARREL)
    b = generate.generate(det, 10, seed=2)
    store = _event(b, empty=())
    rec = _Recorder()
    alg = TrackFittingAlgorithm(TrackFittingAlgorithm.Config(fit=rec, pickTrack=6))
    assert alg.execute(store) == ProcessCode.SUCCESS
    assert rec.calls[0][0].n == 1
    np.testing.assert_array_equal(store["tracks"].proto_track_index, [6])
    store["prototracks"] = store["prototracks"][:-1]
    assert alg.execute(store) == ProcessCode.ABORT
    with pytest.raises(ValueError):
        TrackFittingAlgorithm(TrackFittingAlgorithm.Config())


@pytest.mark.gpu
def test_algorithm_matches_batch_fit_and_oracle():
    from oracle import kforacle

    det = generate.Detector(abi.CKG_BARREL, perigee=True)
    b = generate.generate(det, 3000, seed=21)
    fn = makeKalmanFitterFunction(det, multipleScattering=True, energyLoss=True,
                                  reverseFilteringMomThreshold=1.0, chi2Cut=15.0)
    try:
        store = _event(b)
        alg = TrackFittingAlgorithm(TrackFittingAlgorithm.Config(fit=fn,
                                                                 referenceSurface=det.perigee))
        assert alg.execute(store) == ProcessCode.SUCCESS
        out = store["tracks"]
        sub = b.subset(out.proto_track_index)
        opt = fn.options.to_ck()
        opt.reference_surface = det.perigee
        comps = abi.OUT_ALL | abi.OUT_REFERENCE
        direct = fn.fitter.fit_batch(sub, opt, max_states=24, components=comps)
    finally:
        fn.close()
    got = out.results
    assert opt.smoother == abi.SMOOTHER_MBF and opt.reference_strategy == abi.EXTRAPOLATE_FIRST
    np.testing.assert_array_equal(got.status, direct.status)
    assert (got.status == 0).mean() > 0.99
    for name in ("track_params", "track_cov"):
        np.testing.assert_array_equal(getattr(got, name), getattr(direct, name))
    # some tracks are below the 1 GeV threshold: reverse-filtered
    sm = got.view("smoothed")
    rev = [np.isnan(sm[t, :got.n_states[t], 0]).any() for t in range(got.n)]
    assert 0.02 * got.n < sum(rev) < 0.5 * got.n
    from parity import assert_parity, compare
    ora = Results(sub.n, 24, comps)
    kforacle.fit_batch(det, sub, opt, ora, n_threads=kforacle.hardware_threads())
    rep = compare(got, ora, 1e-9)
    assert_parity(rep, 1e-9)


def test_csv_event_round_trip(tmp_path):
    """An event written as the examples' per-event CSV files (measurements
    with local_key, proto tracks) and read back gives the same batch; a
    measurement of phi is rejected."""
    from acts_gb300 import io_csv

    det = generate.Detector(abi.CKG_STRIPS)
    b = generate.generate(det, 30, seed=4)
    store = _event(b, empty=())
    gids = [(1 << 56) | (s + 1) << 20 for s in range(det.n_surfaces)]   # synthetic identifiers
    mpath = io_csv.per_event_filepath(str(tmp_path), "measurements.csv", 7)
    ppath = io_csv.per_event_filepath(str(tmp_path), "prototracks.csv", 7)
    assert mpath.endswith("event000000007-measurements.csv")
    io_csv.write_measurements(mpath, store["measurements"], gids)
    io_csv.write_proto_tracks(ppath, store["prototracks"])
    meas, ids = io_csv.read_measurements(mpath, {g: s for s, g in enumerate(gids)})
    protos = io_csv.read_proto_tracks(ppath, ids, n_tracks=b.n)
    store2 = dict(store, measurements=meas, prototracks=protos)
    r1, r2 = _Recorder(), _Recorder()
    TrackFittingAlgorithm(TrackFittingAlgorithm.Config(fit=r1)).execute(store)
    TrackFittingAlgorithm(TrackFittingAlgorithm.Config(fit=r2)).execute(store2)
    a, c = r1.calls[0][0], r2.calls[0][0]
    for name in ("meas_offsets", "meas_surfaces", "meas_subspace", "seq_surfaces"):
        np.testing.assert_array_equal(getattr(a, name), getattr(c, name), err_msg=name)
    # values and variances round-trip through the text exactly (repr)
    sub = a.meas_subspace
    np.testing.assert_array_equal(a.meas_values.reshape(-1, 2)[:, 0], c.meas_values.reshape(-1, 2)[:, 0])
    two = sub == abi.MEAS_LOC01
    np.testing.assert_array_equal(a.meas_values.reshape(-1, 2)[two], c.meas_values.reshape(-1, 2)[two])
    np.testing.assert_array_equal(a.meas_cov.reshape(-1, 4)[:, [0, 3]][two], c.meas_cov.reshape(-1, 4)[:, [0, 3]][two])
    text = open(mpath).read().splitlines()
    cols = text[1].split(",")
    cols[2] = str(1 << 3)    # phi
    open(mpath, "w").write("\n".join([text[0], ",".join(cols)] + text[2:]) + "\n")
    with pytest.raises(ValueError):
        io_csv.read_measurements(mpath, {g: s for s, g in enumerate(gids)})
