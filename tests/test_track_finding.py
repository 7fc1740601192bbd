"""The examples' track-finding layer (acts_gb300.track_finding): an event's
measurements in arbitrary order, seeds and surface sequences from a store,
grouped by surface for the search, found tracks reported in the input's
measurement numbering. On the CPU the search is the oracle (as the finder
object); on the GPU the device finder must give the same tracks."""
import numpy as np
import pytest

from acts_gb300 import abi, generate
from acts_gb300.track_finding import TrackFindingAlgorithm
from acts_gb300.track_fitting import Measurements, ProcessCode, TrackParameters
from oracle import kforacle


class OracleFinder:
    """The restatement behind the finder interface (test only)."""

    def __init__(self, det):
        self.det = det

    def find_tracks(self, options, ckf_options, tf):
        kforacle.find_tracks(self.det.surfaces, self.det.field, options, ckf_options, tf,
                             n_threads=kforacle.hardware_threads())
        return tf


def _store(det, n, seed):
    b = generate.generate(det, n, seed=seed)
    nm = int(b.meas_offsets[-1])
    rng = np.random.default_rng(seed)
    perm = rng.permutation(nm)  # the input container's own order
    track = np.repeat(np.arange(n), np.diff(b.meas_offsets))
    meas = Measurements(surfaces=np.asarray(b.meas_surfaces[:nm])[perm],
                        values=b.meas_values.reshape(-1, 2)[:nm][perm],
                        covariances=b.meas_cov.reshape(-1, 4)[:nm][perm])
    initial = TrackParameters(params=b.start_params.reshape(n, 6),
                              covariance=b.start_cov.reshape(n, 6, 6),
                              frames=b.start_frames.reshape(n, 12),
                              particle=b.particle.reshape(n, 2), pdg=b.particle_pdg)
    seqs = [b.seq_surfaces[b.seq_offsets[i]:b.seq_offsets[i + 1]] for i in range(n)]
    store = {"measurements": meas, "initialparameters": initial, "surfacesequences": seqs}
    return store, track[perm]


def _algorithm(det, finder, **kw):
    return TrackFindingAlgorithm(TrackFindingAlgorithm.Config(finder=finder,
                                                              n_surfaces=det.n_surfaces, **kw))


def test_found_tracks_in_input_numbering():
    det = generate.Detector(abi.CKG_BARREL)
    store, truth = _store(det, 200, seed=31)
    alg = _algorithm(det, OracleFinder(det), chi2CutOff=15.0)
    assert alg.execute(store) == ProcessCode.SUCCESS
    found = store["tracks"]
    own = hits = 0
    for s in range(200):
        tr = found.tracks(s)
        assert len(tr) == 1
        own += (truth[tr[0]] == s).sum()
        hits += len(tr[0])
    assert own >= 0.99 * hits


def test_stopper_config_reaches_the_search():
    det = generate.Detector(abi.CKG_BARREL)
    store, _ = _store(det, 100, seed=32)
    alg = _algorithm(det, OracleFinder(det), chi2CutOff=2.0, chi2CutOffOutlier=0.0, maxHoles=0,
                     minMeasurements=3)
    alg.execute(store)
    tf = store["tracks"].finding
    T = np.arange(tf.max_tracks) < tf.n_tracks[:, None]
    assert (tf.track_n_holes[T] <= 1).all() and (tf.track_n_holes[T] == 1).any()


def test_inconsistent_inputs_abort():
    det = generate.Detector(abi.CKG_BARREL)
    store, _ = _store(det, 10, seed=33)
    store["surfacesequences"] = store["surfacesequences"][:5]
    assert _algorithm(det, OracleFinder(det)).execute(store) == ProcessCode.ABORT


@pytest.mark.gpu
def test_device_finder_matches_the_oracle():
    from acts_gb300.fitter import CudaKalman

    det = generate.Detector(abi.CKG_BARREL)
    store, _ = _store(det, 500, seed=34)
    ref = dict(store)
    _algorithm(det, OracleFinder(det), numMeasurementsCutOff=2, chi2CutOff=30.0,
               maxSteps=100000).execute(ref)
    fit = CudaKalman.for_detector(det)
    try:
        _algorithm(det, fit, numMeasurementsCutOff=2, chi2CutOff=30.0,
                   maxSteps=100000).execute(store)
    finally:
        fit.close()
    for s in range(500):
        assert store["tracks"].tracks(s) == ref["tracks"].tracks(s)
