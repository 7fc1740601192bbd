"""The examples' track-finding layer over the batched track finder.

Mirrors the caller side of the reference's CKF
(Examples/Algorithms/TrackFinding/src/TrackFindingAlgorithm.cpp:185-261 and
its Config, include/ActsExamples/TrackFinding/TrackFindingAlgorithm.hpp:
78-145) for what the device search covers: the measurement selector's cuts
(chi2CutOff, chi2CutOffOutlier, numMeasurementsCutOff; one cut bin), the
branch stopper of a single TrackSelector config (minMeasurements, maxHoles,
maxOutliers, maxHolesAndOutliers; StopAndKeep with enough measurements,
else StopAndDrop), maxSteps, the target surface; one search direction along
each seed's DirectNavigator surface sequence. Not covered: two-way and
reverse search, seed deduplication, eta-binned cuts, pixel and strip hole
counts, shared hits, track trimming.

A store is a plain dict keyed by the configured collection names, as for
``track_fitting.TrackFittingAlgorithm``.
"""
from dataclasses import dataclass

import numpy as np

from . import abi
from .track_fitting import Measurements, ProcessCode, TrackParameters  # noqa: F401


@dataclass
class FoundTracks:
    """Output collection: the device search's arrays (an abi.TrackFinding)
    with the measurement numbering of the input container."""
    finding: abi.TrackFinding
    measurement_index: np.ndarray  # input index of each grouped measurement

    def tracks(self, seed):
        """The found tracks of a seed as lists of input measurement indices
        (outliers included), in the order the search kept them."""
        tf = self.finding
        return [[int(self.measurement_index[m]) for m in tf.track_measurements(seed, k)]
                for k in range(int(tf.n_tracks[seed]))]


def group_by_surface(measurements, n_surfaces):
    """Measurements grouped by surface (stable): (offsets [n_surfaces + 1],
    order) with order[i] the input index of grouped measurement i."""
    surf = np.asarray(measurements.surfaces, np.int64)
    if len(surf) and (surf.min() < 0 or surf.max() >= n_surfaces):
        raise ValueError("measurement surface outside the table")
    order = np.argsort(surf, kind="stable")
    offs = np.zeros(n_surfaces + 1, np.int32)
    offs[1:] = np.cumsum(np.bincount(surf, minlength=n_surfaces))
    return offs, order


class TrackFindingAlgorithm:
    """TrackFindingAlgorithm with one device call per event."""

    @dataclass
    class Config:
        inputMeasurements: str = "measurements"
        inputInitialTrackParameters: str = "initialparameters"
        # the DirectNavigator's surface sequence of each seed
        inputSurfaceSequences: str = "surfacesequences"
        outputTracks: str = "tracks"
        finder: object = None  # a CudaKalman on the surface table
        n_surfaces: int = 0
        # MeasurementSelector::Config (one bin)
        chi2CutOff: float = 15.0
        chi2CutOffOutlier: float = float("inf")
        numMeasurementsCutOff: int = 1
        # TrackSelector::Config of the branch stopper (None: no stopping)
        minMeasurements: int = 0
        maxHoles: int = abi.INT32_MAX
        maxOutliers: int = abi.INT32_MAX
        maxHolesAndOutliers: int = abi.INT32_MAX
        maxSteps: int = 100000
        targetSurface: int = -1
        endOfWorld: bool = False
        precision: int = abi.PRECISION_FP64
        maxStates: int = 64
        maxTracks: int = 16
        maxBranches: int = 16

    def __init__(self, config):
        if config.finder is None:
            raise ValueError("Missing track finder")
        for name in ("inputMeasurements", "inputInitialTrackParameters",
                     "inputSurfaceSequences", "outputTracks"):
            if not getattr(config, name):
                raise ValueError("Missing %s" % name)
        self.config = config

    def make_finding(self, measurements, initial, sequences):
        c = self.config
        offs, order = group_by_surface(measurements, c.n_surfaces)
        so = np.zeros(len(sequences) + 1, np.int32)
        so[1:] = np.cumsum([len(s) for s in sequences])
        seq = np.concatenate([np.asarray(s, np.int32) for s in sequences]) if len(sequences) \
            else np.zeros(0, np.int32)
        sub = None
        if measurements.subspaces is not None:
            sub = np.asarray(measurements.subspaces, np.int32)[order]
        tf = abi.TrackFinding(so, seq, np.asarray(initial.params, np.float64).reshape(-1, 6),
                              np.asarray(initial.covariance, np.float64).reshape(-1, 36),
                              np.asarray(initial.frames, np.float64).reshape(-1, 12),
                              np.asarray(initial.particle, np.float32).reshape(-1, 2), offs,
                              np.asarray(measurements.values, np.float64).reshape(-1, 2)[order],
                              np.asarray(measurements.covariances,
                                         np.float64).reshape(-1, 4)[order],
                              meas_subspace=sub,
                              particle_pdg=np.asarray(initial.pdg, np.int32),
                              max_states=c.maxStates, max_tracks=c.maxTracks)
        return tf, order

    def options(self, tf):
        c = self.config
        return tf.options(chi2_cut=c.chi2CutOff, chi2_cut_outlier=c.chi2CutOffOutlier,
                          max_candidates=c.numMeasurementsCutOff,
                          min_measurements=c.minMeasurements, max_holes=c.maxHoles,
                          max_outliers=c.maxOutliers,
                          max_holes_and_outliers=c.maxHolesAndOutliers,
                          target_surface=c.targetSurface, max_branches=c.maxBranches,
                          end_of_world=int(c.endOfWorld))

    def execute(self, store):
        c = self.config
        measurements = store[c.inputMeasurements]
        initial = store[c.inputInitialTrackParameters]
        sequences = store[c.inputSurfaceSequences]
        if len(initial) != len(sequences):
            return ProcessCode.ABORT
        tf, order = self.make_finding(measurements, initial, sequences)
        opt = abi.default_options(precision=c.precision, max_steps=c.maxSteps)
        if tf.n:
            c.finder.find_tracks(opt, self.options(tf), tf)
        store[c.outputTracks] = FoundTracks(tf, order.astype(np.int64))
        return ProcessCode.SUCCESS
