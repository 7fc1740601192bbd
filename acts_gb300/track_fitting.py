"""The examples' track-fitting layer over the batched fitter.

Mirrors the caller side of the reference's fit:

* ``makeKalmanFitterFunction`` (Examples/Algorithms/TrackFitting/src/
  KalmanFitterFunction.cpp:159-200, bound to Python in
  Python/Examples/src/TrackFitting.cpp:50-67): the same arguments, and the
  same fixed choices of the function object — GainMatrixUpdater (Joseph form
  by ``useJosephFormulation``), MbfSmoother, the predicted-chi2 outlier finder
  (``chi2Cut``), the momentum-threshold reverse-filtering logic, the
  extrapolation strategy ``first`` (KalmanFitterFunction.cpp:100-131) — with
  the surface sequence of the direct fitter.
* ``TrackFittingAlgorithm`` (Examples/Algorithms/TrackFitting/src/
  TrackFittingAlgorithm.cpp:38-170): reads the measurements, proto tracks,
  initial parameters and surface sequences of an event from a store, and
  writes the fitted tracks; the perigee surface at the origin is the reference
  surface. The reference calls the fitter once per proto track; here the
  whole event is one batch (empty proto tracks and ``pickTrack`` behave as
  there: no track).

A store is a plain dict keyed by the configured collection names.
"""
from dataclasses import dataclass, field as dc_field
from enum import IntEnum

import numpy as np

from . import abi
from .fitter import CudaKalman, KalmanFitterOptions
from .generate import Batch


class ProcessCode(IntEnum):
    """ActsExamples::ProcessCode"""
    SUCCESS = 0
    ABORT = 1
    END = 2


@dataclass
class Measurements:
    """A measurement container: per measurement its surface id, measured
    local values (2; the second ignored for 1D), 2x2 covariance (row-major)
    and subspace (abi.MEAS_LOC0 / MEAS_LOC1 / MEAS_LOC01)."""
    surfaces: np.ndarray
    values: np.ndarray
    covariances: np.ndarray
    subspaces: np.ndarray = None

    def __len__(self):
        return len(self.surfaces)


@dataclass
class TrackParameters:
    """Bound start parameters of each proto track on its own plane: params
    (n, 6), covariance (n, 6, 6), the plane frame (n, 12: rotation row-major
    then centre), and the particle hypothesis (mass, |q|) with its PDG code."""
    params: np.ndarray
    covariance: np.ndarray
    frames: np.ndarray
    particle: np.ndarray
    pdg: np.ndarray

    def __len__(self):
        return len(self.params)


@dataclass
class FittedTracks:
    """Output collection: the fit results of the fitted proto tracks, in the
    order of ``proto_track_index`` (the proto track each came from)."""
    results: object
    proto_track_index: np.ndarray


class TrackFitterFunction:
    """The function object: holds the device fitter and the fit options."""

    def __init__(self, fitter, options):
        self.fitter = fitter
        self.options = options

    def __call__(self, batch, reference_surface, max_states=24, components=abi.OUT_ALL):
        opt = self.options.to_ck()
        opt.reference_surface = reference_surface
        comps = components | (abi.OUT_REFERENCE if reference_surface >= 0 else 0)
        return self.fitter.fit_batch(batch, opt, max_states=max_states, components=comps)

    def close(self):
        self.fitter.close()


def makeKalmanFitterFunction(detector, multipleScattering=True, energyLoss=True,
                             reverseFilteringMomThreshold=0.0,
                             reverseFilteringCovarianceScaling=100.0,
                             freeToBoundCorrection=False, chi2Cut=float("inf"),
                             useJosephFormulation=False, precision=abi.PRECISION_FP64,
                             fitter=None):
    """KalmanFitterFunction.cpp:159-200. `detector`: an acts_gb300.generate
    Detector (or any object with surfaces / n_surfaces / field); `fitter`: an
    existing CudaKalman to share instead of creating one."""
    opts = KalmanFitterOptions(
        multiple_scattering=bool(multipleScattering),
        energy_loss=bool(energyLoss),
        reverse_filtering_mom_threshold=float(reverseFilteringMomThreshold),
        reverse_filtering_cov_scaling=float(reverseFilteringCovarianceScaling),
        free_to_bound_correction=bool(freeToBoundCorrection),
        outlier_chi2_cut=float(chi2Cut),
        use_joseph=bool(useJosephFormulation),
        smoother=abi.SMOOTHER_MBF,
        reference_strategy=abi.EXTRAPOLATE_FIRST,
        precision=precision,
    )
    return TrackFitterFunction(fitter or CudaKalman.for_detector(detector), opts)


class TrackFittingAlgorithm:
    """TrackFittingAlgorithm with one batched fit per event."""

    @dataclass
    class Config:
        inputMeasurements: str = "measurements"
        inputProtoTracks: str = "prototracks"
        inputInitialTrackParameters: str = "initialparameters"
        # the DirectNavigator's surface sequence of each proto track
        inputSurfaceSequences: str = "surfacesequences"
        outputTracks: str = "tracks"
        fit: object = None
        # the perigee surface at the origin (a line surface of the table), or -1
        referenceSurface: int = -1
        pickTrack: int = -1
        maxStates: int = 24
        components: int = abi.OUT_ALL
        extra: dict = dc_field(default_factory=dict)

    def __init__(self, config):
        if config.fit is None:
            raise ValueError("Missing fit function")
        for name in ("inputMeasurements", "inputProtoTracks", "inputInitialTrackParameters",
                     "inputSurfaceSequences", "outputTracks"):
            if not getattr(config, name):
                raise ValueError("Missing %s" % name)
        self.config = config

    @staticmethod
    def make_batch(measurements, proto_tracks, initial, sequences, selected):
        """The CSR batch of the selected proto tracks (source links by
        measurement index, as the reference's IndexSourceLink)."""
        n = len(selected)
        b = Batch(n, 1)
        so, mo = [0], [0]
        seq, mi = [], []
        for t in selected:
            seq.extend(int(s) for s in sequences[t])
            so.append(len(seq))
            mi.extend(int(m) for m in proto_tracks[t])
            mo.append(len(mi))
        mi = np.asarray(mi, dtype=np.int64)
        b.seq_offsets = np.asarray(so, np.int32)
        b.seq_surfaces = np.asarray(seq, np.int32)
        b.meas_offsets = np.asarray(mo, np.int32)
        b.meas_surfaces = np.ascontiguousarray(np.asarray(measurements.surfaces, np.int32)[mi])
        b.meas_values = np.ascontiguousarray(
            np.asarray(measurements.values, np.float64).reshape(-1, 2)[mi].ravel())
        b.meas_cov = np.ascontiguousarray(
            np.asarray(measurements.covariances, np.float64).reshape(-1, 4)[mi].ravel())
        if measurements.subspaces is not None:
            b.meas_subspace = np.ascontiguousarray(np.asarray(measurements.subspaces, np.int32)[mi])
        sel = np.asarray(selected, dtype=np.int64)
        b.start_params = np.ascontiguousarray(np.asarray(initial.params, np.float64)[sel].ravel())
        b.start_cov = np.ascontiguousarray(np.asarray(initial.covariance, np.float64)[sel].ravel())
        b.start_frames = np.ascontiguousarray(np.asarray(initial.frames, np.float64)[sel].ravel())
        b.particle = np.ascontiguousarray(np.asarray(initial.particle, np.float32)[sel].ravel())
        b.particle_pdg = np.ascontiguousarray(np.asarray(initial.pdg, np.int32)[sel])
        b.truth_meas = np.zeros(6 * len(mi))
        b.meas_outlier = np.zeros(len(mi), np.uint8)
        b.truth_start = np.zeros(6 * n)
        return b

    def execute(self, store):
        c = self.config
        measurements = store[c.inputMeasurements]
        proto_tracks = store[c.inputProtoTracks]
        initial = store[c.inputInitialTrackParameters]
        sequences = store[c.inputSurfaceSequences]
        # consistency cross checks (TrackFittingAlgorithm.cpp:83-88)
        if len(proto_tracks) != len(initial) or len(proto_tracks) != len(sequences):
            return ProcessCode.ABORT
        selected = [t for t in range(len(proto_tracks))
                    if (c.pickTrack < 0 or c.pickTrack == t) and len(proto_tracks[t]) > 0]
        batch = self.make_batch(measurements, proto_tracks, initial, sequences, selected)
        results = c.fit(batch, c.referenceSurface, max_states=c.maxStates,
                        components=c.components)
        store[c.outputTracks] = FittedTracks(results, np.asarray(selected, dtype=np.int64))
        return ProcessCode.SUCCESS
