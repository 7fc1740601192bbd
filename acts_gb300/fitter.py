"""Python host mirror of ActsPlugins::CudaKalman over the C ABI.

CudaKalman keeps the shape of the reference call
    Acts::KalmanFitter<Propagator<EigenStepper<>, DirectNavigator>, ...>
        ::fit(begin, end, startParameters, kfOptions, sSequence, trackContainer)
(Core/include/Acts/TrackFitting/KalmanFitter.hpp:719-731): fit() takes one
track's source links, start parameters, options and DirectNavigator surface
sequence and returns a FitResult that is either a fitted track or the error
name the reference would return (KalmanFitterError / PropagatorError ...).
fit_batch() is the batched entry that replaces the serial per-track loop of
TrackFittingAlgorithm::execute
(Examples/Algorithms/TrackFitting/src/TrackFittingAlgorithm.cpp:117-170).

There is no CPU path: constructing a CudaKalman without the CUDA library or
without a GPU raises.
"""
import ctypes as C
import os
from dataclasses import dataclass, field as dc_field

import numpy as np

from . import abi
from .build import LIBDIR
from .results import Results

_lib = None


class CudaKalmanError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (status %d): %s" % (_status_name(status), status, message))
        self.status = status


def _status_name(s):
    names = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "no CUDA device",
             4: "out of device memory", 5: "unsupported", 6: "budget", 7: "timeout",
             8: "not ready", 9: "scratch limit"}
    return names.get(s, "unknown")


def lib():
    """The loaded libcudakalman.so (raises when it is missing)."""
    global _lib
    if _lib is None:
        path = os.path.join(LIBDIR, "libcudakalman.so")
        if not os.path.exists(path):
            raise CudaKalmanError(abi.CK_ERR_NO_DEVICE,
                                  "libcudakalman.so is not built; run __graft_entry__.build()")
        L = C.CDLL(path)
        P = C.POINTER
        L.ck_api_version.restype = C.c_int32
        L.ck_last_error.restype = C.c_char_p
        L.ck_options_default.argtypes = [P(abi.ck_options)]
        L.ck_create.argtypes = [P(abi.ck_config), P(C.c_void_p)]
        L.ck_destroy.argtypes = [C.c_void_p]
        L.ck_fit_batch.argtypes = [C.c_void_p, P(abi.ck_options), P(abi.ck_batch_in),
                                   P(abi.ck_batch_out), C.c_void_p]
        L.ck_fit_batch_static.argtypes = [C.c_void_p, P(abi.ck_options), P(abi.ck_batch_in),
                                          P(abi.ck_batch_out), C.c_void_p]
        L.ck_static_scratch_bytes.argtypes = [C.c_int32, C.c_int32, C.c_int32]
        L.ck_static_scratch_bytes.restype = C.c_int64
        L.ck_static_scratch_bytes_for.argtypes = [P(abi.ck_options), C.c_int32, C.c_int32]
        L.ck_static_scratch_bytes_for.restype = C.c_int64
        L.ck_static_scratch_capacity.restype = C.c_int64
        L.ck_sync.argtypes = [C.c_void_p]
        L.ck_set_steps_per_round.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
        L.ck_set_grid_blocks.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
        L.ck_set_smoother_staging.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
        L.ck_set_host_chunk_tracks.argtypes = [C.c_void_p, C.c_int32]
        L.ck_last_kernel_split_ms.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
        L.ck_atan2_mixed.argtypes = [C.c_void_p, C.c_int32, P(C.c_double), P(C.c_double),
                                     P(C.c_double)]
        L.ck_last_kernel_ms.argtypes = [C.c_void_p, P(C.c_double)]
        L.ck_last_launch_count.argtypes = [C.c_void_p, P(C.c_int32)]
        L.ck_last_transfer_bytes.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_int64)]
        L.ck_get_launch_config.argtypes = [C.c_void_p, C.c_int32, P(C.c_int32), P(C.c_int32)]
        L.ck_get_launch_variant.argtypes = [C.c_void_p, C.c_int32, P(C.c_int32), P(C.c_int32)]
        L.ck_set_launch_config.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
        L.ck_sort_queue.argtypes = [C.c_void_p, C.c_int32]
        L.ck_set_tail_smoothing.argtypes = [C.c_void_p, C.c_int32]
        L.ck_autotune.argtypes = [C.c_void_p, P(abi.ck_options), P(abi.ck_batch_in),
                                  P(abi.ck_batch_out)]
        L.ck_autotune_log.restype = C.c_char_p
        L.ck_autotune_log.argtypes = [C.c_void_p]
        L.ck_gain_matrix_update.argtypes = ([C.c_void_p, C.c_int32, C.c_int32] + [abi.P_f64] * 4 +
                                            [abi.P_i32] + [abi.P_f64] * 3 + [abi.P_i32])
        L.ck_gain_matrix_smooth.argtypes = [C.c_void_p, C.c_int32, C.c_int32] + [abi.P_f64] * 7 + [abi.P_i32]
        L.ck_mbf_smooth.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_uint32)] + [abi.P_f64] * 9
        L.ck_material_effects.argtypes = [C.c_void_p, C.c_int32, abi.P_i32, abi.P_f32, abi.P_f64,
                                          abi.P_f64, abi.P_f32, abi.P_f32, abi.P_i32, C.c_int32,
                                          C.c_int32, abi.P_f64]
        L.ck_field_lookup.argtypes = [C.c_void_p, C.c_int32, abi.P_f64, abi.P_f64, abi.P_i32]
        L.ck_propagate.argtypes = [C.c_void_p, P(abi.ck_options), P(abi.ck_propagate_in),
                                   P(abi.ck_propagate_out), C.c_void_p]
        L.ck_find_tracks.argtypes = [C.c_void_p, P(abi.ck_options), P(abi.ck_ckf_options),
                                     P(abi.ck_ckf_in), P(abi.ck_ckf_out), C.c_void_p]
        L.ck_ckf_options_default.argtypes = [P(abi.ck_ckf_options)]
        L.ck_ckf_options_default.restype = None
        L.ck_last_ckf_lanes.argtypes = [C.c_void_p]
        L.ck_last_ckf_lanes.restype = C.c_int32
        L.ck_simulate.argtypes = [C.c_void_p, C.c_int32, C.c_uint64, C.c_int64, C.c_int32,
                                  P(abi.ckg_out), C.c_void_p]
        L.ck_field_lookup_precision.argtypes = [C.c_void_p, C.c_int32, C.c_int32, abi.P_f64,
                                                abi.P_f64, abi.P_i32]
        L.ck_fp_peak_gflops.argtypes = [C.c_void_p, C.c_int32, P(C.c_double)]
        L.ck_abi_struct_sizes.argtypes = [P(C.c_int64), C.c_int32]
        L.ck_abi_struct_sizes.restype = None
        _lib = L
    return _lib


def _check(status):
    if status != abi.CK_OK:
        raise CudaKalmanError(status, lib().ck_last_error().decode())


@dataclass
class KalmanFitterOptions:
    """Mirror of Acts::KalmanFitterOptions + the plain stepper / propagator
    options it carries (KalmanFitter.hpp:108-186, StepperOptions.hpp:36-49,
    PropagatorOptions.hpp:28-51), with the fitter's extension choices."""

    multiple_scattering: bool = True
    energy_loss: bool = True
    reverse_filtering: bool = False
    reverse_filtering_cov_scaling: float = 100.0
    reverse_filtering_mom_threshold: float = 0.0  # GeV (the examples' reverseFilteringMomThreshold)
    free_to_bound_correction: bool = False
    reference_surface: int = -1  # a line (perigee) surface of the table, or -1
    reference_strategy: int = abi.EXTRAPOLATE_FIRST_OR_LAST
    use_joseph: bool = False
    outlier_chi2_cut: float = float("inf")
    precision: int = abi.PRECISION_FP64
    step_tolerance: float = 1e-4
    max_steps: int = 1000
    initial_step_size: float = 10000.0
    loop_protection: bool = True
    loop_fraction: float = 0.5
    early_termination: bool = False
    smoother: int = abi.SMOOTHER_GAIN_MATRIX  # or abi.SMOOTHER_MBF (MbfSmoother)
    extra: dict = dc_field(default_factory=dict)

    def to_ck(self):
        o = abi.default_options()
        o.multiple_scattering = int(self.multiple_scattering)
        o.energy_loss = int(self.energy_loss)
        o.reverse_filtering = int(self.reverse_filtering)
        o.reverse_filtering_cov_scaling = float(self.reverse_filtering_cov_scaling)
        o.reverse_filtering_mom_threshold = float(self.reverse_filtering_mom_threshold)
        o.free_to_bound_correction = int(self.free_to_bound_correction)
        o.reference_surface = int(self.reference_surface)
        o.reference_strategy = int(self.reference_strategy)
        o.use_joseph = int(self.use_joseph)
        o.outlier_chi2_cut = float(self.outlier_chi2_cut)
        o.precision = int(self.precision)
        o.step_tolerance = float(self.step_tolerance)
        o.max_steps = int(self.max_steps)
        o.initial_step_size = float(self.initial_step_size)
        o.loop_protection = int(self.loop_protection)
        o.loop_fraction = float(self.loop_fraction)
        o.early_termination = int(self.early_termination)
        o.smoother = int(self.smoother)
        for k, v in self.extra.items():
            setattr(o, k, v)
        return o


@dataclass
class SourceLink:
    """A calibrated 2D measurement on (loc0, loc1) of a surface, what the
    reference's TestSourceLink + testSourceLinkCalibrator provide."""

    surface: int
    value: tuple
    covariance: tuple  # row-major 2x2


@dataclass
class BoundTrackParameters:
    """Start parameters on a plane (rotation 3x3 row-major with the local axes
    as columns, center) with the particle hypothesis."""

    params: np.ndarray
    covariance: np.ndarray
    plane_rotation: np.ndarray
    plane_center: np.ndarray
    mass: float
    abs_charge: float = 1.0
    pdg: int = 211


@dataclass
class TrackState:
    surface: int
    flags: int
    path_length: float
    chi2: float
    predicted: np.ndarray
    predicted_covariance: np.ndarray
    filtered: np.ndarray
    filtered_covariance: np.ndarray
    smoothed: np.ndarray
    smoothed_covariance: np.ndarray
    jacobian: np.ndarray


@dataclass
class FitResult:
    """Result<TrackProxy>: ok() and either the track or the error name."""

    status: int
    states: list = None
    n_measurements: int = 0
    n_holes: int = 0
    n_outliers: int = 0
    chi2: float = 0.0
    ndf: int = 0

    def ok(self):
        return self.status == 0

    @property
    def error(self):
        return None if self.ok() else abi.TRACK_STATUS.get(self.status, "unknown")


class CudaKalman:
    """A fitter bound to one GPU, one surface table and one field."""

    def __init__(self, surfaces, n_surfaces, field, device=0, use_graph=True,
                 autotune_cache=None, threads_per_block=0, blocks_per_sm=0):
        L = lib()
        cfg = abi.ck_config()
        cfg.device = device
        cfg.n_surfaces = n_surfaces
        cfg.surfaces = C.cast(surfaces, C.POINTER(abi.ck_surface))
        cfg.field = field
        cfg.threads_per_block = threads_per_block
        cfg.blocks_per_sm = blocks_per_sm
        cfg.use_graph = int(use_graph)
        cfg.autotune_cache = autotune_cache.encode() if autotune_cache else None
        h = C.c_void_p()
        _check(L.ck_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._keep = (surfaces, field)

    @classmethod
    def for_detector(cls, det, **kw):
        return cls(det.surfaces, det.n_surfaces, det.field, **kw)

    def close(self):
        if getattr(self, "_h", None):
            lib().ck_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # ------------------------------------------------------------ batched
    def fit_batch(self, batch, options, max_states=24, components=abi.OUT_ALL, results=None,
                  sync=True):
        """Fits every track of `batch` (acts_gb300.generate.Batch or an object
        exposing as_batch_in()); returns a Results."""
        if isinstance(options, KalmanFitterOptions):
            options = options.to_ck()
        res = results or Results(batch.n, max_states, components)
        bi = batch.as_batch_in()
        bo = res.as_batch_out()
        _check(lib().ck_fit_batch(self._h, C.byref(options), C.byref(bi), C.byref(bo), None))
        if sync:
            _check(lib().ck_sync(self._h))
        return res

    def fit_batch_raw(self, options, batch_in, batch_out, stream=None):
        _check(lib().ck_fit_batch(self._h, C.byref(options), C.byref(batch_in),
                                  C.byref(batch_out), stream))

    def fit_batch_static(self, options, batch_in, batch_out, stream=None):
        """ck_fit_batch_static: device-resident batch, pipeline scratch in the
        library's static device array (no allocation)."""
        _check(lib().ck_fit_batch_static(self._h, C.byref(options), C.byref(batch_in),
                                         C.byref(batch_out), stream))

    @staticmethod
    def static_scratch_bytes(n_tracks, max_states, precision):
        return lib().ck_static_scratch_bytes(int(n_tracks), int(max_states), int(precision))

    @staticmethod
    def static_scratch_bytes_for(options, n_tracks, max_states):
        """Exact scratch bytes of a ck_fit_batch_static call with these
        options (extrapolation start states included)."""
        return lib().ck_static_scratch_bytes_for(C.byref(options), int(n_tracks), int(max_states))

    @staticmethod
    def static_scratch_capacity():
        return lib().ck_static_scratch_capacity()

    def sync(self):
        _check(lib().ck_sync(self._h))

    def last_kernel_ms(self):
        ms = C.c_double()
        _check(lib().ck_last_kernel_ms(self._h, C.byref(ms)))
        return ms.value

    def last_kernel_split_ms(self):
        """(forward-filter ms, smoother ms) of the most recent timed batch."""
        a, b = C.c_double(), C.c_double()
        _check(lib().ck_last_kernel_split_ms(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_steps_per_round(self, precision, steps):
        _check(lib().ck_set_steps_per_round(self._h, int(precision), int(steps)))

    def set_smoother_staging(self, precision, enable):
        """RTS smoother with warp-cooperative record staging (1) or per-lane
        record reads (0); identical results."""
        _check(lib().ck_set_smoother_staging(self._h, int(precision), int(enable)))

    def set_grid_blocks(self, precision, blocks):
        """Grid of the forward-filter kernel (0: the whole GPU)."""
        _check(lib().ck_set_grid_blocks(self._h, int(precision), int(blocks)))

    def set_host_chunk_tracks(self, tracks):
        """Tracks per chunk of host-memory batches (0: default; < 0: never chunk)."""
        _check(lib().ck_set_host_chunk_tracks(self._h, int(tracks)))

    def last_launch_count(self):
        n = C.c_int32()
        _check(lib().ck_last_launch_count(self._h, C.byref(n)))
        return n.value

    def last_transfer_bytes(self):
        a, b = C.c_int64(), C.c_int64()
        _check(lib().ck_last_transfer_bytes(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def launch_config(self, precision):
        t, b = C.c_int32(), C.c_int32()
        _check(lib().ck_get_launch_config(self._h, precision, C.byref(t), C.byref(b)))
        return t.value, b.value

    def launch_variant(self, precision):
        """(forward-filter kernel variant, Runge-Kutta trials per round)."""
        v, spr = C.c_int32(), C.c_int32()
        _check(lib().ck_get_launch_variant(self._h, int(precision), C.byref(v), C.byref(spr)))
        return v.value, spr.value

    def set_launch_config(self, precision, variant, tpb, bps):
        _check(lib().ck_set_launch_config(self._h, precision, variant, tpb, bps))

    def atan2_mixed(self, y, x):
        """The mixed form's FP64 atan2 on the device (numpy arrays in, out)."""
        y = np.ascontiguousarray(y, np.float64)
        x = np.ascontiguousarray(x, np.float64)
        out = np.empty_like(y)
        _check(lib().ck_atan2_mixed(self._h, y.size, abi.ptr(y, C.c_double), abi.ptr(x, C.c_double),
                                    abi.ptr(out, C.c_double)))
        return out

    def fp_peak_gflops(self, precision):
        g = C.c_double()
        _check(lib().ck_fp_peak_gflops(self._h, precision, C.byref(g)))
        return g.value

    def sort_queue(self, enable):
        _check(lib().ck_sort_queue(self._h, int(enable)))

    def set_tail_smoothing(self, enable):
        """Smoothing in the forward filter's tail (default on; results do not
        depend on it)."""
        _check(lib().ck_set_tail_smoothing(self._h, int(enable)))

    def autotune(self, options, batch_in_device, batch_out_device):
        _check(lib().ck_autotune(self._h, C.byref(options), C.byref(batch_in_device),
                                 C.byref(batch_out_device)))
        return lib().ck_autotune_log(self._h).decode()

    # ------------------------------------------------------- single track
    def fit(self, source_links, start, options, surface_sequence, max_states=64):
        """KalmanFitter::fit for one track (a batch of one)."""
        from .generate import Batch

        b = Batch(1, max(1, len(surface_sequence), len(source_links)))
        b.seq_offsets[:] = [0, len(surface_sequence)]
        b.seq_surfaces = np.ascontiguousarray(np.asarray(surface_sequence, np.int32))
        b.meas_offsets[:] = [0, len(source_links)]
        b.meas_surfaces = np.ascontiguousarray(np.array([s.surface for s in source_links], np.int32))
        b.meas_values = np.ascontiguousarray(
            np.array([v for s in source_links for v in s.value], np.float64))
        b.meas_cov = np.ascontiguousarray(
            np.array([v for s in source_links for v in s.covariance], np.float64))
        b.start_params = np.ascontiguousarray(np.asarray(start.params, np.float64).reshape(6))
        b.start_cov = np.ascontiguousarray(np.asarray(start.covariance, np.float64).reshape(36))
        b.start_frames = np.ascontiguousarray(np.concatenate(
            [np.asarray(start.plane_rotation, np.float64).reshape(9),
             np.asarray(start.plane_center, np.float64).reshape(3)]))
        b.particle = np.array([start.mass, start.abs_charge], np.float32)
        b.particle_pdg = np.array([start.pdg], np.int32)
        res = self.fit_batch(b, options, max_states=max_states)
        return track_result(res, 0)

    # ------------------------------------------------------ unit operators
    def gain_matrix_update(self, pred, pred_cov, meas, meas_cov, joseph=False, subspace=None):
        n = len(pred)
        f = np.zeros((n, 6))
        fc = np.zeros((n, 36))
        chi2 = np.zeros(n)
        st = np.zeros(n, np.int32)
        a = [np.ascontiguousarray(x, np.float64) for x in (pred, pred_cov, meas, meas_cov)]
        sub = None if subspace is None else np.ascontiguousarray(subspace, np.int32)
        _check(lib().ck_gain_matrix_update(self._h, n, int(joseph),
                                           *[abi.ptr(x, C.c_double) for x in a],
                                           abi.ptr(sub, C.c_int32),
                                           abi.ptr(f, C.c_double), abi.ptr(fc, C.c_double),
                                           abi.ptr(chi2, C.c_double), abi.ptr(st, C.c_int32)))
        return f, fc.reshape(n, 6, 6), chi2, st

    def gain_matrix_smooth(self, pred, pred_cov, filt, filt_cov, jac):
        nt, ns = pred.shape[:2]
        s = np.zeros((nt, ns, 6))
        sc = np.zeros((nt, ns, 36))
        st = np.zeros(nt, np.int32)
        a = [np.ascontiguousarray(x, np.float64) for x in (pred, pred_cov, filt, filt_cov, jac)]
        _check(lib().ck_gain_matrix_smooth(self._h, nt, ns, *[abi.ptr(x, C.c_double) for x in a],
                                           abi.ptr(s, C.c_double), abi.ptr(sc, C.c_double),
                                           abi.ptr(st, C.c_int32)))
        return s, sc.reshape(nt, ns, 6, 6), st

    def mbf_smooth(self, flags, pred, pred_cov, filt, filt_cov, jac, meas, meas_cov):
        """MbfSmoother on trajectories (arrays shaped [n_traj, n_states, ...])."""
        nt, ns = pred.shape[:2]
        s = np.zeros((nt, ns, 6))
        sc = np.zeros((nt, ns, 36))
        fl = np.ascontiguousarray(flags, np.uint32)
        a = [np.ascontiguousarray(x, np.float64)
             for x in (pred, pred_cov, filt, filt_cov, jac, meas, meas_cov)]
        _check(lib().ck_mbf_smooth(self._h, nt, ns, abi.ptr(fl, C.c_uint32),
                                   *[abi.ptr(x, C.c_double) for x in a],
                                   abi.ptr(s, C.c_double), abi.ptr(sc, C.c_double)))
        return s, sc.reshape(nt, ns, 6, 6)

    def material_effects(self, surface_ids, scale, directions, qop, mass, absq, pdg, ms=True,
                         el=True):
        n = len(surface_ids)
        out = np.zeros((n, 4))
        arrs = dict(s=np.ascontiguousarray(surface_ids, np.int32),
                    sc=np.ascontiguousarray(scale, np.float32),
                    d=np.ascontiguousarray(directions, np.float64),
                    q=np.ascontiguousarray(qop, np.float64),
                    m=np.ascontiguousarray(mass, np.float32),
                    a=np.ascontiguousarray(absq, np.float32),
                    p=np.ascontiguousarray(pdg, np.int32))
        _check(lib().ck_material_effects(self._h, n, abi.ptr(arrs["s"], C.c_int32),
                                         abi.ptr(arrs["sc"], C.c_float), abi.ptr(arrs["d"], C.c_double),
                                         abi.ptr(arrs["q"], C.c_double), abi.ptr(arrs["m"], C.c_float),
                                         abi.ptr(arrs["a"], C.c_float), abi.ptr(arrs["p"], C.c_int32),
                                         int(ms), int(el), abi.ptr(out, C.c_double)))
        return out

    def propagate(self, options, prop):
        """ck_propagate on an abi.Propagation (host arrays, filled in place):
        Propagator::propagate(start[, target], options) with the fitter's
        stepper in the options' precision form."""
        i, o = prop.as_in(), prop.as_out()
        _check(lib().ck_propagate(self._h, C.byref(options), C.byref(i), C.byref(o), None))
        return prop

    def find_tracks(self, options, ckf_options, tf):
        """ck_find_tracks on an abi.TrackFinding (host arrays, filled in
        place): CombinatorialKalmanFilter::findTracks from each seed along
        its surface sequence, in the options' precision form."""
        i, o = tf.as_in(), tf.as_out()
        self.find_tracks_raw(options, ckf_options, i, o)
        return tf

    def find_tracks_raw(self, options, ckf_options, ck_in, ck_out, stream=None):
        """ck_find_tracks on ck_ckf_in / ck_ckf_out structures (host or
        device memory); `stream` a cudaStream_t as an integer (None: the
        handle's stream)."""
        _check(lib().ck_find_tracks(self._h, C.byref(options), C.byref(ckf_options),
                                    C.byref(ck_in), C.byref(ck_out),
                                    None if stream is None else C.c_void_p(stream)))

    def simulate(self, preset, n_tracks, seed=1, first_track=0, cap=24, device="cuda:0"):
        """ck_simulate: tracks [first_track, first_track + n_tracks) of a
        generator preset simulated and digitised on the GPU through this
        handle's surfaces and field; returns a generate.DeviceBatch (torch
        tensors in device memory, CSR rows of at most `cap` entries)."""
        import torch

        from .generate import DeviceBatch

        b = DeviceBatch(n_tracks, cap, torch, device, strips=preset == abi.CKG_STRIPS)
        o = b.as_ckg_out()
        torch.cuda.synchronize(device)  # (the allocations precede the launches)
        stream = torch.cuda.current_stream(device)
        s = stream.cuda_stream
        _check(lib().ck_simulate(self._h, int(preset), int(seed), int(first_track), int(n_tracks),
                                 C.byref(o), C.c_void_p(s) if s else None))
        if not s:
            self.sync()
        torch.cuda.synchronize(device)
        return b.trim()

    def last_ckf_lanes(self):
        """Lanes per seed of the last track-finding launch."""
        return int(lib().ck_last_ckf_lanes(self._h))

    def field_lookup(self, pos, precision=abi.PRECISION_FP64):
        """getField on the device in a form's stepper arithmetic (FP64, or
        the mixed form's FP32 lookup)."""
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        out = np.zeros_like(pos)
        st = np.zeros(len(pos), np.int32)
        _check(lib().ck_field_lookup_precision(self._h, int(precision), len(pos),
                                               abi.ptr(pos, C.c_double), abi.ptr(out, C.c_double),
                                               abi.ptr(st, C.c_int32)))
        return out, st


def track_result(res, t):
    """FitResult of track t of a Results."""
    st = int(res.status[t])
    if st != 0:
        return FitResult(status=st)
    ns = int(res.n_states[t])
    get = lambda name: None if getattr(res, name) is None else res.view(name)[t, :ns]
    pr, prc, fi, fic, sm, smc, jac = (get(x) for x in ("predicted", "predicted_cov", "filtered",
                                                        "filtered_cov", "smoothed", "smoothed_cov",
                                                        "jacobian"))
    states = []
    for k in range(ns):
        m6 = lambda a: None if a is None else a[k].reshape(6, 6).copy()
        v6 = lambda a: None if a is None else a[k].copy()
        states.append(TrackState(int(res.view("state_surface")[t, k]),
                                 int(res.view("state_flags")[t, k]),
                                 float(res.view("state_path_length")[t, k]),
                                 float(res.view("state_chi2")[t, k]), v6(pr), m6(prc), v6(fi),
                                 m6(fic), v6(sm), m6(smc), m6(jac)))
    return FitResult(status=0, states=states, n_measurements=int(res.n_measurements[t]),
                     n_holes=int(res.n_holes[t]), n_outliers=int(res.n_outliers[t]),
                     chi2=float(res.chi2_sum[t]), ndf=int(res.ndf[t]))
