"""ctypes mirror of the C ABI structs in include/cudakalman.h and include/ckgen.h.

The layouts here must match the C headers field for field; tests/test_abi.py
checks the sizes against the compiled library (ck_abi_struct_sizes).
"""
import ctypes as C

import numpy as np

# ---------------------------------------------------------------- constants
CK_OK = 0
CK_ERR_INVALID_ARGUMENT = 1
CK_ERR_CUDA = 2
CK_ERR_NO_DEVICE = 3
CK_ERR_OUT_OF_MEMORY = 4
CK_ERR_UNSUPPORTED = 5
CK_ERR_BUDGET = 6
CK_ERR_TIMEOUT = 7
CK_ERR_NOT_READY = 8
CK_ERR_SCRATCH_LIMIT = 9

TRACK_STATUS = {
    0: "OK",
    1: "UpdateFailed",
    2: "SmoothFailed",
    3: "NoMeasurementFound",
    4: "StepCountLimitReached",
    5: "NextTargetLimitReached",
    6: "StepSizeStalled",
    7: "StepSizeAdjustmentFailed",
    8: "GlobalPositionNotOnSurface",
    9: "MagneticFieldOutOfBounds",
    10: "TooManyStates",
    11: "NotProcessed",
    12: "InvalidInput",
    13: "CompatibleTrackStateNotFound",
    14: "ReferenceSurfaceUnreachable",
    15: "InconsistentTrackStates",
}

TRACK_OK = 0
TRACK_UPDATE_FAILED = 1
TRACK_STEP_COUNT_LIMIT = 4
TRACK_NOT_ON_SURFACE = 8
TRACK_FIELD_OUT_OF_BOUNDS = 9
TRACK_TOO_MANY_STATES = 10
TRACK_INVALID_INPUT = 12
TRACK_INCONSISTENT_STATES = 15

FLAG_HAS_MEASUREMENT = 1 << 0
FLAG_HAS_PARAMETERS = 1 << 1
FLAG_IS_OUTLIER = 1 << 2
FLAG_IS_HOLE = 1 << 3
FLAG_HAS_MATERIAL = 1 << 4

SURFACE_PLANE = 0
SURFACE_CYLINDER = 1
SURFACE_LINE = 2
SURF_SENSITIVE = 1
SURF_MATERIAL = 2

FIELD_CONSTANT = 0
FIELD_GRID_XYZ = 1

PRECISION_FP64 = 0
PRECISION_MIXED = 1
SMOOTHER_GAIN_MATRIX = 0
SMOOTHER_MBF = 1
MEAS_LOC0 = 1
MEAS_LOC1 = 2
MEAS_LOC01 = 3
NUM_PRECISIONS = 2

MEM_HOST = 0
MEM_DEVICE = 1

OUT_PREDICTED = 1 << 0
OUT_FILTERED = 1 << 1
OUT_SMOOTHED = 1 << 2
OUT_JACOBIAN = 1 << 3
OUT_REFERENCE = 1 << 4
OUT_PACKED_COV = 1 << 5
EXTRAPOLATE_FIRST = 0
EXTRAPOLATE_LAST = 1
EXTRAPOLATE_FIRST_OR_LAST = 2
OUT_ALL = OUT_PREDICTED | OUT_FILTERED | OUT_SMOOTHED | OUT_JACOBIAN

CKG_TELESCOPE = 1
CKG_BARREL = 2
CKG_BARREL_MIXED = 3
CKG_UNEVEN = 4
CKG_SERVING = 5
CKG_STRIPS = 6

P_i32 = C.POINTER(C.c_int32)
P_u32 = C.POINTER(C.c_uint32)
P_f64 = C.POINTER(C.c_double)
P_f32 = C.POINTER(C.c_float)
P_u8 = C.POINTER(C.c_uint8)


class ck_surface(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("flags", C.c_int32),
        ("rotation", C.c_double * 9),
        ("center", C.c_double * 3),
        ("radius", C.c_double),
        ("half_length_z", C.c_double),
        ("half_x", C.c_double),
        ("half_y", C.c_double),
        ("mat_thickness", C.c_float),
        ("mat_x0", C.c_float),
        ("mat_l0", C.c_float),
        ("mat_ar", C.c_float),
        ("mat_z", C.c_float),
        ("mat_molar_rho", C.c_float),
        ("mat_molar_electron_rho", C.c_float),
        ("mat_mean_excitation", C.c_float),
        ("split_factor", C.c_float),
        ("reserved", C.c_float),
    ]


class ck_field(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("n", C.c_int32 * 3),
        ("constant_tesla", C.c_double * 3),
        ("min", C.c_double * 3),
        ("max", C.c_double * 3),
        ("values_tesla", P_f32),
    ]


class ck_options(C.Structure):
    _fields_ = [
        ("step_tolerance", C.c_double),
        ("step_size_cutoff", C.c_double),
        ("initial_step_size", C.c_double),
        ("max_step_size", C.c_double),
        ("max_rk_step_trials", C.c_uint32),
        ("max_steps", C.c_uint32),
        ("max_target_skipping", C.c_uint32),
        ("loop_protection", C.c_int32),
        ("path_limit", C.c_double),
        ("loop_fraction", C.c_double),
        ("surface_tolerance", C.c_double),
        ("near_limit", C.c_double),
        ("multiple_scattering", C.c_int32),
        ("energy_loss", C.c_int32),
        ("use_joseph", C.c_int32),
        ("precision", C.c_int32),
        ("outlier_chi2_cut", C.c_double),
        ("reverse_filtering", C.c_int32),
        ("free_to_bound_correction", C.c_int32),
        ("reference_surface", C.c_int32),
        ("early_termination", C.c_int32),
        ("smoother", C.c_int32),
        ("reference_strategy", C.c_int32),
        ("reverse_filtering_cov_scaling", C.c_double),
        ("reverse_filtering_mom_threshold", C.c_double),
    ]


class ck_config(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("n_surfaces", C.c_int32),
        ("surfaces", C.POINTER(ck_surface)),
        ("field", ck_field),
        ("threads_per_block", C.c_int32),
        ("blocks_per_sm", C.c_int32),
        ("use_graph", C.c_int32),
        ("reserved", C.c_int32),
        ("autotune_cache", C.c_char_p),
    ]


class ck_batch_in(C.Structure):
    _fields_ = [
        ("n_tracks", C.c_int32),
        ("memory", C.c_int32),
        ("seq_offsets", P_i32),
        ("seq_surfaces", P_i32),
        ("meas_offsets", P_i32),
        ("meas_surfaces", P_i32),
        ("meas_values", P_f64),
        ("meas_cov", P_f64),
        ("start_params", P_f64),
        ("start_cov", P_f64),
        ("start_frames", P_f64),
        ("particle", P_f32),
        ("particle_pdg", P_i32),
        ("meas_subspace", P_i32),
    ]


class ck_batch_out(C.Structure):
    _fields_ = [
        ("max_states", C.c_int32),
        ("components", C.c_uint32),
        ("memory", C.c_int32),
        ("reserved", C.c_int32),
        ("status", P_i32),
        ("n_states", P_i32),
        ("n_measurements", P_i32),
        ("n_holes", P_i32),
        ("n_outliers", P_i32),
        ("ndf", P_i32),
        ("chi2_sum", P_f64),
        ("state_surface", P_i32),
        ("state_flags", P_u32),
        ("state_path_length", P_f64),
        ("state_chi2", P_f64),
        ("predicted", P_f64),
        ("predicted_cov", P_f64),
        ("filtered", P_f64),
        ("filtered_cov", P_f64),
        ("smoothed", P_f64),
        ("smoothed_cov", P_f64),
        ("jacobian", P_f64),
        ("track_params", P_f64),
        ("track_cov", P_f64),
    ]


class ck_propagate_in(C.Structure):
    _fields_ = [
        ("n", C.c_int32),
        ("memory", C.c_int32),
        ("start_params", P_f64),
        ("start_cov", P_f64),
        ("start_frames", P_f64),
        ("particle", P_f32),
        ("target", P_i32),
        ("path_limit", P_f64),
    ]


class ck_propagate_out(C.Structure):
    _fields_ = [
        ("status", P_i32),
        ("end_params", P_f64),
        ("end_cov", P_f64),
        ("jacobian", P_f64),
        ("end_frames", P_f64),
        ("path_length", P_f64),
        ("steps", P_i32),
    ]


class Propagation:
    """Host arrays of a batch of propagations (ck_propagate's layout): the
    inputs per track, the outputs [c, n] (structure of arrays)."""

    def __init__(self, start_params, start_frames, particle, path_limit, start_cov=None,
                 target=None):
        f64 = lambda x: np.ascontiguousarray(x, np.float64)
        self.start_params = f64(start_params).reshape(-1, 6)
        self.n = len(self.start_params)
        self.start_frames = f64(start_frames).reshape(self.n, 12)
        self.particle = np.ascontiguousarray(particle, np.float32).reshape(self.n, 2)
        self.path_limit = f64(path_limit).reshape(self.n)
        self.start_cov = None if start_cov is None else f64(start_cov).reshape(self.n, 36)
        self.target = None if target is None else np.ascontiguousarray(target, np.int32)
        n = self.n
        self.status = np.full(n, 11, np.int32)
        self.end_params = np.zeros((6, n))
        self.end_cov = np.zeros((36, n))
        self.jacobian = np.zeros((36, n))
        self.end_frames = np.zeros((n, 12))
        self.path_length = np.zeros(n)
        self.steps = np.zeros(n, np.int32)

    def as_in(self):
        i = ck_propagate_in()
        i.n = self.n
        i.memory = MEM_HOST
        i.start_params = ptr(self.start_params, C.c_double)
        i.start_cov = ptr(self.start_cov, C.c_double)
        i.start_frames = ptr(self.start_frames, C.c_double)
        i.particle = ptr(self.particle, C.c_float)
        i.target = ptr(self.target, C.c_int32)
        i.path_limit = ptr(self.path_limit, C.c_double)
        return i

    def as_out(self):
        o = ck_propagate_out()
        o.status = ptr(self.status, C.c_int32)
        for name in ("end_params", "end_cov", "jacobian", "end_frames", "path_length"):
            setattr(o, name, ptr(getattr(self, name), C.c_double))
        o.steps = ptr(self.steps, C.c_int32)
        return o


class ck_ckf_options(C.Structure):
    _fields_ = [
        ("chi2_cut", C.c_double),
        ("chi2_cut_outlier", C.c_double),
        ("max_candidates", C.c_int32),
        ("min_measurements", C.c_int32),
        ("max_holes", C.c_int32),
        ("max_outliers", C.c_int32),
        ("max_holes_and_outliers", C.c_int32),
        ("target_surface", C.c_int32),
        ("max_states", C.c_int32),
        ("max_tracks", C.c_int32),
        ("max_branches", C.c_int32),
        ("end_of_world", C.c_int32),
        ("lanes_per_seed", C.c_int32),
        ("reserved", C.c_int32),
    ]


INT32_MAX = 2147483647


def ckf_options(**kw):
    """ck_ckf_options with ck_ckf_options_default's values, then `kw`."""
    o = ck_ckf_options()
    o.chi2_cut = 15.0
    o.chi2_cut_outlier = float("inf")
    o.max_candidates = 1
    o.min_measurements = 0
    o.max_holes = INT32_MAX
    o.max_outliers = INT32_MAX
    o.max_holes_and_outliers = INT32_MAX
    o.target_surface = -1
    o.max_states = 64
    o.max_tracks = 16
    o.max_branches = 16
    for k, v in kw.items():
        if not hasattr(o, k):
            raise AttributeError(k)
        setattr(o, k, v)
    return o


class ck_ckf_in(C.Structure):
    _fields_ = [
        ("n_seeds", C.c_int32),
        ("memory", C.c_int32),
        ("seq_offsets", P_i32),
        ("seq_surfaces", P_i32),
        ("start_params", P_f64),
        ("start_cov", P_f64),
        ("start_frames", P_f64),
        ("particle", P_f32),
        ("particle_pdg", P_i32),
        ("n_meas", C.c_int32),
        ("n_surfaces", C.c_int32),
        ("surf_meas_offsets", P_i32),
        ("meas_values", P_f64),
        ("meas_cov", P_f64),
        ("meas_subspace", P_i32),
        ("n_events", C.c_int32),
        ("seed_event", P_i32),
    ]


CKF_OUT_INT = ("status", "n_tracks", "n_states")
CKF_TRACK_FIELDS = (("track_tip", np.int32, 1), ("track_n_measurements", np.int32, 1),
                    ("track_n_holes", np.int32, 1), ("track_n_outliers", np.int32, 1),
                    ("track_ndf", np.int32, 1), ("track_chi2", np.float64, 1),
                    ("track_params", np.float64, 6), ("track_cov", np.float64, 21))
CKF_STATE_FIELDS = (("state_prev", np.int32, 1), ("state_surface", np.int32, 1),
                    ("state_flags", np.uint32, 1), ("state_measurement", np.int32, 1),
                    ("state_chi2", np.float64, 1), ("state_path_length", np.float64, 1),
                    ("predicted", np.float64, 6), ("predicted_cov", np.float64, 21),
                    ("filtered", np.float64, 6), ("filtered_cov", np.float64, 21),
                    ("jacobian", np.float64, 36))
_CTYPE = {np.int32: C.c_int32, np.uint32: C.c_uint32, np.float64: C.c_double}


class ck_ckf_out(C.Structure):
    _fields_ = ([(name, P_i32) for name in CKF_OUT_INT] +
                [(name, C.POINTER(_CTYPE[t])) for name, t, _ in CKF_TRACK_FIELDS] +
                [(name, C.POINTER(_CTYPE[t])) for name, t, _ in CKF_STATE_FIELDS])


class TrackFinding:
    """Host arrays of one track-finding call (ck_find_tracks's layout): the
    seeds with their surface sequences, the event's measurements grouped by
    surface, and the found tracks and track states per seed."""

    def __init__(self, seq_offsets, seq_surfaces, start_params, start_cov, start_frames,
                 particle, surf_meas_offsets, meas_values, meas_cov, meas_subspace=None,
                 particle_pdg=None, max_states=64, max_tracks=16, n_events=1,
                 seed_event=None):
        i32 = lambda x: np.ascontiguousarray(x, np.int32)
        f64 = lambda x: np.ascontiguousarray(x, np.float64)
        self.seq_offsets = i32(seq_offsets)
        self.n = len(self.seq_offsets) - 1
        self.seq_surfaces = i32(seq_surfaces)
        self.start_params = f64(start_params).reshape(self.n, 6)
        self.start_cov = f64(start_cov).reshape(self.n, 36)
        self.start_frames = f64(start_frames).reshape(self.n, 12)
        self.particle = np.ascontiguousarray(particle, np.float32).reshape(self.n, 2)
        self.particle_pdg = None if particle_pdg is None else i32(particle_pdg)
        self.surf_meas_offsets = i32(surf_meas_offsets)
        self.n_events = int(n_events)
        self.seed_event = None if seed_event is None else i32(seed_event)
        self.n_surfaces = (len(self.surf_meas_offsets) - 1) // max(self.n_events, 1)
        self.meas_values = f64(meas_values).reshape(-1, 2)
        self.n_meas = len(self.meas_values)
        self.meas_cov = f64(meas_cov).reshape(self.n_meas, 4)
        self.meas_subspace = None if meas_subspace is None else i32(meas_subspace)
        self.max_states = max_states
        self.max_tracks = max_tracks
        n = self.n
        for name in CKF_OUT_INT:
            setattr(self, name, np.zeros(n, np.int32))
        self.status[:] = 11
        for name, t, c in CKF_TRACK_FIELDS:
            setattr(self, name, np.zeros((n, max_tracks) + ((c,) if c > 1 else ()), t))
        for name, t, c in CKF_STATE_FIELDS:
            setattr(self, name, np.zeros((n, max_states) + ((c,) if c > 1 else ()), t))

    def options(self, **kw):
        """ck_ckf_options with this container's capacities."""
        kw.setdefault("max_states", self.max_states)
        kw.setdefault("max_tracks", self.max_tracks)
        if kw["max_states"] > self.max_states or kw["max_tracks"] > self.max_tracks:
            raise ValueError("capacities above the container's")
        return ckf_options(**kw)

    def as_in(self):
        i = ck_ckf_in()
        i.n_seeds = self.n
        i.memory = MEM_HOST
        i.seq_offsets = ptr(self.seq_offsets, C.c_int32)
        i.seq_surfaces = ptr(self.seq_surfaces, C.c_int32)
        i.start_params = ptr(self.start_params, C.c_double)
        i.start_cov = ptr(self.start_cov, C.c_double)
        i.start_frames = ptr(self.start_frames, C.c_double)
        i.particle = ptr(self.particle, C.c_float)
        i.particle_pdg = ptr(self.particle_pdg, C.c_int32)
        i.n_meas = self.n_meas
        i.n_surfaces = self.n_surfaces
        i.surf_meas_offsets = ptr(self.surf_meas_offsets, C.c_int32)
        i.meas_values = ptr(self.meas_values, C.c_double)
        i.meas_cov = ptr(self.meas_cov, C.c_double)
        i.meas_subspace = ptr(self.meas_subspace, C.c_int32)
        i.n_events = self.n_events
        i.seed_event = ptr(self.seed_event, C.c_int32)
        return i

    def as_out(self):
        o = ck_ckf_out()
        for name in CKF_OUT_INT:
            setattr(o, name, ptr(getattr(self, name), C.c_int32))
        for name, t, _ in CKF_TRACK_FIELDS + CKF_STATE_FIELDS:
            setattr(o, name, ptr(getattr(self, name), _CTYPE[t]))
        return o

    def track_states(self, s, k):
        """State indices of found track k of seed s, first to last."""
        out = []
        i = int(self.track_tip[s, k])
        while i >= 0:
            out.append(i)
            i = int(self.state_prev[s, i])
        return out[::-1]

    def track_measurements(self, s, k):
        """Measurement indices of the measurement states (outliers included)
        of found track k of seed s, first to last."""
        return [int(self.state_measurement[s, i]) for i in self.track_states(s, k)
                if self.state_flags[s, i] & FLAG_HAS_MEASUREMENT]


class ck_server_config(C.Structure):
    _fields_ = [
        ("memory_budget_bytes", C.c_int64),
        ("n_streams", C.c_int32),
        ("max_states", C.c_int32),
        ("max_batch_tracks", C.c_int32),
        ("components", C.c_uint32),
        ("grid_blocks", C.c_int32),
        ("steps_per_round", C.c_int32),
    ]


class ckg_out(C.Structure):
    _fields_ = [
        ("max_per_track", C.c_int32),
        ("seq_offsets", P_i32),
        ("seq_surfaces", P_i32),
        ("meas_offsets", P_i32),
        ("meas_surfaces", P_i32),
        ("meas_values", P_f64),
        ("meas_cov", P_f64),
        ("start_params", P_f64),
        ("start_cov", P_f64),
        ("start_frames", P_f64),
        ("particle", P_f32),
        ("particle_pdg", P_i32),
        ("truth_meas", P_f64),
        ("meas_outlier", P_u8),
        ("truth_start", P_f64),
        ("meas_subspace", P_i32),
    ]


def ptr(a, ctype):
    """ctypes pointer to a contiguous numpy array (None stays NULL)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data_as(C.POINTER(ctype))


def default_options(**kw):
    """Reference defaults (StepperPlainOptions, PropagatorPlainOptions,
    DirectNavigator::Options, KalmanFitterOptions), see ck_options_default."""
    o = ck_options()
    o.step_tolerance = 1e-4
    o.step_size_cutoff = 0.0
    o.initial_step_size = 10000.0
    o.max_step_size = np.finfo(np.float64).max
    o.max_rk_step_trials = 10000
    o.max_steps = 1000
    o.max_target_skipping = 100
    o.loop_protection = 1
    o.path_limit = np.finfo(np.float64).max
    o.loop_fraction = 0.5
    o.surface_tolerance = 1e-4
    o.near_limit = -0.1
    o.multiple_scattering = 1
    o.energy_loss = 1
    o.use_joseph = 0
    o.precision = PRECISION_FP64
    o.outlier_chi2_cut = float("inf")
    o.reverse_filtering = 0
    o.free_to_bound_correction = 0
    o.reference_surface = -1
    o.early_termination = 0
    o.smoother = SMOOTHER_GAIN_MATRIX
    o.reference_strategy = EXTRAPOLATE_FIRST_OR_LAST
    o.reverse_filtering_cov_scaling = 100.0
    o.reverse_filtering_mom_threshold = 0.0
    for k, v in kw.items():
        setattr(o, k, v)
    return o
