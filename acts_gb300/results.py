"""Host-side result buffers in the ck_batch_out layout (include/cudakalman.h).

Per-state arrays are structure-of-arrays with the track index innermost:
element c of state k of track t is at [(k * C + c) * n + t]; the accessors
below reshape them to [n, max_states, C] views for analysis.
"""
import ctypes as C

import numpy as np

from . import abi


# index of full-matrix entry (i, j) in the packed upper triangle (row by row)
UNPACK = np.array([[(min(i, j) * (11 - min(i, j))) // 2 + max(i, j) for j in range(6)]
                   for i in range(6)]).reshape(36)


class Results:
    def __init__(self, n, max_states=24, components=abi.OUT_ALL):
        self.n = n
        self.max_states = max_states
        self.components = components
        z = lambda k, dt: np.zeros(max_states * k * n, dt)
        self.status = np.full(n, 11, np.int32)
        self.n_states = np.zeros(n, np.int32)
        self.n_measurements = np.zeros(n, np.int32)
        self.n_holes = np.zeros(n, np.int32)
        self.n_outliers = np.zeros(n, np.int32)
        self.ndf = np.zeros(n, np.int32)
        self.chi2_sum = np.zeros(n, np.float64)
        self.state_surface = z(1, np.int32)
        self.state_flags = z(1, np.uint32)
        self.state_path_length = z(1, np.float64)
        self.state_chi2 = z(1, np.float64)
        cc = 21 if components & abi.OUT_PACKED_COV else 36
        self.predicted = z(6, np.float64) if components & abi.OUT_PREDICTED else None
        self.predicted_cov = z(cc, np.float64) if components & abi.OUT_PREDICTED else None
        self.filtered = z(6, np.float64) if components & abi.OUT_FILTERED else None
        self.filtered_cov = z(cc, np.float64) if components & abi.OUT_FILTERED else None
        self.smoothed = z(6, np.float64) if components & abi.OUT_SMOOTHED else None
        self.smoothed_cov = z(cc, np.float64) if components & abi.OUT_SMOOTHED else None
        self.jacobian = z(36, np.float64) if components & abi.OUT_JACOBIAN else None
        ref = components & abi.OUT_REFERENCE
        self.track_params = np.zeros(6 * n, np.float64) if ref else None
        self.track_cov = np.zeros(36 * n, np.float64) if ref else None

    ARRAYS = ("status", "n_states", "n_measurements", "n_holes", "n_outliers", "ndf",
              "chi2_sum", "state_surface", "state_flags", "state_path_length", "state_chi2",
              "predicted", "predicted_cov", "filtered", "filtered_cov", "smoothed",
              "smoothed_cov", "jacobian", "track_params", "track_cov")

    def pinned(self):
        """Moves the buffers to page-locked host memory (torch pin_memory),
        which the fit writes in place from the device; returns self."""
        import torch

        self._pinned = []
        for name in self.ARRAYS:
            a = getattr(self, name)
            if a is None:
                continue
            t = torch.from_numpy(a).pin_memory()
            self._pinned.append(t)
            setattr(self, name, t.numpy())
        return self

    def as_batch_out(self):
        o = abi.ck_batch_out()
        o.max_states = self.max_states
        o.components = self.components
        o.memory = abi.MEM_HOST
        for name in ("status", "n_states", "n_measurements", "n_holes", "n_outliers", "ndf",
                     "state_surface"):
            setattr(o, name, abi.ptr(getattr(self, name), C.c_int32))
        o.state_flags = abi.ptr(self.state_flags, C.c_uint32)
        for name in ("chi2_sum", "state_path_length", "state_chi2", "predicted", "predicted_cov",
                     "filtered", "filtered_cov", "smoothed", "smoothed_cov", "jacobian",
                     "track_params", "track_cov"):
            setattr(o, name, abi.ptr(getattr(self, name), C.c_double))
        return o

    def as_batch_out_view(self, m):
        """A ck_batch_out for m <= n tracks over the start of these arrays
        (the SoA layout of m tracks: element c of state k of track t at
        [(k * C + c) * m + t]), for reusing one buffer across events."""
        o = self.as_batch_out()
        assert m <= self.n
        return o

    def track(self, name):
        """Per-track array `name` (track_params / track_cov) as [n, C]."""
        a = getattr(self, name)
        return None if a is None else a.reshape(-1, self.n).T

    def view(self, name, k=None):
        """Array `name` as [n, max_states, C] (or [n, max_states] for scalars);
        packed covariances (CK_OUT_PACKED_COV) are unfolded to C = 36."""
        a = getattr(self, name)
        if a is None:
            return None
        c = a.size // (self.max_states * self.n)
        v = a.reshape(self.max_states, c, self.n).transpose(2, 0, 1)
        if c == 21:
            return v[..., UNPACK]
        return v[..., 0] if c == 1 else v

    def track_states(self, t, name):
        """States 0..n_states-1 of track t for array `name`."""
        v = self.view(name)
        return v[t, : self.n_states[t]]


class TorchResults:
    """Result buffers as torch tensors in device memory (device="cuda:0") or
    page-locked host memory (device="pinned"), in the ck_batch_out layout;
    to_host() copies them into a Results."""

    _SPEC = (("status", 1, "int32"), ("n_states", 1, "int32"), ("n_measurements", 1, "int32"),
             ("n_holes", 1, "int32"), ("n_outliers", 1, "int32"), ("ndf", 1, "int32"),
             ("chi2_sum", 1, "float64"), ("state_surface", -1, "int32"),
             ("state_flags", -1, "int32"), ("state_path_length", -1, "float64"),
             ("state_chi2", -1, "float64"), ("predicted", -6, "float64"),
             ("predicted_cov", -36, "float64"), ("filtered", -6, "float64"),
             ("filtered_cov", -36, "float64"), ("smoothed", -6, "float64"),
             ("smoothed_cov", -36, "float64"), ("jacobian", -36, "float64"))
    _COMP = {"predicted": abi.OUT_PREDICTED, "predicted_cov": abi.OUT_PREDICTED,
             "filtered": abi.OUT_FILTERED, "filtered_cov": abi.OUT_FILTERED,
             "smoothed": abi.OUT_SMOOTHED, "smoothed_cov": abi.OUT_SMOOTHED,
             "jacobian": abi.OUT_JACOBIAN}

    def __init__(self, n, max_states=24, components=abi.OUT_SMOOTHED, device="cuda:0"):
        import torch

        self.n = n
        self.max_states = max_states
        self.components = components
        self.pinned = device == "pinned"
        self.tensors = {}
        for name, per, dt in self._SPEC:
            if name in self._COMP and not components & self._COMP[name]:
                continue
            if per == -36 and name != "jacobian" and components & abi.OUT_PACKED_COV:
                per = -21
            size = n * (per if per > 0 else -per * max_states)
            dtype = getattr(torch, dt)
            if self.pinned:
                t = torch.empty(size, dtype=dtype).pin_memory()
            else:
                t = torch.empty(size, dtype=dtype, device=device)
            self.tensors[name] = t

    def as_batch_out(self):
        o = abi.ck_batch_out()
        o.max_states = self.max_states
        o.components = self.components
        o.memory = abi.MEM_HOST if self.pinned else abi.MEM_DEVICE
        for name, t in self.tensors.items():
            ct = C.c_double if t.element_size() == 8 else (
                C.c_uint32 if name == "state_flags" else C.c_int32)
            setattr(o, name, C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ct)))
        return o

    def to_host(self):
        r = Results(self.n, self.max_states, self.components)
        for name, t in self.tensors.items():
            a = t.cpu().numpy()
            getattr(r, name)[:] = a.view(getattr(r, name).dtype)
        return r
