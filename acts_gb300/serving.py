"""Python binding of the continuous-batching serving loop (ck_server_*).

    srv = FitServer(fitter, options, memory_budget_bytes=40 << 30, n_streams=4)
    srv.submit(event_id, batch)          # returns at once
    eid, results, latency_ms = srv.poll(timeout_ms=100)

Events are admitted against the device-memory budget as stream slots free
up, co-batched with whatever else is pending, and fitted concurrently on the
slots' streams; see acts_gb300/csrc/ck_server.cu.
"""
import ctypes as C

from . import abi
from .fitter import CudaKalmanError, _check, lib
from .results import Results


def _bind():
    L = lib()
    if getattr(L, "_server_bound", False):
        return L
    P = C.POINTER
    L.ck_server_create.argtypes = [C.c_void_p, P(abi.ck_options), P(abi.ck_server_config),
                                   P(C.c_void_p)]
    L.ck_server_submit.argtypes = [C.c_void_p, C.c_int64, P(abi.ck_batch_in)]
    L.ck_server_poll.argtypes = [C.c_void_p, P(C.c_int64), P(abi.ck_batch_out), C.c_int32,
                                 P(C.c_double), C.c_int32]
    L.ck_server_stats.argtypes = [C.c_void_p] + [P(C.c_int64)] * 4
    L.ck_server_capacity.argtypes = [C.c_void_p]
    L.ck_server_capacity.restype = C.c_int32
    L.ck_server_destroy.argtypes = [C.c_void_p]
    L._server_bound = True
    return L


class FitServer:
    def __init__(self, fitter, options, memory_budget_bytes=40 << 30, n_streams=4, max_states=24,
                 max_batch_tracks=200000, components=abi.OUT_SMOOTHED):
        L = _bind()
        cfg = abi.ck_server_config()
        cfg.memory_budget_bytes = int(memory_budget_bytes)
        cfg.n_streams = n_streams
        cfg.max_states = max_states
        cfg.max_batch_tracks = max_batch_tracks
        cfg.components = components
        self.max_states = max_states
        self.components = components
        self._opt = options
        s = C.c_void_p()
        _check(L.ck_server_create(fitter.handle, C.byref(options), C.byref(cfg), C.byref(s)))
        self._s = s
        self._sizes = {}
        self._fitter = fitter

    @property
    def capacity(self):
        return _bind().ck_server_capacity(self._s)

    def submit(self, event_id, batch):
        bi = batch.as_batch_in()
        _check(_bind().ck_server_submit(self._s, int(event_id), C.byref(bi)))
        self._sizes[int(event_id)] = batch.n

    def poll(self, timeout_ms=100):
        """(event_id, Results, latency_ms) of one finished event, or None."""
        L = _bind()
        if not self._sizes:
            return None
        cap = max(self._sizes.values())
        res = Results(cap, self.max_states, self.components)
        eid = C.c_int64()
        lat = C.c_double()
        st = L.ck_server_poll(self._s, C.byref(eid), C.byref(res.as_batch_out()), cap, C.byref(lat),
                              int(timeout_ms))
        if st == abi.CK_ERR_NOT_READY:
            return None
        _check(st)
        n = self._sizes.pop(eid.value)
        return eid.value, _shrink(res, n), lat.value

    def stats(self):
        a, b, c, d = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        _check(_bind().ck_server_stats(self._s, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return {"submitted": a.value, "completed": b.value, "tracks": c.value,
                "bytes_in_use": d.value}

    def close(self):
        if getattr(self, "_s", None):
            _bind().ck_server_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _shrink(res, n):
    """A Results for the first n tracks of a (larger) Results laid out for n."""
    out = Results(n, res.max_states, res.components)
    for name in ("status", "n_states", "n_measurements", "n_holes", "n_outliers", "ndf", "chi2_sum"):
        getattr(out, name)[:] = getattr(res, name)[:n]
    ms = res.max_states
    for name in ("state_surface", "state_flags", "state_path_length", "state_chi2", "predicted",
                 "predicted_cov", "filtered", "filtered_cov", "smoothed", "smoothed_cov",
                 "jacobian"):
        a = getattr(res, name)
        if a is None:
            continue
        c = a.size // (ms * res.n)
        # the server wrote the event's SoA with n innermost at the front
        getattr(out, name)[:] = a[: ms * c * n]
    return out
