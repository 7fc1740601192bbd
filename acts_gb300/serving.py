"""Python binding of the continuous-batching serving loop (ck_server_*).

    srv = FitServer(fitter, options, memory_budget_bytes=40 << 30, n_streams=4)
    srv.submit(event_id, batch)          # returns at once, copies nothing
    eid, results, latency_ms = srv.poll(timeout_ms=100)

Events are admitted against the device-memory budget as stream slots free
up, co-batched with whatever else is pending, and fitted concurrently on the
slots' streams; each event's results are copied straight into its result
buffers (host Results by default; page-locked or device buffers avoid the
staging copy). See acts_gb300/csrc/ck_server.cu.
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
    L.ck_server_submit.argtypes = [C.c_void_p, C.c_int64, P(abi.ck_batch_in),
                                   P(abi.ck_batch_out)]
    L.ck_server_poll.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_double), C.c_int32]
    L.ck_server_stats.argtypes = [C.c_void_p] + [P(C.c_int64)] * 4
    L.ck_server_capacity.argtypes = [C.c_void_p]
    L.ck_server_capacity.restype = C.c_int32
    L.ck_server_destroy.argtypes = [C.c_void_p]
    L._server_bound = True
    return L


class FitServer:
    def __init__(self, fitter, options, memory_budget_bytes=40 << 30, n_streams=4, max_states=24,
                 max_batch_tracks=200000, components=abi.OUT_SMOOTHED, grid_blocks=0,
                 steps_per_round=0):
        L = _bind()
        cfg = abi.ck_server_config()
        cfg.memory_budget_bytes = int(memory_budget_bytes)
        cfg.n_streams = n_streams
        cfg.max_states = max_states
        cfg.max_batch_tracks = max_batch_tracks
        cfg.components = components
        cfg.grid_blocks = int(grid_blocks)
        cfg.steps_per_round = int(steps_per_round)
        self.max_states = max_states
        self.components = components
        self._opt = options
        s = C.c_void_p()
        _check(L.ck_server_create(fitter.handle, C.byref(options), C.byref(cfg), C.byref(s)))
        self._s = s
        self._inflight = {}
        self._fitter = fitter

    @property
    def capacity(self):
        return _bind().ck_server_capacity(self._s)

    def submit(self, event_id, batch, results=None):
        """Queues `batch` (anything with as_batch_in()); its results go to
        `results` (anything with as_batch_out(): host Results by default, or
        page-locked / device buffers). Both are kept alive until polled."""
        if results is None:
            results = Results(batch.n, self.max_states, self.components)
        bi = batch.as_batch_in()
        bo = results.as_batch_out()
        # registered before the submission: the event can finish, and another
        # thread poll it, before ck_server_submit has returned to this one
        key = int(event_id)
        self._inflight[key] = (batch, results, bi, bo)
        try:
            _check(_bind().ck_server_submit(self._s, key, C.byref(bi), C.byref(bo)))
        except Exception:
            self._inflight.pop(key, None)
            raise

    def poll(self, timeout_ms=100):
        """(event_id, results, latency_ms) of one finished event, or None."""
        L = _bind()
        eid = C.c_int64()
        lat = C.c_double()
        st = L.ck_server_poll(self._s, C.byref(eid), C.byref(lat), int(timeout_ms))
        if st == abi.CK_ERR_NOT_READY:
            return None
        entry = self._inflight.pop(eid.value, None)
        _check(st)
        return eid.value, entry[1] if entry is not None else None, lat.value

    def stats(self):
        a, b, c, d = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        _check(_bind().ck_server_stats(self._s, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return {"submitted": a.value, "completed": b.value, "tracks": c.value,
                "bytes_in_use": d.value}

    def close(self):
        if getattr(self, "_s", None):
            _bind().ck_server_destroy(self._s)
            self._s = None
        self._inflight.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
