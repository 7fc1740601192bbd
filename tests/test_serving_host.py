"""Host logic of the Python serving binding (no GPU): an event can finish and
be polled by another thread before ck_server_submit has returned to the
submitting one, so FitServer must know the event before it submits it. The
fake library below polls from inside its submit call, which is that
interleaving made deterministic."""
import ctypes as C

from acts_gb300 import abi, serving


class _Stub:
    def __init__(self, tag):
        self.tag = tag
        self.n = 1

    def as_batch_in(self):
        return abi.ck_batch_in()

    def as_batch_out(self):
        return abi.ck_batch_out()


class _FakeLib:
    """ck_server_submit finishes the event at once and lets the poller take
    it before returning; ck_server_poll hands out the finished event."""

    def __init__(self):
        self.done = []
        self.server = None
        self.polled_during_submit = []
        self.fail_submit = False

    def ck_server_submit(self, s, event_id, bi, bo):
        if self.fail_submit:
            return abi.CK_ERR_BUDGET
        self.done.append(event_id)
        self.polled_during_submit.append(self.server.poll(timeout_ms=0))
        return abi.CK_OK

    def ck_server_poll(self, s, eid_p, lat_p, timeout_ms):
        if not self.done:
            return abi.CK_ERR_NOT_READY
        eid_p._obj.value = self.done.pop(0)
        lat_p._obj.value = 2.5
        return abi.CK_OK


def _server(fake, monkeypatch):
    monkeypatch.setattr(serving, "_bind", lambda: fake)
    srv = serving.FitServer.__new__(serving.FitServer)
    srv._s = C.c_void_p(1)
    srv._inflight = {}
    srv.max_states = 4
    srv.components = abi.OUT_SMOOTHED
    fake.server = srv
    return srv


def test_event_polled_before_submit_returns(monkeypatch):
    fake = _FakeLib()
    srv = _server(fake, monkeypatch)
    try:
        results = _Stub("results")
        srv.submit(7, _Stub("batch"), results)
        eid, res, lat = fake.polled_during_submit[0]
        assert eid == 7 and res is results and lat == 2.5
        assert srv._inflight == {}
    finally:
        srv._s = None  # (no server behind the fake handle to destroy)


def test_failed_submission_forgets_the_event(monkeypatch):
    fake = _FakeLib()
    fake.fail_submit = True
    srv = _server(fake, monkeypatch)
    try:
        try:
            srv.submit(3, _Stub("batch"), _Stub("results"))
        except Exception:
            pass
        else:
            raise AssertionError("a refused submission must raise")
        assert srv._inflight == {}
    finally:
        srv._s = None
