"""Edge cases of the batch fit on the GPU against the oracle: an empty batch,
and one ragged batch mixing tracks the reference treats specially — no
measurement (NoMeasurementFound), no surfaces at all, a measurement on a
surface outside the sequence, two source links on one surface (the first in
input order wins), a single measurement, an invalid surface id
(InvalidInput), more states than the output holds (TooManyStates), a
one-state output capacity — with ordinary tracks between them. Statuses,
counts and flags bit-exact; parameters and covariances within 1e-9."""
import numpy as np
import pytest

from acts_gb300 import abi
from acts_gb300.generate import Batch
from acts_gb300.results import Results
from conftest import batch, detector
from oracle import kforacle
from parity import assert_parity, compare

RTOL = 1e-9


def _ragged(b, tracks):
    """A batch whose track i is built by tracks[i](b) -> (source track,
    sequence surfaces, list of (surface, values, cov) source links)."""
    n = len(tracks)
    out = Batch(n, 32)
    seq, ms, mv, mc = [], [], [], []
    so, mo = [0], [0]
    for i, make in enumerate(tracks):
        src, s, links = make(b)
        seq.extend(s)
        so.append(len(seq))
        for sid, val, cov in links:
            ms.append(sid)
            mv.extend(val)
            mc.extend(cov)
        mo.append(len(ms))
        for name, k in (("start_params", 6), ("start_cov", 36), ("start_frames", 12),
                        ("particle", 2), ("truth_start", 6)):
            getattr(out, name)[k * i:k * (i + 1)] = getattr(b, name)[k * src:k * (src + 1)]
        out.particle_pdg[i] = b.particle_pdg[src]
    out.seq_offsets = np.array(so, np.int32)
    out.seq_surfaces = np.array(seq, np.int32)
    out.meas_offsets = np.array(mo, np.int32)
    out.meas_surfaces = np.array(ms, np.int32)
    out.meas_values = np.array(mv, np.float64)
    out.meas_cov = np.array(mc, np.float64)
    out.truth_meas = np.zeros(6 * len(ms))
    out.meas_outlier = np.zeros(len(ms), np.uint8)
    return out


def _track(t, seq_edit=None, link_edit=None):
    def make(b):
        s = list(b.seq_surfaces[b.seq_offsets[t]:b.seq_offsets[t + 1]])
        links = [(int(b.meas_surfaces[m]), list(b.meas_values[2 * m:2 * m + 2]),
                  list(b.meas_cov[4 * m:4 * m + 4]))
                 for m in range(b.meas_offsets[t], b.meas_offsets[t + 1])]
        if seq_edit:
            s = seq_edit(s)
        if link_edit:
            links = link_edit(links)
        return t, s, links
    return make


def _shift(links, d):
    return [(s, [v[0] + d, v[1]], c) for s, v, c in links]


CASES = [
    _track(0),
    _track(1, link_edit=lambda L: []),                                   # no measurement
    _track(2, seq_edit=lambda s: [], link_edit=lambda L: []),            # no surfaces at all
    _track(3),
    _track(4, link_edit=lambda L: L + [(L[0][0] + 0, L[0][1], L[0][2])][:0] +
           [(L[2][0], [L[2][1][0] + 0.5, L[2][1][1]], L[2][2])]),        # 2nd link on surface 2
    _track(5, link_edit=lambda L: L[:1]),                                # one measurement
    _track(6, seq_edit=lambda s: s[:3] + [-1] + s[3:]),                 # invalid surface id
    _track(7, link_edit=lambda L: [L[0]] + _shift(L[1:], 0.0)),
    _track(8, seq_edit=lambda s: s[:5]),                                 # links beyond the sequence
    _track(9, link_edit=lambda L: L[::-1]),                              # links in reverse order
    _track(10),
]


@pytest.mark.gpu
def test_empty_batch(fitter_factory):
    fit = fitter_factory(abi.CKG_BARREL)
    b = batch(abi.CKG_BARREL, 5).subset(np.arange(0))
    for prec in (abi.PRECISION_FP64, abi.PRECISION_MIXED):
        r = fit.fit_batch(b, abi.default_options(precision=prec), max_states=10)
        assert r.status.size == 0


@pytest.mark.gpu
@pytest.mark.parametrize("max_states", [24, 6, 1])
@pytest.mark.parametrize("reverse", [0, 1], ids=["smoother", "reverse_filtering"])
def test_ragged_edge_case_batch(fitter_factory, max_states, reverse):
    """max_states 6 and 1: the longer tracks end in TooManyStates, as the
    oracle's (and the reference's) state container would overflow. With
    reverse filtering the reversed pass meets the same special tracks (one
    measurement: its first and last measurement state are one; links beyond
    the sequence: neither pass completes)."""
    det = detector(abi.CKG_BARREL)
    src = batch(abi.CKG_BARREL, 16)
    b = _ragged(src, CASES)
    opt = abi.default_options(reverse_filtering=reverse)
    ora = Results(b.n, max_states)
    kforacle.fit_batch(det, b, opt, ora, n_threads=1)
    gpu = fitter_factory(abi.CKG_BARREL).fit_batch(b, opt, max_states=max_states)
    expect = {1: 3, 2: 3, 6: 12}
    for t, st in expect.items():
        assert ora.status[t] == st, (t, ora.status[t])
    if max_states == 24:
        assert (ora.status[[0, 3, 4, 5, 7, 8, 9, 10]] == 0).all()
    else:
        assert (ora.status == 10).any()
    rep = compare(gpu, ora, RTOL)
    assert_parity(rep, RTOL)
    ok = ora.status == 0
    # the duplicate link: the first one (input order) is the state's measurement
    # (slots past a track's n_states are not written: compare its states)
    if max_states == 24 and ok[4]:
        k = ora.n_states[4]
        assert gpu.n_states[4] == k
        np.testing.assert_array_equal(gpu.view("state_surface")[4][:k],
                                      ora.view("state_surface")[4][:k])
