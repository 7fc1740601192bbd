"""Synthetic event generator: determinism, presets and detector response."""
import numpy as np

from acts_gb300 import abi, generate
from conftest import detector


def test_deterministic_and_split_invariant():
    det = detector(abi.CKG_BARREL)
    a = generate.generate(det, 200, seed=9, n_threads=1)
    b = generate.generate(det, 200, seed=9, n_threads=7)
    c1 = generate.generate(det, 120, seed=9)
    c2 = generate.generate(det, 80, seed=9, first_track=120)
    for name in ("seq_offsets", "seq_surfaces", "meas_values", "start_params", "start_cov"):
        np.testing.assert_array_equal(getattr(a, name), getattr(b, name))
    np.testing.assert_array_equal(a.meas_values[: c1.meas_values.size], c1.meas_values)
    np.testing.assert_array_equal(a.meas_values[c1.meas_values.size:], c2.meas_values)
    d = generate.generate(det, 200, seed=10)
    assert not np.array_equal(a.meas_values, d.meas_values)


def test_presets_geometry():
    assert detector(abi.CKG_TELESCOPE).n_surfaces == 10
    assert detector(abi.CKG_BARREL).n_surfaces == 10
    assert detector(abi.CKG_UNEVEN).n_surfaces == 20
    radii = [detector(abi.CKG_BARREL).surfaces[i].radius for i in range(10)]
    assert radii == [32, 72, 116, 172, 260, 360, 500, 660, 820, 1020]
    s = detector(abi.CKG_BARREL).surfaces[0]
    assert abs(s.mat_thickness / s.mat_x0 - 0.0032) < 1e-4  # 0.3 mm Si, x/X0 = 0.32 %


def test_telescope_tracks_hit_every_plane():
    b = generate.generate(detector(abi.CKG_TELESCOPE), 300, seed=2)
    assert (np.diff(b.seq_offsets) == 10).all()
    assert (np.diff(b.meas_offsets) == 10).all()
    # smearing width 50 um
    resid = b.meas_values.reshape(-1, 2) - b.truth_meas.reshape(-1, 6)[:, :2]
    assert abs(resid.std() - 0.05) < 0.005


def test_uneven_holes_outliers_and_lengths():
    b = generate.generate(detector(abi.CKG_UNEVEN), 3000, seed=2)
    nseq = np.diff(b.seq_offsets)
    nmeas = np.diff(b.meas_offsets)
    assert nseq.min() >= 1 and nseq.max() <= 20
    assert 0.07 < 1 - nmeas.sum() / nseq.sum() < 0.13  # hole probability 0.1
    assert 0.035 < b.meas_outlier.mean() < 0.065  # outlier probability 0.05
    assert len(np.unique(nseq)) > 10


def test_grid_field_properties():
    det = detector(abi.CKG_UNEVEN)
    f = det.field
    assert (f.n[0], f.n[1], f.n[2]) == (151, 151, 301)
    v = det.field_values.reshape(151, 151, 301, 3)
    assert abs(v[75, 75, 150, 2] - 2.0) < 1e-6  # 2 T at the centre
    assert abs(v[75, 75, 150, 0]) < 1e-9  # no radial field on the axis
    # Bz(r < 1.2 m, z) = 2 T (1 + (z / 2.5 m)^2)^-1.5
    z = -3000 + 20 * 250
    assert abs(v[75, 75, 250, 2] - 2.0 * (1 + (z / 2500.0) ** 2) ** -1.5) < 1e-5
    # div B ~ 0 in the solenoid body (central differences, 20 mm pitch)
    i, j, k = 90, 80, 200
    h = 20.0
    div = ((v[i + 1, j, k, 0] - v[i - 1, j, k, 0]) + (v[i, j + 1, k, 1] - v[i, j - 1, k, 1]) +
           (v[i, j, k + 1, 2] - v[i, j, k - 1, 2])) / (2 * h)
    assert abs(div) < 1e-5


def test_event_sizes():
    s = generate.event_sizes(4, 200, mean=5000.0)
    assert abs(s.mean() - 5000) < 50 and s.std() > 30
    s = generate.event_sizes(4, 500, lo=100, hi=20000)
    assert s.min() >= 100 and s.max() <= 20000
