"""Pins the CPU oracle against the reference's own known answers (extracted
into tests/golden/reference_known_answers.json by
tests/golden/extract_known_answers.py) and against the structural checks of
the reference's KalmanFitter tests. CPU only."""
import json
import os

import numpy as np
import pytest

from acts_gb300 import abi
from acts_gb300.results import Results
from conftest import batch, detector
from oracle import kforacle

KA = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                 "reference_known_answers.json")))


def _diag(v):
    return np.diag(np.asarray(v, float)).reshape(36)


# ------------------------------------------------ GainMatrixUpdaterTests.cpp
def test_updater_known_answer():
    u = KA["updater"]
    f, fc, chi2, st = kforacle.gain_matrix_update(
        np.array([u["pred"]]), np.array([_diag(u["pred_cov_diag"])]), np.array([u["meas"]]),
        np.array([np.diag(u["meas_cov_diag"]).reshape(4)]))
    assert st[0] == 0
    np.testing.assert_allclose(f[0], u["exp_filtered"], atol=u["tol"])
    np.testing.assert_allclose(np.diag(fc[0]), u["exp_filtered_cov_diag"], atol=u["tol"])
    off = fc[0] - np.diag(np.diag(fc[0]))
    assert np.abs(off).max() <= u["tol"]
    assert abs(chi2[0] - u["exp_chi2"]) <= u["chi2_tol"]


def test_updater_failed():
    u = KA["updater"]
    assert u["failed_case_pred_cov_zero"] and u["failed_case_meas_cov_zero"]
    _, _, _, st = kforacle.gain_matrix_update(np.array([u["pred"]]), np.zeros((1, 36)),
                                              np.array([u["meas"]]), np.zeros((1, 4)))
    assert st[0] == 1  # KalmanFitterError::UpdateFailed


def test_updater_joseph_equals_plain_on_known_answer():
    u = KA["updater"]
    args = (np.array([u["pred"]]), np.array([_diag(u["pred_cov_diag"])]), np.array([u["meas"]]),
            np.array([np.diag(u["meas_cov_diag"]).reshape(4)]))
    a = kforacle.gain_matrix_update(*args, joseph=False)
    b = kforacle.gain_matrix_update(*args, joseph=True)
    np.testing.assert_allclose(a[1], b[1], atol=1e-12)
    np.testing.assert_allclose(a[2], b[2], rtol=1e-12)


# ------------------------------------------------ GainMatrixSmootherTests.cpp
def smoother_inputs():
    s = KA["smoother"]
    cov = _diag(s["cov_diag"])
    pred = np.array([[st["predicted"] for st in s["states"]]])
    filt = np.array([[st["filtered"] for st in s["states"]]])
    covs = np.tile(cov, (1, 3, 1))
    jac = np.tile(np.eye(6).reshape(36), (1, 3, 1))
    return pred, covs, filt, covs.copy(), jac


def test_smoother_known_answer():
    s = KA["smoother"]
    sm, smc, st = kforacle.gain_matrix_smooth(*smoother_inputs())
    assert st[0] == 0
    for k in range(3):
        np.testing.assert_allclose(sm[0, k], s["exp_smoothed"][k], atol=s["tol"])
        np.testing.assert_allclose(np.diag(smc[0, k]), s["exp_cov_diag"], atol=s["tol"])
    # last state: smoothed == filtered; earlier ones differ
    pred, _, filt, _, _ = smoother_inputs()
    assert np.array_equal(sm[0, 2], filt[0, 2])
    assert not np.array_equal(sm[0, 0], filt[0, 0])


def _random_states(n, seed):
    rng = np.random.default_rng(seed)
    scale = np.array([0.05, 0.05, 1e-3, 1e-3, 1e-3, 1.0])
    a = rng.normal(size=(n, 6, 6)) * scale[None, :, None]
    cov = (a @ a.transpose(0, 2, 1) + np.diag(scale ** 2 * 0.1)[None]).reshape(n, 36)
    pred = rng.normal(size=(n, 6)) * scale
    pred[:, 2] = rng.uniform(-3.0, 3.0, n)
    pred[:, 3] = rng.uniform(0.3, 2.8, n)
    meas = pred[:, :2] + rng.normal(size=(n, 2)) * 0.03
    return pred, cov, meas


@pytest.mark.parametrize("h", [0, 1])
@pytest.mark.parametrize("joseph", [False, True])
def test_updater_1d_is_the_2d_limit(h, joseph):
    """visitMeasurementImpl<1> of loc h equals the 2D update in the limit of
    an unmeasured other coordinate (variance 1e16): same filtered state and
    covariance, and the chi2 of the measured coordinate."""
    n = 50
    pred, cov, meas = _random_states(n, 3 + h)
    var = 0.03 ** 2
    m1 = np.zeros((n, 2))
    m1[:, 0] = meas[:, h]
    c1 = np.zeros((n, 4))
    c1[:, 0] = var
    f1, fc1, chi1, st1 = kforacle.gain_matrix_update(pred, cov, m1, c1, joseph=joseph,
                                                     subspace=np.full(n, 1 << h))
    c2 = np.zeros((n, 4))
    c2[:, 3 * h] = var
    c2[:, 3 * (1 - h)] = 1e16
    f2, fc2, chi2, st2 = kforacle.gain_matrix_update(pred, cov, meas, c2, joseph=joseph)
    assert (st1 == 0).all() and (st2 == 0).all()
    np.testing.assert_allclose(f1, f2, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(fc1, fc2, rtol=1e-7, atol=1e-14)
    np.testing.assert_allclose(chi1, chi2, rtol=1e-7)


def test_kf_strip_measurements():
    """Barrel tracks whose outer six layers measure one local coordinate
    (loc0 / loc1 alternating, as the reference's KF test detector): the fits
    succeed where the all-2D barrel fits of the same tracks do, ndf is the
    sum of the measurement dimensions, chi2/ndf ~ 1, and both smoothers
    agree."""
    b = batch(abi.CKG_STRIPS, 300)
    dims = np.where(b.meas_subspace == abi.MEAS_LOC01, 2, 1)
    exp_ndf = np.add.reduceat(dims, b.meas_offsets[:-1])
    r = _fit(abi.CKG_STRIPS, b)
    ok = r.status == 0
    assert ok.mean() > 0.99
    assert np.array_equal(r.status, _fit(abi.CKG_BARREL, batch(abi.CKG_BARREL, 300)).status)
    assert np.array_equal(r.ndf[ok], exp_ndf[ok])
    assert (b.meas_subspace != abi.MEAS_LOC01).sum() > 0.4 * b.meas_subspace.size
    assert 0.9 < r.chi2_sum[ok].sum() / r.ndf[ok].sum() < 1.1
    r2 = _fit(abi.CKG_STRIPS, b, smoother=abi.SMOOTHER_MBF)
    valid = (np.arange(24)[None, :] < r.n_states[:, None]) & ok[:, None]
    np.testing.assert_allclose(r2.view("smoothed")[valid], r.view("smoothed")[valid],
                               rtol=1e-9, atol=1e-12)


def test_kf_strip_outlier_flagged():
    """A 1D measurement displaced by 10 mm is flagged as an outlier by the
    predicted-chi2 cut (outlier finder with a 1D residual)."""
    b = batch(abi.CKG_STRIPS, 100)
    nb = b.subset(np.arange(b.n))
    hit = 0
    for t in range(nb.n):
        for m in range(nb.meas_offsets[t], nb.meas_offsets[t + 1]):
            if nb.meas_subspace[m] != abi.MEAS_LOC01:
                nb.meas_values[2 * m] += 10.0
                hit += 1
                break
    assert hit > 80
    r = _fit(abi.CKG_STRIPS, nb, outlier_chi2_cut=15.0)
    moved = np.array([(nb.meas_subspace[nb.meas_offsets[t]:nb.meas_offsets[t + 1]]
                       != abi.MEAS_LOC01).any() for t in range(nb.n)])
    sel = moved & (r.status == 0)
    assert sel.sum() >= 0.98 * moved.sum()
    assert (r.n_outliers[sel] == 1).all()


def test_invalid_subspace_rejected():
    b = batch(abi.CKG_STRIPS, 10).subset(np.arange(10))
    b.meas_subspace[b.meas_offsets[3]] = 0
    r = _fit(abi.CKG_STRIPS, b)
    assert r.status[3] == 12  # InvalidInput
    assert (np.delete(r.status, 3) != 12).all()


# ------------------------------------------------------ LineSurfaceTests.cpp
def test_line_surface_known_answers():
    ls = KA["line_surface"]
    rot = np.eye(3).reshape(9)
    mom = np.array(ls["g2l_momentum"])
    ok, loc = kforacle.line_global_to_local(ls["center"], rot, ls["g2l_position"],
                                            mom / np.linalg.norm(mom))
    assert ok
    np.testing.assert_allclose(loc, ls["g2l_expected"], atol=1e-6)
    d = np.array(ls["intersect_direction"])
    d = d / np.linalg.norm(d)
    st, path = kforacle.line_intersect(ls["center"], rot, [0.0, 0.0, 0.0], d)
    assert st == 1  # reachable
    np.testing.assert_allclose(path * d, ls["intersect_expected"], atol=1e-6)


def _perigee_fit(preset, n, **kw):
    from acts_gb300 import generate

    det = generate.Detector(preset, perigee=True)
    b = generate.generate(det, n, seed=3)
    res = Results(b.n, 24, abi.OUT_SMOOTHED | abi.OUT_REFERENCE)
    kforacle.fit_batch(det, b, abi.default_options(reference_surface=det.perigee, **kw), res,
                       n_threads=4)
    return det, b, res


@pytest.mark.parametrize("strategy", [abi.EXTRAPOLATE_FIRST, abi.EXTRAPOLATE_FIRST_OR_LAST])
def test_extrapolation_to_perigee_pulls(strategy):
    """extrapolateTrackToReferenceSurface to a PerigeeSurface at the origin
    from the first measurement state (firstOrLast picks it: it is nearer):
    the perigee parameters against the generator truth (d0 = 0, z0 = vertex
    z, and the momentum at the vertex) have pulls of mean 0, width 1."""
    det, b, r = _perigee_fit(abi.CKG_BARREL, 3000, reference_strategy=strategy)
    ok = r.status == 0
    assert ok.mean() > 0.99
    tp, tc = r.track("track_params"), r.track("track_cov")
    ts = b.truth_start.reshape(-1, 6)
    truth = [np.zeros(b.n), b.start_frames.reshape(-1, 12)[:, 11], ts[:, 2], ts[:, 3], ts[:, 4]]
    for i in range(5):
        d = tp[ok, i] - truth[i][ok]
        if i == 2:
            d = (d + np.pi) % (2 * np.pi) - np.pi
        pull = d / np.sqrt(tc[ok, 7 * i])
        assert abs(pull.mean()) < 0.08, (i, pull.mean())
        assert 0.93 < pull.std() < 1.07, (i, pull.std())


def test_extrapolation_strategies_agree_without_material():
    """Without process noise every smoothed state estimates the same
    trajectory: the first, the last and the nearer state give the same
    perigee parameters (telescope), up to the linearisation and the
    Runge-Kutta error of the longer extrapolation (a few % of a sigma)."""
    res = [_perigee_fit(abi.CKG_TELESCOPE, 200, reference_strategy=s)[2]
           for s in (abi.EXTRAPOLATE_FIRST, abi.EXTRAPOLATE_LAST, abi.EXTRAPOLATE_FIRST_OR_LAST)]
    assert all((r.status == 0).all() for r in res)
    sig = np.sqrt(res[0].track("track_cov")[:, [0, 7, 14, 21, 28, 35]])
    for r in res[1:]:
        d = np.abs(r.track("track_params") - res[0].track("track_params")) / sig
        assert d.max() < 0.05, d.max(axis=0)
    np.testing.assert_array_equal(res[2].track("track_params"), res[0].track("track_params"))


def test_line_surface_only_as_reference():
    """A sequence that contains the line surface is invalid input."""
    from acts_gb300 import generate

    det = generate.Detector(abi.CKG_BARREL, perigee=True)
    b = generate.generate(det, 5, seed=3)
    b.seq_surfaces[b.seq_offsets[2]] = det.perigee
    res = Results(b.n, 24)
    kforacle.fit_batch(det, b, abi.default_options(), res, n_threads=1)
    assert res.status[2] == 12
    assert (np.delete(res.status, 2) == 0).all()


# ------------------------------------- CorrectedTransformFreeToBoundTests.cpp
def test_corrected_free_to_bound_known_answer():
    """The unscented free-to-bound correction on the reference's setup: a
    track from the origin (phi 0, theta pi/4, sigma(phi) = sigma(theta) =
    0.25) to a plane at x = 10 mm: loc0 and phi unchanged, loc1 shifted to
    11.2563, sigma(loc0) = 2.5 mm."""
    ka = KA["corrected_free_to_bound"]
    d = ka["distance"]
    # the plane: curvilinear frame of direction x (local x = y, local y = z)
    s = abi.ck_surface()
    s.type = abi.SURFACE_PLANE
    for i, v in enumerate([0, 0, 1, 1, 0, 0, 0, 1, 0]):
        s.rotation[i] = float(v)
    s.center[0] = d
    ph, th = ka["phi"], ka["theta"]
    direction = np.array([np.cos(ph) * np.sin(th), np.sin(ph) * np.sin(th), np.cos(th)])
    path = d / direction[0]
    assert path == pytest.approx(d * np.sqrt(2.0))
    free = np.concatenate([path * direction, [ka["t"]], direction, [ka["qOverP"]]])
    # bound-to-free Jacobian of the plane at the end point (as the test
    # builds it), the bound covariance, the straight-line transport
    j = np.zeros((8, 6))
    j[0:3, 0] = [0, 1, 0]
    j[0:3, 1] = [0, 0, 1]
    j[3, 5] = 1.0
    j[4:7, 2] = [-np.sin(th) * np.sin(ph), np.sin(th) * np.cos(ph), 0.0]
    j[4:7, 3] = [np.cos(th) * np.cos(ph), np.cos(th) * np.sin(ph), -np.sin(th)]
    j[7, 4] = 1.0
    res = [ka["resLoc0"], ka["resLoc1"], ka["resPhi"], ka["resTheta"], ka["resQOverP"],
           ka["resTime"]]
    sfree = j @ np.diag(np.square(res)) @ j.T
    tj = np.eye(8)
    for i in range(3):
        tj[i, 4 + i] = path
    efree = tj @ sfree @ tj.T
    ok, mean, cov = kforacle.corrected_free_to_bound(s, free, efree)
    assert ok
    assert mean[0] == pytest.approx(ka["loc0"], abs=1e-9)
    assert mean[2] == pytest.approx(ka["phi"], abs=1e-9)
    assert mean[1] == pytest.approx(ka["exp_loc1"], rel=ka["eps"])
    assert cov[0, 0] == pytest.approx(ka["exp_loc0_sigma"] ** 2, rel=ka["eps"])


def test_free_to_bound_correction_in_fits():
    """With the correction the fits move by a small fraction of a sigma
    (median < 0.1), except where the sigma points straddle phi = +-pi: the
    reference's unscented transform averages the bound vectors without
    unwrapping, which breaks such a fit (~1 in 2000 barrel tracks)."""
    b = batch(abi.CKG_BARREL, 2000)
    r0 = _fit(abi.CKG_BARREL, b)
    r1 = _fit(abi.CKG_BARREL, b, free_to_bound_correction=1)
    ok = (r0.status == 0) & (r1.status == 0)
    assert ok.mean() > 0.98
    a, c = r0.view("smoothed")[ok, 0], r1.view("smoothed")[ok, 0]
    assert not np.array_equal(a, c)
    sig = np.sqrt(r0.view("smoothed_cov")[ok, 0][:, [0, 7, 14, 21, 28]])
    d = (np.abs(c[:, :5] - a[:, :5]) / sig).max(axis=1)
    assert np.median(d) < 0.1
    broken = d > 1.0
    assert broken.sum() <= 0.002 * ok.sum()
    assert (np.abs(np.abs(a[broken, 2]) - np.pi) < 0.1).all()  # at the seam


# ---------------------------------------------------- MbfSmootherTests.cpp
def mbf_inputs():
    s = KA["mbf_smoother"]
    cov = _diag(s["cov_diag"])
    pred = np.array([[st["predicted"] for st in s["states"]]])
    filt = np.array([[st["filtered"] for st in s["states"]]])
    meas = np.array([[st["calibrated"] for st in s["states"]]])
    mcov = np.array([[st["calibrated_cov"] for st in s["states"]]])
    covs = np.tile(cov, (1, 3, 1))
    jac = np.tile(np.eye(6).reshape(36), (1, 3, 1))
    flags = np.full((1, 3), abi.FLAG_HAS_MEASUREMENT | abi.FLAG_HAS_PARAMETERS, np.uint32)
    return flags, pred, covs, filt, covs.copy(), jac, meas, mcov


def test_mbf_smoother_known_answer():
    s = KA["mbf_smoother"]
    sm, smc = kforacle.mbf_smooth(*mbf_inputs())
    for k in range(3):
        np.testing.assert_allclose(sm[0, k], s["exp_smoothed"][k], atol=s["tol"])
        np.testing.assert_allclose(smc[0, k], np.diag(s["exp_cov_diag"]), atol=s["tol"])
    # the last state: smoothed == filtered; the earlier ones differ
    filt = mbf_inputs()[3]
    assert np.array_equal(sm[0, 2], filt[0, 2])
    assert not np.array_equal(sm[0, 0], filt[0, 0])
    assert not np.array_equal(sm[0, 1], filt[0, 1])


@pytest.mark.parametrize("preset", [abi.CKG_TELESCOPE, abi.CKG_BARREL])
def test_mbf_equals_gain_matrix_smoother(preset):
    """The modified Bryson-Frazier and the Rauch-Tung-Striebel (gain-matrix)
    smoothers are the same estimator (with or without the material noise the
    barrel adds between states): whole fits agree to rounding (measured
    <= 2e-12 relative on the parameters, <= 3e-11 on the covariances)."""
    b = batch(preset, 50)
    r1 = _fit(preset, b)
    r2 = _fit(preset, b, smoother=abi.SMOOTHER_MBF)
    ok = r1.status == 0
    assert ok.mean() > 0.9 and np.array_equal(r1.status, r2.status)
    assert np.array_equal(r1.n_states, r2.n_states)
    valid = (np.arange(24)[None, :] < r1.n_states[:, None]) & ok[:, None]
    a, c = r1.view("smoothed")[valid], r2.view("smoothed")[valid]
    assert not np.array_equal(a, c)  # different arithmetic
    np.testing.assert_allclose(c, a, rtol=1e-9, atol=1e-12)
    a, c = r1.view("smoothed_cov")[valid], r2.view("smoothed_cov")[valid]
    np.testing.assert_allclose(c, a, rtol=1e-8, atol=1e-15)


# ------------------------------------------------------ InteractionsTests.cpp
SI = KA["silicon"]


def _interaction(which, thickness, pdg, m, qop, absq):
    return kforacle.interaction(which, thickness, SI["X0"], SI["L0"], SI["Ar"], SI["Z"],
                                SI["molar_rho"], pdg, m, qop, absq)


def _momenta():
    low = np.arange(0.1, 10.0, 0.1)
    med = np.arange(10.0, 100.0, 10.0)
    high = np.arange(100.0, 10000.0, 100.0)
    return np.concatenate([low, med, high])


PARTICLES = [(11, 0.000511, -1.0), (13, 0.1057, -1.0), (211, 0.1396, 1.0), (2212, 0.9383, 1.0)]


@pytest.mark.parametrize("thickness", KA["interactions"]["consistency"]["thickness"])
@pytest.mark.parametrize("pdg,m,q", PARTICLES)
def test_energy_loss_and_scattering_consistency(thickness, pdg, m, q):
    for p in _momenta()[::7]:
        qop = q / p
        bethe = _interaction(0, thickness, pdg, m, qop, abs(q))
        landau = _interaction(1, thickness, pdg, m, qop, abs(q))
        sig_qop = _interaction(2, thickness, pdg, m, qop, abs(q))
        sigma = _interaction(4, thickness, pdg, m, qop, abs(q)) * 0.42466090014400953
        assert bethe > 0 and landau > 0 and sig_qop > 0 and sigma > 0
        assert sigma <= bethe
        t0 = _interaction(3, thickness, pdg, m, qop, abs(q))
        assert t0 > 0
        assert _interaction(3, thickness, pdg, m, -qop, abs(q)) == t0
        assert _interaction(3, 2 * thickness, pdg, m, qop, abs(q)) > t0
        assert _interaction(3, thickness, pdg, m, q / (2 * p), abs(q)) < t0


def test_vacuum_has_no_interactions():
    for which in range(5):
        v = kforacle.interaction(which, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 13, 0.1057, 1.0, 1.0)
        assert v == 0.0


def test_silicon_bethe_against_pdg():
    c = KA["interactions"]["silicon_bethe"]
    # mass density of silicon in native units (Material::massDensity)
    u = 0.93149410242
    avogadro = 6.02214076e23
    rho = SI["Ar"] * u * np.float32(SI["molar_rho"]) * avogadro
    g = 1.0 / 1.782662e-24
    for p, loss in zip(c["momentum"], c["loss_MeV_cm2_per_g"]):
        de = _interaction(0, c["thickness"], 13, c["mass"], -1.0 / p, 1.0)
        value = de / c["thickness"] / rho / (1e-3 * 100.0 / g)
        assert abs(value - loss) / loss * 100 <= c["percent"], (p, value, loss)


def test_silicon_landau():
    c = KA["interactions"]["silicon_landau"]
    de = _interaction(1, c["thickness"], 13, c["mass"], -1.0 / c["momentum"], 1.0) / 1e-3
    assert abs(de - c["dE_MeV"]) / c["dE_MeV"] * 100 <= c["dE_percent"]
    fw = _interaction(4, c["thickness"], 13, c["mass"], -1.0 / c["momentum"], 1.0) / 1e-3
    assert abs(fw - c["fwhm_MeV"]) / c["fwhm_MeV"] * 100 <= c["fwhm_percent"]


# ------------------------------------------------ InterpolatedBFieldMapTests.cpp
def linear_grid():
    """A small XYZ map filled with a trilinear function: interpolation must
    reproduce it exactly (the RZ bilinear test of the reference, in 3D)."""
    n = (5, 4, 7)
    lo, hi = (-2.0, -1.5, -3.0), (2.0, 1.5, 3.0)
    xs = [np.linspace(lo[i], hi[i], n[i]) for i in range(3)]
    X, Y, Z = np.meshgrid(*xs, indexing="ij")
    vals = np.stack([X * Y + Z, 3 * Y - X * Z, -2 * Z + X * Y * Z], axis=-1).astype(np.float32)
    f = abi.ck_field()
    f.kind = abi.FIELD_GRID_XYZ
    for i in range(3):
        f.n[i] = n[i]
        f.min[i] = lo[i]
        f.max[i] = hi[i]
    vals = np.ascontiguousarray(vals.reshape(-1))
    f.values_tesla = abi.ptr(vals, __import__("ctypes").c_float)
    return f, vals, lo, hi


def field_truth(p):
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    return np.stack([x * y + z, 3 * y - x * z, -2 * z + x * y * z], axis=-1) * 0.000299792458


def test_field_map_trilinear_exact_and_bounds():
    f, keep, lo, hi = linear_grid()
    rng = np.random.default_rng(1)
    pts = rng.uniform(lo, hi, size=(400, 3)) * 0.999
    b, st = kforacle.field_lookup(f, pts)
    assert (st == 0).all()
    # exact up to the float32 node values
    np.testing.assert_allclose(b, field_truth(pts), rtol=2e-6, atol=2e-9)
    # isInside: [min, max) per axis
    edge = np.array([[lo[0], 0.0, 0.0], [hi[0], 0.0, 0.0], [0.0, 0.0, hi[2] - 1e-9],
                     [0.0, lo[1] - 1e-9, 0.0], [0.0, 0.0, 3.5]])
    _, st = kforacle.field_lookup(f, edge)
    assert list(st == 0) == [True, False, True, False, False]


# --------------------------------------------- KalmanFitterTests.cpp structure
def _fit(preset, b, **kw):
    det = detector(preset)
    res = Results(b.n, 24)
    kforacle.fit_batch(det, b, abi.default_options(**kw), res, n_threads=4)
    return res


def test_kf_all_measurements():
    b = batch(abi.CKG_TELESCOPE, 50)
    r = _fit(abi.CKG_TELESCOPE, b)
    assert (r.status == 0).all()
    assert (r.n_measurements == np.diff(b.meas_offsets)).all()
    assert (r.n_holes == 0).all() and (r.n_outliers == 0).all()
    assert (r.ndf == 2 * r.n_measurements).all()


def test_kf_hole_counted_once():
    b = batch(abi.CKG_TELESCOPE, 20)
    for remove in range(1, 9):  # interior measurements
        keep = []
        for t in range(b.n):
            keep.append([m for m in range(b.meas_offsets[t], b.meas_offsets[t + 1])
                         if m - b.meas_offsets[t] != remove])
        nb = _drop_measurements(b, keep)
        r = _fit(abi.CKG_TELESCOPE, nb)
        assert (r.status == 0).all()
        assert (r.n_holes == 1).all(), remove
        assert (r.n_measurements == 9).all()


def test_kf_outlier_flagged():
    b = batch(abi.CKG_TELESCOPE, 20)
    for replace in range(0, 10, 3):
        nb = b.subset(np.arange(b.n))
        for t in range(b.n):
            m = nb.meas_offsets[t] + replace
            nb.meas_values[2 * m] += 10.0  # 10 mm displacement as the reference test
        r = _fit(abi.CKG_TELESCOPE, nb, outlier_chi2_cut=15.0)
        assert (r.status == 0).all()
        assert (r.n_outliers == 1).all(), replace
        assert (r.n_measurements == 9).all()


def test_kf_shuffled_source_links_identical():
    b = batch(abi.CKG_BARREL, 50)
    r1 = _fit(abi.CKG_BARREL, b)
    nb = b.subset(np.arange(b.n))
    rng = np.random.default_rng(5)
    for t in range(b.n):
        a, e = nb.meas_offsets[t], nb.meas_offsets[t + 1]
        perm = rng.permutation(e - a)
        nb.meas_surfaces[a:e] = nb.meas_surfaces[a:e][perm]
        nb.meas_values[2 * a:2 * e] = nb.meas_values[2 * a:2 * e].reshape(-1, 2)[perm].reshape(-1)
        nb.meas_cov[4 * a:4 * e] = nb.meas_cov[4 * a:4 * e].reshape(-1, 4)[perm].reshape(-1)
    r2 = _fit(abi.CKG_BARREL, nb)
    assert np.array_equal(r1.status, r2.status)
    np.testing.assert_array_equal(r1.smoothed, r2.smoothed)


def test_coasting_and_early_termination():
    """The reference keeps propagating after the last surface when outliers
    leave the track incomplete, until the loop-protection path limit; the
    states it adds there are never part of the track. So: tracks that survive
    this coasting are identical under both termination rules, and the tracks
    that fail do so only through propagation errors after the tip (on the
    uneven workload's field map: leaving the map), where the early rule
    succeeds."""
    preset = abi.CKG_UNEVEN
    det = detector(preset)
    b = batch(preset, 300)
    r1, r2 = Results(b.n, 24), Results(b.n, 24)
    kforacle.fit_batch(det, b, abi.default_options(outlier_chi2_cut=15.0), r1, n_threads=4)
    kforacle.fit_batch(det, b, abi.default_options(outlier_chi2_cut=15.0, early_termination=1),
                       r2, n_threads=4)
    assert (r2.n_outliers > 0).sum() > 20  # the case is exercised
    ok = r1.status == 0
    assert ok.sum() > 100
    assert (r2.status[ok] == 0).all()
    for name in ("n_states", "n_measurements", "n_holes", "n_outliers"):
        np.testing.assert_array_equal(getattr(r1, name)[ok], getattr(r2, name)[ok], err_msg=name)
    for name in ("state_flags", "smoothed", "smoothed_cov", "filtered", "predicted", "jacobian"):
        np.testing.assert_array_equal(r1.view(name)[ok], r2.view(name)[ok], err_msg=name)
    failed = ~ok
    assert set(np.unique(r1.status[failed])) <= {abi_status("MagneticFieldOutOfBounds"),
                                                  abi_status("StepCountLimitReached")}
    assert (r2.status[failed] == 0).all()
    assert (r2.n_outliers[failed] > 0).all()


def abi_status(name):
    return [k for k, v in abi.TRACK_STATUS.items() if v == name][0]


def test_no_measurement_found():
    b = batch(abi.CKG_TELESCOPE, 5)
    nb = _drop_measurements(b, [[] for _ in range(b.n)])
    r = _fit(abi.CKG_TELESCOPE, nb)
    assert (r.status == 3).all()  # KalmanFitterError::NoMeasurementFound


def test_invalid_surface_id_rejected():
    b = batch(abi.CKG_TELESCOPE, 5).subset(np.arange(5))
    b.seq_surfaces[0] = 999
    r = _fit(abi.CKG_TELESCOPE, b)
    assert r.status[0] == 12 and (r.status[1:] == 0).all()


def test_logf_restatement_mismatch_rate():
    """ck_logf (correctly rounded) against glibc logf on the arguments the
    material physics sees: the documented deviation is rare."""
    rng = np.random.default_rng(3)
    x = np.exp(rng.uniform(np.log(1e-6), np.log(1e6), 200000)).astype(np.float32)
    bad = kforacle.logf_mismatch(x)
    assert bad / len(x) < 1e-2, bad


def _drop_measurements(b, keep):
    from acts_gb300.generate import Batch

    nb = b.subset(np.arange(b.n))
    ms, mv, mc, tm, mo = [], [], [], [], [0]
    for t in range(b.n):
        for m in keep[t]:
            ms.append(b.meas_surfaces[m])
            mv.extend(b.meas_values[2 * m:2 * m + 2])
            mc.extend(b.meas_cov[4 * m:4 * m + 4])
            tm.extend(b.truth_meas[6 * m:6 * m + 6])
        mo.append(len(ms))
    nb.meas_surfaces = np.ascontiguousarray(np.array(ms, np.int32))
    nb.meas_values = np.ascontiguousarray(np.array(mv, np.float64))
    nb.meas_cov = np.ascontiguousarray(np.array(mc, np.float64))
    nb.truth_meas = np.ascontiguousarray(np.array(tm, np.float64))
    nb.meas_offsets = np.ascontiguousarray(np.array(mo, np.int32))
    nb.meas_outlier = np.zeros(len(ms), np.uint8)
    return nb
