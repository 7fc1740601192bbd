"""Unit operators of the CUDA fitter through the C ABI: the reference's own
known answers (GainMatrixUpdater, GainMatrixSmoother), the float material
physics bit-exact against the oracle, and the field lookup."""
import json
import os

import numpy as np
import pytest

from acts_gb300 import abi
from conftest import batch, detector
from oracle import kforacle

KA = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                 "reference_known_answers.json")))


def _diag(v):
    return np.diag(np.asarray(v, float)).reshape(36)


@pytest.mark.gpu
def test_updater_known_answer_on_gpu(fitter_factory):
    u = KA["updater"]
    fit = fitter_factory(abi.CKG_TELESCOPE)
    args = (np.array([u["pred"]]), np.array([_diag(u["pred_cov_diag"])]), np.array([u["meas"]]),
            np.array([np.diag(u["meas_cov_diag"]).reshape(4)]))
    f, fc, chi2, st = fit.gain_matrix_update(*args)
    assert st[0] == 0
    np.testing.assert_allclose(f[0], u["exp_filtered"], atol=u["tol"])
    np.testing.assert_allclose(np.diag(fc[0]), u["exp_filtered_cov_diag"], atol=u["tol"])
    assert abs(chi2[0] - u["exp_chi2"]) <= u["chi2_tol"]
    # UpdateFailed on zero covariances
    _, _, _, st = fit.gain_matrix_update(args[0], np.zeros((1, 36)), args[2], np.zeros((1, 4)))
    assert st[0] == 1


@pytest.mark.gpu
@pytest.mark.parametrize("joseph", [False, True])
def test_updater_random_states_match_oracle(fitter_factory, joseph):
    rng = np.random.default_rng(4)
    n = 2000
    A = rng.normal(size=(n, 6, 6)) * np.array([0.1, 0.1, 0.01, 0.01, 0.001, 1.0])[None, :, None]
    P = A @ A.transpose(0, 2, 1) + np.eye(6) * 1e-6
    pred = rng.normal(size=(n, 6)) * 0.1
    pred[:, 3] = 1.0 + 0.2 * rng.normal(size=n)
    meas = pred[:, :2] + rng.normal(size=(n, 2)) * 0.05
    V = np.zeros((n, 4))
    V[:, 0] = 0.0025
    V[:, 3] = 0.0025
    fit = fitter_factory(abi.CKG_TELESCOPE)
    g = fit.gain_matrix_update(pred, P.reshape(n, 36), meas, V, joseph)
    o = kforacle.gain_matrix_update(pred, P.reshape(n, 36), meas, V, joseph)
    assert (g[3] == o[3]).all()
    np.testing.assert_allclose(g[0], o[0], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(g[1], o[1], rtol=1e-9, atol=1e-15)
    np.testing.assert_allclose(g[2], o[2], rtol=1e-9)


@pytest.mark.gpu
def test_smoother_known_answer_on_gpu(fitter_factory):
    s = KA["smoother"]
    cov = _diag(s["cov_diag"])
    pred = np.array([[st["predicted"] for st in s["states"]]])
    filt = np.array([[st["filtered"] for st in s["states"]]])
    covs = np.tile(cov, (1, 3, 1))
    jac = np.tile(np.eye(6).reshape(36), (1, 3, 1))
    fit = fitter_factory(abi.CKG_TELESCOPE)
    sm, smc, st = fit.gain_matrix_smooth(pred, covs, filt, covs.copy(), jac)
    assert st[0] == 0
    for k in range(3):
        np.testing.assert_allclose(sm[0, k], s["exp_smoothed"][k], atol=s["tol"])
        np.testing.assert_allclose(np.diag(smc[0, k]), s["exp_cov_diag"], atol=s["tol"])


@pytest.mark.gpu
@pytest.mark.parametrize("joseph", [False, True])
def test_updater_1d_against_oracle(fitter_factory, joseph):
    """visitMeasurementImpl<1> (loc0 or loc1) on random states: device
    against the oracle's restatement."""
    rng = np.random.default_rng(21)
    n = 400
    scale = np.array([0.05, 0.05, 1e-3, 1e-3, 1e-3, 1.0])
    a = rng.normal(size=(n, 6, 6)) * scale[None, :, None]
    cov = (a @ a.transpose(0, 2, 1) + np.diag(scale ** 2 * 0.1)[None]).reshape(n, 36)
    pred = rng.normal(size=(n, 6)) * scale
    pred[:, 2] = rng.uniform(-3.0, 3.0, n)
    pred[:, 3] = rng.uniform(0.3, 2.8, n)
    meas = pred[:, :2] + rng.normal(size=(n, 2)) * 0.03
    mcov = np.zeros((n, 4))
    mcov[:, 0] = 0.1 ** 2
    sub = rng.choice([abi.MEAS_LOC0, abi.MEAS_LOC1], n).astype(np.int32)
    fit = fitter_factory(abi.CKG_TELESCOPE)
    g = fit.gain_matrix_update(pred, cov, meas, mcov, joseph=joseph, subspace=sub)
    o = kforacle.gain_matrix_update(pred, cov, meas, mcov, joseph=joseph, subspace=sub)
    assert (g[3] == 0).all() and (o[3] == 0).all()
    np.testing.assert_allclose(g[0], o[0], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(g[1], o[1], rtol=1e-9, atol=1e-15)
    np.testing.assert_allclose(g[2], o[2], rtol=1e-9)


@pytest.mark.gpu
def test_mbf_smoother_known_answer_on_gpu(fitter_factory):
    s = KA["mbf_smoother"]
    cov = _diag(s["cov_diag"])
    pred = np.array([[st["predicted"] for st in s["states"]]])
    filt = np.array([[st["filtered"] for st in s["states"]]])
    meas = np.array([[st["calibrated"] for st in s["states"]]])
    mcov = np.array([[st["calibrated_cov"] for st in s["states"]]])
    covs = np.tile(cov, (1, 3, 1))
    jac = np.tile(np.eye(6).reshape(36), (1, 3, 1))
    flags = np.full((1, 3), abi.FLAG_HAS_MEASUREMENT | abi.FLAG_HAS_PARAMETERS, np.uint32)
    fit = fitter_factory(abi.CKG_TELESCOPE)
    sm, smc = fit.mbf_smooth(flags, pred, covs, filt, covs.copy(), jac, meas, mcov)
    for k in range(3):
        np.testing.assert_allclose(sm[0, k], s["exp_smoothed"][k], atol=s["tol"])
        np.testing.assert_allclose(smc[0, k], np.diag(s["exp_cov_diag"]), atol=s["tol"])
    assert np.array_equal(sm[0, 2], filt[0, 2])


def _spd(rng, n, scale):
    a = rng.normal(size=(n, 6, 6)) * scale[None, :, None]
    return a @ a.transpose(0, 2, 1) + np.diag(scale ** 2 * 0.1)[None]


@pytest.mark.gpu
def test_mbf_smoother_random_trajectories(fitter_factory):
    """Trajectories with measurement, outlier, hole and material states,
    random covariances and Jacobians: the device MbfSmoother against the
    oracle's restatement within 1e-9 relative."""
    rng = np.random.default_rng(11)
    nt, ns = 200, 12
    scale = np.array([0.05, 0.05, 1e-3, 1e-3, 1e-3, 1.0])
    pc = _spd(rng, nt * ns, scale).reshape(nt, ns, 36)
    fc = (_spd(rng, nt * ns, scale) * 0.5).reshape(nt, ns, 36)
    pred = rng.normal(size=(nt, ns, 6)) * scale
    pred[..., 2] = rng.uniform(-3.0, 3.0, (nt, ns))
    pred[..., 3] = rng.uniform(0.3, 2.8, (nt, ns))
    filt = pred + rng.normal(size=(nt, ns, 6)) * scale * 0.1
    jac = (np.eye(6)[None, None] + rng.normal(size=(nt, ns, 6, 6)) * 0.05).reshape(nt, ns, 36)
    meas = pred[..., :2] + rng.normal(size=(nt, ns, 2)) * 0.02
    mcov = np.tile(np.array([4e-4, 1e-5, 1e-5, 2.5e-3]), (nt, ns, 1))
    kinds = rng.choice([abi.FLAG_HAS_MEASUREMENT,
                        abi.FLAG_HAS_MEASUREMENT | abi.FLAG_IS_OUTLIER,
                        abi.FLAG_IS_HOLE, abi.FLAG_HAS_MATERIAL], size=(nt, ns),
                       p=[0.7, 0.1, 0.1, 0.1])
    flags = (kinds | abi.FLAG_HAS_PARAMETERS).astype(np.uint32)
    args = (flags, pred, pc, filt, fc, jac, meas, mcov)
    fit = fitter_factory(abi.CKG_TELESCOPE)
    g, gc = fit.mbf_smooth(*args)
    o, oc = kforacle.mbf_smooth(*args)
    np.testing.assert_allclose(g, o, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(gc, oc, rtol=1e-9, atol=1e-12 * np.abs(oc).max())


@pytest.mark.gpu
def test_material_effects_bit_exact(fitter_factory):
    """The float Bethe / Landau / Highland physics is reproduced bit for bit
    (un-contracted float arithmetic, shared correctly rounded logf)."""
    det = detector(abi.CKG_BARREL)
    fit = fitter_factory(abi.CKG_BARREL)
    rng = np.random.default_rng(7)
    n = 4000
    sid = rng.integers(0, det.n_surfaces, n).astype(np.int32)
    scale = rng.uniform(1.0, 3.0, n).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    p = np.exp(rng.uniform(np.log(0.05), np.log(500.0), n))
    qop = np.where(rng.uniform(size=n) < 0.5, -1.0, 1.0) / p
    mass = np.full(n, 0.13957039, np.float32)
    absq = np.ones(n, np.float32)
    pdg = np.full(n, 211, np.int32)
    g = fit.material_effects(sid, scale, d, qop, mass, absq, pdg)
    for i in range(0, n, 37):
        o = kforacle.material_effects(det.surfaces[int(sid[i])], float(scale[i]), d[i], qop[i],
                                      float(mass[i]), 1.0, 211)
        assert np.array_equal(g[i], o), (i, g[i], o)


@pytest.mark.gpu
def test_field_lookup_matches_oracle(fitter_factory):
    det = detector(abi.CKG_UNEVEN)
    fit = fitter_factory(abi.CKG_UNEVEN)
    rng = np.random.default_rng(2)
    pts = rng.uniform([-1600, -1600, -3100], [1600, 1600, 3100], size=(20000, 3))
    g, gs = fit.field_lookup(pts)
    o, os_ = kforacle.field_lookup(det.field, pts)
    assert np.array_equal(gs, os_)
    ok = gs == 0
    assert ok.sum() > 10000 and (~ok).sum() > 1000
    np.testing.assert_allclose(g[ok], o[ok], rtol=1e-12, atol=1e-18)


# FP32 field lookup of the mixed form against the FP64 oracle: the float
# nodes are exact in both; the position rounded to float (ulp 2.4e-4 mm at
# 3 m), the float trilinear weights and the float interpolation each give a
# few 1e-7 of the field scale, so every component must agree with the FP64
# lookup within 2e-6 of the map's maximum |B|.
FIELD_FP32_BOUND = 2e-6


@pytest.mark.gpu
def test_field_lookup_fp32_matches_oracle(fitter_factory):
    det = detector(abi.CKG_UNEVEN)
    fit = fitter_factory(abi.CKG_UNEVEN)
    rng = np.random.default_rng(4)
    pts = rng.uniform([-1600, -1600, -3100], [1600, 1600, 3100], size=(50000, 3))
    g, gs = fit.field_lookup(pts, abi.PRECISION_MIXED)
    o, os_ = kforacle.field_lookup(det.field, pts)
    # the status differs only where rounding to float moves a point across
    # the map's edge (a float ulp from it)
    edge = np.zeros(len(pts), bool)
    for i, (lo, hi) in enumerate(((-1500.0, 1500.0), (-1500.0, 1500.0), (-3000.0, 3000.0))):
        edge |= (np.abs(pts[:, i] - lo) < 1e-3) | (np.abs(pts[:, i] - hi) < 1e-3)
    assert np.array_equal(gs[~edge], os_[~edge])
    ok = (gs == 0) & (os_ == 0)
    assert ok.sum() > 25000
    scale = np.abs(o[ok]).max()
    err = np.abs(g[ok] - o[ok]).max() / scale
    print("FP32 field lookup: max |dB| / max |B| = %.3g" % err)
    assert err <= FIELD_FP32_BOUND


@pytest.mark.gpu
def test_mixed_form_atan2_matches_correctly_rounded(fitter_factory):
    """The mixed form's table-driven FP64 atan2 against numpy's arctan2 on
    random directions of all magnitudes and the edge cases (axes, the +-pi
    seam, tiny and huge components): within 4 ulp."""
    fit = fitter_factory(abi.CKG_BARREL)
    rng = np.random.default_rng(3)
    n = 200000
    ang = rng.uniform(-np.pi, np.pi, n)
    mag = 10.0 ** rng.uniform(-8, 4, n)
    y, x = mag * np.sin(ang), mag * np.cos(ang)
    edge_y = np.array([0.0, 0.0, 1.0, -1.0, 1e-300, -1e-300, 1e-12, -1e-12, 1.0, 1.0, 3e3, -2.0])
    edge_x = np.array([1.0, -1.0, 0.0, 0.0, -1.0, -1.0, -1.0, -1.0, 1e-12, -1e-12, 1e-3, 1e-9])
    y = np.concatenate([y, edge_y])
    x = np.concatenate([x, edge_x])
    got = fit.atan2_mixed(y, x)
    ref = np.arctan2(y, x)
    ulp = np.abs(got - ref) / np.spacing(np.abs(ref)).clip(min=np.spacing(1e-300))
    # +-pi for y = -0 / +0 with x < 0 are the same angle
    seam = np.isclose(np.abs(ref), np.pi) & np.isclose(np.abs(got), np.pi)
    ulp[seam] = np.minimum(ulp[seam], np.abs(np.abs(got[seam]) - np.abs(ref[seam])) / np.spacing(np.pi))
    assert ulp.max() <= 4, (ulp.max(), y[ulp.argmax()], x[ulp.argmax()])


@pytest.mark.gpu
def test_reference_surface_must_be_a_line(fitter_factory):
    """A reference surface that is not a line (perigee) surface is rejected
    with CK_ERR_UNSUPPORTED; an index outside the table with
    CK_ERR_INVALID_ARGUMENT."""
    from acts_gb300.fitter import CudaKalmanError

    fit = fitter_factory(abi.CKG_BARREL)
    b = batch(abi.CKG_BARREL, 10)
    with pytest.raises(CudaKalmanError) as e:
        fit.fit_batch(b, abi.default_options(reference_surface=0))
    assert e.value.status == abi.CK_ERR_UNSUPPORTED
    with pytest.raises(CudaKalmanError) as e:
        fit.fit_batch(b, abi.default_options(reference_surface=10 ** 6))
    assert e.value.status == abi.CK_ERR_INVALID_ARGUMENT
