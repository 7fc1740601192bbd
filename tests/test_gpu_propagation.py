"""The fitter's CUDA stepper through ck_propagate, held to the reference's
propagation property tests (PropagationTests.hpp, PropagationEigenConstant.cpp
datasets and tolerances; tests/propagation_cases.py) in both precision
forms, the JacobianEngine identities, and FP64 parity with the oracle's
propagation restatement: statuses and step counts equal, end parameters,
covariances, Jacobians and path lengths within 1e-9 (floors as in the fit
parity: sigma, sqrt(C_ii C_jj), 1e-4 of the Jacobian row, 1 mm)."""
import numpy as np
import pytest

import propagation_cases as pc
from acts_gb300 import abi
from parity import JAC_ROW_FLOOR
from test_oracle_propagation import check_jacobian_engine, jacobian_engine_case

FORMS = [abi.PRECISION_FP64, abi.PRECISION_MIXED]
IDS = ["fp64", "mixed"]
RTOL = 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("precision", FORMS, ids=IDS)
@pytest.mark.parametrize("tesla", pc.FIELDS_T)
def test_forward_backward(tesla, precision):
    rep = pc.forward_backward(pc.CudaBackend(precision), tesla, abi.default_options())
    print(rep)
    assert max(rep.values()) < 1.0, rep


@pytest.mark.gpu
@pytest.mark.parametrize("precision", FORMS, ids=IDS)
@pytest.mark.parametrize("kind", ["plane", "cylinder", "straw"])
@pytest.mark.parametrize("tesla", pc.FIELDS_T)
def test_to_surface(tesla, kind, precision):
    rep = pc.to_surface(pc.CudaBackend(precision), tesla, kind, abi.default_options())
    print(kind, rep)
    assert max(rep.values()) < 1.0, rep


@pytest.mark.gpu
@pytest.mark.parametrize("precision", FORMS, ids=IDS)
@pytest.mark.parametrize("kind", ["curvilinear", "plane", "cylinder", "straw"])
@pytest.mark.parametrize("tesla", pc.FIELDS_T)
def test_covariance_transport(tesla, kind, precision):
    worst, _, _ = pc.covariance(pc.CudaBackend(precision), tesla, kind, abi.default_options())
    print(kind, worst)
    assert worst < 1.0


@pytest.mark.gpu
@pytest.mark.parametrize("precision", FORMS, ids=IDS)
def test_jacobian_engine_identities(precision):
    table, prop = jacobian_engine_case()
    pc.CudaBackend(precision).propagate(pc.constant_field(2.0), table, prop,
                                        abi.default_options())
    check_jacobian_engine(prop, 1e-12 if precision == abi.PRECISION_FP64 else 1e-6)


def _rel(a, b, floor):
    return np.abs(a - b) / np.maximum(np.maximum(np.maximum(np.abs(a), np.abs(b)), floor), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["curvilinear", "plane", "cylinder", "straw"])
@pytest.mark.parametrize("tesla", pc.FIELDS_T)
def test_fp64_parity_with_oracle(tesla, kind):
    opt = abi.default_options()
    _, g, _ = pc.covariance(pc.CudaBackend(abi.PRECISION_FP64), tesla, kind, opt)
    _, o, _ = pc.covariance(pc.OracleBackend(), tesla, kind, opt)
    assert np.array_equal(g.status, o.status)
    assert np.array_equal(g.steps, o.steps)
    cov = o.end_cov.T.reshape(-1, 6, 6)
    sig = np.sqrt(np.abs(np.einsum("nii->ni", cov)))
    dp = np.abs(g.end_params - o.end_params)
    dp[2] = np.abs((g.end_params[2] - o.end_params[2] + np.pi) % (2 * np.pi) - np.pi)
    rp = dp.T / np.maximum(np.maximum(np.abs(g.end_params.T), np.abs(o.end_params.T)), sig)
    rc = _rel(g.end_cov.T, o.end_cov.T, (sig[:, :, None] * sig[:, None, :]).reshape(-1, 36))
    jo = o.jacobian.T.reshape(-1, 6, 6)
    rowmax = np.abs(jo).max(axis=2, keepdims=True) * JAC_ROW_FLOOR
    rj = _rel(g.jacobian.T, o.jacobian.T, np.broadcast_to(rowmax, jo.shape).reshape(-1, 36))
    rl = _rel(g.path_length, o.path_length, 1.0)
    rep = {"params": rp.max(), "cov": rc.max(), "jac": rj.max(), "path": rl.max()}
    print(kind, rep)
    assert max(rep.values()) <= RTOL, rep
