"""Pins the oracle's stepper, transport and intersections to the reference's
own propagation property tests (Tests/IntegrationTests/PropagationTests.hpp
run by PropagationEigenConstant.cpp:65-166): forward-backward closure,
reaching surfaces built from a free propagation (plane, z-cylinder,
z-straw), and the covariance transported with the analytic Jacobian against
the numerically transported one, on the reference's datasets with its
tolerances (tests/propagation_cases.py). Also the JacobianEngine identities
of JacobianEngineTests.cpp:28-110 on a zero-length propagation."""
import numpy as np
import pytest

import propagation_cases as pc
from acts_gb300 import abi


@pytest.fixture(scope="module")
def oracle():
    return pc.OracleBackend()


@pytest.mark.parametrize("tesla", pc.FIELDS_T)
def test_forward_backward(oracle, tesla):
    rep = pc.forward_backward(oracle, tesla, abi.default_options())
    print(rep)
    assert max(rep.values()) < 1.0, rep


@pytest.mark.parametrize("kind", ["plane", "cylinder", "straw"])
@pytest.mark.parametrize("tesla", pc.FIELDS_T)
def test_to_surface(oracle, tesla, kind):
    rep = pc.to_surface(oracle, tesla, kind, abi.default_options())
    print(kind, rep)
    assert max(rep.values()) < 1.0, rep


@pytest.mark.parametrize("kind", ["curvilinear", "plane", "cylinder", "straw"])
@pytest.mark.parametrize("tesla", pc.FIELDS_T)
def test_covariance_transport(oracle, tesla, kind):
    worst, _, _ = pc.covariance(oracle, tesla, kind, abi.default_options())
    print(kind, worst)
    assert worst < 1.0


def jacobian_engine_case():
    """JacobianEngineTests.cpp:28-60: a curvilinear plane through (1, 2, 3)
    with the direction (5, 2, 7), q/p 0.125, time 4, covariance 0.025 I, and
    a plane through the same point normal to (6, 2, 8)."""
    pos = np.array([1.0, 2.0, 3.0])
    d = np.array([5.0, 2.0, 7.0]) / np.linalg.norm([5.0, 2.0, 7.0])
    od = np.array([6.0, 2.0, 8.0]) / np.linalg.norm([6.0, 2.0, 8.0])
    frame = pc.curvilinear_frame(d, pos)
    params = np.array([[0.0, 0.0, np.arctan2(d[1], d[0]), np.arccos(d[2]), 0.125, 4.0]] * 2)
    table = pc._table([pc.plane_surface(frame), pc.plane_surface(pc.curvilinear_frame(od, pos))])
    prop = abi.Propagation(params, np.array([frame, frame]),
                           np.array([[pc.PION_MASS, 1.0]] * 2, np.float32), [1000.0, 1000.0],
                           start_cov=np.tile(0.025 * np.eye(6).reshape(36), (2, 1)),
                           target=np.array([0, 1], np.int32))
    return table, prop


def is_approx(a, b, prec=1e-12):
    """Eigen's isApprox: ||a - b|| <= prec * min(||a||, ||b||)."""
    return np.linalg.norm(a - b) <= prec * min(np.linalg.norm(a), np.linalg.norm(b))


def check_jacobian_engine(prop, prec=1e-12):
    """`prec`: Eigen's double precision (1e-12); the mixed form keeps its
    covariance in float (relative rounding 6e-8)."""
    assert (prop.status == 0).all()
    assert (prop.steps == 0).all() and (np.abs(prop.path_length) == 0).all()
    c0 = 0.025 * np.eye(6)
    same = prop.end_cov[:, 0].reshape(6, 6)
    rotated = prop.end_cov[:, 1].reshape(6, 6)
    # a) no transport onto the same surface keeps the covariance
    assert is_approx(same, c0, prec), same
    np.testing.assert_allclose(prop.jacobian[:, 0].reshape(6, 6), np.eye(6), atol=prec)
    # b) no transport but onto a rotated surface changes it
    assert not is_approx(rotated, c0, prec)


def test_jacobian_engine_identities(oracle):
    table, prop = jacobian_engine_case()
    oracle.propagate(pc.constant_field(2.0), table, prop, abi.default_options())
    check_jacobian_engine(prop)
