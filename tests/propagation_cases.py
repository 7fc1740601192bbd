"""The reference's propagation property tests, restated for any backend of
ck_propagate's interface (the oracle on the CPU, the CUDA stepper in either
precision form).

Datasets and tolerances follow Tests/IntegrationTests/PropagationDatasets.hpp
and PropagationEigenConstant.cpp:37-42 (constant field along z):
  phi    -180..180 deg in 45 deg steps (phiWithoutAmbiguity: -135..135)
  theta  45, 90, 135, 2, 10, 30, 150, 170, 178 deg (thetaWithoutBeam)
  p      0.5, 1, 10, 100 GeV;  q +-1;  path length 10, 100 mm;  B 0.5, 2, 4 T
  epsPos 1 um, epsTime 1 um, epsDir 0.125 mrad, epsMom 1 eV, epsCov 0.025
  (0.125 towards straws).
The checks restate PropagationTests.hpp:
  forward-backward  runForwardBackwardTest (:400-416)
  to surface        runToSurfaceTest (:424-460) with the plane, z-cylinder
                    and z-straw builders (:288-330)
  covariance        runForwardComparisonTest / runToSurfaceComparisonTest
                    (:465-540): the transported covariance against one
                    transported with a numerical Jacobian (the reference's
                    RiddersStepper; here central differences of the same
                    propagator with Richardson extrapolation) under
                    checkCloseCovariance (FloatComparisons.hpp:270-300).
"""
import ctypes as C
import itertools

import numpy as np

from acts_gb300 import abi

DEG = np.pi / 180.0
PHI = np.arange(-180, 181, 45) * DEG
PHI_NO_AMBIGUITY = np.arange(-135, 136, 45) * DEG
THETA = np.array([45, 90, 135, 2, 10, 30, 150, 170, 178]) * DEG
MOMENTA = np.array([0.5, 1.0, 10.0, 100.0])
CHARGES = np.array([1.0, -1.0])
PATHS = np.array([10.0, 100.0])
FIELDS_T = np.array([0.5, 2.0, 4.0])

EPS_POS = 1e-3
EPS_TIME = 1e-3
EPS_DIR = 0.125e-3
EPS_MOM = 1e-9
EPS_COV = 0.025
EPS_COV_STRAW = 0.125

PION_MASS = 0.13957039


def cases(phis=PHI):
    """(phi, theta, p, q, s) of the dataset product for one field value."""
    return np.array(list(itertools.product(phis, THETA, MOMENTA, CHARGES, PATHS)))


def curvilinear_frame(direction, position):
    """createCurvilinearUnitVectors (UnitVectors.hpp:94-150) as a ck_batch_in
    plane frame (rotation row-major with the columns U, V, T; centre)."""
    d = np.asarray(direction, float)
    u = np.array([-d[1], d[0], 0.0])
    sc = np.hypot(u[0], u[1])
    if sc < 16 * np.finfo(float).eps:
        u = np.array([1.0, 0.0, 0.0])
    else:
        u[:2] /= sc
    v = np.cross(d, u)
    v /= np.linalg.norm(v)
    R = np.stack([u, v, d], axis=1)
    return np.concatenate([R.reshape(9), np.asarray(position, float)])


def start_covariance():
    """makeParametersCurvilinearWithCovariance (PropagationTests.hpp:165-190):
    standard deviations 15 um, 80 um, 20 mrad, 30 mrad, 1/(10 GeV), 20 ps
    (in mm: c = 1) and its correlations. The reference assigns the
    (phi, q/p) and (theta, q/p) correlations to one triangle only (the same
    entry twice); a covariance is symmetric, and the packed covariance of the
    fitter holds one triangle, so both triangles carry them here."""
    sd = np.array([15e-3, 80e-3, 20e-3, 30e-3, 0.1, 20 * 0.299792458])
    corr = np.eye(6)
    for (i, j), v in {(0, 1): 0.125, (0, 2): 0.25, (1, 3): -0.25, (5, 4): 0.125, (2, 3): -0.25,
                      (2, 4): -0.125, (3, 4): 0.5}.items():
        corr[i, j] = corr[j, i] = v
    return np.diag(sd) @ corr @ np.diag(sd)


def initial_states(cs, with_cov=False):
    """Curvilinear parameters at the origin (makeParametersCurvilinear,
    PropagationTests.hpp:147-160): params, frames, particle, cov."""
    n = len(cs)
    params = np.zeros((n, 6))
    frames = np.zeros((n, 12))
    for i, (phi, theta, p, q, s) in enumerate(cs):
        params[i] = [0.0, 0.0, phi, theta, q / p, 0.0]
        d = np.array([np.cos(phi) * np.sin(theta), np.sin(phi) * np.sin(theta), np.cos(theta)])
        frames[i] = curvilinear_frame(d, np.zeros(3))
    particle = np.tile(np.array([PION_MASS, 1.0], np.float32), (n, 1))
    cov = np.tile(start_covariance().reshape(36), (n, 1)) if with_cov else None
    return params, frames, particle, cov


def direction(params):
    phi, theta = params[..., 2], params[..., 3]
    return np.stack([np.cos(phi) * np.sin(theta), np.sin(phi) * np.sin(theta), np.cos(theta)], -1)


def surface_position(surf, b):
    """Surface::localToGlobal of bound parameters b on a ck_surface."""
    R = np.array(surf.rotation).reshape(3, 3)
    c = np.array(surf.center)
    if surf.type == abi.SURFACE_PLANE:
        return R @ np.array([b[0], b[1], 0.0]) + c
    if surf.type == abi.SURFACE_CYLINDER:
        r = surf.radius
        a = b[0] / r
        return R @ np.array([r * np.cos(a), r * np.sin(a), b[1]]) + c
    # LineSurface::localToGlobal (LineSurface.cpp:57-68)
    d = direction(b)
    radial = np.cross(R[:, 2], d)
    return R @ np.array([0.0, 0.0, b[1]]) + c + b[0] * radial / np.linalg.norm(radial)


def plane_surface(frame12):
    s = abi.ck_surface()
    s.type = abi.SURFACE_PLANE
    for i in range(9):
        s.rotation[i] = frame12[i]
    for i in range(3):
        s.center[i] = frame12[9 + i]
    s.split_factor = 1.0
    return s


def z_cylinder(position):
    s = abi.ck_surface()
    s.type = abi.SURFACE_CYLINDER
    for i in range(3):
        s.rotation[4 * i] = 1.0
    s.radius = float(np.hypot(position[0], position[1]))
    s.split_factor = 1.0
    return s


def z_straw(position):
    s = abi.ck_surface()
    s.type = abi.SURFACE_LINE
    for i in range(3):
        s.rotation[4 * i] = 1.0
        s.center[i] = position[i]
    s.split_factor = 1.0
    return s


def constant_field(tesla):
    f = abi.ck_field()
    f.kind = abi.FIELD_CONSTANT
    f.constant_tesla[2] = tesla
    return f


def check_close_covariance(val, ref, tol):
    """checkCloseCovariance: |val - ref| < tol * sqrt(ref_ii ref_jj) for
    every entry; returns the worst ratio (< 1 passes)."""
    val = val.reshape(-1, 6, 6)
    ref = ref.reshape(-1, 6, 6)
    d = np.sqrt(np.abs(np.einsum("nii->ni", ref)))
    scale = d[:, :, None] * d[:, None, :] * tol
    return (np.abs(val - ref) / np.maximum(scale, 1e-300)).max(axis=(1, 2))


# numerical Jacobian: step sizes per bound parameter (h and h/2, Richardson)
NUM_STEPS = np.array([2e-3, 2e-3, 2e-5, 2e-5, 0.0, 2e-3])
NUM_QOP_REL = 2e-5


def perturbations(params, frames, particle, target, limit):
    """The start states of a numerical Jacobian: for every track and bound
    parameter j, +-h_j and +-h_j/2. Returns the stacked arrays and the steps
    [n, 6]."""
    n = len(params)
    h = np.tile(NUM_STEPS, (n, 1))
    h[:, 4] = NUM_QOP_REL * np.abs(params[:, 4])
    rows = []
    for scale in (1.0, 0.5):
        for j in range(6):
            for sign in (1.0, -1.0):
                p = params.copy()
                p[:, j] += sign * scale * h[:, j]
                rows.append(p)
    k = len(rows)
    P = np.concatenate(rows)
    return (P, np.tile(frames, (k, 1)), np.tile(particle, (k, 1)),
            None if target is None else np.tile(target, k), np.tile(limit, k), h)


def numerical_jacobian(end, n, h):
    """Richardson-extrapolated central differences from the stacked end
    parameters [6, 24 n] of `perturbations` (phi differences wrapped)."""
    E = end.T.reshape(2, 6, 2, n, 6)  # scale, param j, sign, track, out
    D = E[:, :, 0] - E[:, :, 1]
    D[..., 2] = (D[..., 2] + np.pi) % (2 * np.pi) - np.pi
    D1 = D[0] / (2 * h.T[:, :, None])
    D2 = D[1] / (h.T[:, :, None])
    J = (4 * D2 - D1) / 3  # [j, track, out]
    return np.transpose(J, (1, 2, 0))  # [track, out, j]


# ------------------------------------------------------------------ backends
class OracleBackend:
    """The oracle's propagation restatement (FP64)."""

    def __init__(self, n_threads=None):
        from oracle import kforacle

        self.k = kforacle
        self.n_threads = n_threads or kforacle.hardware_threads()

    def propagate(self, field, table, prop, options):
        self.k.propagate(table, field, options, prop, self.n_threads)
        return prop


class CudaBackend:
    """ck_propagate on the GPU in a precision form; one handle per surface
    table and field."""

    def __init__(self, precision=abi.PRECISION_FP64):
        self.precision = precision

    def propagate(self, field, table, prop, options):
        from acts_gb300.fitter import CudaKalman

        if table is None:
            table, n = (abi.ck_surface * 1)(), 0
        else:
            n = len(table)
        options.precision = self.precision
        fit = CudaKalman(table, n, field)
        try:
            fit.propagate(options, prop)
        finally:
            fit.close()
        return prop


def _table(surfs):
    arr = (abi.ck_surface * len(surfs))()
    for i, s in enumerate(surfs):
        arr[i] = s
    return arr


def _free(backend, field, cs, with_cov, options):
    params, frames, particle, cov = initial_states(cs, with_cov)
    prop = abi.Propagation(params, frames, particle, cs[:, 4], cov)
    return backend.propagate(field, None, prop, options), particle


def _check_consistency(rep, pos, ref_pos, t, ref_t, b, ref_b):
    """checkParametersConsistency's derived quantities: worst |difference| /
    tolerance per kind (< 1 passes)."""
    d = direction(b)
    rd = direction(ref_b)
    rep["pos"] = max(rep.get("pos", 0.0), float(np.abs(pos - ref_pos).max() / EPS_POS))
    rep["time"] = max(rep.get("time", 0.0), float(np.abs(t - ref_t).max() / EPS_TIME))
    dphi = np.abs((b[:, 2] - ref_b[:, 2] + np.pi) % (2 * np.pi) - np.pi)
    ddir = max(float(dphi.max()), float(np.abs(b[:, 3] - ref_b[:, 3]).max()),
               float(np.abs(d - rd).max()))
    rep["dir"] = max(rep.get("dir", 0.0), ddir / EPS_DIR)
    dmom = np.abs(1.0 / np.abs(b[:, 4]) - 1.0 / np.abs(ref_b[:, 4])).max()
    rep["mom"] = max(rep.get("mom", 0.0), float(dmom / EPS_MOM))
    assert np.array_equal(np.sign(b[:, 4]), np.sign(ref_b[:, 4])), "charge differs"
    return rep


def forward_backward(backend, tesla, options):
    """runForwardBackwardTest on the whole dataset for one field value."""
    cs = cases()
    field = constant_field(tesla)
    fwd, particle = _free(backend, field, cs, False, options)
    assert (fwd.status == 0).all(), np.unique(fwd.status, return_counts=True)
    rep = {"fwd_path": float(np.abs(fwd.path_length - cs[:, 4]).max() / EPS_POS)}
    bwd = abi.Propagation(fwd.end_params.T.copy(), fwd.end_frames.copy(), particle, -cs[:, 4])
    backend.propagate(field, None, bwd, options)
    assert (bwd.status == 0).all(), np.unique(bwd.status, return_counts=True)
    rep["bwd_path"] = float(np.abs(bwd.path_length + cs[:, 4]).max() / EPS_POS)
    init, _, _, _ = initial_states(cs)
    b = bwd.end_params.T
    return _check_consistency(rep, bwd.end_frames[:, 9:], np.zeros((len(cs), 3)), b[:, 5],
                              init[:, 5], b, init)


BUILDERS = {"plane": lambda frame, pos: plane_surface(frame),
            "cylinder": lambda frame, pos: z_cylinder(pos),
            "straw": lambda frame, pos: z_straw(pos)}


def to_surface(backend, tesla, kind, options):
    """runToSurfaceTest with the plane / z-cylinder / z-straw builder."""
    cs = cases()
    field = constant_field(tesla)
    fwd, particle = _free(backend, field, cs, False, options)
    assert (fwd.status == 0).all()
    pos = fwd.end_frames[:, 9:]
    table = _table([BUILDERS[kind](fwd.end_frames[i], pos[i]) for i in range(len(cs))])
    params, frames, particle, _ = initial_states(cs)
    prop = abi.Propagation(params, frames, particle, 1.5 * cs[:, 4],
                           target=np.arange(len(cs), dtype=np.int32))
    backend.propagate(field, table, prop, options)
    assert (prop.status == 0).all(), np.unique(prop.status, return_counts=True)
    b = prop.end_params.T
    spos = np.array([surface_position(table[i], b[i]) for i in range(len(cs))])
    rep = {"path": float(np.abs(prop.path_length - cs[:, 4]).max() / EPS_POS)}
    return _check_consistency(rep, spos, pos, b[:, 5], fwd.end_params[5], b, fwd.end_params.T)


def covariance(backend, tesla, kind, options):
    """runForwardComparisonTest (kind "curvilinear") or
    runToSurfaceComparisonTest: the analytic transported covariance against
    the numerically transported one; returns (worst ratio to epsCov, the
    analytic propagation, the numerical Jacobians)."""
    cs = cases(PHI_NO_AMBIGUITY if kind == "cylinder" else PHI)
    n = len(cs)
    field = constant_field(tesla)
    if kind == "curvilinear":
        nominal, particle = _free(backend, field, cs, True, options)
        assert (nominal.status == 0).all()
        table = _table([plane_surface(nominal.end_frames[i]) for i in range(n)])
    else:
        fwd, particle = _free(backend, field, cs, False, options)
        assert (fwd.status == 0).all()
        pos = fwd.end_frames[:, 9:]
        table = _table([BUILDERS[kind](fwd.end_frames[i], pos[i]) for i in range(n)])
        params, frames, particle, cov = initial_states(cs, True)
        nominal = abi.Propagation(params, frames, particle, 1.5 * cs[:, 4], cov,
                                  target=np.arange(n, dtype=np.int32))
        backend.propagate(field, table, nominal, options)
        assert (nominal.status == 0).all(), np.unique(nominal.status, return_counts=True)
    params, frames, particle, cov = initial_states(cs, True)
    P, Fr, Pa, T, L, h = perturbations(params, frames, particle, np.arange(n, dtype=np.int32),
                                       1.5 * cs[:, 4])
    pert = abi.Propagation(P, Fr, Pa, L, target=T)
    backend.propagate(field, table, pert, options)
    assert (pert.status == 0).all(), np.unique(pert.status, return_counts=True)
    J = numerical_jacobian(pert.end_params, n, h)
    C0 = start_covariance()
    cov_num = np.einsum("nij,jk,nlk->nil", J, C0, J)
    cov_ana = nominal.end_cov.T.reshape(n, 6, 6)
    tol = EPS_COV_STRAW if kind == "straw" else EPS_COV
    worst = check_close_covariance(cov_ana, cov_num, tol)
    return float(worst.max()), nominal, J
