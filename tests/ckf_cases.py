"""Track-finding cases shared by the oracle and GPU tests.

cubic_telescope(): the reference's CKF unit-test setup
(Tests/UnitTests/Core/TrackFinding/CombinatorialKalmanFilterTests.cpp:84-105, 204-257
with Tests/CommonHelpers/src/CubicTrackingGeometry.cpp:28-104): six planes
normal to the x axis at x = -2, -1, 1 -+ 1 mm, 2 -+ 1 mm (the last four
rotated by +-0.026 rad about their normal), 0.5 mm of beryllium each; pixel
measurements (25 um, 50 um) on the first two, alternating 1D strips (loc0
100 um, loc1 150 um) on the others; three pions from x = -3 m (phi 0, -1, +1
deg; theta 90, 91, 89 deg; q/p +1, +1, -1 /GeV) whose measurements are the
straight-line intersections, smeared. The reference runs it with zero
field and its full Navigator, where the end of the world ends the search;
with the DirectNavigator of this path a target plane at x = +3 m ends it.
"""
import numpy as np

from acts_gb300 import abi
from propagation_cases import constant_field, curvilinear_frame

DEG = np.pi / 180.0
NS = 299.792458  # 1 ns in mm (the internal time unit)
PION = (0.13957039, 1.0)

LAYER_X = [-2000.0, -1000.0, 999.0, 1001.0, 1999.0, 2001.0]
LAYER_ANGLE = [0.0, 0.0, 0.026, -0.026, 0.026, -0.026]
# measured subspace and resolution per layer
LAYER_SUB = [abi.MEAS_LOC01, abi.MEAS_LOC01, abi.MEAS_LOC0, abi.MEAS_LOC1, abi.MEAS_LOC0,
             abi.MEAS_LOC1]
LAYER_SIGMA = [(0.025, 0.050), (0.025, 0.050), (0.100, 0.0), (0.150, 0.0), (0.100, 0.0),
               (0.150, 0.0)]

START = [((-3000.0, 0.0, 0.0, 1 * NS), 0.0, 90.0, 1.0),
         ((-3000.0, -15.0, -15.0, 2 * NS), -1.0, 91.0, 1.0),
         ((-3000.0, 15.0, 15.0, -1 * NS), 1.0, 89.0, -1.0)]


def _beryllium(s, thickness):
    """makeBeryllium(): X0 352.8 mm, L0 407 mm, Ar 9.012, Z 4, 1.848 g/cm3."""
    s.mat_thickness = thickness
    s.mat_x0 = 352.8
    s.mat_l0 = 407.0
    s.mat_ar = 9.012
    s.mat_z = 4.0
    s.mat_molar_rho = (1.848 / 9.012) / 1000.0
    s.mat_molar_electron_rho = s.mat_z * s.mat_molar_rho
    s.mat_mean_excitation = 16e-9 * 4.0 ** 0.9
    s.flags |= abi.SURF_MATERIAL


def _plane(x, angle):
    s = abi.ck_surface()
    s.type = abi.SURFACE_PLANE
    s.flags = abi.SURF_SENSITIVE
    # base rotation (local x = global z, local y = global y, normal = -x),
    # then the stereo angle about the normal
    ca, sa = np.cos(angle), np.sin(angle)
    lx = np.array([0.0, sa, ca])
    ly = np.array([0.0, ca, -sa])
    n = np.array([-1.0, 0.0, 0.0])
    R = np.stack([lx, ly, n], axis=1)
    for i in range(9):
        s.rotation[i] = R.reshape(9)[i]
    s.center[0] = x
    s.half_x = s.half_y = 500.0
    s.split_factor = 1.0
    _beryllium(s, 0.5)
    return s


class CubicTelescope:
    """Surface table (six layers, then the target plane at x = +3 m) and a
    constant field along z."""

    def __init__(self, bz_tesla=0.0):
        surfs = [_plane(x, a) for x, a in zip(LAYER_X, LAYER_ANGLE)]
        t = abi.ck_surface()
        t.type = abi.SURFACE_PLANE
        fr = curvilinear_frame([1.0, 0.0, 0.0], [3000.0, 0.0, 0.0])
        for i in range(9):
            t.rotation[i] = fr[i]
        for i in range(3):
            t.center[i] = fr[9 + i]
        t.split_factor = 1.0
        surfs.append(t)
        self.surfaces = (abi.ck_surface * len(surfs))(*surfs)
        self.n_surfaces = len(surfs)
        self.target = len(surfs) - 1
        self.field = constant_field(bz_tesla)
        self.preset = -1


def _rotation(s):
    return np.array(list(s.rotation)).reshape(3, 3)


def cubic_event(seed=421235, n_copies=1):
    """The three particles (repeated n_copies times, each copy with its own
    smearing) as one track-finding event on CubicTelescope. Returns
    (detector, TrackFinding, truth track of each measurement)."""
    det = CubicTelescope()
    rng = np.random.default_rng(seed)
    starts = START * n_copies
    n = len(starts)
    sigma = np.array([0.1, 0.1, 2 * DEG, 2 * DEG, 1 / 100.0, 25 * NS])
    cov = np.diag(sigma ** 2).reshape(36)
    params, frames, covs = [], [], []
    meas = [[] for _ in LAYER_X]  # per layer: (track, values, cov, sub)
    for k, (pos4, phi, theta, qop) in enumerate(starts):
        phi, theta = phi * DEG, theta * DEG
        d = np.array([np.cos(phi) * np.sin(theta), np.sin(phi) * np.sin(theta), np.cos(theta)])
        p0 = np.array(pos4[:3])
        frames.append(curvilinear_frame(d, p0))
        params.append([0.0, 0.0, phi, theta, qop, pos4[3]])
        covs.append(cov)
        for li, x in enumerate(LAYER_X):
            s = det.surfaces[li]
            R = _rotation(s)
            c = np.array(list(s.center))
            nrm = R[:, 2]
            t = np.dot(c - p0, nrm) / np.dot(d, nrm)
            loc = R.T @ (p0 + t * d - c)
            s0, s1 = LAYER_SIGMA[li]
            sub = LAYER_SUB[li]
            if sub == abi.MEAS_LOC01:
                v = [loc[0] + s0 * rng.standard_normal(), loc[1] + s1 * rng.standard_normal()]
                V = [s0 * s0, 0.0, 0.0, s1 * s1]
            elif sub == abi.MEAS_LOC0:
                v = [loc[0] + s0 * rng.standard_normal(), 0.0]
                V = [s0 * s0, 0.0, 0.0, 0.0]
            else:
                v = [loc[1] + s0 * rng.standard_normal(), 0.0]
                V = [s0 * s0, 0.0, 0.0, 0.0]
            meas[li].append((k, v, V, sub))
    offs = [0]
    vals, mcov, subs, truth = [], [], [], []
    for li in range(det.n_surfaces):
        rows = meas[li] if li < len(LAYER_X) else []
        for k, v, V, sub in rows:
            truth.append(k)
            vals.append(v)
            mcov.append(V)
            subs.append(sub)
        offs.append(len(vals))
    nseq = len(LAYER_X)
    tf = abi.TrackFinding(np.arange(n + 1) * nseq, np.tile(np.arange(nseq), n), params, covs,
                          frames, [PION] * n, offs, vals, mcov, meas_subspace=subs,
                          max_states=32, max_tracks=8)
    return det, tf, np.array(truth)


class WithTarget:
    """A preset detector's table with a passive target cylinder appended
    (radius 1100 mm, inside the grid field map): the search's branches end
    there instead of running on until the loop-protection path limit, which
    on the grid field leaves the map (a field error of the whole seed)."""

    def __init__(self, det, radius=1100.0):
        t = abi.ck_surface()
        t.type = abi.SURFACE_CYLINDER
        for i in range(3):
            t.rotation[4 * i] = 1.0
        t.radius = radius
        t.half_length_z = 3000.0
        t.split_factor = 1.0
        surfs = list(det.surfaces) + [t]
        self.surfaces = (abi.ck_surface * len(surfs))(*surfs)
        self.n_surfaces = len(surfs)
        self.target = len(surfs) - 1
        self.field = det.field
        self.preset = det.preset
        self._det = det  # owns the field map values

