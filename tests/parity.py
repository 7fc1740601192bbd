"""Comparison of two Results (CUDA fitter vs oracle) with the stated
tolerances: integers and flags bit-exact; floating point within `rtol`
relative to max(|a|, |b|, natural scale of the entry). The natural scales:
sigma of the parameter (its covariance diagonal) for bound parameters,
sqrt(C_ii C_jj) for covariance entries, 1e-4 of the row's largest entry for
Jacobian entries, 1 for path lengths and chi2."""
import numpy as np

from acts_gb300 import abi


# floor of a Jacobian entry's relative comparison, as a fraction of the
# largest entry of its row
JAC_ROW_FLOOR = 1e-4


def _sig(cov):
    # per-state standard deviations from a [..., 36] covariance
    d = cov[..., [0, 7, 14, 21, 28, 35]]
    return np.sqrt(np.abs(d))


def compare(gpu, ora, rtol=1e-9, fields=("predicted", "filtered", "smoothed"), exclude=None):
    """Returns a dict of max normalised errors and mismatch counts. `exclude`:
    tracks left out of the floating-point comparison (statuses still
    compared)."""
    rep = {}
    st_g, st_o = gpu.status, ora.status
    rep["status_mismatch"] = int(np.sum(st_g != st_o))
    ok = (st_g == 0) & (st_o == 0)
    if exclude is not None:
        ok &= ~exclude
    rep["n_ok"] = int(ok.sum())
    for name in ("n_states", "n_measurements", "n_holes", "n_outliers", "ndf"):
        rep[name + "_mismatch"] = int(np.sum(getattr(gpu, name)[ok] != getattr(ora, name)[ok]))
    ms = gpu.max_states
    valid = (np.arange(ms)[None, :] < gpu.n_states[:, None]) & ok[:, None]
    rep["flags_mismatch"] = int(np.sum((gpu.view("state_flags") != ora.view("state_flags")) & valid))
    rep["surface_mismatch"] = int(np.sum((gpu.view("state_surface") != ora.view("state_surface")) & valid))

    def rel(a, b, floor):
        # (0 against 0 with a zero floor counts as equal)
        return np.abs(a - b) / np.maximum(np.maximum(np.maximum(np.abs(a), np.abs(b)), floor),
                                          1e-300)

    m = valid
    for name in ("state_path_length", "state_chi2"):
        a, b = gpu.view(name)[m], ora.view(name)[m]
        rep[name] = float(rel(a, b, 1.0).max()) if a.size else 0.0
    rep["chi2_sum"] = float(rel(gpu.chi2_sum[ok], ora.chi2_sum[ok], 1.0).max()) if ok.any() else 0.0
    for name in fields:
        pa, pb = gpu.view(name), ora.view(name)
        ca, cb = gpu.view(name + "_cov"), ora.view(name + "_cov")
        if pa is None or pb is None:
            continue
        # states without such parameters (reverse filtering: no smoothed
        # parameters but on the first and last measurement state) hold NaN
        # on both sides: the NaN positions must agree, the rest is compared
        for x, y, key in ((pa, pb, name), (ca, cb, name + "_cov")):
            rep[key + "_nan_mismatch"] = int(np.sum((np.isnan(x) != np.isnan(y))[m]))
        pa, pb = np.nan_to_num(pa, nan=0.0), np.nan_to_num(pb, nan=0.0)
        ca, cb = np.nan_to_num(ca, nan=0.0), np.nan_to_num(cb, nan=0.0)
        sig = _sig(cb)
        rp = rel(pa, pb, sig)[m]
        rep[name] = float(rp.max()) if rp.size else 0.0
        scale = np.sqrt(np.abs(cb[..., [0, 7, 14, 21, 28, 35]]))
        floor = (scale[..., :, None] * scale[..., None, :]).reshape(scale.shape[:-1] + (36,))
        rc = rel(ca, cb, floor)[m]
        rep[name + "_cov"] = float(rc.max()) if rc.size else 0.0
    ja, jb = gpu.view("jacobian"), ora.view("jacobian")
    if ja is not None and jb is not None:
        jr = jb.reshape(jb.shape[:-1] + (6, 6))
        # an entry four orders of magnitude below its row's largest is the
        # rounding residue of cancelling products (e.g. the time row's phi and
        # theta derivatives of a 100 GeV track sit 1e-14 from zero in any two
        # FP64 evaluations): those entries are compared at that scale
        rowmax = np.abs(jr).max(axis=-1, keepdims=True) * JAC_ROW_FLOOR
        floor = np.broadcast_to(rowmax, jr.shape).reshape(jb.shape)
        r = rel(ja, jb, floor)[m]
        rep["jacobian"] = float(r.max()) if r.size else 0.0
    ta, tb = getattr(gpu, "track_params", None), getattr(ora, "track_params", None)
    if ta is not None and tb is not None and ok.any():
        # parameters and covariance at the reference surface
        pa, pb = gpu.track("track_params")[ok], ora.track("track_params")[ok]
        ca, cb = gpu.track("track_cov")[ok], ora.track("track_cov")[ok]
        sig = _sig(cb)
        rep["track_params"] = float(rel(pa, pb, sig).max())
        floor = (sig[:, :, None] * sig[:, None, :]).reshape(-1, 36)
        rep["track_cov"] = float(rel(ca, cb, floor).max())
    return rep


def assert_parity(rep, rtol=1e-9):
    for k, v in rep.items():
        if k.endswith("_mismatch"):
            assert v == 0, (k, rep)
    for k in ("state_path_length", "state_chi2", "chi2_sum", "predicted", "predicted_cov",
              "filtered", "filtered_cov", "smoothed", "smoothed_cov", "jacobian", "track_params",
              "track_cov"):
        if k in rep:
            assert rep[k] <= rtol, (k, rep[k], rep)
