"""FP64 parity with the oracle at the sizes of the benchmark configurations,
where the rare paths show up: cylinder-seam tracks (2e-4 of the barrel),
tracks that run into the step limit, tracks that coast out of the field map
after an outlier.

  telescope     1,000 muons, 10 planes, no material (the whole configuration)
  barrel        100,000 pions, 10 silicon cylinders, 2 T (the whole configuration)
  uneven events 50 events with Poisson(5,000) tracks each, 4-20 hits, holes,
                10-sigma outliers, chi2 cut 15, grid field map, as one batch

The tolerance is the parity definition of the plain form (tests/parity.py):
statuses, state counts, surfaces and flags bit-exact; parameters within 1e-9
of max(|x|, sigma_x); covariance entries within 1e-9 of
max(|C_ij|, sqrt(C_ii C_jj)); Jacobian entries within 1e-9 of
max(|J_ij|, 1e-4 max_k |J_ik|); path lengths and chi2 within 1e-9 of
max(|x|, 1). Broken fits — chi2/ndf above 1000, the barrel tracks whose
prediction and measurement straddle a cylinder's phi = +-pi seam and get a
residual of 2 pi R (2e-4 of the tracks) — are fitted identically up to the
filtered states, but their smoothed states come from gain matrices with
condition numbers up to 1e15, where the last bits of any two FP64
evaluations part: they keep every bit-exact check and are compared at 1e-6.
"""
import numpy as np
import pytest

from acts_gb300 import abi, generate
from acts_gb300.results import Results
from conftest import detector
from oracle import kforacle
from parity import assert_parity, compare

RTOL = 1e-9


RTOL_BROKEN = 1e-6
BROKEN_CHI2NDF = 1000.0


def _check(fit, det, b, opt, max_states, components, min_ok):
    n = b.n
    ora = Results(n, max_states, components)
    kforacle.fit_batch(det, b, opt, ora, n_threads=kforacle.hardware_threads())
    gpu = fit.fit_batch(b, opt, max_states=max_states, components=components)
    broken = (ora.status == 0) & (ora.chi2_sum > BROKEN_CHI2NDF * np.maximum(ora.ndf, 1))
    print("broken fits:", int(broken.sum()))
    assert broken.sum() <= 5e-4 * n
    rep = compare(gpu, ora, RTOL, exclude=broken)
    print(n, rep)
    assert rep["n_ok"] >= min_ok * n - broken.sum()
    assert_parity(rep, RTOL)
    if broken.any():
        rep = compare(gpu, ora, RTOL, exclude=~broken)
        print("broken", rep)
        assert_parity({k: v for k, v in rep.items() if k not in ("predicted", "filtered")},
                      RTOL_BROKEN)
        assert max(rep.get("predicted", 0.0), rep.get("filtered", 0.0)) <= RTOL
    return gpu, ora


@pytest.mark.gpu
def test_fp64_parity_telescope_1k(fitter_factory):
    det = detector(abi.CKG_TELESCOPE)
    b = generate.generate(det, 1000, seed=101)
    _check(fitter_factory(abi.CKG_TELESCOPE), det, b, abi.default_options(), 12, abi.OUT_ALL,
           0.99)


@pytest.mark.gpu
def test_fp64_parity_barrel_100k(fitter_factory):
    det = detector(abi.CKG_BARREL)
    b = generate.generate(det, 100000, seed=102)
    gpu, ora = _check(fitter_factory(abi.CKG_BARREL), det, b, abi.default_options(), 12,
                      abi.OUT_ALL, 0.99)
    # the rare outcomes are present and agree track by track
    fails = np.unique(ora.status[ora.status != 0], return_counts=True)
    print("failure statuses (oracle):", dict(zip(fails[0].tolist(), fails[1].tolist())))
    assert (ora.status != 0).sum() >= 1


@pytest.mark.gpu
def test_fp64_parity_uneven_events(fitter_factory):
    det = detector(abi.CKG_UNEVEN)
    sizes = generate.event_sizes(7, 50, mean=5000.0)
    n = int(sizes.sum())
    assert 240000 < n < 260000
    b = generate.generate(det, n, seed=103)
    opt = abi.default_options(outlier_chi2_cut=15.0)
    gpu, ora = _check(fitter_factory(abi.CKG_UNEVEN), det, b, opt, 22,
                      abi.OUT_SMOOTHED | abi.OUT_FILTERED, 0.5)
    st = np.unique(ora.status, return_counts=True)
    print("statuses (oracle):", dict(zip(st[0].tolist(), st[1].tolist())))
    # the coasting tracks that leave the map fail as in the reference
    assert (ora.status == abi.TRACK_FIELD_OUT_OF_BOUNDS).sum() > 0.2 * n
