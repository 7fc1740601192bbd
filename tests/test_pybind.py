"""The pybind11 module acts_gb300._acts_gb300_ext (makeKalmanFitterFunction
of Python/Examples/src/TrackFitting.cpp:50-67 over the C ABI). Built only
where pybind11 is importable; skipped elsewhere.

CPU: the factory carries the reference's keyword names and defaults, and
without a GPU it fails loudly (no CPU fallback). GPU: a fit through the
module equals the ctypes path's fit of the same batch with the same options,
bit for bit."""
import inspect

import numpy as np
import pytest

from acts_gb300 import abi, generate

ext = pytest.importorskip("acts_gb300._acts_gb300_ext")

KEYWORDS = ["trackingGeometry", "magneticField", "multipleScattering", "energyLoss",
            "reverseFilteringMomThreshold", "reverseFilteringCovarianceScaling",
            "freeToBoundCorrection", "chi2Cut", "useJosephFormulation", "level"]


def test_factory_signature():
    doc = ext.makeKalmanFitterFunction.__doc__
    sig = doc[doc.index("(") + 1:doc.index(") ->")]
    names = [p.split(":")[0].strip() for p in sig.split(", ")]
    assert names[:len(KEYWORDS)] == KEYWORDS
    assert "chi2Cut: typing.SupportsFloat" in sig or "chi2Cut: float" in sig
    assert "reverseFilteringCovarianceScaling" in sig and "= 100.0" in sig
    assert hasattr(ext, "TrackFitterFunction")


def test_bad_buffers_raise():
    det = generate.Detector(abi.CKG_BARREL)
    with pytest.raises(ValueError):
        ext.makeKalmanFitterFunction(np.zeros(3, np.uint8), det.field)
    with pytest.raises(ValueError):
        ext.makeKalmanFitterFunction(det.surfaces, np.zeros(3, np.uint8))


def test_no_gpu_fails_loudly():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    det = generate.Detector(abi.CKG_BARREL)
    with pytest.raises(RuntimeError, match="ck_create"):
        ext.makeKalmanFitterFunction(det.surfaces, det.field)


def _args(b):
    return (b.seq_offsets, b.seq_surfaces, b.meas_offsets, b.meas_surfaces, b.meas_values,
            b.meas_cov, b.start_params, b.start_cov, b.start_frames, b.particle,
            b.particle_pdg, b.meas_subspace)


@pytest.mark.gpu
@pytest.mark.parametrize("preset", [abi.CKG_BARREL, abi.CKG_STRIPS])
def test_fit_equals_ctypes_path(preset):
    from acts_gb300.fitter import CudaKalman, KalmanFitterOptions

    det = generate.Detector(preset, perigee=True)
    b = generate.generate(det, 200, seed=21)
    fn = ext.makeKalmanFitterFunction(det.surfaces, det.field, chi2Cut=50.0,
                                      reverseFilteringMomThreshold=0.0)
    comps = abi.OUT_ALL | abi.OUT_PACKED_COV | abi.OUT_REFERENCE
    got = fn(*_args(b), max_states=24, components=comps, reference_surface=det.perigee)
    opts = KalmanFitterOptions(outlier_chi2_cut=50.0, smoother=abi.SMOOTHER_MBF,
                               reference_strategy=abi.EXTRAPOLATE_FIRST,
                               reference_surface=det.perigee)
    ck = CudaKalman.for_detector(det)
    want = ck.fit_batch(b, opts, max_states=24, components=comps)
    ck.close()
    for name in want.ARRAYS:
        w = getattr(want, name)
        if w is None:
            assert name not in got, name
            continue
        np.testing.assert_array_equal(got[name], w, err_msg=name)
    assert (got["status"] == abi.TRACK_OK).mean() > 0.9
