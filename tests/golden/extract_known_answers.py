"""Extracts the known-answer constants of the reference's own unit tests into
tests/golden/reference_known_answers.json.

Run with the path of a checkout of the reference sources as its one
argument. The JSON is committed, so tests never read the
reference at run time. Sources parsed (paths relative to the acts repo):
  Tests/UnitTests/Core/TrackFitting/GainMatrixUpdaterTests.cpp  (Update, UpdateFailed)
  Tests/UnitTests/Core/TrackFitting/GainMatrixSmootherTests.cpp (Smooth)
  Tests/UnitTests/Core/TrackFitting/MbfSmootherTests.cpp        (Smooth)
  Tests/UnitTests/Core/Surfaces/LineSurfaceTests.cpp            (globalToLocal, intersect)
  Tests/UnitTests/Core/EventData/CorrectedTransformFreeToBoundTests.cpp
  Tests/UnitTests/Core/Material/InteractionsTests.cpp           (silicon Bethe, Landau)
  Tests/CommonHelpers/include/ActsTests/CommonHelpers/PredefinedMaterials.hpp (makeSilicon)
"""
import json
import math
import os
import re
import sys

UNITS = {"_GeV": 1.0, "_MeV": 1e-3, "_keV": 1e-6, "_eV": 1e-9, "_TeV": 1e3, "_mm": 1.0,
         "_cm": 10.0, "_um": 1e-3, "_m": 1e3, "_e": 1.0, "_mol": 1.0, "_cm3": 1000.0,
         "_mm2": 1.0, "_g": 1.0 / 1.782662e-24, "_cm2": 100.0,
         "_ns": 299.792458}  # ACTS time unit: mm (1 s = c * 1 s in mm)


def num(expr):
    """Evaluates a C++ numeric expression of the tests (literals, units, pi)."""
    e = expr.strip().rstrip(";")
    e = e.replace("std::numbers::pi", repr(math.pi))
    for u in sorted(UNITS, key=len, reverse=True):
        e = re.sub(r"(\d(?:[\d.eE+-]*\d)?\.?)" + re.escape(u) + r"\b", r"(\1*%r)" % UNITS[u], e)
    e = re.sub(r"(\d)\.(?!\d)", r"\1.0", e)
    return float(eval(e, {"__builtins__": {}}, {}))


def values(stream_text):
    """Numbers of an Eigen comma initialiser 'x << a, b, c;'."""
    rhs = stream_text.split("<<", 1)[1].rstrip(";")
    return [num(v) for v in rhs.split(",")]


def find_after(text, anchor, pattern, start=0):
    i = text.index(anchor, start)
    m = re.compile(pattern, re.S).search(text, i)
    return m, m.end()


def updater(src):
    t = open(os.path.join(src, "Tests/UnitTests/Core/TrackFitting/GainMatrixUpdaterTests.cpp")).read()
    case = t[t.index("BOOST_AUTO_TEST_CASE(Update)"):t.index("BOOST_AUTO_TEST_CASE(UpdateFailed)")]
    mp = re.search(r"Vector2 measPar\(([^)]*)\)", case).group(1).split(",")
    mc = re.search(r"Vector2\(([^)]*)\)\.asDiagonal", case).group(1).split(",")
    tp = values(re.search(r"trkPar <<[^;]*;", case).group(0))
    tc = values(re.search(r"trkCov\.diagonal\(\) <<[^;]*;", case).group(0))
    ep = values(re.search(r"expPar <<[^;]*;", case).group(0))
    ec = values(re.search(r"expCov\.diagonal\(\) <<[^;]*;", case).group(0))
    chi = re.search(r"CHECK_CLOSE_ABS\(ts\.chi2\(\),\s*([0-9.eE+-]+),\s*([0-9.eE+-]+)\)", case)
    tol = re.search(r"tol\s*=\s*([0-9.eE+-]+)", t)
    fcase = t[t.index("BOOST_AUTO_TEST_CASE(UpdateFailed)"):]
    return {
        "source": "Tests/UnitTests/Core/TrackFitting/GainMatrixUpdaterTests.cpp",
        "meas": [num(x) for x in mp], "meas_cov_diag": [num(x) for x in mc],
        "pred": tp, "pred_cov_diag": tc, "exp_filtered": ep, "exp_filtered_cov_diag": ec,
        "exp_chi2": float(chi.group(1)), "chi2_tol": float(chi.group(2)),
        "tol": float(tol.group(1)) if tol else 1e-6,
        "failed_case_pred_cov_zero": "CovarianceMatrix::Zero()" in fcase,
        "failed_case_meas_cov_zero": "SquareMatrix2::Zero()" in fcase,
    }


def smoother(src):
    t = open(os.path.join(src, "Tests/UnitTests/Core/TrackFitting/GainMatrixSmootherTests.cpp")).read()
    cov = values(re.search(r"covTrk\.diagonal\(\) <<[^;]*;", t).group(0))
    pars = [values(m.group(0)) for m in re.finditer(r"parValues <<[^;]*;", t)]
    exp_p = [values(m.group(0)) for m in re.finditer(r"expPars <<[^;]*;", t)]
    exp_c = values(re.search(r"expCov\.diagonal\(\) <<[^;]*;", t).group(0))
    paths = [num(m.group(1)) for m in re.finditer(r"pathLength\(\) = ([^;]*);", t)]
    tol = re.search(r"double tol = ([0-9.eE+-]+);", t)
    states = []
    for k in range(3):
        states.append({"predicted": pars[2 * k], "filtered": pars[2 * k + 1], "path": paths[k]})
    return {"source": "Tests/UnitTests/Core/TrackFitting/GainMatrixSmootherTests.cpp",
            "cov_diag": cov, "states": states, "exp_smoothed": exp_p, "exp_cov_diag": exp_c,
            "tol": float(tol.group(1))}


def mbf_smoother(src):
    t = open(os.path.join(src, "Tests/UnitTests/Core/TrackFitting/MbfSmootherTests.cpp")).read()
    cov = values(re.search(r"covTrk\.diagonal\(\) <<[^;]*;", t).group(0))
    pred = [values(m.group(0)) for m in re.finditer(r"ts\.predicted\(\) <<[^;]*;", t)]
    filt = [values(m.group(0)) for m in re.finditer(r"ts\.filtered\(\) <<[^;]*;", t)]
    cal = [values(m.group(0)) for m in re.finditer(r"ts\.calibrated<2>\(\) <<[^;]*;", t)]
    calc = [values(m.group(0)) for m in re.finditer(r"ts\.calibratedCovariance<2>\(\) <<[^;]*;", t)]
    paths = [num(m.group(1)) for m in re.finditer(r"pathLength\(\) = ([^;]*);", t)]
    exp_p = [values(m.group(0)) for m in re.finditer(r"expPars <<[^;]*;", t)]
    exp_c = values(re.search(r"expCov\.diagonal\(\) <<[^;]*;", t).group(0))
    tol = re.search(r"double tol = ([0-9.eE+-]+);", t)
    states = [{"predicted": pred[k], "filtered": filt[k], "calibrated": cal[k],
               "calibrated_cov": calc[k], "path": paths[k]} for k in range(3)]
    return {"source": "Tests/UnitTests/Core/TrackFitting/MbfSmootherTests.cpp",
            "cov_diag": cov, "states": states, "exp_smoothed": exp_p, "exp_cov_diag": exp_c,
            "tol": float(tol.group(1)), "jacobian": "identity",
            "projector": ["eBoundLoc0", "eBoundLoc1"], "flags": "measurement"}


def line_surface(src):
    t = open(os.path.join(src, "Tests/UnitTests/Core/Surfaces/LineSurfaceTests.cpp")).read()
    case = t[t.index("BOOST_AUTO_TEST_CASE(LineSurface_allNamedMethods_test)"):]
    vec = lambda pat: [num(x) for x in re.search(pat, case).group(1).split(",")]
    return {"source": "Tests/UnitTests/Core/Surfaces/LineSurfaceTests.cpp",
            "center": vec(r"Translation3 translation\{([^}]*)\}"),
            "g2l_position": vec(r"Vector3 gpos\{([^}]*)\}"),
            "g2l_momentum": vec(r"const Vector3 mom\{([^}]*)\}"),
            "g2l_expected": vec(r"const Vector2 expectedResult\{([^}]*)\}"),
            "intersect_direction": vec(r"const Vector3 direction\{([^}]*)\}"),
            "intersect_expected": vec(r"Vector3 expectedIntersection\(([^)]*)\)")}


def corrected_free_to_bound(src):
    t = open(os.path.join(src, "Tests/UnitTests/Core/EventData/CorrectedTransformFreeToBoundTests.cpp")).read()
    v = {}
    for name in ("loc0", "loc1", "phi", "theta", "qOverP", "t", "resLoc0", "resLoc1", "resPhi",
                 "resTheta", "resQOverP", "resTime"):
        v[name] = num(re.search(r"const auto %s = ([^;]*);" % name, t).group(1))
    v["distance"] = num(re.search(r"double distance = ([^;]*);", t).group(1))
    m = re.search(r"CHECK_CLOSE_REL\(eCorrectedBoundParams\[eBoundLoc1\], ([0-9.eE+-]+), eps\)", t)
    v["exp_loc1"] = float(m.group(1))
    m = re.search(r"std::pow\(([0-9.eE+-]+), 2\)", t)
    v["exp_loc0_sigma"] = float(m.group(1))
    v["eps"] = num(re.search(r"constexpr double eps = ([^;]*);", t).group(1))
    v["source"] = "Tests/UnitTests/Core/EventData/CorrectedTransformFreeToBoundTests.cpp"
    v["surface"] = "curvilinear plane at (distance, 0, 0), normal x"
    return v


def interactions(src):
    t = open(os.path.join(src, "Tests/UnitTests/Core/Material/InteractionsTests.cpp")).read()
    mom = re.search(r"static const double momentum\[\] = \{([^}]*)\}", t).group(1)
    loss = re.search(r"static const double energy_loss\[\] = \{([^}]*)\}", t).group(1)
    sil = t[t.index("BOOST_DATA_TEST_CASE(silicon_energy_loss"):]
    thick = re.search(r"const auto thickness = ([^;]*);", sil).group(1)
    mass = re.search(r"const auto m = ([^;]*);", sil).group(1)
    pct = re.search(r"loss, ([0-9.]+)\);", sil).group(1)
    lan = t[t.index("BOOST_AUTO_TEST_CASE(silicon_landau)"):]
    lthick = re.search(r"const auto thickness = ([^;]*);", lan).group(1)
    lmass = re.search(r"const float m = ([^;]*);", lan).group(1)
    lq = re.search(r"q / ([^;]*);", lan).group(1)
    de = re.search(r"BOOST_CHECK_CLOSE\(dE, ([0-9.]+), ([0-9.]+)\)", lan)
    fw = re.search(r"BOOST_CHECK_CLOSE\(fwhm, ([0-9.]+), ([0-9.]+)\)", lan)
    masses = re.search(r"static const double mass\[\] = \{([^}]*)\}", t).group(1)
    thicks = re.search(r"static const double valuesThickness\[\] = \{([^}]*)\}", t).group(1)
    return {
        "source": "Tests/UnitTests/Core/Material/InteractionsTests.cpp",
        "silicon_bethe": {"momentum": [num(x) for x in mom.split(",")],
                          "loss_MeV_cm2_per_g": [num(x) for x in loss.split(",")],
                          "thickness": num(thick), "mass": num(mass), "percent": float(pct)},
        "silicon_landau": {"thickness": num(lthick), "mass": num(lmass), "momentum": num(lq),
                           "dE_MeV": float(de.group(1)), "dE_percent": float(de.group(2)),
                           "fwhm_MeV": float(fw.group(1)), "fwhm_percent": float(fw.group(2))},
        "consistency": {"masses": [num(x) for x in masses.split(",")],
                        "thickness": [num(x) for x in thicks.split(",")]},
    }


def silicon(src):
    t = open(os.path.join(
        src, "Tests/CommonHelpers/include/ActsTests/CommonHelpers/PredefinedMaterials.hpp")).read()
    body = t[t.index("makeSilicon"):]
    m = re.search(r"fromMolarDensity\(([^,]*),([^,]*),([^,]*),([^,]*),\s*\(([^)]*)\)\s*\*\s*1_mol\s*/\s*1_cm3\)",
                  body)
    return {"source": "Tests/CommonHelpers/include/ActsTests/CommonHelpers/PredefinedMaterials.hpp",
            "X0": num(m.group(1)), "L0": num(m.group(2)), "Ar": num(m.group(3)),
            "Z": num(m.group(4)), "molar_rho": num(m.group(5)) / 1000.0}


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: extract_known_answers.py <path of the reference sources>")
    src = sys.argv[1]
    out = {"updater": updater(src), "smoother": smoother(src), "mbf_smoother": mbf_smoother(src),
           "line_surface": line_surface(src),
           "corrected_free_to_bound": corrected_free_to_bound(src),
           "interactions": interactions(src),
           "silicon": silicon(src)}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_known_answers.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(path)


if __name__ == "__main__":
    main()
