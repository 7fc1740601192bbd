"""ctypes binding of the CPU oracle (oracle/_build/libkforacle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU legs as the checker or the timed CPU baseline. The product
package acts_gb300 never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from acts_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libkforacle.so")

_lib = None


def lib():
    global _lib
    if _lib is None:
        subprocess.run(["make", "-s", "-C", HERE], check=True)
        L = C.CDLL(LIB)
        L.kfo_fit_batch.restype = C.c_double
        L.kfo_fit_batch.argtypes = [C.POINTER(abi.ck_options), C.c_int, C.POINTER(abi.ck_surface),
                                    C.POINTER(abi.ck_field), C.POINTER(abi.ck_batch_in),
                                    C.POINTER(abi.ck_batch_out), C.c_int, C.c_int, C.c_int,
                                    C.c_int]
        L.kfo_gain_matrix_update.restype = None
        L.kfo_gain_matrix_update.argtypes = ([C.c_int, C.c_int] + [abi.P_f64] * 4 + [abi.P_i32] +
                                             [abi.P_f64] * 3 + [abi.P_i32])
        L.kfo_gain_matrix_smooth.restype = None
        L.kfo_gain_matrix_smooth.argtypes = [C.c_int, C.c_int] + [abi.P_f64] * 7 + [abi.P_i32]
        L.kfo_mbf_smooth.restype = None
        L.kfo_mbf_smooth.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_uint32)] + [abi.P_f64] * 9
        L.kfo_line_global_to_local.restype = C.c_int
        L.kfo_line_global_to_local.argtypes = [abi.P_f64] * 5
        L.kfo_line_intersect.restype = C.c_int
        L.kfo_line_intersect.argtypes = [abi.P_f64] * 4 + [C.POINTER(C.c_double)]
        L.kfo_corrected_free_to_bound.restype = C.c_int
        L.kfo_corrected_free_to_bound.argtypes = [C.POINTER(abi.ck_surface)] + [abi.P_f64] * 4
        L.kfo_interaction.restype = C.c_float
        L.kfo_interaction.argtypes = [C.c_int] + [C.c_float] * 6 + [C.c_int] + [C.c_float] * 3
        L.kfo_material_effects.restype = None
        L.kfo_material_effects.argtypes = [C.POINTER(abi.ck_surface), C.c_float, abi.P_f64,
                                           C.c_double, C.c_float, C.c_float, C.c_int, C.c_int,
                                           C.c_int, abi.P_f64]
        L.kfo_field_lookup.restype = None
        L.kfo_field_lookup.argtypes = [C.POINTER(abi.ck_field), C.c_int, abi.P_f64, abi.P_f64,
                                       abi.P_i32]
        L.kfo_propagate.restype = None
        L.kfo_propagate.argtypes = [C.POINTER(abi.ck_options), C.c_int, C.POINTER(abi.ck_surface),
                                    C.POINTER(abi.ck_field), C.POINTER(abi.ck_propagate_in),
                                    C.POINTER(abi.ck_propagate_out), C.c_int]
        L.kfo_find_tracks.restype = None
        L.kfo_find_tracks.argtypes = [C.POINTER(abi.ck_options), C.c_int,
                                      C.POINTER(abi.ck_surface), C.POINTER(abi.ck_field),
                                      C.POINTER(abi.ck_ckf_options), C.POINTER(abi.ck_ckf_in),
                                      C.POINTER(abi.ck_ckf_out), C.c_int]
        L.kfo_logf_mismatch.restype = C.c_int
        L.kfo_logf_mismatch.argtypes = [C.c_int, abi.P_f32]
        L.kfo_hardware_threads.restype = C.c_int
        L.kfo_count_flops.restype = C.c_int
        L.kfo_count_flops.argtypes = [C.POINTER(abi.ck_options), C.c_int, C.POINTER(abi.ck_surface),
                                      C.POINTER(abi.ck_field), C.POINTER(abi.ck_batch_in), C.c_int,
                                      C.c_int, C.POINTER(C.c_uint64)]
        _lib = L
    return _lib


def fit_batch(detector, batch, options, results, n_threads=1, coast=None, first=0, count=-1):
    """Fits `batch` (acts_gb300.generate.Batch) into `results`
    (acts_gb300.results.Results). Returns the wall time in seconds."""
    bi = batch.as_batch_in()
    bo = results.as_batch_out()
    c = -1 if coast is None else (1 if coast else 0)
    return lib().kfo_fit_batch(C.byref(options), detector.n_surfaces, detector.surfaces,
                               C.byref(detector.field), C.byref(bi), C.byref(bo), n_threads,
                               c, first, count)


def time_batch(detector, batch, options, n_threads, first=0, count=-1):
    """Fits without writing results (CPU baseline timing)."""
    bi = batch.as_batch_in()
    return lib().kfo_fit_batch(C.byref(options), detector.n_surfaces, detector.surfaces,
                               C.byref(detector.field), C.byref(bi), None, n_threads, -1, first,
                               count)


def _v(x):
    return np.ascontiguousarray(x, np.float64)


def line_global_to_local(center, rotation, pos, direction):
    """LineSurface::globalToLocal: (ok, loc[2])."""
    loc = np.zeros(2)
    a = [_v(center), _v(rotation), _v(pos), _v(direction)]
    ok = lib().kfo_line_global_to_local(*[abi.ptr(x, C.c_double) for x in a],
                                        abi.ptr(loc, C.c_double))
    return bool(ok), loc


def corrected_free_to_bound(surface, free_params, free_cov):
    """CorrectedFreeToBoundTransformer: (ok, mean[6], cov[6, 6])."""
    mean = np.zeros(6)
    cov = np.zeros(36)
    ok = lib().kfo_corrected_free_to_bound(C.byref(surface), abi.ptr(_v(free_params), C.c_double),
                                           abi.ptr(_v(np.reshape(free_cov, 64)), C.c_double),
                                           abi.ptr(mean, C.c_double), abi.ptr(cov, C.c_double))
    return bool(ok), mean, cov.reshape(6, 6)


def line_intersect(center, rotation, pos, direction):
    """LineSurface::intersect: (status 0/1/2, path length)."""
    path = C.c_double()
    a = [_v(center), _v(rotation), _v(pos), _v(direction)]
    st = lib().kfo_line_intersect(*[abi.ptr(x, C.c_double) for x in a], C.byref(path))
    return st, path.value


def gain_matrix_update(pred, pred_cov, meas, meas_cov, joseph=False, subspace=None):
    n = pred.shape[0]
    f = np.zeros((n, 6))
    fc = np.zeros((n, 36))
    chi2 = np.zeros(n)
    st = np.zeros(n, np.int32)
    args = [np.ascontiguousarray(x, dtype=np.float64) for x in (pred, pred_cov, meas, meas_cov)]
    sub = None if subspace is None else np.ascontiguousarray(subspace, np.int32)
    lib().kfo_gain_matrix_update(n, int(joseph), *[abi.ptr(a, C.c_double) for a in args],
                                 abi.ptr(sub, C.c_int32),
                                 abi.ptr(f, C.c_double), abi.ptr(fc, C.c_double),
                                 abi.ptr(chi2, C.c_double), abi.ptr(st, C.c_int32))
    return f, fc.reshape(n, 6, 6), chi2, st


def mbf_smooth(flags, pred, pred_cov, filt, filt_cov, jac, meas, meas_cov):
    """MbfSmoother; arrays shaped [n_traj, n_states, ...]."""
    nt, ns = pred.shape[:2]
    s = np.zeros((nt, ns, 6))
    sc = np.zeros((nt, ns, 36))
    fl = np.ascontiguousarray(flags, np.uint32)
    args = [np.ascontiguousarray(x, dtype=np.float64)
            for x in (pred, pred_cov, filt, filt_cov, jac, meas, meas_cov)]
    lib().kfo_mbf_smooth(nt, ns, abi.ptr(fl, C.c_uint32), *[abi.ptr(a, C.c_double) for a in args],
                         abi.ptr(s, C.c_double), abi.ptr(sc, C.c_double))
    return s, sc.reshape(nt, ns, 6, 6)


def gain_matrix_smooth(pred, pred_cov, filt, filt_cov, jac):
    """Arrays shaped [n_traj, n_states, ...]."""
    nt, ns = pred.shape[:2]
    s = np.zeros((nt, ns, 6))
    sc = np.zeros((nt, ns, 36))
    st = np.zeros(nt, np.int32)
    args = [np.ascontiguousarray(x, dtype=np.float64) for x in (pred, pred_cov, filt, filt_cov, jac)]
    lib().kfo_gain_matrix_smooth(nt, ns, *[abi.ptr(a, C.c_double) for a in args],
                                 abi.ptr(s, C.c_double), abi.ptr(sc, C.c_double),
                                 abi.ptr(st, C.c_int32))
    return s, sc.reshape(nt, ns, 6, 6), st


def interaction(which, thickness, X0, L0, Ar, Z, molar_rho, pdg, m, qop, absq):
    return lib().kfo_interaction(which, thickness, X0, L0, Ar, Z, molar_rho, pdg, m, qop, absq)


def material_effects(surface, scale, direction, qop, mass, absq, pdg, ms=True, el=True):
    out = np.zeros(4)
    d = np.ascontiguousarray(direction, dtype=np.float64)
    lib().kfo_material_effects(C.byref(surface), scale, abi.ptr(d, C.c_double), qop, mass, absq,
                               pdg, int(ms), int(el), abi.ptr(out, C.c_double))
    return out


def field_lookup(field, pos):
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    out = np.zeros_like(pos)
    st = np.zeros(len(pos), np.int32)
    lib().kfo_field_lookup(C.byref(field), len(pos), abi.ptr(pos, C.c_double),
                           abi.ptr(out, C.c_double), abi.ptr(st, C.c_int32))
    return out, st


def propagate(surfaces, field, options, prop, n_threads=1):
    """The propagation restatement on an abi.Propagation (filled in place);
    `surfaces` a ctypes array of ck_surface (the target table)."""
    i, o = prop.as_in(), prop.as_out()
    n_surf = len(surfaces) if surfaces is not None else 0
    lib().kfo_propagate(C.byref(options), n_surf, surfaces, C.byref(field), C.byref(i),
                        C.byref(o), n_threads)
    return prop


def find_tracks(surfaces, field, options, ckf_options, tf, n_threads=1):
    """The track-finding restatement on an abi.TrackFinding (filled in place)."""
    i, o = tf.as_in(), tf.as_out()
    lib().kfo_find_tracks(C.byref(options), len(surfaces), surfaces, C.byref(field),
                          C.byref(ckf_options), C.byref(i), C.byref(o), n_threads)
    return tf


def logf_mismatch(x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    return lib().kfo_logf_mismatch(len(x), abi.ptr(x, C.c_float))


def hardware_threads():
    return lib().kfo_hardware_threads()


def count_flops(detector, batch, options, first=0, count=200):
    """Algorithmic FP64 operation counts of the reference formulation per
    fitted track: dict with add, mul, div, sqrt, trans, cmp, flops, tracks."""
    bi = batch.as_batch_in()
    out = (C.c_uint64 * 6)()
    ok = lib().kfo_count_flops(C.byref(options), detector.n_surfaces, detector.surfaces,
                               C.byref(detector.field), C.byref(bi), first, count, out)
    n = min(count, batch.n - first)
    keys = ("add", "mul", "div", "sqrt", "trans", "cmp")
    d = {k: out[i] / n for i, k in enumerate(keys)}
    d["flops"] = d["add"] + d["mul"] + d["div"] + d["sqrt"]
    d["tracks"] = n
    d["ok"] = ok
    return d
