"""Python binding of the synthetic event generator (include/ckgen.h).

make_workload() returns numpy arrays in the ck_batch_in layout plus the
truth needed for pulls; Batch.as_batch_in() wraps them for the C ABI.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .build import LIBDIR, build_generator

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(LIBDIR, "libckgen.so")
        if not os.path.exists(path):
            build_generator()
        L = C.CDLL(path)
        L.ckg_geometry.restype = C.c_int32
        L.ckg_geometry.argtypes = [C.c_int32, C.POINTER(abi.ck_surface), C.c_int32]
        L.ckg_field_values.restype = C.c_int64
        L.ckg_field_values.argtypes = [C.c_int32]
        L.ckg_field.restype = None
        L.ckg_field.argtypes = [C.c_int32, abi.P_f32, C.POINTER(abi.ck_field), C.c_int32]
        L.ckg_generate.restype = C.c_int64
        L.ckg_generate.argtypes = [C.c_int32, C.c_uint64, C.c_int64, C.c_int32,
                                   C.POINTER(abi.ck_surface), C.c_int32,
                                   C.POINTER(abi.ck_field), C.c_int32, C.POINTER(abi.ckg_out)]
        L.ckg_event_sizes.restype = None
        L.ckg_event_sizes.argtypes = [C.c_uint64, C.c_int32, C.c_double, C.c_int32, C.c_int32,
                                      abi.P_i32]
        _lib = L
    return _lib


class Detector:
    """Surface table and field of a preset (owns the field value buffer)."""

    def __init__(self, preset, n_threads=None, perigee=False):
        """perigee: append a PerigeeSurface (a line along global z through the
        origin) to the table, as the reference surface of the extrapolation;
        its index is `self.perigee`."""
        L = lib()
        self.preset = preset
        arr = (abi.ck_surface * 64)()
        n = L.ckg_geometry(preset, arr, 64)
        if n < 0:
            raise ValueError("unknown preset %r" % preset)
        self.perigee = -1
        if perigee:
            p = abi.ck_surface()
            p.type = abi.SURFACE_LINE
            for i in range(3):
                p.rotation[4 * i] = 1.0
            p.split_factor = 1.0
            arr[n] = p
            self.perigee = n
            n += 1
        self.surfaces = (abi.ck_surface * n)(*arr[:n])
        self.n_surfaces = n
        nv = L.ckg_field_values(preset)
        self.field_values = np.zeros(max(nv, 1), dtype=np.float32)
        self.field = abi.ck_field()
        L.ckg_field(preset, abi.ptr(self.field_values, C.c_float), C.byref(self.field),
                    n_threads or os.cpu_count() or 1)


class Batch:
    """Host arrays of one batch of tracks in the ck_batch_in layout."""

    def __init__(self, n, cap):
        self.n = n
        self.cap = cap
        self.seq_offsets = np.zeros(n + 1, np.int32)
        self.seq_surfaces = np.zeros(n * cap, np.int32)
        self.meas_offsets = np.zeros(n + 1, np.int32)
        self.meas_surfaces = np.zeros(n * cap, np.int32)
        self.meas_values = np.zeros(n * cap * 2, np.float64)
        self.meas_cov = np.zeros(n * cap * 4, np.float64)
        self.start_params = np.zeros(n * 6, np.float64)
        self.start_cov = np.zeros(n * 36, np.float64)
        self.start_frames = np.zeros(n * 12, np.float64)
        self.particle = np.zeros(n * 2, np.float32)
        self.particle_pdg = np.zeros(n, np.int32)
        self.truth_meas = np.zeros(n * cap * 6, np.float64)
        self.meas_outlier = np.zeros(n * cap, np.uint8)
        self.truth_start = np.zeros(n * 6, np.float64)
        # CK_MEAS_* per measurement; None: every source link is 2D
        self.meas_subspace = None

    def trim(self):
        ns = int(self.seq_offsets[-1])
        nm = int(self.meas_offsets[-1])
        self.seq_surfaces = np.ascontiguousarray(self.seq_surfaces[:ns])
        self.meas_surfaces = np.ascontiguousarray(self.meas_surfaces[:nm])
        self.meas_values = np.ascontiguousarray(self.meas_values[: 2 * nm])
        self.meas_cov = np.ascontiguousarray(self.meas_cov[: 4 * nm])
        self.truth_meas = np.ascontiguousarray(self.truth_meas[: 6 * nm])
        self.meas_outlier = np.ascontiguousarray(self.meas_outlier[:nm])
        if self.meas_subspace is not None:
            self.meas_subspace = np.ascontiguousarray(self.meas_subspace[:nm])
        return self

    @property
    def n_meas(self):
        return int(self.meas_offsets[-1])

    def as_batch_in(self, memory=abi.MEM_HOST):
        b = abi.ck_batch_in()
        b.n_tracks = self.n
        b.memory = memory
        b.seq_offsets = abi.ptr(self.seq_offsets, C.c_int32)
        b.seq_surfaces = abi.ptr(self.seq_surfaces, C.c_int32)
        b.meas_offsets = abi.ptr(self.meas_offsets, C.c_int32)
        b.meas_surfaces = abi.ptr(self.meas_surfaces, C.c_int32)
        b.meas_values = abi.ptr(self.meas_values, C.c_double)
        b.meas_cov = abi.ptr(self.meas_cov, C.c_double)
        b.start_params = abi.ptr(self.start_params, C.c_double)
        b.start_cov = abi.ptr(self.start_cov, C.c_double)
        b.start_frames = abi.ptr(self.start_frames, C.c_double)
        b.particle = abi.ptr(self.particle, C.c_float)
        b.particle_pdg = abi.ptr(self.particle_pdg, C.c_int32)
        b.meas_subspace = abi.ptr(self.meas_subspace, C.c_int32)
        return b

    def subset(self, idx):
        """A new Batch holding tracks `idx` (in that order)."""
        idx = np.asarray(idx, dtype=np.int64)
        so, mo = self.seq_offsets, self.meas_offsets
        out = Batch(len(idx), self.cap)
        seq, ms, mv, mc, tm, mol, msub = [], [], [], [], [], [], []
        for j, t in enumerate(idx):
            a, b = so[t], so[t + 1]
            seq.append(self.seq_surfaces[a:b])
            out.seq_offsets[j + 1] = out.seq_offsets[j] + (b - a)
            a, b = mo[t], mo[t + 1]
            ms.append(self.meas_surfaces[a:b])
            mv.append(self.meas_values[2 * a:2 * b])
            mc.append(self.meas_cov[4 * a:4 * b])
            tm.append(self.truth_meas[6 * a:6 * b])
            mol.append(self.meas_outlier[a:b])
            if self.meas_subspace is not None:
                msub.append(self.meas_subspace[a:b])
            out.meas_offsets[j + 1] = out.meas_offsets[j] + (b - a)
        cat = lambda xs, dt: np.ascontiguousarray(np.concatenate(xs).astype(dt)) if xs else np.zeros(0, dt)
        out.seq_surfaces = cat(seq, np.int32)
        out.meas_surfaces = cat(ms, np.int32)
        out.meas_values = cat(mv, np.float64)
        out.meas_cov = cat(mc, np.float64)
        out.truth_meas = cat(tm, np.float64)
        out.meas_outlier = cat(mol, np.uint8)
        out.meas_subspace = cat(msub, np.int32) if self.meas_subspace is not None else None
        for name, k in (("start_params", 6), ("start_cov", 36), ("start_frames", 12),
                        ("particle", 2), ("truth_start", 6)):
            src = getattr(self, name).reshape(self.n, k)
            setattr(out, name, np.ascontiguousarray(src[idx].reshape(-1)))
        out.particle_pdg = np.ascontiguousarray(self.particle_pdg[idx])
        return out


def generate(detector, n_tracks, seed=1, first_track=0, n_threads=None, cap=24):
    L = lib()
    b = Batch(n_tracks, cap)
    o = abi.ckg_out()
    o.max_per_track = cap
    for name in ("seq_offsets", "seq_surfaces", "meas_offsets", "meas_surfaces", "particle_pdg"):
        setattr(o, name, abi.ptr(getattr(b, name), C.c_int32))
    for name in ("meas_values", "meas_cov", "start_params", "start_cov", "start_frames",
                 "truth_meas", "truth_start"):
        setattr(o, name, abi.ptr(getattr(b, name), C.c_double))
    o.particle = abi.ptr(b.particle, C.c_float)
    o.meas_outlier = abi.ptr(b.meas_outlier, C.c_uint8)
    if detector.preset == abi.CKG_STRIPS:
        b.meas_subspace = np.zeros(n_tracks * cap, np.int32)
        o.meas_subspace = abi.ptr(b.meas_subspace, C.c_int32)
    nm = L.ckg_generate(detector.preset, seed, first_track, n_tracks, detector.surfaces,
                        detector.n_surfaces, C.byref(detector.field),
                        n_threads or os.cpu_count() or 1, C.byref(o))
    if nm < 0:
        raise RuntimeError("generator failed")
    return b.trim()


def event_sizes(seed, n_events, mean=-1.0, lo=100, hi=20000):
    out = np.zeros(n_events, np.int32)
    lib().ckg_event_sizes(seed, n_events, mean, lo, hi, abi.ptr(out, C.c_int32))
    return out


def ckf_events(detector, batch, sizes, max_states=64, max_tracks=16):
    """The batch's tracks as consecutive events of `sizes` tracks each, for
    one track-finding call over all of them: every track is a seed of its
    event; the measurements are grouped by event, then surface (stable).
    `meas_track` / `meas_index` as in ckf_event."""
    sizes = np.asarray(sizes, np.int64)
    n = batch.n
    if sizes.sum() != n:
        raise ValueError("event sizes do not add up to the batch")
    n_ev = len(sizes)
    seed_event = np.repeat(np.arange(n_ev, dtype=np.int32), sizes)
    nm = int(batch.meas_offsets[-1])
    ms = np.asarray(batch.meas_surfaces[:nm]).astype(np.int64)
    track_of = np.repeat(np.arange(n, dtype=np.int32), np.diff(batch.meas_offsets))
    seg = seed_event[track_of].astype(np.int64) * detector.n_surfaces + ms
    order = np.argsort(seg, kind="stable")
    counts = np.bincount(seg, minlength=n_ev * detector.n_surfaces)
    offs = np.zeros(n_ev * detector.n_surfaces + 1, np.int32)
    offs[1:] = np.cumsum(counts)
    sub = None if batch.meas_subspace is None else np.asarray(batch.meas_subspace[:nm])[order]
    tf = abi.TrackFinding(batch.seq_offsets, batch.seq_surfaces, batch.start_params,
                          batch.start_cov, batch.start_frames, batch.particle, offs,
                          batch.meas_values.reshape(-1, 2)[:nm][order],
                          batch.meas_cov.reshape(-1, 4)[:nm][order], meas_subspace=sub,
                          particle_pdg=batch.particle_pdg, max_states=max_states,
                          max_tracks=max_tracks, n_events=n_ev, seed_event=seed_event)
    tf.meas_track = track_of[order]
    tf.meas_index = order.astype(np.int64)
    return tf


def ckf_event(detector, batch, max_states=64, max_tracks=16):
    """The batch's tracks as one event for track finding (an
    abi.TrackFinding): every track's start parameters become a seed with the
    track's surface sequence; all measurements of the batch, grouped by
    surface (stable: within a surface in track order), are the candidates.
    `meas_track` gives the generating track of each grouped measurement and
    `meas_index` its index in the batch."""
    n = batch.n
    nm = int(batch.meas_offsets[-1])
    ms = np.asarray(batch.meas_surfaces[:nm])
    order = np.argsort(ms, kind="stable")
    counts = np.bincount(ms, minlength=detector.n_surfaces)
    offs = np.zeros(detector.n_surfaces + 1, np.int32)
    offs[1:] = np.cumsum(counts)
    track_of = np.repeat(np.arange(n, dtype=np.int32), np.diff(batch.meas_offsets))
    sub = None if batch.meas_subspace is None else np.asarray(batch.meas_subspace[:nm])[order]
    tf = abi.TrackFinding(batch.seq_offsets, batch.seq_surfaces, batch.start_params,
                          batch.start_cov, batch.start_frames, batch.particle, offs,
                          batch.meas_values.reshape(-1, 2)[:nm][order],
                          batch.meas_cov.reshape(-1, 4)[:nm][order], meas_subspace=sub,
                          particle_pdg=batch.particle_pdg, max_states=max_states,
                          max_tracks=max_tracks)
    tf.meas_track = track_of[order]
    tf.meas_index = order.astype(np.int64)
    return tf


class DeviceBatch:
    """A generated batch in device memory (torch tensors) in the layout of
    ckg_out / ck_batch_in, as ck_simulate writes it."""

    INT = ("seq_offsets", "seq_surfaces", "meas_offsets", "meas_surfaces", "particle_pdg")
    DBL = ("meas_values", "meas_cov", "start_params", "start_cov", "start_frames",
           "truth_meas", "truth_start")

    def __init__(self, n, cap, torch, device, strips=False):
        self.n, self.cap, self.device = n, cap, device
        t = lambda k, dt: torch.empty(k, dtype=dt, device=device)
        self.seq_offsets = t(n + 1, torch.int32)
        self.meas_offsets = t(n + 1, torch.int32)
        self.seq_surfaces = t(max(n * cap, 1), torch.int32)
        self.meas_surfaces = t(max(n * cap, 1), torch.int32)
        self.meas_values = t(max(n * cap * 2, 1), torch.float64)
        self.meas_cov = t(max(n * cap * 4, 1), torch.float64)
        self.truth_meas = t(max(n * cap * 6, 1), torch.float64)
        self.meas_outlier = t(max(n * cap, 1), torch.uint8)
        self.start_params = t(n * 6, torch.float64)
        self.start_cov = t(n * 36, torch.float64)
        self.start_frames = t(n * 12, torch.float64)
        self.truth_start = t(n * 6, torch.float64)
        self.particle = t(n * 2, torch.float32)
        self.particle_pdg = t(n, torch.int32)
        self.meas_subspace = t(max(n * cap, 1), torch.int32) if strips else None

    @staticmethod
    def _p(x, ct):
        return None if x is None else C.cast(C.c_void_p(x.data_ptr()), C.POINTER(ct))

    def as_ckg_out(self):
        o = abi.ckg_out()
        o.max_per_track = self.cap
        for name in self.INT:
            setattr(o, name, self._p(getattr(self, name), C.c_int32))
        for name in self.DBL:
            setattr(o, name, self._p(getattr(self, name), C.c_double))
        o.particle = self._p(self.particle, C.c_float)
        o.meas_outlier = self._p(self.meas_outlier, C.c_uint8)
        o.meas_subspace = self._p(self.meas_subspace, C.c_int32)
        return o

    def trim(self):
        """Views of the filled part of the row arrays."""
        ns = int(self.seq_offsets[-1])
        nm = int(self.meas_offsets[-1])
        self.seq_surfaces = self.seq_surfaces[:ns]
        self.meas_surfaces = self.meas_surfaces[:nm]
        self.meas_values = self.meas_values[:2 * nm]
        self.meas_cov = self.meas_cov[:4 * nm]
        self.truth_meas = self.truth_meas[:6 * nm]
        self.meas_outlier = self.meas_outlier[:nm]
        if self.meas_subspace is not None:
            self.meas_subspace = self.meas_subspace[:nm]
        return self

    def as_batch_in(self):
        """A ck_batch_in over the device arrays (memory = device)."""
        b = abi.ck_batch_in()
        b.n_tracks = self.n
        b.memory = abi.MEM_DEVICE
        for name in ("seq_offsets", "seq_surfaces", "meas_offsets", "meas_surfaces",
                     "particle_pdg"):
            setattr(b, name, self._p(getattr(self, name), C.c_int32))
        for name in ("meas_values", "meas_cov", "start_params", "start_cov", "start_frames"):
            setattr(b, name, self._p(getattr(self, name), C.c_double))
        b.particle = self._p(self.particle, C.c_float)
        b.meas_subspace = self._p(self.meas_subspace, C.c_int32)
        return b

    def to_host(self):
        """The same batch as a host Batch."""
        out = Batch(self.n, 1)
        for name in self.INT + self.DBL + ("meas_outlier",):
            setattr(out, name, getattr(self, name).cpu().numpy())
        out.particle = self.particle.cpu().numpy()
        out.meas_subspace = None if self.meas_subspace is None else self.meas_subspace.cpu().numpy()
        return out
