"""Per-event CSV files of the examples' I/O (Examples/Io/Csv) for the
track-fitting layer: measurements and proto tracks.

* ``event{N:09d}-measurements.csv`` — one row per measurement with the
  columns of ``MeasurementData`` (Examples/Io/Csv/src/CsvOutputData.hpp:
  236-252): measurement_id, geometry_id, local_key, local0, local1, phi,
  theta, time, var_local0, var_local1, var_phi, var_theta, var_time,
  global_x, global_y, global_z. ``local_key`` marks the measured bound
  parameters with bit (index + 1) (CsvMeasurementReader.cpp:205-240); the
  fitter takes loc0, loc1 or both.
* ``event{N:09d}-prototracks.csv`` — ``ProtoTrackData`` rows (trackId,
  measurementId, x, y, z; CsvOutputData.hpp:443-449), one per hit in
  track order.

File names follow ``perEventFilepath`` (Examples/Framework/src/Utilities/
Paths.cpp:42-54). Geometry identifiers are mapped to the fitter's surface
table by the caller's ``{geometry_id: surface index}``.
"""
import csv
import os

import numpy as np

from . import abi
from .track_fitting import Measurements

MEASUREMENT_COLUMNS = ("measurement_id", "geometry_id", "local_key", "local0", "local1", "phi",
                       "theta", "time", "var_local0", "var_local1", "var_phi", "var_theta",
                       "var_time", "global_x", "global_y", "global_z")
PROTOTRACK_COLUMNS = ("trackId", "measurementId", "x", "y", "z")
_KEY_LOC0, _KEY_LOC1 = 1 << 1, 1 << 2


def per_event_filepath(directory, name, event):
    prefix = "event%09d-" % event
    return prefix + name if not directory else os.path.join(directory, prefix + name)


def write_measurements(path, measurements, geometry_ids):
    """`measurements`: a track_fitting.Measurements (measurement i gets
    measurement_id i); `geometry_ids`: the geometry identifier of each surface
    index."""
    sub = (measurements.subspaces if measurements.subspaces is not None
           else np.full(len(measurements), abi.MEAS_LOC01))
    vals = np.asarray(measurements.values).reshape(-1, 2)
    cov = np.asarray(measurements.covariances).reshape(-1, 4)
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(MEASUREMENT_COLUMNS)
        for i in range(len(measurements)):
            s = int(sub[i])
            key = (_KEY_LOC0 if s in (abi.MEAS_LOC0, abi.MEAS_LOC01) else 0) | \
                  (_KEY_LOC1 if s in (abi.MEAS_LOC1, abi.MEAS_LOC01) else 0)
            # a 1D measurement of loc1 keeps its value in the first slot of the
            # fitter's arrays and in local1 here
            l0, l1 = (vals[i, 0], vals[i, 1]) if s != abi.MEAS_LOC1 else (0.0, vals[i, 0])
            v0, v1 = (cov[i, 0], cov[i, 3]) if s != abi.MEAS_LOC1 else (0.0, cov[i, 0])
            w.writerow([i, int(geometry_ids[int(measurements.surfaces[i])]), key, repr(float(l0)),
                        repr(float(l1)), 0, 0, 0, repr(float(v0)), repr(float(v1)), 0, 0, 0, 0, 0, 0])


def read_measurements(path, surface_of_geometry):
    """A track_fitting.Measurements from a measurements file, in the file's
    measurement_id order; returns (measurements, measurement ids). Only loc0
    / loc1 measurements are accepted; the off-diagonal covariance is 0 (the
    file holds variances)."""
    with open(path, newline="") as f:
        rows = list(csv.DictReader(f))
    rows.sort(key=lambda r: int(r["measurement_id"]))
    n = len(rows)
    surf = np.zeros(n, np.int32)
    vals = np.zeros((n, 2))
    cov = np.zeros((n, 4))
    sub = np.zeros(n, np.int32)
    ids = np.zeros(n, np.int64)
    for i, r in enumerate(rows):
        key = int(r["local_key"])
        if key & ~(_KEY_LOC0 | _KEY_LOC1) or not key:
            raise ValueError("measurement %s measures more than loc0/loc1 (local_key %d)"
                             % (r["measurement_id"], key))
        gid = int(r["geometry_id"])
        if gid not in surface_of_geometry:
            raise ValueError("geometry_id %d is not in the surface table" % gid)
        surf[i] = surface_of_geometry[gid]
        ids[i] = int(r["measurement_id"])
        l0, l1 = float(r["local0"]), float(r["local1"])
        v0, v1 = float(r["var_local0"]), float(r["var_local1"])
        if key == _KEY_LOC0 | _KEY_LOC1:
            sub[i], vals[i], cov[i] = abi.MEAS_LOC01, (l0, l1), (v0, 0.0, 0.0, v1)
        elif key == _KEY_LOC0:
            sub[i], vals[i], cov[i] = abi.MEAS_LOC0, (l0, 0.0), (v0, 0.0, 0.0, 0.0)
        else:
            sub[i], vals[i], cov[i] = abi.MEAS_LOC1, (l1, 0.0), (v1, 0.0, 0.0, 0.0)
    return Measurements(surfaces=surf, values=vals.ravel(), covariances=cov.ravel(),
                        subspaces=sub), ids


def write_proto_tracks(path, proto_tracks):
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(PROTOTRACK_COLUMNS)
        for t, hits in enumerate(proto_tracks):
            for m in hits:
                w.writerow([t, int(m), 0, 0, 0])


def read_proto_tracks(path, measurement_ids, n_tracks=None):
    """Proto tracks as lists of measurement container indices (the position
    of each measurementId in `measurement_ids`), in file order per track."""
    index = {int(m): i for i, m in enumerate(measurement_ids)}
    tracks = {}
    with open(path, newline="") as f:
        for r in csv.DictReader(f):
            tracks.setdefault(int(r["trackId"]), []).append(index[int(r["measurementId"])])
    n = n_tracks if n_tracks is not None else (max(tracks) + 1 if tracks else 0)
    return [tracks.get(t, []) for t in range(n)]
