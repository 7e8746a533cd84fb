"""ERT data container, measurement-scheme generators and analytic geometric
factors.

``DataContainerERT`` keeps what the forward operator reads from the
reference's ``GIMLI::DataContainerERT`` (core/src/bert/bertDataContainer.h:32,
addFourPointData at :62): sensor positions and the four electrode index
columns ``a b m n`` (-1 = electrode at infinity) plus the data fields
``k`` (geometric factor) and ``rhoa``.

The scheme generators restate the loops of pyGIMLi's scheme classes
(pygimli/physics/ert/ertScheme.py: dipole-dipole 476-527, pole-dipole
554-578, Wenner-alpha 652-672) and ``createData`` mirrors
``pg.physics.ert.createData(elecs, schemeName)``.

``geometricFactors`` restates core/src/bert/bertMisc.cpp:131-176 with the
half-space mirror potential of bertMisc.cpp:186-230 (k = 1 / (u_AM - u_BM -
u_AN + u_BN), 2-D sensor positions (x, y) are moved to (x, 0, y) first).
"""
from __future__ import annotations

import os

import numpy as np

# fields every ERT container has (core/src/bert/bertDataContainer.cpp:45-61)
_DEFAULT_TOKENS = ("a", "b", "m", "n", "err", "i", "ip", "iperr", "k", "r", "rhoa", "u", "valid")


class DataContainerERT:
    """Sensors + four-point configurations + data fields."""

    def __init__(self, sensors=None, abmn=None, removeInvalid=True, sensorIndicesFromOne=None):
        """``DataContainerERT(sensors, abmn)``, or like the reference's file
        constructor ``DataContainerERT(fileName, sensorIndicesFromOne=True,
        removeInvalid=True)``."""
        self._sensors = np.zeros((0, 3))
        self._abmn = np.zeros((0, 4), np.int32)
        self._fields = {}
        self._topo = np.zeros((0, 3))
        self._index_from_one = True  # sensor indices on file count from one
        if isinstance(sensors, (str, os.PathLike)):
            if sensorIndicesFromOne is None:
                sensorIndicesFromOne = True if abmn is None else bool(abmn)
            self.load(sensors, sensorIndicesFromOne, removeInvalid)
            return
        if sensors is not None:
            self.setSensorPositions(sensors)
        if abmn is not None:
            ab = np.asarray(abmn, dtype=np.int32).reshape(-1, 4)
            self._abmn = ab.copy()

    # -- sensors ------------------------------------------------------------
    def setSensorPositions(self, pos):
        p = np.asarray(pos, dtype=np.float64)
        if p.ndim == 1:
            p = np.column_stack([p, np.zeros(len(p)), np.zeros(len(p))])
        if p.shape[1] == 2:
            p = np.column_stack([p, np.zeros(len(p))])
        self._sensors = np.ascontiguousarray(p)

    def sensorPositions(self):
        return self._sensors.copy()

    def sensorPosition(self, i):
        return self._sensors[i].copy()

    def sensorCount(self):
        return len(self._sensors)

    def createSensor(self, pos, tolerance=1e-3):
        """Index of the sensor at ``pos``: the last one closer than
        ``tolerance``, else a new one (DataContainer::createSensor,
        core/src/datacontainer.cpp:170-184)."""
        p = np.zeros(3)
        p[:len(pos)] = pos
        if len(self._sensors):
            hit = np.nonzero(np.linalg.norm(self._sensors - p, axis=1) < tolerance)[0]
            if len(hit):
                return int(hit[-1])
        self._sensors = np.vstack([self._sensors, p])
        return len(self._sensors) - 1

    def setSensorPosition(self, i, pos):
        p = np.zeros(3)
        p[:len(pos)] = pos
        self._sensors[int(i)] = p

    def translate(self, vec):
        """Move every sensor by ``vec`` (DataContainer::translate)."""
        v = np.zeros(3)
        v[:len(vec)] = vec
        self._sensors = self._sensors + v

    def scale(self, vec):
        """Scale every sensor position componentwise (DataContainer::scale)."""
        v = np.ones(3)
        v[:len(vec)] = vec
        self._sensors = self._sensors * v

    # -- data -------------------------------------------------------------
    def addFourPointData(self, a, b, m, n):
        self._abmn = np.vstack([self._abmn, np.array([[a, b, m, n]], np.int32)])
        for k, v in self._fields.items():
            self._fields[k] = np.append(v, 1.0 if k == "valid" else 0.0)
        return len(self._abmn) - 1

    def size(self):
        return len(self._abmn)

    def __len__(self):
        return self.size()

    def abmn(self):
        return self._abmn.copy()

    def __getitem__(self, token):
        if token in ("a", "b", "m", "n"):
            return self._abmn[:, "abmn".index(token)].astype(np.float64)
        if token in self._fields:
            return self._fields[token].copy()
        if token == "valid":
            return np.ones(self.size())
        if token in _DEFAULT_TOKENS:
            return np.zeros(self.size())
        raise KeyError(token)

    def __call__(self, token):
        return self[token]

    def get(self, token):
        return self[token]

    def __setitem__(self, token, values):
        self.set(token, values)

    def set(self, token, values):
        v = np.asarray(values, dtype=np.float64)
        if v.shape != (self.size(),):
            raise ValueError(f"field '{token}' needs {self.size()} values")
        if token in ("a", "b", "m", "n"):
            self._abmn[:, "abmn".index(token)] = v.astype(np.int32)
        else:
            self._fields[token] = v.copy()

    def exists(self, token):
        return token in self._fields or token in _DEFAULT_TOKENS

    def haveData(self, token):
        """True when ``token`` holds a value above 1e-12 in magnitude."""
        return self.size() > 0 and self.exists(token) and float(np.max(np.abs(self[token]))) >= 1e-12

    def tokenList(self):
        """Sensor index tokens, then the data fields, each group sorted."""
        from .fileio import token_list
        return token_list(self._field_map())

    def markValid(self, idx, valid=True):
        v = self["valid"]
        v[np.asarray(idx)] = 1.0 if valid else 0.0
        self._fields["valid"] = v

    def markInvalid(self, idx):
        self.markValid(idx, False)

    def remove(self, idx):
        """Drop the data ``idx`` (indices or a boolean mask), as
        DataContainer::remove (markValid(idx, false) + removeInvalid)."""
        idx = np.asarray(idx)
        if idx.dtype == bool:
            idx = np.nonzero(idx)[0]
        self.markInvalid(idx)
        self.removeInvalid()

    def resize(self, n):
        """n data: new rows get sensor index -1 and field value 0, 'valid' 0
        (DataContainer::resize, datacontainer.cpp:742-754)."""
        n = int(n)
        old = self.size()
        if n <= old:
            self._abmn = self._abmn[:n].copy()
            self._fields = {k: v[:n].copy() for k, v in self._fields.items()}
            return
        self._abmn = np.vstack([self._abmn, np.full((n - old, 4), -1, np.int32)])
        self._fields = {k: np.concatenate([v, np.zeros(n - old)]) for k, v in self._fields.items()}

    def add(self, other, snap=1e-3):
        """Append ``other``'s data: its sensors merged into this container's
        (createSensor with tolerance ``snap``), its sensor indices mapped onto
        them, the fields of this container filled from ``other``
        (DataContainer::add, core/src/datacontainer.cpp:139-168)."""
        start = self.size()
        perm = np.array([self.createSensor(p, snap) for p in other.sensorPositions()], np.int64)
        ab = other.abmn().astype(np.int64)
        ok = (ab > -1) & (ab < len(perm))
        mapped = np.where(ok, perm[np.where(ok, ab, 0)], -1).astype(np.int32)
        mine = self._field_map()
        theirs = other._field_map()
        self._abmn = np.vstack([self._abmn, mapped]).reshape(-1, 4)
        n = self.size()
        for k, v in mine.items():
            if k in "abmn":
                continue
            add = theirs[k] if k in theirs else np.zeros(n - start)
            self._fields[k] = np.concatenate([v, add])

    def removeInvalid(self):
        """Drop every datum whose 'valid' flag is not 1."""
        keep = np.nonzero(self["valid"] == 1)[0]
        self._abmn = self._abmn[keep].copy()
        self._fields = {k: v[keep].copy() for k, v in self._fields.items()}

    def checkDataValidity(self, remove=True):
        """Validity rules of the reference's loader (non-finite values,
        sensor indices out of range, rhoa or |r| below 1e-12, coinciding
        electrodes); ``remove`` drops what they mark."""
        from .fileio import check_validity
        self._set_field_map(check_validity(self._field_map(), self.sensorCount(), remove=remove))

    def removeUnusedSensors(self):
        from .fileio import _remove_unused_sensors
        sensors, f = _remove_unused_sensors(self._sensors, self._field_map())
        self._sensors = np.ascontiguousarray(sensors)
        self._set_field_map(f)

    def estimateError(self, *args, **kwargs):
        """Set 'err' from estimateError (geometric factors first if missing)."""
        if not self.haveData("k"):
            self.set("k", geometricFactors(self, 3 if np.ptp(self._sensors[:, 1]) > 0 else 2))
        self.set("err", estimateError(self, *args, **kwargs))

    def additionalPoints(self):
        """Additional (topography) points read from a file."""
        return self._topo.copy()

    # -- unified data format -------------------------------------------------
    def _field_map(self):
        f = {t: self._abmn[:, j].astype(np.float64) for j, t in enumerate("abmn")}
        for t in _DEFAULT_TOKENS[4:]:
            f[t] = self[t]
        for k, v in self._fields.items():
            f[k] = v.copy()
        return f

    def _set_field_map(self, f):
        n = len(f["valid"])
        self._abmn = np.column_stack([f[t] for t in "abmn"]).astype(np.int32).reshape(n, 4)
        self._fields = {k: np.asarray(v, np.float64).copy() for k, v in f.items() if k not in "abmn"}

    def load(self, fileName, sensorIndicesFromOne=True, removeInvalid=True):
        """Read a unified data file (the reference's DataContainer::load,
        core/src/datacontainer.cpp:209-470): sensors with an optional
        '# x y z' format line, data columns named by the '#' line after the
        data count (aliases such as c1 c2 p1 p2, rho_a, u/mV, err/% are
        translated and scaled), sensor indices counted from one on file,
        duplicated sensors merged, invalid data dropped."""
        from .fileio import read_unified
        u = read_unified(fileName, sensorIndicesFromOne, removeInvalid)
        self._sensors = np.ascontiguousarray(u.sensors)
        self._set_field_map(u.fields)
        self._topo = u.topo
        self._index_from_one = bool(sensorIndicesFromOne)
        return 1

    def save(self, fileName, formatData="all", formatSensor="x y z", noFilter=False, verbose=False):
        """Write a unified data file (DataContainer::save,
        core/src/datacontainer.cpp:518-615); ``formatData`` names the
        columns ("all": every field and datum, else only valid data)."""
        from .fileio import write_unified
        return write_unified(fileName, self._sensors, self._field_map(), formatData, formatSensor, noFilter,
                             self._index_from_one)

    def allNonZero(self, token):
        return token in self._fields and bool(np.all(self._fields[token] != 0))

    def copy(self):
        d = DataContainerERT(self._sensors, self._abmn)
        d._fields = {k: v.copy() for k, v in self._fields.items()}
        d._topo = self._topo.copy()
        d._index_from_one = self._index_from_one
        return d

    def __repr__(self):
        return f"DataContainerERT(sensors={self.sensorCount()}, data={self.size()}, fields={sorted(self._fields)})"


# -- measurement schemes (pygimli/physics/ert/ertScheme.py) -----------------

def _scheme_dd(nE, spacings=(1,), max_separation=999):
    out = []
    for space in spacings:
        max_sep = nE - space
        max_inj = nE - space
        if max_separation < max_sep:
            max_sep = max_separation
        for sep in range(1, max_sep + 1):
            for i in range(max_inj - sep):
                a = i
                b = (a + space) % nE
                m = (b + sep) % nE
                n = (m + space) % nE
                if m + space < nE:
                    out.append((a, b, m, n))
    return out


def _scheme_pd(nE, max_separation=999):
    out = []
    b = -1
    for a in range(nE):
        for m in range(a + 1, nE - 1):
            n = m + 1
            if m - a > max_separation:
                break
            out.append((a, b, m, n))
    return out


def _scheme_wa(nE, max_separation=999):
    out = []
    max_sep = nE - 2
    if max_separation < max_sep:
        max_sep = max_separation
    for sep in range(1, max_sep + 1):
        for i in range((nE - 2) - sep):
            a = i
            m = a + sep
            n = m + sep
            b = n + sep
            if max(a, b, m, n) < nE:
                out.append((a, b, m, n))
    return out


def createData(elecs, schemeName="dd", **kwargs):
    """Create a data container for the electrode positions ``elecs``
    (array of x, or (N, 2|3) positions) and a scheme name
    (``dd`` dipole-dipole, ``pd`` pole-dipole, ``wa`` Wenner-alpha)."""
    e = np.asarray(elecs, dtype=np.float64)
    if e.ndim == 1:
        e = np.column_stack([e, np.zeros(len(e)), np.zeros(len(e))])
    nE = len(e)
    max_sep = kwargs.pop("maxSeparation", 999)
    if schemeName == "dd":
        rows = _scheme_dd(nE, kwargs.pop("spacings", (1,)), max_sep)
    elif schemeName == "pd":
        rows = _scheme_pd(nE, max_sep)
    elif schemeName == "wa":
        rows = _scheme_wa(nE, max_sep)
    else:
        raise ValueError(f"unknown scheme '{schemeName}'")
    d = DataContainerERT(e, np.array(rows, np.int32).reshape(-1, 4))
    return d


def grid_line_scheme(electrode_grid, kind="dd", max_separation=999):
    """Dipole-dipole / pole-dipole / Wenner lines along x and along y of a rectangular
    surface electrode grid ``electrode_grid`` (nx, ny) whose electrode index
    is ``ix * ny + iy``."""
    nx, ny = electrode_grid
    rows = []
    lines = [[ix * ny + iy for ix in range(nx)] for iy in range(ny)]
    lines += [[ix * ny + iy for iy in range(ny)] for ix in range(nx)]
    gens = {"dd": lambda m: _scheme_dd(m, (1,), max_separation),
            "pd": lambda m: _scheme_pd(m, max_separation=max_separation),
            "wa": lambda m: _scheme_wa(m, max_separation=max_separation)}
    if kind not in gens:
        raise ValueError(f"unknown line scheme {kind!r}")
    for line in lines:
        loc = gens[kind](len(line))
        for (a, b, m, n) in loc:
            rows.append(tuple(line[i] if i >= 0 else -1 for i in (a, b, m, n)))
    return np.array(rows, np.int32).reshape(-1, 4)


def grid_scheme_3d(nx, ny, max_line_offset=3):
    """Surface-grid scheme for an (nx, ny) electrode grid (electrode index
    ``ix * ny + iy``): inline dipole-dipole along every x and y line,
    pole-dipole along the x lines, and cross-line dipole-dipole (current
    dipole on one x line, potential dipoles of unit length on the x lines
    up to ``max_line_offset`` lines away).  For 12 x 8 electrodes and offset
    3 this gives 5336 configurations."""
    def idx(ix, iy):
        return ix * ny + iy
    rows = []
    xl = [[idx(ix, iy) for ix in range(nx)] for iy in range(ny)]
    yl = [[idx(ix, iy) for iy in range(ny)] for ix in range(nx)]
    for line in xl + yl:
        for (a, b, m, n) in _scheme_dd(len(line)):
            rows.append((line[a], line[b], line[m], line[n]))
    for line in xl:
        for (a, _, m, n) in _scheme_pd(len(line)):
            rows.append((line[a], -1, line[m], line[n]))
    for iy in range(ny):
        for jy in range(ny):
            if jy == iy or abs(jy - iy) > max_line_offset:
                continue
            for a in range(nx - 1):
                for m in range(nx - 1):
                    rows.append((idx(a, iy), idx(a + 1, iy), idx(m, jy), idx(m + 1, jy)))
    return np.array(rows, np.int32).reshape(-1, 4)


# -- geometric factors (core/src/bert/bertMisc.cpp:131-230) ---------------

def _u_half(p, s):
    """3-D half-space potential of a unit source at ``s`` observed at ``p``
    with the mirror source above z=0 (bertMisc.cpp:186-230 with k = 0,
    surfaceZ = 0): (1/r + 1/r') / (4 pi)."""
    r = np.linalg.norm(p - s, axis=-1)
    sm = s.copy()
    sm[..., 2] = -s[..., 2]
    rm = np.linalg.norm(p - sm, axis=-1)
    with np.errstate(divide="ignore"):
        return (1.0 / r + 1.0 / rm) / (4.0 * np.pi)


def estimateError(data, relativeError=0.03, absoluteUError=None, absoluteError=0, absoluteCurrent=0.1):
    """Relative data error from a relative and an absolute part
    (pygimli/physics/ert/ert.py:482-540): relativeError + |absoluteError /
    rhoa|, or with ``absoluteUError`` (V) relativeError + |absoluteUError /
    u| where u comes from 'u', else r * i, else rhoa / k * i (i: 'i' or
    absoluteCurrent).  A relativeError of 0.5 or more is taken as percent."""
    if relativeError >= 0.5:
        relativeError /= 100.0
    if absoluteUError is None:
        if not data.allNonZero("rhoa"):
            raise ValueError("We need apparent resistivity values (rhoa) in the data to estimate a data error.")
        return relativeError + np.abs(absoluteError / data["rhoa"])
    i = data["i"] if data.haveData("i") else absoluteCurrent
    if data.haveData("u"):
        u = data["u"]
    elif data.haveData("r"):
        u = data["r"] * i
    elif data.haveData("rhoa"):
        if not data.haveData("k"):
            raise ValueError("We need (rhoa) and (k) in the data to estimate data error.")
        u = data["rhoa"] / data["k"] * i
    else:
        raise ValueError("We need apparent resistivity values (rhoa) or impedances (r) in the data to estimate "
                         "data error.")
    return np.abs(absoluteUError / u) + relativeError


def geometricFactors(data, dim=3):
    """Analytic half-space geometric factors for every datum."""
    pos = data.sensorPositions().copy()
    if dim == 2:
        # (x, y) -> (x, 0, y) when y differs from 0 (bertMisc.cpp:134-145)
        mv = pos[:, 1] != 0.0
        pos[mv, 2] = pos[mv, 1]
        pos[mv, 1] = 0.0
    ab = data.abmn()
    k = np.empty(len(ab))
    for i, (a, b, m, n) in enumerate(ab):
        uam = _u_half(pos[m], pos[a]) if (a > -1 and m > -1) else 0.0
        ubm = _u_half(pos[m], pos[b]) if (b > -1 and m > -1) else 0.0
        uan = _u_half(pos[n], pos[a]) if (a > -1 and n > -1) else 0.0
        ubn = _u_half(pos[n], pos[b]) if (b > -1 and n > -1) else 0.0
        k[i] = 1.0 / (uam - ubm - uan + ubn)
    return k
