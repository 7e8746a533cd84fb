"""The reference's file formats for ERT data and meshes.

Unified data format (``.dat`` / ``.ohm`` / ``.shm``), read and written by
``GIMLI::DataContainer`` (core/src/datacontainer.cpp: ``load`` 209-470,
``write`` 527-615) with the ERT token aliases of
core/src/bert/bertDataContainer.cpp:64-90 and the validity rules of
datacontainer.cpp:480-516 and bertDataContainer.cpp:92-148::

    <number of sensors>
    # x y z                       (optional sensor format line)
    <one row per sensor>
    <number of data>
    # a b m n rhoa err ...        (data format line)
    <one row per datum; sensor indices count from one on file>
    <number of additional (topography) points, optional>

Binary mesh format (``.bms``, version 3), ``Mesh::saveBinaryV2`` /
``Mesh::loadBinaryV2`` (core/src/mesh_io.cpp:391-662), little-endian::

    u8 dim, u8 version (3), u8[128] (byte 0: geometry flag),
    u32 nNodes, f64[3 nNodes] positions, i32[nNodes] node markers,
    u32 nCells, u8[nCells] node counts, u32[sum] node ids, i32[nCells] markers,
    u32 nBounds, u8[nBounds] node counts, u32[sum] node ids, i32 markers,
    i32[nBounds] left cell, i32[nBounds] right cell (-1: none),
    u64 nData, then per entry: u64 name length, name, u64 length, f64[length]

Legacy ASCII VTK export (``Mesh::exportVTK``, core/src/mesh_io.cpp:674-992).

Everything here is host-side file handling with numpy; nothing of it runs
on the GPU.
"""
from __future__ import annotations

import os
import re
import struct
import warnings

import numpy as np

TOLERANCE = 1e-12  # core/src/gimli.h:206

# Token aliases, inserted in this order into a map that keeps the first
# entry of a key (DataContainer::initTokenTranslator, datacontainer.cpp:82-95,
# then DataContainerERT::initTokenTranslator, bertDataContainer.cpp:64-90).
_BASE_ALIASES = (("err", "err std error err/%"), ("t", "t t/s t/ms t/(ms)"))
_ERT_ALIASES = (
    ("a", "a c1"), ("b", "b c2"), ("eca", "ECa EC_a"), ("i", "i i/A i(A) i/mA i(mA)"),
    ("ip", "ip ip/mrad ip/° phase phase/mrad phase/° phi phi/mrad phi/°"),
    ("iperr", "iperr iperr/mrad iperr/° phierr phierr/mrad phierr/°"), ("k", "k"),
    ("m", "m p1"), ("n", "n p2"), ("r", "r rho r(Ohm) imp z u/i"),
    ("rhoa", "rhoa rho_a ra rs rhos rhoa/Ohmm rhoa(Ohmm)"),
    ("u", "u u/V u(V) u/mV u(mV) v v/V v(V) v/mV v(mV)"),
)


def _translator():
    tt = {}
    for groups in (_BASE_ALIASES, _ERT_ALIASES):
        for token, aliases in groups:
            for a in aliases.split():
                tt.setdefault(a, token)
    return tt


TOKEN_TRANSLATOR = _translator()
SENSOR_INDEX_TOKENS = ("a", "b", "m", "n")
ERT_DEFAULT_FIELDS = ("err", "i", "ip", "iperr", "k", "r", "rhoa", "u")


def translate_alias(alias):
    """Token for ``alias`` (first character compared in lower case), or
    None (DataContainer::translateAlias, datacontainer.cpp:96-108)."""
    if not alias:
        return None
    return TOKEN_TRANSLATOR.get(alias[0].lower() + alias[1:])


_FLOAT_PREFIX = re.compile(
    r"\s*([+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan))", re.IGNORECASE)
_INT_PREFIX = re.compile(r"\s*([+-]?\d+)")


def _strtod(s):
    """Leading number of ``s`` like C ``strtod`` (0.0 when there is none)."""
    m = _FLOAT_PREFIX.match(s)
    return float(m.group(1)) if m else 0.0


def _atoi(s):
    m = _INT_PREFIX.match(s)
    return int(m.group(1)) if m else 0


class _Rows:
    """Line reader with the reference's row rules: text after '#' is a
    comment, rows split on whitespace, empty rows are skipped, and a format
    line is a line that starts with '#' directly after a count row."""

    def __init__(self, text):
        self.lines = text.split("\n")
        if self.lines and self.lines[-1] == "":
            self.lines.pop()
        self.pos = 0

    def row(self):
        if self.pos >= len(self.lines):
            return None
        line = self.lines[self.pos]
        self.pos += 1
        return line.split("#", 1)[0].split()

    def non_empty(self):
        while True:
            r = self.row()
            if r is None:
                return []
            if r:
                return r

    def format_line(self):
        if self.pos < len(self.lines) and self.lines[self.pos].startswith("#"):
            line = self.lines[self.pos][1:]
            self.pos += 1
            return line.split("#", 1)[0].split()
        return None


_SENSOR_COLS = {"x": 0, "X": 0, "x/m": 0, "X/m": 0, "y": 1, "Y": 1, "y/m": 1, "Y/m": 1,
                "z": 2, "Z": 2, "z/m": 2, "Z/m": 2}
# the reference's z/mm test lists "z/mm" twice, so "Z/mm" is an unknown column
_SENSOR_MM = {"x/mm": 0, "X/mm": 0, "y/mm": 1, "Y/mm": 1, "z/mm": 2}


class UnifiedData:
    """Parsed content of a unified data file: sensors (S, 3), fields
    (token -> float64 array, sensor indices counted from zero, -1 = none),
    the additional points and the format strings read."""

    def __init__(self, sensors, fields, topo, sensor_format, data_format):
        self.sensors = sensors
        self.fields = fields
        self.topo = topo
        self.sensor_format = sensor_format
        self.data_format = data_format


def read_unified(path, sensorIndicesFromOne=True, removeInvalid=True, verbose=False):
    """``DataContainerERT::load`` (datacontainer.cpp:209-470) restated."""
    with open(path, "r", encoding="utf-8", errors="replace") as f:
        rows = _Rows(f.read())
    row = rows.non_empty()
    if len(row) != 1:
        raise ValueError(f"{path}: cannot determine data format ({len(row)} values in the first row)")
    n_s = _atoi(row[0])
    if n_s < 1:
        raise ValueError(f"{path}: cannot determine sensor count {row[0]}")
    fmt = rows.format_line()
    if fmt is None:
        fmt = ["x", "y", "z"]
    sensor_format = " ".join(fmt)
    xyz = np.zeros((n_s, 3))
    for i in range(n_s):
        row = rows.non_empty()
        if not row:
            raise ValueError(f"{path}: too few sensors, {n_s} expected but {i} found")
        for j, v in enumerate(row):
            if j == len(fmt):
                break
            t = fmt[j]
            if t in _SENSOR_COLS:
                xyz[i, _SENSOR_COLS[t]] = _strtod(v)
            elif t in _SENSOR_MM:
                xyz[i, _SENSOR_MM[t]] = _strtod(v) / 1000.0
            elif verbose:
                warnings.warn(f"sensor format token '{t}' unknown, column ignored")
    xyz = np.rint(xyz / 1e-12) * 1e-12

    # DataContainer::createSensor (datacontainer.cpp:170-184): the last
    # earlier sensor closer than 1e-3 is a duplicate; the sensor is kept for
    # now and its indices are moved to that sensor below.
    duplicated = []
    for i in range(n_s):
        if i:
            d = np.sqrt(((xyz[:i] - xyz[i]) ** 2).sum(axis=1))
            hit = np.nonzero(d < 1e-3)[0]
            if len(hit):
                duplicated.append((i, int(hit[-1])))

    row = rows.non_empty()
    if len(row) != 1:
        raise ValueError(f"{path}: cannot determine data size")
    n_d = _atoi(row[0])
    fields = {t: np.full(max(n_d, 0), -1.0) for t in SENSOR_INDEX_TOKENS}
    fields.update({t: np.zeros(max(n_d, 0)) for t in ERT_DEFAULT_FIELDS})
    dfmt = fmt
    if n_d > 0:
        g = rows.format_line()
        if g is not None:
            if not g:
                raise ValueError(f"{path}: cannot determine data format")
            dfmt = g
    tmp = {}
    for d in range(max(n_d, 0)):
        row = rows.non_empty()
        if not row:
            raise ValueError(f"{path}: too few data, {n_d} expected and {d} found")
        for j, v in enumerate(row):
            if j == len(dfmt):
                break
            if dfmt[j] not in tmp:
                tmp[dfmt[j]] = np.zeros(n_d)
            tmp[dfmt[j]][d] = _strtod(v)
    for name in sorted(tmp):
        tok = translate_alias(name)
        if tok is not None:
            scale = 1.0
            if "mV" in name or "mA" in name or "ms" in name:
                scale = 1.0 / 1000.0
            if "%" in name:
                scale = 1.0 / 100.0
            fields[tok] = tmp[name] * scale
        else:
            fields[name] = tmp[name]
    data_format = " ".join(translate_alias(t) or t for t in dfmt)
    if sensorIndicesFromOne and n_d > 0:
        for t in SENSOR_INDEX_TOKENS:
            fields[t] = fields[t] - 1.0
    fields["valid"] = np.ones(max(n_d, 0))

    sensors = xyz
    if duplicated:
        for old, new in duplicated:
            for t in SENSOR_INDEX_TOKENS:
                v = fields[t]
                v[v == old] = new
        sensors, fields = _remove_unused_sensors(sensors, fields)

    fields = check_validity(fields, len(sensors), remove=removeInvalid, verbose=verbose)

    topo = np.zeros((0, 3))
    row = rows.non_empty()
    if len(row) == 1:
        n_t = _atoi(row[0])
        if n_t > 0:
            tf = rows.format_line()
            if tf is None or tf[0] not in ("x", "X"):
                tf = ["x", "y", "z"]
            topo = np.zeros((n_t, 3))
            for i in range(n_t):
                row = rows.non_empty()
                if not row:
                    raise ValueError(f"{path}: too few topography points, {n_t} expected and {i} found")
                for j, v in enumerate(row):
                    if j == len(tf):
                        break
                    c = {"x": 0, "X": 0, "y": 1, "Y": 1, "z": 2, "Z": 2}.get(tf[j])
                    if c is not None:
                        topo[i, c] = _strtod(v)
    return UnifiedData(sensors, fields, topo, sensor_format, data_format)


def _remove_unused_sensors(sensors, fields):
    """DataContainer::removeUnusedSensors (datacontainer.cpp:801-840)."""
    S = len(sensors)
    active = np.zeros(S, bool)
    for t in SENSOR_INDEX_TOKENS:
        v = fields[t].astype(np.int64)
        ok = (v > -1) & (v < S)
        active[v[ok]] = True
    perm = np.cumsum(active) - 1
    out = dict(fields)
    for t in SENSOR_INDEX_TOKENS:
        v = fields[t].copy()
        iv = v.astype(np.int64)
        ok = (iv > -1) & (iv < S)
        v[ok] = perm[iv[ok]]
        out[t] = v
    return sensors[active], out


def check_validity(fields, n_sensors, remove=True, verbose=False):
    """DataContainer::checkDataValidity (datacontainer.cpp:480-516) with the
    ERT rules of DataContainerERT::checkDataValidityLocal
    (bertDataContainer.cpp:92-148): non-finite values, sensor indices
    outside [-1, sensors), rhoa < 1e-12, |r| < 1e-12 and coinciding
    electrodes mark a datum invalid; ``remove`` drops the invalid data."""
    fields = {k: np.asarray(v, np.float64).copy() for k, v in fields.items()}
    n = len(fields["valid"])
    valid = fields["valid"]
    for k in sorted(fields):
        valid[~np.isfinite(fields[k])] = 0.0
    for t in SENSOR_INDEX_TOKENS:
        v = fields[t]
        valid[(v < -1) | (v >= float(n_sensors))] = 0.0

    def have(t):
        return t in fields and len(fields[t]) > 0 and not (np.max(np.abs(fields[t])) < TOLERANCE)

    def all_nonzero(t):
        return t in fields and len(fields[t]) > 0 and np.min(np.abs(fields[t])) > TOLERANCE

    if n > 0:
        if have("rhoa") or have("r") or have("u"):
            if not all_nonzero("rhoa") and not all_nonzero("r"):
                if all_nonzero("i") and all_nonzero("u"):
                    fields["r"] = fields["u"] / fields["i"]
                elif verbose:
                    warnings.warn("zero current or voltage in the data")
        if have("rhoa"):
            valid[fields["rhoa"] < TOLERANCE] = 0.0
        if have("r"):
            valid[np.abs(fields["r"]) < TOLERANCE] = 0.0
        a, b, m, nn = (fields[t] for t in SENSOR_INDEX_TOKENS)
        bad = (((np.abs(a - b) < TOLERANCE) & (a > 0)) | ((np.abs(a - m) < TOLERANCE) & (a > 0))
               | ((np.abs(a - nn) < TOLERANCE) & (a > 0)) | ((np.abs(b - m) < TOLERANCE) & (b > 0))
               | ((np.abs(b - nn) < TOLERANCE) & (b > 0)) | ((np.abs(m - nn) < TOLERANCE) & (m > 0)))
        valid[bad] = 0.0
    fields["valid"] = valid
    if remove and np.any(valid < 1):
        keep = np.nonzero(valid == 1)[0]
        fields = {k: v[keep] for k, v in fields.items()}
    return fields


def token_list(fields):
    """DataContainer::tokenList(false): sensor index tokens, then the other
    fields, each group in byte order, each token followed by a space."""
    idx = sorted(t for t in fields if t in SENSOR_INDEX_TOKENS)
    rest = sorted(t for t in fields if t not in SENSOR_INDEX_TOKENS)
    return "".join(t + " " for t in idx + rest)


def write_unified(path, sensors, fields, formatData="all", formatSensor="x y z", noFilter=False,
                  sensorIndicesFromOne=True):
    """``DataContainer::save`` / ``write`` (datacontainer.cpp:518-615):
    sensor coordinates with 14 significant digits, sensor indices as
    integers counted from one, other fields in scientific notation with 14
    decimals, tab-separated; ``formatData="all"`` writes every field and
    every datum, otherwise only the valid ones unless ``noFilter``."""
    sensors = np.asarray(sensors, np.float64).reshape(-1, 3)
    valid = fields["valid"]
    out = [f"{len(sensors)}", f"# {formatSensor}"]
    sfmt = formatSensor.split()
    cols = {"x": 0, "X": 0, "y": 1, "Y": 1, "z": 2, "Z": 2}
    for p in sensors:
        out.append("\t".join(("%.14g" % p[cols[t]]) if t in cols else "" for t in sfmt))
    if formatData.lower() == "all":
        idx = np.nonzero(valid > -1)[0]
        fmt = token_list(fields)
    else:
        idx = np.nonzero(valid > -1)[0] if noFilter else np.nonzero(valid == 1)[0]
        fmt = formatData
    tokens = fmt.split()
    vecs = []
    for t in tokens:
        name = translate_alias(t) or t
        if name not in fields:
            raise KeyError(f"no such data: {name}")
        vecs.append((t, name, fields[name]))
    out.append(f"{len(idx)}")
    out.append(f"# {fmt}")
    one = 1 if sensorIndicesFromOne else 0
    for i in idx:
        vals = []
        for t, name, v in vecs:
            if name in SENSOR_INDEX_TOKENS:
                vals.append("%d" % (int(v[i]) + one))
            elif t == "valid":
                vals.append("%d" % int(v[i]))
            else:
                vals.append("%.14e" % v[i])
        out.append("\t".join(vals))
    out.append("0")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    return 1


# -- binary mesh -------------------------------------------------------------

def _bms_name(path):
    path = os.fspath(path)
    return path[:path.rfind(".bms")] + ".bms" if ".bms" in path else path + ".bms"


def write_bms(path, dim, nodes, node_markers, cells, cell_markers, boundaries, boundary_markers,
              left, right, data=None, geometry=False):
    """Mesh::saveBinaryV2 (mesh_io.cpp:391-538), version 3."""
    nodes = np.ascontiguousarray(nodes, "<f8").reshape(-1, 3)
    parts = [struct.pack("<BB", dim, 3), bytes([1 if geometry else 0]) + bytes(127),
             struct.pack("<I", len(nodes))]
    if len(nodes):
        parts += [nodes.tobytes(), np.ascontiguousarray(node_markers, "<i4").tobytes()]

    def elems(conn, markers, extra=()):
        n = len(conn)
        b = [struct.pack("<I", n)]
        if n:
            conn = np.asarray(conn)
            b += [np.full(n, conn.shape[1], np.uint8).tobytes(), np.ascontiguousarray(conn, "<u4").tobytes(),
                  np.ascontiguousarray(markers, "<i4").tobytes()]
            b += [np.ascontiguousarray(e, "<i4").tobytes() for e in extra]
        return b

    parts += elems(cells, cell_markers)
    parts += elems(boundaries, boundary_markers, (left, right))
    data = data or {}
    parts.append(struct.pack("<Q", len(data)))
    for name, v in data.items():
        v = np.ascontiguousarray(v, "<f8")
        nb = name.encode()
        if len(nb) and len(v):
            parts += [struct.pack("<Q", len(nb)), nb, struct.pack("<Q", len(v)), v.tobytes()]
    fname = _bms_name(path)
    with open(fname, "wb") as f:
        f.write(b"".join(parts))
    return fname


def write_bms_v1(path, dim, nodes, node_markers, cells, cell_markers, boundaries, boundary_markers, left, right,
                 geometry=False):
    """The first binary format, Mesh::saveBinary (mesh_io.cpp:98-246): int32
    counts with 127-int32 header blocks, ``dim`` coordinates per node and
    the cell markers as float64 attributes."""
    nodes = np.asarray(nodes, np.float64).reshape(-1, 3)
    head = np.zeros(127, "<i4")
    head[0] = 1 if geometry else 0
    i4 = lambda a: np.ascontiguousarray(a, "<i4").tobytes()  # noqa: E731
    parts = [struct.pack("<i", dim), head.tobytes(), struct.pack("<i", len(nodes)),
             np.ascontiguousarray(nodes[:, :dim], "<f8").tobytes(), i4(node_markers)]
    np0 = np.zeros(127, "<i4").tobytes()
    cells = np.asarray(cells)
    parts += [np0, struct.pack("<i", len(cells)), i4(np.full(len(cells), cells.shape[1] if len(cells) else 0)),
              i4(cells.reshape(-1)), np.ascontiguousarray(cell_markers, "<f8").tobytes()]
    boundaries = np.asarray(boundaries)
    parts += [np0, struct.pack("<i", len(boundaries)),
              i4(np.full(len(boundaries), boundaries.shape[1] if len(boundaries) else 0)),
              i4(boundaries.reshape(-1)), i4(boundary_markers), i4(left), i4(right)]
    fname = _bms_name(path)
    with open(fname, "wb") as f:
        f.write(b"".join(parts))
    return fname


def _read_bms_v1(buf):
    """Mesh::loadBinary (mesh_io.cpp:248-389)."""
    off = 0

    def take(fmt, count=1):
        nonlocal off
        dt = np.dtype(fmt)
        a = np.frombuffer(buf, dt, count, off)
        off += dt.itemsize * count
        return a

    dim = int(take("<i4")[0])
    if dim not in (2, 3):
        raise ValueError(f"cannot determine dimension {dim}")
    geometry = bool(take("<i4", 127)[0])
    n = int(take("<i4")[0])
    nodes = np.zeros((n, 3))
    nodes[:, :dim] = take("<f8", dim * n).reshape(n, dim)
    nmark = take("<i4", n).copy()

    def elems():
        take("<i4", 127)
        c = int(take("<i4")[0])
        nv = take("<i4", c)
        idx = take("<i4", int(nv.sum(dtype=np.int64)))
        if c and np.all(nv == nv[0]):
            return c, idx.reshape(c, int(nv[0])).astype(np.int32)
        if c == 0:
            return 0, np.zeros((0, 0), np.int32)
        cs = np.concatenate([[0], np.cumsum(nv, dtype=np.int64)])
        return c, [idx[cs[i]:cs[i + 1]].astype(np.int32) for i in range(c)]

    C, cells = elems()
    cmark = np.rint(take("<f8", C)).astype(np.int32)
    B, bnd = elems()
    bmark = take("<i4", B).copy()
    left = take("<i4", B).copy()
    right = take("<i4", B).copy()
    return {"dim": dim, "geometry": geometry, "nodes": nodes, "node_markers": nmark, "cells": cells,
            "cell_markers": cmark, "boundaries": bnd, "boundary_markers": bmark, "left": left, "right": right,
            "data": {}}


def read_bms(path):
    """Mesh::load of a binary mesh (mesh_io.cpp:30-49): the v2/v3 format of
    Mesh::loadBinaryV2 (mesh_io.cpp:540-662), else the first format.
    Returns a dict of the arrays (cells and boundaries as (count, nodes)
    arrays when their node counts are uniform)."""
    with open(_bms_name(path), "rb") as f:
        buf = f.read()
    try:
        return _read_bms_v2(buf)
    except ValueError:
        return _read_bms_v1(buf)


def _read_bms_v2(buf):
    off = 0

    def take(fmt, count=1):
        nonlocal off
        dt = np.dtype(fmt)
        a = np.frombuffer(buf, dt, count, off)
        off += dt.itemsize * count
        return a

    dim = int(take("u1")[0])
    if dim not in (2, 3):
        raise ValueError(f"cannot determine dimension {dim}")
    version = int(take("u1")[0])
    geometry = False
    if version == 3:
        geometry = bool(take("u1", 128)[0])
    elif version != 2:
        raise ValueError(f"wrong version {version}")
    n = int(take("<u4")[0])
    if n > 1e9:
        raise ValueError("node count above 1e9")
    nodes = take("<f8", 3 * n).reshape(n, 3).copy() if n else np.zeros((0, 3))
    nmark = take("<i4", n).copy() if n else np.zeros(0, np.int32)

    def elems(with_neighbours):
        c = int(take("<u4")[0])
        if c == 0:
            z = np.zeros((0, 0), np.int32)
            e = np.zeros(0, np.int32)
            return (z, e, e, e) if with_neighbours else (z, e)
        nv = take("u1", c)
        idx = take("<u4", int(nv.sum(dtype=np.int64)))
        mk = take("<i4", c).copy()
        if np.all(nv == nv[0]):
            conn = idx.reshape(c, int(nv[0])).astype(np.int32)
        else:
            cs = np.concatenate([[0], np.cumsum(nv, dtype=np.int64)])
            conn = [idx[cs[i]:cs[i + 1]].astype(np.int32) for i in range(c)]
        if with_neighbours:
            return conn, mk, take("<i4", c).copy(), take("<i4", c).copy()
        return conn, mk

    cells, cmark = elems(False)
    bnd, bmark, left, right = elems(True)
    data = {}
    nd = int(take("<u8")[0])
    for _ in range(nd):
        ln = int(take("<u8")[0])
        name = bytes(take("u1", ln)).decode()
        ld = int(take("<u8")[0])
        data[name] = take("<f8", ld).copy()
    return {"dim": dim, "geometry": geometry, "nodes": nodes, "node_markers": nmark, "cells": cells,
            "cell_markers": cmark, "boundaries": bnd, "boundary_markers": bmark, "left": left, "right": right,
            "data": data}


# -- VTK ----------------------------------------------------------------------

_VTK_CELL_TYPE = {(2, 3): 5, (2, 6): 22, (3, 4): 10, (3, 10): 24}
_VTK_BOUNDARY_TYPE = {(2, 2): 3, (2, 3): 21, (3, 3): 5, (3, 6): 22}
# Tetrahedron10 nodes as exportVTK writes them (old Tet10 numbering style)
_VTK_TET10 = (0, 1, 2, 3, 4, 7, 5, 6, 9, 8)


def _g(v):
    return "%.14g" % v


def write_vtk(path, dim, nodes, cells, cell_markers, boundaries, boundary_markers, data=None,
              write_cells=True, comment="created by pygimli_gb300"):
    """Mesh::exportVTK (mesh_io.cpp:674-992), ASCII legacy format: points,
    cells (or boundaries when ``write_cells`` is false or there are no
    cells) with their types, the cell (boundary) data of matching length
    plus ``Marker``, and the point data of matching length."""
    fname = path[:path.rfind(".vtk")] + ".vtk" if ".vtk" in path else path + ".vtk"
    data = dict(data or {})
    nodes = np.asarray(nodes, np.float64)
    n, C, B = len(nodes), len(cells), len(boundaries)
    out = ["# vtk DataFile Version 3.0", f"d-{dim}__ {comment}", "ASCII", "DATASET UNSTRUCTURED_GRID",
           f"POINTS {n} double"]
    out += [f"{_g(p[0])}\t{_g(p[1])}\t{_g(p[2])}" for p in nodes]

    def scalars(items, count):
        lines = []
        for name in sorted(items):
            v = np.asarray(items[name])
            if len(v) == count:
                lines.append(f"SCALARS {name.replace(' ', '_')} double 1")
                lines.append("LOOKUP_TABLE default")
                lines.append("".join(_g(x) + " " for x in v))
        return lines

    if write_cells and C > 0:
        nv = cells.shape[1]
        out.append(f"CELLS {C} {C * (nv + 1)}")
        if (dim, nv) == (3, 10):
            out += [f"{nv}\t" + "\t".join(str(c[j]) for j in _VTK_TET10) for c in cells]
        else:
            out += [f"{nv}\t" + "".join(f"{x}\t" for x in c) for c in cells]
        out.append(f"CELL_TYPES {C}")
        out.append(f"{_VTK_CELL_TYPE[(dim, nv)]} " * C)
        cdata = dict(data)
        cdata.setdefault("Marker", np.asarray(cell_markers, np.float64))
        out.append(f"CELL_DATA {C}")
        out += scalars(cdata, C)
    elif B > 0:
        nvb = boundaries.shape[1]
        out.append(f"CELLS {B} {B * (nvb + 1)}")
        out += [f"{nvb}\t" + "".join(f"{x}\t" for x in b) for b in boundaries]
        out.append(f"CELL_TYPES {B}")
        out.append(f"{_VTK_BOUNDARY_TYPE[(dim, nvb)]} " * B)
        bdata = dict(data)
        bdata.setdefault("Marker", np.asarray(boundary_markers, np.float64))
        out.append(f"CELL_DATA {B}")
        out += scalars(bdata, B)
    if data:
        out.append(f"POINT_DATA {n}")
        out += scalars(data, n)
    with open(fname, "w") as f:
        f.write("\n".join(out) + "\n")
    return fname


def read_vtk(path):
    """Mesh::importVTK for a legacy ASCII unstructured grid (mesh_io.cpp:
    importVTK, readVTKPoints_, readVTKCells_, readVTKScalars_): the
    dimension from the 'd-2__' / 'd-3__' comment line or the coordinates (no
    z: 2-D; no y but z: 2-D with y and z swapped), POINTS, CELLS (node order as
    written), every SCALARS array into the data map and 'Marker' as the cell
    markers.  CELL_TYPES, boundaries and node markers are not in the file's
    reach of the reference either (markers 0)."""
    fname = path[:path.rfind(".vtk")] + ".vtk" if ".vtk" in path else path + ".vtk"
    with open(fname) as f:
        lines = f.read().split("\n")
    comment = lines[1] if len(lines) > 1 else ""
    dim = 2 if "d-2__" in comment else (3 if "d-3__" in comment else 0)
    i = 2
    while i < len(lines) and lines[i].split()[:1] not in (["ASCII"], ["BINARY"]):
        i += 1
    if i < len(lines) and lines[i].split()[:1] == ["BINARY"]:
        raise ValueError("binary VTK files are not supported")
    i += 1
    if i >= len(lines) or not lines[i].split() or lines[i].split()[-1] != "UNSTRUCTURED_GRID":
        raise ValueError("only unstructured grids are supported")
    toks = " ".join(lines[i + 1:]).split()
    pos = 0
    nodes = np.zeros((0, 3))
    cells = []
    data = {}
    while pos < len(toks):
        t = toks[pos]
        if t == "POINTS":
            nv = int(toks[pos + 1])
            pos += 3
            nodes = np.array([float(v) for v in toks[pos:pos + 3 * nv]]).reshape(nv, 3)
            pos += 3 * nv
            y0 = not np.any(np.abs(nodes[:, 1]) > 1e-12)
            z0 = not np.any(np.abs(nodes[:, 2]) > 1e-12)
            if y0 and not z0:
                dim = 2
                nodes[:, 1], nodes[:, 2] = nodes[:, 2].copy(), 0.0
            elif z0:
                dim = 2
        elif t == "CELLS":
            nc = int(toks[pos + 1])
            pos += 3
            for _ in range(nc):
                k = int(toks[pos])
                cells.append([int(v) for v in toks[pos + 1:pos + 1 + k]])
                pos += 1 + k
        elif t == "SCALARS":
            name = toks[pos + 1]
            pos += 4 if pos + 3 < len(toks) and toks[pos + 3] == "1" else 3
            if toks[pos] == "LOOKUP_TABLE":
                pos += 2
            vals = []
            while pos < len(toks) and toks[pos] not in ("SCALARS", "CELL_DATA", "POINT_DATA", "VECTORS",
                                                           "FIELD", "CELLS", "POINTS", "CELL_TYPES"):
                vals.append(float(toks[pos]))
                pos += 1
            data[name] = np.array(vals)
        else:
            pos += 1
    if dim == 0:
        dim = 3
    nv = {len(c) for c in cells}
    if len(nv) > 1:
        raise ValueError("mixed cell types: only simplex meshes are supported")
    C = len(cells)
    cell_arr = np.array(cells, np.int32).reshape(C, nv.pop() if nv else dim + 1)
    mk = data.get("Marker")
    markers = mk.astype(np.int32) if mk is not None and len(mk) == C else np.zeros(C, np.int32)
    return {"dim": dim, "nodes": nodes, "cells": cell_arr, "cell_markers": markers, "data": data}
