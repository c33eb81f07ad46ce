"""VTK XML files the PanNDE runners read and write, without the VTK library.

* ``write_vtu`` / ``read_vtu``: unstructured grids of 8-node hexahedra with
  PointData, CellData and FieldData (``encoding``: ``"binary"`` inline base64,
  ``"ascii"``, or ``"appended"`` raw bytes; ``compress=True`` writes
  vtkZLibDataCompressor blocks).
* ``read_vtt``: tables (RowData columns, FieldData).
* ``read_transducer_job`` / ``read_water_column_job``: the problem a
  TransducerModel / WaterColumnModel runner builds from a job file, as a
  ``cases.Case`` (mesh, per-cell materials, dt, excitation windows).
* ``write_transducer_job``: a TransducerModel job for a ``cases.Case`` in the
  key names of PanNDE's StandardNames.hpp (density and C11..C66 CELL fields;
  FieldData dt, write_times, NTransducers, XD<i>/XCenter, YCenter, ZCenter,
  Radius, SignalTimes, SignalValues) -- the layout the reference's case makers
  produce.

The same subset is read and written in C++ by include/pn_vtu.hpp.
"""
from __future__ import annotations

import base64
import struct
import xml.etree.ElementTree as ET
import zlib

import numpy as np

_TYPES = {"Float64": "<f8", "Float32": "<f4", "Int64": "<i8", "UInt64": "<u8", "Int32": "<i4",
          "UInt32": "<u4", "Int16": "<i2", "UInt16": "<u2", "Int8": "<i1", "UInt8": "<u1"}


def _block(data: bytes, compress: bool) -> bytes:
    """header + data of one array, UInt64 headers"""
    if not compress:
        return struct.pack("<Q", len(data)) + data
    comp = zlib.compress(data)
    return struct.pack("<QQQQ", 1, len(data), len(data), len(comp)) + comp


class _Writer:
    def __init__(self, encoding: str, compress: bool):
        self.encoding, self.compress = encoding, compress
        self.appended = bytearray()

    def array(self, name, values, vtype="Float64", components=1, tuples=None):
        a = np.ascontiguousarray(values, dtype=_TYPES[vtype]).reshape(-1)
        attrs = f'type="{vtype}"' + (f' Name="{name}"' if name else "")
        if components != 1:
            attrs += f' NumberOfComponents="{components}"'
        if tuples is not None:
            attrs += f' NumberOfTuples="{tuples}"'
        if self.encoding == "ascii":
            body = " ".join(repr(float(v)) if vtype.startswith("Float") else str(int(v)) for v in a)
            return f'<DataArray {attrs} format="ascii">{body}</DataArray>'
        blk = _block(a.tobytes(), self.compress)
        if self.encoding == "appended":
            off = len(self.appended)
            self.appended += blk
            return f'<DataArray {attrs} format="appended" offset="{off}"/>'
        if self.compress:  # header and data as two base64 units
            hdr_len = 8 * 4
            text = base64.b64encode(blk[:hdr_len]).decode() + base64.b64encode(blk[hdr_len:]).decode()
        else:
            text = base64.b64encode(blk).decode()
        return f'<DataArray {attrs} format="binary">{text}</DataArray>'


def write_vtu(path, points, hexes, point_data=None, cell_data=None, field_data=None,
              encoding="binary", compress=False):
    """points [n, 3], hexes [m, 8] (corner order as PanNDE's meshes);
    *_data: {name: array}; field_data arrays are 1-D."""
    w = _Writer(encoding, compress)
    pts = np.asarray(points, dtype=np.float64).reshape(-1, 3)
    hx = np.asarray(hexes, dtype=np.int64).reshape(-1, 8)
    parts = []
    if field_data:
        parts.append("<FieldData>" + "".join(
            w.array(k, np.atleast_1d(v), tuples=np.atleast_1d(v).size) for k, v in field_data.items())
            + "</FieldData>")
    piece = [f'<Piece NumberOfPoints="{len(pts)}" NumberOfCells="{len(hx)}">',
             "<PointData>" + "".join(w.array(k, v) for k, v in (point_data or {}).items()) + "</PointData>",
             "<CellData>" + "".join(w.array(k, v) for k, v in (cell_data or {}).items()) + "</CellData>",
             "<Points>" + w.array("Points", pts, components=3) + "</Points>",
             "<Cells>" + w.array("connectivity", hx, "Int64") +
             w.array("offsets", 8 * np.arange(1, len(hx) + 1), "Int64") +
             w.array("types", np.full(len(hx), 12), "UInt8") + "</Cells>", "</Piece>"]
    head = ('<?xml version="1.0"?>\n<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" '
            'header_type="UInt64"' + (' compressor="vtkZLibDataCompressor"' if compress else "") + ">")
    xml = head + "<UnstructuredGrid>" + "".join(parts) + "".join(piece) + "</UnstructuredGrid>"
    with open(path, "wb") as f:
        f.write(xml.encode())
        if encoding == "appended":
            f.write(b'<AppendedData encoding="raw">_' + bytes(w.appended) + b"</AppendedData>")
        f.write(b"</VTKFile>\n")


def _decode(elem, info, appended):
    vtype = elem.get("type", "Float64")
    fmt = elem.get("format", "ascii")
    dt = np.dtype(_TYPES[vtype])
    if fmt == "ascii":
        return np.array((elem.text or "").split(), dtype=np.float64).astype(dt)
    hs = 8 if info["header"] == "UInt64" else 4
    hc = "Q" if hs == 8 else "I"
    hfmt = "<" + hc
    if fmt == "binary":
        text = "".join((elem.text or "").split())
        if info["zlib"]:
            raise ValueError("inline compressed arrays: use the C++ reader")
        raw = base64.b64decode(text)
        n = struct.unpack(hfmt, raw[:hs])[0]
        return np.frombuffer(raw[hs:hs + n], dtype=dt)
    off = int(elem.get("offset", "0"))
    data = appended[off:]
    if info["zlib"]:
        nb = struct.unpack(hfmt, data[:hs])[0]
        sizes = struct.unpack("<" + hc * nb, data[3 * hs:(3 + nb) * hs])
        p = (3 + nb) * hs
        out = b""
        for s in sizes:
            out += zlib.decompress(data[p:p + s])
            p += s
        return np.frombuffer(out, dtype=dt)
    n = struct.unpack(hfmt, data[:hs])[0]
    return np.frombuffer(data[hs:hs + n], dtype=dt)


def _parse(path):
    raw = open(path, "rb").read()
    appended = b""
    k = raw.find(b"<AppendedData")
    if k >= 0:  # raw bytes follow: parse the XML before them, closed by hand
        us = raw.index(b"_", k)
        appended = raw[us + 1:raw.rindex(b"</AppendedData>")]
        raw = raw[:k] + b"</VTKFile>"
    root = ET.fromstring(raw)
    info = {"header": root.get("header_type", "UInt32"), "zlib": "ZLib" in root.get("compressor", "")}
    return root, info, appended


def read_vtu(path) -> dict:
    """{"points" [n,3], "hexes" [m,8], "point_data", "cell_data", "field_data"}"""
    root, info, app = _parse(path)
    out = {"point_data": {}, "cell_data": {}, "field_data": {}}
    for sec, key in (("PointData", "point_data"), ("CellData", "cell_data"), ("FieldData", "field_data")):
        for s in root.iter(sec):
            for e in s.iter("DataArray"):
                out[key][e.get("Name")] = _decode(e, info, app)
    pts = next(root.iter("Points")).find("DataArray")
    out["points"] = _decode(pts, info, app).astype(np.float64).reshape(-1, 3)
    cells = {e.get("Name"): _decode(e, info, app) for e in next(root.iter("Cells")).iter("DataArray")}
    out["hexes"] = cells["connectivity"].astype(np.int64).reshape(-1, 8)
    return out


def read_vtt(path) -> dict:
    """{"columns": {name: array}, "field_data": {name: array}}"""
    root, info, app = _parse(path)
    cols = {e.get("Name"): _decode(e, info, app) for s in root.iter("RowData") for e in s.iter("DataArray")}
    fd = {e.get("Name"): _decode(e, info, app) for s in root.iter("FieldData") for e in s.iter("DataArray")}
    return {"columns": cols, "field_data": fd}


CIJ_NAMES = [f"C{i + 1}{j + 1}" for i in range(6) for j in range(i, 6)]  # the 21 in StandardNames order


def write_transducer_job(path, case, write_times, **kw):
    """A TransducerModel job for ``case`` (its force sources become XD<i>
    transducers: centre, radius, signal; the runners take the window
    thickness from the mesh)."""
    from . import _native as N
    m = case.mesh
    cell = {"density": case.density[case.cell_material]}
    for k, name in enumerate(CIJ_NAMES):
        cell[name] = case.cij[case.cell_material, k]
    xds = [s for s in case.sources if s.kind == N.PN_SOURCE_FORCE and s.component == 2]
    fd = {"dt": np.array([case.dt]), "write_times": np.asarray(write_times, dtype=np.float64),
          "NTransducers": np.array([float(len(xds))])}
    for i, s in enumerate(xds):
        fd[f"XD{i}/XCenter"] = np.array([s.center[0]])
        fd[f"XD{i}/YCenter"] = np.array([s.center[1]])
        fd[f"XD{i}/ZCenter"] = np.array([s.center[2]])
        fd[f"XD{i}/Radius"] = np.array([s.radius])
        fd[f"XD{i}/SignalTimes"] = np.asarray(s.times, dtype=np.float64)
        fd[f"XD{i}/SignalValues"] = np.asarray(s.values, dtype=np.float64)
    pts = np.stack([m.x, m.y, m.z], axis=1)
    write_vtu(path, pts, m.hexes, cell_data=cell, field_data=fd, **kw)


def write_water_column_job(path, case, write_times, **kw):
    """A WaterColumnModel job for ``case``: its moment sources, grouped, become
    WC<i> excitations (centre, radius, signal times and the sigma_xx / yy /
    zz signals of components 0 / 1 / 2)."""
    from . import _native as N
    m = case.mesh
    cell = {"density": case.density[case.cell_material]}
    for k, name in enumerate(CIJ_NAMES):
        cell[name] = case.cij[case.cell_material, k]
    groups = {}
    for s in case.sources:
        if s.kind == N.PN_SOURCE_MOMENT and s.component in (0, 1, 2):
            groups.setdefault(s.group, {})[s.component] = s
    fd = {"dt": np.array([case.dt]), "write_times": np.asarray(write_times, dtype=np.float64),
          "NWaterColumns": np.array([float(len(groups))])}
    for i, g in enumerate(sorted(groups)):
        comp = groups[g]
        s0 = comp[min(comp)]
        fd[f"WC{i}/XCenter"] = np.array([s0.center[0]])
        fd[f"WC{i}/YCenter"] = np.array([s0.center[1]])
        fd[f"WC{i}/ZCenter"] = np.array([s0.center[2]])
        fd[f"WC{i}/Radius"] = np.array([s0.radius])
        fd[f"WC{i}/SignalTimes"] = np.asarray(s0.times, dtype=np.float64)
        for c, key in ((0, "SignalSigmaXX"), (1, "SignalSigmaYY"), (2, "SignalSigmaZZ")):
            vals = comp[c].values if c in comp else np.zeros_like(s0.values)
            fd[f"WC{i}/{key}"] = np.asarray(vals, dtype=np.float64)
    pts = np.stack([m.x, m.y, m.z], axis=1)
    write_vtu(path, pts, m.hexes, cell_data=cell, field_data=fd, **kw)


def _job_base(path):
    """Mesh, materials (the cells' density and C11..C66, one row per distinct
    cell) and FieldData of a job file."""
    from . import cases
    d = read_vtu(path)
    pts, hexes = d["points"], d["hexes"].astype(np.int32)
    mesh = cases.HexMesh(pts[:, 0].copy(), pts[:, 1].copy(), pts[:, 2].copy(), hexes)
    cd = d["cell_data"]
    rows = np.stack([np.asarray(cd["density"], np.float64)] +
                    [np.asarray(cd[k], np.float64) for k in CIJ_NAMES], axis=1)
    uniq, cell_mat = np.unique(rows, axis=0, return_inverse=True)
    fd = d["field_data"]
    # window thickness: |z(corner 0) - z(corner 6)| of cell 0 (Boss.hpp:530-536, 650-658)
    ds = abs(float(mesh.z[hexes[0, 0]]) - float(mesh.z[hexes[0, 6]]))
    return mesh, uniq[:, 0].copy(), uniq[:, 1:].copy(), cell_mat.reshape(-1).astype(np.int32), fd, ds


def read_transducer_job(path, sensors=None, nsteps=0):
    """The problem TransducerModel builds from a job: each XD<i> a z-force
    window (HostNormalXDZ: centre, Radius, the thickness of cell 0) with its
    SignalTimes / SignalValues (Boss.hpp:496-524)."""
    from . import _native as N
    from . import cases
    mesh, rho, cij, cell_mat, fd, ds = _job_base(path)
    src = []
    for i in range(int(fd["NTransducers"][0])):
        center = tuple(float(fd[f"XD{i}/{a}Center"][0]) for a in "XYZ")
        src.append(cases.WindowSource(N.PN_SOURCE_FORCE, i, 2, center, float(fd[f"XD{i}/Radius"][0]), ds,
                                      np.asarray(fd[f"XD{i}/SignalTimes"], np.float64),
                                      np.asarray(fd[f"XD{i}/SignalValues"], np.float64)))
    sens = np.zeros(0, np.int32) if sensors is None else np.asarray(sensors, np.int32)
    return cases.Case(str(path), mesh, rho, cij, cell_mat, float(fd["dt"][0]), src, sens, nsteps,
                      dict(write_times=np.asarray(fd["write_times"], np.float64)))


def read_water_column_job(path, sensors=None, nsteps=0):
    """The problem WaterColumnModel builds from a job: each WC<i> three
    moment windows (xx, yy, zz: SignalSigmaXX / YY / ZZ over SignalTimes) at
    one centre and radius, thickness of cell 0 (Boss.hpp:580-660)."""
    from . import _native as N
    from . import cases
    mesh, rho, cij, cell_mat, fd, ds = _job_base(path)
    src = []
    for i in range(int(fd["NWaterColumns"][0])):
        center = tuple(float(fd[f"WC{i}/{a}Center"][0]) for a in "XYZ")
        t = np.asarray(fd[f"WC{i}/SignalTimes"], np.float64)
        for comp, key in ((0, "SignalSigmaXX"), (1, "SignalSigmaYY"), (2, "SignalSigmaZZ")):
            src.append(cases.WindowSource(N.PN_SOURCE_MOMENT, i, comp, center, float(fd[f"WC{i}/Radius"][0]), ds,
                                          t, np.asarray(fd[f"WC{i}/{key}"], np.float64)))
    sens = np.zeros(0, np.int32) if sensors is None else np.asarray(sensors, np.int32)
    return cases.Case(str(path), mesh, rho, cij, cell_mat, float(fd["dt"][0]), src, sens, nsteps,
                      dict(write_times=np.asarray(fd["write_times"], np.float64)))
