"""On-disk formats around a solve.

* MetaImage (`.mhd` header + `.raw` data, or one `.mha`): the images the
  reference's GHMF_Segment reads and writes with vtkMetaImageReader /
  vtkMetaImageWriter (Applications/MaxFlow/GHMF_Segment.cxx:182-246).
  Arrays are [z, y, x] (plus a trailing channel axis for multi-channel
  images), x fastest, as VTK stores scalars.
* Legacy VTK graph files (ASCII): the label hierarchy GHMF_Segment reads
  with vtkGraphReader / vtkTreeReader (:125-140) -- DATASET DIRECTED_GRAPH or
  TREE with VERTICES, EDGES and FIELD arrays in VERTEX_DATA / EDGE_DATA
  (string, integer and floating arrays; strings %-encoded as the VTK legacy
  writer encodes them).
"""
from __future__ import annotations

import os
import re
import zlib
from dataclasses import dataclass, field

import numpy as np

__all__ = ["read_metaimage", "write_metaimage", "Graph", "read_vtk_graph", "write_vtk_graph"]

_MET_TYPES = {
    "MET_CHAR": np.int8, "MET_UCHAR": np.uint8, "MET_SHORT": np.int16, "MET_USHORT": np.uint16,
    "MET_INT": np.int32, "MET_UINT": np.uint32, "MET_LONG": np.int32, "MET_ULONG": np.uint32,
    "MET_LONG_LONG": np.int64, "MET_ULONG_LONG": np.uint64, "MET_FLOAT": np.float32, "MET_DOUBLE": np.float64,
}
_NP_TO_MET = {np.dtype(np.int8): "MET_CHAR", np.dtype(np.uint8): "MET_UCHAR", np.dtype(np.int16): "MET_SHORT",
              np.dtype(np.uint16): "MET_USHORT", np.dtype(np.int32): "MET_INT", np.dtype(np.uint32): "MET_UINT",
              np.dtype(np.int64): "MET_LONG_LONG", np.dtype(np.uint64): "MET_ULONG_LONG",
              np.dtype(np.float32): "MET_FLOAT", np.dtype(np.float64): "MET_DOUBLE"}


def _true(v: str) -> bool:
    return v.strip().lower() in ("true", "1", "yes")


def read_metaimage(path: str):
    """Returns (array, meta): meta holds 'spacing' and 'origin' (x, y, z) and
    the raw header fields under 'header'."""
    with open(path, "rb") as f:
        blob = f.read()
    header = {}
    pos = 0
    data_file = None
    while pos < len(blob):
        end = blob.find(b"\n", pos)
        if end < 0:
            end = len(blob)
        line = blob[pos:end].decode("latin-1").strip()
        pos = end + 1
        if not line or "=" not in line:
            continue
        key, val = (s.strip() for s in line.split("=", 1))
        header[key] = val
        if key == "ElementDataFile":
            data_file = val
            break
    if data_file is None:
        raise ValueError("%s: no ElementDataFile" % path)
    ndims = int(header.get("NDims", "3"))
    dims = [int(v) for v in header["DimSize"].split()][:ndims]
    while len(dims) < 3:
        dims.append(1)
    etype = header.get("ElementType", "MET_FLOAT")
    if etype not in _MET_TYPES:
        raise ValueError("%s: unsupported ElementType %s" % (path, etype))
    dtype = np.dtype(_MET_TYPES[etype])
    msb = _true(header.get("BinaryDataByteOrderMSB", header.get("ElementByteOrderMSB", "False")))
    dtype = dtype.newbyteorder(">" if msb else "<")
    channels = int(header.get("ElementNumberOfChannels", "1"))
    count = dims[0] * dims[1] * dims[2] * channels
    if data_file == "LOCAL":
        raw = blob[pos:]
    else:
        if data_file.startswith("LIST") or "%" in data_file:
            raise ValueError("%s: multi-file MetaImages are not supported" % path)
        with open(os.path.join(os.path.dirname(path), data_file), "rb") as f:
            raw = f.read()
    if _true(header.get("CompressedData", "False")):
        raw = zlib.decompress(raw)
    hs = int(header.get("HeaderSize", "0"))
    nbytes = count * dtype.itemsize
    if hs == -1:
        raw = raw[len(raw) - nbytes:]
    elif hs > 0:
        raw = raw[hs:]
    if len(raw) < nbytes:
        raise ValueError("%s: %d data bytes, %d expected" % (path, len(raw), nbytes))
    arr = np.frombuffer(raw[:nbytes], dtype=dtype).astype(dtype.newbyteorder("="))
    shape = (dims[2], dims[1], dims[0]) + ((channels,) if channels > 1 else ())
    sp = [float(v) for v in header.get("ElementSpacing", header.get("ElementSize", "1 1 1")).split()]
    org = [float(v) for v in header.get("Offset", header.get("Position", header.get("Origin", "0 0 0"))).split()]
    meta = {"spacing": tuple((sp + [1.0] * 3)[:3]), "origin": tuple((org + [0.0] * 3)[:3]), "header": header}
    return arr.reshape(shape), meta


def write_metaimage(path: str, array, spacing=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0), raw_path: str | None = None,
                    compress: bool = False) -> None:
    """Writes `array` ([z, y, x] or [z, y, x, c]) as `path` (.mhd) plus the
    data file `raw_path` (default: path with .raw), the fields vtkMetaImageWriter
    writes; a .mha path keeps the data in the same file."""
    a = np.ascontiguousarray(array)
    if a.dtype not in _NP_TO_MET:
        raise ValueError("unsupported element type %s" % a.dtype)
    channels = a.shape[3] if a.ndim == 4 else 1
    z, y, x = a.shape[:3]
    local = path.lower().endswith(".mha")
    if raw_path is None and not local:
        raw_path = os.path.splitext(path)[0] + ".raw"
    payload = a.astype(a.dtype.newbyteorder("<")).tobytes()
    if compress:
        payload = zlib.compress(payload)
    lines = ["ObjectType = Image", "NDims = 3", "BinaryData = True", "BinaryDataByteOrderMSB = False",
             "CompressedData = %s" % ("True" if compress else "False")]
    if compress:
        lines.append("CompressedDataSize = %d" % len(payload))
    lines += ["TransformMatrix = 1 0 0 0 1 0 0 0 1", "Offset = %s" % " ".join("%.17g" % v for v in origin),
              "CenterOfRotation = 0 0 0", "AnatomicalOrientation = RAI",
              "ElementSpacing = %s" % " ".join("%.17g" % v for v in spacing), "DimSize = %d %d %d" % (x, y, z)]
    if channels > 1:
        lines.append("ElementNumberOfChannels = %d" % channels)
    lines += ["ElementType = %s" % _NP_TO_MET[a.dtype],
              "ElementDataFile = %s" % ("LOCAL" if local else os.path.basename(raw_path))]
    text = ("\n".join(lines) + "\n").encode("latin-1")
    with open(path, "wb") as f:
        f.write(text)
        if local:
            f.write(payload)
    if not local:
        with open(raw_path, "wb") as f:
            f.write(payload)


@dataclass
class Graph:
    """A graph file's content: vertices 0..n-1, edges (source, target) in edge
    order, vertex / edge arrays by name (one value per vertex / edge)."""
    n: int
    edges: list
    kind: str = "DIRECTED_GRAPH"
    vertex_data: dict = field(default_factory=dict)
    edge_data: dict = field(default_factory=dict)

    def parents(self, v):
        return [s for s, t in self.edges if t == v]

    def children(self, v):
        return [t for s, t in self.edges if s == v]


def _decode(s: str) -> str:
    return re.sub(r"%([0-9A-Fa-f]{2})", lambda m: chr(int(m.group(1), 16)), s)


def _encode(s: str) -> str:
    return "".join(c if (c.isprintable() and c not in " %\"") else "%%%02X" % ord(c) for c in s)


_INT_TYPES = {"bit", "char", "unsigned_char", "short", "unsigned_short", "int", "unsigned_int", "long",
              "unsigned_long", "vtkIdType", "vtktypeint64", "vtktypeuint64", "idtype"}


def read_vtk_graph(path: str) -> Graph:
    """Reads a legacy ASCII VTK graph or tree file."""
    with open(path, "r", encoding="latin-1") as f:
        lines = [ln.rstrip("\n") for ln in f]
    if len(lines) < 4 or not lines[0].startswith("# vtk DataFile"):
        raise ValueError("%s: not a legacy VTK file" % path)
    if lines[2].strip().upper() != "ASCII":
        raise ValueError("%s: only ASCII legacy files are supported" % path)
    i = 3

    def next_line():
        nonlocal i
        while i < len(lines) and not lines[i].strip():
            i += 1
        if i >= len(lines):
            return None
        ln = lines[i]
        i += 1
        return ln

    def numbers(count, conv):
        out = []
        while len(out) < count:
            ln = next_line()
            if ln is None:
                raise ValueError("%s: unexpected end of file" % path)
            out.extend(conv(t) for t in ln.split())
        return out[:count]

    def read_arrays(n_arrays):
        nonlocal i
        arrays = {}
        for _ in range(n_arrays):
            head = next_line().split()
            name, comps, tuples, typ = _decode(head[0]), int(head[1]), int(head[2]), head[3].lower()
            count = comps * tuples
            if typ == "string" or typ == "utf8_string":
                vals = []  # one value per line, empty lines included
                while len(vals) < count:
                    if i >= len(lines):
                        raise ValueError("%s: unexpected end of file" % path)
                    vals.append(_decode(lines[i].strip()))
                    i += 1
            elif typ in _INT_TYPES:
                vals = numbers(count, int)
            else:
                vals = numbers(count, float)
            if comps > 1:
                vals = [vals[k * comps:(k + 1) * comps] for k in range(tuples)]
            arrays[name] = vals
        return arrays

    kind, n, edges = "DIRECTED_GRAPH", None, []
    vdata, edata = {}, {}
    target = None
    while True:
        ln = next_line()
        if ln is None:
            break
        parts = ln.split()
        key = parts[0].upper()
        if key == "DATASET":
            kind = parts[1].upper()
        elif key == "POINTS":
            numbers(3 * int(parts[1]), float)
        elif key == "VERTICES":
            n = int(parts[1])
        elif key == "EDGES":
            m = int(parts[1])
            vals = numbers(2 * m, int)
            edges = [(vals[2 * k], vals[2 * k + 1]) for k in range(m)]
        elif key == "VERTEX_DATA":
            target = vdata
        elif key == "EDGE_DATA":
            target = edata
        elif key == "FIELD":
            arrays = read_arrays(int(parts[2]))
            if target is not None:
                target.update(arrays)
        elif key in ("SCALARS",):
            name, typ = _decode(parts[1]), parts[2].lower()
            comps = int(parts[3]) if len(parts) > 3 else 1
            count_owner = n if target is vdata else len(edges)
            nxt = next_line()
            if not nxt.upper().startswith("LOOKUP_TABLE"):
                i -= 1
            vals = numbers(comps * count_owner, int if typ in _INT_TYPES else float)
            if target is not None:
                target[name] = vals
        else:
            raise ValueError("%s: unsupported section %s" % (path, parts[0]))
    if n is None:
        n = 1 + max([max(e) for e in edges] or [0])
    return Graph(n=n, edges=edges, kind=kind, vertex_data=vdata, edge_data=edata)


def write_vtk_graph(path: str, g: Graph) -> None:
    """Writes a legacy ASCII VTK graph file (the layout read_vtk_graph reads)."""
    out = ["# vtk DataFile Version 3.0", "vtk output", "ASCII", "DATASET %s" % g.kind,
           "POINTS %d float" % g.n]
    out += ["0 0 0"] * g.n
    out += ["VERTICES %d" % g.n, "EDGES %d" % len(g.edges)] + ["%d %d" % e for e in g.edges]

    def arrays(header, count, data):
        if not data:
            return []
        lines = ["%s %d" % (header, count), "FIELD FieldData %d" % len(data)]
        for name, vals in data.items():
            if vals and isinstance(vals[0], str):
                lines.append("%s 1 %d string" % (_encode(name), len(vals)))
                lines += [_encode(v) for v in vals]
            elif vals and all(isinstance(v, (int, np.integer)) for v in vals):
                lines.append("%s 1 %d int" % (_encode(name), len(vals)))
                lines.append(" ".join(str(int(v)) for v in vals))
            else:
                lines.append("%s 1 %d double" % (_encode(name), len(vals)))
                lines.append(" ".join("%.17g" % float(v) for v in vals))
        return lines

    out += arrays("EDGE_DATA", len(g.edges), g.edge_data)
    out += arrays("VERTEX_DATA", g.n, g.vertex_data)
    with open(path, "w", encoding="latin-1") as f:
        f.write("\n".join(out) + "\n")
