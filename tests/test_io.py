"""MetaImage and legacy VTK graph files (robartsvtk_gb300.io) and the
GHMF_Segment argument handling.  CPU only."""
import os
import zlib

import numpy as np
import pytest

from robartsvtk_gb300 import ghmf_segment
from robartsvtk_gb300.io import read_metaimage, read_vtk_graph, write_metaimage, write_vtk_graph


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32, np.uint8, np.int16, np.uint16])
@pytest.mark.parametrize("compress", [False, True])
def test_metaimage_round_trip(tmp_path, dtype, compress):
    rng = np.random.default_rng(1)
    a = (rng.random((5, 7, 9)) * 100).astype(dtype)
    p = str(tmp_path / "img.mhd")
    write_metaimage(p, a, spacing=(0.5, 0.25, 2.0), origin=(1.0, -2.0, 3.5), compress=compress)
    assert os.path.exists(str(tmp_path / "img.raw"))
    b, meta = read_metaimage(p)
    assert b.dtype == a.dtype and b.shape == a.shape and np.array_equal(a, b)
    assert meta["spacing"] == (0.5, 0.25, 2.0) and meta["origin"] == (1.0, -2.0, 3.5)


def test_metaimage_local_big_endian_channels_and_2d(tmp_path):
    a = np.arange(2 * 3 * 4 * 2, dtype=np.int16).reshape(2, 3, 4, 2)
    p = str(tmp_path / "one.mha")
    write_metaimage(p, a)
    b, _ = read_metaimage(p)
    assert np.array_equal(a, b)
    # a hand-written header: MSB data, 2-D, separate file, HeaderSize
    raw = np.arange(12, dtype=">f4").tobytes()
    with open(tmp_path / "d.bin", "wb") as f:
        f.write(b"JUNK" + raw)
    with open(tmp_path / "h.mhd", "w") as f:
        f.write("ObjectType = Image\nNDims = 2\nDimSize = 4 3\nElementType = MET_FLOAT\n"
                "BinaryDataByteOrderMSB = True\nHeaderSize = 4\nElementDataFile = d.bin\n")
    c, _ = read_metaimage(str(tmp_path / "h.mhd"))
    assert c.shape == (1, 3, 4) and np.array_equal(c.reshape(-1), np.arange(12, dtype=np.float32))
    with open(tmp_path / "z.mhd", "w") as f:
        f.write("NDims = 3\nDimSize = 2 2 1\nElementType = MET_UCHAR\nCompressedData = True\n"
                "ElementDataFile = z.raw\n")
    with open(tmp_path / "z.raw", "wb") as f:
        f.write(zlib.compress(bytes([1, 2, 3, 4])))
    assert read_metaimage(str(tmp_path / "z.mhd"))[0].reshape(-1).tolist() == [1, 2, 3, 4]


GRAPH_TEXT = """# vtk DataFile Version 3.0
vtk output
ASCII
DATASET DIRECTED_GRAPH
POINTS 4 float
0 0 0 0 0 0
0 0 0 0 0 0
VERTICES 4
EDGES 4
0 1
0 2
1 3
2 3
EDGE_DATA 4
FIELD FieldData 1
Weights 1 4 float
1 0.5 0.25 2
VERTEX_DATA 4
FIELD FieldData 3
DataTerm 1 4 string

%20
%20
leaf%20three.mhd
Alpha 1 4 double
0 0.1 0.2
0.3
Identifier 1 4 int
0 0 0 7
"""


def test_graph_file(tmp_path):
    p = tmp_path / "g.vtk"
    p.write_text(GRAPH_TEXT)
    g = read_vtk_graph(str(p))
    assert g.n == 4 and g.edges == [(0, 1), (0, 2), (1, 3), (2, 3)] and g.kind == "DIRECTED_GRAPH"
    assert g.edge_data["Weights"] == [1.0, 0.5, 0.25, 2.0]
    assert g.vertex_data["DataTerm"][3] == "leaf three.mhd"
    assert g.vertex_data["Alpha"] == [0.0, 0.1, 0.2, 0.3] and g.vertex_data["Identifier"] == [0, 0, 0, 7]
    q = tmp_path / "h.vtk"
    write_vtk_graph(str(q), g)
    h = read_vtk_graph(str(q))
    assert (h.n, h.edges, h.edge_data, h.vertex_data) == (g.n, g.edges, g.edge_data, g.vertex_data)


def test_cli_arguments():
    assert ghmf_segment.parse(["x"]) is None
    assert ghmf_segment.parse(["x", "--HELP"]) == "help"
    assert ghmf_segment.parse(["x", "t.vtk", "10", "1"]) is None
    o = ghmf_segment.parse(["x", "t.vtk", "10", "2", "0", "3", "-output", "seg", "-step", "0.2", "-cc", "0.5"])
    assert o == {"tree": "t.vtk", "iterations": 10, "devices": [0, 3], "output": "seg", "step": 0.2, "cc": 0.5}
    assert ghmf_segment.parse(["x", "t.vtk", "10", "1", "0", "-bogus", "1"]) is None


def test_cli_without_devices_reports(tmp_path, capsys):
    p = tmp_path / "g.vtk"
    p.write_text(GRAPH_TEXT)
    rc = ghmf_segment.run({"tree": str(p), "iterations": 3, "devices": [], "output": None, "step": 0.1, "cc": 0.25})
    assert rc == 1 and "not available" in capsys.readouterr().err
