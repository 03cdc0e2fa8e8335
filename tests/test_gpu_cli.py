"""python -m robartsvtk_gb300.ghmf_segment end to end: a weighted DAG problem
written as MetaImages and a legacy VTK graph file, solved and merged, against
DAGSolver + vote on the same inputs.  GPU only."""
import os
import subprocess
import sys

import numpy as np
import pytest

from robartsvtk_gb300 import REF_CUDA, DAGSolver, vote
from robartsvtk_gb300.io import Graph, read_metaimage, write_metaimage, write_vtk_graph
from tests.golden.cases import dag_problem

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_ghmf_segment_cli(tmp_path):
    w = dag_problem("dag_weighted_11x6x7")
    n = w.n
    data_term, out_loc, ident = [""] * n, [""] * n, [0] * n
    for k, (leaf, d) in enumerate(sorted(w.data.items())):
        p = str(tmp_path / ("d%d.mhd" % leaf))
        write_metaimage(p, d, spacing=(0.5, 0.5, 1.5))
        data_term[leaf] = p
        out_loc[leaf] = str(tmp_path / ("u%d" % leaf))
        ident[leaf] = 10 + k
    smooth_term = [""] * n
    for v, S in w.smooth.items():
        p = str(tmp_path / ("s%d.mhd" % v))
        write_metaimage(p, S)
        smooth_term[v] = p
    alpha = [float(w.alpha.get(v, 0.0)) for v in range(n)]
    g = Graph(n=n, edges=w.edges, vertex_data={"DataTerm": data_term, "SmoothnessTerm": smooth_term,
                                                 "OutputLocation": out_loc, "Alpha": alpha, "Identifier": ident},
              edge_data={"Weights": list(w.weights)})
    tree = str(tmp_path / "tree.vtk")
    write_vtk_graph(tree, g)
    seg = str(tmp_path / "seg")
    r = subprocess.run([sys.executable, "-m", "robartsvtk_gb300.ghmf_segment", tree, str(w.iterations), "1", "0",
                        "-output", seg, "-step", "0.1", "-cc", "0.25"], cwd=ROOT, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    s = DAGSolver(w.dims, n, w.edges, w.weights)
    for leaf, d in w.data.items():
        s.set_data(leaf, d)
    for v, S in w.smooth.items():
        s.set_smoothness(v, S)
    for v in range(1, n):
        s.set_smoothness_scalar(v, alpha[v])
    s.set_params(w.iterations, 0.1, 0.25)
    s.solve()
    labels = {leaf: s.labels(leaf) for leaf in s.leaves}
    for leaf in s.leaves:
        u, meta = read_metaimage(out_loc[leaf] + ".mhd")
        assert np.array_equal(u, labels[leaf]) and meta["spacing"] == (0.5, 0.5, 1.5)
    merged, _ = read_metaimage(seg + ".mhd")
    want = vote([labels[l] for l in s.leaves], [ident[l] for l in s.leaves], semantics=REF_CUDA)
    assert merged.dtype == np.int32 and np.array_equal(merged, want)
    s.close()
