"""GHMF_Segment on this library (Applications/MaxFlow/GHMF_Segment.cxx:66-283).

    python -m robartsvtk_gb300.ghmf_segment TreeFilename NumberOfIterations NumberOfDevices Device1 ... DeviceN
        [-output OutputFilename] [-step StepSize] [-cc VanishingRatio]

The tree is a legacy VTK graph file (DIRECTED_GRAPH or TREE) with vertex
arrays "DataTerm" (MetaImage of each leaf's cost), optional "SmoothnessTerm",
"OutputLocation" (file base for a leaf's probabilistic label), "Alpha" and
"Identifier" (the value of a leaf in the merged label map written to
OutputFilename), and optional edge "Weights".  As in the reference, the
labels are solved by the DAG solver (vtkCudaDirectedAcyclicGraphMaxFlowSegmentation)
and merged with the CUDA vote (vtkCudaImageVote: the last leaf of a tie, in
forward-iterator order, wins).  Only one device is used (the first listed).
NumberOfDevices 0 selects the reference's CPU DAG class, which is not
available: its flow magnitude reads past its buffers.
"""
from __future__ import annotations

import sys

import numpy as np

from . import io as hio
from .segmentation import DAGSolver, HMFError, REF_CUDA, vote


def usage() -> str:
    return ("Usage:\t TreeFilename NumberOfIterations NumberOfDevices Device1 ... DeviceN "
            "[-output OutputFilename] [-step StepSize] [-cc VanishingRatio]")


def long_help() -> str:
    return "\n".join([
        "Description:",
        "This file is a utility for applying the GHMF solver. It will take a brief description of the GHMF "
        "hierarchy with associated smoothness/data terms and alphas as well as identifiers and output values",
        "", usage(),
        "The tree is saved in a VTK file with the following attributes:",
        '"DataTerm": (mandatory) filename for the data term',
        '"SmoothnessTerm": (optional) filename for the smoothness term',
        '"OutputLocation": (optional) filename to save probabilistic label to',
        '"Alpha": (optional) filename for the smoothness term',
        '"Identifier": (mandatory iff OutputFilename is specified) unique label integer to associate in merged '
        "file (discrete segmentation)"])


def parse(argv):
    """The reference's argument handling (:77-122): None when it would print
    the usage and stop."""
    if len(argv) < 2:
        return None
    if "help" in argv[1].lower():
        return "help"
    if len(argv) < 5:
        return None
    its, ndev = int(argv[2]), int(argv[3])
    devices = [int(a) for a in argv[4:4 + ndev]]
    nflags = (len(argv) - (3 + ndev) - 1) // 2
    opts = {"tree": argv[1], "iterations": its, "devices": devices, "output": None, "step": 0.1, "cc": 0.25}
    for k in range(nflags):
        cmd, val = argv[4 + ndev + 2 * k], argv[5 + ndev + 2 * k]
        if cmd == "-output":
            opts["output"] = val
        elif cmd == "-step":
            opts["step"] = float(val)
        elif cmd == "-cc":
            opts["cc"] = float(val)
        else:
            return None
    return opts


def run(opts, out=None, err=None) -> int:
    out = out or sys.stdout
    err = err or sys.stderr
    g = hio.read_vtk_graph(opts["tree"])
    if not opts["devices"]:
        print("the CPU DAG solver is not available: the reference's CPU class reads past its flow buffers "
              "(vtkMaxFlowSegmentationUtilities.cxx:197-200); give a CUDA device", file=err)
        return 1
    weights = g.edge_data.get("Weights")
    data_terms = g.vertex_data.get("DataTerm")
    smooth_terms = g.vertex_data.get("SmoothnessTerm")
    out_loc = g.vertex_data.get("OutputLocation")
    alphas = g.vertex_data.get("Alpha")
    identifiers = g.vertex_data.get("Identifier")
    if data_terms is None:
        print('No data terms provided in tree file. (No field named "DataTerm".)', file=out)
    # the image size from the leaves' data terms
    kids = {s for s, _ in g.edges}
    leaves_any = [v for v in range(g.n) if v not in kids]
    images = {}
    meta = None
    for v in leaves_any:
        images[v], m = hio.read_metaimage(data_terms[v])
        meta = meta or m
    shape = next(iter(images.values())).shape
    dims = (shape[2], shape[1], shape[0])
    solver = DAGSolver(dims, g.n, g.edges, weights, device=opts["devices"][0])
    try:
        root = solver.parent.index(-1)
        seen_alpha = set()
        for v in range(g.n):
            if v == root:
                continue
            if v in images:
                solver.set_data(v, np.ascontiguousarray(images[v], dtype=np.float32))
            if smooth_terms and len(smooth_terms) > 0 and smooth_terms[v]:
                s, _ = hio.read_metaimage(smooth_terms[v])
                solver.set_smoothness(v, np.ascontiguousarray(s, dtype=np.float32))
            if alphas is not None and v not in seen_alpha and float(alphas[v]) >= 0.0:
                solver.set_smoothness_scalar(v, float(alphas[v]))  # std::map::insert: the first value stays
                seen_alpha.add(v)
        solver.set_params(opts["iterations"], opts["step"], opts["cc"])
        solver.solve()
        labels = {leaf: solver.labels(leaf) for leaf in solver.leaves}
        for leaf in solver.leaves:
            if out_loc is None or len(out_loc[leaf]) < 1:
                continue
            hio.write_metaimage(out_loc[leaf] + ".mhd", labels[leaf], meta["spacing"], meta["origin"],
                                raw_path=out_loc[leaf] + ".raw")
        if opts["output"] and identifiers is not None:
            ids = [int(identifiers[leaf]) for leaf in solver.leaves]
            merged = vote([labels[leaf] for leaf in solver.leaves], ids, semantics=REF_CUDA)
            hio.write_metaimage(opts["output"] + ".mhd", merged.astype(np.int32), meta["spacing"], meta["origin"],
                                raw_path=opts["output"] + ".raw")
        elif opts["output"]:
            print('Identifiers not given in tree file. (No field named "Identifier".) ', file=err)
    except HMFError as e:
        print("ERROR: %s" % e, file=err)
        return 1
    finally:
        solver.close()
    return 0


def main(argv=None) -> int:
    argv = sys.argv if argv is None else argv
    opts = parse(argv)
    if opts is None:
        print(usage(), file=sys.stderr)
        return 0
    if opts == "help":
        print(long_help(), file=sys.stderr)
        return 0
    return run(opts)


if __name__ == "__main__":
    sys.exit(main())
