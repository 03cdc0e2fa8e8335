"""The C ABI library without a GPU: it builds for sm_103a, loads, exports every
symbol include/hmf.h declares, and fails cleanly where a device is needed."""
import ctypes
import os
import re

import numpy as np
import pytest

from tests.conftest import gpu_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\**\s*\b(hmf_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_abi():
    syms = declared_symbols()
    for must in ("hmf_create", "hmf_destroy", "hmf_set_data", "hmf_set_smoothness", "hmf_set_smoothness_scalar",
                 "hmf_set_params", "hmf_solve", "hmf_get_labels", "hmf_last_error"):
        assert must in syms


def test_library_exports_every_declared_symbol(hmf_lib):
    for name in declared_symbols():
        assert hasattr(hmf_lib, name), name


def test_python_binding_covers_the_header():
    from robartsvtk_gb300 import _capi
    bound = {n for n, _, _ in _capi.SIGNATURES}
    assert bound == set(declared_symbols())


@pytest.mark.skipif(gpu_available(), reason="checks the no-device error path")
def test_create_without_device_reports_error(hmf_lib):
    ctx = ctypes.c_void_p()
    par = (ctypes.c_int * 3)(-1, 0, 0)
    rc = hmf_lib.hmf_create(ctypes.byref(ctx), 4, 4, 4, par, 3, 0, 0)
    assert rc == -4  # HMF_ERR_CUDA
    assert hmf_lib.hmf_last_error(None)
    assert not ctx.value


@pytest.mark.parametrize("parent,code", [
    ([-1], -2), ([1, 0], -2), ([-1, -1, 0], -2), ([-1, 3, 0], -2),
])
def test_create_rejects_bad_trees_before_touching_the_device(hmf_lib, parent, code):
    ctx = ctypes.c_void_p()
    par = (ctypes.c_int * len(parent))(*parent)
    assert hmf_lib.hmf_create(ctypes.byref(ctx), 4, 4, 4, par, len(parent), 0, 0) == code


def test_create_rejects_bad_dims_and_semantics(hmf_lib):
    ctx = ctypes.c_void_p()
    par = (ctypes.c_int * 3)(-1, 0, 0)
    assert hmf_lib.hmf_create(ctypes.byref(ctx), 0, 4, 4, par, 3, 0, 0) == -1
    assert hmf_lib.hmf_create(ctypes.byref(ctx), 4, 4, 4, par, 3, 7, 0) == -1
    assert hmf_lib.hmf_create(ctypes.byref(ctx), (1 << 30) + 1, 4, 4, par, 3, 0, 0) == -1
    assert b"2^30" in hmf_lib.hmf_last_error(None)
    assert hmf_lib.hmf_create(ctypes.byref(ctx), 4, 4, 2**31 - 1, par, 3, 0, 0) == -1
    assert not ctx.value
    f0 = ctypes.c_double()
    f = (ctypes.c_double * 3)()
    assert hmf_lib.hmf_decomposition_energy((1 << 30) + 1, 1, 1, par, 3, None, None, None, 0,
                                            ctypes.byref(f0), f, None) == -1


def test_null_context_is_rejected(hmf_lib):
    assert hmf_lib.hmf_solve(None, None) == -1
    assert hmf_lib.hmf_set_params(None, 1, 0.1, 0.25) == -1
    assert hmf_lib.hmf_destroy(None) == 0


def test_facade_reports_missing_hierarchy():
    from robartsvtk_gb300 import HierarchicalMaxFlowSegmentation
    f = HierarchicalMaxFlowSegmentation()
    assert f.Update() == -1
    assert "Hierarchy" in f.GetLastError()
    f.SetStructure([-1, 0, 0])
    f.SetDataInputDataObject(1, np.zeros((2, 2, 2), np.float32))
    f.SetDataInputDataObject(2, np.zeros((2, 3, 2), np.float32))
    assert f.Update() == -1
    assert "extent" in f.GetLastError()


def test_facade_continue_update_needs_an_update():
    """ContinueUpdate without an Update on the same hierarchy and extent is
    refused before any device work; the graph filter refuses it always."""
    from robartsvtk_gb300 import DirectedAcyclicGraphMaxFlowSegmentation, HierarchicalMaxFlowSegmentation
    f = HierarchicalMaxFlowSegmentation()
    f.SetStructure([-1, 0, 0])
    f.SetDataInputDataObject(1, np.zeros((2, 2, 2), np.float32))
    f.SetDataInputDataObject(2, np.zeros((2, 2, 2), np.float32))
    assert f.ContinueUpdate() == -1
    assert "ContinueUpdate follows an Update" in f.GetLastError()
    g = DirectedAcyclicGraphMaxFlowSegmentation()
    g.SetStructure(3, [(0, 1), (0, 2)])
    assert g.ContinueUpdate() == -1
    assert "label trees" in g.GetLastError()


def test_continue_without_context_is_rejected(hmf_lib):
    assert hmf_lib.hmf_solve_continue(None, None) == -1


def test_facade_clamps_like_vtk():
    from robartsvtk_gb300 import HierarchicalMaxFlowSegmentation
    f = HierarchicalMaxFlowSegmentation()
    f.SetCC(3.0)
    f.SetStepSize(-1.0)
    f.SetNumberOfIterations(-5)
    assert (f.GetCC(), f.GetStepSize(), f.GetNumberOfIterations()) == (1.0, 0.0, 0)
    f.AddSmoothnessScalar(2, 0.5)
    f.AddSmoothnessScalar(2, 0.7)     # std::map::insert keeps the first
    f.AddSmoothnessScalar(3, -1.0)    # rejected
    assert f.SmoothnessScalars == {2: 0.5}
