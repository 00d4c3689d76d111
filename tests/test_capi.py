"""The C-ABI library loads and exports every declared entry point (CPU)."""
import os
import re

import pytest

import spoa_gb300 as sg
from conftest import ROOT


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"\b(spoa_gb300_\w+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol():
    L = sg.lib()
    declared = _declared()
    assert declared, "no declarations found"
    missing = [n for n in declared if not hasattr(L, n)]
    assert not missing, missing
    assert set(sg.EXPORTED) >= declared


def test_status_strings():
    L = sg.lib()
    assert L.spoa_gb300_status_string(0) == b"ok"
    assert L.spoa_gb300_status_string(3) == b"possible overflow!"


def test_invalid_arguments_rejected_before_any_device_work():
    with pytest.raises(sg.SpoaError, match="invalid alignment type"):
        sg.AlignmentEngine.create(7, 1, -1, -1)
    with pytest.raises(sg.SpoaError, match="gap extension penalty must be non-positive"):
        sg.AlignmentEngine.create(0, 1, -1, -2, 3)


@pytest.mark.skipif(sg.lib().spoa_gb300_device_count() > 0, reason="a GPU is visible")
def test_no_gpu_fails_loudly():
    """No CPU fallback: without a device the compute entry points refuse."""
    with pytest.raises(sg.SpoaError) as ei:
        sg.AlignmentEngine.create(0, 5, -4, -8)
    assert ei.value.status == 10
    with pytest.raises(sg.SpoaError):
        sg.Graph()


def test_graph_entry_points_reject_null_handles():
    """Argument checks of the graph entry points that need no device: null
    handles and missing outputs are refused before any CUDA call."""
    import ctypes as C
    L = sg.lib()
    n = C.c_uint64()
    assert L.spoa_gb300_graph_save(None, None, 0, C.byref(n)) == 1
    assert L.spoa_gb300_graph_load(None, None, 0) == 1
    m = (C.c_uint32 * 4)()
    assert L.spoa_gb300_graph_subgraph(None, 0, 0, None, m, 4) == 1
    assert L.spoa_gb300_graph_export(None, *([None] * 18)) == 1
