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


def test_every_entry_point_refuses_bad_arguments_before_any_device_call():
    """The C ABI's argument checks that need no device, through ctypes: null
    handles and outputs, unknown types, positive penalties, malformed batch
    offsets and no-alloc sizes past the limits are refused with their status
    (1 invalid argument, 2 too large), on a machine with or without a GPU."""
    import ctypes as C
    L = sg.lib()
    INVALID, TOO_LARGE = 1, 2
    h, u32, u64, i32 = C.c_void_p(), C.c_uint32(), C.c_uint64(), C.c_int32()
    # engines and graphs
    assert L.spoa_gb300_engine_create(3, 5, -4, -8, -6, -10, -4, C.byref(h)) == INVALID
    assert L.spoa_gb300_engine_create(0, 5, -4, 1, -6, -10, -4, C.byref(h)) == INVALID
    assert L.spoa_gb300_engine_create(0, 5, -4, -8, -6, -10, 2, C.byref(h)) == INVALID
    assert L.spoa_gb300_engine_create(0, 5, -4, -8, -6, -10, -4, None) == INVALID
    assert L.spoa_gb300_engine_params(None, None, None, None) == INVALID
    assert L.spoa_gb300_engine_prealloc(None, 100, 4) == INVALID
    assert L.spoa_gb300_engine_align(None, b"ACGT", 4, None, None, None, None, 0, None) == INVALID
    assert L.spoa_gb300_graph_create(None) == INVALID
    assert L.spoa_gb300_graph_clear(None) == INVALID
    assert L.spoa_gb300_graph_add_alignment(None, None, 0, b"A", 1, None, 0) == INVALID
    assert L.spoa_gb300_align_add(None, None, b"A", 1, None, 0, None, None) == INVALID
    assert L.spoa_gb300_graph_consensus(None, None, 0, C.byref(u32)) == INVALID
    assert L.spoa_gb300_graph_msa(None, 0, None, 0, C.byref(u32), C.byref(u32)) == INVALID
    assert L.spoa_gb300_graph_counts(*([None] * 7)) == INVALID
    assert L.spoa_gb300_graph_gfa(None, None, None, 0, None, 0, C.byref(u64)) == INVALID
    L.spoa_gb300_engine_destroy(None)
    L.spoa_gb300_graph_destroy(None)
    # batches
    reads = [b"ACGTACGT", b"ACGTTCGT", b"ACGAACGT"]
    blob = b"".join(reads)
    off = (C.c_uint64 * 4)(0, 8, 16, 24)

    def desc(wro, types=None, **kw):
        d = sg._BatchDesc(type=kw.get("type", 2), m=5, n=-4, g=kw.get("g", -8), e=-6, q=-10,
                          c=-4, n_windows=len(wro) - 1)
        d.window_read_off = C.cast((C.c_uint32 * len(wro))(*wro), C.c_void_p)
        if types is not None:
            d.window_type = C.cast((C.c_int8 * len(types))(*types), C.c_void_p)
        d.seqs = C.cast(C.c_char_p(blob), C.c_void_p)
        d.seq_off = C.cast(off, C.c_void_p)
        return d

    out = C.c_void_p()
    assert L.spoa_gb300_batch_create(None, C.byref(out)) == INVALID
    assert L.spoa_gb300_batch_create(C.byref(desc([0, 3])), None) == INVALID
    assert L.spoa_gb300_batch_create(C.byref(desc([0, 3], type=5)), C.byref(out)) == INVALID
    assert L.spoa_gb300_batch_create(C.byref(desc([0, 3], g=3)), C.byref(out)) == INVALID
    assert L.spoa_gb300_batch_create(C.byref(desc([1, 3])), C.byref(out)) == INVALID
    assert L.spoa_gb300_batch_create(C.byref(desc([0, 3, 1])), C.byref(out)) == INVALID
    assert L.spoa_gb300_batch_create(C.byref(desc([0, 1, 3], types=[2, 9])),
                                     C.byref(out)) == INVALID
    assert not out.value
    assert L.spoa_gb300_batch_launch(None, None) == INVALID
    assert L.spoa_gb300_batch_launch_plain(None, None) == INVALID
    assert L.spoa_gb300_batch_fetch(None, None) == INVALID
    L.spoa_gb300_batch_destroy(None)
    # servers
    assert L.spoa_gb300_server_create(None, C.byref(out)) == INVALID
    assert L.spoa_gb300_server_submit(None, blob, off, 3, 2, 0, 0.0, C.byref(u64)) == INVALID
    assert L.spoa_gb300_server_wait(None, 0, 0.1, None, 0, None, C.byref(i32), None) == INVALID
    assert L.spoa_gb300_server_stats(None, None, None) == INVALID
    assert L.spoa_gb300_server_resident_stats(None, None, None) == INVALID
    L.spoa_gb300_server_destroy(None)
    # the single window that allocates nothing: host-checked arguments and limits
    params = (5, -4, -8, -6, -10, -4)

    dummy = C.c_void_p(1)  # never dereferenced: every call below is refused first

    def noalloc(type_=2, pen=params, n_reads=3, max_len=8, ptr=dummy):
        return L.spoa_gb300_window_poa_noalloc(type_, *pen, 0, n_reads, max_len, ptr, ptr, None,
                                               ptr, 64, ptr, None, ptr, None)
    assert noalloc(type_=4) == INVALID
    assert noalloc(pen=(5, -4, 2, -6, -10, -4)) == INVALID
    assert noalloc(ptr=None) == INVALID
    assert noalloc(n_reads=0) == INVALID
    assert noalloc(n_reads=257) == TOO_LARGE
    assert noalloc(max_len=641) == TOO_LARGE
    assert noalloc(max_len=0) == TOO_LARGE
