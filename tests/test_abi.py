"""The C-ABI library loads without a GPU and exports every entry point that
include/clbm.h declares; calls that need a device fail with a status code."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (REPO / "include" / "clbm.h").read_text()
    return sorted(set(re.findall(r"\b(clbm_[a-z0-9_]+)\s*\(", text)))


def test_header_declarations_are_known(clbm_lib):
    assert declared_symbols() == sorted(clbm_lib.EXPORTS)


def test_every_declared_symbol_is_exported(clbm_lib):
    L = clbm_lib.lib()
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing


def test_status_strings(clbm_lib):
    L = clbm_lib.lib()
    assert L.clbm_strerror(0) == b"ok"
    assert L.clbm_strerror(-3) == b"device error word set"
    assert L.clbm_version() >= 10000


def test_invalid_arguments_are_rejected(clbm_lib):
    L = clbm_lib.lib()
    h = C.c_void_p()
    assert L.clbm_create(None, 1, 0, 10, 0, C.byref(h)) == clbm_lib.ERR_INVALID
    bad = clbm_lib.RunDesc(width=2, height=2, nclones=1, tau=0.6)
    assert L.clbm_create(C.byref(bad), 1, 0, 10, 0, C.byref(h)) == clbm_lib.ERR_INVALID
    ok = clbm_lib.RunDesc(width=16, height=8, xmin=4, xmax=6, ymin=2, ymax=4, nclones=3, ranks=2, tau=0.6)
    assert L.clbm_create(C.byref(ok), 1, 0, 10, 0, C.byref(h)) == clbm_lib.ERR_INVALID  # ranks
    g = clbm_lib.Geom(2, 2, 0, 0, 0, 0)
    assert L.clbm_ref_walls_bb(C.byref(g), None, None, None) == clbm_lib.ERR_INVALID
    m = np.zeros(16)
    assert L.clbm_ref_random_field(2, 8, 3.0, 1, 0, m.ctypes.data_as(C.c_void_p), None) == clbm_lib.ERR_INVALID
    assert L.clbm_ref_random_field(8, 8, -1.0, 1, 0, m.ctypes.data_as(C.c_void_p), None) == clbm_lib.ERR_INVALID
    assert L.clbm_ref_random_field(8, 8, 3.0, 1, 0, None, None) == clbm_lib.ERR_INVALID


def test_no_device_means_status_not_fallback(clbm_lib):
    if clbm_lib.device_count() > 0:
        pytest.skip("a GPU is present")
    ok = clbm_lib.RunDesc(width=16, height=8, xmin=4, xmax=6, ymin=2, ymax=4, nclones=2, ranks=1, tau=0.6)
    h = C.c_void_p()
    assert clbm_lib.lib().clbm_create(C.byref(ok), 1, 0, 10, 0, C.byref(h)) == clbm_lib.ERR_CUDA


def test_variant_numbering(clbm_lib):
    """The autotuner's variant numbers: 8 streaming launch shapes, then the
    cluster-resident kernel per cluster size (1, 2, 4, 8, 16, 3, 5, 6, 7, 9,
    10, in that order: the sizes that are not powers of two appended) times
    three thread counts (the numbering include/clbm.h documents)."""
    assert clbm_lib.describe_variant(7) == {"kind": "streaming", "kernel": "k_step_f32", "variant": 7}
    sizes = (1, 2, 4, 8, 16, 3, 5, 6, 7, 9, 10)
    for q, cs in enumerate(sizes):
        for tv, threads in enumerate((1024, 512, 256)):
            d = clbm_lib.describe_variant(8 + 3 * q + tv)
            assert (d["kind"], d["cluster_size"], d["threads"]) == ("cluster-resident", cs, threads)
    assert clbm_lib.describe_variant(14)["cluster_size"] == 4  # the powers of two keep their numbers
    assert clbm_lib.describe_variant(23)["cluster_size"] == 3
