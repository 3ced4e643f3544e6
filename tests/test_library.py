"""The C-ABI library builds, loads and exports every symbol the header declares
(no GPU needed: nothing here launches a kernel)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "flowket_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fk_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def built():
    from flowket_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    names = _declared()
    for must in ("fk_find_conn_heisenberg", "fk_ar2d_forward", "fk_ar2d_sample", "fk_ar2d_backward",
                 "fk_local_energy_reduce", "fk_adam_step"):
        assert must in names


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_binding_covers_header(built):
    from flowket_gb300 import _lib
    _lib.load()
    bound = set(_lib._SIGNATURES)
    missing = [n for n in _declared() if n not in bound]
    assert not missing, missing


def test_descriptor_queries_without_gpu(built):
    from flowket_gb300 import _lib
    from flowket_gb300.machines import ar2d_param_layout
    lib = _lib.load()
    for (h, w, d, f, wn) in [(4, 4, 5, 16, 0), (10, 10, 10, 32, 1), (16, 16, 20, 64, 1)]:
        desc = _lib.Ar2dDesc(h, w, d, f, wn, 1)
        n = lib.fk_ar2d_num_params(ctypes.byref(desc))
        assert n == ar2d_param_layout(d, f, bool(wn))[1]
        assert lib.fk_ar2d_workspace_bytes(ctypes.byref(desc), 4096, 1) > 0
    # 42,756 parameters for depth 5, 16 channels without weight norm (the reference's 4x4 machine)
    assert lib.fk_ar2d_num_params(ctypes.byref(_lib.Ar2dDesc(4, 4, 5, 16, 0, 1))) == 42756
    # the FP16-operand format has the BF16 layout and workspace sizes
    d16, d32 = _lib.Ar2dDesc(10, 10, 10, 32, 1, 2), _lib.Ar2dDesc(10, 10, 10, 32, 1, 1)
    assert lib.fk_ar2d_packed_bytes(ctypes.byref(d16)) == lib.fk_ar2d_packed_bytes(ctypes.byref(d32)) > 0
    assert (lib.fk_ar2d_workspace_bytes(ctypes.byref(d16), 4096, 1) ==
            lib.fk_ar2d_workspace_bytes(ctypes.byref(d32), 4096, 1))
    assert lib.fk_ar2d_num_params(ctypes.byref(_lib.Ar2dDesc(4, 4, 5, 16, 0, 3))) < 0
    bad = _lib.Ar2dDesc(4, 4, 5, 24, 0, 1)
    assert lib.fk_ar2d_num_params(ctypes.byref(bad)) < 0
    assert b"channels" in lib.fk_last_error()


def test_bad_arguments_are_rejected_without_launch(built):
    from flowket_gb300 import _lib
    lib = _lib.load()
    st = lib.fk_find_conn_heisenberg(None, 1, 4, 4, 2, 1, 1, None, None, None, None, None)
    assert st == -1 and b"NULL" in lib.fk_last_error()
    st = lib.fk_adam_step(None, None, None, None, 4, 0, 1e-3, 0.9, 0.999, 1e-7, None)
    assert st == -1


def test_sr_gram_entry_points_check_arguments_without_launch(built):
    """The block-by-block and split-operand Gram entry points and the
    streamed SR Gram reject bad arguments on the host, before any launch,
    and their size queries answer without a GPU."""
    import ctypes
    from flowket_gb300 import _lib
    lib = _lib.load()
    # split operands: rows padded to 32, columns to 256, bf16 hi + lo
    assert lib.fk_sr_gram_split_bytes(100, 300) == 2 * 128 * 512 * 2
    assert lib.fk_sr_gram_split_bytes(0, 8) == 0
    assert lib.fk_sr_gram_split_bytes(-1, 8) == -1
    assert lib.fk_sr_gram_split(None, None, 8, 8, 4, 8, None, 0, None) == -1
    assert lib.fk_sr_center_split(None, None, 8, 8, 4, 16, 1, None, 0, None) == -1
    assert lib.fk_sr_gram_split_accumulate(None, 4, 8, None, None) == -1
    assert lib.fk_sr_gram_accumulate(None, 4, 8, None, 0, None) == -1
    assert lib.fk_sr_gram_mirror(None, 8, None) == -1
    d = _lib.Ar2dDesc(4, 4, 3, 16, 1, _lib.PRECISIONS["bf16"], 0)
    assert lib.fk_ar2d_sr_gram_workspace_bytes(ctypes.byref(d), 64) > 0
    cc = lib.fk_ar2d_sr_gram_min_rows(ctypes.byref(d), 64, 0)
    tc = lib.fk_ar2d_sr_gram_min_rows(ctypes.byref(d), 64, 1)
    assert 0 < cc < tc
    assert lib.fk_ar2d_sr_gram(ctypes.byref(d), None, None, None, 64, None, 0, None, 0, None, 0, None, 1,
                               None) == -1
    assert b"NULL" in lib.fk_last_error()
