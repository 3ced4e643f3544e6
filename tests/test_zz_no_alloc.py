"""fk_sr_solve_noalloc: the SR solve for callers that cannot give the library
device memory (their GPU memory is owned by another allocator, or cudaMalloc
is not allowed where they solve). It keeps its conjugate-gradient scratch in a
fixed array inside the library (n <= 8192) and must give the same answer as
fk_sr_solve, which takes a caller-provided workspace.

This file is collected last on purpose; it runs the entry point alone in a
fresh process as well as after the other tests."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _system(n, p, seed):
    from flowket_gb300 import _lib
    rng = np.random.default_rng(seed)
    a = torch.as_tensor(rng.normal(size=(p, n // 2)).astype(np.float32)).cuda()
    c = torch.as_tensor(rng.normal(size=(p, n // 2)).astype(np.float32)).cuda()
    gram = torch.empty((n, n), dtype=torch.float64, device="cuda")
    _lib.call("fk_sr_gram", _lib.ptr(a), _lib.ptr(c), p, n // 2, _lib.ptr(gram), n * n, _lib.stream_ptr())
    return gram


def _solve_with_workspace(gram, n, rhs, p):
    from flowket_gb300 import _lib
    x = torch.empty(n, dtype=torch.float64, device="cuda")
    stats = torch.zeros(3, dtype=torch.float64, device="cuda")
    ws = torch.empty(_lib.load().fk_sr_solve_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    _lib.call("fk_sr_solve", _lib.ptr(gram), n, 1.0 / p, 0.05, _lib.ptr(rhs), 1e-10, 300, _lib.ptr(x),
              _lib.ptr(stats), _lib.ptr(ws), ws.numel(), _lib.stream_ptr())
    return x, stats


def _solve_noalloc(gram, n, rhs, p):
    from flowket_gb300 import _lib
    x = torch.empty(n, dtype=torch.float64, device="cuda")
    stats = torch.zeros(3, dtype=torch.float64, device="cuda")
    _lib.call("fk_sr_solve_noalloc", _lib.ptr(gram), n, 1.0 / p, 0.05, _lib.ptr(rhs), 1e-10, 300, _lib.ptr(x),
              _lib.ptr(stats), _lib.stream_ptr())
    return x, stats


def test_noalloc_solve_matches_workspace_solve_twice(cuda):
    n, p = 384, 2000
    gram = _system(n, p, 0)
    rng = np.random.default_rng(1)
    for call in range(2):  # the second call reuses the array the first one left behind
        rhs = torch.as_tensor(rng.normal(size=n)).cuda()
        want, want_stats = _solve_with_workspace(gram, n, rhs, p)
        got, got_stats = _solve_noalloc(gram, n, rhs, p)
        torch.cuda.synchronize()
        np.testing.assert_allclose(got.cpu().numpy(), want.cpu().numpy(), rtol=1e-8, atol=1e-10)
        assert got_stats[0].item() == want_stats[0].item() > 0


def test_noalloc_solve_rejects_sizes_beyond_its_scratch(cuda):
    from flowket_gb300 import _lib
    lib = _lib.load()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    st = lib.fk_sr_solve_noalloc(_lib.ptr(buf), 8193, 1.0, 0.1, _lib.ptr(buf), 1e-3, 10, _lib.ptr(buf), None,
                                 _lib.stream_ptr())
    assert st == -1
    assert b"8192" in lib.fk_last_error()
