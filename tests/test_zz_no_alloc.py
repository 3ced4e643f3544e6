"""fk_sr_solve_noalloc: the SR solve for callers that cannot give the library
device memory (their GPU memory is owned by another allocator, or cudaMalloc
is not allowed where they solve). It keeps its conjugate-gradient scratch in a
fixed array inside the library (n <= 8192) and must give the same answer as
fk_sr_solve, which takes a caller-provided workspace.

This file is collected last on purpose, so that a run stopping at the first
failure has run every other test before it. It checks the entry point after
the other tests (in the shared session) and as the first library call of a
fresh child process, where the per-device lookup of the array runs."""
import os
import subprocess
import sys

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


_FRESH = r"""
import sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
from flowket_gb300 import _lib
n, p = 256, 1000
g = torch.Generator(device="cuda").manual_seed(0)
y = torch.randn((p, n), generator=g, device="cuda", dtype=torch.float64)
gram = (y.T @ y).contiguous()
res = []
for k in range(2):
    rhs = torch.randn(n, generator=g, device="cuda", dtype=torch.float64)
    x0 = torch.empty(n, dtype=torch.float64, device="cuda")
    _lib.call("fk_sr_solve_noalloc", _lib.ptr(gram), n, 1.0 / p, 0.05, _lib.ptr(rhs), 1e-10, 300, _lib.ptr(x0),
              None, _lib.stream_ptr())
    ws = torch.empty(_lib.load().fk_sr_solve_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    x1 = torch.empty(n, dtype=torch.float64, device="cuda")
    _lib.call("fk_sr_solve", _lib.ptr(gram), n, 1.0 / p, 0.05, _lib.ptr(rhs), 1e-10, 300, _lib.ptr(x1), None,
              _lib.ptr(ws), ws.numel(), _lib.stream_ptr())
    torch.cuda.synchronize()
    res.append(float((x0 - x1).abs().max() / x1.abs().max()))
print("max-rel", max(res))
assert max(res) < 1e-8, res
"""


def test_noalloc_solve_as_first_call_of_a_fresh_process(cuda):
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _FRESH, root], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "max-rel" in r.stdout
