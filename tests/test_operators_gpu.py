"""Kernel (c): GPU enumeration is bit-exact against the oracle restatement."""
import numpy as np
import pytest
import torch

from oracle import operators as ref

pytestmark = pytest.mark.gpu


def _rand_spins(b, shape, seed):
    rng = np.random.default_rng(seed)
    return rng.choice([-1, 1], size=(b,) + shape).astype(np.int8)


def _check(got, want):
    conn, mel, use = got
    wc, wm, wu = want
    assert conn.shape == wc.shape
    assert np.array_equal(conn.cpu().numpy().astype(np.int64), wc.astype(np.int64))
    assert np.array_equal(use.cpu().numpy(), wu)
    assert np.array_equal(mel.cpu().numpy(), np.real(wm))


@pytest.mark.parametrize("shape,pbc", [((4, 4), True), ((4, 4), False), ((10, 10), True), ((3, 5), True),
                                       ((16, 16), True), ((2, 3), True)])
@pytest.mark.parametrize("rot", [True, False])
def test_heisenberg_2d(cuda, shape, pbc, rot):
    from flowket_gb300.operators import Heisenberg
    s = _rand_spins(37, shape, 1)
    op = Heisenberg(hilbert_state_shape=shape, pbc=pbc, unitary_rotation=rot)
    _check(op.find_conn(torch.as_tensor(s).cuda()), ref.heisenberg_find_conn(s, pbc=pbc, unitary_rotation=rot))


@pytest.mark.parametrize("length,pbc", [(7, True), (64, True), (20, False)])
def test_heisenberg_chain(cuda, length, pbc):
    from flowket_gb300.operators import Heisenberg
    s = _rand_spins(130, (length,), 2)
    op = Heisenberg(hilbert_state_shape=(length,), pbc=pbc)
    _check(op.find_conn(torch.as_tensor(s).cuda()), ref.heisenberg_find_conn(s, pbc=pbc))


@pytest.mark.parametrize("shape,pbc", [((10, 10), True), ((4, 4), False), ((16,), False), ((1, 8), True)])
def test_ising(cuda, shape, pbc):
    from flowket_gb300.operators import Ising
    s = _rand_spins(65, shape, 3)
    op = Ising(h=3.0, hilbert_state_shape=shape, pbc=pbc)
    _check(op.find_conn(torch.as_tensor(s).cuda()), ref.ising_find_conn(s, h=3.0, pbc=pbc))


@pytest.mark.parametrize("shape,pbc", [((4, 4), False), ((10, 10), True), ((4, 6), True)])
def test_j1j2(cuda, shape, pbc):
    from flowket_gb300.operators import J1J2
    s = _rand_spins(33, shape, 4)
    op = J1J2(hilbert_state_shape=shape, j2=0.5, pbc=pbc)
    _check(op.find_conn(torch.as_tensor(s).cuda()), ref.j1j2_find_conn(s, j2=0.5, pbc=pbc))


def test_empty_batch(cuda):
    from flowket_gb300.operators import Heisenberg
    op = Heisenberg(hilbert_state_shape=(4, 4))
    conn, mel, use = op.find_conn(torch.empty((0, 4, 4), dtype=torch.int8, device="cuda"))
    assert conn.shape == (33, 0, 4, 4) and mel.shape == (33, 0)


def test_compaction_and_local_energy_match_oracle(cuda):
    """Unbalanced-path restatement: compact the used slots, evaluate a simple
    complex-linear wave function, reduce E_loc on the GPU."""
    from flowket_gb300 import _lib
    from flowket_gb300.operators import Heisenberg
    from oracle import local_energy as le
    shape = (4, 4)
    s = _rand_spins(300, shape, 5)
    op = Heisenberg(hilbert_state_shape=shape, pbc=True)
    flips, mel, use, spins = op.enumerate(torch.as_tensor(s).cuda())
    b, n, c = 300, 16, op.max_number_of_local_connections
    ws = torch.empty(_lib.load().fk_compact_workspace_bytes(b), dtype=torch.uint8, device="cuda")
    max_rows = b * c
    configs = torch.empty((max_rows, n), dtype=torch.int8, device="cuda")
    owner = torch.empty(max_rows, dtype=torch.int32, device="cuda")
    cmel = torch.empty(max_rows, dtype=torch.float64, device="cuda")
    cflips = torch.empty((max_rows, 2), dtype=torch.int16, device="cuda")
    offsets = torch.empty(b + 1, dtype=torch.int64, device="cuda")
    nrows = torch.empty(1, dtype=torch.int64, device="cuda")
    _lib.call("fk_compact_connections", _lib.ptr(spins), b, n, c, _lib.ptr(flips), _lib.ptr(mel), _lib.ptr(use), 1,
              _lib.ptr(configs), _lib.ptr(owner), _lib.ptr(cmel), _lib.ptr(cflips), _lib.ptr(offsets), max_rows,
              _lib.ptr(nrows), _lib.ptr(ws), ws.numel(), _lib.stream_ptr())
    r = int(nrows.item())
    w = torch.linspace(-0.3, 0.4, n, dtype=torch.float64) + 1j * torch.linspace(0.2, -0.1, n, dtype=torch.float64)
    def lp_of(x):
        v = x.to(torch.complex128).cpu() @ w
        return torch.stack([v.real, v.imag], 1).to(torch.float32).cuda()
    lp_rows = lp_of(configs[:r])
    lp_self = lp_of(spins)
    local = torch.empty((b, 2), dtype=torch.float64, device="cuda")
    _lib.call("fk_local_energy_reduce", _lib.ptr(lp_self), _lib.ptr(mel[0].contiguous()), b, _lib.ptr(lp_rows),
              _lib.ptr(offsets), _lib.ptr(cmel), _lib.ptr(local), _lib.stream_ptr())
    wnp = w.numpy()
    conn_np, mel_np, use_np = ref.heisenberg_find_conn(s, pbc=True)
    f = lambda x: (x.reshape(x.shape[0], -1) @ wnp).astype(np.complex64).astype(np.complex128)
    want = le.local_values(f, conn_np, mel_np, use_np)
    got = local[:, 0].cpu().numpy() + 1j * local[:, 1].cpu().numpy()
    assert r == int(use_np[1:].sum())
    np.testing.assert_allclose(got, want, rtol=2e-5, atol=2e-5)


def test_find_conn_equals_golden_fixture(cuda):
    """Bit-exact against the committed fixture tests/golden/connections_4x4.json."""
    import json
    import os
    from flowket_gb300 import operators as ops
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "connections_4x4.json")))
    s = torch.as_tensor(np.array(gold["configs"], dtype=np.int8)).cuda()
    shape = (4, 4)
    for name, op in (("heisenberg", ops.Heisenberg(hilbert_state_shape=shape, pbc=True)),
                     ("ising", ops.Ising(h=3.0, hilbert_state_shape=shape, pbc=True)),
                     ("j1j2", ops.J1J2(hilbert_state_shape=shape, j2=0.5, pbc=True))):
        conn, mel, use = op.find_conn(s)
        g = gold[name]
        assert np.array_equal(conn.cpu().numpy(), np.array(g["conn"], dtype=np.int8)), name
        m = mel.cpu().numpy()
        m = m.real if np.iscomplexobj(m) else m
        assert np.array_equal(m, np.array(g["mel"])), name
        assert np.array_equal(use.cpu().numpy(), np.array(g["use"], dtype=bool)), name
