"""The CUDA path against golden vectors written by the reference's own numpy
code (tests/golden/make_reference_fixtures.py): the GPU enumeration equals
operators/heisenberg.py / operators/ising.py find_conn bit for bit, the GPU
local energies equal observables/monte_carlo/operator.py's local_values, and
fk_energy_stats equals observable.py's estimate."""
import os

import numpy as np
import pytest
import torch

from test_reference_fixtures import FIND_CONN, FIND_CONN_ARGS, LOCAL

pytestmark = pytest.mark.gpu


def _operator(op, shape, kw):
    from flowket_gb300.operators import Heisenberg, Ising
    return (Heisenberg if op == "heisenberg" else Ising)(hilbert_state_shape=shape, **kw)


@pytest.mark.parametrize("name", sorted(FIND_CONN_ARGS))
def test_gpu_enumeration_equals_reference_find_conn(cuda, name):
    op, kw = FIND_CONN_ARGS[name]
    s = FIND_CONN[name + "/spins"]
    ham = _operator(op, s.shape[1:], kw)
    flips, mel, use, _ = ham.enumerate(torch.as_tensor(s).cuda())
    use_ref = FIND_CONN[name + "/use"]
    np.testing.assert_array_equal(use.cpu().numpy().astype(bool), use_ref)
    np.testing.assert_array_equal(mel.cpu().numpy(), FIND_CONN[name + "/mel"])
    got = np.sort(flips.cpu().numpy().astype(np.int64), axis=-1)
    want = FIND_CONN[name + "/diff"].astype(np.int64)
    # a site pair sorted ascending, -1 (none) first
    want = np.sort(want, axis=-1)
    used = use_ref.copy()
    used[0] = False
    np.testing.assert_array_equal(got[used], want[used])
    # the dense connected configurations as well
    conn, _, _ = ham.find_conn(torch.as_tensor(s).cuda())
    conn = conn.cpu().numpy().reshape(conn.shape[0], s.shape[0], -1)
    flat = s.reshape(s.shape[0], -1)
    for c in range(conn.shape[0]):
        d = conn[c] != flat
        for i in range(s.shape[0]):
            sites = np.nonzero(d[i])[0]
            ref = FIND_CONN[name + "/diff"][c, i]
            np.testing.assert_array_equal(sites, ref[ref >= 0])


@pytest.mark.parametrize("name,op,kw", [("rbm_heis_4x4_pbc", "heisenberg", dict(pbc=True)),
                                        ("rbm_ising_4x4_pbc_h3", "ising", dict(pbc=True, h=3.0)),
                                        ("rbm_heis_chain16_obc", "heisenberg", dict(pbc=False))])
def test_gpu_rbm_local_energy_equals_reference_local_values(cuda, name, op, kw):
    from flowket_gb300.machines import RBM
    from flowket_gb300.observables import Observable, energy_stats
    s = LOCAL[name + "/spins"]
    a, b, w = LOCAL[name + "/a"], LOCAL[name + "/b"], LOCAL[name + "/W"]
    full = np.concatenate([a, b, w.reshape(-1)])
    params = np.stack([full.real, full.imag], axis=1).reshape(-1).astype(np.float32)
    m = RBM(s.shape[1:], alpha=b.shape[0] // a.shape[0], params=params)
    obs = Observable(_operator(op, s.shape[1:], kw))
    local = obs.local_values(m, torch.as_tensor(s).cuda())
    got = local.cpu().numpy()
    got = got[:, 0] + 1j * got[:, 1]
    want = LOCAL[name + "/local"]
    np.testing.assert_allclose(got, want, rtol=0, atol=2e-5 * np.abs(want).max())
    # fk_energy_stats on the reference's own local values equals its estimate
    ref_local = torch.as_tensor(np.stack([want.real, want.imag], axis=1)).cuda()
    stats, _ = energy_stats(ref_local)
    st = stats.cpu().numpy()
    mean, var = LOCAL[name + "/mean"], float(LOCAL[name + "/var"])
    assert abs(complex(st[0], st[1]) - mean) <= 1e-12 * abs(mean)
    assert abs(st[2] - var) <= 1e-11 * var


@pytest.mark.parametrize("reuse", [False, True])
@pytest.mark.parametrize("name,op,kw", [("ar_heis_4x4_pbc", "heisenberg", dict(pbc=True)),
                                        ("ar_ising_4x4_pbc_h3", "ising", dict(pbc=True, h=3.0))])
def test_gpu_ar_local_energy_equals_reference_local_values(cuda, name, op, kw, reuse):
    """FP32 path, full forward of every connected configuration or causal
    reuse of the base activations."""
    from flowket_gb300 import _lib
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.observables import Observable
    s = LOCAL[name + "/spins"]
    m = ConvNetAutoregressive2D((4, 4), 3, 16, weights_normalization=True, precision="fp32",
                                params=LOCAL[name + "/params"])
    obs = Observable(_operator(op, (4, 4), kw))
    st = torch.as_tensor(s).cuda()
    if reuse:
        lp, _, saved = m.forward(st, mode=_lib.FK_AR2D_SAVE)
        local = obs.local_values(m, st, log_psi=lp, base_saved=saved)
    else:
        local = obs.local_values(m, st)
    got = local.cpu().numpy()
    got = got[:, 0] + 1j * got[:, 1]
    want = LOCAL[name + "/local"]
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-5 * np.abs(want).max())
