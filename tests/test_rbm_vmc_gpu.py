"""RBM machines through the VMC driver: RBMSym tied parameters, the complex
loss gradient, Metropolis-Hastings samplers as the driver's samplers, and
complex-parameter stochastic reconfiguration, against the oracle; the
reference's SR example (examples/rbm_heisenberg_1d_sr.py:14-37) reaching its
exact ground-state energy."""
import numpy as np
import pytest
import torch

from oracle import rbm as ref_rbm, sr as ref_sr

pytestmark = pytest.mark.gpu


def _spins(n, b, seed):
    return np.random.default_rng(seed).choice([-1, 1], size=(b, n)).astype(np.int8)


def test_rbm_sym_log_psi_and_log_derivatives_match_oracle(cuda):
    from flowket_gb300.machines import RBMSym
    shape, alpha = (3, 4), 2
    m = RBMSym(shape, alpha=alpha, stddev=0.2, seed=3)
    bare = {k: v.numpy() for k, v in m.bare.items()}
    s = _spins(12, 90, 0)
    st = torch.as_tensor(s).cuda()
    got = m.log_psi(st).cpu().numpy()
    want = ref_rbm.rbm_log_psi(ref_rbm.rbm_sym_full_params(bare, shape), s)
    np.testing.assert_allclose(got.real, want.real, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(np.exp(1j * got.imag), np.exp(1j * want.imag), atol=1e-5)
    o = m.log_derivatives(st).cpu().numpy().T
    want_o = ref_rbm.rbm_sym_log_derivatives(bare, shape, s)
    assert o.shape == want_o.shape == (90, 1 + alpha + 12 * alpha)
    np.testing.assert_allclose(o, want_o, rtol=1e-4, atol=2e-5)


@pytest.mark.parametrize("sym", [False, True])
def test_rbm_backward_is_the_complex_loss_gradient(cuda, sym):
    """grad of sum_b (w_re Re log psi_b + w_im Im log psi_b) with respect to the
    stored (re, im) pairs: (sum w_re Re O + w_im Im O, sum w_im Re O - w_re Im O)."""
    from flowket_gb300.machines import RBM, RBMSym
    shape = (10,)
    m = (RBMSym if sym else RBM)(shape, alpha=2, stddev=0.1, seed=4)
    s = _spins(10, 150, 1)
    w = np.random.default_rng(2).normal(size=(150, 2)).astype(np.float32)
    g = m.backward(torch.as_tensor(s).cuda(), torch.as_tensor(w).cuda()).cpu().numpy().astype(np.float64)
    if sym:
        o = ref_rbm.rbm_sym_log_derivatives({k: v.numpy() for k, v in m.bare.items()}, shape, s)
    else:
        p = {k: v.detach().cpu().numpy().astype(np.complex128) for k, v in m.complex_params().items()}
        o = ref_rbm.rbm_log_derivatives(p, s)
    wr, wi = w[:, 0:1].astype(np.float64), w[:, 1:2].astype(np.float64)
    gu = (wr * o.real + wi * o.imag).sum(0)
    gv = (wi * o.real - wr * o.imag).sum(0)
    want = np.stack([gu, gv], axis=1).reshape(-1)
    np.testing.assert_allclose(g, want, rtol=1e-4, atol=1e-4 * np.abs(want).max())
    # finite difference of the loss along a random direction of the stored pairs
    d = np.random.default_rng(5).normal(size=m.num_params)
    base = m.params.clone()
    eps = 1e-3

    def loss(params):
        m.params.copy_(torch.as_tensor(params, dtype=torch.float32).cuda())
        m.params_updated()
        lp = m.log_psi(torch.as_tensor(s).cuda()).cpu().numpy().astype(np.complex128)
        return float((w[:, 0] * lp.real + w[:, 1] * lp.imag).sum())

    p0 = base.cpu().numpy().astype(np.float64)
    fd = (loss(p0 + eps * d) - loss(p0 - eps * d)) / (2 * eps)
    m.params.copy_(base)
    m.params_updated()
    assert abs(fd - float(g @ d)) < 2e-2 * max(1.0, abs(fd)), (fd, float(g @ d))


@pytest.mark.parametrize("sampler_kind", ["local", "exchange", "hamiltonian"])
def test_vmc_step_runs_metropolis_hastings_samplers_on_rbm(cuda, sampler_kind):
    """VariationalMonteCarlo drives every Metropolis-Hastings sampler over an
    RBM (the reference's MCMC path) with Adam and lowers the energy."""
    from flowket_gb300.machines import RBM
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.optimization import VariationalMonteCarlo
    from flowket_gb300.optimizers import Adam
    from flowket_gb300.samplers import (MetropolisHastingsExchange, MetropolisHastingsHamiltonian,
                                        MetropolisHastingsLocal)
    shape = (12,)
    op = Heisenberg(hilbert_state_shape=shape, pbc=True)
    m = RBM(shape, alpha=1, stddev=0.01, seed=1)
    if sampler_kind == "local":
        sampler = MetropolisHastingsLocal(m, 512, num_of_chains=64, unused_sampels=12, seed=2)
    elif sampler_kind == "exchange":
        sampler = MetropolisHastingsExchange(m, 512, num_of_chains=64, unused_sampels=12, seed=2)
    else:
        sampler = MetropolisHastingsHamiltonian(m, 512, op, num_of_chains=64, unused_sampels=12, seed=2)
    vmc = VariationalMonteCarlo(m, op, sampler)
    opt = Adam(m, lr=1e-2)
    energies = []
    for _ in range(40):
        vmc.step(opt)
        energies.append(vmc.current_energy.real)
    assert np.all(np.isfinite(energies))
    assert np.mean(energies[-5:]) < np.mean(energies[:5]) - 1.0, energies
    x, y = next(iter(vmc.to_generator()))
    assert x.shape == (512,) + shape and y.shape == (512,)


@pytest.mark.parametrize("sym", [False, True])
def test_complex_sr_direction_matches_oracle_parameter_space_solve(cuda, sym):
    """Sample-space complex SR (Hermitian Gram, real embedding, FP64 CG) equals
    the reference's parameter-space solve (optimizer.py:55-114 with Cholesky)."""
    from flowket_gb300.machines import RBM, RBMSym
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.optimizers import ComplexValuesStochasticReconfiguration
    from flowket_gb300.samplers import MetropolisHastingsLocal
    shape = (8,)
    m = (RBMSym if sym else RBM)(shape, alpha=2, stddev=0.2, seed=6)
    sampler = MetropolisHastingsLocal(m, 256, num_of_chains=32, unused_sampels=8, seed=3)
    s = next(sampler)
    local = m.local_energy(Heisenberg(hilbert_state_shape=shape, pbc=True), s)
    opt = ComplexValuesStochasticReconfiguration(m, lr=0.05, diag_shift=0.1, iterative_solver=False)
    x = opt.direction(s, local).cpu().numpy().astype(np.float64)
    x = x[0::2] + 1j * x[1::2]
    e = local.cpu().numpy()
    e = e[:, 0] + 1j * e[:, 1]
    y = np.conj(e - e.mean()) / e.shape[0]
    o_gpu = m.log_derivatives(s).cpu().numpy().T.astype(np.complex128)
    want = ref_sr.sr_complex(o_gpu, y, 0.1)
    np.testing.assert_allclose(x, want, rtol=0, atol=1e-5 * np.abs(want).max())
    sn = s.cpu().numpy().reshape(256, -1)
    if sym:
        o_ref = ref_rbm.rbm_sym_log_derivatives({k: v.numpy() for k, v in m.bare.items()}, shape, sn)
    else:
        p = {k: v.detach().cpu().numpy().astype(np.complex128) for k, v in m.complex_params().items()}
        o_ref = ref_rbm.rbm_log_derivatives(p, sn)
    want_ref = ref_sr.sr_complex(o_ref, y, 0.1)
    np.testing.assert_allclose(x, want_ref, rtol=0, atol=1e-3 * np.abs(want_ref).max())


def test_rbm_sym_heisenberg_chain_sr_reaches_exact_energy(cuda):
    """examples/rbm_heisenberg_1d_sr.py:14-37 on this stack: RBMSym (alpha 1,
    stddev 0.01) on the 20-site periodic Heisenberg chain (Marshall sign),
    MetropolisHastingsHamiltonian with 20 chains and 20 unused sweeps, 1000
    samples per step, SR lr 0.05, diag_shift 0.1, direct solve, 300 steps.
    The energy reaches the exact -35.6175461195 within 1e-3 relative."""
    from flowket_gb300.machines import RBMSym
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.optimization import VariationalMonteCarlo
    from flowket_gb300.optimizers import ComplexValuesStochasticReconfiguration
    from flowket_gb300.samplers import MetropolisHastingsHamiltonian
    shape = (20, 1)
    e0 = -35.6175461195
    m = RBMSym(shape, stddev=0.01, seed=0)
    op = Heisenberg(hilbert_state_shape=shape, pbc=True)
    sampler = MetropolisHastingsHamiltonian(m, 1000, op, num_of_chains=20, unused_sampels=20, seed=11)
    vmc = VariationalMonteCarlo(m, op, sampler)
    opt = ComplexValuesStochasticReconfiguration(m, lr=0.05, diag_shift=0.1, iterative_solver=False)
    energies = []
    for _ in range(300):
        vmc.step(opt)
        energies.append(vmc.current_energy.real)
    tail = float(np.mean(energies[-30:]))
    assert abs(tail - e0) / abs(e0) < 1e-3, (tail, energies[-10:])
