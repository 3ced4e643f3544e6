"""Local energy through the GPU pipeline (kernel c + batched AR passes) and a
full VMC step, against the oracle."""
import numpy as np
import pytest
import torch

from oracle import ar2d, exact, local_energy, operators as ref_ops

pytestmark = pytest.mark.gpu


def _ops(shape):
    from flowket_gb300 import operators as ops
    return [
        (ops.Heisenberg(hilbert_state_shape=shape, pbc=True), lambda s: ref_ops.heisenberg_find_conn(s, pbc=True)),
        (ops.Ising(h=3.0, hilbert_state_shape=shape, pbc=True), lambda s: ref_ops.ising_find_conn(s, h=3.0, pbc=True)),
        (ops.J1J2(hilbert_state_shape=shape, j2=0.5, pbc=True), lambda s: ref_ops.j1j2_find_conn(s, j2=0.5, pbc=True)),
    ]


@pytest.mark.parametrize("which", [0, 1, 2])
def test_local_energy_matches_oracle(cuda, which):
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.observables import Observable
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape, depth = (4, 4), 3
    m = ConvNetAutoregressive2D(shape, depth, 16, weights_normalization=True, precision="fp32", seed=1)
    op, ref_fc = _ops(shape)[which]
    spins, lp, _ = FastAutoregressiveSampler(m, 256, seed=4).sample()
    got = Observable(op).local_values(m, spins, log_psi=lp)
    got = got[:, 0].cpu().numpy() + 1j * got[:, 1].cpu().numpy()
    s = spins.cpu().numpy()
    params = m.params_dict_cpu()
    wf = lambda x: ar2d.log_psi_numpy(params, np.asarray(x).astype(np.int8), depth, True)
    conn, mel, use = ref_fc(s)
    want = local_energy.local_values(wf, conn, mel, use)
    np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-4 * np.abs(want).max())


def test_vmc_step_decreases_energy_heisenberg_4x4(cuda):
    """A short run of the plain path (4x4 Heisenberg PBC, Marshall sign, AR net,
    Adam): the variational energy approaches the Lanczos ground state."""
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.optimization import VariationalMonteCarlo
    from flowket_gb300.optimizers import Adam
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape = (4, 4)
    e0 = exact.lanczos_ground_energy(lambda s: ref_ops.heisenberg_find_conn(s, pbc=True), shape,
                                     basis=exact.sz_sector(shape, 0))
    m = ConvNetAutoregressive2D(shape, 3, 16, weights_normalization=False, precision="fp32", seed=0)
    vmc = VariationalMonteCarlo(m, Heisenberg(hilbert_state_shape=shape, pbc=True),
                                FastAutoregressiveSampler(m, 256, seed=11))
    opt = Adam(m, lr=1e-2)
    energies = []
    for _ in range(120):
        vmc.step(opt)
        energies.append(vmc.current_energy.real)
    first, last = np.mean(energies[:5]), np.mean(energies[-10:])
    assert last < first
    assert (last - e0) / abs(e0) < 0.1, (last, e0)
    assert set(vmc.times) == {"sampling", "local_energy", "gradient", "update"}


@pytest.mark.parametrize("precision,which", [("bf16", 0), ("bf16", 1), ("fp32", 2), ("bf16", 2), ("fp16", 0),
                                             ("fp16", 2)])
def test_causal_reuse_equals_full_forward(cuda, precision, which):
    """Connected configurations evaluated from the base samples' saved
    activations (rows >= first flipped row only) give bitwise the full forward."""
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.observables import Observable
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape = (5, 6)
    m = ConvNetAutoregressive2D(shape, 4, 16, weights_normalization=True, precision=precision, seed=2)
    op = _ops(shape)[which][0]
    spins, lp, saved = FastAutoregressiveSampler(m, 300, seed=8).sample()
    obs = Observable(op, evaluation_batch_size=1024)
    _, _, bf, rows = obs.connections(spins)
    full = m.forward(bf["configs"][:rows])[0]
    reuse = m.forward_connections(bf["configs"], bf["owner"], bf["cflips"], rows, saved, 300, chunk=1024)
    assert torch.equal(full, reuse[:rows])
    e_full = obs.local_values(m, spins, log_psi=lp).clone()
    e_reuse = obs.local_values(m, spins, log_psi=lp, base_saved=saved)
    assert torch.equal(e_full, e_reuse)


@pytest.mark.parametrize("precision,which,shape,depth,f", [("bf16", 0, (10, 10), 4, 32), ("fp16", 1, (6, 7), 3, 32),
                                                         ("bf16", 1, (6, 6), 3, 64), ("fp32", 0, (6, 6), 3, 32),
                                                         ("bf16", 2, (4, 4), 5, 16)])
def test_causal_reuse_equals_full_forward_engines(cuda, precision, which, shape, depth, f):
    """The causal-reuse forward (every op from the first flipped row rk, the
    rows above and the rows the first evaluated row's taps read gathered from
    the base activations) gives bitwise the full forward on every engine:
    pipelined (F = 32), per-pixel (F = 64) and FP32. (The V stream of row r
    depends on the spins of row r: its taps include row r, and the shift
    that makes the network autoregressive comes after it, when row r's V
    output feeds Cat at row r + 1; so the V ops of row rk are evaluated too.)"""
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.observables import Observable
    from flowket_gb300.samplers import FastAutoregressiveSampler
    m = ConvNetAutoregressive2D(shape, depth, f, weights_normalization=True, precision=precision, seed=4)
    op = _ops(shape)[which][0]
    spins, lp, saved = FastAutoregressiveSampler(m, 200, seed=9).sample()
    obs = Observable(op, evaluation_batch_size=1024)
    _, _, bf, rows = obs.connections(spins)
    full = m.forward(bf["configs"][:rows])[0]
    reuse = m.forward_connections(bf["configs"], bf["owner"], bf["cflips"], rows, saved, 200, chunk=1024)
    assert torch.equal(full, reuse[:rows])


def test_exact_variational_matches_oracle_and_finite_differences(cuda):
    """ExactVariational (exact_variational.py:96-155) on 3x3 Heisenberg PBC:
    the energy, variance and probabilities equal the oracle's closed form over
    all 512 configurations, and the adjoint gradient of the exact energy
    matches a central finite difference of the oracle's FP64 exact energy
    along a random direction. The parameters are moved off the initial zero
    biases first: a ReLU at exactly zero has no derivative a finite
    difference can see."""
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.optimization import ExactVariational
    shape, depth = (3, 3), 2
    m = ConvNetAutoregressive2D(shape, depth, 16, weights_normalization=True, precision="fp32", seed=3)
    g = torch.Generator().manual_seed(1)
    m.params.add_((0.02 * torch.randn(m.num_params, generator=g)).cuda())
    m.params_updated()
    ev = ExactVariational(m, Heisenberg(hilbert_state_shape=shape, pbc=True), batch_size=64)
    e = ev.machine_updated()
    params = m.params_dict_cpu()
    fc = lambda s: ref_ops.heisenberg_find_conn(s, pbc=True)

    def oracle_energy(p):
        wf = lambda x: ar2d.log_psi_numpy(p, np.asarray(x).astype(np.int8), depth, True)
        return exact.exact_energy(wf, fc, shape)

    want, want_var, probs, _ = oracle_energy(params)
    assert abs(e - want) < 1e-4 * abs(want), (e, want)
    assert ev.current_local_energy_variance == pytest.approx(want_var, rel=1e-3, abs=1e-4)
    np.testing.assert_allclose(ev.probs.cpu().numpy(), probs, rtol=1e-4, atol=1e-9)
    grad = m.backward(ev.states, ev._w, ev._saved).double().cpu()
    d = torch.randn(m.num_params, generator=torch.Generator().manual_seed(0), dtype=torch.float64)
    dd = {name: d[off:off + int(np.prod(shp))].reshape(shp) for name, shp, off in m.layout}
    eps = 1e-6
    plus = oracle_energy({k: v + eps * dd[k] for k, v in params.items()})[0].real
    minus = oracle_energy({k: v - eps * dd[k] for k, v in params.items()})[0].real
    fd = (plus - minus) / (2 * eps)
    got = float((grad * d).sum())
    assert abs(got - fd) < 2e-3 * abs(fd) + 1e-4, (got, fd)
    # the generator serves (configurations, coefficients) in batch_size pieces
    x, y = next(iter(ev))
    assert x.shape == (64, 3, 3) and y.shape == (64,)


@pytest.mark.parametrize("kind", ["ar_adam", "rbm_sr"])
def test_checkpoint_resume_continues_a_vmc_run_identically(cuda, tmp_path, kind):
    """A real VMC run checkpointed after 3 steps (parameters, optimiser state,
    sampler position; callbacks/checkpoint.py:9-73) and resumed in fresh
    objects repeats the uninterrupted run's next steps: bit for bit with Adam
    (every reduction of that step has a fixed order); with SR to rounding,
    because the Gram's K-split partial sums and CG's dot products are added
    with atomics in a varying order."""
    from flowket_gb300 import checkpoint
    from flowket_gb300.machines import RBM, ConvNetAutoregressive2D
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.optimization import VariationalMonteCarlo
    from flowket_gb300.optimizers import Adam, ComplexValuesStochasticReconfiguration
    from flowket_gb300.samplers import FastAutoregressiveSampler, MetropolisHastingsLocal

    def build():
        if kind == "ar_adam":
            shape = (4, 4)
            m = ConvNetAutoregressive2D(shape, 3, 16, weights_normalization=True, precision="bf16", seed=1)
            smp = FastAutoregressiveSampler(m, 256, seed=5)
            opt = Adam(m, lr=3e-3)
        else:
            shape = (10,)
            m = RBM(shape, alpha=2, stddev=0.05, seed=1)
            smp = MetropolisHastingsLocal(m, 256, num_of_chains=32, unused_sampels=4, seed=5)
            opt = ComplexValuesStochasticReconfiguration(m, lr=0.05, diag_shift=0.1)
        return m, smp, opt, VariationalMonteCarlo(m, Heisenberg(hilbert_state_shape=shape, pbc=True), smp)

    m, smp, opt, vmc = build()
    for _ in range(3):
        vmc.step(opt)
    path = str(tmp_path / "ckpt")
    checkpoint.save_weights(m, path)
    if kind == "ar_adam":
        checkpoint.save_optimizer_weights(opt, path, 0, 3)
    checkpoint.save_sampler_state(smp, path)
    # SR: one resumed step, whose sampling and energy depend only on the
    # restored state (the update itself is reproduced to rounding)
    n_more = 3 if kind == "ar_adam" else 1
    want = []
    for _ in range(n_more):
        vmc.step(opt)
        want.append(vmc.current_energy)
    want_params = m.params.clone()
    m2, smp2, opt2, vmc2 = build()
    checkpoint.load_weights(m2, path)
    if kind == "ar_adam":
        assert checkpoint.load_optimizer_weights(opt2, path) == (0, 3)
    assert checkpoint.load_sampler_state(smp2, path)
    got = []
    for _ in range(n_more):
        vmc2.step(opt2)
        got.append(vmc2.current_energy)
    assert got == want
    if kind == "ar_adam":
        assert torch.equal(m2.params, want_params)
    else:
        assert torch.allclose(m2.params, want_params, rtol=1e-4, atol=1e-6)
