"""EqualUpDownSpins (abstract_machine.py:52-53, layers/spins_invariants.py:13-22)
through the CUDA path: forward (per-pixel and pipelined engines, both
precisions), exact sampler, adjoint and local energy against the oracle."""
import numpy as np
import pytest
import torch

from oracle import ar2d, exact, local_energy, operators as ref_ops

pytestmark = pytest.mark.gpu


def _machine(shape, depth, f, precision, seed=0):
    from flowket_gb300.machines import ConvNetAutoregressive2D
    m = ConvNetAutoregressive2D(shape, depth, f, weights_normalization=True, precision=precision, seed=seed,
                                equal_up_down_spins=True)
    g = torch.Generator().manual_seed(seed + 11)
    m.params.add_((0.05 * torch.randn(m.num_params, generator=g)).cuda())
    m.params_updated()
    return m


def _configs(shape, b, seed):
    rng = np.random.default_rng(seed)
    n = int(np.prod(shape))
    half = np.array([1] * (n // 2) + [-1] * (n - n // 2), dtype=np.int8)
    sz0 = np.stack([rng.permutation(half) for _ in range(b // 2)])
    rand = rng.choice([-1, 1], size=(b - b // 2, n)).astype(np.int8)
    return np.concatenate([sz0, rand]).reshape((b,) + shape)


@pytest.mark.parametrize("shape,depth,f,precision", [((4, 4), 3, 16, "fp32"), ((3, 5), 2, 32, "fp32"),
                                                     ((4, 4), 3, 16, "bf16"), ((6, 6), 4, 32, "bf16")])
def test_forward_with_mask_matches_oracle(cuda, shape, depth, f, precision):
    m = _machine(shape, depth, f, precision)
    s = _configs(shape, 200, 1)
    got = m.log_psi(torch.as_tensor(s).cuda()).cpu().numpy().astype(np.complex128)
    want = ar2d.log_psi_numpy(m.params_dict_cpu(), s, depth, True, equal_up_down=True)
    inf = np.isneginf(want.real)
    assert np.array_equal(np.isneginf(got.real), inf)
    if int(np.prod(shape)) % 2 == 0:
        # psi vanishes exactly off the Sz = 0 sector
        assert np.array_equal(inf, s.reshape(len(s), -1).sum(axis=1) != 0)
    tol = 1e-5 if precision == "fp32" else 2e-2
    np.testing.assert_allclose(got.real[~inf], want.real[~inf], rtol=tol, atol=tol * max(1.0, np.abs(want.real[~inf]).max()))


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_sampler_with_mask_stays_in_sector(cuda, precision):
    """Every draw has Sz = 0; sampler log psi equals the forward's bitwise; the
    exact distribution sums to one over the Sz = 0 sector and is zero outside."""
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape = (4, 4)
    m = _machine(shape, 3, 16, precision, seed=2)
    spins, lp, _ = FastAutoregressiveSampler(m, 512, seed=7).sample()
    assert np.all(spins.view(512, -1).sum(dim=1).cpu().numpy() == 0)
    fwd, _, _ = m.forward(spins)
    assert torch.equal(fwd, lp)
    states = torch.as_tensor(exact.all_states(shape)).cuda()
    lp_all = m.log_psi(states).real.double().cpu().numpy()
    p = np.exp(2 * lp_all)
    sz0 = exact.all_states(shape).reshape(-1, 16).sum(axis=1) == 0
    assert np.all(p[~sz0] == 0.0)
    assert p[sz0].sum() == pytest.approx(1.0, abs=2e-4 if precision == "fp32" else 2e-2)


def test_pipelined_engine_with_mask_equals_per_pixel(cuda, tmp_path):
    """The pipelined engine's head applies the same mask bits as the per-pixel
    engine: bitwise equal log psi (BF16, 10x10)."""
    import os
    import subprocess
    import sys
    s = _configs((10, 10), 256, 3)
    np.save(tmp_path / "s.npy", s)
    code = (
        "import sys, numpy as np, torch\n"
        "sys.path.insert(0, %r)\n"
        "from tests.test_equal_up_down_gpu import _machine\n"
        "m = _machine((10, 10), 4, 32, 'bf16', seed=4)\n"
        "s = torch.as_tensor(np.load(%r)).cuda()\n"
        "lp, _, _ = m.forward(s)\n"
        "np.save(%r, lp.cpu().numpy())\n")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    outs = []
    for engine in ("pipe", "rowwise"):
        out = tmp_path / f"{engine}.npy"
        env = dict(os.environ)
        if engine == "rowwise":
            env["FK_AR2D_ENGINE"] = "rowwise"
        else:
            env.pop("FK_AR2D_ENGINE", None)
        subprocess.run([sys.executable, "-c", code % (root, str(tmp_path / "s.npy"), str(out))], check=True, env=env,
                       cwd=root)
        outs.append(np.load(out))
    assert np.array_equal(outs[0], outs[1])
    assert np.isneginf(outs[0][:, 0]).sum() > 0


def test_gradient_with_mask_matches_oracle(cuda):
    from flowket_gb300 import _lib
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape, depth = (4, 4), 3
    m = _machine(shape, depth, 16, "fp32", seed=5)
    spins, _, _ = FastAutoregressiveSampler(m, 150, seed=3).sample()
    _, _, saved = m.forward(spins, mode=_lib.FK_AR2D_SAVE)
    w = np.random.default_rng(0).normal(size=(150, 2)).astype(np.float32)
    got = m.backward(spins, w, saved).cpu().numpy().astype(np.float64)
    g = ar2d.weighted_gradient(m.params_dict_cpu(), spins.cpu().numpy(), depth, True, w[:, 0], w[:, 1],
                               equal_up_down=True)
    ref = torch.cat([g[name].reshape(-1) for name, _, _ in m.layout]).numpy()
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert rel < 1e-4, rel


@pytest.mark.parametrize("which", ["heisenberg", "ising"])
def test_local_energy_with_mask_matches_oracle(cuda, which):
    """Heisenberg keeps the connections in the sector; Ising's single flips leave
    it, where psi = 0: those terms vanish. Through the causal-reuse path."""
    from flowket_gb300.observables import Observable
    from flowket_gb300.operators import Heisenberg, Ising
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape, depth = (4, 4), 3
    m = _machine(shape, depth, 16, "fp32", seed=6)
    if which == "heisenberg":
        op, fc = Heisenberg(hilbert_state_shape=shape, pbc=True), lambda s: ref_ops.heisenberg_find_conn(s, pbc=True)
    else:
        op, fc = Ising(h=3.0, hilbert_state_shape=shape, pbc=True), lambda s: ref_ops.ising_find_conn(s, h=3.0, pbc=True)
    spins, lp, saved = FastAutoregressiveSampler(m, 128, seed=8).sample()
    got = Observable(op).local_values(m, spins, log_psi=lp, base_saved=saved)
    got = got[:, 0].cpu().numpy() + 1j * got[:, 1].cpu().numpy()
    params = m.params_dict_cpu()
    wf = lambda x: ar2d.log_psi_numpy(params, np.asarray(x).astype(np.int8), depth, True, equal_up_down=True)
    conn, mel, use = fc(spins.cpu().numpy())
    want = local_energy.local_values(wf, conn, mel, use)
    assert np.all(np.isfinite(got))
    np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-4 * np.abs(want).max())
