"""Kernels (a) and (b): AR2D forward and exact sampler against the oracle.

Tolerances: FP32 path log psi within 1e-5 relative of the FP64 oracle (the
reference runs FP32). Tensor-core paths (16-bit operands and stored
activations, FP32 accumulation): |d log psi| <= bound * max(1, |log psi|)
per sample, the bound 3x the worst case measured over 5 seeds on these
cases (BF16 8.4e-4, FP16 1.05e-4, both on the 4x4 depth-5 network).
"""
import numpy as np
import pytest
import torch

from oracle import ar2d, exact, philox

pytestmark = pytest.mark.gpu

FP32_RTOL = 1e-5
TC_BOUND = {"bf16": 2.6e-3, "fp16": 3.2e-4}


def _machine(shape, depth, f, wn, precision, seed=0):
    from flowket_gb300.machines import ConvNetAutoregressive2D
    return ConvNetAutoregressive2D(shape, depth, f, weights_normalization=wn, precision=precision, seed=seed)


def _spins(b, shape, seed):
    rng = np.random.default_rng(seed)
    return rng.choice([-1, 1], size=(b,) + shape).astype(np.int8)


CASES = [((4, 4), 5, 16, False), ((3, 5), 3, 32, True), ((4, 4), 2, 64, True), ((10, 10), 3, 32, True),
         ((1, 12), 4, 16, False)]


def test_init_matches_oracle_init(cuda):
    m = _machine((4, 4), 5, 16, True, "fp32", seed=7)
    want = ar2d.init_params((4, 4), 5, 16, True, seed=7, dtype=torch.float64)
    got = m.params_dict_cpu()
    assert set(got) == set(want)
    for k in want:
        assert torch.allclose(got[k], want[k].to(torch.float32).to(torch.float64), atol=0, rtol=0), k


@pytest.mark.parametrize("shape,depth,f,wn", CASES)
def test_forward_fp32_matches_oracle(cuda, shape, depth, f, wn):
    m = _machine(shape, depth, f, wn, "fp32")
    s = _spins(200, shape, 1)
    got = m.log_psi(torch.as_tensor(s).cuda()).cpu().numpy()
    want = ar2d.log_psi_numpy(m.params_dict_cpu(), s, depth, wn)
    err = np.abs(got - want) / np.maximum(1.0, np.abs(want))
    assert err.max() < FP32_RTOL, err.max()


@pytest.mark.parametrize("precision", ["bf16", "fp16"])
@pytest.mark.parametrize("shape,depth,f,wn", CASES)
def test_forward_tensor_core_within_bound(cuda, shape, depth, f, wn, precision):
    m = _machine(shape, depth, f, wn, precision)
    s = _spins(300, shape, 2)
    got = m.log_psi(torch.as_tensor(s).cuda()).cpu().numpy()
    want = ar2d.log_psi_numpy(m.params_dict_cpu(), s, depth, wn)
    err = np.abs(got - want) / np.maximum(1.0, np.abs(want))
    assert err.max() < TC_BOUND[precision], err.max()


def test_conditionals_fp32(cuda):
    shape, depth = (4, 3), 3
    m = _machine(shape, depth, 16, True, "fp32")
    s = _spins(130, shape, 3)
    got = m.conditional_log_probs(torch.as_tensor(s).cuda()).cpu().numpy()
    re, _ = ar2d.conditional_log_wave_function(m.params_dict_cpu(), torch.as_tensor(s), depth, True)
    np.testing.assert_allclose(got, 2 * re.numpy(), atol=2e-5)


@pytest.mark.parametrize("precision", ["fp32", "bf16", "fp16"])
def test_distribution_normalised_4x4(cuda, precision):
    """tests/test_autoregressive.py:18-30 on the GPU path: sum |psi|^2 = 1."""
    m = _machine((4, 4), 4, 16, False, precision)
    states = torch.as_tensor(exact.all_states((4, 4))).cuda()
    lp = m.log_psi(states).real.double()
    total = torch.logsumexp(2 * lp, 0).exp().item()
    assert total == pytest.approx(1.0, abs=1e-5 if precision == "fp32" else 1e-3)


@pytest.mark.parametrize("precision", ["fp32", "bf16", "fp16"])
def test_sampler_reproduces_oracle_draw(cuda, precision):
    """Same Philox uniforms -> the same samples as the oracle's raster sampler
    run on this machine's own conditionals; sampler log psi == forward log psi."""
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape, depth = (3, 4), 3
    m = _machine(shape, depth, 16, True, precision)
    b = 300
    sampler = FastAutoregressiveSampler(m, b, seed=99, offset=5)
    spins, lp, _ = sampler.sample()
    got = spins.cpu().numpy()

    def cond_lp(batch):
        return m.conditional_log_probs(torch.as_tensor(batch.astype(np.int8)).cuda()).cpu().numpy().astype(np.float64)

    u = philox.ar_site_uniforms(99, 5, b, 12)
    batch = np.zeros((b,) + shape)
    for k in range(12):
        i, j = divmod(k, 4)
        lpk = cond_lp(batch)
        batch[:, i, j] = np.where(np.exp(lpk[:, i, j, 0]) > u[:, k], 1.0, -1.0)
        # later sites in the draw depend only on sampled ones: keep the GPU's
        # draw where the two sides are within rounding of the threshold
        near = np.abs(np.exp(lpk[:, i, j, 0]) - u[:, k]) < 1e-5
        batch[near, i, j] = got[near, i, j]
    assert np.array_equal(batch.astype(np.int8), got)
    fwd = m.log_psi(spins).cpu().numpy()
    samp = torch.complex(lp[:, 0], lp[:, 1]).cpu().numpy()
    assert np.array_equal(fwd, samp)


@pytest.mark.parametrize("precision", ["fp32", "bf16", "fp16"])
def test_sampler_matches_exact_distribution(cuda, precision):
    """tests/test_samplers.py:49-82: closeness statistic z <= sqrt(n) against
    |psi|^2 enumerated with the same machine."""
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape = (3, 3)
    m = _machine(shape, 2, 16, False, precision, seed=3)
    n = 2 ** 15
    states = torch.as_tensor(exact.all_states(shape)).cuda()
    lp = m.log_psi(states).real.double().cpu().numpy()
    probs, _ = exact.exact_distribution(lp)
    got = FastAutoregressiveSampler(m, n, seed=5).sample()[0].cpu().numpy()
    ref = exact.exact_sample(probs, shape, n, np.random.default_rng(0))
    x = np.bincount(exact.states_to_index(got), minlength=512)
    y = np.bincount(exact.states_to_index(ref), minlength=512)
    z = ((np.square(x - y) - x - y) / (x + y + 1e-20)).sum()
    assert z <= np.sqrt(n), z


@pytest.mark.parametrize("precision", ["bf16", "fp16"])
@pytest.mark.parametrize("f", [16, 32])
def test_pipelined_engine_equals_per_pixel_engine(cuda, f, precision, tmp_path):
    """The persistent pipelined tensor-core engine and the per-pixel engine
    give bitwise the same log psi (same MMA sequence, same epilogue)."""
    import subprocess
    import sys
    code = (
        "import sys, numpy as np, torch; sys.path.insert(0, %r);"
        "from flowket_gb300.machines import ConvNetAutoregressive2D;"
        "m = ConvNetAutoregressive2D((5, 7), 4, %d, weights_normalization=True, precision=%r, seed=3);"
        "s = torch.as_tensor(np.random.default_rng(9).choice([-1, 1], size=(700, 5, 7)).astype(np.int8)).cuda();"
        "np.save(%r, m.log_psi(s).cpu().numpy())"
    ) % (str(__import__("os").path.dirname(__import__("os").path.dirname(__file__))), f, precision,
         str(tmp_path / "a.npy"))
    env = dict(__import__("os").environ, FK_AR2D_ENGINE="rowwise")
    subprocess.run([sys.executable, "-c", code], check=True, env=env)
    ref = np.load(tmp_path / "a.npy")
    m = _machine((5, 7), 4, f, True, precision, seed=3)
    s = torch.as_tensor(np.random.default_rng(9).choice([-1, 1], size=(700, 5, 7)).astype(np.int8)).cuda()
    got = m.log_psi(s).cpu().numpy()
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("precision", ["bf16", "fp16"])
@pytest.mark.parametrize("shape,f", [((3, 20), 32), ((2, 40), 16)])
def test_sampler_wide_rows_equals_forward(cuda, shape, f, precision):
    """Rows wider than the TMEM holds at once (W * F > 512): the sampler's
    row-end V ops fall back to one op per pixel; log psi stays bitwise equal
    to the forward's and the draw follows the model (normalised conditionals)."""
    from flowket_gb300.samplers import FastAutoregressiveSampler
    m = _machine(shape, 3, f, True, precision)
    spins, lp, _ = FastAutoregressiveSampler(m, 200, seed=5).sample()
    fwd, _, _ = m.forward(spins)
    assert torch.equal(fwd, lp)
    assert torch.all(torch.isfinite(lp))


@pytest.mark.parametrize("precision", ["bf16", "fp16"])
@pytest.mark.parametrize("updown", [False, True])
def test_sampler_f64_equals_forward(cuda, updown, precision):
    """F = 64 runs the sampler's per-pixel ops; log psi bitwise equal to the
    forward's, with and without the EqualUpDownSpins mask."""
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.samplers import FastAutoregressiveSampler
    m = ConvNetAutoregressive2D((4, 4), 2, 64, weights_normalization=True, precision=precision, seed=3,
                                equal_up_down_spins=updown)
    spins, lp, _ = FastAutoregressiveSampler(m, 256, seed=9).sample()
    fwd, _, _ = m.forward(spins)
    assert torch.equal(fwd, lp)
    if updown:
        assert torch.all(spins.view(256, -1).sum(dim=1) == 0)
