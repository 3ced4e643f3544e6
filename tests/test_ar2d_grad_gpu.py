"""Adjoint kernel: gradients against the oracle's autograd (float64).

Tolerances: FP32 path ||g - g_ref|| / ||g_ref|| < 1e-4. BF16 path (bf16
activations from the tensor-core forward, fp32 weights and gradients; with
F = 32 the adjoint itself runs on tensor cores with bf16 gradients between
its ops): the stated bound is ||g - g_ref|| / ||g_ref|| < 1e-1 with cosine
similarity > 0.995, for random +-seeds (which maximise cancellation between
samples). The tensor-core adjoint against the CUDA-core adjoint on the same
bf16 activations: relative difference < 3e-2, cosine > 0.999.
"""
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

from oracle import ar2d

pytestmark = pytest.mark.gpu

CASES = [((4, 4), 3, 16, True), ((3, 5), 4, 32, False), ((4, 4), 2, 64, True), ((1, 12), 4, 16, True)]


def _setup(shape, depth, f, wn, precision, b=150, seed=0):
    from flowket_gb300 import _lib
    from flowket_gb300.machines import ConvNetAutoregressive2D
    m = ConvNetAutoregressive2D(shape, depth, f, weights_normalization=wn, precision=precision, seed=seed)
    rng = np.random.default_rng(seed + 1)
    s = rng.choice([-1, 1], size=(b,) + shape).astype(np.int8)
    w = rng.normal(size=(b, 2)).astype(np.float32)
    sc = torch.as_tensor(s).cuda()
    _, _, saved = m.forward(sc, mode=_lib.FK_AR2D_SAVE)
    return m, s, sc, w, saved


def _flat(m, grads):
    return torch.cat([grads[name].reshape(-1) for name, _, _ in m.layout]).numpy()


@pytest.mark.parametrize("shape,depth,f,wn", CASES)
def test_gradient_fp32_matches_autograd(cuda, shape, depth, f, wn):
    m, s, sc, w, saved = _setup(shape, depth, f, wn, "fp32")
    got = m.backward(sc, w, saved).cpu().numpy().astype(np.float64)
    ref = _flat(m, ar2d.weighted_gradient(m.params_dict_cpu(), s, depth, wn, w[:, 0], w[:, 1]))
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert rel < 1e-4, rel


BF16_CASES = CASES[:2] + [((10, 10), 10, 32, True), ((1, 12), 4, 32, True), ((6, 3), 5, 32, True)]


@pytest.mark.parametrize("shape,depth,f,wn", BF16_CASES)
def test_gradient_bf16_within_bound(cuda, shape, depth, f, wn):
    m, s, sc, w, saved = _setup(shape, depth, f, wn, "bf16")
    got = m.backward(sc, w, saved).cpu().numpy().astype(np.float64)
    ref = _flat(m, ar2d.weighted_gradient(m.params_dict_cpu(), s, depth, wn, w[:, 0], w[:, 1]))
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    cos = got @ ref / (np.linalg.norm(got) * np.linalg.norm(ref))
    assert rel < 1e-1 and cos > 0.995, (rel, cos)


def test_per_sample_rows_match_autograd(cuda):
    shape, depth, f, wn = (3, 4), 3, 16, True
    m, s, sc, w, saved = _setup(shape, depth, f, wn, "fp32", b=130)
    o = m.log_derivatives(sc, saved).cpu().numpy()
    for b in (0, 77, 129):
        e = np.zeros(130)
        e[b] = 1.0
        gre = _flat(m, ar2d.weighted_gradient(m.params_dict_cpu(), s, depth, wn, e, 0 * e))
        gim = _flat(m, ar2d.weighted_gradient(m.params_dict_cpu(), s, depth, wn, 0 * e, e))
        ref = gre + 1j * gim
        assert np.linalg.norm(o[:, b] - ref) / np.linalg.norm(ref) < 1e-4
    # the summed gradient is the seed-weighted sum of the rows
    summed = m.backward(sc, w, saved).cpu().numpy()
    np.testing.assert_allclose(o.real @ w[:, 0] + o.imag @ w[:, 1], summed, rtol=1e-3, atol=1e-5)


@pytest.mark.parametrize("precision", ["fp32", "bf16", "fp16"])
def test_sampler_activations_feed_the_adjoint(cuda, precision):
    """The sampler's workspace holds the same activations as a forward pass."""
    from flowket_gb300 import _lib
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.samplers import FastAutoregressiveSampler
    m = ConvNetAutoregressive2D((4, 4), 3, 16, weights_normalization=True, precision=precision, seed=2)
    spins, lp, saved = FastAutoregressiveSampler(m, 200, seed=3).sample()
    w = torch.randn((200, 2), device="cuda")
    g1 = m.backward(spins, w, saved).clone()
    _, _, saved2 = m.forward(spins, mode=_lib.FK_AR2D_SAVE)
    g2 = m.backward(spins, w, saved2)
    assert torch.equal(g1, g2)


@pytest.mark.parametrize("precision", ["bf16", "fp16"])
@pytest.mark.parametrize("shape,depth", [((5, 7), 4), ((10, 10), 10)])
def test_tensor_core_adjoint_matches_cuda_core_adjoint(cuda, tmp_path, shape, depth, precision):
    """F = 32, BF16: the tcgen05 adjoint (bf16 gradients between ops,
    deterministic sums) against the CUDA-core adjoint on the same saved
    activations (FK_AR2D_ENGINE=rowwise selects the CUDA-core adjoint and the
    per-pixel forward, which computes bitwise the same activations)."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = (
        "import sys; sys.path.insert(0, %r);"
        "import numpy as np, torch;"
        "from flowket_gb300 import _lib;"
        "from flowket_gb300.machines import ConvNetAutoregressive2D;"
        "m = ConvNetAutoregressive2D(%r, %d, 32, weights_normalization=True, precision=%r, seed=5);"
        "rng = np.random.default_rng(6);"
        "s = torch.as_tensor(rng.choice([-1, 1], size=(300,) + %r).astype(np.int8)).cuda();"
        "w = torch.as_tensor(rng.normal(size=(300, 2)).astype(np.float32)).cuda();"
        "_, _, saved = m.forward(s, mode=_lib.FK_AR2D_SAVE);"
        "np.save(%r, m.backward(s, w, saved).cpu().numpy())"
    ) % (root, shape, depth, precision, shape, str(tmp_path / "g.npy"))
    env = dict(os.environ, FK_AR2D_ENGINE="rowwise")
    subprocess.run([sys.executable, "-c", code], check=True, env=env)
    ref = np.load(tmp_path / "g.npy").astype(np.float64)
    from flowket_gb300 import _lib
    from flowket_gb300.machines import ConvNetAutoregressive2D
    m = ConvNetAutoregressive2D(shape, depth, 32, weights_normalization=True, precision=precision, seed=5)
    rng = np.random.default_rng(6)
    s = torch.as_tensor(rng.choice([-1, 1], size=(300,) + shape).astype(np.int8)).cuda()
    w = torch.as_tensor(rng.normal(size=(300, 2)).astype(np.float32)).cuda()
    _, _, saved = m.forward(s, mode=_lib.FK_AR2D_SAVE)
    g1 = m.backward(s, w, saved).clone()
    g2 = m.backward(s, w, saved)
    assert torch.equal(g1, g2)  # fixed-order sums: deterministic
    got = g1.cpu().numpy().astype(np.float64)
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    cos = got @ ref / (np.linalg.norm(got) * np.linalg.norm(ref))
    assert rel < 3e-2 and cos > 0.999, (rel, cos)


@pytest.mark.parametrize("recompute", [None, 48])
@pytest.mark.parametrize("precision", ["fp32", "bf16", "fp16"])
def test_autograd_function_equals_machine_backward(cuda, precision, recompute):
    """torch.autograd through Ar2dLogPsi (with and without chunked activation
    recomputation) gives the gradient of m.backward on the same seeds."""
    from flowket_gb300 import _lib
    shape, depth, f, wn = (4, 4), 3, 32, True
    m, s, sc, w, saved = _setup(shape, depth, f, wn, precision, b=150)
    want = m.backward(sc, w, saved).cpu().numpy().astype(np.float64)
    p = m.params.detach().requires_grad_(True)
    lp = m.log_psi_autograd(sc, params=p, recompute_chunk=recompute)
    loss = (lp * torch.as_tensor(w).cuda()).sum()
    loss.backward()
    got = p.grad.cpu().numpy().astype(np.float64)
    if recompute is None:
        # same activations, same adjoint: bitwise
        np.testing.assert_array_equal(got, want)
    rel = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert rel < 1e-5, rel
    # the oracle's gradient agrees as well (FP32 path)
    if precision == "fp32":
        ref = _flat(m, ar2d.weighted_gradient(m.params_dict_cpu(), s, depth, wn, w[:, 0], w[:, 1]))
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-4


def test_backward_recompute_equals_saved_adjoint(cuda):
    shape, depth, f, wn = (10, 10), 10, 32, True
    m, s, sc, w, saved = _setup(shape, depth, f, wn, "bf16", b=256)
    want = m.backward(sc, w, saved).cpu().numpy().astype(np.float64)
    got = m.backward_recompute(sc, w, chunk=128).cpu().numpy().astype(np.float64)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-5


@pytest.mark.parametrize("precision", ["bf16", "fp16"])
def test_tensor_core_per_sample_rows_match_cuda_core(cuda, tmp_path, precision):
    """Per-sample O on the tensor-core path (data gradients on tcgen05 with
    16-bit gradients between ops, per-sample weight gradients on CUDA cores)
    against the CUDA-core adjoint's rows on the same saved activations
    (FK_AR2D_ENGINE=rowwise): the same bound as the summed gradients
    (relative < 3e-2, cosine > 0.999), per sample and overall."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    shape, depth, b = (5, 7), 4, 160
    code = (
        "import sys; sys.path.insert(0, %r);"
        "import numpy as np, torch;"
        "from flowket_gb300 import _lib;"
        "from flowket_gb300.machines import ConvNetAutoregressive2D;"
        "m = ConvNetAutoregressive2D(%r, %d, 32, weights_normalization=True, precision=%r, seed=5);"
        "rng = np.random.default_rng(6);"
        "s = torch.as_tensor(rng.choice([-1, 1], size=(%d,) + %r).astype(np.int8)).cuda();"
        "_, _, saved = m.forward(s, mode=_lib.FK_AR2D_SAVE);"
        "np.save(%r, m.log_derivatives(s, saved).cpu().numpy())"
    ) % (root, shape, depth, precision, b, shape, str(tmp_path / "o.npy"))
    env = dict(os.environ, FK_AR2D_ENGINE="rowwise")
    subprocess.run([sys.executable, "-c", code], check=True, env=env)
    ref = np.load(tmp_path / "o.npy").astype(np.complex128)
    from flowket_gb300 import _lib
    from flowket_gb300.machines import ConvNetAutoregressive2D
    m = ConvNetAutoregressive2D(shape, depth, 32, weights_normalization=True, precision=precision, seed=5)
    rng = np.random.default_rng(6)
    s = torch.as_tensor(rng.choice([-1, 1], size=(b,) + shape).astype(np.int8)).cuda()
    _, _, saved = m.forward(s, mode=_lib.FK_AR2D_SAVE)
    got = m.log_derivatives(s, saved).cpu().numpy().astype(np.complex128)
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert rel < 3e-2, rel
    for part in (np.real, np.imag):
        g, r = part(got), part(ref)
        cos = (g * r).sum(0) / (np.linalg.norm(g, axis=0) * np.linalg.norm(r, axis=0))
        assert cos.min() > 0.999, cos.min()
    # the rows weighted by the seeds sum to the summed tensor-core gradient
    w = rng.normal(size=(b, 2)).astype(np.float32)
    summed = m.backward(s, torch.as_tensor(w).cuda(), saved).cpu().numpy().astype(np.float64)
    from_rows = got.real @ w[:, 0] + got.imag @ w[:, 1]
    assert np.linalg.norm(from_rows - summed) / np.linalg.norm(summed) < 3e-2


@pytest.mark.parametrize("precision", ["bf16", "fp16"])
@pytest.mark.parametrize("shape,depth,b", [((5, 7), 4, 130), ((10, 10), 5, 256), ((16, 16), 3, 64)])
def test_per_sample_weight_gradients_on_tensor_cores(cuda, tmp_path, shape, depth, b, precision):
    """The per-sample weight and bias gradients of the tensor-core adjoint on
    the tensor cores (wgrad_rows_tc_kernel: per sample, the tap-shifted input
    activations times the output gradients over K = pixels) against the
    CUDA-core per-sample kernel on the same 16-bit gradient tensors
    (FK_AR2D_ROWS=cuda): both sum the same products in FP32, in different
    orders. A batch that is not a multiple of 8 (130) has a partial last
    group of samples; 16x16 stages one sample at a time."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = (
        "import sys; sys.path.insert(0, %r);"
        "import numpy as np, torch;"
        "from flowket_gb300 import _lib;"
        "from flowket_gb300.machines import ConvNetAutoregressive2D;"
        "m = ConvNetAutoregressive2D(%r, %d, 32, weights_normalization=True, precision=%r, seed=9);"
        "rng = np.random.default_rng(10);"
        "s = torch.as_tensor(rng.choice([-1, 1], size=(%d,) + %r).astype(np.int8)).cuda();"
        "_, _, saved = m.forward(s, mode=_lib.FK_AR2D_SAVE);"
        "np.save(%r, m.log_derivatives(s, saved).cpu().numpy())"
    ) % (root, shape, depth, precision, b, shape, str(tmp_path / "o.npy"))
    env = dict(os.environ, FK_AR2D_ROWS="cuda")
    subprocess.run([sys.executable, "-c", code], check=True, env=env)
    ref = np.load(tmp_path / "o.npy").astype(np.complex128)
    from flowket_gb300 import _lib
    from flowket_gb300.machines import ConvNetAutoregressive2D
    m = ConvNetAutoregressive2D(shape, depth, 32, weights_normalization=True, precision=precision, seed=9)
    rng = np.random.default_rng(10)
    s = torch.as_tensor(rng.choice([-1, 1], size=(b,) + shape).astype(np.int8)).cuda()
    _, _, saved = m.forward(s, mode=_lib.FK_AR2D_SAVE)
    got = m.log_derivatives(s, saved).cpu().numpy().astype(np.complex128)
    assert got.shape == ref.shape == (m.num_params, b)
    err = np.abs(got - ref).max(axis=0) / np.abs(ref).max(axis=0)
    assert err.max() < 1e-5, err.max()


@pytest.mark.parametrize("shape,depth,b", [((6, 6), 3, 130), ((16, 16), 2, 40)])
def test_per_sample_weight_gradients_on_tensor_cores_f64(cuda, tmp_path, shape, depth, b):
    """64 channels (the CUDA-core adjoint of the BF16 path, float gradients):
    the per-sample weight gradients on the tensor cores, the float gradients
    rounded to bf16 operands, against the CUDA-core per-sample kernel on the
    same float gradients (FK_AR2D_ROWS=cuda). max |d row| / max |row| per
    sample, from the bf16 rounding of the gradients: measured 7.6e-4 (6x6)
    and 5.5e-4 (16x16); bound 3e-3."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = (
        "import sys; sys.path.insert(0, %r);"
        "import numpy as np, torch;"
        "from flowket_gb300 import _lib;"
        "from flowket_gb300.machines import ConvNetAutoregressive2D;"
        "m = ConvNetAutoregressive2D(%r, %d, 64, weights_normalization=True, precision='bf16', seed=11);"
        "rng = np.random.default_rng(12);"
        "s = torch.as_tensor(rng.choice([-1, 1], size=(%d,) + %r).astype(np.int8)).cuda();"
        "_, _, saved = m.forward(s, mode=_lib.FK_AR2D_SAVE);"
        "np.save(%r, m.log_derivatives(s, saved).cpu().numpy())"
    ) % (root, shape, depth, b, shape, str(tmp_path / "o.npy"))
    env = dict(os.environ, FK_AR2D_ROWS="cuda")
    subprocess.run([sys.executable, "-c", code], check=True, env=env)
    ref = np.load(tmp_path / "o.npy").astype(np.complex128)
    from flowket_gb300 import _lib
    from flowket_gb300.machines import ConvNetAutoregressive2D
    m = ConvNetAutoregressive2D(shape, depth, 64, weights_normalization=True, precision="bf16", seed=11)
    rng = np.random.default_rng(12)
    s = torch.as_tensor(rng.choice([-1, 1], size=(b,) + shape).astype(np.int8)).cuda()
    _, _, saved = m.forward(s, mode=_lib.FK_AR2D_SAVE)
    got = m.log_derivatives(s, saved).cpu().numpy().astype(np.complex128)
    err = np.abs(got - ref).max(axis=0) / np.abs(ref).max(axis=0)
    assert err.max() < 3e-3, err.max()
