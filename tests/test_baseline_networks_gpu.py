"""Parity at the networks of the benchmark workloads, against the FP64
oracle (oracle/ar2d.py, which restates machines/conv_net_autoregressive_2D.py:24-74):

* net4x4_d5_f16: 4x4, depth 5, 16 channels (no weight norm) -- Heisenberg, Lanczos case;
* net10x10_d10_f32: 10x10, depth 10, 32 channels -- the bench workload (TFIM h=3);
* net10x10_d20_f32: 10x10, depth 20, 32 channels -- the J1-J2 SR case;
* net1x64_d4_f16: 1x64, depth 4, 16 channels -- the learned proposal of the chain;
* net16x16_d20_f64: 16x16, depth 20, 64 channels -- Heisenberg 16x16.

Bounds. FP32 log psi: 1e-5 relative (the reference computes in FP32; the
measured worst case over 5 seeds per network is 3.8e-7). The tensor-core
formats (BF16, FP16 operands and stored activations, FP32 accumulation):
per network, 3x the worst |d log psi| / max(1, |log psi|) measured over 5
seeds of weights and spins (``TC_FORWARD``). Adjoint: ||g - g_ref|| / ||g_ref||
and the cosine for random +-seeds (the worst case: every sample's gradient
cancels against the others'), 3x the measured worst relative error and 3x
the measured worst cosine's distance from 1 (``FP32_ADJOINT``, where ReLU
masks that flip under FP32 rounding set the error, and ``TC_ADJOINT``)."""
import numpy as np
import pytest
import torch

from oracle import ar2d, local_energy as ref_le, operators as ref_ops

pytestmark = pytest.mark.gpu

NETWORKS = {
    "net4x4_d5_f16": ((4, 4), 5, 16, False),
    "net10x10_d10_f32": ((10, 10), 10, 32, True),
    "net10x10_d20_f32": ((10, 10), 20, 32, True),
    "net1x64_d4_f16": ((1, 64), 4, 16, True),
    "net16x16_d20_f64": ((16, 16), 20, 64, True),
}
BATCH = {"net4x4_d5_f16": 256, "net10x10_d10_f32": 64, "net10x10_d20_f32": 32, "net1x64_d4_f16": 128,
         "net16x16_d20_f64": 12}
GRAD_BATCH = {"net4x4_d5_f16": 128, "net10x10_d10_f32": 48, "net10x10_d20_f32": 24, "net1x64_d4_f16": 64,
              "net16x16_d20_f64": 6}

# Measured worst over 5 seeds (weights and spins) per network, with the
# helpers below (forward: max_b |d log psi_b| / max(1, |log psi_b|); adjoint:
# relative error and cosine):
#   net               FP32 fwd  BF16 fwd  FP16 fwd | FP32 adj  BF16 adj (cos)    FP16 adj (cos)
#   net4x4_d5_f16     9.8e-8    6.6e-4    1.0e-4   | 3.0e-7    0.079 (0.99686)   0.026 (0.99966)
#   net10x10_d10_f32  1.1e-7    1.4e-3    1.1e-4   | 1.1e-4    0.087 (0.99629)   0.031 (0.99953)
#   net10x10_d20_f32  1.7e-7    2.5e-3    3.0e-4   | 1.5e-5    0.133 (0.99134)   0.063 (0.99803)
#   net1x64_d4_f16    6.1e-8    1.5e-4    1.9e-5   | 7.2e-7    0.117 (0.99366)   0.031 (0.99953)
#   net16x16_d20_f64  3.8e-7    3.0e-3    4.5e-4   | 7.0e-4    0.123 (0.99272)   0.038 (0.99927)
# Bounds: 3x the worst error (the cosine's distance from 1 times 3).
TC_FORWARD = {
    "bf16": {"net4x4_d5_f16": 2.0e-3, "net10x10_d10_f32": 4.5e-3, "net10x10_d20_f32": 7.5e-3,
             "net1x64_d4_f16": 5.0e-4, "net16x16_d20_f64": 9.0e-3},
    "fp16": {"net4x4_d5_f16": 3.1e-4, "net10x10_d10_f32": 3.5e-4, "net10x10_d20_f32": 9.0e-4,
             "net1x64_d4_f16": 6.0e-5, "net16x16_d20_f64": 1.4e-3},
}
FP32_FORWARD = 1e-5
# (relative error bound, cosine bound)
FP32_ADJOINT = {"net4x4_d5_f16": (1e-6, 1 - 1e-12), "net10x10_d10_f32": (3.3e-4, 1 - 2e-8),
                "net10x10_d20_f32": (4.5e-5, 1 - 4e-10), "net1x64_d4_f16": (2.2e-6, 1 - 1e-12),
                "net16x16_d20_f64": (2.1e-3, 1 - 7.5e-7)}
TC_ADJOINT = {
    "bf16": {"net4x4_d5_f16": (0.24, 0.9906), "net10x10_d10_f32": (0.26, 0.9889), "net10x10_d20_f32": (0.40, 0.9740),
             "net1x64_d4_f16": (0.35, 0.9810), "net16x16_d20_f64": (0.37, 0.9782)},
    "fp16": {"net4x4_d5_f16": (0.078, 0.9990), "net10x10_d10_f32": (0.093, 0.9986),
             "net10x10_d20_f32": (0.19, 0.9941), "net1x64_d4_f16": (0.094, 0.9986),
             "net16x16_d20_f64": (0.115, 0.9978)},
}


def _machine(net, precision, seed):
    from flowket_gb300.machines import ConvNetAutoregressive2D
    shape, depth, f, wn = NETWORKS[net]
    return ConvNetAutoregressive2D(shape, depth, f, weights_normalization=wn, precision=precision, seed=seed)


def _spins(net, b, seed):
    shape = NETWORKS[net][0]
    return np.random.default_rng(1000 + seed).choice([-1, 1], size=(b,) + shape).astype(np.int8)


def _forward_error(net, precision, seed):
    shape, depth, f, wn = NETWORKS[net]
    m = _machine(net, precision, seed)
    s = _spins(net, BATCH[net], seed)
    got = m.log_psi(torch.as_tensor(s).cuda()).cpu().numpy().astype(np.complex128)
    want = ar2d.log_psi_numpy(m.params_dict_cpu(), s, depth, wn)
    d = got - want
    # the imaginary part is a phase: compare it modulo 2 pi
    d = d.real + 1j * np.angle(np.exp(1j * d.imag))
    return float((np.abs(d) / np.maximum(1.0, np.abs(want))).max())


@pytest.mark.parametrize("net", sorted(NETWORKS))
def test_fp32_forward_at_benchmark_network(cuda, net):
    err = _forward_error(net, "fp32", 0)
    assert err < FP32_FORWARD, err


@pytest.mark.parametrize("precision", ["bf16", "fp16"])
@pytest.mark.parametrize("net", sorted(NETWORKS))
def test_tensor_core_forward_at_benchmark_network(cuda, net, precision):
    for seed in (0, 1):
        err = _forward_error(net, precision, seed)
        assert err < TC_FORWARD[precision][net], (seed, err)


def _adjoint_error(net, precision, seed):
    from flowket_gb300 import _lib
    shape, depth, f, wn = NETWORKS[net]
    b = GRAD_BATCH[net]
    m = _machine(net, precision, seed)
    rng = np.random.default_rng(2000 + seed)
    s = rng.choice([-1, 1], size=(b,) + shape).astype(np.int8)
    w = rng.normal(size=(b, 2)).astype(np.float32)
    sc = torch.as_tensor(s).cuda()
    _, _, saved = m.forward(sc, mode=_lib.FK_AR2D_SAVE)
    got = m.backward(sc, w, saved).cpu().numpy().astype(np.float64)
    g = ar2d.weighted_gradient(m.params_dict_cpu(), s, depth, wn, w[:, 0], w[:, 1])
    ref = torch.cat([g[name].reshape(-1) for name, _, _ in m.layout]).numpy()
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    cos = got @ ref / (np.linalg.norm(got) * np.linalg.norm(ref))
    return float(rel), float(cos)


@pytest.mark.parametrize("precision", ["fp32", "bf16", "fp16"])
@pytest.mark.parametrize("net", sorted(NETWORKS))
def test_adjoint_at_benchmark_network(cuda, net, precision):
    rel, cos = _adjoint_error(net, precision, 0)
    bound, cos_bound = FP32_ADJOINT[net] if precision == "fp32" else TC_ADJOINT[precision][net]
    assert rel < bound and cos > cos_bound, (rel, cos)


@pytest.mark.parametrize("precision", ["fp32", "bf16", "fp16"])
@pytest.mark.parametrize("net", ["net10x10_d10_f32", "net16x16_d20_f64"])
def test_sampler_equals_forward_at_benchmark_network(cuda, net, precision):
    """The persistent sampler's log psi is bitwise the forward's on the drawn
    configurations, and its saved activations feed the adjoint like a
    forward's."""
    from flowket_gb300 import _lib
    from flowket_gb300.samplers import FastAutoregressiveSampler
    m = _machine(net, precision, 0)
    b = 256 if net == "net10x10_d10_f32" else 128
    spins, lp, saved = FastAutoregressiveSampler(m, b, seed=31).sample()
    fwd, _, saved2 = m.forward(spins, mode=_lib.FK_AR2D_SAVE)
    assert torch.equal(fwd, lp)
    w = torch.randn((b, 2), device="cuda", generator=torch.Generator(device="cuda").manual_seed(3))
    g1 = m.backward(spins, w, saved).clone()
    g2 = m.backward(spins, w, saved2)
    assert torch.equal(g1, g2)


# local energies of the bench workload (TFIM 10x10 PBC, h = 3) on the net10x10_d10_f32
# network: the reference's local-values algorithm over the oracle's FP64
# log psi; bounds relative to max |E_loc|
ELOC = {"fp32": 1e-5, "bf16": 2e-2, "fp16": 4e-3}


@pytest.mark.parametrize("precision", ["fp32", "bf16", "fp16"])
def test_local_energy_at_bench_workload(cuda, precision):
    from flowket_gb300.observables import Observable
    from flowket_gb300.operators import Ising
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape, depth, f, wn = NETWORKS["net10x10_d10_f32"]
    m = _machine("net10x10_d10_f32", precision, 0)
    spins, lp, saved = FastAutoregressiveSampler(m, 16, seed=5).sample()
    local = Observable(Ising(h=3.0, hilbert_state_shape=shape, pbc=True)).local_values(m, spins, log_psi=lp,
                                                                                      base_saved=saved)
    got = local.cpu().numpy()
    got = got[:, 0] + 1j * got[:, 1]
    s = spins.cpu().numpy()
    conn, mel, use = ref_ops.ising_find_conn(s, h=3.0, pbc=True)
    params = m.params_dict_cpu()
    want = ref_le.local_values(
        lambda x: ar2d.log_psi_numpy(params, np.asarray(x).astype(np.int8), depth, wn), conn, mel, use)
    err = np.abs(got - want).max() / np.abs(want).max()
    assert err < ELOC[precision], err
