"""Kernel set (d): sample-space SR against the oracle's parameter-space solve."""
import numpy as np
import pytest
import torch

from oracle import ar2d, sr as ref_sr

pytestmark = pytest.mark.gpu


def test_gram_and_solve_match_numpy(cuda):
    from flowket_gb300 import _lib
    rng = np.random.default_rng(0)
    p, b = 3000, 96
    a = rng.normal(size=(p, b)).astype(np.float32)
    c = rng.normal(size=(p, b)).astype(np.float32)
    ta, tc = torch.as_tensor(a).cuda(), torch.as_tensor(c).cuda()
    n = 2 * b
    gram = torch.empty((n, n), dtype=torch.float64, device="cuda")
    _lib.call("fk_sr_gram", _lib.ptr(ta), _lib.ptr(tc), p, b, _lib.ptr(gram), n * n, _lib.stream_ptr())
    y = np.concatenate([a, c], axis=1).astype(np.float64)
    want = y.T @ y
    np.testing.assert_allclose(gram.cpu().numpy(), want, rtol=1e-5, atol=1e-3)
    rhs = torch.as_tensor(rng.normal(size=n)).cuda()
    x = torch.empty(n, dtype=torch.float64, device="cuda")
    stats = torch.zeros(3, dtype=torch.float64, device="cuda")
    ws = torch.empty(_lib.load().fk_sr_solve_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    _lib.call("fk_sr_solve", _lib.ptr(gram), n, 1.0 / p, 0.05, _lib.ptr(rhs), 1e-12, 500, _lib.ptr(x),
              _lib.ptr(stats), _lib.ptr(ws), ws.numel(), _lib.stream_ptr())
    # the solver against a dense FP64 solve of the same (GPU-built) matrix
    ref = np.linalg.solve(gram.cpu().numpy() / p + 0.05 * np.eye(n), rhs.cpu().numpy())
    np.testing.assert_allclose(x.cpu().numpy(), ref, rtol=1e-8, atol=1e-10)
    assert 0 < stats[0].item() <= 500


@pytest.mark.parametrize("p,b,complex_", [(3000, 96, True), (4133, 200, True), (70_000, 512, True),
                                         (1000, 40, False), (64, 8, True)])
def test_tensor_core_gram_matches_fp64(cuda, p, b, complex_):
    """fk_sr_gram_tc (tcgen05, split-BF16 products, FP32 accumulation) against
    the FP64 Gram of the same FP32 rows, relative to sqrt(T_ii T_jj): 5e-5
    (the tensor core sums a 4096-parameter range in FP32: 2e-5 measured on
    the diagonal, where every term is positive; 2e-7 off it), and the
    CUDA-core fk_sr_gram at 1e-5. Sizes not multiples of the 128 x 256 tiles
    or of the 64 parameters per stage, and a single tile."""
    from flowket_gb300 import _lib
    rng = np.random.default_rng(p + b)
    a = rng.normal(size=(p, b)).astype(np.float32)
    c = rng.normal(size=(p, b)).astype(np.float32) if complex_ else None
    ta = torch.as_tensor(a).cuda()
    tc = torch.as_tensor(c).cuda() if complex_ else None
    n = 2 * b if complex_ else b
    y = np.concatenate([a, c], axis=1).astype(np.float64) if complex_ else a.astype(np.float64)
    want = y.T @ y
    scale = np.sqrt(np.outer(np.diag(want), np.diag(want)))
    for entry in ("fk_sr_gram_tc", "fk_sr_gram"):
        gram = torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
        _lib.call(entry, _lib.ptr(ta), _lib.ptr(tc), p, b, _lib.ptr(gram), n * n, _lib.stream_ptr())
        got = gram.cpu().numpy()
        err = np.abs(got - want) / scale
        assert err.max() < (5e-5 if entry == "fk_sr_gram_tc" else 1e-5), (entry, err.max())
        off = err[~np.eye(n, dtype=bool)]
        assert off.max() < 2e-6, (entry, off.max())
        np.testing.assert_array_equal(got, got.T)


def test_tensor_core_gram_rejects_unsupported_shapes(cuda):
    from flowket_gb300 import _lib
    lib = _lib.load()
    buf = torch.zeros(1024, dtype=torch.float32, device="cuda")
    g = torch.zeros(1024, dtype=torch.float64, device="cuda")
    assert lib.fk_sr_gram_tc(_lib.ptr(buf), None, 10, 12, _lib.ptr(g), 1024, _lib.stream_ptr()) == -1
    assert b"multiple of 8" in lib.fk_last_error()


@pytest.mark.parametrize("gram", ["fp32", "tc"])
def test_sr_direction_matches_parameter_space_solve(cuda, gram):
    """(Re<O_c^* O_c> + lambda) x = Re<O_c^* E_c>: the sample-space GPU solve
    (Gram on the CUDA cores or on the tensor cores) equals the oracle's
    parameter-space solve on the same O and E_loc."""
    from flowket_gb300 import _lib
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.observables import Observable
    from flowket_gb300.optimizers import ComplexValuesStochasticReconfiguration
    shape, depth, f = (3, 4), 2, 16
    m = ConvNetAutoregressive2D(shape, depth, f, weights_normalization=False, precision="fp32", seed=1)
    rng = np.random.default_rng(2)
    s = torch.as_tensor(rng.choice([-1, 1], size=(96,) + shape).astype(np.int8)).cuda()
    _, _, saved = m.forward(s, mode=_lib.FK_AR2D_SAVE)
    local = Observable(Heisenberg(hilbert_state_shape=shape, pbc=True)).local_values(m, s)
    opt = ComplexValuesStochasticReconfiguration(m, lr=0.05, diag_shift=1e-2, iterative_solver=False, gram=gram)
    x = opt.direction(s, local, saved).cpu().numpy().astype(np.float64)
    o = m.log_derivatives(s, saved).cpu().numpy().T.astype(np.complex128)
    e = local[:, 0].cpu().numpy() + 1j * local[:, 1].cpu().numpy()
    want = ref_sr.sr_real(o, e, 1e-2)
    assert np.linalg.norm(x - want) / np.linalg.norm(want) < 1e-3


def test_vmc_with_sr_lowers_energy(cuda):
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.optimization import VariationalMonteCarlo
    from flowket_gb300.optimizers import ComplexValuesStochasticReconfiguration
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape = (4, 4)
    m = ConvNetAutoregressive2D(shape, 3, 16, weights_normalization=True, precision="fp32", seed=0)
    vmc = VariationalMonteCarlo(m, Heisenberg(hilbert_state_shape=shape, pbc=True),
                                FastAutoregressiveSampler(m, 256, seed=3))
    opt = ComplexValuesStochasticReconfiguration(m, lr=0.05, diag_shift=1e-3)
    energies = []
    for _ in range(30):
        vmc.step(opt)
        energies.append(vmc.current_energy.real)
    assert np.mean(energies[-5:]) < np.mean(energies[:3]) - 1.0
