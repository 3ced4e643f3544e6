"""Symmetrised ensembles (machines/ensemble.py:14-69): the combination rules
and the symmetry images on the host (CPU), the ensemble log psi against the
oracle and its invariances on the GPU."""
import math

import numpy as np
import pytest
import torch

from oracle import ar2d


class _Stub:
    """A machine whose log psi is a fixed function of the configuration."""

    def __init__(self, shape, fn):
        self.hilbert_state_shape = shape
        self.device = torch.device("cpu")
        self.fn = fn

    def forward(self, spins, mode=0, with_cond=False, workspace=None):
        return self.fn(spins), None, None


def _members(x):
    # an arbitrary, asymmetric function of the configuration
    h, w = x.shape[1:]
    wts = torch.arange(1, h * w + 1, dtype=torch.float32).view(1, h, w)
    s = (x.float() * wts).sum((1, 2))
    return torch.stack((0.01 * s, 0.1 * s), dim=1)


def test_combination_rules_match_complex_arithmetic():
    from flowket_gb300.ensemble import EnsembleMachine
    g = torch.Generator().manual_seed(0)
    lp = torch.randn((5, 6, 2), generator=g, dtype=torch.float64)
    z = np.exp(lp[..., 0].numpy() + 1j * lp[..., 1].numpy())
    e = EnsembleMachine(_Stub((2, 2), None), [lambda x: x] * 6, probabilistic=True)
    got = e._combine(lp).double().numpy()
    want_re = 0.5 * np.log(np.mean(np.abs(z) ** 2, axis=1))
    want_im = np.angle(np.mean(np.exp(1j * lp[..., 1].numpy()), axis=1))
    np.testing.assert_allclose(got[:, 0], want_re, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(got[:, 1], want_im, rtol=1e-6, atol=1e-6)
    e.probabilistic = False
    got = e._combine(lp).double().numpy()
    m = np.mean(z, axis=1)
    np.testing.assert_allclose(got[:, 0], np.log(np.abs(m)), rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(got[:, 1], np.angle(m), rtol=1e-6, atol=1e-6)
    # identical members: the ensemble is the member
    one = lp[:, :1].expand(5, 6, 2)
    e.probabilistic = True
    np.testing.assert_allclose(e._combine(one).double().numpy(), lp[:, 0].numpy(), rtol=1e-6, atol=1e-6)


def test_images_are_the_symmetry_group():
    from flowket_gb300.ensemble import make_2d_obc_invariants, make_pbc_invariants, make_up_down_invariant
    x = torch.tensor([[[1, -1, -1], [1, 1, -1], [-1, -1, -1]]], dtype=torch.int8)
    stub = _Stub((3, 3), _members)
    d4 = make_2d_obc_invariants(stub)
    imgs = d4._images(x)[0]
    assert imgs.shape == (8, 3, 3)
    assert len({tuple(i.flatten().tolist()) for i in imgs}) == 8  # an asymmetric configuration has 8 images
    # the image set is closed under the group: a rotated input gives the same set
    imgs_r = d4._images(torch.rot90(x, 1, dims=(1, 2)))[0]
    assert {tuple(i.flatten().tolist()) for i in imgs} == {tuple(i.flatten().tolist()) for i in imgs_r}
    pbc = make_pbc_invariants(stub, apply_also_obc_invariants=False)
    assert pbc.ensemble_size == 9
    assert torch.equal(pbc._images(x)[0, 4], torch.roll(x[0], shifts=(1, 1), dims=(0, 1)))
    ud = make_up_down_invariant(stub)
    assert torch.equal(ud._images(x)[0, 1], -x[0])
    # invariance of the combined value (host stub)
    full = make_pbc_invariants(stub)
    a, _, _ = full.forward(x)
    b, _, _ = full.forward(torch.roll(torch.flip(x, dims=(2,)), shifts=(2, 1), dims=(1, 2)))
    np.testing.assert_allclose(a.numpy(), b.numpy(), rtol=1e-6, atol=1e-6)
    with pytest.raises(ValueError):
        make_2d_obc_invariants(_Stub((2, 3), _members))


@pytest.mark.gpu
@pytest.mark.parametrize("probabilistic", [True, False])
def test_ensemble_log_psi_matches_oracle(cuda, probabilistic):
    from flowket_gb300.ensemble import make_2d_obc_invariants, make_up_down_invariant
    from flowket_gb300.machines import ConvNetAutoregressive2D
    shape, depth = (4, 4), 3
    m = ConvNetAutoregressive2D(shape, depth, 16, weights_normalization=True, precision="fp32", seed=2)
    e = make_up_down_invariant(make_2d_obc_invariants(m, probabilistic), probabilistic)
    g = torch.Generator().manual_seed(0)
    x = (2 * torch.randint(0, 2, (64, 4, 4), generator=g) - 1).to(torch.int8)
    got, _, _ = e.forward(x.cuda())
    got = got.double().cpu().numpy()
    params = m.params_dict_cpu()
    xs = x.numpy()
    imgs = []
    for k in range(4):
        r = np.rot90(xs, k, axes=(1, 2))
        imgs += [r, r[:, :, ::-1]]
    lps = np.stack([ar2d.log_psi_numpy(params, np.ascontiguousarray(i).astype(np.int8), depth, True) for i in imgs], 1)

    def comb(lp):
        if probabilistic:
            re = 0.5 * np.log(np.mean(np.exp(2 * lp.real), axis=1))
            return re + 1j * np.angle(np.mean(np.exp(1j * lp.imag), axis=1))
        return np.log(np.mean(np.exp(lp), axis=1))

    inner = comb(lps)
    lps_f = np.stack([ar2d.log_psi_numpy(params, np.ascontiguousarray(-i).astype(np.int8), depth, True) for i in imgs], 1)
    want = comb(np.stack([inner, comb(lps_f)], 1))
    np.testing.assert_allclose(got[:, 0], want.real, rtol=1e-5, atol=1e-4)
    dphase = np.angle(np.exp(1j * (got[:, 1] - want.imag)))
    assert np.abs(dphase).max() < 1e-4
    # invariance under the group on the GPU
    b, _, _ = e.forward(torch.flip(torch.rot90(x, 1, dims=(1, 2)), dims=(2,)).cuda() * -1)
    np.testing.assert_allclose(b.double().cpu().numpy()[:, 0], got[:, 0], rtol=1e-5, atol=1e-5)


@pytest.mark.gpu
def test_vmc_evaluates_ensemble_with_base_sampler(cuda):
    """The reference's evaluation (experiments/run_evaluation.py:12-24): samples
    of the base machine, local energies of the ensemble."""
    from flowket_gb300.ensemble import make_2d_obc_invariants
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.observables import Observable
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.optimization import VariationalMonteCarlo
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape = (4, 4)
    m = ConvNetAutoregressive2D(shape, 3, 16, weights_normalization=False, precision="fp32", seed=0)
    e = make_2d_obc_invariants(m)
    op = Heisenberg(hilbert_state_shape=shape, pbc=True)
    vmc = VariationalMonteCarlo(e, op, FastAutoregressiveSampler(m, 128, seed=5))
    spins, y = vmc.next_batch()
    want = Observable(op).local_values(e, spins)
    got = vmc.current_local_energy
    np.testing.assert_allclose(got.real.cpu().numpy(), want[:, 0].cpu().numpy(), rtol=1e-6, atol=1e-6)
    assert math.isfinite(vmc.current_energy.real)
