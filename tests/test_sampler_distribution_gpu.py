"""The sampled distribution against exact |psi|^2 on the 4x4 lattice (65,536
configurations), for the exact autoregressive sampler in each precision:

* the closeness statistic of tests/test_samplers.py:49-82 (arXiv:1308.3946)
  between the sampler's histogram and an exact sampler's, z <= sqrt(n), with
  n = max(2^16, 16 * 2^16) samples as the reference test takes;
* Pearson's chi-square goodness of fit of the histogram against n |psi|^2
  (bins with expectation < 5 pooled): p-value > 1e-4;
* KL(empirical || |psi|^2) within 10% (+1e-3) of the KL of an exact sampler's
  histogram of the same size (the finite-sample floor, about (k-1)/2n).
|psi|^2 is the machine's own forward over all configurations, normalised in
FP64 (the sampler's log psi is bitwise the forward's)."""
import numpy as np
import pytest
import torch
from scipy import stats

from oracle import exact

pytestmark = pytest.mark.gpu


def _kl(counts, p):
    q = counts / counts.sum()
    nz = q > 0
    return float((q[nz] * np.log(q[nz] / p[nz])).sum())


@pytest.mark.parametrize("precision", ["fp32", "bf16", "fp16"])
def test_sampler_distribution_4x4_kl_and_chi_square(cuda, precision):
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape = (4, 4)
    m = ConvNetAutoregressive2D(shape, 5, 16, weights_normalization=False, precision=precision, seed=11)
    states = torch.as_tensor(exact.all_states(shape)).cuda()
    lp = m.log_psi(states).real.double().cpu().numpy()
    p, _ = exact.exact_distribution(lp)
    n_states = p.shape[0]
    n = max(2 ** 16, 16 * n_states)
    sampler = FastAutoregressiveSampler(m, 1 << 16, seed=77)
    got = np.concatenate([sampler.sample()[0].cpu().numpy() for _ in range(n // (1 << 16))])
    x = np.bincount(exact.states_to_index(got), minlength=n_states).astype(np.float64)
    ref = exact.exact_sample(p, shape, n, np.random.default_rng(3))
    y = np.bincount(exact.states_to_index(ref), minlength=n_states).astype(np.float64)
    z = ((np.square(x - y) - x - y) / (x + y + 1e-20)).sum()
    assert z <= np.sqrt(n), z
    e = n * p
    big = e >= 5
    obs = np.concatenate([x[big], [x[~big].sum()]])
    exp = np.concatenate([e[big], [e[~big].sum()]])
    if exp[-1] < 5:
        obs, exp = obs[:-1], exp[:-1]
    chi2 = float(((obs - exp) ** 2 / exp).sum())
    pval = float(stats.chi2.sf(chi2, obs.shape[0] - 1))
    assert pval > 1e-4, (chi2, obs.shape[0] - 1, pval)
    kl, kl_ref = _kl(x, p), _kl(y, p)
    assert kl < 1.1 * kl_ref + 1e-3, (kl, kl_ref)
