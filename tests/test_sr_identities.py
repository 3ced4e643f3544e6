"""The sample-space SR arithmetic of the streamed route, on the CPU in FP64,
against the oracle's parameter-space solve (oracle/sr.py, which restates
optimizers/stochastic_reconfiguration/optimizer.py:55-114):

* the Gram of the centred rows Y = [Re O_c | Im O_c] accumulated block by
  block over parameter rows, each block centred on its own (what
  fk_ar2d_sr_gram does conv by conv), equals the Gram of the whole array;
* the update x = Y_c alpha / B equals the seed-weighted sum of the
  uncentred rows with the centred seeds (alpha_b - mean, alpha_{B+b} - mean)
  / B (what the streamed route computes with one summed adjoint);
* x equals the parameter-space solve (Re<O_c^* O_c> + lambda) x =
  Re<O_c^* E_c> (the Woodbury identity behind the sample-space solve)."""
import numpy as np
import pytest

from oracle import sr as ref_sr


@pytest.mark.parametrize("p,b,lam", [(300, 40, 1e-2), (57, 96, 1e-3), (1000, 8, 0.1)])
def test_streamed_sample_space_sr_equals_parameter_space_solve(p, b, lam):
    rng = np.random.default_rng(p + b)
    o = rng.normal(size=(b, p)) + 1j * rng.normal(size=(b, p))   # O[b][p] = d log psi_b / d theta_p
    e = rng.normal(size=b) + 1j * rng.normal(size=b)
    y = np.concatenate([o.real.T, o.imag.T], axis=1)                # P x 2B, uncentred
    yc = np.concatenate([o.real.T - o.real.T.mean(1, keepdims=True),
                         o.imag.T - o.imag.T.mean(1, keepdims=True)], axis=1)
    # the Gram block by block over parameter rows, each block centred alone
    gram = np.zeros((2 * b, 2 * b))
    edges = [0, 7, 8, p // 3, p // 2 + 1, p]
    for r0, r1 in zip(edges[:-1], edges[1:]):
        blk = y[r0:r1]
        blk = np.concatenate([blk[:, :b] - blk[:, :b].mean(1, keepdims=True),
                              blk[:, b:] - blk[:, b:].mean(1, keepdims=True)], axis=1)
        gram += blk.T @ blk
    np.testing.assert_allclose(gram, yc.T @ yc, rtol=1e-12, atol=1e-12 * np.abs(gram).max())
    ec = e - e.mean()
    alpha = np.linalg.solve(gram / b + lam * np.eye(2 * b), np.concatenate([ec.real, ec.imag]))
    x_stored = yc @ alpha / b
    seeds = np.stack([alpha[:b] - alpha[:b].mean(), alpha[b:] - alpha[b:].mean()], axis=1) / b
    x_summed = y[:, :b] @ seeds[:, 0] + y[:, b:] @ seeds[:, 1]
    np.testing.assert_allclose(x_summed, x_stored, rtol=1e-10, atol=1e-12 * np.abs(x_stored).max())
    x_param = ref_sr.sr_real(o, e, lam)
    np.testing.assert_allclose(x_stored, x_param, rtol=1e-8, atol=1e-10 * np.abs(x_param).max())
