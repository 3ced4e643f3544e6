"""RBMSym's tied-parameter map (host logic, no GPU): expanding a bare
parameter vector through the product's index map gives the oracle's dense
RBM (machines/rbm.py:51-65, layers/complex/dense.py:53-85)."""
import numpy as np
import pytest

from oracle import rbm as ref_rbm


@pytest.mark.parametrize("shape,alpha", [((6,), 2), ((3, 4), 1), ((20, 1), 1), ((4, 4), 3)])
def test_rbm_sym_tied_index_matches_oracle_expansion(shape, alpha):
    from flowket_gb300.machines import rbm_sym_tied_index
    n = int(np.prod(shape))
    rng = np.random.default_rng(n + alpha)
    vec = rng.normal(size=1 + alpha + n * alpha) + 1j * rng.normal(size=1 + alpha + n * alpha)
    idx = rbm_sym_tied_index(shape, alpha).numpy()
    assert idx.shape == (n + alpha * n + n * alpha * n,)
    full = ref_rbm.rbm_sym_full_params(ref_rbm.rbm_sym_bare_dict(vec, shape, alpha), shape)
    want = np.concatenate([full["a"], full["b"], full["W"].reshape(-1)])
    np.testing.assert_array_equal(vec[idx], want)
