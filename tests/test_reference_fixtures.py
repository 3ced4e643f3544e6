"""The oracle and the product's host-side estimators against golden vectors
written by the reference's own numpy code (tests/golden/make_reference_fixtures.py):
find_conn of operators/heisenberg.py and operators/ising.py (bit-exact),
Observable.local_values / estimate of observables/monte_carlo/ (1e-12) and
calc_r_hat_value of samplers/metropolis_hastings.py (1e-12). No GPU."""
import os

import numpy as np
import pytest

from oracle import local_energy as ref_le, operators as ref_ops, samplers as ref_samplers

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def _cases(data):
    return sorted({k.split("/")[0] for k in data.files})


FIND_CONN = _load("reference_find_conn.npz")
LOCAL = _load("reference_local_values.npz")
RHAT = _load("reference_r_hat.npz")

# name -> (operator, shape, kwargs) as the generator wrote them
FIND_CONN_ARGS = {
    "heis_4x4_pbc": ("heisenberg", dict(pbc=True)), "heis_4x4_obc": ("heisenberg", dict(pbc=False)),
    "heis_4x4_pbc_norot": ("heisenberg", dict(pbc=True, unitary_rotation=False)),
    "heis_10x10_pbc": ("heisenberg", dict(pbc=True)), "heis_16x16_pbc": ("heisenberg", dict(pbc=True)),
    "heis_chain64_pbc": ("heisenberg", dict(pbc=True)), "heis_20x1_pbc": ("heisenberg", dict(pbc=True)),
    "ising_4x4_pbc_h3": ("ising", dict(pbc=True, h=3.0)), "ising_10x10_pbc_h3": ("ising", dict(pbc=True, h=3.0)),
    "ising_12x12_obc_h2.5": ("ising", dict(pbc=False, h=2.5)),
    "ising_3x5_obc_j0.7": ("ising", dict(pbc=False, h=1.5, j=0.7)),
}


def _diff_sites(conn, spins):
    b = spins.shape[0]
    conn = conn.reshape(conn.shape[0], b, -1)
    flat = spins.reshape(b, -1)
    out = np.full(conn.shape[:2] + (2,), -1, dtype=np.int16)
    for c in range(conn.shape[0]):
        for i in range(b):
            d = np.nonzero(conn[c, i] != flat[i])[0]
            out[c, i, :d.size] = d
    return out


def test_fixture_covers_every_case():
    assert _cases(FIND_CONN) == sorted(FIND_CONN_ARGS)


@pytest.mark.parametrize("name", sorted(FIND_CONN_ARGS))
def test_oracle_find_conn_equals_reference_output(name):
    op, kw = FIND_CONN_ARGS[name]
    s = FIND_CONN[name + "/spins"]
    fn = ref_ops.heisenberg_find_conn if op == "heisenberg" else ref_ops.ising_find_conn
    conn, mel, use = fn(s, **kw)
    np.testing.assert_array_equal(use, FIND_CONN[name + "/use"])
    np.testing.assert_array_equal(mel, FIND_CONN[name + "/mel"])
    np.testing.assert_array_equal(_diff_sites(np.asarray(conn), s), FIND_CONN[name + "/diff"])


def rbm_wave_function(a, b, w):
    def wf(x):
        s = np.asarray(x, dtype=np.float64).reshape(x.shape[0], -1)
        return s @ a + np.log(np.cosh(s @ w + b[None, :])).sum(axis=1)
    return wf


@pytest.mark.parametrize("name,op,kw", [("rbm_heis_4x4_pbc", "heisenberg", dict(pbc=True)),
                                        ("rbm_ising_4x4_pbc_h3", "ising", dict(pbc=True, h=3.0)),
                                        ("rbm_heis_chain16_obc", "heisenberg", dict(pbc=False))])
def test_oracle_local_values_equal_reference_output(name, op, kw):
    s = LOCAL[name + "/spins"]
    fn = ref_ops.heisenberg_find_conn if op == "heisenberg" else ref_ops.ising_find_conn
    conn, mel, use = fn(s, **kw)
    wf = rbm_wave_function(LOCAL[name + "/a"], LOCAL[name + "/b"], LOCAL[name + "/W"])
    got = ref_le.local_values(wf, conn, mel, use)
    np.testing.assert_allclose(got, LOCAL[name + "/local"], rtol=1e-12, atol=1e-12)
    mean, var, _ = ref_le.estimate(got)
    assert abs(mean - LOCAL[name + "/mean"]) <= 1e-12 * abs(mean)
    assert abs(var - LOCAL[name + "/var"]) <= 1e-12 * abs(var)


@pytest.mark.parametrize("name", sorted({k.split("/")[0] for k in RHAT.files}))
def test_r_hat_and_correlations_equal_reference_output(name):
    from flowket_gb300.samplers import r_hat_and_correlations
    values = RHAT[name + "/values"]
    chains = int(RHAT[name + "/chains"])
    want = RHAT[name + "/result"]
    got = np.array(r_hat_and_correlations(values, chains), dtype=np.float64)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)
    got_oracle = np.array(ref_samplers.r_hat_and_correlations(values, chains), dtype=np.float64)
    np.testing.assert_allclose(got_oracle, want, rtol=1e-12, atol=1e-12)
