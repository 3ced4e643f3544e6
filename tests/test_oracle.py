"""The CPU oracle against the reference's own known answers (no GPU)."""
import numpy as np
import pytest
import torch

from oracle import ar2d, exact, local_energy, operators, philox, rbm, samplers, sr

# tests/test_tensorflow_complex_numbers_ops.py:6
COMPLEX_NUMBERS = [2, 3j, 1 + 7j, 10 - 3j, -6]


@pytest.mark.parametrize("z", COMPLEX_NUMBERS)
def test_lncosh_matches_log_cosh(z):
    # test_tensorflow_complex_numbers_ops.py:9-19 (1e-8 in complex128)
    assert abs(rbm.lncosh(np.array([z]))[0] - np.log(np.cosh(z))) < 1e-8


@pytest.mark.parametrize("z", COMPLEX_NUMBERS)
def test_lncosh_derivative_is_tanh(z):
    # test_tensorflow_complex_numbers_ops.py:22-33: the gradient of Re lncosh
    # is tanh z (u_x - i u_y for f = u + iv); Re is free of the log branch cut.
    h = 1e-6
    u = lambda w: np.real(rbm.lncosh(np.array([w]))[0])
    d = (u(z + h) - u(z - h)) / (2 * h) - 1j * (u(z + 1j * h) - u(z - 1j * h)) / (2 * h)
    assert abs(d - np.tanh(z)) < 1e-7


def test_unbalanced_equals_balanced_hand_fixture():
    """tests/test_variational.py:18-46 with the reference's hand-built arrays."""
    rng = np.random.default_rng(0)
    sample = np.array([[1, 1, 1, -1, -1, -1, -1],
                       [1, 1, 1, -1, 1, -1, -1],
                       [1, -1, 1, 1, -1, -1, -1]])
    conn = rng.choice([-1, 1], size=(5, 3, 7))
    conn[0] = sample
    mel = np.array([[2.0, 7j + 8, 0.0, 0.0, 3],
                    [0.0, 0.0, 0.0, 0.0, -1.0],
                    [5.0, 3j, 0.0, -2, 9]]).T
    use = np.array([[True, True, False, False, True],
                    [True, False, False, False, True],
                    [True, True, False, True, True]]).T
    w = rng.normal(size=7) + 1j * rng.normal(size=7)

    def wave_function(x):
        return x.reshape(x.shape[0], -1) @ w

    u = np.mean(local_energy.local_values_unbalanced(wave_function, conn, mel, use))
    b = np.mean(local_energy.local_values_balanced(wave_function, conn, mel))
    assert np.allclose(u, b)


# Exact ground-state energies hard-coded in the reference examples.
def test_lanczos_ising_4x4_obc():
    # examples/basic_autoregressive_2d.py:27,38
    e = exact.lanczos_ground_energy(lambda s: operators.ising_find_conn(s, h=3.0, pbc=False), (4, 4))
    assert e == pytest.approx(-50.18662388277671, abs=1e-8)


def test_lanczos_ising_chain_16_obc():
    # examples/basic_autoregressive_monte_carlo_gradient.py:29,41
    e = exact.lanczos_ground_energy(lambda s: operators.ising_find_conn(s, h=3.0, pbc=False), (16,))
    assert e == pytest.approx(-49.257706531889006, abs=1e-8)


def test_lanczos_heisenberg_chain_20_pbc():
    # examples/rbm_heisenberg_1d_sr.py:35,69 (the Sz=0 sector holds the ground state)
    basis = exact.sz_sector((20,), 0)
    e = exact.lanczos_ground_energy(lambda s: operators.heisenberg_find_conn(s, pbc=True), (20,), basis=basis)
    assert e == pytest.approx(-35.6175461195, abs=1e-8)


def test_lanczos_heisenberg_4x4_pbc():
    # the exact energy the 4x4 training case of bench.py is compared with
    import bench
    e = exact.lanczos_ground_energy(lambda s: operators.heisenberg_find_conn(s, pbc=True), (4, 4))
    assert e == pytest.approx(bench.HEISENBERG_4X4_PBC_E0, abs=1e-8)
    assert e == pytest.approx(-44.91393283371548, abs=1e-8)


def test_lanczos_j1j2_4x4_obc():
    # examples/j1j2_2d_monte_carlo_4.py:43,48
    basis = exact.sz_sector((4, 4), 0)
    e = exact.lanczos_ground_energy(lambda s: operators.j1j2_find_conn(s, j2=0.5, pbc=False), (4, 4), basis=basis)
    assert e == pytest.approx(-30.022227800323677, abs=1e-8)


def test_heisenberg_marshall_rotation_is_unitary():
    """The Marshall sign rotation (heisenberg.py:11-14) changes no eigenvalue on
    a bipartite lattice."""
    f_rot = lambda s: operators.heisenberg_find_conn(s, pbc=True, unitary_rotation=True)
    f_raw = lambda s: operators.heisenberg_find_conn(s, pbc=True, unitary_rotation=False)
    basis = exact.sz_sector((4, 4), 0)
    assert exact.lanczos_ground_energy(f_rot, (4, 4), basis=basis) == pytest.approx(
        exact.lanczos_ground_energy(f_raw, (4, 4), basis=basis), abs=1e-9)


def test_heisenberg_slot_layout():
    s = np.array([[[1, -1], [1, 1]]])
    conn, mel, use = operators.heisenberg_find_conn(s, pbc=False)
    assert conn.shape == (2 * 4 + 1, 1, 2, 2)
    # site (0,0): vertical bond to (1,0) equal spins -> unused; horizontal to (0,1) antiparallel -> used
    assert not use[1, 0] and use[2, 0] and mel[2, 0] == -2.0
    assert np.array_equal(conn[2, 0], np.array([[-1, 1], [1, 1]]))
    # diagonal: (0,0)-(1,0): +1, (0,0)-(0,1): -1, (0,1)-(1,1): -1, (1,0)-(1,1): +1
    assert mel[0, 0] == 0.0


@pytest.mark.parametrize("depth,shape", [(2, (4, 3)), (4, (4, 4))])
def test_autoregressive_distribution_is_normalised(depth, shape):
    """tests/test_autoregressive.py:18-30: sum_s |psi(s)|^2 = 1 (1e-5)."""
    params = ar2d.init_params(shape, depth, 16, weights_normalization=False, seed=3)
    states = exact.all_states(shape)
    lp = ar2d.log_psi_numpy(params, states, depth, False)
    total = np.exp(np.logaddexp.reduce(2 * np.real(lp)))
    assert total == pytest.approx(1.0, abs=1e-5)


def test_autoregressive_weight_normalisation_is_scale_free():
    params = ar2d.init_params((3, 3), 3, 8, weights_normalization=True, seed=1)
    states = exact.all_states((3, 3))[:64]
    a = ar2d.log_psi_numpy(params, states, 3, True)
    scaled = dict(params)
    scaled["cc1.c.kernel"] = params["cc1.c.kernel"] * 3.0
    b = ar2d.log_psi_numpy(scaled, states, 3, True)
    assert np.allclose(a, b, atol=1e-12)


def test_autoregressive_sampler_matches_exact_distribution():
    """tests/test_samplers.py:49-82 closeness statistic z <= sqrt(n)."""
    shape, depth = (3, 3), 2
    params = ar2d.init_params(shape, depth, 8, weights_normalization=False, seed=5)

    def cond_lp(batch):
        re, _ = ar2d.conditional_log_wave_function(ar2d.params_to(params, torch.float64),
                                                   torch.as_tensor(batch), depth, False)
        return 2.0 * re.detach().numpy()

    n = 2 ** 13
    got = samplers.autoregressive_sample(cond_lp, shape, n, seed=7, offset=0)
    probs, _ = exact.exact_distribution(ar2d.log_psi_numpy(params, exact.all_states(shape), depth, False))
    ref = exact.exact_sample(probs, shape, n, np.random.default_rng(1))
    x = np.bincount(exact.states_to_index(got.astype(np.int8)), minlength=512)
    y = np.bincount(exact.states_to_index(ref), minlength=512)
    z = ((np.square(x - y) - x - y) / (x + y + 1e-20)).sum()
    assert z <= np.sqrt(n)


def test_metropolis_local_matches_exact_distribution():
    shape = (8,)
    rng = np.random.default_rng(2)
    params = {"W": 0.3 * (rng.normal(size=(8, 16)) + 1j * rng.normal(size=(8, 16))),
              "b": 0.1 * (rng.normal(size=16) + 1j * rng.normal(size=16)),
              "a": 0.1 * (rng.normal(size=8) + 1j * rng.normal(size=8))}
    fn = lambda s: rbm.rbm_log_psi(params, s)
    init = rng.choice([-1, 1], size=(64, 8)).astype(np.float64)
    batch, ratio, _ = samplers.metropolis_hastings(fn, init, "local", 128, 8, 10, seed=11)
    n = batch.shape[0]
    probs, _ = exact.exact_distribution(fn(exact.all_states(shape)))
    ref = exact.exact_sample(probs, shape, n, np.random.default_rng(3))
    x = np.bincount(exact.states_to_index(batch.astype(np.int8)), minlength=256)
    y = np.bincount(exact.states_to_index(ref), minlength=256)
    z = ((np.square(x - y) - x - y) / (x + y + 1e-20)).sum()
    assert 0 < ratio <= 1
    assert z <= 2 * np.sqrt(n)  # chains are correlated; the reference thins by 2N sweeps


def test_sr_direct_and_cg_match_pinv():
    """tests/test_stochastic_reconfiguration.py:32-72 on the `Linear` machine
    (O = s): direct and CG solves agree with the pseudo-inverse to 1e-5."""
    rng = np.random.default_rng(4)
    s = rng.choice([-1.0, 1.0], size=(128, 16)).astype(np.complex128)
    y = rng.normal(size=128) + 1j * rng.normal(size=128)
    jc = s - s.mean(axis=0, keepdims=True)
    smat = jc.conj().T @ jc / 128 + 0.01 * np.eye(16)
    f = jc.conj().T @ np.conj(y)
    want = np.linalg.pinv(smat) @ f
    for it in (False, True):
        got = sr.sr_complex(s, y, 0.01, iterative=it, tol=1e-6)
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-5


def test_accumulate_gradient_known_answers():
    """tests/test_gradients_aggregation.py:36-111 (w0 = 1, loss = w x, SGD lr 1)."""
    hist, _ = sr.accumulate_gradient_sgd(1.0, [2.0, 3.0], 1.0, 2, mean=True)
    assert hist == [1.0, -1.5]
    hist, _ = sr.accumulate_gradient_sgd(1.0, [2.0, 3.0], 1.0, 1, mean=True)
    assert hist[-1] == -4.0
    hist, ema = sr.accumulate_gradient_sgd(1.0, [2.0, 3.0], 1.0, 1, mean=True, ema_decay=0.9)
    assert hist == [-1.0, -4.0] and ema == pytest.approx(-2.5789473684210527)
    hist, ema = sr.accumulate_gradient_sgd(1.0, [2.0, 3.0], 1.0, 2, mean=True, ema_decay=0.9)
    assert hist[-1] == -1.5 and ema == pytest.approx(-1.5)


def test_r_hat_of_identical_chains():
    v = np.tile(np.sin(np.arange(50.0)), 4)
    r_hat, var, cs, ess = samplers.r_hat_and_correlations(v, 4)
    assert r_hat < 1.0 and var > 0 and ess > 0


def test_philox_is_deterministic_and_uniform():
    a = philox.ar_site_uniforms(1234, 0, 256, 64)
    b = philox.ar_site_uniforms(1234, 0, 256, 64)
    c = philox.ar_site_uniforms(1234, 1, 256, 64)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert 0 < a.min() and a.max() < 1 and abs(a.mean() - 0.5) < 0.01


def test_rbm_log_derivatives_match_finite_differences():
    rng = np.random.default_rng(6)
    p = {"W": 0.2 * (rng.normal(size=(6, 12)) + 1j * rng.normal(size=(6, 12))),
         "b": 0.1 * (rng.normal(size=12) + 1j * rng.normal(size=12)),
         "a": 0.1 * (rng.normal(size=6) + 1j * rng.normal(size=6))}
    s = rng.choice([-1.0, 1.0], size=(5, 6))
    o = rbm.rbm_log_derivatives(p, s)
    h = 1e-6
    q = {k: v.copy() for k, v in p.items()}
    q["W"][2, 3] += h
    fd = (rbm.rbm_log_psi(q, s) - rbm.rbm_log_psi(p, s)) / h
    assert np.allclose(fd, o[:, 6 + 12 + 2 * 12 + 3], atol=1e-5)


def test_oracle_gradient_matches_finite_differences():
    """The oracle's autograd (the reference for the adjoint kernel) against
    central differences in float64."""
    shape, depth, f = (3, 3), 3, 8
    params = ar2d.params_to(ar2d.init_params(shape, depth, f, True, seed=4), torch.float64)
    rng = np.random.default_rng(7)
    for k in params:  # biases off zero so that no relu sits on its kink
        if k.endswith(".bias"):
            params[k] = torch.as_tensor(rng.normal(scale=0.1, size=params[k].shape))
    s = rng.choice([-1, 1], size=(5,) + shape).astype(np.int8)
    wre, wim = rng.normal(size=5), rng.normal(size=5)
    g = ar2d.weighted_gradient(params, s, depth, True, wre, wim)

    def loss(p):
        lp = ar2d.log_psi_numpy(p, s, depth, True)
        return float(np.sum(wre * lp.real + wim * lp.imag))

    for name, idx in [("cc1.c.kernel", (1, 2, 3, 4)), ("cc0.v.kernel", (2, 1, 0, 5)), ("cc2.y.g", (1,)),
                      ("out.bias", (2,)), ("cc3.x.bias", (3,))]:
        h = 1e-6
        p1 = {k: v.clone() for k, v in params.items()}
        p2 = {k: v.clone() for k, v in params.items()}
        p1[name][idx] += h
        p2[name][idx] -= h
        fd = (loss(p1) - loss(p2)) / (2 * h)
        assert fd == pytest.approx(float(g[name][idx]), rel=1e-5, abs=1e-8), name


def test_fast_sampler_restatement_equals_slow_sampler():
    """deepar/samplers/fast_autoregressive.py and deepar/samplers/autoregressive.py
    draw the same samples from the same uniforms."""
    from oracle.fast_sampler import FastSamplerCPU
    shape, depth = (3, 4), 4
    params = ar2d.init_params(shape, depth, 8, True, seed=2)
    fast = FastSamplerCPU(params, shape, depth, True, dtype=torch.float64).sample(64, seed=3, offset=1)

    def cond_lp(batch):
        re, _ = ar2d.conditional_log_wave_function(ar2d.params_to(params, torch.float64), torch.as_tensor(batch),
                                                   depth, True)
        return 2.0 * re.detach().numpy()

    slow = samplers.autoregressive_sample(cond_lp, shape, 64, seed=3, offset=1)
    assert np.array_equal(fast, slow.astype(np.int8))


def test_equal_up_down_mask_restricts_the_distribution_to_sz0():
    """EqualUpDownSpins (layers/spins_invariants.py:13-22): the masked AR
    network is normalised over the Sz = 0 sector and zero outside it; the
    mask marks outcome k once N/2 earlier sites hold it."""
    import torch
    x = torch.tensor([[[1, 1], [-1, 1]]], dtype=torch.int8)
    m = ar2d.equal_up_down_mask(x)[0].reshape(4, 2)
    # earlier +1 counts 0, 1, 2, 2 -> outcome 0 masked from the third site on
    assert m[:, 0].tolist() == [False, False, True, True]
    assert m[:, 1].tolist() == [False, False, False, False]
    shape = (3, 4)
    params = ar2d.init_params(shape, 3, 16, True, seed=5, dtype=torch.float64)
    g = torch.Generator().manual_seed(1)
    params = {k: v + 0.05 * torch.randn(v.shape, generator=g, dtype=torch.float64) for k, v in params.items()}
    states = exact.all_states(shape)
    lp = ar2d.log_psi_numpy(params, states, 3, True, equal_up_down=True)
    p = np.exp(2 * lp.real)
    sz0 = states.reshape(states.shape[0], -1).sum(axis=1) == 0
    assert np.all(p[~sz0] == 0.0)
    assert p[sz0].sum() == pytest.approx(1.0, abs=1e-12)
    lp0 = ar2d.log_psi_numpy(params, states, 3, True)
    assert np.exp(2 * lp0.real).sum() == pytest.approx(1.0, abs=1e-12)


def test_oracle_reproduces_golden_connections():
    """tests/golden/connections_4x4.json (written by tests/golden/make_golden.py)."""
    import json
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "connections_4x4.json")
    gold = json.load(open(path))
    s = np.array(gold["configs"], dtype=np.float64)
    fcs = {"heisenberg": lambda x: operators.heisenberg_find_conn(x, pbc=True),
           "ising": lambda x: operators.ising_find_conn(x, h=3.0, pbc=True),
           "j1j2": lambda x: operators.j1j2_find_conn(x, j2=0.5, pbc=True)}
    for name, fc in fcs.items():
        conn, mel, use = fc(s)
        g = gold[name]
        assert np.array_equal(np.asarray(conn).astype(np.int8), np.array(g["conn"], dtype=np.int8)), name
        assert np.array_equal(np.asarray(mel, dtype=np.complex128).real, np.array(g["mel"])), name
        assert np.array_equal(np.asarray(use, dtype=bool), np.array(g["use"], dtype=bool)), name
