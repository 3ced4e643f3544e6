"""Writes golden fixtures produced by the reference itself (FlowKet's pure-numpy
modules, imported straight from a FlowKet checkout without its TensorFlow
package initialisers):

* reference_find_conn.npz -- operators/heisenberg.py:47-121 and
  operators/ising.py:17-46 find_conn on seeded configurations: the use flags,
  matrix elements and, per slot, the sites where the connected configuration
  differs from the sample;
* reference_local_values.npz -- observables/monte_carlo/operator.py:13-53
  (Observable.local_values, balanced and unbalanced paths) and
  observables/monte_carlo/observable.py:10-14 (estimate) for a complex RBM
  wave function written out below in numpy, and for the 4x4 autoregressive
  network evaluated by the oracle;
* reference_r_hat.npz -- samplers/metropolis_hastings.py:8-12,67-89
  (calc_r_hat_value, sum_correlations) on seeded chain series.

Run from the repository root with the FlowKet source tree as argument:
    python tests/golden/make_reference_fixtures.py /root/reference/src/flowket
The reference uses numpy.bool (removed from numpy 1.24); this script binds
that name to bool before loading it. Nothing at test time reads the reference.
"""
import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def load_reference(src):
    """Registers empty packages for the FlowKet tree (so relative imports
    resolve file by file) and loads the numpy-only modules."""
    if not hasattr(np, "bool"):
        np.bool = bool
    pkgs = ["fkref", "fkref.operators", "fkref.observables", "fkref.observables.monte_carlo", "fkref.deepar",
            "fkref.deepar.samplers", "fkref.samplers"]
    for name in pkgs:
        mod = types.ModuleType(name)
        rel = name.split(".")[1:]
        mod.__path__ = [os.path.join(src, *rel)]
        sys.modules[name] = mod

    def load(name, rel):
        spec = importlib.util.spec_from_file_location(name, os.path.join(src, rel))
        mod = importlib.util.module_from_spec(spec)
        mod.__package__ = name.rpartition(".")[0]
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
        return mod

    load("fkref.operators.operator", "operators/operator.py")
    heis = load("fkref.operators.heisenberg", "operators/heisenberg.py")
    ising = load("fkref.operators.ising", "operators/ising.py")
    load("fkref.observables.monte_carlo.observable", "observables/monte_carlo/observable.py")
    obs = load("fkref.observables.monte_carlo.operator", "observables/monte_carlo/operator.py")
    load("fkref.deepar.samplers.base_sampler", "deepar/samplers/base_sampler.py")
    mh = load("fkref.samplers.metropolis_hastings", "samplers/metropolis_hastings.py")
    return heis.Heisenberg, ising.Ising, obs.Observable, mh


def spins(shape, b, seed):
    return np.random.default_rng(seed).choice([-1, 1], size=(b,) + tuple(shape)).astype(np.int8)


FIND_CONN_CASES = [
    # name, operator, shape, kwargs, batch
    ("heis_4x4_pbc", "heisenberg", (4, 4), dict(pbc=True), 8),
    ("heis_4x4_obc", "heisenberg", (4, 4), dict(pbc=False), 8),
    ("heis_4x4_pbc_norot", "heisenberg", (4, 4), dict(pbc=True, unitary_rotation=False), 8),
    ("heis_10x10_pbc", "heisenberg", (10, 10), dict(pbc=True), 6),
    ("heis_16x16_pbc", "heisenberg", (16, 16), dict(pbc=True), 4),
    ("heis_chain64_pbc", "heisenberg", (64,), dict(pbc=True), 8),
    ("heis_20x1_pbc", "heisenberg", (20, 1), dict(pbc=True), 8),
    ("ising_4x4_pbc_h3", "ising", (4, 4), dict(pbc=True, h=3.0), 8),
    ("ising_10x10_pbc_h3", "ising", (10, 10), dict(pbc=True, h=3.0), 6),
    ("ising_12x12_obc_h2.5", "ising", (12, 12), dict(pbc=False, h=2.5), 4),
    ("ising_3x5_obc_j0.7", "ising", (3, 5), dict(pbc=False, h=1.5, j=0.7), 8),
]


def find_conn_fixture(Heisenberg, Ising):
    out = {}
    for k, (name, op, shape, kw, b) in enumerate(FIND_CONN_CASES):
        s = spins(shape, b, 100 + k)
        ham = (Heisenberg if op == "heisenberg" else Ising)(hilbert_state_shape=shape, **kw)
        conn, mel, use = ham.find_conn(s.astype(np.float64))
        conn = np.asarray(conn).reshape(conn.shape[0], b, -1)
        flat = s.reshape(b, -1)
        diff = np.full(conn.shape[:2] + (2,), -1, dtype=np.int16)
        for c in range(conn.shape[0]):
            for i in range(b):
                d = np.nonzero(conn[c, i] != flat[i])[0]
                assert d.size <= 2
                diff[c, i, :d.size] = d
        out[name + "/spins"] = s
        out[name + "/use"] = np.asarray(use, dtype=bool)
        out[name + "/mel"] = np.asarray(mel, dtype=np.float64)
        out[name + "/diff"] = diff
    return out


def rbm_wave_function(params):
    """log psi = s.a + sum_j log cosh(b_j + W_j.s) in complex128 (small
    parameters: the plain log cosh is exact enough)."""
    def wf(x):
        s = np.asarray(x, dtype=np.float64).reshape(x.shape[0], -1)
        theta = s @ params["W"] + params["b"][None, :]
        return (s @ params["a"] + np.log(np.cosh(theta)).sum(axis=1))[:, None]
    return wf


def rbm_params(n, alpha, stddev, seed):
    rng = np.random.default_rng(seed)
    m = alpha * n

    def c(*shape):
        # complex64-representable values, so the GPU sees the same parameters
        return (rng.normal(size=shape) * stddev).astype(np.float32) + 1j * (rng.normal(size=shape) * stddev).astype(
            np.float32)

    return {"a": c(n).astype(np.complex128), "b": c(m).astype(np.complex128), "W": c(n, m).astype(np.complex128)}


LOCAL_CASES = [
    ("rbm_heis_4x4_pbc", "heisenberg", (4, 4), dict(pbc=True), 64),
    ("rbm_ising_4x4_pbc_h3", "ising", (4, 4), dict(pbc=True, h=3.0), 64),
    ("rbm_heis_chain16_obc", "heisenberg", (16,), dict(pbc=False), 64),
]


def local_values_fixture(Heisenberg, Ising, Observable):
    out = {}
    for k, (name, op, shape, kw, b) in enumerate(LOCAL_CASES):
        n = int(np.prod(shape))
        p = rbm_params(n, 2, 0.1, 200 + k)
        s = spins(shape, b, 300 + k)
        ham = (Heisenberg if op == "heisenberg" else Ising)(hilbert_state_shape=shape, **kw)
        obs = Observable(ham)
        mean, var, local = obs.estimate(rbm_wave_function(p), s.astype(np.float64))
        out[name + "/spins"] = s
        for key in ("a", "b", "W"):
            out[name + "/" + key] = p[key]
        out[name + "/local"] = np.asarray(local, dtype=np.complex128)
        out[name + "/mean"] = np.complex128(mean)
        out[name + "/var"] = np.float64(var)
    # the autoregressive network (depth 3, 16 channels, weight norm) on the
    # 4x4 Heisenberg and Ising operators, log psi from the oracle in FP64
    sys.path.insert(0, ROOT)
    import torch
    from oracle import ar2d
    from flowket_gb300.machines import ar2d_param_layout, glorot_uniform_init
    layout, _ = ar2d_param_layout(3, 16, True)
    init = glorot_uniform_init(layout, 5, True)
    flat = np.concatenate([init[nm].reshape(-1).numpy() for nm, _, _ in layout]).astype(np.float32)
    params = {nm: torch.as_tensor(flat[off:off + int(np.prod(shp))].astype(np.float64)).reshape(shp)
              for nm, shp, off in layout}

    def ar_wf(x):
        return ar2d.log_psi_numpy(params, np.asarray(x).reshape(x.shape[0], 4, 4).astype(np.int8), 3, True)[:, None]

    for k, (name, op, kw) in enumerate([("ar_heis_4x4_pbc", "heisenberg", dict(pbc=True)),
                                        ("ar_ising_4x4_pbc_h3", "ising", dict(pbc=True, h=3.0))]):
        s = spins((4, 4), 48, 400 + k)
        ham = (Heisenberg if op == "heisenberg" else Ising)(hilbert_state_shape=(4, 4), **kw)
        mean, var, local = Observable(ham).estimate(ar_wf, s.astype(np.float64))
        out[name + "/spins"] = s
        out[name + "/params"] = flat
        out[name + "/local"] = np.asarray(local, dtype=np.complex128)
        out[name + "/mean"] = np.complex128(mean)
        out[name + "/var"] = np.float64(var)
    return out


R_HAT_CASES = [("ar1_rho0.5_c8_s64", 8, 64, 0.5), ("ar1_rho0.9_c16_s100", 16, 100, 0.9),
               ("white_c32_s20", 32, 20, 0.0), ("ar1_rho0.99_c4_s300", 4, 300, 0.99), ("single_c6_s1", 6, 1, 0.3)]


def r_hat_fixture(mh):
    out = {}
    for k, (name, chains, spc, rho) in enumerate(R_HAT_CASES):
        rng = np.random.default_rng(500 + k)
        x = np.zeros((chains, spc))
        x[:, 0] = rng.normal(size=chains) + rng.normal(size=chains) * 0.3
        for t in range(1, spc):
            x[:, t] = rho * x[:, t - 1] + np.sqrt(1 - rho * rho) * rng.normal(size=chains)
        x += 0.1 * np.arange(chains)[:, None]
        flat = x.reshape(-1)
        holder = types.SimpleNamespace(batch_size=chains * spc, num_of_chains=chains)
        res = mh.MetropolisHastingsSampler.calc_r_hat_value(holder, flat.copy())
        out[name + "/values"] = flat
        out[name + "/chains"] = np.int64(chains)
        out[name + "/result"] = np.array([float(v) for v in res], dtype=np.float64)
    return out


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else "/root/reference/src/flowket"
    Heisenberg, Ising, Observable, mh = load_reference(src)
    np.savez_compressed(os.path.join(HERE, "reference_find_conn.npz"), **find_conn_fixture(Heisenberg, Ising))
    np.savez_compressed(os.path.join(HERE, "reference_local_values.npz"),
                        **local_values_fixture(Heisenberg, Ising, Observable))
    np.savez_compressed(os.path.join(HERE, "reference_r_hat.npz"), **r_hat_fixture(mh))
    for f in ("reference_find_conn.npz", "reference_local_values.npz", "reference_r_hat.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


if __name__ == "__main__":
    main()
