"""Oracle: complex RBM wave functions (numpy complex128).

Restates machines/rbm.py:12-65 with layers/complex/dense.py:11-85 and
layers/complex/tensorflow_ops.py:69-85 (the overflow-safe lncosh). Parameters
are held as plain complex arrays: the reference stores (Re, -Im) pairs
(layers/complex/base_layer.py:18-35) but the wave function only sees the
complex value. Test infrastructure only.
"""
import itertools

import numpy as np


def lncosh(z):
    """tensorflow_ops.py:79-85: |Re z| - ln 2 + log(e^{z-|Re z|} + e^{-z-|Re z|})
    with log = log|.| + i atan2 (tensorflow_ops.py:69-76)."""
    z = np.asarray(z, dtype=np.complex128)
    a = np.abs(np.real(z))
    w = np.exp(z - a) + np.exp(-z - a)
    return a - np.log(2.0) + np.log(np.abs(w)) + 1j * np.arctan2(np.imag(w), np.real(w))


def rbm_log_psi(params, spins):
    """rbm.py:35-48: s.a + sum_j lncosh(b_j + W_j . s). spins (B, *shape)."""
    s = np.asarray(spins, dtype=np.float64).reshape(spins.shape[0], -1)
    theta = s @ params["W"] + params["b"][None, :]
    return s @ params["a"] + lncosh(theta).sum(axis=1)


def rbm_sym_full_params(bare, shape):
    """rbm.py:51-65 / dense.py:53-85: expand the translation-invariant kernel
    (shape + (alpha,)) into the dense (N, alpha*N) kernel, column f*T + t for
    feature f and translation t (itertools order over the lattice), bias
    repeated per translation, visible bias a on every site."""
    kern = bare["W"]
    alpha = kern.shape[-1]
    n = int(np.prod(shape))
    axes = tuple(range(len(shape)))
    trans = [np.roll(kern, t, axes) for t in itertools.product(*[range(d) for d in shape])]
    w = np.stack(trans, axis=-1).reshape(n, alpha * len(trans))
    b = np.repeat(bare["b"], n)
    a = np.full(n, bare["a"], dtype=np.complex128)
    return {"W": w, "b": b, "a": a}


def rbm_log_derivatives(params, spins):
    """O_k = d log psi / d p_k for p = (a, b, W), complex-holomorphic."""
    s = np.asarray(spins, dtype=np.float64).reshape(spins.shape[0], -1)
    theta = s @ params["W"] + params["b"][None, :]
    t = np.tanh(theta)
    o_w = (s[:, :, None] * t[:, None, :]).reshape(s.shape[0], -1)
    return np.concatenate([s.astype(np.complex128), t, o_w], axis=1)


def rbm_sym_bare_vector(bare):
    """The bare RBMSym parameters as one complex vector [a (1) | b (alpha) | W (shape + (alpha,))]."""
    return np.concatenate([np.ravel(bare["a"])[:1], np.ravel(bare["b"]), np.ravel(bare["W"])]).astype(np.complex128)


def rbm_sym_bare_dict(vec, shape, alpha):
    vec = np.asarray(vec, dtype=np.complex128)
    return {"a": vec[0], "b": vec[1:1 + alpha], "W": vec[1 + alpha:].reshape(tuple(shape) + (alpha,))}


def rbm_sym_log_derivatives(bare, shape, spins):
    """O_k = d log psi / d bare_k of RBMSym (rbm.py:51-65). The dense
    parameters are linear in the bare ones (copies), so by the chain rule
    d log psi / d bare_k = sum_j O_dense_j * d dense_j / d bare_k, with
    d dense / d bare_k the expansion of the k-th unit vector."""
    alpha = np.asarray(bare["b"]).shape[0]
    vec = rbm_sym_bare_vector(bare)
    full = rbm_sym_full_params(bare, shape)
    o_dense = rbm_log_derivatives(full, spins)
    cols = []
    for k in range(vec.shape[0]):
        e = np.zeros_like(vec)
        e[k] = 1.0
        u = rbm_sym_full_params(rbm_sym_bare_dict(e, shape, alpha), shape)
        cols.append(np.concatenate([u["a"], u["b"], u["W"].reshape(-1)]))
    jac = np.stack(cols, axis=1)
    return o_dense @ jac
