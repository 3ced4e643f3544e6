"""Oracle: stochastic reconfiguration and the Keras optimisers (numpy).

* ``sr_complex`` restates optimizers/stochastic_reconfiguration/optimizer.py:55-114
  in parameter space: J_c = J - mean(J), F = J_c^H conj(y), S = J_c^H J_c / B
  + lambda I, solved by Cholesky (:63-64) or by CG (linear_equations.py:34-137,
  residual-norm stop relative to ||F||); the update is W <- W - lr x
  (complex_values_optimizer.py:48-58).
* ``sr_real`` is the real-parameter form used for real-weight networks with a
  complex output: S = Re<O_c^* O_c>, F = Re<O_c^* E_c>.
* ``keras_adam`` restates tf.keras Adam (TF 1.x, epsilon = K.epsilon() = 1e-7).
* ``accumulate_gradient_sgd`` restates optimizers/accumulate_gradient_optimizer.py:13-88
  for plain SGD with mean/sum accumulation and an EMA of the weights.
Test infrastructure only.
"""
import numpy as np


def conjugate_gradient(apply, rhs, tol=1e-3, max_iter=200):
    """linear_equations.py:34-137 without preconditioner, x0 = 0; stops when
    ||r|| <= tol * ||rhs|| or after max_iter steps."""
    x = np.zeros_like(rhs)
    r = rhs.copy()
    p = r.copy()
    gamma = np.vdot(r, r)
    stop = tol * np.linalg.norm(rhs)
    i = 0
    while (max_iter is None or i < max_iter) and np.linalg.norm(r) > stop:
        z = apply(p)
        alpha = gamma / np.vdot(p, z)
        x = x + alpha * p
        r = r - alpha * z
        g2 = np.vdot(r, r)
        p = r + (g2 / gamma) * p
        gamma = g2
        i += 1
    return x, i, np.linalg.norm(r)


def sr_complex(jac, y, diag_shift, iterative=False, tol=1e-6, max_iter=None):
    """jac (B, P) complex O_k; y (B,) loss coefficients conj(E-Ebar)/B.
    Returns the solution x (the update is W <- W - lr x)."""
    b = jac.shape[0]
    jc = jac - jac.mean(axis=0, keepdims=True)
    f = jc.conj().T @ np.conj(y)
    if iterative:
        def apply(v):
            return jc.conj().T @ (jc @ v) / b + diag_shift * v
        x, _, _ = conjugate_gradient(apply, f, tol=tol, max_iter=max_iter)
        return x
    s = jc.conj().T @ jc / b + diag_shift * np.eye(jac.shape[1])
    lchol = np.linalg.cholesky(s)
    return np.linalg.solve(lchol.conj().T, np.linalg.solve(lchol, f))


def sr_real(o, local_energy, diag_shift):
    """o (B, P) complex d log psi / d theta for real theta; local_energy (B,).
    Solves (Re<O_c^* O_c> + lambda I) x = Re<O_c^* (E - Ebar)>."""
    b = o.shape[0]
    oc = o - o.mean(axis=0, keepdims=True)
    ec = local_energy - local_energy.mean()
    s = np.real(oc.conj().T @ oc) / b + diag_shift * np.eye(o.shape[1])
    f = np.real(oc.conj().T @ ec) / b
    return np.linalg.solve(s, f)


def keras_adam(params, grads, state, lr=1e-3, beta_1=0.9, beta_2=0.999, epsilon=1e-7):
    """One tf.keras (TF 1.x) Adam step on dicts of arrays; state holds m, v, t."""
    t = state.get("t", 0) + 1
    lr_t = lr * np.sqrt(1.0 - beta_2 ** t) / (1.0 - beta_1 ** t)
    out = {}
    for k, p in params.items():
        g = grads[k]
        m = beta_1 * state.get("m_" + k, np.zeros_like(p)) + (1 - beta_1) * g
        v = beta_2 * state.get("v_" + k, np.zeros_like(p)) + (1 - beta_2) * g * g
        state["m_" + k], state["v_" + k] = m, v
        out[k] = p - lr_t * m / (np.sqrt(v) + epsilon)
    state["t"] = t
    return out


def accumulate_gradient_sgd(w0, grads, lr, update_every, mean=True, ema_decay=None):
    """SGD that applies the accumulated gradient every `update_every` calls
    (accumulate_gradient_optimizer.py:13-88). Returns the weight after each
    call and the final EMA of the applied weights (bias-corrected)."""
    w = float(w0)
    acc = 0.0
    k = 0
    history = []
    ema = 0.0
    n_updates = 0
    for g in grads:
        acc += g
        k += 1
        if k == update_every:
            step = acc / update_every if mean else acc
            w = w - lr * step
            acc = 0.0
            k = 0
            n_updates += 1
            if ema_decay is not None:
                ema = ema_decay * ema + (1 - ema_decay) * w
        history.append(w)
    ema_w = ema / (1 - ema_decay ** n_updates) if (ema_decay is not None and n_updates) else None
    return history, ema_w
