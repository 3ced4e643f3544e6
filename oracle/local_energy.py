"""Oracle: local energy and its statistics (numpy, complex128).

Restates observables/monte_carlo/operator.py:6-53 (both connection paths) and
observables/monte_carlo/observable.py:10-14. Test infrastructure only.
"""
import numpy as np


def local_values_unbalanced(wave_function, conn, mel, use):
    """operator.py:20-34: evaluate only the used connections, then a per-sample
    loop sum mel * exp(logpsi' - logpsi_0)."""
    b = use.shape[1]
    reshaped = np.moveaxis(conn, 1, 0).reshape((-1,) + conn.shape[2:])
    flat_conn = reshaped[use.astype(bool).T.flatten()]
    flat_log = wave_function(flat_conn)
    per = use.sum(axis=0).astype(np.int64)
    out = np.zeros(b, dtype=np.complex128)
    idx = 0
    for i in range(b):
        lv = flat_log[idx:idx + per[i]]
        idx += per[i]
        out[i] = (mel[use[:, i].astype(bool), i] * np.exp(lv - lv[0])).sum()
    return out


def local_values_balanced(wave_function, conn, mel):
    """operator.py:36-42: evaluate every slot, vectorised reduction."""
    flat = conn.reshape((-1,) + conn.shape[2:])
    lv = wave_function(flat).reshape(conn.shape[0:2])
    return (mel * np.exp(lv - lv[0, :])).sum(axis=0)


def local_values(wave_function, conn, mel, use):
    """operator.py:44-53 dispatch on mean(use) < 0.95."""
    if use.mean() < 0.95:
        return local_values_unbalanced(wave_function, conn, mel, use)
    return local_values_balanced(wave_function, conn, mel)


def estimate(local):
    """observable.py:10-14: (mean, var(Re), local values)."""
    return np.mean(local), np.var(np.real(local)), local


def loss_coefficients(local, batch_size):
    """variational_monte_carlo.py:38-40,50: conj(E_loc - mean)/B."""
    return np.conj(local - np.mean(local)) / batch_size
