"""Oracle: exact enumeration and FP64 Lanczos ground states.

Restates exact/utils.py:39-78 (bit <-> index maps, log-sum-exp norm),
optimization/exact_variational.py:98-152 (|psi|^2 over all 2^N states, exact
energy and variance) and samplers/exact_sampler.py:7-20. The Lanczos ground
state (scipy.sparse.linalg.eigsh on the sparse H assembled from the
find_conn restatement) is new; it is pinned by the exact energies hard-coded
in the reference examples. Test infrastructure only.
"""
import numpy as np
import scipy.sparse
import scipy.sparse.linalg


def all_states(shape):
    """utils.py:49-58 with zero_one_base=False: bit k of the index is flat site
    k, bit 1 -> +1, bit 0 -> -1."""
    n = int(np.prod(shape))
    idx = np.arange(2 ** n, dtype=np.int64)
    bits = (idx[:, None] >> np.arange(n)[None, :]) & 1
    return (2 * bits - 1).reshape((2 ** n,) + tuple(shape)).astype(np.int8)


def states_to_index(states):
    """utils.py:39-46: +1 digits are the set bits."""
    b = states.shape[0]
    flat = states.reshape(b, -1)
    return ((flat == 1).astype(np.int64) << np.arange(flat.shape[1])[None, :]).sum(axis=1)


def exact_distribution(log_psi_all):
    """exact_variational.py:132-139: probs = |psi|^2 / Z with a max-shifted log-sum-exp."""
    re2 = 2.0 * np.real(log_psi_all)
    m = re2.max()
    log_z = np.log(np.sum(np.exp(re2 - m))) + m
    return np.exp(re2 - log_z), log_z


def sparse_hamiltonian(find_conn, shape, batch=4096, basis=None):
    """Sparse H over a basis (all 2^N states by default, or a sub-basis closed
    under H, e.g. the Sz=0 sector)."""
    if basis is None:
        basis = all_states(shape)
    index = states_to_index(basis)
    pos = {int(k): i for i, k in enumerate(index)} if len(index) < 2 ** int(np.prod(shape)) else None
    rows, cols, vals = [], [], []
    for s in range(0, basis.shape[0], batch):
        chunk = basis[s:s + batch]
        conn, mel, use = find_conn(chunk)
        c = conn.shape[0]
        b = chunk.shape[0]
        cidx = states_to_index(conn.reshape((c * b,) + conn.shape[2:])).reshape(c, b)
        for k in range(c):
            m = use[k] & (mel[k] != 0)
            if not np.any(m):
                continue
            r = np.arange(s, s + b)[m]
            cc = cidx[k][m]
            if pos is not None:
                cc = np.array([pos[int(x)] for x in cc], dtype=np.int64)
            rows.append(r)
            cols.append(cc)
            vals.append(mel[k][m])
    rows = np.concatenate(rows)
    cols = np.concatenate(cols)
    vals = np.concatenate(vals).astype(np.complex128)
    n = basis.shape[0]
    # <s|H|s'> with s' connected from s: row s, column s'. Real symmetric for these models.
    h = scipy.sparse.csr_matrix((vals, (rows, cols)), shape=(n, n))
    if np.all(np.imag(h.data) == 0):
        h = h.real
    return h


def sz_sector(shape, total_sz=0):
    n = int(np.prod(shape))
    allst = all_states(shape)
    keep = allst.reshape(allst.shape[0], -1).sum(axis=1) == total_sz
    return allst[keep]


def lanczos_ground_energy(find_conn, shape, basis=None, tol=1e-12):
    h = sparse_hamiltonian(find_conn, shape, basis=basis)
    val = scipy.sparse.linalg.eigsh(h, k=1, which="SA", tol=tol, return_eigenvectors=False)
    return float(val[0])


def exact_energy(log_psi_fn, find_conn, shape, batch=4096):
    """exact_variational.py:75-95 in closed form: E = sum_s p(s) E_loc(s),
    var = sum_s p(s) (Re E_loc(s) - E)^2. Returns (E, var, probs, local)."""
    states = all_states(shape)
    lp = np.concatenate([log_psi_fn(states[i:i + batch]) for i in range(0, states.shape[0], batch)])
    probs, _ = exact_distribution(lp)
    local = np.zeros(states.shape[0], dtype=np.complex128)
    for s in range(0, states.shape[0], batch):
        chunk = states[s:s + batch]
        conn, mel, use = find_conn(chunk)
        c, b = mel.shape
        cidx = states_to_index(conn.reshape((c * b,) + conn.shape[2:]).astype(np.int8)).reshape(c, b)
        lv = lp[cidx]
        contrib = np.where(use, mel * np.exp(lv - lv[0:1]), 0.0)
        local[s:s + b] = contrib.sum(axis=0)
    e = np.sum(probs * local)
    var = np.sum(probs * (np.real(local) - np.real(e)) ** 2)
    return e, var, probs, local


def exact_sample(probs, shape, n, rng):
    """exact_sampler.py:13-19."""
    idx = rng.choice(probs.shape[0], size=n, p=probs / probs.sum())
    return all_states(shape)[idx]
