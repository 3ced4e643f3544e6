"""Oracle: connected-configuration enumeration (numpy, integer-exact).

Restates operators/heisenberg.py:6-121, operators/ising.py:8-46,
operators/j1j2.py:7-69 and operators/netket_operator.py:46-66.
Every function returns the reference's triple
``(all_conn (C,B,*shape), mel (C,B), use (C,B) bool)`` with index 0 = the
sample itself. Test infrastructure only.
"""
import numpy as np


def _as_2d(sample):
    """A 1D shape is treated as (L, 1) (heisenberg.py:58-59, :73-74)."""
    if sample.ndim == 2:
        return sample[:, :, None], True
    return sample, False


def heisenberg_find_conn(sample, pbc=True, unitary_rotation=True):
    """heisenberg.py:47-121. Off-diagonal slot 1 + (site*dim + dim_idx), site
    row-major, dim_idx 0 = the bond to (i+1, j), 1 = the bond to (i, j+1); a
    slot is used iff the two spins differ; mel = -2 with the Marshall rotation
    (heisenberg.py:11-14), +2 without. dim = number of axes of the original
    shape, so a 1D chain has L+1 slots."""
    sample = np.asarray(sample)
    orig_dim = sample.ndim - 1
    s, was_1d = _as_2d(sample)
    b, hh, ww = s.shape
    n = hh * ww
    dim = orig_dim
    off = -2.0 if unitary_rotation else 2.0
    n_conn = n * dim + 1
    conn = np.broadcast_to(s[None], (n_conn, b, hh, ww)).astype(np.float64).copy()
    mel = np.zeros((n_conn, b), dtype=np.float64)
    use = np.zeros((n_conn, b), dtype=bool)
    use[0] = True
    diag = np.zeros(b, dtype=np.float64)
    for i in range(hh):
        for j in range(ww):
            d = 0
            if hh > 1:
                slot = 1 + (i * ww + j) * dim + d
                if i + 1 < hh or pbc:
                    i2 = i + 1 if i + 1 < hh else 0
                    diag += s[:, i, j] * s[:, i2, j]
                    u = s[:, i, j] != s[:, i2, j]
                    use[slot] = u
                    conn[slot, :, i, j] = s[:, i2, j]
                    conn[slot, :, i2, j] = s[:, i, j]
                    mel[slot] = np.where(u, off, 0.0)
                d += 1
            if ww > 1:
                slot = 1 + (i * ww + j) * dim + d
                if j + 1 < ww or pbc:
                    j2 = j + 1 if j + 1 < ww else 0
                    diag += s[:, i, j] * s[:, i, j2]
                    u = s[:, i, j] != s[:, i, j2]
                    use[slot] = u
                    conn[slot, :, i, j] = s[:, i, j2]
                    conn[slot, :, i, j2] = s[:, i, j]
                    mel[slot] = np.where(u, off, 0.0)
    mel[0] = diag
    if was_1d:
        conn = conn[..., 0]
    return conn, mel, use


def ising_find_conn(sample, h=1.0, j=1.0, pbc=True):
    """ising.py:17-46. Slot 0 diagonal -J sum s_i (s_down + s_right) computed in
    float32 (ising.py:25), slots 1..N flip one site in row-major order, mel -h,
    all used."""
    sample = np.asarray(sample)
    b = sample.shape[0]
    shape = sample.shape[1:]
    n = int(np.prod(shape))
    flat = sample.reshape(b, n)
    mel_site = np.zeros(sample.shape, dtype=np.float32)
    if len(shape) == 1:
        (ll,) = shape
        for i in range(ll):
            nb = sample[:, i + 1] if i + 1 < ll else (sample[:, 0] if pbc else 0)
            mel_site[:, i] -= np.float32(j) * sample[:, i] * nb
    else:
        hh, ww = shape
        for i in range(hh):
            for k in range(ww):
                if hh > 1:
                    nb = sample[:, i + 1, k] if i + 1 < hh else (sample[:, 0, k] if pbc else 0)
                    mel_site[:, i, k] -= np.float32(j) * sample[:, i, k] * nb
                if ww > 1:
                    nb = sample[:, i, k + 1] if k + 1 < ww else (sample[:, i, 0] if pbc else 0)
                    mel_site[:, i, k] -= np.float32(j) * sample[:, i, k] * nb
    self_mel = mel_site.reshape(b, n).sum(axis=1, dtype=np.float32)
    conn = np.broadcast_to(flat[None], (n + 1, b, n)).astype(np.float64).copy()
    for k in range(n):
        conn[k + 1, :, k] *= -1
    mel = np.full((n + 1, b), -h, dtype=np.float64)
    mel[0] = self_mel
    return conn.reshape((n + 1, b) + shape), mel, np.ones((n + 1, b), dtype=bool)


def j1j2_edges(hh, ww, pbc=True):
    """Edge list with colours (1 = J1, 2 = J2), restating the construction of
    j1j2.py:13-35 (sites numbered w + ww*h)."""
    edges = []
    for h in range(hh):
        for w in range(ww - 1):
            edges.append((w + ww * h, w + 1 + ww * h, 1))
            if h < hh - 1:
                edges.append((w + ww * h, w + ww * (h + 1), 1))
                edges.append((w + ww * h, w + 1 + ww * (h + 1), 2))
            elif pbc:
                edges.append((w + ww * h, w, 1))
                edges.append((w + ww * h, w + 1, 2))
            if h > 0:
                edges.append((w + ww * h, w + 1 + ww * (h - 1), 2))
            elif pbc:
                edges.append((w + ww * h, w + 1 + ww * (hh - 1), 2))
        w = ww - 1
        if pbc:
            edges.append((ww - 1 + ww * h, ww * h, 1))
            edges.append((w + ww * h, ww * ((h + 1) % hh), 2))
            edges.append((w + ww * h, ww * ((hh + h - 1) % hh), 2))
        if h < hh - 1:
            edges.append((w + ww * h, w + ww * (h + 1), 1))
        elif pbc:
            edges.append((w + ww * h, w, 1))
    return edges


def j1j2_find_conn(sample, j2=0.5, pbc=True):
    """J1-J2 bond operator J_c (sz sz + sx sx + sy sy) on the j1j2.py:13-35
    edges (j1j2.py:37-48). Diagonal = sum_edges J_c s_i s_j; each antiparallel
    edge gives one exchange connection with element 2 J_c. Connections are
    packed in edge order behind the diagonal and padded to 4N+1 slots with
    zero configurations, mel 0 and use = (mel != 0) (netket_operator.py:46-66).
    NetKet's own ordering of the connections is not pinned by any reference
    test; only the multiset of (configuration, element) pairs is."""
    sample = np.asarray(sample)
    b, hh, ww = sample.shape
    n = hh * ww
    jc = {1: 1.0, 2: float(j2)}
    edges = j1j2_edges(hh, ww, pbc)
    n_conn = n * 2 * 2 + 1
    flat = sample.reshape(b, n).astype(np.float64)
    conn = np.zeros((n_conn, b, n), dtype=np.float64)
    mel = np.zeros((n_conn, b), dtype=np.complex128)
    conn[0] = flat
    for bi in range(b):
        s = flat[bi]
        diag = 0.0
        k = 1
        for (a, c, col) in edges:
            diag += jc[col] * s[a] * s[c]
        for (a, c, col) in edges:
            if s[a] != s[c]:
                t = s.copy()
                t[a], t[c] = s[c], s[a]
                conn[k, bi] = t
                mel[k, bi] = 2.0 * jc[col]
                k += 1
        mel[0, bi] = diag
    use = mel != 0.0
    use[0] = True
    return conn.reshape((n_conn, b, hh, ww)), mel, use
