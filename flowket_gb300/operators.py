"""Hamiltonians (flowket.operators drop-ins) enumerated on the GPU.

``find_conn(sample)`` returns the reference's triple
``(all_conn (C,B,*shape) int8, mel (C,B) float64, use (C,B) bool)`` with
slot 0 = the sample itself, bit-identical to operators/heisenberg.py:84-127,
operators/ising.py:17-46 and operators/j1j2.py:37-69. ``enumerate(sample)``
returns the compact form used by the local-energy path (flip pairs, elements,
use flags) without materialising configurations.
"""
import numpy as np
import torch

from . import _lib


class Operator:
    """operators/operator.py:6-30."""

    def __init__(self, hilbert_state_shape):
        self.hilbert_state_shape = tuple(int(x) for x in hilbert_state_shape)
        self.max_number_of_local_connections = None

    @property
    def n_sites(self):
        return int(np.prod(self.hilbert_state_shape))

    def random_states(self, num_of_states, generator=None):
        x = torch.randint(0, 2, (num_of_states,) + self.hilbert_state_shape, generator=generator)
        return (2 * x - 1).to(torch.int8)

    def use_state(self, state):
        return True

    def _grid(self):
        shape = self.hilbert_state_shape
        if len(shape) == 1:
            return shape[0], 1
        if len(shape) == 2:
            return shape
        raise ValueError("operators support 1D and 2D lattices (heisenberg.py:101-102, ising.py:27)")

    def _prep(self, sample):
        s = torch.as_tensor(sample)
        if not s.is_cuda or s.dtype != torch.int8:
            s = s.to(device="cuda" if not s.is_cuda else s.device, dtype=torch.int8)
        return s.reshape(s.shape[0], self.n_sites).contiguous()

    def enumerate(self, sample):
        """(flips (C,B,2) int16, mel (C,B) float64, use (C,B) uint8, spins (B,N) int8)."""
        s = self._prep(sample)
        b = s.shape[0]
        c = self.max_number_of_local_connections
        flips = torch.empty((c, b, 2), dtype=torch.int16, device=s.device)
        mel = torch.empty((c, b), dtype=torch.float64, device=s.device)
        use = torch.empty((c, b), dtype=torch.uint8, device=s.device)
        self._launch(s, b, flips, mel, use, None)
        return flips, mel, use, s

    def find_conn(self, sample):
        s = self._prep(sample)
        b = s.shape[0]
        c = self.max_number_of_local_connections
        flips = torch.empty((c, b, 2), dtype=torch.int16, device=s.device)
        mel = torch.empty((c, b), dtype=torch.float64, device=s.device)
        use = torch.empty((c, b), dtype=torch.uint8, device=s.device)
        conn = torch.empty((c, b, s.shape[1]), dtype=torch.int8, device=s.device)
        self._launch(s, b, flips, mel, use, conn)
        return conn.view((c, b) + self.hilbert_state_shape), mel, use.bool()


class OperatorOnGrid(Operator):
    """operators/operator.py:40-46."""

    def __init__(self, hilbert_state_shape=None, pbc=True):
        if hilbert_state_shape is None:
            hilbert_state_shape = (20, 1)
        super().__init__(hilbert_state_shape)
        self.pbc = pbc


class Heisenberg(OperatorOnGrid):
    """operators/heisenberg.py:6-44 (Marshall-rotated by default: off-diagonal -2)."""

    def __init__(self, total_sz=0.0, unitary_rotation=True, **kwargs):
        super().__init__(**kwargs)
        self.unitary_rotation = unitary_rotation
        self.total_sz = total_sz
        self.dim = len(self.hilbert_state_shape)
        self.max_number_of_local_connections = self.n_sites * self.dim + 1

    def random_states(self, num_of_states, generator=None):
        """Random states in the total_sz sector (heisenberg.py:20-31)."""
        if self.total_sz is None:
            return super().random_states(num_of_states, generator)
        n = self.n_sites
        half = n // 2
        base = torch.cat([torch.ones(half + int(self.total_sz)), -torch.ones(half - int(self.total_sz))])
        out = torch.empty((num_of_states, n), dtype=torch.int8)
        for i in range(num_of_states):
            out[i] = base[torch.randperm(n, generator=generator)].to(torch.int8)
        return out.view((num_of_states,) + self.hilbert_state_shape)

    def use_state(self, state):
        if self.total_sz is None:
            return True
        return float(torch.as_tensor(state).sum()) == self.total_sz

    def _launch(self, s, b, flips, mel, use, conn):
        h, w = self._grid()
        _lib.call("fk_find_conn_heisenberg", _lib.ptr(s), b, h, w, self.dim, 1 if self.pbc else 0,
                  1 if self.unitary_rotation else 0, _lib.ptr(flips), _lib.ptr(mel), _lib.ptr(use),
                  _lib.ptr(conn), _lib.stream_ptr())


class Ising(OperatorOnGrid):
    """operators/ising.py:8-46 (transverse field h, coupling j). Every slot
    is used (ising.py:46), so the local energy knows its row count on the
    host."""

    all_connections_used = True

    def __init__(self, h=1.0, j=1.0, **kwargs):
        super().__init__(**kwargs)
        self.h = float(h)
        self.j = float(j)
        self.max_number_of_local_connections = self.n_sites + 1

    def _launch(self, s, b, flips, mel, use, conn):
        h, w = self._grid()
        _lib.call("fk_find_conn_ising", _lib.ptr(s), b, h, w, self.h, self.j, 1 if self.pbc else 0,
                  _lib.ptr(flips), _lib.ptr(mel), _lib.ptr(use), _lib.ptr(conn), _lib.stream_ptr())


class J1J2(Operator):
    """operators/j1j2.py:7-69 (j1j2_two_dim_operator): J1 = 1 on nearest and J2
    on next-nearest neighbours, no Marshall rotation, 4N+1 padded slots."""

    def __init__(self, hilbert_state_shape, j2=0.5, pbc=False):
        super().__init__(hilbert_state_shape)
        if len(self.hilbert_state_shape) != 2:
            raise ValueError("J1J2 needs a 2D hilbert_state_shape (j1j2.py:58)")
        self.j2 = float(j2)
        self.pbc = pbc
        self.max_number_of_local_connections = self.n_sites * 2 * 2 + 1

    def _launch(self, s, b, flips, mel, use, conn):
        h, w = self.hilbert_state_shape
        _lib.call("fk_find_conn_j1j2", _lib.ptr(s), b, h, w, self.j2, 1 if self.pbc else 0, _lib.ptr(flips),
                  _lib.ptr(mel), _lib.ptr(use), _lib.ptr(conn), _lib.stream_ptr())
