"""Samplers (flowket.samplers drop-ins).

* ``FastAutoregressiveSampler`` / ``AutoregressiveSampler``: exact raster-order
  sampling of an autoregressive machine (deepar/samplers/fast_autoregressive.py:13-76,
  deepar/samplers/autoregressive.py:10-48 with the +-1 convention of
  samplers/__init__.py:8-14). Both run the persistent sampling kernel, which
  evaluates each (layer, site) once -- the fast sampler's work -- and draws
  every site with Philox4x32-10; the slow sampler's N full forward passes give
  the same distribution and are not re-implemented.
* ``MetropolisHastingsLocal`` / ``MetropolisHastingsExchange``: on-device
  Markov chains for RBM machines (samplers/metropolis_hastings.py:15-145).
* ``MetropolisHastingsIndependent``: the learned independent proposal (an
  autoregressive network sampled exactly) with the exact acceptance
  min(1, |psi(s')|^2 q(s) / (|psi(s)|^2 q(s'))).
__next__ returns an int8 CUDA tensor (B, *shape) of +-1.
"""
import copy

import torch

from . import _lib


class Sampler:
    """deepar/samplers/base_sampler.py:4-25."""

    def __init__(self, input_size, batch_size, mini_batch_size=None):
        self.input_size = tuple(input_size)
        self._set_batch_size(batch_size, mini_batch_size)

    def _set_batch_size(self, batch_size, mini_batch_size=None):
        if mini_batch_size is None or mini_batch_size > batch_size:
            mini_batch_size = batch_size
        self.batch_size = int(batch_size)
        self.mini_batch_size = int(mini_batch_size)

    def copy_with_new_batch_size(self, batch_size, mini_batch_size=None):
        new = copy.copy(self)
        new._set_batch_size(batch_size, mini_batch_size)
        return new

    def __iter__(self):
        return self


class FastAutoregressiveSampler(Sampler):
    """Persistent-kernel exact sampler. ``seed`` keys Philox; every draw uses a
    fresh counter offset (``offset`` increments per call)."""

    def __init__(self, machine, batch_size, mini_batch_size=None, seed=1234, offset=0):
        super().__init__(machine.hilbert_state_shape, batch_size, mini_batch_size)
        self.machine = machine
        self.seed = int(seed)
        self.offset = int(offset)
        self.last_log_psi = None
        self.last_workspace = None

    def sample(self, offset=None):
        """One draw: (spins (B, H, W) int8, log_psi (B, 2) float32, activation workspace)."""
        m = self.machine
        b = self.batch_size
        h, w = m.hilbert_state_shape
        spins = torch.empty((b, h * w), dtype=torch.int8, device=m.device)
        lp = torch.empty((b, 2), dtype=torch.float32, device=m.device)
        ws = m.workspace(b, _lib.FK_AR2D_SAVE)
        off = self.offset if offset is None else int(offset)
        _lib.call("fk_ar2d_sample", ctypes_ref(m.desc), _lib.ptr(m.packed()), b, self.seed, off, _lib.ptr(spins),
                  _lib.ptr(lp), _lib.ptr(ws), ws.numel(), _lib.stream_ptr())
        if offset is None:
            self.offset += 1
        self.last_log_psi = lp
        self.last_workspace = ws
        return spins.view(b, h, w), lp, ws

    def __next__(self):
        return self.sample()[0]


class AutoregressiveSampler(FastAutoregressiveSampler):
    """deepar/samplers/autoregressive.py:10-48: same exact distribution."""


def ctypes_ref(struct):
    import ctypes
    return ctypes.byref(struct)
