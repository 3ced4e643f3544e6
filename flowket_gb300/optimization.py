"""VMC driver (flowket.optimization drop-in).

``VariationalMonteCarlo`` restates optimization/variational_monte_carlo.py:12-50
(sample -> local energy -> loss coefficients y = conj(E_loc - Ebar)/B) and adds
``step(optimizer)``: one full step on the GPU (exact sampling, local energy,
adjoint gradient of loss_for_energy_minimization (optimization/loss.py:4-5),
optimiser update) with CUDA-event timings per stage, the split of
callbacks/monte_carlo/runtime_stats.py:11-16.
"""
import math

import torch

from . import _lib
from .observables import Observable, BaseObservable, energy_stats


def loss_for_energy_minimization(y_true, y_pred):
    """optimization/loss.py:4-5: 2 Re(logpsi * y)."""
    return 2.0 * torch.real(y_pred * y_true)


class MiniBatchGenerator:
    """optimization/mini_batch_generator.py:5-45."""

    def __init__(self, batch_size, mini_batch_size):
        self.set_batch_size(batch_size, mini_batch_size)

    def set_batch_size(self, batch_size, mini_batch_size=None):
        if mini_batch_size is None or mini_batch_size > batch_size:
            mini_batch_size = batch_size
        self.batch_size = batch_size
        self.mini_batch_size = mini_batch_size
        self._idx = batch_size
        self.update_params_frequency = math.ceil(batch_size / float(mini_batch_size))
        return self.update_params_frequency

    def next_mini_batch_size(self):
        if self._idx + self.mini_batch_size > self.batch_size:
            self._x, self._y = self.next_batch()
            self._idx = 0
        self._idx += self.mini_batch_size
        return self._x[self._idx - self.mini_batch_size:self._idx], self._y[self._idx - self.mini_batch_size:self._idx]

    def __iter__(self):
        return self

    def __next__(self):
        return self.next_mini_batch_size()

    def to_generator(self):
        while True:
            yield next(self)


class VariationalMonteCarlo(MiniBatchGenerator):
    def __init__(self, model, operator, sampler, mini_batch_size=None, wave_function_evaluation_batch_size=None):
        super().__init__(sampler.batch_size, mini_batch_size)
        self.model = model
        self.operator = operator
        self.sampler = sampler
        self.energy_observable = operator if isinstance(operator, BaseObservable) else Observable(
            operator, evaluation_batch_size=wave_function_evaluation_batch_size or (1 << 17))
        self.current_batch = None
        self.current_local_energy = None
        self.current_energy = None
        self.current_local_energy_variance = None
        self.times = {}
        # evaluate connected configurations from the sampler's saved activations
        self.causal_reuse = True

    def _sample(self):
        out = self.sampler.sample()
        if isinstance(out, tuple):
            return out
        return out, None, None

    def _local_energy(self, spins, log_psi, saved=None):
        if saved is not None:
            return self.energy_observable.local_values(self.model, spins, log_psi=log_psi, base_saved=saved)
        return self.energy_observable.local_values(self.model, spins, log_psi=log_psi)

    def next_batch(self):
        spins, lp, _ = self._sample()
        local = self._local_energy(spins, lp)
        stats, _ = energy_stats(local)
        self.current_batch = spins
        self.current_local_energy = torch.complex(local[:, 0], local[:, 1])
        self.current_energy = complex(stats[0].item(), stats[1].item())
        self.current_local_energy_variance = stats[2].item()
        y = torch.conj(self.current_local_energy - self.current_energy) / self.batch_size
        return spins, y

    def step(self, optimizer, sync=True):
        """One VMC step. Returns the stats tensor [Re E, Im E, var] (device)."""
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        ev[0].record()
        spins, lp, saved = self._sample()
        ev[1].record()
        local = self._local_energy(spins, lp, saved if self.causal_reuse else None)
        stats, w = energy_stats(local)
        ev[2].record()
        if hasattr(optimizer, "update"):
            optimizer.update(spins, local, w, saved)
            ev[3].record()
        else:
            grad = self.model.backward(spins, w, saved)
            ev[3].record()
            optimizer.apply_gradient(grad)
        ev[4].record()
        self.current_batch = spins
        self._stats = stats
        self._events = ev
        self._local = local
        if sync:
            self.finish_step()
        return stats

    def finish_step(self):
        torch.cuda.current_stream().synchronize()
        ev = self._events
        self.times = {"sampling": ev[0].elapsed_time(ev[1]), "local_energy": ev[1].elapsed_time(ev[2]),
                      "gradient": ev[2].elapsed_time(ev[3]), "update": ev[3].elapsed_time(ev[4])}
        st = self._stats.tolist()
        self.current_energy = complex(st[0], st[1])
        self.current_local_energy_variance = st[2]
        self.current_local_energy = torch.complex(self._local[:, 0], self._local[:, 1])
        return self.times
