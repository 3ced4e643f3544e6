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
        """(spins, log psi or None, activation workspace or None) from the
        sampler's ``sample_with_log_psi()``, or ``next(sampler)`` for a plain
        iterator (the reference driver's call, variational_monte_carlo.py:46)."""
        if hasattr(self.sampler, "sample_with_log_psi"):
            out = self.sampler.sample_with_log_psi()
        else:
            out = (next(self.sampler), None, None)
        if getattr(self.sampler, "machine", self.model) is not self.model:
            # drawn from another machine (the base of a symmetrised ensemble,
            # experiments/run_evaluation.py:12-24): log psi and the local
            # energy's connected configurations come from the model itself
            return out[0], None, None
        return out

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
        """Waits for the step, raises if a kernel recorded a failure (a
        timed-out device wait or a non-finite energy) and publishes the
        energy, variance, local energies and stage times."""
        _lib.check_device("VariationalMonteCarlo.step")
        ev = self._events
        self.times = {"sampling": ev[0].elapsed_time(ev[1]), "local_energy": ev[1].elapsed_time(ev[2]),
                      "gradient": ev[2].elapsed_time(ev[3]), "update": ev[3].elapsed_time(ev[4])}
        st = self._stats.tolist()
        self.current_energy = complex(st[0], st[1])
        self.current_local_energy_variance = st[2]
        self.current_local_energy = torch.complex(self._local[:, 0], self._local[:, 1])
        return self.times


class ExactVariational:
    """Exact-enumeration driver (optimization/exact_variational.py:96-155).

    All 2^N configurations (site i = bit i of the index, bit 1 -> +1, as
    exact/utils.py:48-57) are evaluated on the GPU, |psi|^2 is normalised
    over them (exact_variational.py:124-130, FP64 log-sum-exp), E_loc is
    computed for every configuration (the connected configurations reuse
    the base activations), E = sum_s p_s E_loc(s) and
    var = sum_s p_s (Re E_loc(s) - Re E)^2 in FP64
    (exact_variational.py:91-95), and the loss coefficients are
    y_s = p_s conj(E_loc(s) - E) (exact_variational.py:132-135).

    ``step(optimizer)`` takes one optimizer step per enumeration with the
    exact energy gradient 2 Re sum_s y_s dlogpsi_s, i.e. the reference's
    generator with ``batch_size`` = 2^N without Keras' division by the
    mini-batch size (a constant factor). ``to_generator()`` yields
    (configurations, y) batches of ``batch_size`` as the reference's does.
    Sampling-free: for lattices up to ~24 sites."""

    def __init__(self, model, operator, batch_size=None):
        h, w = model.hilbert_state_shape
        n = h * w
        if n > 24:
            raise ValueError("ExactVariational enumerates 2^N configurations; N <= 24")
        self.model = model
        self.operator = operator
        self.num_of_states = 1 << n
        bs = self.num_of_states if batch_size is None else min(int(batch_size), self.num_of_states)
        if self.num_of_states % bs != 0:
            raise ValueError("In exact the batch size must divide the total number of states in the system")
        self.batch_size = bs
        idx = torch.arange(self.num_of_states, device=model.device, dtype=torch.int64)
        bits = (idx[:, None] >> torch.arange(n, device=model.device, dtype=torch.int64)[None, :]) & 1
        self.states = (2 * bits - 1).to(torch.int8).view(-1, h, w)
        self.energy_observable = Observable(operator)
        self.probs = None
        self.current_energy = None
        self.current_local_energy = None
        self.current_local_energy_variance = None
        self._w = None
        self._saved = None

    def machine_updated(self):
        """wave function, probabilities, local energies, energy and coefficients."""
        lp, _, saved = self.model.forward(self.states, mode=_lib.FK_AR2D_SAVE)
        local = self.energy_observable.local_values(self.model, self.states, log_psi=lp, base_saved=saved)
        lr2 = 2.0 * lp[:, 0].double()
        p = torch.exp(lr2 - torch.logsumexp(lr2, 0))
        e = (p[:, None] * local).sum(0)
        d_re = local[:, 0] - e[0]
        d_im = local[:, 1] - e[1]
        self.probs = p
        self.current_local_energy = torch.complex(local[:, 0], local[:, 1])
        self.current_energy = complex(e[0].item(), e[1].item())
        self.current_local_energy_variance = float((p * d_re * d_re).sum().item())
        self.y = torch.complex(p * d_re, -p * d_im)
        # adjoint seeds of 2 Re(logpsi y): (d/dRe logpsi, d/dIm logpsi)
        self._w = torch.stack((2.0 * p * d_re, 2.0 * p * d_im), dim=1).float().contiguous()
        self._saved = saved
        return self.current_energy

    def step(self, optimizer):
        self.machine_updated()
        if hasattr(optimizer, "update"):
            raise ValueError("ExactVariational takes gradient optimizers (the SR Gram is sample-space)")
        grad = self.model.backward(self.states, self._w, self._saved)
        optimizer.apply_gradient(grad)
        return self.current_energy

    def to_generator(self):
        while True:
            self.machine_updated()
            for i in range(0, self.num_of_states, self.batch_size):
                yield self.states[i:i + self.batch_size], self.y[i:i + self.batch_size]

    def __iter__(self):
        return self.to_generator()
