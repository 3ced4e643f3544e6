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
__next__ returns an int8 CUDA tensor (B, *shape) of +-1. As in the reference,
the Metropolis-Hastings samplers keep their chain state in the attribute
``sample`` (samplers/metropolis_hastings.py:28); every sampler also has
``sample_with_log_psi()`` -> (spins, log psi or None, activation workspace or
None), the call the VMC driver makes.
"""
import copy

import numpy as np

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

    def state_dict(self):
        """The draw position: with these the next draws repeat exactly."""
        return {"seed": self.seed, "offset": self.offset}

    def load_state_dict(self, state):
        self.seed = int(state["seed"])
        self.offset = int(state["offset"])

    def sample_with_log_psi(self):
        """(spins, log_psi, activation workspace) of one draw: the driver's
        sampler protocol (the workspace lets the local energy reuse the base
        activations and the adjoint skip a forward)."""
        return self.sample()

    def __next__(self):
        return self.sample()[0]


class AutoregressiveSampler(FastAutoregressiveSampler):
    """deepar/samplers/autoregressive.py:10-48: same exact distribution."""


def ctypes_ref(struct):
    import ctypes
    return ctypes.byref(struct)


def sum_correlations(corr):
    """metropolis_hastings.py:8-12: truncate at the first negative pair sum."""
    c = corr.tolist()
    for i in range(1, len(c) // 2):
        if c[2 * i - 1] + c[2 * i] < 0:
            return float(sum(c[:2 * i]))
    return float(sum(c))


def r_hat_and_correlations(values, n_chains):
    """metropolis_hastings.py:67-89 on a (chains x samples) series (chain-major
    flat input): Gelman-Rubin R-hat, variance, sum of the variogram
    autocorrelations (tau_int = 1 + 2 sum) and the effective sample size."""
    v = torch.as_tensor(values, dtype=torch.float64).reshape(n_chains, -1)
    spc = v.shape[1]
    b = v.numel()
    cm = v.mean(dim=1)
    mean = cm.mean()
    between = (spc / (n_chains - 1.0)) * ((cm - mean) ** 2).sum()
    if spc == 1:
        return 1.0, float(between), 0.0, float(b)
    within = ((v - cm[:, None]) ** 2).sum(dim=1).mean() / (spc - 1)
    var = ((spc - 1) * within + between) / spc
    r_hat = torch.sqrt(var / within)
    vt = torch.stack([((v[:, t + 1:] - v[:, :spc - t - 1]) ** 2).mean(dim=1).mean() for t in range(spc - 1)])
    corr = 1 - vt / (2 * var)
    cs = sum_correlations(corr)
    return float(r_hat), float(var), cs, b / (1 + 2 * cs)


class MetropolisHastingsSampler(Sampler):
    """samplers/metropolis_hastings.py:15-89 for RBM machines: all sweeps of a
    draw run in one persistent kernel (warp per chain)."""

    kind = 0

    def __init__(self, machine, batch_size, num_of_chains=1, unused_sampels=0, discard_ratio=10, seed=4321,
                 mini_batch_size=None):
        super().__init__(machine.hilbert_state_shape, batch_size, mini_batch_size)
        if batch_size % num_of_chains != 0:
            raise ValueError("Num of samplers must divide the batch size")
        self.machine = machine
        self.num_of_chains = int(num_of_chains)
        self.unused_sampels = int(unused_sampels)
        self.discard_ratio = int(discard_ratio)
        self.seed = int(seed)
        self.sweep = 0
        gen = torch.Generator().manual_seed(self.seed)
        n = machine.n
        self.sample = (2 * torch.randint(0, 2, (self.num_of_chains, n), generator=gen) - 1).to(torch.int8).to(
            machine.device)
        self.log_psi = torch.empty((self.num_of_chains, 2), dtype=torch.float32, device=machine.device)
        self.accepted = torch.zeros(1, dtype=torch.int64, device=machine.device)
        self.acceptance_ratio = 1.0

    def _grid(self):
        shape = self.input_size
        return (shape[0], 1) if len(shape) == 1 else (shape[0], int(np.prod(shape[1:])))

    def __next__(self):
        m = self.machine
        spc = self.batch_size // self.num_of_chains
        warm = (spc // self.discard_ratio) * self.unused_sampels if self.discard_ratio > 0 else 0
        out = torch.empty((self.num_of_chains, spc, m.n), dtype=torch.int8, device=m.device)
        self.accepted.zero_()
        h, w = self._grid()
        _lib.call("fk_rbm_mh_sweeps", _lib.ptr(m.kernel_params()), m.n, m.m, h, w, self.kind, _lib.ptr(self.sample),
                  _lib.ptr(self.log_psi), self.num_of_chains, warm, spc, self.unused_sampels, self.seed, self.sweep,
                  _lib.ptr(out), _lib.ptr(self.accepted), _lib.stream_ptr())
        self.sweep += warm + spc * (self.unused_sampels + 1)
        self._accepted_pending = (self.accepted, self.batch_size * (self.unused_sampels + 1))
        return out.view((self.batch_size,) + tuple(self.input_size))

    def sample_with_log_psi(self):
        return self.__next__(), None, None

    def update_acceptance_ratio(self):
        acc, total = self._accepted_pending
        self.acceptance_ratio = int(acc.item()) / total
        return self.acceptance_ratio

    def calc_r_hat_value(self, estimated_values):
        return r_hat_and_correlations(estimated_values, self.num_of_chains)

    def state_dict(self):
        """Chains, their log psi and the sweep counter of the Philox stream."""
        return {"sample": self.sample, "log_psi": self.log_psi, "seed": self.seed, "sweep": self.sweep}

    def load_state_dict(self, state):
        self.sample.copy_(state["sample"])
        self.log_psi.copy_(state["log_psi"])
        self.seed = int(state["seed"])
        self.sweep = int(state["sweep"])


class MetropolisHastingsLocal(MetropolisHastingsSampler):
    """metropolis_hastings.py:119-127: flip one random site."""
    kind = 0


class MetropolisHastingsExchange(MetropolisHastingsSampler):
    """metropolis_hastings.py:130-145: swap a random site with a random
    neighbour (offset in {-1, 0, 1} per axis, periodic)."""
    kind = 1


class MetropolisHastingsHamiltonian(Sampler):
    """metropolis_hastings.py:170-195: each sweep proposes, per chain, one of
    the operator's used connections of the current configuration (uniformly,
    slot 0 included when used) and accepts it with
    min(1, |psi(s')|^2 n(s) / (|psi(s)|^2 n(s'))), n = number of used
    connections. Chains start from ``hamiltonian.random_states`` (the
    total_sz sector when the operator has one). The warm-up and thinning
    schedule is the one of the other Metropolis-Hastings samplers. One sweep =
    enumeration of the chains' connections, the propose kernel, enumeration of
    the candidates' connections, the machine's log psi of the candidates and
    the accept kernel. Works with RBM and ConvNetAutoregressive2D machines."""

    def __init__(self, machine, batch_size, hamiltonian, num_of_chains=1, unused_sampels=0, discard_ratio=10,
                 seed=4321, mini_batch_size=None):
        super().__init__(machine.hilbert_state_shape, batch_size, mini_batch_size)
        if batch_size % num_of_chains != 0:
            raise ValueError("Num of samplers must divide the batch size")
        self.machine = machine
        self.hamiltonian = hamiltonian
        self.num_of_chains = int(num_of_chains)
        self.unused_sampels = int(unused_sampels)
        self.discard_ratio = int(discard_ratio)
        self.seed = int(seed)
        self.sweep = 0
        self.n_sites = int(np.prod(machine.hilbert_state_shape))
        gen = torch.Generator().manual_seed(self.seed)
        init = hamiltonian.random_states(self.num_of_chains, generator=gen)
        self.sample = torch.as_tensor(init).to(device=machine.device, dtype=torch.int8).reshape(
            self.num_of_chains, self.n_sites).contiguous()
        self.lp = self._log_psi(self.sample)
        self.cand = torch.empty_like(self.sample)
        self.n_conn = torch.empty(self.num_of_chains, dtype=torch.int32, device=machine.device)
        self.accepted = torch.zeros(1, dtype=torch.int64, device=machine.device)
        self.acceptance_ratio = 1.0

    def _log_psi(self, x):
        m = self.machine
        if hasattr(m, "log_psi_pairs"):
            return m.log_psi_pairs(x).contiguous()
        lp, _, _ = m.forward(x.view((-1,) + tuple(m.hilbert_state_shape)))
        return lp.contiguous()

    def _sweep(self, accepted):
        op = self.hamiltonian
        flips, _, use, _ = op.enumerate(self.sample)
        n_slots = use.shape[0]
        _lib.call("fk_mh_hamiltonian_propose", _lib.ptr(self.sample), _lib.ptr(flips), _lib.ptr(use), n_slots,
                  self.num_of_chains, self.n_sites, self.seed, self.sweep, _lib.ptr(self.cand),
                  _lib.ptr(self.n_conn), _lib.stream_ptr())
        _, _, use_c, _ = op.enumerate(self.cand)
        lp_c = self._log_psi(self.cand)
        _lib.call("fk_mh_hamiltonian_accept", _lib.ptr(self.sample), _lib.ptr(self.lp), _lib.ptr(self.cand),
                  _lib.ptr(lp_c), _lib.ptr(self.n_conn), _lib.ptr(use_c), n_slots, self.num_of_chains, self.n_sites,
                  self.seed, self.sweep, _lib.ptr(accepted) if accepted is not None else None,
                  _lib.stream_ptr())
        self.sweep += 1

    def __next__(self):
        spc = self.batch_size // self.num_of_chains
        warm = (spc // self.discard_ratio) * self.unused_sampels if self.discard_ratio > 0 else 0
        out = torch.empty((self.num_of_chains, spc, self.n_sites), dtype=torch.int8, device=self.machine.device)
        self.accepted.zero_()
        for _ in range(warm):
            self._sweep(None)
        for i in range(spc):
            for _ in range(self.unused_sampels + 1):
                self._sweep(self.accepted)
            out[:, i].copy_(self.sample)
        self._accepted_pending = (self.accepted, self.batch_size * (self.unused_sampels + 1))
        return out.view((self.batch_size,) + tuple(self.input_size))

    def sample_with_log_psi(self):
        return self.__next__(), None, None

    def update_acceptance_ratio(self):
        acc, total = self._accepted_pending
        self.acceptance_ratio = int(acc.item()) / total
        return self.acceptance_ratio

    def calc_r_hat_value(self, estimated_values):
        return r_hat_and_correlations(estimated_values, self.num_of_chains)

    def state_dict(self):
        return {"sample": self.sample, "log_psi": self.lp, "seed": self.seed, "sweep": self.sweep}

    def load_state_dict(self, state):
        self.sample.copy_(state["sample"])
        self.lp.copy_(state["log_psi"])
        self.seed = int(state["seed"])
        self.sweep = int(state["sweep"])


class MetropolisHastingsIndependent(Sampler):
    """Independent Metropolis-Hastings with a learned autoregressive proposal.

    Candidates s' are exact samples of the proposal network q (a
    ConvNetAutoregressive2D on the lattice, sampled by the persistent kernel);
    acceptance uses the exact ratio min(1, |psi(s')|^2 q(s) / (|psi(s)|^2 q(s'))),
    so |psi|^2 stays the stationary distribution whatever q is (the reference's
    MetropolisHastingsGlobal, metropolis_hastings.py:148-157, omits the q
    ratio). The proposal is fitted by maximum likelihood to the chain's own
    samples with the project's forward, adjoint and Adam kernels
    (``fit_proposal``)."""

    def __init__(self, machine, proposal, batch_size, num_of_chains, seed=777, init_chains=None):
        super().__init__(machine.hilbert_state_shape, batch_size)
        if batch_size % num_of_chains != 0:
            raise ValueError("Num of samplers must divide the batch size")
        self.machine = machine
        self.proposal = proposal
        self.num_of_chains = int(num_of_chains)
        self.seed = int(seed)
        self.step_count = 0
        self.proposal_sampler = FastAutoregressiveSampler(proposal, self.num_of_chains, seed=self.seed + 1)
        n = machine.n
        if init_chains is None:
            gen = torch.Generator().manual_seed(self.seed)
            init_chains = (2 * torch.randint(0, 2, (self.num_of_chains, n), generator=gen) - 1).to(torch.int8)
        self.sample = torch.as_tensor(init_chains).to(device=machine.device, dtype=torch.int8).reshape(
            self.num_of_chains, n).contiguous()
        self.accepted = torch.zeros(1, dtype=torch.int64, device=machine.device)
        self.acceptance_ratio = 1.0
        self._opt = None
        self._refresh()

    def _refresh(self):
        self.lp = self.machine.log_psi_pairs(self.sample).contiguous()
        lq, _, _ = self.proposal.forward(self.sample.view((-1,) + self.proposal.hilbert_state_shape))
        self.lq = lq.contiguous()

    def fit_proposal(self, samples, steps=50, lr=3e-3, batch=None):
        """Maximum likelihood: minimise -mean log q(s) = -mean 2 Re log psi_q(s)."""
        from .optimizers import Adam
        q = self.proposal
        if self._opt is None or self._opt.lr != lr:
            self._opt = Adam(q, lr=lr)
        s = torch.as_tensor(samples).to(device=q.device, dtype=torch.int8).reshape(
            (-1,) + q.hilbert_state_shape)
        b = s.shape[0] if batch is None else min(batch, s.shape[0])
        w = torch.zeros((b, 2), dtype=torch.float32, device=q.device)
        w[:, 0] = -2.0 / b
        gen = torch.Generator(device=q.device).manual_seed(self.seed + 17)
        for _ in range(steps):
            idx = torch.randint(0, s.shape[0], (b,), device=q.device, generator=gen) if b < s.shape[0] else None
            x = s[idx] if idx is not None else s
            _, _, saved = q.forward(x, mode=_lib.FK_AR2D_SAVE)
            self._opt.apply_gradient(q.backward(x, w, saved))
        self._refresh()

    def mean_log_likelihood(self, samples):
        lq = self.proposal.log_psi(torch.as_tensor(samples).to(self.proposal.device).reshape(
            (-1,) + self.proposal.hilbert_state_shape)).real
        return float((2 * lq).mean())

    def step(self):
        m = self.machine
        cand, lq_c, _ = self.proposal_sampler.sample()
        cand = cand.reshape(self.num_of_chains, m.n).contiguous()
        lp_c = m.log_psi_pairs(cand).contiguous()
        _lib.call("fk_mh_independent_step", _lib.ptr(self.sample), _lib.ptr(self.lp), _lib.ptr(self.lq),
                  _lib.ptr(cand), _lib.ptr(lp_c), _lib.ptr(lq_c.contiguous()), self.num_of_chains, m.n, self.seed,
                  self.step_count, _lib.ptr(self.accepted), _lib.stream_ptr())
        self.step_count += 1

    def __next__(self):
        spc = self.batch_size // self.num_of_chains
        out = torch.empty((self.num_of_chains, spc, self.machine.n), dtype=torch.int8, device=self.machine.device)
        self.accepted.zero_()
        for i in range(spc):
            self.step()
            out[:, i] = self.sample
        self._accepted_pending = (self.accepted, self.batch_size)
        return out.view((self.batch_size,) + tuple(self.input_size))

    def sample_with_log_psi(self):
        return self.__next__(), None, None

    def update_acceptance_ratio(self):
        acc, total = self._accepted_pending
        self.acceptance_ratio = int(acc.item()) / total
        return self.acceptance_ratio

    def calc_r_hat_value(self, estimated_values):
        return r_hat_and_correlations(estimated_values, self.num_of_chains)
