"""Local-energy observables (flowket.observables.monte_carlo drop-ins).

``Observable(operator).local_values(machine, configurations)`` restates
observables/monte_carlo/operator.py:13-53 on the GPU: the operator enumerates
the connected configurations (kernel c), the used ones are compacted
(operator.py:6-10), their log psi is evaluated in batched network passes and
E_loc(s) = sum_c mel_c exp(log psi(s_c) - log psi(s)) is reduced per sample
with a compensated sum. ``estimate`` returns (mean, var(Re), local values)
(observable.py:10-14).
"""
import torch

from . import _lib


class BaseObservable:
    def estimate(self, machine, configurations, log_psi=None):
        local = self.local_values(machine, configurations, log_psi=log_psi)
        stats, _ = energy_stats(local)
        return complex(stats[0].item(), stats[1].item()), stats[2].item(), local


def energy_stats(local):
    """(stats float64 [Re mean, Im mean, var Re], loss weights float32 (B, 2))."""
    b = local.shape[0]
    stats = torch.empty(3, dtype=torch.float64, device=local.device)
    w = torch.empty((b, 2), dtype=torch.float32, device=local.device)
    _lib.call("fk_energy_stats", _lib.ptr(local), b, _lib.ptr(stats), _lib.ptr(w), _lib.stream_ptr())
    return stats, w


class Observable(BaseObservable):
    def __init__(self, operator, evaluation_batch_size=1 << 17):
        self.operator = operator
        self.evaluation_batch_size = int(evaluation_batch_size)
        self._buf = {}
        # optional CUDA-event timing of the batched network passes (bench)
        self.record_forward = False
        self.forward_events = []
        self.last_forward = (0.0, 0)

    def _buffers(self, b, c, n, device):
        key = (b, c, n)
        if key not in self._buf:
            rows = b * (c - 1)
            self._buf = {key: dict(
                configs=torch.empty((rows, n), dtype=torch.int8, device=device),
                owner=torch.empty(rows, dtype=torch.int32, device=device),
                cmel=torch.empty(rows, dtype=torch.float64, device=device),
                cflips=torch.empty((rows, 2), dtype=torch.int16, device=device),
                offsets=torch.empty(b + 1, dtype=torch.int64, device=device),
                nrows=torch.empty(1, dtype=torch.int64, device=device),
                ws=torch.empty(_lib.load().fk_compact_workspace_bytes(b), dtype=torch.uint8, device=device),
                local=torch.empty((b, 2), dtype=torch.float64, device=device))}
        return self._buf[key]

    def connections(self, configurations):
        """Compact list of used connections (slot 0 excluded)."""
        flips, mel, use, spins = self.operator.enumerate(configurations)
        c, b = mel.shape
        n = spins.shape[1]
        bf = self._buffers(b, c, n, spins.device)
        _lib.call("fk_compact_connections", _lib.ptr(spins), b, n, c, _lib.ptr(flips), _lib.ptr(mel), _lib.ptr(use), 1,
                  _lib.ptr(bf["configs"]), _lib.ptr(bf["owner"]), _lib.ptr(bf["cmel"]), _lib.ptr(bf["cflips"]),
                  _lib.ptr(bf["offsets"]), b * (c - 1), _lib.ptr(bf["nrows"]), _lib.ptr(bf["ws"]), bf["ws"].numel(),
                  _lib.stream_ptr())
        if getattr(self.operator, "all_connections_used", False):
            # every slot is a connection (Ising): the row count is known on
            # the host and the step needs no device synchronisation here
            rows = b * (c - 1)
        else:
            rows = int(bf["nrows"].item())
        return spins, mel, bf, rows

    def local_values(self, machine, configurations, log_psi=None, base_saved=None):
        """E_loc per sample ((B, 2) float64). With `base_saved` (the sampler's
        or a FK_AR2D_SAVE forward's workspace for these configurations) the
        connected configurations reuse the base activations (causal reuse).
        Machines with their own local-energy kernel (the RBM family: ratios
        from incremental theta updates) evaluate it directly."""
        if hasattr(machine, "local_energy"):
            return machine.local_energy(self.operator, configurations)
        spins, mel, bf, rows = self.connections(configurations)
        b = spins.shape[0]
        if log_psi is None:
            lp_self, _, _ = machine.forward(spins)
        else:
            lp_self = log_psi
        if self.record_forward:
            ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ev[0].record()
        if base_saved is not None and hasattr(machine, "forward_connections"):
            lp_rows = machine.forward_connections(bf["configs"], bf["owner"], bf["cflips"], rows, base_saved, b,
                                                  chunk=self.evaluation_batch_size)
        else:
            lp_rows = torch.empty((max(rows, 1), 2), dtype=torch.float32, device=spins.device)
            for i in range(0, rows, self.evaluation_batch_size):
                j = min(rows, i + self.evaluation_batch_size)
                lp, _, _ = machine.forward(bf["configs"][i:j])
                lp_rows[i:j] = lp
        if self.record_forward:
            ev[1].record()
            self.forward_events.append(ev)
        self.last_forward = (0.0, rows)
        mel0 = mel[0].contiguous()
        _lib.call("fk_local_energy_reduce", _lib.ptr(lp_self), _lib.ptr(mel0), b, _lib.ptr(lp_rows),
                  _lib.ptr(bf["offsets"]), _lib.ptr(bf["cmel"]), _lib.ptr(bf["local"]), _lib.stream_ptr())
        return bf["local"]
