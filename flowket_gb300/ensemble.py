"""Symmetrised ensembles of a machine (flowket.machines.ensemble drop-in).

A machine's log psi is evaluated on symmetry images of each configuration
and combined per configuration (machines/ensemble.py:14-69):

* probabilistic (default, ensemble.py:14-19): Re = 1/2 logsumexp(2 Re_t) -
  1/2 log n, Im = angle(mean_t exp(i Im_t)), i.e. |psi|^2 is averaged;
* average (ensemble.py:22-23): log(mean_t psi_t).

Images: ``make_2d_obc_invariants`` the 4 rotations (layers/dihedral_4_invariants.py,
tf.image.rot90) and their left-right flips; ``make_pbc_invariants`` every
translation (layers/transition_invariants.py, tf.roll), composed by default
with the 2D OBC invariants; ``make_up_down_invariant`` the configuration and
its spin flip. The wrapped machine evaluates every image on the GPU in one
batched pass per chunk; the combination is FP64. Ensembles are evaluation
machines: ``forward`` gives log psi only (no conditionals, no saved
activations), so the local energy evaluates connected configurations in full
and ``VariationalMonteCarlo`` with a sampler of the base machine recomputes
the sample's log psi with the ensemble, as the reference's evaluation does
(experiments/run_evaluation.py:12-24).
"""
import itertools
import math

import torch

from . import _lib


class EnsembleMachine:
    def __init__(self, machine, transforms, probabilistic=True, chunk=1 << 16):
        self.machine = machine
        self.transforms = list(transforms)
        self.probabilistic = bool(probabilistic)
        self.hilbert_state_shape = tuple(machine.hilbert_state_shape)
        self.device = machine.device
        self.chunk = int(chunk)

    @property
    def ensemble_size(self):
        return len(self.transforms)

    def _images(self, x):
        return torch.stack([t(x) for t in self.transforms], dim=1)  # (B, n, H, W)

    def _combine(self, lp):
        """lp (B, n, 2) float -> (B, 2) float32."""
        re = lp[..., 0].double()
        im = lp[..., 1].double()
        n = lp.shape[1]
        if self.probabilistic:
            new_re = 0.5 * torch.logsumexp(2.0 * re, dim=1) - 0.5 * math.log(n)
            new_im = torch.atan2(torch.sin(im).mean(dim=1), torch.cos(im).mean(dim=1))
        else:
            # log(mean_t exp(re_t + i im_t)), scaled by the largest amplitude
            mx = re.max(dim=1, keepdim=True).values
            mag = torch.exp(re - mx)
            zr = (mag * torch.cos(im)).mean(dim=1)
            zi = (mag * torch.sin(im)).mean(dim=1)
            new_re = mx[:, 0] + 0.5 * torch.log(zr * zr + zi * zi)
            new_im = torch.atan2(zi, zr)
        return torch.stack((new_re, new_im), dim=1).float()

    def forward(self, spins, mode=_lib.FK_AR2D_INFER, with_cond=False, workspace=None):
        if mode != _lib.FK_AR2D_INFER or with_cond:
            raise ValueError("an ensemble machine evaluates log psi only")
        h, w = self.hilbert_state_shape
        x = torch.as_tensor(spins, device=self.device).to(torch.int8).reshape(-1, h, w)
        b = x.shape[0]
        n = self.ensemble_size
        out = torch.empty((b, 2), dtype=torch.float32, device=self.device)
        step = max(1, self.chunk // n)
        for i in range(0, b, step):
            j = min(b, i + step)
            imgs = self._images(x[i:j]).reshape(-1, h, w).contiguous()
            lp, _, _ = self.machine.forward(imgs)
            out[i:j] = self._combine(lp.reshape(j - i, n, 2))
        return out, None, None

    def log_psi(self, spins, chunk=None):
        lp, _, _ = self.forward(spins)
        return torch.complex(lp[:, 0], lp[:, 1])

    def predict(self, spins, batch_size=None):
        return self.log_psi(spins).unsqueeze(1)


def _check_square(shape):
    if len(shape) != 2 or shape[0] != shape[1]:
        raise ValueError("rotation invariants need a square lattice, got %s" % (shape,))


def make_2d_obc_invariants(machine, probabilistic=True):
    """ensemble.py:41-48: rotations by 0..3 quarter turns and their left-right flips."""
    _check_square(machine.hilbert_state_shape)
    rots = [lambda x, k=k: torch.rot90(x, k, dims=(1, 2)) for k in range(4)]
    flips = [lambda x, r=r: torch.flip(r(x), dims=(2,)) for r in rots]
    return EnsembleMachine(machine, rots + flips, probabilistic)


def make_pbc_invariants(machine, apply_also_obc_invariants=True, probabilistic=True):
    """ensemble.py:51-58: every translation (tf.roll by (i, j)), each
    evaluated by the 2D OBC ensemble when ``apply_also_obc_invariants``."""
    inner = make_2d_obc_invariants(machine, probabilistic) if apply_also_obc_invariants else machine
    h, w = machine.hilbert_state_shape
    rolls = [lambda x, s=s: torch.roll(x, shifts=s, dims=(1, 2)) for s in itertools.product(range(h), range(w))]
    return EnsembleMachine(inner, rolls, probabilistic)


def make_up_down_invariant(machine, probabilistic=True):
    """ensemble.py:61-66: the configuration and its global spin flip."""
    return EnsembleMachine(machine, [lambda x: x, lambda x: -x], probabilistic)
