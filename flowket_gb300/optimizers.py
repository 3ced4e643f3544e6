"""Optimisers (flowket.optimizers / tf.keras drop-ins) updating a machine's
flat parameter vector on the GPU.

* ``Adam``: tf.keras Adam of TF 1.x (lr_t = lr sqrt(1-b2^t)/(1-b1^t),
  epsilon = K.epsilon() = 1e-7), the optimiser of experiments/train.py:52
  and the examples.
* ``ComplexValuesStochasticReconfiguration``: optimizers/stochastic_reconfiguration/optimizer.py:14-183,
  solved in sample space on the GPU.
"""
import torch

from . import _lib


class Adam:
    def __init__(self, machine, lr=1e-3, beta_1=0.9, beta_2=0.999, epsilon=1e-7):
        self.machine = machine
        self.lr, self.beta_1, self.beta_2, self.epsilon = float(lr), float(beta_1), float(beta_2), float(epsilon)
        self.m = torch.zeros_like(machine.params)
        self.v = torch.zeros_like(machine.params)
        self.iterations = 0

    def apply_gradient(self, grad):
        self.iterations += 1
        _lib.call("fk_adam_step", _lib.ptr(self.machine.params), _lib.ptr(grad), _lib.ptr(self.m), _lib.ptr(self.v),
                  self.machine.num_params, self.iterations, self.lr, self.beta_1, self.beta_2, self.epsilon,
                  _lib.stream_ptr())
        self.machine.params_updated()

    def state_dict(self):
        return {"m": self.m, "v": self.v, "iterations": self.iterations}

    def load_state_dict(self, state):
        self.m.copy_(state["m"])
        self.v.copy_(state["v"])
        self.iterations = int(state["iterations"])


class ComplexValuesStochasticReconfiguration:
    """Stochastic reconfiguration (optimizers/stochastic_reconfiguration/optimizer.py:14-183)
    in sample space on the GPU.

    Complex parameters (the RBM family, the reference's own use of SR,
    complex_values_optimizer.py:28-82): S = <O_c^* O_c> + diag_shift I,
    F = <O_c^* (E - Ebar)>, solved through the B x B Hermitian Gram
    T = O_c O_c^H: z = (T / B + diag_shift I)^-1 (E - Ebar), x = O_c^H z / B,
    theta <- theta - lr x (fk_sr_hermitian_embed, fk_sr_solve on the real
    embedding, fk_sr_complex_backmap).

    Real parameters with a complex log psi (the AR network): S = Re<O_c^* O_c>
    + diag_shift I and F = Re<O_c^* (E - Ebar)>, via the 2B x 2B Gram of
    Y = [Re O_c | Im O_c]: alpha = (Y^T Y / B + diag_shift I)^-1 [Re E_c; Im E_c],
    x = Y alpha / B.

    The solve is FP64 CG with the reference's tolerance rule
    (linear_equations.py:34-137); ``iterative_solver=False`` runs CG to 1e-10
    instead of a Cholesky factorisation.

    ``gram``: "tc" builds the Gram on the tensor cores (split-BF16 products,
    FP32-level accuracy: fk_sr_gram_split + fk_sr_gram_split_accumulate),
    "fp32" on the CUDA cores (fk_sr_gram); "auto" takes the tensor cores for
    a machine on the tensor-core path (BF16/FP16), the CUDA cores otherwise
    (the plain FP32 path stays on CUDA cores throughout).

    ``rows_bytes``: for the AR network, the per-sample rows Y (num_params x
    2B float32) are stored whole when they take at most
    ``STORED_ROWS_LIMIT`` bytes; otherwise (or whenever ``rows_bytes`` is
    given) they are streamed: fk_ar2d_sr_gram builds the Gram conv by conv
    through a row buffer of ``rows_bytes`` (default ``STREAM_BUFFER_BYTES``)
    from the two per-sample adjoints (seeds (1, 0) and (0, 1)) run together
    over the step's activations, and the update x = Y alpha / B is the summed
    adjoint with the centred seeds (alpha_b - mean, alpha_{B+b} - mean) / B,
    so that Y is never held: the memory on top of the step's is two adjoint
    workspaces, the buffer and the Gram."""

    STORED_ROWS_LIMIT = 32 << 30
    STREAM_BUFFER_BYTES = 16 << 30

    def __init__(self, machine, predictions_jacobian=None, lr=0.01, diag_shift=0.05, iterative_solver=True,
                 compute_jvp_instead_of_full_jacobian=False, use_cholesky=True, conjugate_gradient_tol=1e-3,
                 iterative_solver_max_iterations=200, gram="auto", rows_bytes=None, **kwargs):
        if gram not in ("auto", "tc", "fp32"):
            raise ValueError("gram must be 'auto', 'tc' or 'fp32'")
        if rows_bytes is not None and int(rows_bytes) <= 0:
            raise ValueError("rows_bytes must be positive")
        self.gram = gram
        self.rows_bytes = None if rows_bytes is None else int(rows_bytes)
        self.streamed = False
        self.machine = machine
        self.lr = float(lr)
        self.diag_shift = float(diag_shift)
        self.iterative_solver = iterative_solver
        self.tol = float(conjugate_gradient_tol) if iterative_solver else 1e-10
        self.max_iter = int(iterative_solver_max_iterations or 1000) if iterative_solver else 2000
        self.iterations = 0
        self.last_stats = None
        self._buf = {}

    def _buffers(self, n, dev):
        if n not in self._buf:
            lib = _lib.load()
            self._buf = {n: dict(gram=torch.empty((n, n), dtype=torch.float64, device=dev),
                                 alpha=torch.empty(n, dtype=torch.float64, device=dev),
                                 rhs=torch.empty(n, dtype=torch.float64, device=dev),
                                 stats=torch.zeros(3, dtype=torch.float64, device=dev),
                                 ws=torch.empty(lib.fk_sr_solve_workspace_bytes(n), dtype=torch.uint8, device=dev))}
        return self._buf[n]

    def update(self, spins, local, w, saved):
        m = self.machine
        if getattr(m, "is_complex", False):
            self._complex_solve(spins, local, self.lr, m.params, None)
        else:
            x = self.direction(spins, local, saved)
            _lib.call("fk_axpy", m.num_params, -self.lr, _lib.ptr(x), _lib.ptr(m.params), _lib.stream_ptr())
        m.params_updated()
        self.iterations += 1
        self.last_stats = self._buf[2 * spins.shape[0]]["stats"]

    def _gram_entry(self, b):
        if self.gram == "tc":
            return "fk_sr_gram_tc"
        if self.gram == "fp32":
            return "fk_sr_gram"
        tc = getattr(self.machine, "precision", "fp32") in ("bf16", "fp16")
        return "fk_sr_gram_tc" if tc else "fk_sr_gram"

    def _center_gram(self, o_re, o_im, p, b, gram, st):
        """Centres the rows of o_re and o_im (p x b each) in place and builds
        gram = Y^T Y, Y = [o_re | o_im] (p x 2b): on the tensor cores from
        operands split into bf16 hi + lo once, centring and split in one pass
        (fk_sr_center_split, then fk_sr_gram_split_accumulate), or on the CUDA
        cores (fk_center_columns, fk_sr_gram)."""
        n = 2 * b
        if self._gram_entry(b) == "fk_sr_gram":
            _lib.call("fk_center_columns", _lib.ptr(o_re), p, b, None, st)
            _lib.call("fk_center_columns", _lib.ptr(o_im), p, b, None, st)
            _lib.call("fk_sr_gram", _lib.ptr(o_re), _lib.ptr(o_im), p, b, _lib.ptr(gram), n * n, st)
            return
        nbytes = _lib.load().fk_sr_gram_split_bytes(p, n)
        split = torch.empty(nbytes, dtype=torch.uint8, device=gram.device)
        _lib.call("fk_sr_center_split", _lib.ptr(o_re), _lib.ptr(o_im), b, b, p, n, 1, _lib.ptr(split), nbytes, st)
        gram.zero_()
        _lib.call("fk_sr_gram_split_accumulate", _lib.ptr(split), p, n, _lib.ptr(gram), st)
        _lib.call("fk_sr_gram_mirror", _lib.ptr(gram), n, st)

    def _max_iter(self, n, n_complex_params):
        if self.iterative_solver:
            return self.max_iter
        # T / B has rank <= P (complex), its real embedding <= 2P: CG on the
        # shifted system terminates after at most 2P + 1 distinct eigenvalues
        return min(self.max_iter, 4 * n_complex_params + 20, n + 20)

    def _complex_solve(self, spins, local, lr, params, x_out):
        m = self.machine
        b = spins.shape[0]
        o_re, o_im = m.log_derivatives_split(spins)
        p = o_re.shape[0]
        st = _lib.stream_ptr()
        n = 2 * b
        bf = self._buffers(n, m.device)
        self._center_gram(o_re, o_im, p, b, bf["gram"], st)
        _lib.call("fk_sr_hermitian_embed", _lib.ptr(bf["gram"]), b, st)
        bf["rhs"][:b] = local[:, 0] - local[:, 0].mean()
        bf["rhs"][b:] = local[:, 1] - local[:, 1].mean()
        _lib.call("fk_sr_solve", _lib.ptr(bf["gram"]), n, 1.0 / b, self.diag_shift, _lib.ptr(bf["rhs"]), self.tol,
                  self._max_iter(n, p), _lib.ptr(bf["alpha"]), _lib.ptr(bf["stats"]), _lib.ptr(bf["ws"]),
                  bf["ws"].numel(), st)
        _lib.call("fk_sr_complex_backmap", _lib.ptr(o_re), _lib.ptr(o_im), p, b, _lib.ptr(bf["alpha"]), 1.0 / b,
                  lr, _lib.ptr(params), _lib.ptr(x_out), st)

    def direction(self, spins, local, saved=None):
        """The solution x of the SR system (no update): float32 (num_params,);
        for complex parameters interleaved (re, im)."""
        m = self.machine
        if getattr(m, "is_complex", False):
            x = torch.empty(m.num_params, dtype=torch.float32, device=m.device)
            self._complex_solve(spins, local, 0.0, None, x)
            return x
        b = spins.shape[0]
        p = m.num_params
        self.streamed = self.rows_bytes is not None or 2 * p * b * 4 > self.STORED_ROWS_LIMIT
        if self.streamed:
            return self._streamed_direction(spins, local, saved)
        ones = torch.zeros((b, 2), dtype=torch.float32, device=m.device)
        ones[:, 0] = 1
        o_re = m.backward(spins, ones, saved, per_sample=True)
        ones[:, 0] = 0
        ones[:, 1] = 1
        o_im = m.backward(spins, ones, saved, per_sample=True)
        p = m.num_params
        st = _lib.stream_ptr()
        n = 2 * b
        bf = self._buffers(n, m.device)
        self._center_gram(o_re, o_im, p, b, bf["gram"], st)
        bf["rhs"][:b] = local[:, 0] - local[:, 0].mean()
        bf["rhs"][b:] = local[:, 1] - local[:, 1].mean()
        _lib.call("fk_sr_solve", _lib.ptr(bf["gram"]), n, 1.0 / b, self.diag_shift, _lib.ptr(bf["rhs"]), self.tol,
                  self.max_iter, _lib.ptr(bf["alpha"]), _lib.ptr(bf["stats"]), _lib.ptr(bf["ws"]), bf["ws"].numel(),
                  st)
        x = torch.empty(p, dtype=torch.float32, device=m.device)
        _lib.call("fk_sr_backmap", _lib.ptr(o_re), _lib.ptr(o_im), p, b, _lib.ptr(bf["alpha"]), 1.0 / b, 0.0, None,
                  _lib.ptr(x), st)
        return x

    def _streamed_direction(self, spins, local, saved):
        from .machines import ctypes_ref
        m = self.machine
        lib = _lib.load()
        s = m._spins(spins)
        b = s.shape[0]
        n = 2 * b
        st = _lib.stream_ptr()
        if saved is None:
            _, _, saved = m.forward(s, mode=_lib.FK_AR2D_SAVE)
        ws = torch.empty(lib.fk_ar2d_sr_gram_workspace_bytes(ctypes_ref(m.desc), b), dtype=torch.uint8,
                         device=m.device)
        tc = 1 if self._gram_entry(b) == "fk_sr_gram_tc" else 0
        budget = self.rows_bytes if self.rows_bytes is not None else self.STREAM_BUFFER_BYTES
        floats = min(budget // 4, m.num_params * n * (2 if tc else 1))
        floats = max(floats, lib.fk_ar2d_sr_gram_min_rows(ctypes_ref(m.desc), b, tc))
        rows = torch.empty(floats, dtype=torch.float32, device=m.device)
        bf = self._buffers(n, m.device)
        _lib.call("fk_ar2d_sr_gram", ctypes_ref(m.desc), _lib.ptr(m.packed()), _lib.ptr(m.params), _lib.ptr(s), b,
                  _lib.ptr(saved), saved.numel(), _lib.ptr(ws), ws.numel(), _lib.ptr(rows), rows.numel(),
                  _lib.ptr(bf["gram"]), tc, st)
        del rows, ws
        bf["rhs"][:b] = local[:, 0] - local[:, 0].mean()
        bf["rhs"][b:] = local[:, 1] - local[:, 1].mean()
        _lib.call("fk_sr_solve", _lib.ptr(bf["gram"]), n, 1.0 / b, self.diag_shift, _lib.ptr(bf["rhs"]), self.tol,
                  self.max_iter, _lib.ptr(bf["alpha"]), _lib.ptr(bf["stats"]), _lib.ptr(bf["ws"]), bf["ws"].numel(),
                  st)
        # x = Y alpha / B = sum_b (alpha_b - mean) Re O_b + (alpha_{B+b} - mean) Im O_b, all / B: the
        # summed adjoint with these seeds
        a = bf["alpha"]
        w = torch.stack([a[:b] - a[:b].mean(), a[b:] - a[b:].mean()], dim=1).div_(b).to(torch.float32).contiguous()
        return m.backward(s, w, saved)


class AccumulateGradientOptimizer:
    """optimizers/accumulate_gradient_optimizer.py:13-88: gradients of
    ``update_params_frequency`` consecutive steps are summed (or averaged:
    each divided by the frequency) in a device buffer and applied by the
    wrapped optimiser on every ``update_params_frequency``-th call, which
    then clears the buffer. With ``ema_decay`` > 0 an exponential moving
    average of the parameters after each applied update is kept;
    ``set_weights_ema`` loads its bias-corrected value
    (ema / (1 - decay^updates)). One GPU per process: there is no Horovod
    allreduce (replicas only)."""

    def __init__(self, optimizer, update_params_frequency, accumulate_sum_or_mean=True, ema_decay=0,
                 use_horovod=False):
        if update_params_frequency < 1:
            raise ValueError("update_params_frequency must be >= 1")
        if use_horovod:
            raise ValueError("no Horovod allreduce: one process per GPU runs independent replicas")
        self.optimizer = optimizer
        self.machine = optimizer.machine
        self.update_params_frequency = int(update_params_frequency)
        self.accumulate_sum = bool(accumulate_sum_or_mean)
        self.ema_decay = float(ema_decay)
        self.accumulated_iterations = 0
        self.total_iterations = 0
        self.accumulated_gradient = torch.zeros_like(self.machine.params)
        self.params_ema = torch.zeros_like(self.machine.params) if self.ema_decay > 0 else None

    def set_update_params_frequency(self, update_params_frequency):
        self.update_params_frequency = int(update_params_frequency)

    def apply_gradient(self, grad):
        if self.accumulate_sum:
            self.accumulated_gradient.add_(grad)
        else:
            self.accumulated_gradient.add_(grad, alpha=1.0 / self.update_params_frequency)
        self.accumulated_iterations += 1
        if self.accumulated_iterations % self.update_params_frequency != 0:
            return
        self.optimizer.apply_gradient(self.accumulated_gradient)
        self.accumulated_gradient.zero_()
        if self.params_ema is not None:
            self.total_iterations += 1
            self.params_ema.mul_(self.ema_decay).add_(self.machine.params, alpha=1.0 - self.ema_decay)

    def set_weights_ema(self):
        if self.params_ema is None or self.total_iterations == 0:
            return
        self.machine.params.copy_(self.params_ema / (1.0 - self.ema_decay ** self.total_iterations))
        self.machine.params_updated()

    def state_dict(self):
        return {"optimizer": self.optimizer.state_dict(), "accumulated_gradient": self.accumulated_gradient,
                "accumulated_iterations": self.accumulated_iterations, "total_iterations": self.total_iterations,
                "params_ema": self.params_ema}

    def load_state_dict(self, state):
        self.optimizer.load_state_dict(state["optimizer"])
        self.accumulated_gradient.copy_(state["accumulated_gradient"])
        self.accumulated_iterations = int(state["accumulated_iterations"])
        self.total_iterations = int(state["total_iterations"])
        if self.params_ema is not None and state["params_ema"] is not None:
            self.params_ema.copy_(state["params_ema"])


def convert_to_accumulate_gradient_optimizer(orig_optimizer, update_params_frequency, accumulate_sum_or_mean=True,
                                             ema_decay=0, use_horovod=False):
    """accumulate_gradient_optimizer.py:13: the wrapped optimiser."""
    return AccumulateGradientOptimizer(orig_optimizer, update_params_frequency, accumulate_sum_or_mean, ema_decay,
                                       use_horovod)
