"""Wave-function machines (flowket.machines drop-ins) over the CUDA library.

``ConvNetAutoregressive2D`` mirrors machines/conv_net_autoregressive_2D.py:8-78
(the PixelCNN-style causal conv net with vertical/horizontal streams, weight
normalisation with exponential norm, auto-normalised conditionals of
machines/abstract_machine.py:49-71). ``RBM`` mirrors machines/rbm.py:35-48 and
``RBMSym`` machines/rbm.py:51-65.

Parameters live in one flat FP32 CUDA tensor in Keras layer order; every
evaluation calls the library (no CPU fallback).
"""
import math

import numpy as np
import torch

from . import _lib


def _device(device):
    if device is None:
        device = torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else None
    if device is None:
        raise _lib.FlowketError("flowket_gb300 machines need a CUDA device")
    return torch.device(device)


def ar2d_param_layout(depth, channels, weights_normalization):
    """(name, shape, offset) of every parameter in the flat vector, matching
    the library's layout: per causal conv i and conv in (v, h, x, y, c):
    kernel (kh, kw, cin, cout), bias, [g]; then out.kernel, out.bias."""
    f = channels
    out = []
    off = 0

    def add(name, shape):
        nonlocal off
        out.append((name, shape, off))
        off += int(np.prod(shape))

    for i in range(2 * depth - 2):
        cin = 1 if i == 0 else f
        for conv, shape in (("v", (3, 3, cin, f)), ("h", (1, 3, cin, f)), ("x", (1, 1, f, f // 2)),
                            ("y", (1, 1, f, f // 2)), ("c", (3, 3, f, f))):
            add(f"cc{i}.{conv}.kernel", shape)
            add(f"cc{i}.{conv}.bias", (shape[-1],))
            if weights_normalization:
                add(f"cc{i}.{conv}.g", (shape[-1],))
    add("out.kernel", (1, 1, f, 4))
    add("out.bias", (4,))
    return out, off


def glorot_uniform_init(layout, seed, weights_normalization):
    """Seeded Glorot-uniform kernels (limit sqrt(6/(fan_in+fan_out)), keras
    Conv2D default), zero biases, g = log(||v|| + 1e-10) (deepar/layers/wrappers.py:26-39)."""
    gen = torch.Generator().manual_seed(seed)
    flat = {}
    for name, shape, _ in layout:
        if name.endswith(".kernel"):
            kh, kw, cin, cout = shape
            limit = math.sqrt(6.0 / (kh * kw * cin + kh * kw * cout))
            k = (torch.rand(shape, generator=gen, dtype=torch.float64) * 2 - 1) * limit
            flat[name] = k
            base = name[:-len(".kernel")]
            flat[base + ".bias"] = torch.zeros(cout, dtype=torch.float64)
            if weights_normalization and base != "out":
                flat[base + ".g"] = torch.log(torch.sqrt((k * k).sum(dim=(0, 1, 2))) + 1e-10)
    return flat


class ConvNetAutoregressive2D:
    """flowket.machines.ConvNetAutoregressive2D on GB300.

    ``hilbert_state_shape`` replaces the Keras input layer (H, W).
    ``precision`` selects the tcgen05 tensor-core path with BF16 operands
    ('bf16') or FP16 operands ('fp16'; the same kernels and speed, 10
    instead of 7 mantissa bits in every stored activation, so the log psi
    ratios of the local energy carry about 8x less rounding noise), or the
    plain FP32 CUDA-core path ('fp32')."""

    def __init__(self, hilbert_state_shape, depth, num_of_channels, kernel_size=3, weights_normalization=True,
                 exponential_norm=True, precision="bf16", seed=0, device=None, params=None,
                 equal_up_down_spins=False):
        if kernel_size != 3 or not exponential_norm:
            raise ValueError("only kernel_size=3 with exponential_norm=True (the reference defaults) is supported")
        shape = tuple(int(x) for x in hilbert_state_shape)
        if len(shape) != 2:
            raise ValueError("ConvNetAutoregressive2D needs a 2D hilbert_state_shape (use (1, L) for a chain)")
        self.hilbert_state_shape = shape
        self.depth = int(depth)
        self.num_of_channels = int(num_of_channels)
        self.weights_normalization = bool(weights_normalization)
        self.precision = precision
        self.device = _device(device)
        self.equal_up_down_spins = bool(equal_up_down_spins)
        if precision not in _lib.PRECISIONS:
            raise ValueError("precision must be one of %s" % sorted(_lib.PRECISIONS))
        self.desc = _lib.Ar2dDesc(shape[0], shape[1], self.depth, self.num_of_channels,
                                  1 if self.weights_normalization else 0, _lib.PRECISIONS[precision],
                                  1 if self.equal_up_down_spins else 0)
        lib = _lib.load()
        self.layout, n = ar2d_param_layout(self.depth, self.num_of_channels, self.weights_normalization)
        n_lib = lib.fk_ar2d_num_params(ctypes_ref(self.desc))
        if n_lib < 0:
            _lib.check(-1, "ConvNetAutoregressive2D")
        assert n_lib == n, (n_lib, n)
        self.num_params = n
        if params is None:
            init = glorot_uniform_init(self.layout, seed, self.weights_normalization)
            flat = torch.cat([init[name].reshape(-1) for name, _, _ in self.layout]).to(torch.float32)
        else:
            flat = torch.as_tensor(params, dtype=torch.float32).reshape(-1)
            assert flat.numel() == n
        self.params = flat.to(self.device).contiguous()
        self._packed = torch.empty(lib.fk_ar2d_packed_bytes(ctypes_ref(self.desc)), dtype=torch.uint8,
                                   device=self.device)
        self._packed_version = None
        self._manual_version = 0
        self._ws = {}

    # ------------------------------------------------------------------ params
    def named_params(self):
        return {name: self.params[off:off + int(np.prod(shape))].view(shape) for name, shape, off in self.layout}

    def params_dict_cpu(self, dtype=torch.float64):
        return {k: v.detach().cpu().to(dtype).clone() for k, v in self.named_params().items()}

    def count_params(self):
        return self.num_params

    def load_weights(self, filepath):
        """Keras ``model.load_weights`` of a weight file saved by the reference's
        ConvNetAutoregressive2D (HDF5, see flowket_gb300.h5weights)."""
        from .h5weights import load_conv_net_autoregressive_2d
        return load_conv_net_autoregressive_2d(self, filepath)

    def params_updated(self):
        """Call after writing `params` through a raw pointer (the optimisers do)."""
        self._manual_version += 1

    def packed(self):
        """Weight-normalised, operand-layout weights (repacked after updates)."""
        ver = (self.params._version, self._manual_version)
        if self._packed_version != ver:
            _lib.call("fk_ar2d_pack", ctypes_ref(self.desc), _lib.ptr(self.params), _lib.ptr(self._packed),
                      _lib.stream_ptr())
            self._packed_version = ver
        return self._packed

    def workspace(self, batch, mode):
        key = (mode, batch)
        ws = self._ws.get(key)
        if ws is None:
            nbytes = _lib.load().fk_ar2d_workspace_bytes(ctypes_ref(self.desc), batch, mode)
            if nbytes < 0:
                _lib.check(-1, "fk_ar2d_workspace_bytes")
            ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            if len(self._ws) > 8:
                self._ws.clear()
            self._ws[key] = ws
        return ws

    # ------------------------------------------------------------------ evaluation
    def _spins(self, spins):
        s = torch.as_tensor(spins)
        if s.device != self.device or s.dtype != torch.int8:
            s = s.to(device=self.device, dtype=torch.int8)
        return s.reshape(s.shape[0], self.hilbert_state_shape[0] * self.hilbert_state_shape[1]).contiguous()

    def forward(self, spins, mode=_lib.FK_AR2D_INFER, with_cond=False, workspace=None):
        """Returns (log_psi float32 (B, 2) (re, im), cond (B, N, 4) or None, workspace)."""
        s = self._spins(spins)
        b = s.shape[0]
        lp = torch.empty((b, 2), dtype=torch.float32, device=self.device)
        cond = torch.empty((b, s.shape[1], 4), dtype=torch.float32, device=self.device) if with_cond else None
        ws = workspace if workspace is not None else self.workspace(b, mode)
        _lib.call("fk_ar2d_forward", ctypes_ref(self.desc), _lib.ptr(self.packed()), _lib.ptr(s), b,
                  _lib.ptr(lp), _lib.ptr(cond), _lib.ptr(ws), ws.numel(), mode, _lib.stream_ptr())
        return lp, cond, ws

    def log_psi(self, spins, chunk=1 << 16):
        """Complex log psi (B,) (machines/abstract_machine.py:31-46)."""
        s = self._spins(spins)
        outs = []
        for i in range(0, s.shape[0], chunk):
            lp, _, _ = self.forward(s[i:i + chunk])
            outs.append(torch.complex(lp[:, 0], lp[:, 1]))
        return torch.cat(outs) if outs else torch.empty(0, dtype=torch.complex64, device=self.device)

    def predict(self, spins, batch_size=None):
        """Keras model.predict drop-in: (B, 1) complex64."""
        return self.log_psi(spins, chunk=batch_size or (1 << 16)).unsqueeze(1)

    __call__ = predict

    def conditional_log_wave_function(self, spins):
        """(B, H, W, 2) complex normalised conditionals (abstract_machine.py:56-57)."""
        _, cond, _ = self.forward(spins, with_cond=True)
        h, w = self.hilbert_state_shape
        c = cond.view(-1, h, w, 4)
        return torch.complex(c[..., 0:2], c[..., 2:4])

    def conditional_log_probs(self, spins):
        """(B, H, W, 2) log-probabilities 2 Re cond (abstract_machine.py:56-57)."""
        _, cond, _ = self.forward(spins, with_cond=True)
        h, w = self.hilbert_state_shape
        return 2.0 * cond.view(-1, h, w, 4)[..., 0:2]


def ctypes_ref(struct):
    import ctypes
    return ctypes.byref(struct)


def _ar2d_backward(machine, spins, seeds, saved, per_sample=False):
    """Adjoint of sum_b (w_re Re log psi_b + w_im Im log psi_b): flat gradient
    (num_params,) or per-sample rows O (num_params, B) (param-major)."""
    s = machine._spins(spins)
    b = s.shape[0]
    w = torch.as_tensor(seeds, dtype=torch.float32, device=machine.device).reshape(b, 2).contiguous()
    lib = _lib.load()
    nbytes = lib.fk_ar2d_backward_workspace_bytes(ctypes_ref(machine.desc), b)
    key = ("bwd", b)
    ws = machine._ws.get(key)
    if ws is None or ws.numel() < nbytes:
        ws = torch.empty(nbytes, dtype=torch.uint8, device=machine.device)
        machine._ws[key] = ws
    if per_sample:
        out = torch.empty((machine.num_params, b), dtype=torch.float32, device=machine.device)
        grad_p, ps_p = None, _lib.ptr(out)
    else:
        out = torch.empty(machine.num_params, dtype=torch.float32, device=machine.device)
        grad_p, ps_p = _lib.ptr(out), None
    _lib.call("fk_ar2d_backward", ctypes_ref(machine.desc), _lib.ptr(machine.packed()), _lib.ptr(machine.params),
              _lib.ptr(s), b, _lib.ptr(w), _lib.ptr(saved), saved.numel(), _lib.ptr(ws), ws.numel(), grad_p, ps_p,
              _lib.stream_ptr())
    return out


ConvNetAutoregressive2D.backward = _ar2d_backward


class Ar2dLogPsi(torch.autograd.Function):
    """log psi of ConvNetAutoregressive2D as a differentiable torch op: the
    forward kernels produce (B, 2) = (Re, Im) log psi, the hand-written
    adjoint (fk_ar2d_backward) maps the incoming gradient (B, 2) to the
    gradient of the flat parameter vector (the role of the reference's
    Keras gradient through the model, optimization/loss.py:4-5, and of
    machines/abstract_machine.py:24-28's jacobian hook for the summed case).

    With ``recompute_chunk`` = c the forward keeps no activations: the adjoint
    re-runs the forward over c samples at a time (FK_AR2D_SAVE into a
    c-sample workspace) and accumulates the chunks' gradients, so the memory
    held between forward and backward is the log psi alone and the adjoint's
    workspace is bounded by c samples instead of B."""

    @staticmethod
    def forward(ctx, params, machine, spins, recompute_chunk):
        if recompute_chunk:
            lp, _, _ = machine.forward(spins, mode=_lib.FK_AR2D_INFER)
            ctx.saved_ws = None
        else:
            # a private workspace (the machine's cached one is reused by the
            # next forward of the same batch size)
            nbytes = _lib.load().fk_ar2d_workspace_bytes(ctypes_ref(machine.desc), spins.shape[0],
                                                         _lib.FK_AR2D_SAVE)
            ws = torch.empty(nbytes, dtype=torch.uint8, device=machine.device)
            lp, _, _ = machine.forward(spins, mode=_lib.FK_AR2D_SAVE, workspace=ws)
            ctx.saved_ws = ws
        ctx.machine = machine
        ctx.chunk = recompute_chunk
        ctx.save_for_backward(spins)
        return lp.clone()

    @staticmethod
    def backward(ctx, grad_lp):
        (spins,) = ctx.saved_tensors
        m = ctx.machine
        g = grad_lp.to(torch.float32).contiguous()
        if ctx.saved_ws is not None:
            grad = m.backward(spins, g, ctx.saved_ws)
        else:
            grad = torch.zeros(m.num_params, dtype=torch.float32, device=m.device)
            for i in range(0, spins.shape[0], ctx.chunk):
                x = spins[i:i + ctx.chunk]
                _, _, ws = m.forward(x, mode=_lib.FK_AR2D_SAVE)
                grad.add_(m.backward(x, g[i:i + ctx.chunk], ws))
        return grad, None, None, None


def _ar2d_log_psi_autograd(machine, spins, params=None, recompute_chunk=None):
    """Differentiable log psi (B, 2) (Re, Im) through Ar2dLogPsi. `params`
    defaults to ``machine.params`` (set ``requires_grad`` on it, or pass a
    leaf tensor that aliases it)."""
    s = machine._spins(spins)
    p = machine.params if params is None else params
    return Ar2dLogPsi.apply(p, machine, s, recompute_chunk)


ConvNetAutoregressive2D.log_psi_autograd = _ar2d_log_psi_autograd


def _ar2d_backward_recompute(machine, spins, seeds, chunk=1024):
    """Summed adjoint without stored activations: the forward is re-run in
    chunks of `chunk` samples (activation recomputation for lattices whose
    full-batch activations would not fit next to the rest of the step)."""
    s = machine._spins(spins)
    w = torch.as_tensor(seeds, dtype=torch.float32, device=machine.device).reshape(s.shape[0], 2).contiguous()
    grad = torch.zeros(machine.num_params, dtype=torch.float32, device=machine.device)
    for i in range(0, s.shape[0], chunk):
        x = s[i:i + chunk]
        _, _, ws = machine.forward(x, mode=_lib.FK_AR2D_SAVE)
        grad.add_(machine.backward(x, w[i:i + chunk], ws))
    return grad


ConvNetAutoregressive2D.backward_recompute = _ar2d_backward_recompute


def _ar2d_log_derivatives(machine, spins, saved=None):
    """Per-sample complex O_k = d log psi / d theta_k (num_params, B) complex64
    (the reference's predictions_jacobian, machines/abstract_machine.py:24-28)."""
    s = machine._spins(spins)
    if saved is None:
        _, _, saved = machine.forward(s, mode=_lib.FK_AR2D_SAVE)
    b = s.shape[0]
    ones = torch.zeros((b, 2), dtype=torch.float32, device=machine.device)
    ones[:, 0] = 1
    o_re = machine.backward(s, ones, saved, per_sample=True)
    ones[:, 0] = 0
    ones[:, 1] = 1
    o_im = machine.backward(s, ones, saved, per_sample=True)
    return torch.complex(o_re, o_im)


ConvNetAutoregressive2D.log_derivatives = _ar2d_log_derivatives


class RBM:
    """flowket.machines.RBM (machines/rbm.py:35-48): complex RBM with alpha*N
    hidden units, log psi = a.s + sum_j lncosh(b_j + W_j.s). Parameters are
    one float32 tensor of interleaved complex values [a | b | W]; real and
    imaginary parts are initialised N(0, stddev) (rbm.py:23).

    The machine protocol of the driver: ``forward`` (log psi), ``backward``
    (the loss gradient with respect to the stored (re, im) pairs),
    ``log_derivatives_split`` (per-sample complex O for SR) and
    ``local_energy`` (E_loc from the operator's enumeration, ratios from
    incremental theta updates)."""

    is_complex = True

    def __init__(self, hilbert_state_shape, alpha=1, stddev=1.0, use_float64_ops=False, seed=0, device=None,
                 params=None):
        if use_float64_ops:
            raise ValueError("the GPU RBM computes in complex64 (use_float64_ops=False)")
        self.hilbert_state_shape = tuple(int(x) for x in hilbert_state_shape)
        self.n = int(np.prod(self.hilbert_state_shape))
        self.m = int(alpha) * self.n
        self.alpha = int(alpha)
        self.device = _device(device)
        self.num_complex_params = self.n + self.m + self.n * self.m
        if params is None:
            gen = torch.Generator().manual_seed(seed)
            params = torch.randn(2 * self.num_complex_params, generator=gen, dtype=torch.float64) * stddev
        self.params = torch.as_tensor(params, dtype=torch.float32).reshape(-1).to(self.device).contiguous()
        assert self.params.numel() == 2 * self.num_complex_params
        self.num_params = self.params.numel()

    def params_updated(self):
        pass

    def count_params(self):
        return self.num_params

    def kernel_params(self):
        """The dense [a | b | W] parameters the RBM kernels read."""
        return self.params

    def complex_params(self):
        c = torch.view_as_complex(self.kernel_params().view(-1, 2))
        n, m = self.n, self.m
        return {"a": c[:n], "b": c[n:n + m], "W": c[n + m:].view(n, m)}

    def _spins(self, spins):
        s = torch.as_tensor(spins)
        if s.device != self.device or s.dtype != torch.int8:
            s = s.to(device=self.device, dtype=torch.int8)
        return s.reshape(s.shape[0], self.n).contiguous()

    def log_psi_pairs(self, spins):
        s = self._spins(spins)
        out = torch.empty((s.shape[0], 2), dtype=torch.float32, device=self.device)
        _lib.call("fk_rbm_log_psi", _lib.ptr(self.kernel_params()), self.n, self.m, _lib.ptr(s), s.shape[0],
                  _lib.ptr(out), _lib.stream_ptr())
        return out

    def forward(self, spins, mode=_lib.FK_AR2D_INFER, with_cond=False, workspace=None):
        """(log_psi float32 (B, 2) (re, im), None, None): the RBM keeps no
        activations (the adjoint recomputes theta)."""
        if with_cond:
            raise ValueError("an RBM has no autoregressive conditionals")
        return self.log_psi_pairs(spins), None, None

    def log_psi(self, spins):
        lp = self.log_psi_pairs(spins)
        return torch.complex(lp[:, 0], lp[:, 1])

    def predict(self, spins, batch_size=None):
        return self.log_psi(spins).unsqueeze(1)

    __call__ = predict

    def local_energy(self, operator, spins):
        flips, mel, use, s = operator.enumerate(spins)
        local = torch.empty((s.shape[0], 2), dtype=torch.float64, device=self.device)
        _lib.call("fk_rbm_local_energy", _lib.ptr(self.kernel_params()), self.n, self.m, _lib.ptr(s), s.shape[0],
                  _lib.ptr(flips), _lib.ptr(mel), _lib.ptr(use), mel.shape[0], _lib.ptr(local), _lib.stream_ptr())
        return local

    def _dense_log_derivatives(self, s):
        b = s.shape[0]
        o_re = torch.empty((self.n + self.m + self.n * self.m, b), dtype=torch.float32, device=self.device)
        o_im = torch.empty_like(o_re)
        _lib.call("fk_rbm_log_derivatives", _lib.ptr(self.kernel_params()), self.n, self.m, _lib.ptr(s), b,
                  _lib.ptr(o_re), _lib.ptr(o_im), _lib.stream_ptr())
        return o_re, o_im

    def log_derivatives_split(self, spins):
        """(O_re, O_im) parameter-major (num_complex_params, B): O_k = d log psi / d theta_k
        (holomorphic) for the trainable complex parameters."""
        return self._dense_log_derivatives(self._spins(spins))

    def log_derivatives(self, spins):
        o_re, o_im = self.log_derivatives_split(spins)
        return torch.complex(o_re, o_im)

    def backward(self, spins, seeds, saved=None, per_sample=False):
        """Gradient of sum_b (w_re Re log psi_b + w_im Im log psi_b) with respect
        to the stored (re, im) parameter pairs (num_params,) float32."""
        if per_sample:
            raise ValueError("RBM: per-sample rows are log_derivatives_split (complex O)")
        s = self._spins(spins)
        b = s.shape[0]
        w = torch.as_tensor(seeds, dtype=torch.float32, device=self.device).reshape(b, 2).contiguous()
        o_re, o_im = self.log_derivatives_split(s)
        grad = torch.empty(self.num_params, dtype=torch.float32, device=self.device)
        _lib.call("fk_complex_param_gradient", _lib.ptr(o_re), _lib.ptr(o_im), self.num_params // 2, b, _lib.ptr(w),
                  _lib.ptr(grad), _lib.stream_ptr())
        return grad


def rbm_sym_tied_index(shape, alpha):
    """Index map dense -> bare of RBMSym (machines/rbm.py:51-65 with
    layers/complex/dense.py:53-85): bare = [a (1) | b (alpha) | W (shape + (alpha,))];
    dense = [a (N) | b (alpha*N) | W (N x alpha*N)], kernel column u*T + t the
    bare kernel rolled by translation t (itertools order over the lattice),
    bias u*N + t = bare bias u, every visible bias = the single bare a
    (Flatten -> sum -> ComplexDense(1) in rbm.py:59-62)."""
    import itertools
    n = int(np.prod(shape))
    dims = tuple(range(len(shape)))
    w_idx = torch.arange(n * alpha, dtype=torch.int64).reshape(tuple(shape) + (alpha,))
    trans = [torch.roll(w_idx, t, dims) for t in itertools.product(*[range(d) for d in shape])]
    w_map = torch.stack(trans, dim=-1).reshape(n, alpha * len(trans)) + 1 + alpha
    b_map = torch.arange(alpha, dtype=torch.int64).repeat_interleave(n) + 1
    a_map = torch.zeros(n, dtype=torch.int64)
    return torch.cat([a_map, b_map, w_map.reshape(-1)])


class RBMSym(RBM):
    """flowket.machines.RBMSym (machines/rbm.py:51-65): translation-invariant
    kernel (shape + (alpha,)), one hidden bias per feature and a single
    visible bias. The trainable ``params`` are the bare complex values
    [a (1) | b (alpha) | W (shape + (alpha,))] interleaved (re, im); the
    kernels evaluate the dense RBM, expanded from them on the device
    (fk_gather_complex) whenever they change, and the per-sample O of a bare
    parameter is the sum of its dense copies' (fk_segment_sum_rows)."""

    def __init__(self, hilbert_state_shape, alpha=1, stddev=1.0, use_float64_ops=False, seed=0, device=None,
                 params=None):
        if use_float64_ops:
            raise ValueError("the GPU RBM computes in complex64 (use_float64_ops=False)")
        shape = tuple(int(x) for x in hilbert_state_shape)
        self.hilbert_state_shape = shape
        self.n = int(np.prod(shape))
        self.alpha = int(alpha)
        self.m = self.alpha * self.n
        self.device = _device(device)
        n_bare = 1 + self.alpha + self.n * self.alpha
        if params is None:
            gen = torch.Generator().manual_seed(seed)
            bare_w = torch.complex(torch.randn(shape + (alpha,), generator=gen, dtype=torch.float64) * stddev,
                                   torch.randn(shape + (alpha,), generator=gen, dtype=torch.float64) * stddev)
            bare_b = torch.complex(torch.randn(alpha, generator=gen, dtype=torch.float64) * stddev,
                                   torch.randn(alpha, generator=gen, dtype=torch.float64) * stddev)
            bare_a = torch.complex(torch.randn(1, generator=gen, dtype=torch.float64) * stddev,
                                   torch.randn(1, generator=gen, dtype=torch.float64) * stddev)
            params = torch.view_as_real(torch.cat([bare_a, bare_b, bare_w.reshape(-1)])).reshape(-1)
        self.params = torch.as_tensor(params, dtype=torch.float32).reshape(-1).to(self.device).contiguous()
        assert self.params.numel() == 2 * n_bare
        self.num_complex_params = n_bare
        self.num_params = 2 * n_bare
        self.num_dense_complex_params = self.n + self.m + self.n * self.m
        tied = rbm_sym_tied_index(shape, self.alpha)
        self._tied = tied.to(torch.int32).to(self.device)
        order = torch.argsort(tied, stable=True)
        counts = torch.bincount(tied, minlength=n_bare)
        offsets = torch.zeros(n_bare + 1, dtype=torch.int64)
        offsets[1:] = torch.cumsum(counts, 0)
        self._seg_rows = order.to(torch.int32).to(self.device)
        self._seg_offsets = offsets.to(self.device)
        self._dense = torch.empty(2 * self.num_dense_complex_params, dtype=torch.float32, device=self.device)
        self._dense_version = None
        self._manual_version = 0

    @property
    def bare(self):
        c = torch.view_as_complex(self.params.view(-1, 2)).detach().cpu().to(torch.complex128)
        al = self.alpha
        return {"a": c[:1], "b": c[1:1 + al], "W": c[1 + al:].view(self.hilbert_state_shape + (al,))}

    def params_updated(self):
        self._manual_version += 1

    def kernel_params(self):
        ver = (self.params._version, self._manual_version)
        if self._dense_version != ver:
            _lib.call("fk_gather_complex", _lib.ptr(self.params), _lib.ptr(self._tied), self.num_dense_complex_params,
                      _lib.ptr(self._dense), _lib.stream_ptr())
            self._dense_version = ver
        return self._dense

    def log_derivatives_split(self, spins):
        s = self._spins(spins)
        d_re, d_im = self._dense_log_derivatives(s)
        b = s.shape[0]
        o_re = torch.empty((self.num_complex_params, b), dtype=torch.float32, device=self.device)
        o_im = torch.empty_like(o_re)
        st = _lib.stream_ptr()
        for src, dst in ((d_re, o_re), (d_im, o_im)):
            _lib.call("fk_segment_sum_rows", _lib.ptr(src), _lib.ptr(self._seg_offsets), _lib.ptr(self._seg_rows),
                      self.num_complex_params, b, _lib.ptr(dst), st)
        return o_re, o_im


def _ar2d_forward_connections(machine, configs, owner, cflips, n_rows, base_saved, base_batch, chunk=1 << 17):
    """log psi (n_rows, 2) of connected configurations with causal reuse of the
    base samples' saved activations (fk_ar2d_forward_connections)."""
    lib = _lib.load()
    max_rows = configs.shape[0]
    chunk = min(chunk, ((n_rows + 127) // 128) * 128) if n_rows else 128
    nbytes = lib.fk_ar2d_connections_workspace_bytes(ctypes_ref(machine.desc), max_rows, chunk)
    key = ("conn", max_rows, chunk)
    ws = machine._ws.get(key)
    if ws is None:
        ws = torch.empty(nbytes, dtype=torch.uint8, device=machine.device)
        machine._ws[key] = ws
    out = torch.empty((max(n_rows, 1), 2), dtype=torch.float32, device=machine.device)
    _lib.call("fk_ar2d_forward_connections", ctypes_ref(machine.desc), _lib.ptr(machine.packed()), _lib.ptr(configs),
              _lib.ptr(owner), _lib.ptr(cflips), n_rows, _lib.ptr(base_saved), base_saved.numel(), base_batch,
              _lib.ptr(out), _lib.ptr(ws), ws.numel(), chunk, _lib.stream_ptr())
    return out


ConvNetAutoregressive2D.forward_connections = _ar2d_forward_connections
