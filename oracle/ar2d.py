"""Oracle: ConvNetAutoregressive2D forward pass (CPU, torch float64/float32).

Restates machines/conv_net_autoregressive_2D.py:24-74 together with
machines/abstract_machine.py:49-71 (normalisation + combination),
deepar/layers/masking.py:8-19 (down/right shift),
deepar/layers/autoregressive.py:7-22 (log-space normalisation, combination),
deepar/layers/one_hot.py:7-9 (+1 -> index 0, -1 -> index 1),
layers/complex/casting.py:16-24 (channels [0:2] real, [2:4] imaginary) and
deepar/layers/wrappers.py:114-134 (weight normalisation with exponential norm).

Written with torch on the CPU so that autograd gives the reference gradient
for the adjoint-kernel parity tests. Test infrastructure only.
"""
import math

import numpy as np
import torch

CONV_NAMES = ("v", "h", "x", "y", "c")


def num_causal_convs(depth):
    """First causal conv + (depth-2) residual blocks of two + final masked one
    (conv_net_autoregressive_2D.py:68-72)."""
    return 2 * depth - 2


def kernel_shapes(depth, channels):
    """Keras kernel shapes (kh, kw, Cin, Cout) of every conv, in layer order."""
    f = channels
    shapes = {}
    for i in range(num_causal_convs(depth)):
        cin = 1 if i == 0 else f
        shapes[f"cc{i}.v"] = (3, 3, cin, f)       # conv_net_autoregressive_2D.py:38
        shapes[f"cc{i}.h"] = (1, 3, cin, f)       # :39
        shapes[f"cc{i}.x"] = (1, 1, f, f // 2)    # :43
        shapes[f"cc{i}.y"] = (1, 1, f, f // 2)    # :45
        shapes[f"cc{i}.c"] = (3, 3, f, f)         # :50
    shapes["out"] = (1, 1, f, 4)                  # :73 (never weight-normalised)
    return shapes


def effective_kernel(params, name, weights_normalization, exponential_norm=True):
    """Kernel actually used by the conv (wrappers.py:123-134)."""
    v = params[name + ".kernel"]
    if not weights_normalization or name == "out":
        return v
    g = params[name + ".g"]
    if exponential_norm:
        g = torch.exp(g)
    sq = (v * v).sum(dim=(0, 1, 2))
    # tf.nn.l2_normalize: x * rsqrt(max(sum(x^2), 1e-12))
    return v * torch.rsqrt(torch.clamp(sq, min=1e-12)) * g


def _pad(x, top, left, right):
    # x: (B, H, W, C) -> zero padded
    return torch.nn.functional.pad(x, (0, 0, left, right, top, 0))


def _conv_valid(xp, k, b):
    kh, kw = k.shape[0], k.shape[1]
    h = xp.shape[1] - kh + 1
    w = xp.shape[2] - kw + 1
    out = None
    for i in range(kh):
        for j in range(kw):
            term = xp[:, i:i + h, j:j + w, :] @ k[i, j]
            out = term if out is None else out + term
    return out + b


def _down_shift(x):
    return torch.cat([torch.zeros_like(x[:, :1]), x[:, :-1]], dim=1)


def _right_shift(x):
    return torch.cat([torch.zeros_like(x[:, :, :1]), x[:, :, :-1]], dim=2)


def _causal_conv(params, i, v, h, wn, final):
    """conv_net_autoregressive_2D.py:33-51."""
    relu = torch.relu
    kv = effective_kernel(params, f"cc{i}.v", wn)
    kh = effective_kernel(params, f"cc{i}.h", wn)
    kx = effective_kernel(params, f"cc{i}.x", wn)
    ky = effective_kernel(params, f"cc{i}.y", wn)
    kc = effective_kernel(params, f"cc{i}.c", wn)
    vp = _conv_valid(_pad(v, 2, 1, 1), kv, params[f"cc{i}.v.bias"])
    x = relu(_conv_valid(_pad(h, 0, 2, 0), kh, params[f"cc{i}.h.bias"]))
    if final:
        x = _right_shift(x)
    x = _conv_valid(x, kx, params[f"cc{i}.x.bias"])
    y = _down_shift(relu(vp))
    y = _conv_valid(y, ky, params[f"cc{i}.y.bias"])
    cat = torch.cat([relu(x), relu(y)], dim=-1)
    hp = _conv_valid(_pad(cat, 2, 2, 0), kc, params[f"cc{i}.c.bias"])
    return vp, hp


def logits(params, spins, depth, weights_normalization):
    """Unnormalised per-site outputs (B, H, W, 4) (conv_net_autoregressive_2D.py:64-74)."""
    relu = torch.relu
    dtype = params["out.kernel"].dtype
    x = spins.to(dtype).unsqueeze(-1)
    n_cc = num_causal_convs(depth)
    v, h = _causal_conv(params, 0, x, x, weights_normalization, final=False)
    v, h = relu(v), relu(h)
    for b in range(depth - 2):
        v0, h0 = v, h
        v, h = _causal_conv(params, 1 + 2 * b, v, h, weights_normalization, final=False)
        v, h = relu(v), relu(h)
        v, h = _causal_conv(params, 2 + 2 * b, v, h, weights_normalization, final=False)
        v, h = relu(v0 + v), relu(h0 + h)
    _, h = _causal_conv(params, n_cc - 1, v, h, weights_normalization, final=True)
    return _conv_valid(relu(h), params["out.kernel"], params["out.bias"])


def equal_up_down_mask(spins):
    """layers/spins_invariants.py:13-22: outcome k (0: spin +1, 1: spin -1) of
    a site is masked when the number of earlier sites in raster order
    holding outcome k (exclusive cumulative sum) is >= N/2. (B,H,W,2) bool."""
    b = spins.shape[0]
    n = int(np.prod(spins.shape[1:]))
    idx = ((1 - spins.to(torch.int64)) // 2).reshape(b, n)
    onehot = torch.nn.functional.one_hot(idx, 2).to(torch.float64)
    cum = torch.cumsum(onehot, dim=1) - onehot
    return (cum >= n / 2.0).reshape(tuple(spins.shape) + (2,))


def conditional_log_wave_function(params, spins, depth, weights_normalization, equal_up_down=False):
    """(B,H,W,2) real and imaginary parts of the normalised conditionals
    (abstract_machine.py:56-57 with norm_type=2; autoregressive.py:7-15).
    With ``equal_up_down`` the EqualUpDownSpins mask (abstract_machine.py:52-53)
    adds LOG_ZERO (-1e300, -inf in float32) to the masked outcomes' real part
    before the normalisation; -inf is used here."""
    out = logits(params, spins, depth, weights_normalization)
    re, im = out[..., 0:2], out[..., 2:4]
    if equal_up_down:
        re = torch.where(equal_up_down_mask(spins), torch.full_like(re, -math.inf), re)
    re = re - 0.5 * torch.logsumexp(2.0 * re, dim=-1, keepdim=True)
    return re, im


def log_psi(params, spins, depth, weights_normalization, equal_up_down=False):
    """log psi(s) = sum over sites of the conditional picked by the one-hot spin
    (abstract_machine.py:31-46, autoregressive.py:18-22). Returns (re, im)."""
    re, im = conditional_log_wave_function(params, spins, depth, weights_normalization, equal_up_down)
    idx = ((1 - spins.to(torch.int64)) // 2).unsqueeze(-1)
    re_s = torch.gather(re, -1, idx).squeeze(-1)
    im_s = torch.gather(im, -1, idx).squeeze(-1)
    return re_s.sum(dim=(1, 2)), im_s.sum(dim=(1, 2))


def init_params(hilbert_state_shape, depth, channels, weights_normalization, seed=0,
                dtype=torch.float32):
    """Seeded Glorot-uniform kernels, zero biases; g = log(||v|| + 1e-10)
    (keras Conv2D defaults; wrappers.py:26-39). The same initialiser is used by
    the product's machine so that both sides start from identical weights."""
    gen = torch.Generator().manual_seed(seed)
    params = {}
    for name, shape in kernel_shapes(depth, channels).items():
        kh, kw, cin, cout = shape
        fan_in, fan_out = kh * kw * cin, kh * kw * cout
        limit = math.sqrt(6.0 / (fan_in + fan_out))
        k = (torch.rand(shape, generator=gen, dtype=torch.float64) * 2 - 1) * limit
        params[name + ".kernel"] = k.to(dtype)
        params[name + ".bias"] = torch.zeros(cout, dtype=dtype)
        if weights_normalization and name != "out":
            norm = torch.sqrt((k * k).sum(dim=(0, 1, 2)))
            params[name + ".g"] = torch.log(norm + 1e-10).to(dtype)
    return params


def params_to(params, dtype):
    return {k: v.detach().to(dtype).clone() for k, v in params.items()}


def log_psi_numpy(params, spins, depth, weights_normalization, dtype=torch.float64, equal_up_down=False):
    p = params_to(params, dtype)
    with torch.no_grad():
        re, im = log_psi(p, torch.as_tensor(np.asarray(spins)), depth, weights_normalization, equal_up_down)
    return re.numpy() + 1j * im.numpy()


def weighted_gradient(params, spins, depth, weights_normalization, w_re, w_im,
                      dtype=torch.float64, equal_up_down=False):
    """d/dtheta sum_s (w_re[s] Re log psi(s) + w_im[s] Im log psi(s)) by autograd.
    This is the loss gradient of optimization/loss.py:4-5 when
    w = 2 Re(y)/B, -2 Im(y)/B, and the per-sample O_k rows when w is one-hot."""
    p = {k: v.detach().to(dtype).clone().requires_grad_(True) for k, v in params.items()}
    re, im = log_psi(p, torch.as_tensor(np.asarray(spins)), depth, weights_normalization, equal_up_down)
    loss = (torch.as_tensor(w_re, dtype=dtype) * re).sum() + (torch.as_tensor(w_im, dtype=dtype) * im).sum()
    loss.backward()
    return {k: v.grad.detach() for k, v in p.items()}
