"""Optimiser kernels against the oracle's restatement of tf.keras Adam (TF 1.x:
lr_t = lr sqrt(1 - b2^t) / (1 - b1^t), epsilon = K.epsilon() = 1e-7), the
optimiser of the reference's examples and experiments/train.py:52, over
several steps with both beta_2 settings the reference uses."""
import numpy as np
import pytest
import torch

from oracle import sr as ref_sr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("beta_2", [0.999, 0.9])
def test_adam_step_matches_keras_adam(cuda, beta_2):
    from flowket_gb300 import _lib
    rng = np.random.default_rng(4)
    n = 10_000
    p0 = rng.normal(size=n).astype(np.float32)
    params = torch.as_tensor(p0).cuda()
    m = torch.zeros_like(params)
    v = torch.zeros_like(params)
    state = {}
    want = {"w": p0.astype(np.float64)}
    for t in range(1, 8):
        g = (rng.normal(size=n) * (0.1 * t)).astype(np.float32)
        _lib.call("fk_adam_step", _lib.ptr(params), _lib.ptr(torch.as_tensor(g).cuda()), _lib.ptr(m), _lib.ptr(v), n,
                  t, 1e-3, 0.9, beta_2, 1e-7, _lib.stream_ptr())
        want = ref_sr.keras_adam(want, {"w": g.astype(np.float64)}, state, lr=1e-3, beta_1=0.9, beta_2=beta_2,
                                 epsilon=1e-7)
        got = params.cpu().numpy().astype(np.float64)
        step = np.abs(want["w"] - p0)
        assert np.abs(got - want["w"]).max() <= 1e-6 * max(1.0, step.max()) + 1e-7, t


def test_adam_optimizer_class_matches_keras_adam(cuda):
    """optimizers.Adam over a machine's flat parameters (the driver's update)."""
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.optimizers import Adam
    mach = ConvNetAutoregressive2D((4, 4), 2, 16, weights_normalization=True, precision="fp32", seed=0)
    p0 = mach.params.cpu().numpy().astype(np.float64)
    opt = Adam(mach, lr=3e-3)
    rng = np.random.default_rng(8)
    state, want = {}, {"w": p0}
    for _ in range(5):
        g = rng.normal(size=p0.shape).astype(np.float32)
        opt.apply_gradient(torch.as_tensor(g).cuda())
        want = ref_sr.keras_adam(want, {"w": g.astype(np.float64)}, state, lr=3e-3)
    got = mach.params.cpu().numpy().astype(np.float64)
    assert np.abs(got - want["w"]).max() < 2e-6
    assert opt.iterations == 5
