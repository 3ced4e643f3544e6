"""Gradient accumulation / EMA (optimizers/accumulate_gradient_optimizer.py:13-88)
against the oracle's restatement, which is pinned to the reference's test
numbers, and checkpoint-resume of parameters and optimiser state (host)."""
import numpy as np
import pytest
import torch

from oracle import sr


class _Machine:
    def __init__(self, w0):
        self.params = torch.tensor([float(w0)], dtype=torch.float64)
        self.layout = [("w", (1,), 0)]
        self.updates = 0

    def params_updated(self):
        self.updates += 1


class _SGD:
    def __init__(self, machine, lr):
        self.machine, self.lr = machine, lr
        self.iterations = 0

    def apply_gradient(self, grad):
        self.iterations += 1
        self.machine.params.sub_(self.lr * grad)
        self.machine.params_updated()

    def state_dict(self):
        return {"iterations": self.iterations}

    def load_state_dict(self, state):
        self.iterations = int(state["iterations"])


@pytest.mark.parametrize("every,mean,ema", [(2, True, None), (1, True, None), (1, True, 0.9), (2, True, 0.9),
                                            (3, False, 0.5), (2, False, None)])
def test_accumulation_matches_oracle(every, mean, ema):
    from flowket_gb300.optimizers import convert_to_accumulate_gradient_optimizer
    grads = [2.0, 3.0, -1.0, 0.5, 4.0, 1.5]
    want_hist, want_ema = sr.accumulate_gradient_sgd(1.0, grads, 1.0, every, mean=mean, ema_decay=ema)
    m = _Machine(1.0)
    opt = convert_to_accumulate_gradient_optimizer(_SGD(m, 1.0), every, accumulate_sum_or_mean=not mean,
                                                   ema_decay=ema or 0)
    hist = []
    for g in grads:
        opt.apply_gradient(torch.tensor([g], dtype=torch.float64))
        hist.append(float(m.params[0]))
    np.testing.assert_allclose(hist, want_hist, rtol=1e-12, atol=1e-12)
    if ema is not None:
        opt.set_weights_ema()
        assert float(m.params[0]) == pytest.approx(want_ema, rel=1e-12)


def test_accumulation_rejects_bad_arguments():
    from flowket_gb300.optimizers import convert_to_accumulate_gradient_optimizer
    with pytest.raises(ValueError):
        convert_to_accumulate_gradient_optimizer(_SGD(_Machine(0.0), 1.0), 0)
    with pytest.raises(ValueError):
        convert_to_accumulate_gradient_optimizer(_SGD(_Machine(0.0), 1.0), 2, use_horovod=True)


def test_checkpoint_resume_continues_identically(tmp_path):
    from flowket_gb300.checkpoint import CheckpointByTime, load_optimizer_weights, load_weights
    from flowket_gb300.optimizers import convert_to_accumulate_gradient_optimizer
    grads = [torch.tensor([g], dtype=torch.float64) for g in (2.0, 3.0, -1.0, 0.5, 4.0, 1.5, -2.0)]
    m = _Machine(1.0)
    opt = convert_to_accumulate_gradient_optimizer(_SGD(m, 0.5), 2, ema_decay=0.9)
    for g in grads[:3]:
        opt.apply_gradient(g)
    cb = CheckpointByTime(m, opt, str(tmp_path / "ckpt_{tag}"), save_frequency_in_minutes=0)
    cb.on_epoch_begin(4)
    cb.on_batch_end(17, logs={"tag": "a"})
    for g in grads[3:]:
        opt.apply_gradient(g)
    want = float(m.params[0])
    m2 = _Machine(-5.0)
    opt2 = convert_to_accumulate_gradient_optimizer(_SGD(m2, 0.5), 2, ema_decay=0.9)
    load_weights(m2, str(tmp_path / "ckpt_a"))
    assert load_optimizer_weights(opt2, str(tmp_path / "ckpt_a")) == (4, 17)
    for g in grads[3:]:
        opt2.apply_gradient(g)
    assert float(m2.params[0]) == want
    assert load_optimizer_weights(opt2, str(tmp_path / "missing")) is None
    bad = _Machine(0.0)
    bad.params = torch.zeros(2, dtype=torch.float64)
    bad.layout = [("w", (2,), 0)]
    with pytest.raises(ValueError):
        load_weights(bad, str(tmp_path / "ckpt_a"))
