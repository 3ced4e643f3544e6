"""Failure detection without a GPU fault: a bounded device wait that runs out
(an mbarrier that nothing arrives at) sets FK_STATUS_TIMEOUT and returns, the
host raises at the end of the step, and the context stays usable; non-finite
weights injected on the host surface as NonFiniteError (the reference raises
on a non-finite wave function, samplers/metropolis_hastings.py:103-105)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ar_problem(precision="bf16"):
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.operators import Ising
    from flowket_gb300.optimization import VariationalMonteCarlo
    from flowket_gb300.optimizers import Adam
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape = (4, 4)
    m = ConvNetAutoregressive2D(shape, 3, 16, weights_normalization=True, precision=precision, seed=0)
    vmc = VariationalMonteCarlo(m, Ising(h=3.0, hilbert_state_shape=shape, pbc=True),
                                FastAutoregressiveSampler(m, 256, seed=1))
    return m, vmc, Adam(m, lr=1e-3)


def test_bounded_wait_times_out_and_reports(cuda):
    from flowket_gb300 import _lib
    _lib.check_device()
    _lib.call("fk_selftest_wait_timeout", 4096, _lib.stream_ptr())
    st = _lib.device_status(clear=False)
    assert st & _lib.FK_STATUS_TIMEOUT
    with pytest.raises(_lib.DeviceTimeout):
        _lib.check_device("selftest")
    assert _lib.device_status() == 0
    # the context still works: a full step after the timeout
    m, vmc, opt = _ar_problem()
    vmc.step(opt)
    assert np.isfinite(vmc.current_energy.real)


def test_vmc_step_raises_on_a_recorded_timeout_then_recovers(cuda):
    from flowket_gb300 import _lib
    m, vmc, opt = _ar_problem()
    vmc.step(opt)
    _lib.call("fk_selftest_wait_timeout", 4096, _lib.stream_ptr())
    with pytest.raises(_lib.DeviceTimeout):
        vmc.step(opt)
    vmc.step(opt)
    assert np.isfinite(vmc.current_energy.real)


@pytest.mark.parametrize("precision", ["bf16", "fp32"])
def test_nonfinite_weight_injection_is_reported(cuda, precision):
    from flowket_gb300 import _lib
    m, vmc, opt = _ar_problem(precision)
    vmc.step(opt)
    good = m.params.clone()
    # a non-finite output-layer bias makes every log psi non-finite (a NaN
    # inside a hidden layer can be absorbed: ReLU as max(x, 0) maps NaN to 0)
    with torch.no_grad():
        m.named_params()["out.bias"][0] = float("nan")
    m.params_updated()
    with pytest.raises(_lib.NonFiniteError):
        vmc.step(opt)
    m.params.copy_(good)
    m.params_updated()
    opt.m.zero_()
    opt.v.zero_()
    vmc.step(opt)
    assert np.isfinite(vmc.current_energy.real)


def test_nonfinite_rbm_is_reported(cuda):
    from flowket_gb300 import _lib
    from flowket_gb300.machines import RBM
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.optimization import VariationalMonteCarlo
    from flowket_gb300.optimizers import Adam
    from flowket_gb300.samplers import MetropolisHastingsLocal
    shape = (8,)
    m = RBM(shape, alpha=1, stddev=0.05, seed=0)
    vmc = VariationalMonteCarlo(m, Heisenberg(hilbert_state_shape=shape, pbc=True),
                                MetropolisHastingsLocal(m, 128, num_of_chains=16, seed=1))
    opt = Adam(m, lr=1e-3)
    vmc.step(opt)
    with torch.no_grad():
        m.params[3] = float("inf")
    with pytest.raises(_lib.NonFiniteError):
        vmc.step(opt)
