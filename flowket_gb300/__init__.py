"""flowket_gb300: the variational Monte Carlo hot path of FlowKet on GB300.

Host code is Python over PyTorch CUDA tensors; every computation runs in the
hand-written sm_103a kernels of libflowket_gb300.so (C ABI in
include/flowket_gb300.h). Module names follow the reference package:
machines, operators, samplers, observables, optimization, optimizers.
"""
from . import _lib  # noqa: F401

__all__ = ["machines", "operators", "samplers", "observables", "optimization", "optimizers"]
