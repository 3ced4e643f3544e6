"""CPU restatement of FlowKet's variational-Monte-Carlo hot path.

TEST INFRASTRUCTURE ONLY. Nothing in the product (``flowket_gb300``) imports,
calls or links anything in this package; only ``tests/``, the smoke check in
``__graft_entry__.py`` and the CPU-baseline leg of ``bench.py`` use it, and
only to check results or as the timed CPU baseline.

Each function cites the reference file:line it restates (paths relative to the
FlowKet source tree). The reference itself (TensorFlow 1.x / tf.keras) cannot
run here, so parity is pinned by the reference's own known-answer tests and
published constants (see ``tests/test_oracle.py``):

* lncosh values at the reference test points (tests/test_tensorflow_complex_numbers_ops.py:6);
* the balanced == unbalanced local-energy fixture (tests/test_variational.py:18-46);
* the exact ground-state energies hard-coded in the reference examples
  (examples/basic_autoregressive_2d.py:38, examples/basic_autoregressive_monte_carlo_gradient.py:41,
  examples/rbm_heisenberg_1d_sr.py:35, examples/j1j2_2d_monte_carlo_4.py:43);
* normalisation of the autoregressive distribution (tests/test_autoregressive.py:18-30);
* the SR solve vs a pseudo-inverse (tests/test_stochastic_reconfiguration.py:32-72);
* the gradient-accumulation numbers (tests/test_gradients_aggregation.py:36-111).
"""
