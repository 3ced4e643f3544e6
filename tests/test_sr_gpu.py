"""Kernel set (d): sample-space SR against the oracle's parameter-space solve."""
import numpy as np
import pytest
import torch

from oracle import ar2d, sr as ref_sr

pytestmark = pytest.mark.gpu


def test_gram_and_solve_match_numpy(cuda):
    from flowket_gb300 import _lib
    rng = np.random.default_rng(0)
    p, b = 3000, 96
    a = rng.normal(size=(p, b)).astype(np.float32)
    c = rng.normal(size=(p, b)).astype(np.float32)
    ta, tc = torch.as_tensor(a).cuda(), torch.as_tensor(c).cuda()
    n = 2 * b
    gram = torch.empty((n, n), dtype=torch.float64, device="cuda")
    _lib.call("fk_sr_gram", _lib.ptr(ta), _lib.ptr(tc), p, b, _lib.ptr(gram), n * n, _lib.stream_ptr())
    y = np.concatenate([a, c], axis=1).astype(np.float64)
    want = y.T @ y
    np.testing.assert_allclose(gram.cpu().numpy(), want, rtol=1e-5, atol=1e-3)
    rhs = torch.as_tensor(rng.normal(size=n)).cuda()
    x = torch.empty(n, dtype=torch.float64, device="cuda")
    stats = torch.zeros(3, dtype=torch.float64, device="cuda")
    ws = torch.empty(_lib.load().fk_sr_solve_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    _lib.call("fk_sr_solve", _lib.ptr(gram), n, 1.0 / p, 0.05, _lib.ptr(rhs), 1e-12, 500, _lib.ptr(x),
              _lib.ptr(stats), _lib.ptr(ws), ws.numel(), _lib.stream_ptr())
    # the solver against a dense FP64 solve of the same (GPU-built) matrix
    ref = np.linalg.solve(gram.cpu().numpy() / p + 0.05 * np.eye(n), rhs.cpu().numpy())
    np.testing.assert_allclose(x.cpu().numpy(), ref, rtol=1e-8, atol=1e-10)
    assert 0 < stats[0].item() <= 500


@pytest.mark.parametrize("p,b,complex_", [(3000, 96, True), (4133, 200, True), (70_000, 512, True),
                                         (1000, 40, False), (64, 8, True)])
def test_tensor_core_gram_matches_fp64(cuda, p, b, complex_):
    """fk_sr_gram_tc (tcgen05, split-BF16 products, FP32 accumulation) against
    the FP64 Gram of the same FP32 rows, relative to sqrt(T_ii T_jj): 5e-5
    (the tensor core sums a 4096-parameter range in FP32: 2e-5 measured on
    the diagonal, where every term is positive; 2e-7 off it), and the
    CUDA-core fk_sr_gram at 1e-5. Sizes not multiples of the 128 x 256 tiles
    or of the 64 parameters per stage, and a single tile."""
    from flowket_gb300 import _lib
    rng = np.random.default_rng(p + b)
    a = rng.normal(size=(p, b)).astype(np.float32)
    c = rng.normal(size=(p, b)).astype(np.float32) if complex_ else None
    ta = torch.as_tensor(a).cuda()
    tc = torch.as_tensor(c).cuda() if complex_ else None
    n = 2 * b if complex_ else b
    y = np.concatenate([a, c], axis=1).astype(np.float64) if complex_ else a.astype(np.float64)
    want = y.T @ y
    scale = np.sqrt(np.outer(np.diag(want), np.diag(want)))
    for entry in ("fk_sr_gram_tc", "fk_sr_gram"):
        gram = torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
        _lib.call(entry, _lib.ptr(ta), _lib.ptr(tc), p, b, _lib.ptr(gram), n * n, _lib.stream_ptr())
        got = gram.cpu().numpy()
        err = np.abs(got - want) / scale
        assert err.max() < (5e-5 if entry == "fk_sr_gram_tc" else 1e-5), (entry, err.max())
        off = err[~np.eye(n, dtype=bool)]
        assert off.max() < 2e-6, (entry, off.max())
        np.testing.assert_array_equal(got, got.T)


@pytest.mark.parametrize("p,b,complex_", [(3000, 96, True), (4133, 200, True), (70_000, 512, True),
                                         (1000, 45, True), (64, 8, True), (33, 300, False), (9000, 1030, False),
                                         (300, 4100, True)])
def test_split_tensor_core_gram_matches_fp64(cuda, p, b, complex_):
    """fk_sr_gram_split (bf16 hi + lo written once in the blocked operand
    layout) + fk_sr_gram_split_accumulate (bulk-copied operands, the same
    split-BF16 products) + fk_sr_gram_mirror against the FP64 Gram of the
    same FP32 rows, with fk_sr_gram_tc's bounds; column counts that are not
    multiples of 8, 128 or 256 and row counts that are not multiples of 32;
    8,200 columns: 65 x 33 tiles in bands of 8 tile rows, the last one
    partial. Each call adds into the Gram: a second call doubles it."""
    from flowket_gb300 import _lib
    rng = np.random.default_rng(p + 3 * b)
    a = rng.normal(size=(p, b)).astype(np.float32)
    c = rng.normal(size=(p, b)).astype(np.float32) if complex_ else None
    ta = torch.as_tensor(a).cuda()
    tc = torch.as_tensor(c).cuda() if complex_ else None
    n = 2 * b if complex_ else b
    y = np.concatenate([a, c], axis=1).astype(np.float64) if complex_ else a.astype(np.float64)
    want = y.T @ y
    scale = np.sqrt(np.outer(np.diag(want), np.diag(want)))
    lib = _lib.load()
    nbytes = lib.fk_sr_gram_split_bytes(p, n)
    split = torch.full((nbytes,), 255, dtype=torch.uint8, device="cuda")
    st = _lib.stream_ptr()
    _lib.call("fk_sr_gram_split", _lib.ptr(ta), _lib.ptr(tc), b, b if complex_ else n, p, n, _lib.ptr(split), nbytes,
              st)
    gram = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    _lib.call("fk_sr_gram_split_accumulate", _lib.ptr(split), p, n, _lib.ptr(gram), st)
    _lib.call("fk_sr_gram_mirror", _lib.ptr(gram), n, st)
    got = gram.cpu().numpy()
    err = np.abs(got - want) / scale
    assert err.max() < 5e-5, err.max()
    # off the diagonal: <= 3 * 2^-18 per product (lo*lo dropped, lo rounded);
    # over >= 1000 random rows the errors average to 2e-7, over 33 to 5e-6
    assert err[~np.eye(n, dtype=bool)].max() < (2e-6 if p >= 1000 else 1.5e-5)
    np.testing.assert_array_equal(got, got.T)
    # a second accumulation adds the same tile sums again
    _lib.call("fk_sr_gram_split_accumulate", _lib.ptr(split), p, n, _lib.ptr(gram), st)
    _lib.call("fk_sr_gram_mirror", _lib.ptr(gram), n, st)
    np.testing.assert_allclose(gram.cpu().numpy(), 2 * got, rtol=1e-12, atol=0)
    assert lib.fk_sr_gram_split(_lib.ptr(ta), _lib.ptr(tc), b, b if complex_ else n, p, n, _lib.ptr(split),
                                nbytes - 1, st) == -1
    assert b"split buffer" in lib.fk_last_error()


@pytest.mark.parametrize("p,b", [(1000, 96), (77, 45), (300, 1030)])
def test_center_split_equals_center_then_split(cuda, p, b):
    """fk_sr_center_split (centring of each row within [0, b) and [b, 2b),
    written back, and the split in one pass) gives bitwise the rows of
    fk_center_columns on each half and the split operands of
    fk_sr_gram_split on them; without write-back the rows stay as they were."""
    from flowket_gb300 import _lib
    rng = np.random.default_rng(p + b)
    a = torch.as_tensor(rng.normal(1.0, 2.0, size=(p, b)).astype(np.float32)).cuda()
    c = torch.as_tensor(rng.normal(-0.5, 1.0, size=(p, b)).astype(np.float32)).cuda()
    lib = _lib.load()
    n = 2 * b
    nbytes = lib.fk_sr_gram_split_bytes(p, n)
    st = _lib.stream_ptr()
    a1, c1 = a.clone(), c.clone()
    split1 = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
    _lib.call("fk_sr_center_split", _lib.ptr(a1), _lib.ptr(c1), b, b, p, n, 1, _lib.ptr(split1), nbytes, st)
    a2, c2 = a.clone(), c.clone()
    _lib.call("fk_center_columns", _lib.ptr(a2), p, b, None, st)
    _lib.call("fk_center_columns", _lib.ptr(c2), p, b, None, st)
    split2 = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
    _lib.call("fk_sr_gram_split", _lib.ptr(a2), _lib.ptr(c2), b, b, p, n, _lib.ptr(split2), nbytes, st)
    assert torch.equal(a1, a2) and torch.equal(c1, c2)
    assert torch.equal(split1, split2)
    a3, c3 = a.clone(), c.clone()
    split3 = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
    _lib.call("fk_sr_center_split", _lib.ptr(a3), _lib.ptr(c3), b, b, p, n, 0, _lib.ptr(split3), nbytes, st)
    assert torch.equal(a3, a) and torch.equal(c3, c) and torch.equal(split3, split2)


def test_tensor_core_gram_rejects_unsupported_shapes(cuda):
    from flowket_gb300 import _lib
    lib = _lib.load()
    buf = torch.zeros(1024, dtype=torch.float32, device="cuda")
    g = torch.zeros(1024, dtype=torch.float64, device="cuda")
    assert lib.fk_sr_gram_tc(_lib.ptr(buf), None, 10, 12, _lib.ptr(g), 1024, _lib.stream_ptr()) == -1
    assert b"multiple of 8" in lib.fk_last_error()


@pytest.mark.parametrize("gram", ["fp32", "tc"])
def test_sr_direction_matches_parameter_space_solve(cuda, gram):
    """(Re<O_c^* O_c> + lambda) x = Re<O_c^* E_c>: the sample-space GPU solve
    (Gram on the CUDA cores or on the tensor cores) equals the oracle's
    parameter-space solve on the same O and E_loc."""
    from flowket_gb300 import _lib
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.observables import Observable
    from flowket_gb300.optimizers import ComplexValuesStochasticReconfiguration
    shape, depth, f = (3, 4), 2, 16
    m = ConvNetAutoregressive2D(shape, depth, f, weights_normalization=False, precision="fp32", seed=1)
    rng = np.random.default_rng(2)
    s = torch.as_tensor(rng.choice([-1, 1], size=(96,) + shape).astype(np.int8)).cuda()
    _, _, saved = m.forward(s, mode=_lib.FK_AR2D_SAVE)
    local = Observable(Heisenberg(hilbert_state_shape=shape, pbc=True)).local_values(m, s)
    opt = ComplexValuesStochasticReconfiguration(m, lr=0.05, diag_shift=1e-2, iterative_solver=False, gram=gram)
    x = opt.direction(s, local, saved).cpu().numpy().astype(np.float64)
    o = m.log_derivatives(s, saved).cpu().numpy().T.astype(np.complex128)
    e = local[:, 0].cpu().numpy() + 1j * local[:, 1].cpu().numpy()
    want = ref_sr.sr_real(o, e, 1e-2)
    assert np.linalg.norm(x - want) / np.linalg.norm(want) < 1e-3


@pytest.mark.parametrize("rows_bytes", [None, 4])
def test_vmc_with_sr_lowers_energy(cuda, rows_bytes):
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.optimization import VariationalMonteCarlo
    from flowket_gb300.optimizers import ComplexValuesStochasticReconfiguration
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape = (4, 4)
    m = ConvNetAutoregressive2D(shape, 3, 16, weights_normalization=True, precision="fp32", seed=0)
    vmc = VariationalMonteCarlo(m, Heisenberg(hilbert_state_shape=shape, pbc=True),
                                FastAutoregressiveSampler(m, 256, seed=3))
    opt = ComplexValuesStochasticReconfiguration(m, lr=0.05, diag_shift=1e-3, rows_bytes=rows_bytes)
    energies = []
    for _ in range(30):
        vmc.step(opt)
        energies.append(vmc.current_energy.real)
    assert opt.streamed == (rows_bytes is not None)
    assert np.mean(energies[-5:]) < np.mean(energies[:3]) - 1.0


@pytest.mark.parametrize("tensor_cores", [0, 1])
def test_gram_accumulated_by_row_blocks(cuda, tensor_cores):
    """fk_sr_gram_accumulate over row blocks of Y, then fk_sr_gram_mirror,
    against the FP64 Gram of the same rows: the block-by-block Gram of the
    streamed SR path (same bounds as the whole-array kernels)."""
    from flowket_gb300 import _lib
    rng = np.random.default_rng(11)
    p, n = 9000, 264
    y = rng.normal(size=(p, n)).astype(np.float32)
    ty = torch.as_tensor(y).cuda()
    gram = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    for r0, r1 in ((0, 1000), (1000, 1008), (1008, 6100), (6100, p)):
        _lib.call("fk_sr_gram_accumulate", _lib.ptr(ty[r0:]), r1 - r0, n, _lib.ptr(gram), tensor_cores,
                  _lib.stream_ptr())
    _lib.call("fk_sr_gram_mirror", _lib.ptr(gram), n, _lib.stream_ptr())
    want = y.astype(np.float64).T @ y.astype(np.float64)
    err = np.abs(gram.cpu().numpy() - want) / np.sqrt(np.outer(np.diag(want), np.diag(want)))
    assert err.max() < (5e-5 if tensor_cores else 1e-5), err.max()
    assert err[~np.eye(n, dtype=bool)].max() < 2e-6


# (shape, depth, channels, weight norm, precision): CUDA-core adjoint (F = 16,
# FP32), the tensor-core adjoint's per-sample rows (F = 32, BF16 and FP16)
STREAMED_NETS = [((4, 4), 3, 16, True, "fp32"), ((6, 6), 3, 32, True, "bf16"), ((5, 6), 2, 32, True, "fp16"),
                 ((4, 4), 2, 16, False, "bf16")]


def _stored_rows(m, s, saved):
    """Y = [Re O_c | Im O_c] (num_params x 2B) from the stored per-sample rows."""
    b = s.shape[0]
    ones = torch.zeros((b, 2), dtype=torch.float32, device="cuda")
    ones[:, 0] = 1
    o_re = m.backward(s, ones, saved, per_sample=True).double()
    ones[:, 0], ones[:, 1] = 0, 1
    o_im = m.backward(s, ones, saved, per_sample=True).double()
    y = torch.cat([o_re - o_re.mean(1, keepdim=True), o_im - o_im.mean(1, keepdim=True)], dim=1)
    return y.cpu().numpy()


@pytest.mark.parametrize("tensor_cores", [0, 1])
@pytest.mark.parametrize("net", range(len(STREAMED_NETS)))
def test_streamed_sr_gram_equals_gram_of_stored_rows(cuda, net, tensor_cores):
    """fk_ar2d_sr_gram (both per-sample adjoints over one set of activations,
    rows streamed conv by conv through the smallest row buffer allowed: a
    flush at almost every step, weight-norm chain rule and centring per
    buffer) against the FP64 Gram of the stored, centred per-sample rows of
    fk_ar2d_backward: the streamed rows are the same numbers, so the bounds
    are the Gram kernels' own."""
    from flowket_gb300 import _lib
    from flowket_gb300.machines import ConvNetAutoregressive2D, ctypes_ref
    shape, depth, f, wn, prec = STREAMED_NETS[net]
    m = ConvNetAutoregressive2D(shape, depth, f, weights_normalization=wn, precision=prec, seed=3 + net)
    b = 64
    s = m._spins(torch.as_tensor(np.random.default_rng(net).choice([-1, 1], size=(b,) + shape).astype(np.int8)))
    _, _, saved = m.forward(s, mode=_lib.FK_AR2D_SAVE)
    y = _stored_rows(m, s, saved)
    want = y.T @ y
    n = 2 * b
    lib = _lib.load()
    d = ctypes_ref(m.desc)
    ws = torch.empty(lib.fk_ar2d_sr_gram_workspace_bytes(d, b), dtype=torch.uint8, device="cuda")
    min_rows = lib.fk_ar2d_sr_gram_min_rows(d, b, tensor_cores)
    rows = torch.empty(min_rows + 7, dtype=torch.float32, device="cuda")
    gram = torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
    _lib.call("fk_ar2d_sr_gram", d, _lib.ptr(m.packed()), _lib.ptr(m.params), _lib.ptr(s), b, _lib.ptr(saved),
              saved.numel(), _lib.ptr(ws), ws.numel(), _lib.ptr(rows), rows.numel(), _lib.ptr(gram), tensor_cores,
              _lib.stream_ptr())
    got = gram.cpu().numpy()
    np.testing.assert_array_equal(got, got.T)
    err = np.abs(got - want) / np.sqrt(np.outer(np.diag(want), np.diag(want)))
    assert err.max() < (5e-5 if tensor_cores else 1e-5), err.max()
    # off the diagonal the split-BF16 products (lo*lo dropped, lo rounded:
    # <= 3 * 2^-18 of sum |y_pi y_pj| <= sqrt(T_ii T_jj)) reach 5.7e-6 on
    # these rows, whose entries share signs (2e-7 on random rows)
    assert err[~np.eye(n, dtype=bool)].max() < (1.5e-5 if tensor_cores else 2e-6)
    # a buffer below the minimum, or a short workspace, is an argument error
    args = [d, _lib.ptr(m.packed()), _lib.ptr(m.params), _lib.ptr(s), b, _lib.ptr(saved), saved.numel(),
            _lib.ptr(ws), ws.numel(), _lib.ptr(rows), min_rows - 1, _lib.ptr(gram), tensor_cores, _lib.stream_ptr()]
    assert lib.fk_ar2d_sr_gram(*args) == -1 and b"row buffer" in lib.fk_last_error()
    args[10], args[8] = min_rows, ws.numel() - 1
    assert lib.fk_ar2d_sr_gram(*args) == -1 and b"workspace" in lib.fk_last_error()


# ||x_streamed - x_stored|| / ||x_stored||, 3x the worst of 5 seeds per
# network (6.2e-6, 8.0e-3, 1.0e-3, 6.5e-6): the CUDA-core adjoints keep FP32
# gradient tensors (rounding only); on the tensor-core adjoint (F = 32, BF16
# and FP16) the update's seeds pass through its 16-bit gradient tensors
STREAMED_X = [2e-5, 2.5e-2, 3e-3, 2e-5]


@pytest.mark.parametrize("with_saved", [True, False])
@pytest.mark.parametrize("net", range(len(STREAMED_NETS)))
def test_streamed_sr_direction_equals_stored(cuda, net, with_saved):
    """ComplexValuesStochasticReconfiguration with ``rows_bytes`` (the
    streamed route: Gram through fk_ar2d_sr_gram, update as the summed
    adjoint with the centred solution as seeds) against the stored route on
    the same samples and local energies."""
    from flowket_gb300 import _lib
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.observables import Observable
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.optimizers import ComplexValuesStochasticReconfiguration
    shape, depth, f, wn, prec = STREAMED_NETS[net]
    m = ConvNetAutoregressive2D(shape, depth, f, weights_normalization=wn, precision=prec, seed=7 + net)
    b = 128
    s = m._spins(torch.as_tensor(np.random.default_rng(20 + net).choice([-1, 1], size=(b,) + shape)
                                 .astype(np.int8)))
    _, _, saved = m.forward(s, mode=_lib.FK_AR2D_SAVE)
    local = Observable(Heisenberg(hilbert_state_shape=shape, pbc=True)).local_values(m, s)
    ref = ComplexValuesStochasticReconfiguration(m, lr=0.05, diag_shift=1e-2, iterative_solver=False)
    x_ref = ref.direction(s, local, saved).double()
    assert not ref.streamed
    opt = ComplexValuesStochasticReconfiguration(m, lr=0.05, diag_shift=1e-2, iterative_solver=False,
                                                 rows_bytes=4)  # the smallest buffer allowed
    x = opt.direction(s, local, saved if with_saved else None).double()
    assert opt.streamed
    rel = (torch.linalg.norm(x - x_ref) / torch.linalg.norm(x_ref)).item()
    assert rel < STREAMED_X[net], rel
