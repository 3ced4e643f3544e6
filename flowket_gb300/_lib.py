"""ctypes binding of libflowket_gb300.so (the C ABI in include/flowket_gb300.h).

The library is built in-tree (flowket_gb300/build.py). There is no CPU
fallback: every product path calls into this library and raises if it is
missing or if a call returns a non-zero status.
"""
import ctypes
import os

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libflowket_gb300.so")

FK_PRECISION_FP32 = 0
FK_PRECISION_BF16 = 1
FK_PRECISION_FP16 = 2
PRECISIONS = {"fp32": FK_PRECISION_FP32, "bf16": FK_PRECISION_BF16, "fp16": FK_PRECISION_FP16}
FK_AR2D_INFER = 0
FK_AR2D_SAVE = 1

c_i32, c_i64, c_u64, c_f32, c_f64, c_p = (ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64, ctypes.c_float,
                                          ctypes.c_double, ctypes.c_void_p)


class Ar2dDesc(ctypes.Structure):
    _fields_ = [("height", c_i32), ("width", c_i32), ("depth", c_i32), ("channels", c_i32),
                ("weights_normalization", c_i32), ("precision", c_i32), ("equal_up_down_spins", c_i32)]


class RbmDesc(ctypes.Structure):
    _fields_ = [("n_visible", c_i32), ("n_hidden", c_i32)]


_SIGNATURES = {
    "fk_last_error": (ctypes.c_char_p, []),
    "fk_version": (ctypes.c_char_p, []),
    "fk_kernel_launches": (c_i64, []),
    "fk_device_status": (c_i32, [c_p, c_i32, c_p]),
    "fk_find_conn_heisenberg": (c_i32, [c_p, c_i64, c_i32, c_i32, c_i32, c_i32, c_i32, c_p, c_p, c_p, c_p, c_p]),
    "fk_find_conn_ising": (c_i32, [c_p, c_i64, c_i32, c_i32, c_f64, c_f64, c_i32, c_p, c_p, c_p, c_p, c_p]),
    "fk_find_conn_j1j2": (c_i32, [c_p, c_i64, c_i32, c_i32, c_f64, c_i32, c_p, c_p, c_p, c_p, c_p]),
    "fk_compact_workspace_bytes": (c_i64, [c_i64]),
    "fk_compact_connections": (c_i32, [c_p, c_i64, c_i32, c_i32, c_p, c_p, c_p, c_i32, c_p, c_p, c_p, c_p, c_p,
                                       c_i64, c_p, c_p, c_i64, c_p]),
    "fk_local_energy_reduce": (c_i32, [c_p, c_p, c_i64, c_p, c_p, c_p, c_p, c_p]),
    "fk_energy_stats": (c_i32, [c_p, c_i64, c_p, c_p, c_p]),
    "fk_ar2d_num_params": (c_i64, [c_p]),
    "fk_ar2d_packed_bytes": (c_i64, [c_p]),
    "fk_ar2d_pack": (c_i32, [c_p, c_p, c_p, c_p]),
    "fk_ar2d_workspace_bytes": (c_i64, [c_p, c_i64, c_i32]),
    "fk_ar2d_forward": (c_i32, [c_p, c_p, c_p, c_i64, c_p, c_p, c_p, c_i64, c_i32, c_p]),
    "fk_ar2d_sample": (c_i32, [c_p, c_p, c_i64, c_u64, c_u64, c_p, c_p, c_p, c_i64, c_p]),
    "fk_ar2d_connections_workspace_bytes": (c_i64, [c_p, c_i64, c_i64]),
    "fk_ar2d_forward_connections": (c_i32, [c_p, c_p, c_p, c_p, c_p, c_i64, c_p, c_i64, c_i64, c_p, c_p, c_i64,
                                            c_i64, c_p]),
    "fk_ar2d_backward_workspace_bytes": (c_i64, [c_p, c_i64]),
    "fk_ar2d_backward": (c_i32, [c_p, c_p, c_p, c_p, c_i64, c_p, c_p, c_i64, c_p, c_i64, c_p, c_p, c_p]),
    "fk_ar2d_sr_gram_workspace_bytes": (c_i64, [c_p, c_i64]),
    "fk_ar2d_sr_gram_min_rows": (c_i64, [c_p, c_i64, c_i32]),
    "fk_ar2d_sr_gram": (c_i32, [c_p, c_p, c_p, c_p, c_i64, c_p, c_i64, c_p, c_i64, c_p, c_i64, c_p, c_i32, c_p]),
    "fk_axpy": (c_i32, [c_i64, c_f32, c_p, c_p, c_p]),
    "fk_adam_step": (c_i32, [c_p, c_p, c_p, c_p, c_i64, c_i64, c_f32, c_f32, c_f32, c_f32, c_p]),
    "fk_sr_gram_workspace_bytes": (c_i64, [c_i64, c_i64]),
    "fk_sr_gram": (c_i32, [c_p, c_p, c_i64, c_i64, c_p, c_i64, c_p]),
    "fk_sr_gram_tc": (c_i32, [c_p, c_p, c_i64, c_i64, c_p, c_i64, c_p]),
    "fk_sr_gram_accumulate": (c_i32, [c_p, c_i64, c_i64, c_p, c_i32, c_p]),
    "fk_sr_gram_mirror": (c_i32, [c_p, c_i64, c_p]),
    "fk_sr_gram_split_bytes": (c_i64, [c_i64, c_i64]),
    "fk_sr_gram_split": (c_i32, [c_p, c_p, c_i64, c_i64, c_i64, c_i64, c_p, c_i64, c_p]),
    "fk_sr_gram_split_accumulate": (c_i32, [c_p, c_i64, c_i64, c_p, c_p]),
    "fk_sr_center_split": (c_i32, [c_p, c_p, c_i64, c_i64, c_i64, c_i64, c_i32, c_p, c_i64, c_p]),
    "fk_sr_solve_workspace_bytes": (c_i64, [c_i64]),
    "fk_sr_solve": (c_i32, [c_p, c_i64, c_f64, c_f64, c_p, c_f64, c_i32, c_p, c_p, c_p, c_i64, c_p]),
    "fk_sr_solve_noalloc": (c_i32, [c_p, c_i64, c_f64, c_f64, c_p, c_f64, c_i32, c_p, c_p, c_p]),
    "fk_sr_backmap": (c_i32, [c_p, c_p, c_i64, c_i64, c_p, c_f64, c_f32, c_p, c_p, c_p]),
    "fk_sr_hermitian_embed": (c_i32, [c_p, c_i64, c_p]),
    "fk_sr_complex_backmap": (c_i32, [c_p, c_p, c_i64, c_i64, c_p, c_f64, c_f32, c_p, c_p, c_p]),
    "fk_selftest_wait_timeout": (c_i32, [c_i32, c_p]),
    "fk_gather_complex": (c_i32, [c_p, c_p, c_i64, c_p, c_p]),
    "fk_segment_sum_rows": (c_i32, [c_p, c_p, c_p, c_i64, c_i64, c_p, c_p]),
    "fk_complex_param_gradient": (c_i32, [c_p, c_p, c_i64, c_i64, c_p, c_p, c_p]),
    "fk_center_columns": (c_i32, [c_p, c_i64, c_i64, c_p, c_p]),
    "fk_rbm_log_psi": (c_i32, [c_p, c_i32, c_i32, c_p, c_i64, c_p, c_p]),
    "fk_rbm_local_energy": (c_i32, [c_p, c_i32, c_i32, c_p, c_i64, c_p, c_p, c_p, c_i32, c_p, c_p]),
    "fk_rbm_log_derivatives": (c_i32, [c_p, c_i32, c_i32, c_p, c_i64, c_p, c_p, c_p]),
    "fk_rbm_mh_sweeps": (c_i32, [c_p, c_i32, c_i32, c_i32, c_i32, c_i32, c_p, c_p, c_i64, c_i64, c_i32, c_i32, c_u64,
                                 c_u64, c_p, c_p, c_p]),
    "fk_mh_independent_step": (c_i32, [c_p, c_p, c_p, c_p, c_p, c_p, c_i64, c_i32, c_u64, c_u64, c_p, c_p]),
    "fk_mh_hamiltonian_propose": (c_i32, [c_p, c_p, c_p, c_i32, c_i64, c_i32, c_u64, c_u64, c_p, c_p, c_p]),
    "fk_mh_hamiltonian_accept": (c_i32, [c_p, c_p, c_p, c_p, c_p, c_p, c_i32, c_i64, c_i32, c_u64, c_u64, c_p, c_p]),
}

_lib = None


class FlowketError(RuntimeError):
    pass


def load():
    """Loads the in-tree library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FlowketError(
            "libflowket_gb300.so is not built (run `python -m flowket_gb300.build` or "
            "`python -c 'import __graft_entry__ as g; g.build()'`); there is no CPU fallback")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    lib = load()
    return [n for n in _SIGNATURES if getattr(lib, n, None) is not None]


def check(status, what=""):
    if status != 0:
        msg = load().fk_last_error().decode(errors="replace")
        if status == -1:
            raise ValueError(f"{what}: {msg}")
        raise FlowketError(f"{what} failed ({status}): {msg}")


def call(name, *args):
    lib = load()
    check(getattr(lib, name)(*args), name)


def ptr(t):
    if t is None:
        return None
    if not isinstance(t, torch.Tensor):
        raise TypeError("expected a torch tensor")
    if t.numel() and not t.is_cuda:
        raise ValueError("flowket_gb300 kernels take CUDA tensors (no CPU fallback)")
    return ctypes.c_void_p(t.data_ptr())


def stream_ptr(device=None):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


FK_STATUS_TIMEOUT = 1
FK_STATUS_NONFINITE = 2


class DeviceTimeout(FlowketError):
    """A bounded device-side wait gave up; the kernel's outputs are incomplete."""


class NonFiniteError(FlowketError):
    """A non-finite energy statistic (the reference raises on a non-finite
    wave function, samplers/metropolis_hastings.py:103-105)."""


def device_status(clear=True):
    out = ctypes.c_int32(0)
    check(load().fk_device_status(ctypes.byref(out), 1 if clear else 0, stream_ptr()), "fk_device_status")
    return out.value


def check_device(what="flowket_gb300"):
    """Reads and clears the device error word (synchronises the current
    stream) and raises if a kernel recorded a failure since the last check."""
    st = device_status(clear=True)
    if st & FK_STATUS_TIMEOUT:
        raise DeviceTimeout(f"{what}: a device-side wait timed out; results of this step are incomplete")
    if st & FK_STATUS_NONFINITE:
        raise NonFiniteError(f"{what}: non-finite local energy (the wave function is not finite)")
    if st:
        raise FlowketError(f"{what}: device error word {st:#x}")
