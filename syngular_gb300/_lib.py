"""ctypes binding of ``libsyngular_gb300.so`` (the C ABI in ``include/syngular_gb300.h``).

The shared library is the only compute path: when it is missing, or when no
CUDA device is present, every operation raises instead of falling back to the
CPU.  Site cores are ``torch.float64`` CUDA tensors; PyTorch provides device
memory (its caching allocator also serves the workspaces) and the current
stream, nothing else.
"""
from __future__ import annotations

import ctypes
import os
from typing import Sequence

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libsyngular_gb300.so")

SGT_OK = 0
SGT_ERR_INVALID = 1
SGT_ERR_NOT_CONVERGED = 2
SGT_ERR_CUDA = 3
SGT_ERR_WORKSPACE = 4
SGT_ERR_SHAPE = 5

PREC_F64 = 0
PREC_TF32 = 1
PREC_BF16 = 2
PREC_BF16X3 = 3
PREC_TF32X3 = 4
PREC_BF16X6 = 5

TUNE_SLICED_SPLIT_CTAS = 0
TUNE_SLICED_SPLIT_MIN_KTILES = 1
TUNE_PCHOL_BLOCKED = 2
TUNE_PURIFY_CLEANUP = 3
TUNE_PURIFY_VECTOR_STEP = 4

_c_i64 = ctypes.c_int64
_c_vp = ctypes.c_void_p
_c_int = ctypes.c_int
_c_size = ctypes.c_size_t
_c_dbl = ctypes.c_double
_PP = ctypes.POINTER(ctypes.c_void_p)
_PI64 = ctypes.POINTER(ctypes.c_int64)

# name -> (restype, argtypes)
SIGNATURES = {
    "sgt_version": (_c_int, []),
    "sgt_last_error": (ctypes.c_char_p, []),
    "sgt_site_contract_mpo_mps": (_c_int, [_c_vp, _c_i64, _c_i64, _c_i64, _c_vp, _c_i64, _c_i64, _c_i64, _c_vp, _c_vp]),
    "sgt_site_contract_mpo_mpo": (_c_int, [_c_vp, _c_i64, _c_i64, _c_i64, _c_i64, _c_vp, _c_i64, _c_i64, _c_i64, _c_vp, _c_vp]),
    "sgt_bond_concat": (_c_int, [_c_vp, _c_i64, _c_i64, _c_i64, _c_vp, _c_i64, _c_i64, _c_int, _c_vp, _c_vp]),
    "sgt_bond_concat_chain": (_c_int, [_c_int, _PP, _PI64, _PP, _PI64, _PP, _c_vp, _c_size, _c_vp]),
    "sgt_bond_concat_chain_workspace_size": (_c_size, [_c_int]),
    "sgt_overlap_workspace_size": (_c_size, [_c_int, _PI64, _PI64]),
    "sgt_overlap_sweep": (_c_int, [_c_int, _PP, _PI64, _PP, _PI64, _c_vp, _c_vp, _c_size, _c_vp]),
    "sgt_overlap_prec_workspace_size": (_c_size, [_c_int, _PI64, _PI64, _c_int]),
    "sgt_overlap_sweep_prec": (_c_int, [_c_int, _PP, _PI64, _PP, _PI64, _c_int, _c_vp, _c_vp, _c_size, _c_vp]),
    "sgt_overlap_sweep_noalloc": (_c_int, [_c_int, _PP, _PI64, _PP, _PI64, _c_vp, _c_vp]),
    "sgt_qr_truncate_workspace_size": (_c_size, [_c_int, _PI64, _c_i64]),
    "sgt_qr_truncate_sweep": (_c_int, [_c_int, _PP, _PI64, _c_i64, _PP, _c_vp, _c_size, _c_vp]),
    "sgt_decompose_workspace_size": (_c_size, [_c_int, _PI64, _PI64, _c_int]),
    "sgt_decompose": (_c_int, [_c_vp, _c_int, _PI64, _PI64, _c_int, _PP, _c_vp, _c_size, _c_vp]),
    "sgt_normalize": (_c_int, [_c_vp, _c_i64, _c_vp, _c_vp]),
    "sgt_orthonormalize_workspace_size": (_c_size, [_c_int, _PI64]),
    "sgt_left_orthonormalize": (_c_int, [_c_int, _PP, _PI64, _c_vp, _c_size, _c_vp]),
    "sgt_right_orthonormalize": (_c_int, [_c_int, _PP, _PI64, _c_vp, _c_size, _c_vp]),
    "sgt_orthogonality": (_c_int, [_c_vp, _c_i64, _c_i64, _c_i64, _c_int, _c_vp, _c_vp]),
    "sgt_svd_round_shapes": (_c_int, [_c_int, _PI64, _c_i64, _PI64, _PI64]),
    "sgt_svd_round_workspace_size": (_c_size, [_c_int, _PI64, _c_i64, _c_int]),
    "sgt_svd_round": (_c_int, [_c_int, _PP, _PI64, _c_i64, _c_int, _PP, _c_vp, _c_vp, _c_vp, _c_vp, _c_size, _c_vp]),
    "sgt_gemm_f64": (_c_int, [_c_int, _c_int, _c_i64, _c_i64, _c_i64, _c_dbl, _c_vp, _c_i64, _c_i64, _c_vp, _c_i64, _c_i64, _c_dbl, _c_vp, _c_i64, _c_i64, _c_i64, _c_vp]),
    "sgt_qr_workspace_size": (_c_size, [_c_i64, _c_i64, _c_i64]),
    "sgt_qr": (_c_int, [_c_vp, _c_i64, _c_i64, _c_i64, _c_vp, _c_vp, _c_i64, _c_vp, _c_size, _c_vp]),
    "sgt_jacobi_svd_workspace_size": (_c_size, [_c_i64, _c_i64]),
    "sgt_jacobi_svd": (_c_int, [_c_vp, _c_i64, _c_i64, _c_vp, _c_vp, _c_vp, _c_vp, _c_size, _c_vp]),
    "sgt_tc_gemm_f32": (_c_int, [_c_int, _c_i64, _c_i64, _c_i64, ctypes.c_float, _c_vp, _c_vp, _c_i64, _c_vp, _c_vp, _c_i64, ctypes.c_float, _c_vp, _c_i64, _c_vp, _c_vp]),
    "sgt_tc_gemm_f32_workspace_size": (_c_size, [_c_i64, _c_i64, _c_i64]),
    "sgt_tc_gemm_f32_ws": (_c_int, [_c_int, _c_i64, _c_i64, _c_i64, ctypes.c_float, _c_vp, _c_vp, _c_i64, _c_vp, _c_vp, _c_i64, ctypes.c_float, _c_vp, _c_i64, _c_vp, _c_vp, _c_size, _c_vp]),
    "sgt_split_tf32": (_c_int, [_c_vp, _c_vp, _c_vp, _c_i64, _c_vp]),
    "sgt_gemm_f64_sliced_workspace_size": (_c_size, [_c_i64, _c_i64, _c_i64]),
    "sgt_gemm_f64_sliced": (_c_int, [_c_i64, _c_i64, _c_i64, _c_dbl, _c_vp, _c_i64, _c_vp, _c_i64, _c_dbl, _c_vp, _c_i64, _c_vp, _c_size, _c_vp]),
    "sgt_set_tuning": (_c_int, [_c_int, _c_int]),
    "sgt_get_tuning": (_c_int, [_c_int]),
    "sgt_phase_profile": (_c_int, [_c_int, ctypes.POINTER(ctypes.c_double), _c_int]),
    "sgt_sliced_profile": (_c_int, [_c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)]),
    "sgt_launch_count": (ctypes.c_ulonglong, []),
    "sgt_sym_eig_f32_workspace_size": (_c_size, [_c_i64]),
    "sgt_sym_eig_f32": (_c_int, [_c_vp, _c_i64, _c_vp, _c_vp, _c_vp, _c_int, _c_vp, _c_size, _c_vp]),
    "sgt_eig_method": (_c_int, [_c_int]),
    "sgt_batched_plan_create": (_c_int, [_c_int, _c_vp, _c_vp, _c_vp, _c_vp, _c_int, _c_int, _c_vp, _c_vp]),
    "sgt_batched_plan_lane": (_c_int, [_c_vp, _c_int]),
    "sgt_batched_plan_out_shape": (_c_int, [_c_vp, _c_int, _c_vp]),
    "sgt_batched_launch": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_size, _c_vp]),
    "sgt_batched_plan_destroy": (None, [_c_vp]),
    "sgt_tc_profile": (_c_int, [_c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)]),
    "sgt_eig_profile": (_c_int, [_c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)]),
    "sgt_env_blocks_workspace_size": (_c_size, [_c_int, _PI64, _PI64, _PI64, _c_int, _c_int]),
    "sgt_env_blocks": (_c_int, [_c_int, _PP, _PI64, _PP, _PI64, _PP, _PI64, _c_int, _c_int, _PP, _c_vp, _c_size, _c_vp]),
    "sgt_env_two_site_workspace_size": (_c_size, [_PI64, _PI64, _PI64, _PI64, _PI64]),
    "sgt_env_two_site": (_c_int, [_c_vp, _PI64, _c_vp, _PI64, _c_vp, _PI64, _c_vp, _PI64, _c_vp, _PI64, _c_vp, _c_vp, _c_size, _c_vp]),
    "sgt_mpo_mps_zipup_shapes": (_c_int, [_c_int, _PI64, _PI64, _c_i64, _PI64]),
    "sgt_mpo_mps_zipup_workspace_size": (_c_size, [_c_int, _PI64, _PI64, _c_i64]),
    "sgt_mpo_mps_zipup": (_c_int, [_c_int, _PP, _PI64, _PP, _PI64, _c_i64, _PP, _c_vp, _c_vp, _c_vp, _c_size, _c_vp]),
    "sgt_mpo_mps_round_workspace_size":(_c_size, [_c_int, _PI64, _PI64, _c_i64, _c_int]),
    "sgt_mpo_mps_round": (_c_int, [_c_int, _PP, _PI64, _PP, _PI64, _c_i64, _c_int, _PP, _c_vp, _c_vp, _c_vp, _c_vp, _c_size, _c_vp]),
}

_lib = None


class SyngularError(RuntimeError):
    """A nonzero status from the C ABI."""

    def __init__(self, fn, code, msg):
        super().__init__("%s failed (status %d): %s" % (fn, code, msg))
        self.code = code


def load():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            "libsyngular_gb300.so is not built (%s); run `python -c \"import __graft_entry__ as g; "
            "g.build()\"` first -- there is no CPU fallback" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def call(name, *args):
    lib = load()
    code = getattr(lib, name)(*args)
    if code != SGT_OK:
        msg = lib.sgt_last_error().decode(errors="replace")
        if code == SGT_ERR_SHAPE:
            raise ValueError(msg)
        raise SyngularError(name, code, msg)
    return code


def query(name, *args) -> int:
    return int(getattr(load(), name)(*args))


# ---------------------------------------------------------------------------
# marshalling helpers
# ---------------------------------------------------------------------------

def device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("syngular_gb300 needs a CUDA device (GB300, sm_103a); there is no CPU fallback")
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr():
    return _c_vp(torch.cuda.current_stream().cuda_stream)


def ptr(t: torch.Tensor):
    return _c_vp(t.data_ptr())


def ptr_array(tensors: Sequence[torch.Tensor]):
    arr = (ctypes.c_void_p * len(tensors))(*[t.data_ptr() for t in tensors])
    return ctypes.cast(arr, _PP), arr


def i64_array(values: Sequence[int]):
    arr = (ctypes.c_int64 * len(values))(*[int(v) for v in values])
    return ctypes.cast(arr, _PI64), arr


def shape_array(shapes):
    flat = []
    for s in shapes:
        flat += [int(s[0]), int(s[1]), int(s[2])]
    return i64_array(flat)


def workspace(nbytes: int) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device())


def as_device(t) -> torch.Tensor:
    """float64, contiguous, on the current CUDA device (host arrays are copied)."""
    dev = device()
    if isinstance(t, torch.Tensor):
        return t.to(device=dev, dtype=torch.float64).contiguous()
    import numpy as np

    return torch.from_numpy(np.ascontiguousarray(np.asarray(t, dtype=np.float64))).to(dev)
