"""ctypes binding of ``libedgpu.so`` (the C ABI declared in ``include/edgpu.h``).

The library is loaded from ``impuritymodel_gb300/_lib/libedgpu.so`` (built in-tree by
``impuritymodel_gb300.nvcc_build``).  There is no fallback: if the library is missing the
import of the engine raises.
"""

from __future__ import annotations

import ctypes as C
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libedgpu.so")

EDGPU_OK = 0
EDGPU_ERR_ARG = 1
EDGPU_ERR_OVERFLOW = 2
EDGPU_ERR_BREAKDOWN = 3
EDGPU_ERR_NAN = 4
EDGPU_ERR_NOCONV = 5
EDGPU_ERR_CUDA = 6
EDGPU_ERR_WORKSPACE = 7

FILTER_NONE = 0
FILTER_IN_BASIS = 1
FILTER_NOT_IN_BASIS = 2

ABI_VERSION = 2  # EDGPU_ABI_VERSION in include/edgpu.h
MAX_RESTRICTIONS = 8
MAX_WORDS = 8

# Exported symbols and their signatures (restype, argtypes).
_P = C.c_void_p
_I64 = C.c_int64
_I = C.c_int
_D = C.c_double
_SZ = C.c_size_t


class Terms(C.Structure):
    _fields_ = [("ops", _P), ("coeff", _P), ("flags", _P), ("n_terms", C.c_int32)]


class Restrictions(C.Structure):
    _fields_ = [
        ("n", C.c_int32),
        ("lo", C.c_int32 * MAX_RESTRICTIONS),
        ("hi", C.c_int32 * MAX_RESTRICTIONS),
        ("mask", (C.c_uint64 * MAX_WORDS) * MAX_RESTRICTIONS),
    ]


class Ragged(C.Structure):
    _fields_ = [
        ("n_sectors", _I),
        ("n_runs", _I),
        ("sec_row0", _P),
        ("run_sec", _P),
        ("run_vec0", _P),
        ("max_rows", _I64),
    ]


class CSR(C.Structure):
    _fields_ = [
        ("n", _I64),
        ("nnz", _I64),
        ("row_ptr", _P),
        ("col", _P),
        ("val_c", _P),
        ("val_r", _P),
        ("val_cf", _P),
        ("val_rf", _P),
        ("val_df", _P),
    ]


SIGNATURES = {
    "edgpu_abi_version": (_I, []),
    "edgpu_status_string": (C.c_char_p, [_I]),
    "edgpu_apply_columns": (
        _I,
        [_I, _P, _I64, C.POINTER(Terms), C.POINTER(Restrictions), _D, _P, _I64, _I, _P, _P, _P, _P, _P, _I, _I, _P, _P],
    ),
    "edgpu_apply_vector": (_I, [_I, _P, _P, _I64, C.POINTER(Terms), C.POINTER(Restrictions), _P, _P, _P, _P, _P]),
    "edgpu_sort_states_workspace": (_SZ, [_I, _I64]),
    "edgpu_sort_states": (_I, [_I, _P, _P, _I64, C.POINTER(C.c_uint64), _P, _SZ, _P]),
    "edgpu_vary_mask": (_I, [_I, _P, _I64, _P, _P]),
    "edgpu_scan_workspace": (_SZ, [_I64]),
    "edgpu_scan_i64": (_I, [_P, _P, _I64, _P, _SZ, _P]),
    "edgpu_segment_heads": (_I, [_I, _P, _I64, _P, _P]),
    "edgpu_segment_reduce": (_I, [_I, _P, _P, _I64, _P, _P, _P, _P, _P, _P]),
    "edgpu_merge_states": (_I, [_I, _P, _I64, _P, _I64, _P, _P]),
    "edgpu_lookup_states": (_I, [_I, _P, _I64, _P, _I64, _P, _P]),
    "edgpu_spmv": (_I, [C.POINTER(CSR), _P, _P, _I, _P]),
    "edgpu_spmv_c64": (_I, [C.POINTER(CSR), _P, _P, _I, _P]),
    "edgpu_spmv_plan_workspace": (_SZ, [_I64]),
    "edgpu_spmv_plan": (_I, [C.POINTER(CSR), _I64, _I, _P, C.POINTER(_I64), _P, _SZ, _P]),
    "edgpu_spmv_planned": (_I, [C.POINTER(CSR), _P, _I64, _I, _I, _P, _P, _I, _P]),
    "edgpu_spmv_planned_c64": (_I, [C.POINTER(CSR), _P, _I64, _I, _I, _P, _P, _I, _P]),
    "edgpu_spmv_pages_workspace": (_SZ, [_I64, _I]),
    "edgpu_spmv_pages_build": (_I, [C.POINTER(CSR), _P, _I64, _I, _I, _I, _P, _I64, C.POINTER(_I64), _P, _SZ, _P]),
    "edgpu_spmv_paged": (_I, [C.POINTER(CSR), _P, _I64, _I, _I, _I, _P, _P, _I, _P]),
    "edgpu_spmv_paged_c64": (_I, [C.POINTER(CSR), _P, _I64, _I, _I, _I, _P, _P, _I, _P]),
    "edgpu_spmv_paged_tma_c64": (_I, [C.POINTER(CSR), _P, _I64, _I, _I, _P, _P, _I, _P, _P]),
    "edgpu_hv_diag": (_I, [_I, _P, _I64, C.POINTER(Terms), _P, _P]),
    "edgpu_state_hash_build": (_I, [_I, _P, _I64, _P, _I64, _P]),
    "edgpu_hv_matfree": (_I, [_I, _P, _I64, _P, _I64, _I, _P, C.POINTER(Terms), _I, C.POINTER(Restrictions), _P, _D,
                              _P, _P, _I, _P]),
    "edgpu_hv_matfree_c64": (_I, [_I, _P, _I64, _P, _I64, _I, _P, C.POINTER(Terms), _I, C.POINTER(Restrictions), _P,
                                  _D, _P, _P, _I, _P]),
    "edgpu_krylov_workspace": (_SZ, [_I64, _I, _I]),
    "edgpu_krylov_dot": (_I, [_I, _P, _I64, _I, _I64, _I, _P, _P, _P, _SZ, _P]),
    "edgpu_krylov_project": (_I, [_I, _P, _I64, _I, _I64, _I, _P, _P, _I, _P, _SZ, _P]),
    "edgpu_krylov_normalize": (_I, [_I, _I64, _I, _P, _P, _P, _P, _P, _SZ, _P]),
    "edgpu_build_csr_workspace": (_SZ, [_I, _I64, _I64]),
    "edgpu_build_csr": (_I, [_I, C.POINTER(Terms), C.POINTER(Restrictions), _D, _P, _I64, _I, _P, _P, _P, _I64,
                             C.POINTER(_I64), _P, _P, _SZ, _P]),
    "edgpu_expand_workspace": (_SZ, [_I, _I64, _I64]),
    "edgpu_expand": (_I, [_I, C.POINTER(Terms), C.POINTER(Restrictions), _D, _P, _I64, _I64, _I64, _P, _P,
                          C.POINTER(_I64), _P, _P, _SZ, _P]),
    "edgpu_eig_lowest_workspace": (_SZ, [_I64, _I]),
    "edgpu_eig_lowest": (_I, [C.POINTER(CSR), _I, _D, _I, C.c_uint64, C.POINTER(_D), _P, C.POINTER(_I), _P, _P,
                              _SZ, _P]),
    "edgpu_lanczos_workspace": (_SZ, [_I64, _I, _I, _I]),
    "edgpu_lanczos": (_I, [C.POINTER(CSR), _P, _I, _P, _I, _I, _P, _P, _P, _P, _SZ, _P]),
    "edgpu_lanczos_timed": (_I, [C.POINTER(CSR), _P, _I, _P, _I, _I, _P, _P, _P, _P, _SZ, _P, C.POINTER(_D)]),
    "edgpu_launch_count": (C.c_longlong, []),
    "edgpu_lanczos_noalloc": (_I, [C.POINTER(CSR), _P, _I, _P, _I, _I, _P, _P, _P, _P]),
    "edgpu_lanczos_noalloc_bytes": (_SZ, []),
    "edgpu_lanczos_noalloc_forget": (None, []),
    "edgpu_lanczos_reorth_workspace": (_SZ, [_I64, _I]),
    "edgpu_lanczos_reorth": (_I, [C.POINTER(CSR), _P, _I, _I, _I, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "edgpu_lanczos_reorth_df": (_I, [C.POINTER(CSR), _P, _I, _I, _I, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "edgpu_set_reorth_fused": (None, [_I]),
    "edgpu_set_small_reserve": (None, [_I]),
    "edgpu_set_lanczos_cta": (None, [_I]),
    "edgpu_shifted_solve_workspace": (_SZ, [_I64, _I, _I, _I]),
    "edgpu_shifted_solve": (_I, [C.POINTER(CSR), _P, _I, _P, _I, _I, _D, _P, _P, _P, _P, _SZ, _P]),
    "edgpu_shifted_solve_df": (_I, [C.POINTER(CSR), _P, _I, _P, _I, _I, _D, _P, _P, _P, _P, _SZ, _P]),
    "edgpu_combine": (_I, [_P, _I, _I64, _P, _I, _P, _P]),
    "edgpu_lanczos_ragged_smem": (_SZ, [_I64]),
    "edgpu_lanczos_ragged": (_I, [C.POINTER(CSR), C.c_void_p, _P, _P, _I, _P, _P, _P, _P]),
    "edgpu_lanczos_reorth_ragged_smem": (_SZ, [_I64, _I]),
    "edgpu_lanczos_reorth_ragged": (_I, [C.POINTER(CSR), C.c_void_p, _P, _P, _I, _P, _P, _P, _P, _P, _P]),
    "edgpu_combine_ragged": (_I, [_P, C.c_void_p, _P, _P, _P, _I, _I, _P, _P]),
    "edgpu_gemm_bf16": (_I, [_P, _P, _I, _I, _I, _P, _P, _P]),
    "edgpu_density_matrix": (_I, [_I, _P, _P, _P, _I, _P, _I, _P, _P]),
    "edgpu_components": (_I, [C.POINTER(CSR), _P, _P, _P]),
    "edgpu_gemm_bf16_epi": (_I, [_I, _P, _P, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
    "edgpu_gemm_tile_width": (_I, [_I, _I]),
    "edgpu_mlp_bits": (_I, [_P, _I, _I64, _I, _P, _P, _P]),
    "edgpu_mlp_head": (_I, [_P, _P, _P, _I64, _I, _P, _P]),
    "edgpu_mlp_head_backward": (_I, [_P, _P, _P, _P, _I64, _I, _P, _P, _P, _P]),
    "edgpu_mlp_row_dot": (_I, [_P, _I, _I64, _P, _P, _P]),
    "edgpu_mlp_adam": (_I, [_P, _P, _P, _P, _I64, C.c_float, C.c_float, C.c_float, C.c_float, _P]),
    "edgpu_mlp_to_bf16": (_I, [_P, _I, _I, _P, _P, _P]),
    "edgpu_cfrac": (_I, [_P, _P, _P, _I, _I, _P, _I, _D, _P, _P, _P, _P]),
    "edgpu_cfrac_f32_workspace": (_SZ, [_I, _I]),
    "edgpu_cfrac_f32": (_I, [_P, _P, _P, _I, _I, _P, _I, _D, _P, _P, _P, _P, _SZ, _P]),
}

_lib = None


class EdgpuError(RuntimeError):
    def __init__(self, status, where=""):
        self.status = status
        msg = _status_string(status)
        super().__init__("edgpu %s failed: %s (status %d)" % (where, msg, status))


def _status_string(status):
    try:
        return load().edgpu_status_string(int(status)).decode()
    except Exception:
        return "status %d" % status


def load(path=None):
    """Load ``libedgpu.so`` and declare its signatures (raises if it is missing)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(
            "libedgpu.so not found at %s; build it with `python -m impuritymodel_gb300.nvcc_build` "
            "(there is no CPU fallback)" % p
        )
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def noalloc_bytes():
    """Size of the static scratch array of ``edgpu_lanczos_noalloc``, read from the library."""
    return int(load().edgpu_lanczos_noalloc_bytes())


def check(rc, where):
    if rc != EDGPU_OK:
        raise EdgpuError(rc, where)
