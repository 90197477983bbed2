"""ctypes binding of ``libfvgb.so`` (the C ABI declared in ``include/fvgb.h``).

The library is built in-tree by ``aquaflux_gb300.build.build_library`` (``__graft_entry__.build()``).
There is no CPU fallback: every entry point of this package runs on the CUDA library, and importing
:func:`lib` without it raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfvgb.so")

c_int, c_long, c_double, c_void_p, c_char_p = (ctypes.c_int, ctypes.c_long, ctypes.c_double,
                                               ctypes.c_void_p, ctypes.c_char_p)
P = ctypes.c_void_p  # device / host pointers are passed as integers

FV_OK, FV_ERR_ARG, FV_ERR_CUDA, FV_ERR_NO_DIAG, FV_ERR_ZERO_PIVOT = 0, 1, 2, 3, 4
FV_ERR_NONFINITE, FV_ERR_NOT_CONVERGED, FV_ERR_TIMEOUT = 5, 6, 7


class FvCaseDesc(ctypes.Structure):
    _fields_ = [("turbulent", c_int), ("mu", c_double), ("rho", c_double),
                ("pressure_pin", c_int), ("pressure_pin_value", c_double),
                ("gradient_sweeps", c_int), ("gradient_relaxation", c_double),
                ("advection", c_int), ("limiter_k", c_double),
                ("scalar_transform", c_int), ("scalar_advection", c_int),
                ("scalar_limiter_k", c_double)]


# name -> (restype, argtypes); this table is the binding a ctypes user of the C ABI adds.
SIGNATURES = {
    "fv_last_error": (c_char_p, []),
    "fv_last_error_index": (c_long, []),
    "fv_version": (c_char_p, []),
    "fv_mesh_create": (c_int, [c_int, c_int, c_int, c_int, P, P, P, P, P, P, P]),
    "fv_mesh_destroy": (c_int, [P]),
    "fv_mesh_set_nodes": (c_int, [P, P, P]),
    "fv_case_refresh_geometry": (c_int, [P, P]),
    "fv_mesh_geometry": (c_int, [P, P, P, P, P, P, P]),
    "fv_mesh_sizes": (c_int, [P, P, P, P, P]),
    "fv_case_create": (c_int, [P, ctypes.POINTER(FvCaseDesc), P, P, P, P, P, P, P, P, P, P]),
    "fv_case_destroy": (c_int, [P]),
    "fv_case_set_params": (c_int, [P, c_double, c_double]),
    "fv_case_wall_distance": (c_int, [P, P, P, P]),
    "fv_case_set_wall_distance": (c_int, [P, P, P]),
    "fv_case_n_unknowns": (c_long, [P]),
    "fv_case_profile_begin": (c_int, [P, c_int]),
    "fv_case_profile_end": (c_int, [P, P, c_int, P]),
    "fv_residual": (c_int, [P, P, P, P]),
    "fv_eddy_viscosity": (c_int, [P, P, P, P]),
    "fv_jvp": (c_int, [P, P, P, P, P, P]),
    "fv_jvp_shift": (c_int, [P, P, P, P, P, P]),
    "fv_jvp_frozen": (c_int, [P, P, P, P, P]),
    "fv_linearise": (c_int, [P, P, P, P]),
    "fv_jvp_linearised": (c_int, [P, P, P, P, P, P]),
    "fv_probe_jacobian": (c_int, [P, P, c_int, P, c_int, P, P, P, P]),
    "fv_jvp_batch": (c_int, [P, P, P, c_int, P, P]),
    "fv_node_vjp": (c_int, [P, P, P, P, P]),
    "fv_hold_forward": (c_int, [P, P, P, P]),
    "fv_vjp_held": (c_int, [P, P, P, P, P]),
    "fv_case_set_viscosity_field": (c_int, [P, P, P]),
    "fv_case_set_block_size": (c_int, [P, c_int]),
    "fv_case_set_persistent": (c_int, [P, c_int, c_int, c_int]),
    "fv_case_set_cell_order": (c_int, [P, c_int, P]),
    "fv_case_autotune_persistent": (c_int, [P, P, P, P, P, P, P, P]),
    "fv_case_autotune": (c_int, [P, P, P, P, P, P]),
    "fv_case_block_sizes": (c_int, [P, P, c_int]),
    "fv_segment_dot": (c_int, [c_int, P, c_int, c_int, P, P, P, P]),
    "fv_face_functional": (c_int, [P, P, P, c_int, P, P, P, P, P]),
    "fv_assemble_jacobian": (c_int, [P, P, P, P, P, P]),
    "fv_assemble_jacobian_f32": (c_int, [P, P, P, P, P, P]),
    "fv_jvp_f32": (c_int, [P, P, P, P, P]),
    "fv_param_jvp": (c_int, [P, P, P, P, P]),
    "fv_vjp": (c_int, [P, P, P, P, P, P]),
    "fv_param_vjp": (c_int, [P, P, P, P, P]),
    "fv_bsr_spmv_f64": (c_int, [c_int, c_int, P, P, P, P, P, c_int, P]),
    "fv_bsr_spmv_f32": (c_int, [c_int, c_int, P, P, P, P, P, c_int, P]),
    "fv_bsr_spmv_t_f64_noalloc": (c_int, [c_int, c_long, c_int, P, P, P, P, P, P]),
    "fv_ilu0_create": (c_int, [c_int, c_int, P, P, c_int, P, P]),
    "fv_ilu0_clone": (c_int, [P, c_int, P, P]),
    "fv_ilu0_destroy": (c_int, [P]),
    "fv_ilu0_factor": (c_int, [P, P, c_int, P]),
    "fv_ilu0_apply": (c_int, [P, P, P, c_int, P]),
    "fv_ilu0_factor_values": (c_int, [P, P, P]),
    "fv_dot_f64": (c_int, [c_long, P, P, P, P]),
    "fv_cell_graph": (c_int, [c_int, c_long, P, P, P, P, P, P]),
    "fv_rcm_permutation": (c_int, [c_int, P, P, P, P, P, P]),
    "fv_krylov_create": (c_int, [c_int, P]),
    "fv_krylov_destroy": (c_int, [P]),
    "fv_krylov_start": (c_int, [P, c_long, P, P, P, P]),
    "fv_krylov_arnoldi": (c_int, [P, c_int, c_long, P, P, P, P]),
    "fv_krylov_update": (c_int, [P, c_int, c_long, P, P, P]),
    "fv_krylov_norm": (c_int, [P, c_long, P, P, P]),
    "fv_saturation_colouring": (c_int, [c_int, P, P, P, P]),
    "fv_greedy_colouring": (c_int, [c_int, P, P, P, P]),
    "fv_coarsen": (c_int, [c_int, P, P, P, c_int, P, P, P, P, P, P, P]),
    "fv_colour_aggregates": (c_int, [c_int, P, P, P, c_int, P, P]),
    "fv_cell_pattern": (c_int, [c_int, c_long, P, P, P, P]),
    "fv_aggregate": (c_int, [c_int, P, P, P, P]),
    "fv_galerkin_f32": (c_int, [c_long, c_int, P, P, P, c_int, P, P]),
    "fv_restrict_f32": (c_int, [c_int, c_int, P, P, P, P, P]),
    "fv_prolong_add_f32": (c_int, [c_int, c_int, P, P, P, P]),
    "fv_galerkin_f64": (c_int, [c_long, c_int, P, P, P, c_int, P, P]),
    "fv_permute_pattern": (c_int, [c_int, P, P, P, P, P, P]),
    "fv_gather_blocks": (c_int, [c_long, c_int, P, P, c_int, P, c_int, P]),
    "fv_to_cells": (c_int, [c_int, c_int, P, P, P, P, c_int, P]),
    "fv_from_cells": (c_int, [c_int, c_int, P, P, P, c_int, P, P]),
    "fv_bsr_transpose_map": (c_int, [c_int, P, P, P, P, P]),
    "fv_bsr_spmv_t_mapped": (c_int, [c_int, c_int, P, P, P, P, P, P, c_int, P]),
    "fv_bsr_transpose_blocks": (c_int, [c_long, c_int, P, P, P, c_int, P]),
    "fv_bsr_shift_equilibrate": (c_int, [c_int, c_int, P, P, P, P, c_int, P, P, P, c_int, P]),
    "fv_restrict_f64": (c_int, [c_int, c_int, P, P, P, P, P]),
    "fv_prolong_add_f64": (c_int, [c_int, c_int, P, P, P, P]),
}

_lib = None


class FvError(RuntimeError):
    """A non-OK status from the C ABI (code in ``.code``, associated row in ``.index``)."""

    def __init__(self, code: int, message: str, index: int = -1):
        super().__init__(f"[fv status {code}] {message}")
        self.code, self.message, self.index = code, message, index


def lib():
    """Load ``libfvgb.so`` once; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"the CUDA library {LIB_PATH} is missing: run __graft_entry__.build() "
                "(there is no CPU fallback)")
        handle = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def check(rc: int) -> None:
    if rc != FV_OK:
        L = lib()
        raise FvError(rc, L.fv_last_error().decode(), int(L.fv_last_error_index()))


def ptr(t) -> int:
    """Raw data pointer of a torch tensor (contiguous) or numpy array, or 0 for None."""
    if t is None:
        return 0
    if hasattr(t, "data_ptr"):
        return int(t.data_ptr())
    return int(t.ctypes.data)
