"""ctypes binding of libgb300fea.so (the C ABI declared in include/gfea.h).

The library is loaded from ``easyfea_gb300/lib``; there is no fallback: when
it is missing or no GPU is present, every compute entry point raises
``GfeaError``.
"""

from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_double, c_float, c_int, c_int32, c_int64, c_size_t, c_uint8, c_void_p

from . import _build

ABI_VERSION = 1

OK = 0
ERR_NOT_CONVERGED = 5
ERR_TIMEOUT = 9

F64 = 0
F32 = 1

ELEM_CODE = {"SEG2": 0, "TRI3": 1, "QUAD4": 2, "QUAD9": 3, "HEXA8": 4, "TETRA4": 5, "TRI6": 6, "QUAD8": 7,
             "TETRA10": 8, "SEG3": 9, "HEXA20": 10, "HEXA27": 11, "PRISM6": 12, "PRISM15": 13,
             "PRISM18": 14, "TRI10": 15, "TRI15": 16, "SEG4": 17, "SEG5": 18}
SPLIT_CODE = {"Bourdin": 0, "Amor": 1, "Miehe": 2, "Zhang": 3, "Stress": 4, "He": 5, "AnisotStrain": 6,
              "AnisotStrain_PM": 7, "AnisotStrain_MP": 8, "AnisotStrain_NoCross": 9, "AnisotStress": 10,
              "AnisotStress_PM": 11, "AnisotStress_MP": 12, "AnisotStress_NoCross": 13}
REGU_CODE = {"AT1": 0, "AT2": 1}


class GfeaError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        msg = _status_string(status) if _LIB is not None else str(status)
        super().__init__(f"{what}: {msg} (status {status})")


class System(ctypes.Structure):
    _fields_ = [
        ("version", c_int32),
        ("dof_n", c_int32),
        ("n_nodes", c_int64),
        ("n_pairs", c_int64),
        ("node_ptr", c_void_p),
        ("nbr", c_void_p),
        ("vals64", c_void_p),
        ("vals32", c_void_p),
        ("known", c_void_p),
        ("translation_invariant", c_int32),
        ("pad", c_int32),
        ("coord", c_void_p),
    ]


class PcgOpts(ctypes.Structure):
    _fields_ = [
        ("version", c_int32),
        ("precision", c_int32),
        ("max_iters", c_int32),
        ("check_every", c_int32),
        ("rtol", c_double),
        ("inner_rtol", c_double),
        ("max_refine", c_int32),
        ("lanes", c_int32),
        ("coarse", c_int32),
        ("coarse_reuse", c_int32),
    ]


class PcgResult(ctypes.Structure):
    _fields_ = [
        ("status", c_int32),
        ("iterations", c_int32),
        ("refinements", c_int32),
        ("pad", c_int32),
        ("rel_residual", c_double),
        ("floor_rel", c_double),
    ]


class CoarseLevel(ctypes.Structure):
    _fields_ = [
        ("n_agg", c_int32),
        ("nr", c_int32),
        ("nc", c_int32),
        ("pad", c_int32),
        ("agg", c_void_p),
        ("off", c_void_p),
        ("agg_ptr", c_void_p),
        ("agg_nodes", c_void_p),
        ("inv", c_void_p),
        ("inv32", c_void_p),
        ("rc", c_void_p),
        ("ec", c_void_p),
    ]


class BatchInstance(ctypes.Structure):
    _fields_ = [
        ("version", c_int32),
        ("dof_n", c_int32),
        ("n_nodes", c_int64),
        ("n_pairs", c_int64),
        ("node_ptr", c_void_p),
        ("nbr", c_void_p),
        ("vals64", c_void_p),
        ("vals32", c_void_p),
        ("known", c_void_p),
        ("translation_invariant", c_int32),
        ("max_iters", c_int32),
        ("rtol", c_double),
        ("b", c_void_p),
        ("x", c_void_p),
        ("work", c_void_p),
        ("result", c_void_p),
        ("coarse", CoarseLevel),
    ]


class PfParams(ctypes.Structure):
    _fields_ = [
        ("version", c_int32),
        ("split", c_int32),
        ("regularization", c_int32),
        ("dim", c_int32),
        ("lambda_", c_double),
        ("mu", c_double),
        ("Gc", c_double),
        ("l0", c_double),
        ("thickness", c_double),
        ("A", c_double * 9),
        ("C", c_double * 36),
        ("k_res", c_double),
        ("plane_stress", c_int32),
        ("pad", c_int32),
        ("S", c_double * 36),
    ]


class Fields(ctypes.Structure):
    """gfea_fields: inputs and outputs of gfea_element_fields."""

    _fields_ = [
        ("version", c_int32),
        ("gauss", c_int32),
        ("coef", c_double),
        ("thickness", c_double),
        ("C", c_void_p),
        ("c_per_elem", c_int32),
        ("pad", c_int32),
        ("pf", POINTER(PfParams)),
        ("d", c_void_p),
        ("H_old", c_void_p),
        ("sigma_n", c_void_p),
        ("strain_e", c_void_p),
        ("stress_e", c_void_p),
        ("vm_e", c_void_p),
        ("energy_e", c_void_p),
        ("psiP_e", c_void_p),
    ]


class PartPlan(ctypes.Structure):
    """gfea_part_plan: the row-owned assembly's parts and visit lists (device arrays)."""

    _fields_ = [
        ("version", c_int32),
        ("n_parts", c_int32),
        ("max_part_values", c_int32),
        ("threads", c_int32),
        ("node_off", c_void_p),
        ("part_node_ptr", c_void_p),
        ("part_nodes", c_void_p),
        ("part_nvals", c_void_p),
        ("visit_ptr", c_void_p),
        ("visit_elem", c_void_p),
        ("visit_mask", c_void_p),
    ]


_LIB = None

# name -> (restype, argtypes); the complete list of exported entry points
SIGNATURES = {
    "gfea_version": (ctypes.c_char_p, []),
    "gfea_status_string": (ctypes.c_char_p, [c_int]),
    "gfea_graph_workspace_size": (c_int, [c_int64, c_int64, c_int, POINTER(c_size_t)]),
    "gfea_graph_count": (c_int, [c_void_p, c_int64, c_int, c_int64, c_void_p, POINTER(c_int64), c_void_p,
                                 c_size_t, c_void_p]),
    "gfea_graph_fill": (c_int, [c_void_p, c_int64, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                c_size_t, c_void_p]),
    "gfea_csr_pattern": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p, c_void_p, c_void_p]),
    "gfea_assemble_elastic": (c_int, [c_int, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int,
                                      c_double, c_int, c_void_p, c_int64, c_int, c_void_p]),
    "gfea_assemble_mass": (c_int, [c_int, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_int, c_double,
                                   c_double, c_int, c_void_p, c_int64, c_int, c_void_p]),
    "gfea_surface_load": (c_int, [c_int, c_void_p, c_void_p, c_int64, c_void_p, c_int, c_int, POINTER(c_int32),
                                  POINTER(c_double), c_double, c_void_p, c_void_p]),
    "gfea_boundary_gauss_points": (c_int, [c_int, c_void_p, c_void_p, c_int64, c_void_p, POINTER(c_int32),
                                           c_void_p]),
    "gfea_surface_load_field": (c_int, [c_int, c_void_p, c_void_p, c_int64, c_void_p, c_int, c_int, c_int,
                                        c_void_p, c_double, c_void_p, c_void_p]),
    "gfea_pf_damage": (c_int, [c_int, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p,
                               POINTER(PfParams), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "gfea_pf_elastic": (c_int, [c_int, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                POINTER(PfParams), c_int, c_void_p, c_void_p]),
    "gfea_pf_split": (c_int, [c_void_p, c_int64, POINTER(PfParams), c_void_p, c_void_p, c_void_p, c_void_p,
                              c_void_p]),
    "gfea_part_plan_host": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_int64, c_void_p, c_int, c_int32,
                                    c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                    POINTER(c_int32), POINTER(c_int64)]),
    "gfea_part_smem_bytes": (c_size_t, [c_int, c_int, c_int32, c_int]),
    "gfea_assemble_elastic_parts": (c_int, [c_int, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int,
                                            c_double, c_int, c_void_p, POINTER(PartPlan), c_void_p]),
    "gfea_element_fields": (c_int, [c_int, c_void_p, c_void_p, c_int64, c_void_p, POINTER(Fields), c_void_p]),
    "gfea_node_incidence": (c_int, [c_void_p, c_int64, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_size_t,
                                    c_void_p]),
    "gfea_node_average": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int, c_void_p, c_void_p]),
    "gfea_spmv": (c_int, [POINTER(System), c_int, c_void_p, c_void_p, c_void_p]),
    "gfea_pcg_workspace_size": (c_int, [POINTER(System), POINTER(PcgOpts), POINTER(c_size_t)]),
    "gfea_pcg_solve": (c_int, [POINTER(System), c_void_p, c_void_p, POINTER(PcgOpts), c_void_p, c_size_t,
                               POINTER(PcgResult), c_void_p]),
    "gfea_pcg_solve_noalloc": (c_int, [POINTER(System), c_void_p, c_void_p, POINTER(PcgOpts), POINTER(PcgResult),
                                       c_void_p]),
    "gfea_coarse_workspace_size": (c_int, [POINTER(System), POINTER(PcgOpts), POINTER(c_size_t)]),
    "gfea_coarse_setup": (c_int, [POINTER(System), POINTER(PcgOpts), c_int, c_void_p, c_size_t, POINTER(CoarseLevel),
                                  c_void_p]),
    "gfea_coarse_batch_scratch_size": (c_size_t, [c_int]),
    "gfea_coarse_batch_prepare": (c_int, [POINTER(System), POINTER(PcgOpts), c_int, POINTER(c_void_p),
                                          POINTER(CoarseLevel), c_void_p, c_size_t, c_void_p]),
    "gfea_coarse_batch_build": (c_int, [c_void_p, c_int, POINTER(c_int32), c_int, c_int, c_void_p]),
    "gfea_batch_workspace_size": (c_size_t, [c_int64, c_int, c_int]),
    "gfea_batch_scratch_size": (c_size_t, [c_int]),
    "gfea_batch_pcg": (c_int, [POINTER(BatchInstance), c_int, c_void_p, c_size_t, POINTER(PcgOpts), c_void_p]),
    "gfea_batch_prepare": (c_int, [POINTER(BatchInstance), c_int, c_void_p, c_size_t, POINTER(PcgOpts), c_void_p]),
    "gfea_batch_launch": (c_int, [c_void_p, c_int, POINTER(PcgOpts), c_void_p]),
    "gfea_reduce_workspace_size": (c_size_t, []),
    "gfea_reaction_energy": (c_int, [POINTER(System), c_void_p, c_void_p, c_int64, c_void_p, POINTER(c_double),
                                     c_void_p, c_void_p]),
    "gfea_max_abs_diff": (c_int, [c_void_p, c_void_p, c_int64, POINTER(c_double), c_void_p, c_void_p]),
    "gfea_cast_f64_f32": (c_int, [c_void_p, c_void_p, c_int64, c_void_p]),
    "gfea_launch_count": (ctypes.c_longlong, []),
    "gfea_cuda_graph_count": (ctypes.c_longlong, []),
    "gfea_profile_enable": (c_int, [c_int]),
    "gfea_profile_read": (c_int, [POINTER(c_double), POINTER(ctypes.c_longlong)]),
    "gfea_selftest_wait": (c_int, [c_int32, c_int32, POINTER(c_int32), c_void_p]),
    "gfea_tune_mode": (c_int, [c_int]),
    "gfea_tune_clear": (c_int, []),
    "gfea_tune_spmv": (c_int, [POINTER(System), c_int, c_void_p, c_void_p, POINTER(c_int32), POINTER(c_float),
                               c_void_p]),
    "gfea_tune_assemble_elastic": (c_int, [c_int, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int,
                                           c_double, c_int, c_void_p, c_int64, POINTER(c_int32), POINTER(c_float),
                                           c_void_p]),
    "gfea_tune_export": (c_int, [POINTER(c_int64), POINTER(c_int32), c_int, POINTER(c_int)]),
    "gfea_tune_import": (c_int, [POINTER(c_int64), POINTER(c_int32), c_int]),
}


def load(path: str | None = None):
    """Load (once) and return the library; raises GfeaError if it is not built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = path or _build.lib_path()
    if not os.path.exists(path):
        raise GfeaError(-1, f"{path} is not built (run __graft_entry__.build() or easyfea_gb300._build.build())")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def _status_string(status: int) -> str:
    try:
        return _LIB.gfea_status_string(status).decode()
    except Exception:  # pragma: no cover
        return str(status)


def check(status: int, what: str, allow=(OK,)):
    if status not in allow:
        raise GfeaError(status, what)
    return status


def ptr(t) -> int:
    """Device pointer of a torch tensor (None -> NULL)."""
    return 0 if t is None else t.data_ptr()


def stream() -> int:
    import torch

    return torch.cuda.current_stream().cuda_stream


def require_gpu():
    import torch

    if not torch.cuda.is_available():
        raise GfeaError(-1, "no CUDA device: the easyfea_gb300 compute path runs only on the GPU")
    load()
