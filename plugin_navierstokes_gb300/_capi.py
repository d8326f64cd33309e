"""ctypes binding of the native C ABI (include/nsfv1_gb300.h).

The library ``lib/libnsfv1_gb300.so`` is built in-tree by ``build.py``. There is
no fallback: if the library is missing, ``load()`` raises.
"""
from __future__ import annotations

import ctypes
import re
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_void_p
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "lib" / "libnsfv1_gb300.so"
HEADER = HERE.parent / "include" / "nsfv1_gb300.h"

OK = 0
ERR_ARGUMENT = 1
ERR_STATE = 2
ERR_CUDA = 3
ERR_NOT_CONVERGED = 4
ERR_BREAKDOWN = 5
ERR_NONFINITE = 6
ERR_GEOMETRY = 7
ERR_TIMEOUT = 8

TRIANGLE = 2
QUADRILATERAL = 3
TETRAHEDRON = 4
PRISM = 6
HEXAHEDRON = 8
NSH = {TRIANGLE: 3, QUADRILATERAL: 4, TETRAHEDRON: 4, PRISM: 6, HEXAHEDRON: 8}
DIM = {TRIANGLE: 2, QUADRILATERAL: 2, TETRAHEDRON: 3, PRISM: 3, HEXAHEDRON: 3}

F64 = 0
F32 = 1
BICGSTAB = 0
GMRES = 1

STATUS_NAMES = {
    OK: "ok", ERR_ARGUMENT: "argument", ERR_STATE: "state", ERR_CUDA: "cuda", ERR_NOT_CONVERGED: "not_converged",
    ERR_BREAKDOWN: "breakdown", ERR_NONFINITE: "nonfinite", ERR_GEOMETRY: "geometry", ERR_TIMEOUT: "timeout",
}


class NewtonParams(ctypes.Structure):
    _fields_ = [
        ("rtol", c_double), ("atol", c_double), ("max_iter", c_int), ("lin_rtol", c_double), ("lin_max_iter", c_int),
        ("line_search_steps", c_int), ("jacobian_prec", c_int), ("linear_solver", c_int), ("gmres_restart", c_int),
    ]


class NewtonResult(ctypes.Structure):
    _fields_ = [
        ("iterations", c_int), ("linear_iterations", c_int), ("initial_defect", c_double), ("final_defect", c_double),
        ("status", c_int),
    ]


class BatchOptions(ctypes.Structure):
    _fields_ = [("cluster_size", c_int), ("max_clusters", c_int), ("mg_levels", c_int), ("smooth_steps", c_int),
                ("coarse_steps", c_int), ("smooth_omega", c_double), ("defect_reference", c_int), ("zero_fallback", c_int),
                ("forcing_max", c_double), ("graph", c_int), ("tail_clusters", c_int)]


class MlpConfig(ctypes.Structure):
    _fields_ = [("max_points", c_int), ("max_slots", c_int)]


class MlpDataset(ctypes.Structure):
    _fields_ = [("n_train", ctypes.c_int64), ("n_nodes", ctypes.c_int64), ("coords", c_void_p), ("targets", c_void_p),
                ("cond", c_void_p)]


class MlpTrainParams(ctypes.Structure):
    _fields_ = [("steps", c_int), ("slots", c_int), ("points_per_slot", c_int), ("lr", ctypes.c_float),
                ("lr_final", ctypes.c_float), ("seed", ctypes.c_uint64), ("step_offset", ctypes.c_int64)]


class NSFV1Error(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{STATUS_NAMES.get(status, status)}] {message}")
        self.status = status


_lib = None

_SIGS = {
    "nsfv1_create": (c_int, [c_int, POINTER(c_void_p)]),
    "nsfv1_destroy": (c_int, [c_void_p]),
    "nsfv1_last_error": (c_char_p, [c_void_p]),
    "nsfv1_disc_type": (c_char_p, [c_void_p]),
    "nsfv1_set_kinematic_viscosity": (c_int, [c_void_p, c_double]),
    "nsfv1_set_density": (c_int, [c_void_p, c_double]),
    "nsfv1_set_source": (c_int, [c_void_p, c_void_p, c_int]),
    "nsfv1_set_exact_jacobian": (c_int, [c_void_p, c_double]),
    "nsfv1_set_stokes": (c_int, [c_void_p, c_int]),
    "nsfv1_set_laplace": (c_int, [c_void_p, c_int]),
    "nsfv1_set_peclet_blend": (c_int, [c_void_p, c_int]),
    "nsfv1_set_upwind": (c_int, [c_void_p, c_char_p]),
    "nsfv1_set_stabilization": (c_int, [c_void_p, c_char_p, c_char_p]),
    "nsfv1_set_stabilization_upwind": (c_int, [c_void_p, c_char_p]),
    "nsfv1_set_pac_upwind": (c_int, [c_void_p, c_int]),
    "nsfv1_set_mesh": (c_int, [c_void_p, c_int, c_int64, c_void_p, c_int64, c_void_p]),
    "nsfv1_pattern_info": (c_int, [c_void_p, POINTER(c_int64), POINTER(c_int64), POINTER(c_int), POINTER(c_int)]),
    "nsfv1_mesh_pattern": (c_int, [c_int, c_int64, c_int64, c_void_p, POINTER(c_int64), POINTER(c_int), c_void_p, c_void_p, c_void_p]),
    "nsfv1_get_pattern": (c_int, [c_void_p, c_void_p, c_void_p]),
    "nsfv1_get_coloring": (c_int, [c_void_p, c_void_p]),
    "nsfv1_device_pattern": (c_int, [c_void_p, POINTER(c_void_p), POINTER(c_void_p)]),
    "nsfv1_set_dirichlet": (c_int, [c_void_p, c_int64, c_void_p, c_void_p]),
    "nsfv1_add_dirichlet": (c_int, [c_void_p, c_int64, c_void_p, c_void_p]),
    "nsfv1_add_wall": (c_int, [c_void_p, c_int64, c_void_p]),
    "nsfv1_add_inflow": (c_int, [c_void_p, c_int64, c_int, c_void_p, c_void_p]),
    "nsfv1_clear_boundary": (c_int, [c_void_p]),
    "nsfv1_add_outflow": (c_int, [c_void_p, c_int64, c_int, c_void_p]),
    "nsfv1_assemble_defect": (c_int, [c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_void_p]),
    "nsfv1_assemble_jacobian": (c_int, [c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_int, c_void_p]),
    "nsfv1_assemble_defect_jacobian": (c_int, [c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_void_p, c_int, c_void_p]),
    "nsfv1_elem_batch": (c_int, [c_void_p, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_void_p,
                                 c_void_p, c_void_p, c_void_p, c_void_p]),
    "nsfv1_elem_batch_host": (c_int, [c_void_p, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_void_p]),
    "nsfv1_vorticity": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "nsfv1_eval_points": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_int, c_void_p, c_void_p]),
    "nsfv1_export": (c_int, [c_void_p, c_int, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_double, c_int, c_int, c_void_p,
                             c_void_p, c_void_p, c_void_p]),
    "nsfv1_bsr_mv": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "nsfv1_split_vector": (c_int, [c_int64, c_void_p, c_void_p, c_void_p]),
    "nsfv1_bsr_mv_split": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "nsfv1_block_jacobi": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "nsfv1_block_jacobi_noalloc": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "nsfv1_newton_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_double, POINTER(NewtonParams), POINTER(NewtonResult), c_void_p]),
    "nsfv1_linear_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, POINTER(NewtonParams), POINTER(c_int), POINTER(c_double),
                                   POINTER(c_int), c_void_p]),
    "nsfv1_set_elem_viscosity": (c_int, [c_void_p, c_void_p]),
    "nsfv1_set_instances": (c_int, [c_void_p, c_int, c_void_p]),
    "nsfv1_set_instance_grids": (c_int, [c_void_p, c_void_p]),
    "nsfv1_newton_solve_batched": (c_int, [c_void_p, c_void_p, c_void_p, c_double, POINTER(NewtonParams), POINTER(BatchOptions),
                                           c_void_p, c_void_p]),
    "nsfv1_set_assembly_threads": (c_int, [c_void_p, c_int]),
    "nsfv1_get_assembly_threads": (c_int, [c_void_p]),
    "nsfv1_assembly_autotune": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p]),
    "nsfv1_batch_stats": (c_int, [c_void_p, c_void_p, c_int]),
    "nsfv1_batch_autotune": (c_int, [c_void_p, c_void_p, c_void_p, c_double, POINTER(NewtonParams), POINTER(BatchOptions), c_void_p,
                                     c_int, c_void_p, c_void_p]),
    "nsfv1_ref_tables": (c_int, [c_int, POINTER(c_int), POINTER(c_int), c_void_p, POINTER(c_int), c_void_p, c_void_p, c_void_p]),
    "nsfv1_mlp_create": (c_int, [POINTER(MlpConfig), POINTER(c_void_p)]),
    "nsfv1_mlp_destroy": (None, [c_void_p]),
    "nsfv1_mlp_last_error": (c_char_p, [c_void_p]),
    "nsfv1_mlp_num_params": (ctypes.c_int64, [c_void_p]),
    "nsfv1_mlp_condition": (None, [c_double, c_double, c_void_p]),
    "nsfv1_mlp_init": (c_int, [c_void_p, ctypes.c_uint64]),
    "nsfv1_mlp_get_params": (c_int, [c_void_p, c_void_p, ctypes.c_int64]),
    "nsfv1_mlp_set_params": (c_int, [c_void_p, c_void_p, ctypes.c_int64]),
    "nsfv1_mlp_forward": (c_int, [c_void_p, ctypes.c_int64, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "nsfv1_mlp_loss_grad": (c_int, [c_void_p, ctypes.c_int64, c_void_p, c_int, c_void_p, c_void_p, c_void_p, POINTER(c_double),
                                    c_void_p, c_void_p]),
    "nsfv1_mlp_train": (c_int, [c_void_p, POINTER(MlpDataset), POINTER(MlpTrainParams), c_void_p, c_void_p]),
    "nsfv1_mlp_targets": (c_int, [ctypes.c_int64, ctypes.c_int64, c_void_p, c_void_p, c_void_p, c_void_p]),
    "nsfv1_mlp_predict": (c_int, [c_void_p, ctypes.c_int64, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "nsfv1_gemm_bf16": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "nsfv1_gemm_bf16_splits": (c_int, [c_int, c_int]),
}


NOALLOC_MAX_NODES = 32768


def header_symbols() -> list[str]:
    """Every function declared in include/nsfv1_gb300.h."""
    txt = HEADER.read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(nsfv1_[a-z0-9_]+)\s*\(", txt)))


def load() -> ctypes.CDLL:
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"native library missing: {LIB_PATH} (run plugin_navierstokes_gb300/build.py)")
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(h, status: int) -> None:
    if status != OK:
        msg = load().nsfv1_last_error(h).decode() if h else ""
        raise NSFV1Error(status, msg)
