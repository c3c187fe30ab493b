"""ctypes binding of the C ABI in include/vfvm_gb300.h.

The library is the product: there is no CPU fallback.  If the shared library is
missing or no CUDA device is present, calls fail with a RuntimeError.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

P = ctypes.POINTER
c_d, c_i32, c_i64, c_vp = ctypes.c_double, ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p

# status codes (vfvm_gb300.h)
OK, ERR_CONVERGENCE, ERR_ASSEMBLY, ERR_LINEAR, ERR_TIMEOUT, ERR_INPUT, ERR_CUDA, ERR_EMBEDDING = range(8)
ERR_NOALLOC_LIMIT = 8
NOALLOC_MAX_ROWS = 131072  # VFVM_NOALLOC_MAX_ROWS
COARSE_MAX = 208           # VFVM_COARSE_MAX

PHYSICS_IDS = {
    "ex105": 1, "ex106": 2, "ex110": 3, "ex160": 4, "ex207": 5, "ex301": 6, "ex440": 7,
    "laplace_dirichlet": 8, "nlpoisson": 11, "porous": 12, "bipolar": 13, "rd2": 14, "kappa_exp": 15,
    "surface_heat": 16, "boundary_species": 17, "edge_reaction": 18, "joule_heat": 19, "ex161": 20,
    "testfunction": 21, "ex430": 22, "outflow": 23, "ex210": 24, "ex102": 25, "ex107": 26, "ex115": 27,
    "ex215": 28, "ex220": 29, "ex203": 30,
}
# physics whose first parameters carry derivatives (NPD in the device functor)
PHYSICS_NPD = {22: 1}


def physics_npd(physics_id: int) -> int:
    return PHYSICS_NPD.get(physics_id, 0)


PHYSICS_NSPEC = {1: 1, 2: 1, 3: 2, 4: 2, 5: 1, 6: 1, 7: 1, 8: 1, 11: 1, 12: 1, 13: 3, 14: 2, 15: 1, 16: 1, 17: 2, 18: 1, 19: 2, 20: 3, 21: 1, 22: 1, 23: 2, 24: 2,
                 25: 1, 26: 1, 27: 3, 28: 2, 29: 3, 30: 1}

KRYLOV = {"bicgstab": 0, "gmres": 1}
PRECON = {"jacobi": 0, "ilu0": 1, "block_ilu0": 2}
PRECISION = {"fp64": 0, "mixed": 1}
ENGINE = {"graph": 0, "persistent": 1, "auto": 2}
COORD = {"cartesian": 0, "polar1d": 1, "spherical1d": 2, "cylindrical2d": 3}  # VFVM_COORD_*


class Grid_t(ctypes.Structure):
    _fields_ = [("dim", c_i32), ("nnodes", c_i32), ("ncells", c_i32), ("nbfaces", c_i32),
                ("coord", P(c_d)), ("cellnodes", P(c_i32)), ("cellregions", P(c_i32)),
                ("bfacenodes", P(c_i32)), ("bfaceregions", P(c_i32)), ("coordsystem", c_i32)]


class Physics_t(ctypes.Structure):
    _fields_ = [("physics_id", c_i32), ("nparams", c_i32), ("params", P(c_d)),
                ("nnodedata", c_i32), ("nodedata", P(c_d)),
                ("nbregions", c_i32), ("bfactors", P(c_d)), ("bvalues", P(c_d)),
                ("ncellregions_species", c_i32), ("region_species", P(c_i32)),
                ("nbregions_species", c_i32), ("bregion_species", P(c_i32))]


class Control_t(ctypes.Structure):
    _fields_ = [("abstol", c_d), ("reltol", c_d), ("maxiters", c_i32),
                ("tol_round", c_d), ("tol_mono", c_d), ("damp_initial", c_d), ("damp_growth", c_d),
                ("max_round", c_i32), ("is_linear", c_i32), ("updatecontrol", c_i32),
                ("reltol_linear", c_d), ("abstol_linear", c_d), ("maxiters_linear", c_i32),
                ("krylov", c_i32), ("precon", c_i32), ("precision", c_i32), ("gmres_restart", c_i32),
                ("dt", c_d), ("dt_min", c_d), ("dt_max", c_d), ("dt_grow", c_d), ("dt_decrease", c_d),
                ("dp", c_d), ("dp_min", c_d), ("dp_max", c_d), ("dp_grow", c_d), ("dp_decrease", c_d),
                ("du_opt", c_d), ("du_max_factor", c_d),
                ("num_final_steps", c_i32), ("force_first_step", c_i32), ("handle_exceptions", c_i32),
                ("store_all", c_i32), ("engine", c_i32), ("team_ctas", c_i32),
                ("coarse", c_i32), ("batch_krylov_tail", c_i32)]


class History_t(ctypes.Structure):
    _fields_ = [("nnewton", c_i32), ("nlin", c_i32), ("nsteps", c_i32), ("status", c_i32),
                ("updatenorm", c_d), ("resnorm", c_d), ("time_ms", c_d), ("tasm_ms", c_d),
                ("tlinsolve_ms", c_d)]


# exported symbol -> (restype, argtypes)
SIGNATURES = {
    "vfvm_control_default": (None, [P(Control_t)]),
    "vfvm_create": (c_vp, [P(Grid_t), P(Physics_t), P(ctypes.c_int)]),
    "vfvm_destroy": (None, [c_vp]),
    "vfvm_info": (ctypes.c_int, [c_vp, P(c_i64)]),
    "vfvm_pattern": (ctypes.c_int, [c_vp, P(c_i64), P(c_i32)]),
    "vfvm_geometry": (ctypes.c_int, [c_vp, P(c_d), P(c_d), P(c_i32)]),
    "vfvm_set_params": (ctypes.c_int, [c_vp, P(c_d), c_i32]),
    "vfvm_init_dirichlet": (ctypes.c_int, [c_vp, P(c_d), c_d, c_d]),
    "vfvm_integrate": (ctypes.c_int, [c_vp, P(c_d), P(c_d), P(c_d), c_d, c_d, P(c_d)]),
    "vfvm_mass_matrix": (ctypes.c_int, [c_vp, P(c_d)]),
    "vfvm_parameter_derivatives": (ctypes.c_int, [c_vp, P(c_d), c_d, c_d, c_d, P(c_d), P(c_i32)]),
    "vfvm_assemble": (ctypes.c_int, [c_vp, P(c_d), P(c_d), c_d, c_d, c_d, P(c_d), P(c_d)]),
    "vfvm_solve": (ctypes.c_int, [c_vp, P(Control_t), P(c_d), P(c_d), c_d, c_d, c_d, P(History_t)]),
    "vfvm_evolve": (ctypes.c_int, [c_vp, P(Control_t), P(c_d), P(c_d), c_i32, c_i32, c_d, P(c_d), P(c_d),
                                   c_i32, P(c_i32), P(History_t)]),
    "vfvm_evolve_device": (ctypes.c_int, [c_vp, P(Control_t), P(c_d), P(c_d), c_i32, c_i32, c_d, P(c_d), P(c_d),
                                          c_i32, P(c_i32), P(History_t), P(c_i32)]),
    "vfvm_solve_device": (ctypes.c_int, [c_vp, P(Control_t), c_vp, c_vp, c_d, c_d, c_d, P(History_t)]),
    "vfvm_evolve_fixed_device": (ctypes.c_int, [c_vp, P(Control_t), c_vp, c_d, c_d, c_i32, P(History_t)]),
    "vfvm_stream": (c_vp, [c_vp]),
    "vfvm_assemble_device": (ctypes.c_int, [c_vp, c_vp, c_vp, c_d, c_d, c_d, c_vp, c_i32]),
    "vfvm_linsolve_csr": (ctypes.c_int, [c_i32, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_d, c_d, c_i32, P(c_i32),
                                         P(c_d)]),
    "vfvm_batch_create": (c_vp, [c_i32, P(Grid_t), P(Physics_t), P(ctypes.c_int)]),
    "vfvm_batch_destroy": (None, [c_vp]),
    "vfvm_batch_offsets": (ctypes.c_int, [c_vp, P(c_i64)]),
    "vfvm_batch_info": (ctypes.c_int, [c_vp, P(c_i64)]),
    "vfvm_batch_set_instance": (ctypes.c_int, [c_vp, c_i32, P(c_d), c_i32, P(c_d), c_i32]),
    "vfvm_batch_load_device": (ctypes.c_int, [c_vp, c_vp, c_i32, c_vp, c_i32]),
    "vfvm_set_nodedata": (ctypes.c_int, [c_vp, P(c_d), c_i32]),
    "vfvm_batch_solve": (ctypes.c_int, [c_vp, P(Control_t), P(c_d), P(c_d), c_d, c_d, c_d, P(History_t)]),
    "vfvm_batch_solve_device": (ctypes.c_int, [c_vp, P(Control_t), c_vp, c_vp, c_d, c_d, c_d, P(History_t)]),
    "vfvm_batch_solve_guarded_device": (ctypes.c_int, [c_vp, P(Control_t), c_vp, c_vp, c_vp, c_d, c_d, c_d,
                                                       P(History_t), P(c_i32)]),
    "vfvm_batch_tune": (ctypes.c_int, [c_vp, P(Control_t), c_vp, P(c_i32), P(ctypes.c_float), c_i32, P(c_i32)]),
    "vfvm_linsolve_csr_noalloc": (ctypes.c_int, [c_i32, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_d, c_d, c_i32,
                                                 P(c_i32), P(c_d)]),
    "vfvm_mlp_create": (c_vp, [c_i32, P(c_i32), c_i32, ctypes.c_uint64, P(ctypes.c_int)]),
    "vfvm_mlp_destroy": (None, [c_vp]),
    "vfvm_mlp_nparams": (ctypes.c_int, [c_vp, P(c_i64)]),
    "vfvm_mlp_params": (ctypes.c_int, [c_vp, P(ctypes.c_float), P(ctypes.c_float)]),
    "vfvm_mlp_forward": (ctypes.c_int, [c_vp, c_i32, c_vp, c_vp]),
    "vfvm_mlp_gradients": (ctypes.c_int, [c_vp, c_i32, c_vp, c_vp, P(ctypes.c_float), P(ctypes.c_float)]),
    "vfvm_mlp_train_step": (ctypes.c_int, [c_vp, c_i32, c_vp, c_vp, ctypes.c_float, P(ctypes.c_float)]),
    "vfvm_prolong_bilinear": (ctypes.c_int, [c_i32, c_i32, c_i32, c_vp, c_i64, c_d, c_d, c_vp, c_vp, c_i64, c_vp]),
    "vfvm_check_bounded_wait": (ctypes.c_int, [c_i32, P(c_i32), P(ctypes.c_float)]),
    "vfvm_coarse_log_features": (ctypes.c_int, [c_i32, c_i32, c_i32, c_i32, c_vp, c_i64, c_vp, c_vp, c_vp]),
}

_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the CUDA library (building it first when asked)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build_library()
        else:
            raise RuntimeError(f"CUDA library not built: {path} (run __graft_entry__.build())")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def ptr(a, ct=c_d):
    return a.ctypes.data_as(P(ct))
