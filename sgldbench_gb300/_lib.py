"""ctypes binding of ``libsgld_gb300.so`` (the C ABI of ``include/sgld_gpu.h``).

The library is the product: there is no CPU fallback.  ``load()`` raises if
the shared library is missing or cannot be loaded, so every caller fails
loudly instead of silently computing something else.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsgld_gb300.so")

SGLD_OK = 0
SGLD_PREC_FP64 = 0
SGLD_PREC_MIXED = 1
SGLD_PREC_MIXED_DF = 2

# exported symbols and their signatures (mirrors include/sgld_gpu.h)
vp, i32, i64, dbl = C.c_void_p, C.c_int, C.c_int64, C.c_double


class Options(C.Structure):
    _fields_ = [("num_levels", i32), ("non_dyadic", i32), ("poisson_ratio", dbl), ("cell_size", dbl),
                ("omega", dbl), ("device", i32)]


class SolveOpts(C.Structure):
    _fields_ = [("tol", dbl), ("maxit", i32), ("use_x0", i32), ("precision", i32), ("inner_its", i32),
                ("history", vp), ("profile", i32), ("inner_tol", dbl)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", i32), ("converged", i32), ("relres", dbl), ("true_relres", dbl),
                ("inner_iterations", i32), ("seconds", dbl), ("kbyu_seconds", dbl), ("kbyu_launches", i32),
                ("precond_seconds", dbl), ("fallback", i32), ("replacements", i32)]


class CasesStats(C.Structure):
    _fields_ = [("diagnostics", i32), ("basis", i32), ("net_used", i32), ("net_accepted", i32), ("net_ratio", dbl),
                ("basis_ratio", dbl), ("start_ratio", dbl), ("net_loss_before", dbl), ("net_loss", dbl), ("t_start", dbl), ("t_solve", dbl),
                ("t_train", dbl)]


class TopOptOpts(C.Structure):
    _fields_ = [("volfrac", dbl), ("rmin", dbl), ("move", dbl), ("n_loop", i32), ("min_change", dbl),
                ("max_sharpness", dbl), ("penalty", dbl), ("E0", dbl), ("Emin", dbl), ("solve", SolveOpts),
                ("optimizer", i32), ("learned", i32), ("net_level", i32), ("net_train_steps", i32),
                ("net_lr", C.c_float), ("xphys0", vp), ("U0", vp), ("loop0", i32), ("x_out", vp)]


class TopOptProjectedOpts(C.Structure):
    _fields_ = [("constraint", i32), ("volfrac", dbl), ("rmin", dbl), ("rhat", dbl), ("alpha", dbl), ("pnorm", dbl), ("move", dbl), ("n_loop", i32),
                ("min_change", dbl), ("max_sharpness", dbl), ("simp_penalty", dbl), ("penalty", dbl),
                ("penalty_increment", dbl), ("penalty_interval", i32), ("beta", dbl), ("eta", dbl),
                ("beta_max", dbl), ("beta_interval", i32), ("E0", dbl), ("Emin", dbl), ("solve", SolveOpts)]


class TopOptIter(C.Structure):
    _fields_ = [("loop", i32), ("cg_iterations", i32), ("compliance", dbl), ("volume", dbl), ("sharpness", dbl),
                ("change", dbl), ("constraint", dbl), ("t_assemble", dbl), ("t_solve", dbl), ("t_opt", dbl),
                ("t_filter", dbl), ("net_used", i32), ("net_accepted", i32), ("net_r0_ratio", dbl),
                ("ext_r0_ratio", dbl),
                ("net_loss", dbl), ("t_net", dbl), ("inner_iterations", i32)]


SIGNATURES = {
    "sgld_default_options": (None, [vp]),
    "sgld_reference_num_levels": (i32, [i64, i64]),
    "sgld_create": (i32, [i32, i32, i32, vp, vp, vp]),
    "sgld_destroy": (None, [vp]),
    "sgld_last_error": (C.c_char_p, [vp]),
    "sgld_level_info": (i32, [vp, i32, vp, vp, vp, vp]),
    "sgld_num_levels": (i32, [vp]),
    "sgld_node_map": (i32, [vp, i32, vp]),
    "sgld_element_map": (i32, [vp, i32, vp]),
    "sgld_get_ke": (i32, [vp, vp]),
    "sgld_set_ke": (i32, [vp, vp]),
    "sgld_set_fixed_dofs": (i32, [vp, vp]),
    "sgld_get_free_dofs": (i32, [vp, i32, vp]),
    "sgld_set_modulus": (i32, [vp, vp]),
    "sgld_set_modulus_device": (i32, [vp, vp]),
    "sgld_assemble": (i32, [vp]),
    "sgld_get_diag": (i32, [vp, i32, vp]),
    "sgld_get_ks": (i32, [vp, i32, vp]),
    "sgld_kbyu": (i32, [vp, vp, vp]),
    "sgld_kbyu_df": (i32, [vp, vp, vp]),
    "sgld_kbyu_prec": (i32, [vp, vp, vp, i32]),
    "sgld_vcycle_prec": (i32, [vp, vp, vp, i32]),
    "sgld_build_hierarchy": (i32, [vp, i32, i32]),
    "sgld_kbyu_device": (i32, [vp, vp, vp]),
    "sgld_restrict": (i32, [vp, i32, vp, vp]),
    "sgld_restrict_prec": (i32, [vp, i32, vp, vp, i32]),
    "sgld_interpolate": (i32, [vp, i32, vp, vp]),
    "sgld_vcycle": (i32, [vp, vp, vp]),
    "sgld_pcg": (i32, [vp, vp, vp, vp, vp]),
    "sgld_pcg_device": (i32, [vp, vp, vp, vp, vp]),
    "sgld_solve_block": (i32, [vp, i32, vp, vp, vp, vp]),
    "sgld_solve": (i32, [vp, i32, vp, vp, dbl, i32, i32, vp, vp]),
    "sgld_compliance": (i32, [vp, vp, vp, vp]),
    "sgld_stress": (i32, [vp, vp, vp, vp, vp]),
    "sgld_vonmises": (i32, [vp, vp, vp, vp]),
    "sgld_principal_stress": (i32, [vp, vp, vp, vp]),
    "sgld_pde_filter": (i32, [vp, dbl, vp, vp, dbl, i32, vp]),
    "sgld_mma_update": (i32, [vp, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    "sgld_set_passive": (i32, [vp, i64, vp]),
    "sgld_get_stream": (vp, [vp]),
    "sgld_kernel_launches": (i64, []),
    "sgld_time_op": (i32, [vp, i32, i32, vp]),
    "sgld_kbyu_tile": (i32, [vp, vp, vp]),
    "sgld_inject_fault": (i32, [vp, i32]),
    "sgld_net_create": (i32, [i32, i32, i32, i32, i32, i32, vp, C.c_ulonglong, vp]),
    "sgld_net_destroy": (None, [vp]),
    "sgld_net_last_error": (C.c_char_p, [vp]),
    "sgld_net_num_params": (i64, [vp]),
    "sgld_net_get_params": (i32, [vp, vp]),
    "sgld_net_set_params": (i32, [vp, vp]),
    "sgld_net_forward": (i32, [vp, vp, vp]),
    "sgld_net_grad": (i32, [vp, vp, vp, vp, vp, vp]),
    "sgld_net_train_step": (i32, [vp, vp, vp, vp, C.c_float, vp]),
    "sgld_kbyu_dot_noalloc": (i32, [vp, vp, vp, vp, vp]),
    "sgld_density_filter": (i32, [vp, dbl, vp, vp]),
    "sgld_topopt": (i32, [vp, vp, vp, vp, vp, vp, vp]),
    "sgld_topopt_displacement": (i32, [vp, vp]),
    "sgld_topopt_projected": (i32, [vp, vp, vp, vp, vp, vp]),
    "sgld_cases_create": (i32, [vp, i32, i32, i32, vp]),
    "sgld_cases_destroy": (None, [vp]),
    "sgld_cases_basis_size": (i32, [vp]),
    "sgld_cases_solve": (i32, [vp, vp, vp, vp, i32, i32, vp, vp]),
    "sgld_cases_solve_device": (i32, [vp, vp, vp, vp, i32, i32, vp, vp]),
}

_lib = None


class SgldError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"sgld error {code}: {msg}")
        self.code = code


def load(path: str = LIB_PATH):
    """Load the CUDA library (raises if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is not built; run sgldbench_gb300.build.build() "
                          "(or __graft_entry__.build()) first")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib
