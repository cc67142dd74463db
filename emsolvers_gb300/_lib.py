"""ctypes binding of libems (include/ems.h).

The shared library is built in-tree by ``emsolvers_gb300.build``; loading
fails loudly when it is missing — there is no CPU fallback.
"""
import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libems.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "ems.h")

EMS_OK = 0
FP64, FP32 = 0, 1
LEAPFROG, SYMP2, SYMP4, ABM = 0, 1, 2, 3
WAVE_REFERENCE, WAVE_RICKER = 0, 1

_lib = None


class EmsError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status


class FdtdParams(C.Structure):
    _fields_ = [("grid", C.c_int * 3), ("h", C.c_double), ("dt", C.c_double), ("permittivity", C.c_double),
                ("permeability", C.c_double), ("time_frequency", C.c_int), ("precision", C.c_int),
                ("pml_cells", C.c_int), ("pml_order", C.c_double), ("pml_kappa_max", C.c_double),
                ("pml_alpha_max", C.c_double), ("pml_reflection", C.c_double)]


class HexFemParams(C.Structure):
    _fields_ = [("order", C.c_int), ("grid", C.c_int * 3), ("h", C.c_double), ("dt", C.c_double),
                ("permittivity", C.c_double), ("permeability", C.c_double), ("time_frequency", C.c_int),
                ("use_ofem", C.c_int), ("integrator", C.c_int), ("precision", C.c_int), ("kmat_dir", C.c_char_p)]


class FemStabParams(C.Structure):
    _fields_ = [("grid", C.c_int * 3), ("h", C.c_double), ("dt", C.c_double), ("permittivity", C.c_double),
                ("permeability", C.c_double), ("time_frequency", C.c_int), ("stabilization_factor", C.c_double),
                ("use_ofem", C.c_int), ("precision", C.c_int)]


class TetFemParams(C.Structure):
    _fields_ = [("cells", C.c_int * 3), ("h", C.c_double), ("order", C.c_int), ("integrator", C.c_int),
                ("precision", C.c_int), ("dt", C.c_double), ("cfl_fraction", C.c_double),
                ("time_frequency", C.c_int)]


def declared_functions():
    """Names of the functions declared in include/ems.h."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\s*\*|void)\s*(ems_\w+)\s*\(", txt, re.M)))


def lib():
    """Loads libems.so (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build
        build.build()
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libems.so not found at {LIB_PATH}; run python -m emsolvers_gb300.build")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int)
    sig = {
        "ems_abi_version": (C.c_int, []),
        "ems_status_string": (C.c_char_p, [C.c_int]),
        "ems_last_error": (C.c_char_p, [vp]),
        "ems_device_count": (C.c_int, []),
        "ems_fdtd_create": (C.c_int, [C.POINTER(FdtdParams), C.POINTER(vp)]),
        "ems_fdtd_set_source": (C.c_int, [vp, C.c_int, ip, C.c_int, C.c_double, C.c_double]),
        "ems_fdtd_add_observation": (C.c_int, [vp, ip, C.c_int, ip, C.c_int, ip, C.c_int]),
        "ems_fdtd_set_material": (C.c_int, [vp, dp, dp]),
        "ems_hexfem_create": (C.c_int, [C.POINTER(HexFemParams), C.POINTER(vp)]),
        "ems_hexfem_set_source": (C.c_int, [vp, C.c_int, ip]),
        "ems_hexfem_add_observation": (C.c_int, [vp, ip]),
        "ems_hexfem_add_dipole": (C.c_int, [vp, ip]),
        "ems_hexfem_add_observation_edges": (C.c_int, [vp, ip, C.c_int, ip, C.c_int, ip, C.c_int]),
        "ems_femstab_create": (C.c_int, [C.POINTER(FemStabParams), C.POINTER(vp)]),
        "ems_femstab_element_matrix": (C.c_int, [vp, dp, C.c_size_t]),
        "ems_tetfem_create": (C.c_int, [C.POINTER(TetFemParams), C.POINTER(vp)]),
        "ems_tetfem_element_matrices": (C.c_int, [C.c_int, C.c_int, dp, dp, C.c_size_t]),
        "ems_tetbatch_create": (C.c_int, [C.POINTER(TetFemParams), C.c_int, ip, C.POINTER(vp)]),
        "ems_tetbatch_add_dipole": (C.c_int, [vp, C.c_int, dp, dp, C.c_int, C.c_double, C.c_double]),
        "ems_tetbatch_add_receiver": (C.c_int, [vp, C.c_int, dp]),
        "ems_tetfem_set_material": (C.c_int, [vp, dp, dp]),
        "ems_tetfem_add_dipole": (C.c_int, [vp, dp, dp, C.c_int, C.c_double, C.c_double]),
        "ems_tetfem_add_receiver": (C.c_int, [vp, dp]),
        "ems_tetfem_time_step": (C.c_int, [vp, dp, dp]),
        "ems_tetfem_apply_stiffness": (C.c_int, [vp, dp, dp, C.c_size_t]),
        "ems_tetfem_set_checkpoints": (C.c_int, [vp, C.c_int]),
        "ems_tetfem_backward": (C.c_int, [vp, dp, C.c_size_t, dp, dp, C.c_size_t]),
        "ems_tetfem_energy": (C.c_int, [vp, dp, C.c_int]),

        "ems_trace_misfit": (C.c_int, [C.c_int, C.c_int, C.c_int, dp, dp, dp, dp, dp]),
        "ems_tetfem_gradient": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, dp, dp, dp, dp, dp, C.c_size_t]),
        "ems_tet_stiffness_apply_static": (C.c_int, [ip, vp, vp, vp]),
        "ems_run": (C.c_int, [vp, C.c_int]),
        "ems_trace_shape": (C.c_int, [vp, ip, ip, ip]),
        "ems_get_traces": (C.c_int, [vp, dp, C.c_size_t]),
        "ems_save_results": (C.c_int, [vp, C.c_char_p]),
        "ems_save_trace_component": (C.c_int, [vp, C.c_int, C.c_int, C.c_char_p]),
        "ems_field_size": (C.c_int, [vp, C.c_int, C.POINTER(C.c_size_t)]),
        "ems_get_field": (C.c_int, [vp, C.c_int, dp, C.c_size_t]),
        "ems_set_field": (C.c_int, [vp, C.c_int, dp, C.c_size_t]),
        "ems_last_run_stats": (C.c_int, [vp, dp, C.POINTER(C.c_longlong)]),
        "ems_time_dominant_kernel": (C.c_int, [vp, C.c_int, dp, dp, C.c_char_p, C.c_size_t]),
        "ems_launch_shape": (C.c_int, [vp, C.POINTER(C.c_int)]),
        "ems_reset": (C.c_int, [vp]),
        "ems_destroy": (C.c_int, [vp]),
    }
    for name, (res, args) in sig.items():
        if hasattr(L, name):
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
    _lib = L
    return L


def check(status, handle=None):
    if status != EMS_OK:
        L = lib()
        msg = L.ems_last_error(handle)
        raise EmsError(status, (msg or b"").decode() or L.ems_status_string(status).decode())
