"""ctypes bindings of include/mfbem.h (the library's C-ABI) and of the
caller-side mesh preparation exported by the same shared object.

The library is loaded from this package's _lib/ directory only; a missing or
unloadable library raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmfbem.so")

c_int32 = ctypes.c_int32
c_double = ctypes.c_double
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)

MFBEM_OK = 0
MFBEM_EARG = -1
MFBEM_ECUDA = -2
MFBEM_ENOMEM = -3
MFBEM_ETIMEOUT = -4
MFBEM_EGEOMETRY = -5
MFBEM_ENOCONV = -6
MFBEM_EUNSUPPORTED = -7
MFBEM_DEVICE_PTRS = 0x1
MFBEM_OVERWRITE = 0x2

# every symbol include/mfbem.h declares
ABI_SYMBOLS = [
    "mfbem_mesh_upload", "mfbem_mesh_release", "mfbem_assemble_staela", "mfbem_assemble_harela",
    "mfbem_solve_r", "mfbem_solve_c", "mfbem_solve_report", "mfbem_internal_points_staela",
    "mfbem_internal_points_harela", "mfbem_trim_device_cache", "mfbem_sweep_harela", "mfbem_solve_staela", "mfbem_last_stats",
    "mfbem_last_error", "mfbem_version", "mfbem_solve_c_static",
    "mfbem_qlearn_label", "mfbem_mlp_size", "mfbem_mlp_forward", "mfbem_mlp_loss_grad", "mfbem_mlp_train",
    "mfbem_set_learned_quadrature", "mfbem_sweep_harela_batch", "mfbem_msh_read", "mfbem_msh_error",
    "mfbem_msh_sizes", "mfbem_msh_parts", "mfbem_msh_nodes", "mfbem_msh_elements", "mfbem_msh_free",
    "mfbem_nso_write", "mfbem_nso_error", "mfbem_fortran_format", "mfbem_set_halfspace", "mfbem_mesh_upload_dual",
    "mfbem_internal_points_faces_staela", "mfbem_internal_points_faces_harela",
]
PREP_SYMBOLS = ["mfbem_prep_create", "mfbem_prep_desc", "mfbem_prep_free", "mfbem_prep_dof",
                "mfbem_prep_set_formulation", "mfbem_prep_set_crack", "mfbem_prep_dof2", "mfbem_prep_dual"]


class MeshDesc(ctypes.Structure):
    _fields_ = [
        ("n_nodes", c_int32), ("n_elements", c_int32), ("n_dof", c_int32),
        ("x_gn", _dp), ("element_node", _ip), ("csize", _dp), ("n_phi", _ip), ("bball", _dp), ("reversion", _ip),
        ("n_gn", _dp), ("tbp_gn", _dp),
        ("row", _ip), ("col", _ip), ("ctype", _ip), ("cvalue", _dp), ("sbie", _ip),
        ("xi_i_sbie_mca", _dp), ("x_i_sbie_mca", _dp),
        ("qsi_relative_error", c_double), ("qsi_ns_max", c_int32), ("n_precalsets", c_int32),
        ("precalset_gln", _ip), ("geometric_tolerance", c_double),
    ]


class DualDesc(ctypes.Structure):
    _fields_ = [("hbie", _ip), ("dual", _ip), ("dual_is_common", _ip), ("alpha", _dp), ("xi_i_hbie", _dp),
                ("x_i_hbie", _dp), ("n_i_hbie", _dp), ("crack_el", _ip), ("ctype2", _ip), ("cvalue2", _dp)]


class Stats(ctypes.Structure):
    _fields_ = [
        ("pairs_regular", ctypes.c_int64), ("pairs_adaptive", ctypes.c_int64), ("pairs_singular", ctypes.c_int64),
        ("points_regular", ctypes.c_int64), ("points_adaptive", ctypes.c_int64), ("points_singular", ctypes.c_int64),
        ("adaptive_leaves", c_int32), ("refinement_iterations", c_int32), ("max_backward_error", c_double),
        ("ms_assemble", c_double), ("ms_factor", c_double), ("ms_solve", c_double),
        ("ms_regular", c_double), ("ms_adaptive", c_double), ("ms_singular", c_double), ("ms_free", c_double),
        ("kernel_launches", ctypes.c_int64), ("gmres_iterations", c_int32), ("refactorizations", c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MfbemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"mfbem error {code}: {msg}")
        self.code = code


_lib = None


def load():
    """Load (building first if needed) the native library."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _b
        _b.build()
    L = ctypes.CDLL(LIB_PATH)
    vp = ctypes.c_void_p
    L.mfbem_mesh_upload.argtypes = [ctypes.POINTER(MeshDesc), ctypes.POINTER(vp)]
    L.mfbem_mesh_release.argtypes = [vp]
    L.mfbem_assemble_staela.argtypes = [vp, c_double, c_double, _dp, c_int32, _dp, c_int32]
    L.mfbem_assemble_harela.argtypes = [vp, _dp, _dp, c_double, _dp, c_double, _dp, c_int32, _dp, c_int32]
    solve_args = [c_int32, _dp, _ip, c_int32, _dp, ctypes.c_char_p, _dp, _dp, c_int32, _dp, c_int32, c_int32, c_int32,
                  c_int32]
    L.mfbem_solve_r.argtypes = solve_args
    L.mfbem_solve_c.argtypes = solve_args
    L.mfbem_solve_report.argtypes = [_dp, c_int32, _dp, _dp]
    L.mfbem_internal_points_staela.argtypes = [vp, c_double, c_double, c_int32, _dp, _dp, _dp, _dp, _dp]
    L.mfbem_internal_points_harela.argtypes = [vp, _dp, _dp, c_double, c_double, c_int32, _dp, _dp, _dp, _dp, _dp]
    L.mfbem_internal_points_faces_staela.argtypes = [vp, c_double, c_double, c_int32, _dp, _dp, _dp, _dp, _dp, _dp,
                                                     _dp]
    L.mfbem_internal_points_faces_harela.argtypes = [vp, _dp, _dp, c_double, c_double, c_int32, _dp, _dp, _dp, _dp,
                                                     _dp, _dp, _dp]
    L.mfbem_sweep_harela.argtypes = [vp, _dp, _dp, c_double, _dp, c_int32, _dp, c_int32, c_double, _dp, c_int32,
                                     ctypes.POINTER(Stats)]
    L.mfbem_solve_staela.argtypes = [vp, c_double, c_double, c_int32, c_double, _dp, c_int32, ctypes.POINTER(Stats)]
    L.mfbem_last_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    L.mfbem_solve_c_static.argtypes = [c_int32, _dp, _ip, c_int32, _dp, c_int32]
    L.mfbem_last_error.restype = ctypes.c_char_p
    L.mfbem_version.restype = ctypes.c_char_p
    L.mfbem_prep_create.restype = vp
    L.mfbem_prep_create.argtypes = [c_int32, _dp, c_int32, _ip, _ip, _dp, c_double, c_int32, c_int32, _ip, c_double]
    L.mfbem_prep_desc.restype = ctypes.POINTER(MeshDesc)
    L.mfbem_prep_desc.argtypes = [vp]
    L.mfbem_prep_free.argtypes = [vp]
    L.mfbem_prep_dof.argtypes = [vp, _ip, _ip]
    L.mfbem_prep_set_formulation.argtypes = [vp, _ip, _dp, _dp]
    L.mfbem_prep_set_crack.argtypes = [vp, _ip, _ip, _dp]
    L.mfbem_prep_dof2.argtypes = [vp, _ip]
    L.mfbem_prep_dual.restype = ctypes.POINTER(DualDesc)
    L.mfbem_prep_dual.argtypes = [vp]
    L.mfbem_mesh_upload_dual.argtypes = [ctypes.POINTER(MeshDesc), ctypes.POINTER(DualDesc), ctypes.POINTER(vp)]
    _lib = L
    return L


def check(rc):
    if rc != 0:
        msg = load().mfbem_last_error().decode(errors="replace")
        raise MfbemError(rc, msg)
    return rc
