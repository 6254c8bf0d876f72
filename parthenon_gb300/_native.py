"""ctypes binding of libparthenon_gb300.so (the C ABI declared in include/parthenon_gb300.h).

There is no fallback: if the native library is missing or cannot be loaded, every
entry point raises. Build it with `python -m parthenon_gb300.build` (or
`__graft_entry__.build()`).
"""
import ctypes
import os

from . import build as _build

_lib = None

I32P = ctypes.POINTER(ctypes.c_int32)
I64P = ctypes.POINTER(ctypes.c_int64)
DP = ctypes.POINTER(ctypes.c_double)
VP = ctypes.c_void_p


class MeshSpec(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32 * 3), ("block_nx", ctypes.c_int32 * 3), ("nghost", ctypes.c_int32),
                ("xmin", ctypes.c_double * 3), ("xmax", ctypes.c_double * 3)]


class MeshInfo(ctypes.Structure):
    _fields_ = [("nblocks", ctypes.c_int32), ("multilevel", ctypes.c_int32), ("root_level", ctypes.c_int32),
                ("max_level", ctypes.c_int32), ("N", ctypes.c_int32 * 3), ("Nc", ctypes.c_int32 * 3),
                ("npairs", ctypes.c_int32), ("buffer_elems", ctypes.c_int64), ("nflux_corr", ctypes.c_int32)]


class GmgParams(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("ncoarsen", ctypes.c_int32), ("stages", ctypes.c_int32),
                ("jacobi", ctypes.c_int32), ("weight", ctypes.c_double), ("coarse_sweeps", ctypes.c_int32),
                ("exact", ctypes.c_int32), ("xmin", ctypes.c_double), ("xmax", ctypes.c_double)]


class MgParams(ctypes.Structure):
    _fields_ = [("stages", ctypes.c_int32), ("jacobi", ctypes.c_int32), ("weight", ctypes.c_double),
                ("coarse_sweeps", ctypes.c_int32), ("max_coarsenings", ctypes.c_int32), ("D", ctypes.c_double),
                ("alpha", ctypes.c_double), ("exact", ctypes.c_int32), ("flux_correct", ctypes.c_int32)]


class StageParams(ctypes.Structure):
    _fields_ = [("physics", ctypes.c_int32), ("recon", ctypes.c_int32), ("exact", ctypes.c_int32),
                ("ncomp_vel", ctypes.c_int32), ("vel", ctypes.c_double * 3), ("cfl", ctypes.c_double),
                ("comp_vel", DP)]


class SparseParams(ctypes.Structure):
    _fields_ = [("ncomp", ctypes.c_int32), ("dealloc_count", ctypes.c_int32), ("alloc_threshold", DP),
                ("dealloc_threshold", DP), ("default_value", DP)]


# name -> (argtypes); every function returns int32 status unless noted
_SIGNATURES = {
    "pgb_version": [],
    "pgb_mesh_create": [ctypes.POINTER(MeshSpec), ctypes.c_int32, VP, ctypes.POINTER(VP)],
    "pgb_mesh_destroy": [VP],
    "pgb_mesh_get_info": [VP, ctypes.POINTER(MeshInfo)],
    "pgb_mesh_block_info": [VP, VP, VP],
    "pgb_mesh_boundaries": [VP, VP, ctypes.c_int32],
    "pgb_mesh_upload": [VP],
    "pgb_mesh_validate": [VP],
    "pgb_exchange": [VP, VP, VP, ctypes.c_int32, ctypes.c_int32, VP, VP],
    "pgb_pack_buffers": [VP, VP, VP, ctypes.c_int32, VP, VP],
    "pgb_exchange_static_buffer": [VP, VP, VP, ctypes.c_int32, ctypes.c_int32, VP],
    "pgb_flux_correct": [VP, VP, ctypes.c_int32, VP],
    "pgb_stage": [VP, ctypes.POINTER(StageParams), VP, VP, VP, VP, VP, VP, ctypes.c_double, ctypes.c_double,
                  ctypes.c_double, ctypes.c_int32, VP],
    "pgb_estimate_dt": [VP, ctypes.POINTER(StageParams), VP, ctypes.c_int32, VP, ctypes.c_int32, VP],
    "pgb_fill_derived": [VP, VP, ctypes.c_int32, VP, VP],
    "pgb_set_derived": [VP, VP],
    "pgb_rk2_cycles": [VP, ctypes.POINTER(StageParams), VP, VP, VP, VP, VP, VP, ctypes.c_int32, VP,
                       ctypes.c_int32, ctypes.c_int32, VP],
    "pgb_run_host": [VP, ctypes.POINTER(StageParams), VP, VP, ctypes.c_int32, ctypes.c_int32, DP],
    "pgb_run_host_dt": [VP, ctypes.POINTER(StageParams), VP, VP, ctypes.c_int32, ctypes.c_int32, DP, DP],
    "pgb_release_host_workspace": [VP],
    "pgb_gmg_create": [ctypes.POINTER(GmgParams), ctypes.POINTER(VP)],
    "pgb_gmg_destroy": [VP],
    "pgb_gmg_vcycles": [VP, VP, VP, ctypes.c_int32, VP, VP],
    "pgb_gmg_solve": [VP, VP, VP, ctypes.c_int32, ctypes.c_double, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                      DP, VP],
    "pgb_gmg_bicgstab": [VP, VP, VP, ctypes.c_int32, ctypes.c_double, ctypes.c_int32, ctypes.c_int32,
                         ctypes.POINTER(ctypes.c_int32), DP, VP],
    "pgb_gmg_solve_blocks": [VP, VP, VP, VP, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                             ctypes.c_double, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), DP, VP],
    "pgb_mg_create": [VP, ctypes.POINTER(MgParams), ctypes.POINTER(VP)],
    "pgb_mg_destroy": [VP],
    "pgb_mg_info": [VP, VP],
    "pgb_mg_boundaries": [VP, ctypes.c_int32, VP, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)],
    "pgb_mg_vcycles": [VP, VP, VP, ctypes.c_int32, VP, VP],
    "pgb_mg_solve": [VP, VP, VP, ctypes.c_double, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                     ctypes.POINTER(ctypes.c_int32), DP, VP],
    "pgb_mg_set_coefficient": [VP, VP, VP],
    "pgb_mg_bicgstab": [VP, VP, VP, ctypes.c_int32, ctypes.c_double, ctypes.c_int32, ctypes.c_int32,
                        ctypes.POINTER(ctypes.c_int32), DP, VP],
    "pgb_mg_layout": [VP, I32P],
    "pgb_mg_store_info": [VP, ctypes.c_int32, I32P, DP, I32P],
    "pgb_mg_grid_info": [VP, ctypes.c_int32, I32P, I32P, I32P],
    "pgb_mg_field_exchange": [VP, ctypes.c_int32, VP, VP],
    "pgb_mg_field_restrict": [VP, ctypes.c_int32, VP, VP, VP],
    "pgb_mg_field_prolongate": [VP, ctypes.c_int32, VP, VP, VP],
    "pgb_mg_face_restrict": [VP, ctypes.c_int32, VP, VP, VP],
    "pgb_history_mass": [VP, VP, ctypes.c_int32, VP, ctypes.c_int32, ctypes.c_double, VP, VP],
    "pgb_tune_report": [ctypes.c_char_p, ctypes.c_int32],
    "pgb_amr_block_criterion": [VP, VP, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, VP, VP],
    "pgb_amr_set_refinement": [VP, VP, ctypes.c_double, ctypes.c_double, ctypes.c_int32, ctypes.c_int32,
                               ctypes.c_int32, VP],
    "pgb_amr_remesh": [VP, VP, ctypes.POINTER(VP)],
    "pgb_amr_transfer": [VP, VP, VP, VP, ctypes.c_int32, VP],
    "pgb_sparse_enable": [VP, ctypes.POINTER(SparseParams)],
    "pgb_sparse_set_alloc": [VP, VP, VP],
    "pgb_sparse_get_alloc": [VP, VP, VP, VP],
    "pgb_sparse_dealloc": [VP, VP, VP, ctypes.c_int32, VP, ctypes.c_int32, VP, VP],
    "pgb_sparse_tag": [VP, VP, ctypes.c_double, ctypes.c_double, VP, VP],
}


class NativeError(RuntimeError):
    pass


def lib_path():
    return _build.LIB


def lib():
    """Load the native library (raises if it is absent: no CPU fallback exists)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise NativeError("libparthenon_gb300.so is not built (%s); run parthenon_gb300.build.build()" % path)
        L = ctypes.CDLL(path)
        for name, args in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int32
        L.pgb_last_error.argtypes = []
        L.pgb_last_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def check(rc, what=""):
    if rc != 0:
        msg = lib().pgb_last_error().decode(errors="replace")
        raise NativeError("%s failed (%d): %s" % (what, rc, msg))
    return rc


def exported_symbols():
    return sorted(list(_SIGNATURES) + ["pgb_last_error"])


def tune_report():
    """Launch shapes chosen by the autotuner so far: {key: (choice, [ms per candidate])}."""
    buf = ctypes.create_string_buffer(8192)
    check(lib().pgb_tune_report(buf, len(buf)), "pgb_tune_report")
    out = {}
    for item in buf.value.decode().split(" ; "):
        if "=" not in item:
            continue
        key, rest = item.rsplit("=", 1)
        choice, ms = rest.split(" (", 1)
        out[key] = (int(choice), [float(x) for x in ms.rstrip(" ms)").split()])
    return out
