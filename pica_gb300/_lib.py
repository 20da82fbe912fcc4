"""ctypes binding of the pica_gb300 C ABI (include/pica_gb300.h).

The library is built in-tree (pica_gb300/_build/libpica_gb300.so).  There is
no fallback: if the library is missing and cannot be built, importing the
binding raises.
"""
import ctypes as C
import os

from . import build as _build

_LIB = None


class PicaConfig(C.Structure):
    _fields_ = [
        ("n", C.c_int32 * 3), ("sc", C.c_int32 * 3), ("h", C.c_double * 3), ("dt", C.c_double),
        ("form", C.c_int32), ("shape", C.c_int32), ("deposit", C.c_int32), ("nspecies", C.c_int32),
        ("mass", C.c_double * 4), ("charge", C.c_double * 4), ("slack", C.c_double),
        ("resort_every", C.c_int32), ("threads", C.c_int32),
    ]


class PicaDiag(C.Structure):
    _fields_ = [("field_energy", C.c_double), ("kinetic_energy", C.c_double), ("total_charge", C.c_double),
                ("gauss_max", C.c_double), ("rho_max", C.c_double), ("pad_", C.c_double * 3)]


class PicaPlasmaSpec(C.Structure):
    _fields_ = [
        ("n", C.c_int32 * 3), ("species", C.c_int32), ("h", C.c_double * 3), ("ppc", C.c_double),
        ("density_mod", C.c_double), ("drift_u", C.c_double), ("sigma_u", C.c_double), ("weight", C.c_double),
        ("seed", C.c_uint64), ("nbeams", C.c_int32), ("drift_axis", C.c_int32),
    ]


# Every exported symbol of include/pica_gb300.h with its ctypes signature.
_vp, _dp, _ip, _i64, _i32 = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_int64, C.c_int32
SIGNATURES = {
    "pica_abi_version": (C.c_int, []),
    "pica_status_string": (C.c_char_p, [C.c_int]),
    "pica_ctx_create": (C.c_int, [C.POINTER(PicaConfig), C.POINTER(_vp)]),
    "pica_ctx_destroy": (C.c_int, [_vp]),
    "pica_set_stream": (C.c_int, [_vp, _vp]),
    "pica_synchronize": (C.c_int, [_vp]),
    "pica_last_error": (C.c_char_p, [_vp]),
    "pica_launch_count": (_i64, [_vp]),
    "pica_set_variant": (C.c_int, [_vp, _i32]),
    "pica_get_variant": (C.c_int, [_vp, _ip, _ip]),
    "pica_upload_particles": (C.c_int, [_vp, _i64] + [_dp] * 7 + [_ip]),
    "pica_num_particles": (_i64, [_vp]),
    "pica_download_particles": (C.c_int, [_vp] + [_dp] * 7 + [_ip, _ip]),
    "pica_get_counts": (C.c_int, [_vp, _ip]),
    "pica_record_migrations": (C.c_int, [_vp, _i32]),
    "pica_num_migrations": (_i64, [_vp]),
    "pica_get_migrations": (C.c_int, [_vp, _ip, _ip, _ip, _ip]),
    "pica_upload_fields": (C.c_int, [_vp, C.POINTER(_dp)]),
    "pica_download_fields": (C.c_int, [_vp, C.POINTER(_dp)]),
    "pica_push_deposit": (C.c_int, [_vp]),
    "pica_update_b": (C.c_int, [_vp, C.c_double]),
    "pica_update_e": (C.c_int, [_vp, C.c_double]),
    "pica_migrate": (C.c_int, [_vp]),
    "pica_step": (C.c_int, [_vp, _i32]),
    "pica_diagnostics": (C.c_int, [_vp, C.c_double, C.POINTER(PicaDiag)]),
    "pica_charge_density": (C.c_int, [_vp, _dp]),
    "pica_field_energy": (C.c_int, [_vp, _dp]),
    "pica_field_energy_noalloc": (C.c_int, [C.POINTER(_vp), _i32, _ip, _dp, _vp, _dp]),
    "pica_checkpoint_save": (C.c_int, [_vp, C.c_char_p]),
    "pica_step_count": (_i64, [_vp]),
    "pica_checkpoint_load": (C.c_int, [_vp, C.c_char_p]),
    "pica_batch_create": (C.c_int, [C.POINTER(PicaConfig), _i32, C.POINTER(_vp)]),
    "pica_batch_destroy": (C.c_int, [_vp]),
    "pica_batch_member": (_vp, [_vp, _i32]),
    "pica_batch_set_options": (C.c_int, [_vp, _i32, _i32]),
    "pica_batch_step": (C.c_int, [_vp, _i32]),
    "pica_batch_stats": (C.c_int, [_vp, C.POINTER(C.c_int64)]),
    "pica_batch_last_error": (C.c_char_p, [_vp]),
    "pica_state_slots": (_i64, [_vp, _i32]),
    "pica_state_copy": (C.c_int, [_vp, _i32, _i32, _vp, _i32]),
    "pica_state_packed_slots": (_i64, [_vp, _i32]),
    "pica_state_copy_packed": (C.c_int, [_vp, _i32, _i32, _vp, _i32]),
    "pica_state_copy_packed_range": (C.c_int, [_vp, _i32, _i32, _vp, _i32, _i32, _i32]),
    "pica_state_copy_packed_range_on": (C.c_int, [_vp, _i32, _i32, _vp, _i32, _i32, _i32, _vp]),
    "pica_state_copy_range_on": (C.c_int, [_vp, _i32, _i32, _vp, _i32, _i32, _i32, _vp]),
    "pica_push_deposit_chunked": (C.c_int, [_vp, _i32, C.POINTER(_vp)]),
    "pica_push_deposit_ranges": (C.c_int, [_vp, _i32, C.POINTER(_i32), C.POINTER(_vp)]),
    "pica_reorder": (C.c_int, [_vp]),
    "pica_order_by_position": (C.c_int, [_i64, _i32, _vp, _vp, _vp, _vp, _vp]),
    "pica_push_flat": (C.c_int, [_vp, _i64] + [_vp] * 8 + [_i32]),
    "pica_order_by_position_host": (C.c_int, [_i64, _i32, _dp, _dp, _dp, C.POINTER(_i64)]),
    "pica_push_flat_host": (C.c_int, [_vp, _i64] + [_dp] * 7 + [_ip, _i32]),
    "pica_field_slab": (C.c_int, [_vp, _i32, _i32, _i32, _vp, _i32]),
    "pica_take_supercells": (_i64, [_vp, _i32, _i32, _i32, C.POINTER(_vp), _i64, _ip]),
    "pica_append_to_supercells": (C.c_int, [_vp, _i32, _i32, _i32, _ip, C.POINTER(_vp), _i32]),
    "pica_generate_plasma": (C.c_int, [_vp, C.POINTER(PicaPlasmaSpec), _i32]),
    "pica_plasma_count": (_i64, [C.POINTER(PicaPlasmaSpec)]),
    "pica_plasma_generate": (C.c_int, [C.POINTER(PicaPlasmaSpec), _i32] + [_dp] * 7 + [_ip]),
}


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load (building first if needed) the CUDA library and bind every ABI symbol."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if build_if_missing and (not os.path.exists(path) or _build._stale()):
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"pica_gb300 CUDA library not built ({path}); run pica_gb300.build.build()")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype, fn.argtypes = res, args
    _LIB = lib
    return lib
