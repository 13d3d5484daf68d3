"""ctypes binding of libommp_gb300.so (include/openmmpol_gb300.h).

The shared library is built in-tree by ``openmmpol_gb300.build``.  Loading
fails with an explicit error when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libommp_gb300.so")

_vp = C.c_void_p
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)

# name -> (restype, argtypes); every symbol declared in include/openmmpol_gb300.h
SIGNATURES = {
    "ommp_init_mmp": (_vp, [C.c_char_p]),
    "ommp_set_default_solver": (None, [_vp, C.c_int32]),
    "ommp_set_default_matv": (None, [_vp, C.c_int32]),
    "ommp_terminate": (None, [_vp]),
    "ommp_set_verbose": (None, [C.c_int32]),
    "ommp_set_outputfile": (None, [C.c_char_p]),
    "ommp_close_outputfile": (None, []),
    "ommp_message": (None, [C.c_char_p, C.c_int32, C.c_char_p]),
    "ommp_fatal": (None, [C.c_char_p]),
    "ommp_time_pull": (None, [C.c_char_p]),
    "ommp_time_push": (None, []),
    "ommp_get_polelec_energy": (C.c_double, [_vp]),
    "ommp_get_fixedelec_energy": (C.c_double, [_vp]),
    "ommp_get_full_ele_energy": (C.c_double, [_vp]),
    "ommp_gpu_get_fixedelec_energy": (C.c_int32, [_vp, _dp]),
    "ommp_set_external_field": (None, [_vp, _dp, C.c_int32, C.c_int32]),
    "ommp_set_external_field_nomm": (None, [_vp, _dp, C.c_int32, C.c_int32]),
    "ommp_ff_is_amoeba": (C.c_bool, [_vp]),
    "ommp_get_n_ipd": (C.c_int32, [_vp]),
    "ommp_get_ld_cart": (C.c_int32, [_vp]),
    "ommp_get_mm_atoms": (C.c_int32, [_vp]),
    "ommp_get_pol_atoms": (C.c_int32, [_vp]),
    "ommp_get_cmm": (_dp, [_vp]),
    "ommp_get_cpol": (_dp, [_vp]),
    "ommp_get_q": (_dp, [_vp]),
    "ommp_get_ipd": (_dp, [_vp]),
    "ommp_get_polar_mm": (_ip, [_vp]),
    "ommp_update_coordinates": (None, [_vp, _dp]),
    "ommp_enable_fmm": (None, [_vp]),
    "ommp_disable_fmm": (None, [_vp]),
    "ommp_use_fmm": (C.c_bool, [_vp]),
    "ommp_gpu_init_mmp": (C.c_int32, [C.c_char_p, C.POINTER(_vp)]),
    "ommp_gpu_set_external_field": (C.c_int32, [_vp, _dp, C.c_int32, C.c_int32, C.c_int32]),
    "ommp_gpu_set_external_field_status": (C.c_int32, [_vp, _dp, C.c_int32, C.c_int32, C.c_int32]),
    "ommp_gpu_set_external_field_device": (C.c_int32, [_vp, _vp, C.c_int32, C.c_int32, C.c_int32]),
    "ommp_gpu_get_polelec_energy": (C.c_int32, [_vp, _dp]),
    "ommp_gpu_update_coordinates": (C.c_int32, [_vp, _dp]),
    "ommp_gpu_set_default_solver": (C.c_int32, [_vp, C.c_int32]),
    "ommp_gpu_set_default_matv": (C.c_int32, [_vp, C.c_int32]),
    "ommp_gpu_last_error": (C.c_char_p, []),
    "ommp_gpu_set_solver_tol": (None, [_vp, C.c_double]),
    "ommp_gpu_set_solver_maxiter": (None, [_vp, C.c_int32]),
    "ommp_gpu_set_precision": (None, [_vp, C.c_int32]),
    "ommp_gpu_set_fp64_kernel": (C.c_int32, [_vp, C.c_int32]),
    "ommp_gpu_set_fp32_kernel": (C.c_int32, [_vp, C.c_int32]),
    "ommp_gpu_get_fp32_shape": (C.c_int32, [_vp, C.c_int32, C.POINTER(C.c_int32)]),
    "ommp_gpu_set_inner_preconditioner": (C.c_int32, [_vp, C.c_int32]),
    "ommp_gpu_set_inner_blocks": (C.c_int32, [_vp, C.c_int32, C.c_double]),
    "ommp_gpu_potential_ext": (C.c_int32, [_vp, C.c_int32, C.c_int32, _dp, _dp]),
    "ommp_gpu_field_ext": (C.c_int32, [_vp, C.c_int32, C.c_int32, _dp, _dp]),
    "ommp_potential_mmpol2ext": (None, [_vp, C.c_int32, _dp, _dp]),
    "ommp_potential_mm2ext": (None, [_vp, C.c_int32, _dp, _dp]),
    "ommp_potential_pol2ext": (None, [_vp, C.c_int32, _dp, _dp]),
    "ommp_field_mmpol2ext": (None, [_vp, C.c_int32, _dp, _dp]),
    "ommp_field_mm2ext": (None, [_vp, C.c_int32, _dp, _dp]),
    "ommp_field_pol2ext": (None, [_vp, C.c_int32, _dp, _dp]),
    "ommp_polelec_geomgrad": (None, [_vp, _dp]),
    "ommp_gpu_polelec_geomgrad": (C.c_int32, [_vp, _dp]),
    "ommp_fixedelec_geomgrad": (None, [_vp, _dp]),
    "ommp_gpu_fixedelec_geomgrad": (C.c_int32, [_vp, _dp]),
    "ommp_rotation_geomgrad": (None, [_vp, _dp, _dp, _dp]),
    "ommp_gpu_rotation_geomgrad": (C.c_int32, [_vp, _dp, _dp, _dp]),
    "ommp_gpu_set_fmm": (C.c_int32, [_vp, C.c_int32, C.c_int32]),
    "ommp_set_fmm_lmax_pol": (None, [_vp, C.c_int32]),
    "ommp_set_fmm_lmax": (None, [_vp, C.c_int32]),
    "ommp_set_fmm_distance": (None, [_vp, C.c_double]),
    "ommp_set_fmm_min_cell_size": (None, [_vp, C.c_double]),
    "ommp_gpu_set_fmm_lmax_pol": (C.c_int32, [_vp, C.c_int32]),
    "ommp_gpu_set_fmm_lmax": (C.c_int32, [_vp, C.c_int32]),
    "ommp_gpu_set_fmm_distance": (C.c_int32, [_vp, C.c_double]),
    "ommp_gpu_set_fmm_min_cell_size": (C.c_int32, [_vp, C.c_double]),
    "ommp_gpu_get_fmm_settings": (None, [_vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), _dp]),
    "ommp_gpu_set_fmm_auto": (None, [C.c_int32]),
    "ommp_init_qm_helper": (_vp, [C.c_int32, _dp, _dp, _ip]),
    "ommp_gpu_init_qm_helper": (C.c_int32, [C.c_int32, _dp, _dp, _ip, C.POINTER(_vp)]),
    "ommp_terminate_qm_helper": (None, [_vp]),
    "ommp_qm_helper_update_coord": (None, [_vp, _dp]),
    "ommp_prepare_qm_ele_ene": (None, [_vp, _vp]),
    "ommp_prepare_qm_ele_grd": (None, [_vp, _vp]),
    "ommp_gpu_prepare_qm_ele_ene": (C.c_int32, [_vp, _vp]),
    "ommp_gpu_prepare_qm_ele_grd": (C.c_int32, [_vp, _vp]),
    "ommp_qm_helper_get_V_m2n": (_dp, [_vp]),
    "ommp_qm_helper_get_V_p2n": (_dp, [_vp]),
    "ommp_qm_helper_get_E_m2n": (_dp, [_vp]),
    "ommp_qm_helper_get_E_p2n": (_dp, [_vp]),
    "ommp_qm_helper_get_E_n2p": (_dp, [_vp]),
    "ommp_qm_helper_get_G_n2p": (_dp, [_vp]),
    "ommp_qm_helper_get_E_n2m": (_dp, [_vp]),
    "ommp_qm_helper_get_G_n2m": (_dp, [_vp]),
    "ommp_qm_helper_get_H_n2m": (_dp, [_vp]),
    "ommp_qm_helper_get_cqm": (_dp, [_vp]),
    "ommp_qm_helper_get_npol": (C.c_int32, [_vp]),
    "ommp_qm_helper_get_nmm": (C.c_int32, [_vp]),
    "ommp_qm_helper_get_qm_atoms": (C.c_int32, [_vp]),
    "ommp_gpu_set_use_graphs": (None, [_vp, C.c_int32]),
    "ommp_gpu_set_block_cg": (None, [_vp, C.c_int32]),
    "ommp_gpu_set_residual_update": (C.c_int32, [_vp, C.c_int32]),
    "ommp_gpu_set_external_fields_batch": (C.c_int32, [_vp, C.c_int32, _dp, _dp, _dp]),
    "ommp_gpu_set_external_fields_batch_device": (C.c_int32, [_vp, C.c_int32, _vp, _vp, _dp]),
    "ommp_gpu_clear_guess": (None, [_vp]),
    "ommp_gpu_get_iterations": (C.c_int32, [_vp, C.c_int32]),
    "ommp_gpu_get_residual_history": (C.c_int32, [_vp, C.c_int32, _dp, C.c_int32]),
    "ommp_gpu_get_counter": (C.c_int64, [_vp, C.c_int32]),
    "ommp_gpu_last_solve_ms": (C.c_double, [_vp]),
    "ommp_gpu_get_e_m2d": (C.c_int32, [_vp, _dp]),
    "ommp_gpu_tmatvec": (C.c_int32, [_vp, _dp, _dp, C.c_int32, C.c_int32, C.c_int32]),
    "ommp_gpu_tmatvec_fp32": (C.c_int32, [_vp, _dp, _dp, C.c_int32]),
    "ommp_gpu_tmatvec_ds": (C.c_int32, [_vp, _dp, _dp, C.c_int32]),
    "ommp_gpu_enable_kernel_timing": (None, [_vp, C.c_int32]),
    "ommp_gpu_kernel_stats": (None, [_vp, C.c_int32, _i64p, _dp, _i64p]),
    "ommp_gpu_synchronize": (C.c_int32, [_vp]),
    "ommp_gpu_reset_kernel_stats": (None, [_vp]),
    "ommp_gpu_timer_record": (C.c_int32, [_vp, C.c_int32]),
    "ommp_gpu_timer_elapsed": (C.c_int32, [_vp, C.c_int32, C.c_int32, _dp]),
    "ommp_gpu_flush_l2": (C.c_int32, [_vp, C.c_int64]),
    "ommp_gpu_kernel_launch_count": (C.c_int64, []),
    "ommp_gpu_device_alloc": (C.c_int32, [C.c_int64, C.POINTER(_vp)]),
    "ommp_gpu_device_free": (C.c_int32, [_vp]),
    "ommp_gpu_copy_to_device": (C.c_int32, [_vp, _vp, C.c_int64]),
    "ommp_gpu_device_mem_info": (C.c_int32, [C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "ommp_gpu_copy_to_host": (C.c_int32, [_vp, _vp, C.c_int64]),
    "ommp_gpu_measure_pipe_peak": (C.c_int32, [C.c_int32, _dp]),
    "ommp_gpu_device_sm_count": (C.c_int32, []),
    "ommp_gpu_tmatvec_noalloc": (C.c_int32, [_vp, _vp, _vp, C.c_int32, C.c_int32]),
    "ommp_gpu_solve_multi": (C.c_int32, [C.c_int32, C.POINTER(_vp), C.POINTER(_dp), _dp, _i64p]),
    "ommp_gpu_server_create": (C.c_int32, [C.c_int64, C.c_int32, C.c_int32, C.c_double, C.POINTER(_vp)]),
    "ommp_gpu_server_destroy": (None, [_vp]),
    "ommp_gpu_server_submit": (C.c_int32, [_vp, C.c_char_p, _dp, C.c_int32, _i64p]),
    "ommp_gpu_server_submit_followup": (C.c_int32, [_vp, C.c_int64, _dp, C.c_int32, _i64p]),
    "ommp_gpu_server_wait": (C.c_int32, [_vp, C.c_int64, _dp, _dp, _i64p, _dp]),
    "ommp_gpu_server_release": (None, [_vp, C.c_int64]),
    "ommp_gpu_server_cancel": (C.c_int32, [_vp, C.c_int64]),
    "ommp_gpu_server_stats": (None, [_vp, _dp]),
    "ommp_gpu_server_engine_stats": (None, [_vp, _i64p]),
    "ommp_gpu_server_phase_stats": (None, [_vp, _dp]),
    "ommp_gpu_server_engine_times": (None, [_vp, _dp]),
    "ommp_gpu_server_set_round_ms": (C.c_int32, [_vp, C.c_double]),
}

_lib = None


class LibraryMissing(RuntimeError):
    pass


def load(path: str | None = None):
    """Load (once) and type the library; raises LibraryMissing if absent."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise LibraryMissing(
            f"{p} not found: build it with `python -m openmmpol_gb300.build` "
            "(CUDA toolkit with sm_103a support required); there is no CPU fallback")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
