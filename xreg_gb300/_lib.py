"""ctypes binding of libxreg_gb300.so (the C ABI declared in include/xreg_gb300.h).

The library is built in-tree by xreg_gb300.build; importing this module never
falls back to any other implementation: if the shared library is missing the
import raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from .build import LIB_PATH

XR_OK = 0
XR_ERR_INVALID_ARG = -1
XR_ERR_CUDA = -2
XR_ERR_OUT_OF_MEMORY = -3
XR_ERR_UNSUPPORTED = -4
XR_ERR_NOT_ALLOCATED = -5
XR_ERR_DEVICE_CHECK = -6

XR_VOXEL_F32, XR_VOXEL_F16, XR_VOXEL_BF16 = 0, 1, 2
XR_LINE_INT_SUM, XR_LINE_INT_MAX = 0, 1
XR_PROJ_STORE_REPLACE, XR_PROJ_STORE_ACCUM = 0, 1
XR_REGI_CMAES, XR_REGI_DFO = 0, 1
XR_INTERP_LINEAR, XR_INTERP_NN, XR_INTERP_SINC, XR_INTERP_BSPLINE = 0, 1, 2, 3
XR_CAM_FOCAL_POS_Z, XR_CAM_FOCAL_NEG_Z, XR_CAM_ON_DETECTOR = 0, 1, 2
XR_LAYOUT_AUTO, XR_LAYOUT_LINEAR, XR_LAYOUT_CELL8 = -1, 0, 1
XR_SIM_NCC, XR_SIM_GRAD_NCC, XR_SIM_PATCH_NCC, XR_SIM_PATCH_GRAD_NCC = 0, 1, 2, 3


class xr_volume_desc(C.Structure):
    _fields_ = [("n", C.c_int64 * 3), ("spacing", C.c_double * 3), ("origin", C.c_double * 3),
                ("direction", C.c_double * 9)]


class xr_camera_desc(C.Structure):
    _fields_ = [("intrins", C.c_double * 9), ("extrins", C.c_double * 16), ("num_det_rows", C.c_int64),
                ("num_det_cols", C.c_int64), ("det_row_spacing", C.c_double), ("det_col_spacing", C.c_double),
                ("focal_len", C.c_double), ("coord_frame_type", C.c_int32), ("reserved", C.c_int32)]


class xr_patch_options(C.Structure):
    _fields_ = [("use_mask_for_weighting", C.c_int32), ("use_mask_for_patch_stats", C.c_int32),
                ("normalize_weights_as_prob", C.c_int32), ("weight_patch_sims_in_combine", C.c_int32),
                ("compute_mean_of_patch_sims", C.c_int32), ("use_fixed_img_patch_variances_as_wgts", C.c_int32),
                ("use_mov_img_patch_variances_as_wgts", C.c_int32),
                ("use_variances_in_grad_imgs_as_wgts", C.c_int32), ("choose_rand_patches", C.c_int32),
                ("mask_only_for_weights", C.c_int32), ("save_all_per_patch_scores", C.c_int32),
                ("reserved0", C.c_int32), ("num_rand_patches", C.c_int64), ("rand_patch_min_pixels_sep", C.c_double),
                ("rand_seed", C.c_uint64)]


class xr_regi_level_params(C.Structure):
    _fields_ = [("optimizer", C.c_int32), ("lambda_", C.c_int32), ("sigma", C.c_double * 6),
                ("bounds", C.c_double * 6), ("max_iters", C.c_int64), ("tol_fun", C.c_double),
                ("tol_x", C.c_double), ("rho_beg", C.c_double), ("rho_end", C.c_double), ("seed", C.c_uint64)]


class xr_regi_step_job(C.Structure):
    _fields_ = [("obj", C.c_void_p), ("optimizer", C.c_int32), ("reserved", C.c_int32), ("opt", C.c_void_p),
                ("centre", C.c_double * 16), ("start_pose", C.c_double * 16), ("bounds", C.c_double * 6)]


class XRegError(RuntimeError):
    """A C-ABI call returned a non-zero xr_status."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"[xr_status {status}] {msg}")
        self.status = status


H = C.c_void_p
P = C.c_void_p
i32, i64, u64, f32, f64 = C.c_int32, C.c_int64, C.c_uint64, C.c_float, C.c_double

# name -> argtypes (restype is xr_status unless listed in _RESTYPES)
_SIGS = {
    "xr_last_error": [],
    "xr_version": [],
    "xr_camera_setup_naive": [f64, i64, i64, f64, f64, i32, C.POINTER(xr_camera_desc)],
    "xr_camera_downsample": [C.POINTER(xr_camera_desc), f64, i32, C.POINTER(xr_camera_desc)],
    "xr_rc_create": [i32, C.POINTER(H)],
    "xr_rc_destroy": [H],
    "xr_rc_set_stream": [H, P],
    "xr_rc_synchronize": [H],
    "xr_rc_set_volumes": [H, i32, C.POINTER(xr_volume_desc), C.POINTER(P), i32, f32],
    "xr_rc_set_volumes_device": [H, i32, C.POINTER(xr_volume_desc), C.POINTER(P), i32, f32],
    "xr_rc_set_camera_models": [H, i32, C.POINTER(xr_camera_desc)],
    "xr_rc_set_num_projs": [H, i64],
    "xr_rc_num_projs": [H, C.POINTER(i64)],
    "xr_rc_set_ray_step_size": [H, f32],
    "xr_rc_set_interp_method": [H, i32],
    "xr_rc_set_proj_store_method": [H, i32],
    "xr_rc_set_default_bg_pixel_val": [H, f32],
    "xr_rc_set_kernel_id": [H, i32],
    "xr_rc_set_bg_projs": [H, C.POINTER(P), i32],
    "xr_rc_set_use_bg_projs": [H, i32],
    "xr_rc_set_xforms_cam_to_itk_phys": [H, i64, P],
    "xr_rc_distribute_xforms_among_cam_models": [H, i64, P],
    "xr_rc_distribute_xforms_device": [H, i64, P],
    "xr_rc_set_camera_model_proj_associations": [H, i64, P],
    "xr_rc_camera_model_proj_associations": [H, i64, P, C.POINTER(i64)],
    "xr_rc_set_proj_cam_model": [H, i64, i32],
    "xr_rc_xforms_cam_to_itk_phys": [H, i64, P, C.POINTER(i64)],
    "xr_rc_pre_multiply_all_xforms": [H, P],
    "xr_rc_post_multiply_all_xforms": [H, P],
    "xr_rc_num_vols": [H, C.POINTER(i32)],
    "xr_rc_num_camera_models": [H, C.POINTER(i32)],
    "xr_rc_xform_img_center_to_itk_phys": [H, i32, P],
    "xr_rc_xform_cam_wrt_carm_center_of_rot": [H, i32, P],
    "xr_rc_allocate_resources": [H],
    "xr_rc_max_num_projs_possible": [H, C.POINTER(i64)],
    "xr_rc_compute": [H, i32],
    "xr_rc_proj": [H, i64, P],
    "xr_rc_copy_projs_to_host": [H, P],
    "xr_rc_device_pixel_buf": [H, C.POINTER(P)],
    "xr_rc_use_other_proj_buf": [H, H],
    "xr_rc_use_external_host_pixel_buf": [H, P],
    "xr_rc_last_num_samples": [H, C.POINTER(u64)],
    "xr_rc_last_num_loaded_samples": [H, C.POINTER(u64)],
    "xr_measure_l2_read_bandwidth": [C.c_int32, C.c_int64, C.c_int32, C.POINTER(C.c_double)],
    "xr_rc_set_count_samples": [H, i32],
    "xr_rc_set_launch_config": [H, i32, i32, i32],
    "xr_rc_get_launch_config": [H, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)],
    "xr_rc_set_launch_config_ex": [H, i32, i32, i32, i32],
    "xr_rc_get_launch_config_ex": [H, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)],
    "xr_rc_set_build_cell_layout": [H, i32],
    "xr_rc_set_empty_space_skipping": [H, i32],
    "xr_sm_create": [i32, i32, C.POINTER(H)],
    "xr_sm_destroy": [H],
    "xr_sm_set_stream": [H, P],
    "xr_sm_set_fixed_image": [H, P, i64, i64],
    "xr_sm_set_mask": [H, P],
    "xr_sm_set_num_moving_images": [H, i64],
    "xr_sm_set_mov_imgs_buf_from_ray_caster": [H, H, i64],
    "xr_sm_set_mov_imgs_device_buf": [H, P, i64],
    "xr_sm_set_mov_imgs_host_buf": [H, P],
    "xr_sm_set_smooth_img_before_sobel_kernel_radius": [H, i32],
    "xr_sm_set_patch_radius": [H, i32],
    "xr_sm_set_patch_stride": [H, i32],
    "xr_patch_options_default": [C.POINTER(xr_patch_options)],
    "xr_sm_set_patch_options": [H, C.POINTER(xr_patch_options)],
    "xr_sm_get_patch_options": [H, C.POINTER(xr_patch_options)],
    "xr_sm_set_patch_wgt_img": [H, P],
    "xr_sm_patch_indices_used": [H, i64, P, C.POINTER(i64)],
    "xr_sm_patch_scores": [H, i64, i64, P, C.POINTER(i64)],
    "xr_sm_set_patches_to_use": [H, i64, P],
    "xr_sm_fixed_image": [H, i64, P, C.POINTER(i64), C.POINTER(i64)],
    "xr_sm_mask": [H, i64, P, C.POINTER(i32)],
    "xr_sm_num_pix_per_proj": [H, C.POINTER(i64)],
    "xr_sm_num_moving_images": [H, C.POINTER(i64)],
    "xr_sm_allocate_resources": [H],
    "xr_sm_compute": [H],
    "xr_sm_sim_vals": [H, P],
    "xr_sm_device_sim_vals": [H, C.POINTER(P)],
    "xr_obj_create": [H, i32, i32, C.POINTER(H), i64, C.POINTER(H)],
    "xr_obj_destroy": [H],
    "xr_obj_eval": [H, i64, P, P],
    "xr_obj_eval_device": [H, i64, P, P],
    "xr_obj_set_fused": [H, i32],
    "xr_grad_ncc_noalloc": [P, P, i64, i64, i64, i32, P, P],
    "xr_cmaes_create": [i32, P, P, i32, u64, C.POINTER(H)],
    "xr_cmaes_destroy": [H],
    "xr_cmaes_set_stop": [H, f64, f64, i64],
    "xr_cmaes_sample_population": [H, P],
    "xr_cmaes_resample_single": [H, i32, P],
    "xr_cmaes_update_distribution": [H, P],
    "xr_cmaes_test_termination": [H, C.POINTER(i32)],
    "xr_cmaes_get": [H, P, P, C.POINTER(f64), C.POINTER(f64), C.POINTER(i64)],
    "xr_cmaes_state_bytes": [H, C.POINTER(i64)],
    "xr_dfo_set_batch": [H, i32],
    "xr_jobset_set_pose_groups": [H, i32],
    "xr_jobset_last_pose_grouped": [H, C.POINTER(i32)],
    "xr_dfo_evaluations": [H, C.POINTER(i64)],
    "xr_cmaes_export_state": [H, P, i64],
    "xr_cmaes_attach_device": [H, i32],
    "xr_cmaes_detach_device": [H],
    "xr_dfo_create": [i32, P, P, P, f64, f64, i64, C.POINTER(H)],
    "xr_dfo_destroy": [H],
    "xr_dfo_ask": [H, P, C.POINTER(i32)],
    "xr_dfo_tell": [H, P],
    "xr_dfo_test_termination": [H, C.POINTER(i32)],
    "xr_dfo_get": [H, P, C.POINTER(f64), C.POINTER(f64), C.POINTER(i64)],
    "xr_hu_to_lin_att": [P, i64, P, P],
    "xr_downsample_image_size": [i64, i64, f64, C.POINTER(i64), C.POINTER(i64)],
    "xr_downsample_image": [P, i64, i64, f64, P, P, P],
    "xr_camera_crop_boundary": [P, i64, P],
    "xr_crop_image_boundary": [P, i64, i64, i64, P, P],
    "xr_log_remap": [P, i64, i64, i32, f32, P, P, P],
    "xr_regi_level_params_default": [i32, C.POINTER(xr_regi_level_params)],
    "xr_regi_run_level": [H, P, P, C.POINTER(xr_regi_level_params), P, C.POINTER(f64), C.POINTER(i64),
                          C.POINTER(i32)],
    "xr_jobset_create": [i32, C.POINTER(H)],
    "xr_jobset_destroy": [H],
    "xr_jobset_set_stream": [H, P],
    "xr_jobset_eval": [H, i32, C.POINTER(H), C.POINTER(i64), C.POINTER(P), C.POINTER(P)],
    "xr_jobset_eval_device": [H, i32, C.POINTER(H), C.POINTER(i64), C.POINTER(P), C.POINTER(P)],
    "xr_jobset_last_launch": [H, C.POINTER(i64), C.POINTER(i32)],
    "xr_jobset_set_fused": [H, i32],
    "xr_jobset_last_kernel_launches": [H, C.POINTER(i32)],
    "xr_regi_pose_map": [C.c_void_p, C.c_void_p, i64, C.c_void_p, C.c_void_p],
    "xr_regi_jobset_step": [H, i32, C.POINTER(xr_regi_step_job), C.POINTER(i32), C.POINTER(i32)],
    "xr_cmaes_lambda": [H, C.POINTER(i32)],
    "xr_itk_affine_transform_read": [C.c_char_p, P],
    "xr_itk_slicer_affine_transform_read": [C.c_char_p, P],
    "xr_itk_affine_transform_write": [C.c_char_p, P],
}
_RESTYPES = {"xr_last_error": C.c_char_p, "xr_version": C.c_char_p}

EXPORTED = tuple(_SIGS)

_lib = None


def lib_path() -> Path:
    return LIB_PATH


def load() -> C.CDLL:
    """Loads the in-tree shared library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: run `python -m xreg_gb300.build` (or __graft_entry__.build())")
    lib = C.CDLL(str(LIB_PATH))
    for name, args in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, C.c_int32)
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != XR_OK:
        raise XRegError(status, load().xr_last_error().decode(errors="replace"))


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))
