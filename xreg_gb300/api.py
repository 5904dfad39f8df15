"""Python mirror of xReg's ray caster / similarity-metric operator surface over
the C ABI.  Method names follow xReg (lib/ray_cast/xregRayCastInterface.h,
lib/regi/sim_metrics_2d/xregImgSimMetric2D.h) so code written against xReg's
objects reads the same; every call goes to libxreg_gb300.so.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from ._lib import call, load


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


# --------------------------------------------------------------------- camera
class CameraModel:
    """xreg::CameraModel (xregPerspectiveXform.h:108-273) as an xr_camera_desc."""

    def __init__(self, desc: L.xr_camera_desc | None = None, recipe: tuple | None = None):
        self.desc = desc if desc is not None else L.xr_camera_desc()
        # How the model was built (set-up, downsampling, crop, extrinsics), step
        # by step; None for a model given as a raw descriptor.
        self.recipe = recipe

    def _derived(self, d, step) -> "CameraModel":
        return CameraModel(d, None if self.recipe is None else self.recipe + (step,))

    @classmethod
    def naive(cls, focal_len: float, num_rows: int, num_cols: int, row_spacing: float, col_spacing: float,
              coord_frame_type: int = L.XR_CAM_FOCAL_NEG_Z) -> "CameraModel":
        """CameraModel::setup(f, nr, nc, rs, cs) (xregPerspectiveXform.cpp:230-254)."""
        d = L.xr_camera_desc()
        args = (float(focal_len), int(num_rows), int(num_cols), float(row_spacing), float(col_spacing),
                int(coord_frame_type))
        call("xr_camera_setup_naive", *args, C.byref(d))
        return cls(d, (("naive",) + args,))

    def downsample(self, ds_factor: float, force_even_dims: bool = False) -> "CameraModel":
        """DownsampleCameraModel (xregPerspectiveXform.cpp:654-689)."""
        d = L.xr_camera_desc()
        call("xr_camera_downsample", C.byref(self.desc), float(ds_factor), int(force_even_dims), C.byref(d))
        return self._derived(d, ("downsample", float(ds_factor), bool(force_even_dims)))

    def crop_boundary(self, width: int) -> "CameraModel":
        """The camera of CropBoundaryPixels (xregProjData.cpp:543-567 ->
        UpdateCameraModelFor2DROI, xregPerspectiveXform.cpp:482-503)."""
        d = L.xr_camera_desc()
        call("xr_camera_crop_boundary", C.byref(self.desc), int(width), C.byref(d))
        return self._derived(d, ("crop", int(width)))

    @property
    def num_det_rows(self) -> int:
        return int(self.desc.num_det_rows)

    @property
    def num_det_cols(self) -> int:
        return int(self.desc.num_det_cols)

    @property
    def focal_len(self) -> float:
        return float(self.desc.focal_len)

    @property
    def intrins(self) -> np.ndarray:
        return np.array(self.desc.intrins[:], dtype=np.float64).reshape(3, 3)

    @property
    def extrins(self) -> np.ndarray:
        return np.array(self.desc.extrins[:], dtype=np.float64).reshape(4, 4)

    def set_extrins(self, extrins: np.ndarray) -> None:
        """The world -> camera transform; CameraModel holds it in float."""
        e = np.asarray(extrins, dtype=np.float64).reshape(16).astype(np.float32)
        for i in range(16):
            self.desc.extrins[i] = float(e[i])
        if self.recipe is not None:
            self.recipe = self.recipe + (("extrins", tuple(float(v) for v in e)),)

    def as_tuple(self):
        d = self.desc
        return (tuple(d.intrins), tuple(d.extrins), d.num_det_rows, d.num_det_cols, d.det_row_spacing,
                d.det_col_spacing, d.focal_len, d.coord_frame_type)


# --------------------------------------------------------------------- volume
@dataclass
class Volume:
    """A float32 attenuation volume in ITK conventions: voxels[z, y, x] (x fastest),
    physical = origin + direction @ diag(spacing) @ index."""

    voxels: np.ndarray
    spacing: tuple = (1.0, 1.0, 1.0)
    origin: tuple = (0.0, 0.0, 0.0)
    direction: np.ndarray = field(default_factory=lambda: np.eye(3))

    def __post_init__(self):
        self.voxels = np.ascontiguousarray(self.voxels, dtype=np.float32)
        assert self.voxels.ndim == 3

    @property
    def size(self) -> tuple:
        nz, ny, nx = self.voxels.shape
        return (nx, ny, nz)

    def desc(self) -> L.xr_volume_desc:
        d = L.xr_volume_desc()
        nx, ny, nz = self.size
        d.n[0], d.n[1], d.n[2] = nx, ny, nz
        for i in range(3):
            d.spacing[i] = float(self.spacing[i])
            d.origin[i] = float(self.origin[i])
        dirm = np.asarray(self.direction, dtype=np.float64).reshape(9)
        for i in range(9):
            d.direction[i] = float(dirm[i])
        return d

    def index_to_phys(self) -> np.ndarray:
        """ITKImagePhysicalPointTransformsAsEigen (xregITKBasicImageUtils.h:133-165)."""
        T = np.eye(4)
        T[:3, :3] = np.asarray(self.direction, dtype=np.float64) @ np.diag(np.asarray(self.spacing, dtype=np.float64))
        T[:3, 3] = np.asarray(self.origin, dtype=np.float64)
        return T

    def xform_img_center_to_itk_phys(self) -> np.ndarray:
        """RayCaster::xform_img_center_to_itk_phys (xregRayCastInterface.cpp:200-224):
        translation to the physical point of continuous index size/2."""
        c = np.array(self.size, dtype=np.float64) / 2.0
        T = np.eye(4)
        T[:3, 3] = (self.index_to_phys() @ np.append(c, 1.0))[:3]
        return T


# ----------------------------------------------------------------- ray caster
class RayCasterLineIntCUDA:
    """Line-integral DRR ray caster on the GPU with RayCaster's method names."""

    def __init__(self, device: int = -1):
        load()
        h = C.c_void_p()
        call("xr_rc_create", int(device), C.byref(h))
        self._h = h
        self._cams: list[CameraModel] = []
        self._num_projs = 0
        self._vols: list[Volume] = []

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                load().xr_rc_destroy(h)
            except Exception:
                pass
            self._h = None

    def close(self):
        self.__del__()

    # state
    def set_stream(self, cuda_stream: int | None) -> None:
        call("xr_rc_set_stream", self._h, C.c_void_p(cuda_stream or 0))

    def synchronize(self) -> None:
        call("xr_rc_synchronize", self._h)

    def set_volume(self, vol: Volume, voxel_type: int = L.XR_VOXEL_F32, scale: float = 0.0) -> None:
        self.set_volumes([vol], voxel_type, scale)

    def set_volumes(self, vols, voxel_type: int = L.XR_VOXEL_F32, scale: float = 0.0) -> None:
        descs = (L.xr_volume_desc * len(vols))(*[v.desc() for v in vols])
        ptrs = (C.c_void_p * len(vols))(*[v.voxels.ctypes.data for v in vols])
        call("xr_rc_set_volumes", self._h, len(vols), descs, ptrs, int(voxel_type), float(scale))
        self._vols = list(vols)

    def set_volumes_device(self, vols, device_ptrs, voxel_type: int = L.XR_VOXEL_F32, scale: float = 0.0):
        descs = (L.xr_volume_desc * len(vols))(*[v.desc() for v in vols])
        ptrs = (C.c_void_p * len(vols))(*[int(p) for p in device_ptrs])
        call("xr_rc_set_volumes_device", self._h, len(vols), descs, ptrs, int(voxel_type), float(scale))
        self._vols = list(vols)

    def set_camera_model(self, cam: CameraModel) -> None:
        self.set_camera_models([cam])

    def set_camera_models(self, cams) -> None:
        arr = (L.xr_camera_desc * len(cams))(*[c.desc for c in cams])
        call("xr_rc_set_camera_models", self._h, len(cams), arr)
        self._cams = list(cams)

    def camera_models(self):
        return list(self._cams)

    def num_camera_models(self) -> int:
        return len(self._cams)

    def set_num_projs(self, n: int) -> None:
        call("xr_rc_set_num_projs", self._h, int(n))
        self._num_projs = int(n)

    def num_projs(self) -> int:
        v = C.c_int64()
        call("xr_rc_num_projs", self._h, C.byref(v))
        return int(v.value)

    def set_ray_step_size(self, step: float) -> None:
        call("xr_rc_set_ray_step_size", self._h, float(step))

    def set_interp_method(self, m: int) -> None:
        call("xr_rc_set_interp_method", self._h, int(m))

    def use_linear_interp(self) -> None:
        self.set_interp_method(L.XR_INTERP_LINEAR)

    def use_proj_store_replace_method(self) -> None:
        call("xr_rc_set_proj_store_method", self._h, L.XR_PROJ_STORE_REPLACE)

    def use_proj_store_accum_method(self) -> None:
        call("xr_rc_set_proj_store_method", self._h, L.XR_PROJ_STORE_ACCUM)

    def set_default_bg_pixel_val(self, v: float) -> None:
        call("xr_rc_set_default_bg_pixel_val", self._h, float(v))

    def set_kernel_id(self, k: int) -> None:
        call("xr_rc_set_kernel_id", self._h, int(k))

    def set_bg_projs(self, imgs, use_bg_projs: bool = True) -> None:
        arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in imgs]
        ptrs = (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        call("xr_rc_set_bg_projs", self._h, ptrs, int(bool(use_bg_projs)))

    def set_use_bg_projs(self, use: bool) -> None:
        call("xr_rc_set_use_bg_projs", self._h, int(bool(use)))

    def set_xforms_cam_to_itk_phys(self, xforms) -> None:
        x = np.ascontiguousarray(np.asarray(xforms, dtype=np.float64).reshape(-1, 16))
        call("xr_rc_set_xforms_cam_to_itk_phys", self._h, x.shape[0], _ptr(x))
        self._num_projs = x.shape[0]

    def distribute_xforms_among_cam_models(self, xforms) -> None:
        x = np.ascontiguousarray(np.asarray(xforms, dtype=np.float64).reshape(-1, 16))
        call("xr_rc_distribute_xforms_among_cam_models", self._h, x.shape[0], _ptr(x))

    def distribute_xforms_device(self, n: int, d_xforms: int) -> None:
        call("xr_rc_distribute_xforms_device", self._h, int(n), C.c_void_p(int(d_xforms)))

    def set_camera_model_proj_associations(self, cam_idx) -> None:
        a = np.ascontiguousarray(np.asarray(cam_idx, dtype=np.int32))
        call("xr_rc_set_camera_model_proj_associations", self._h, a.shape[0], _ptr(a))

    def camera_model_proj_associations(self) -> np.ndarray:
        n = C.c_int64()
        call("xr_rc_camera_model_proj_associations", self._h, 0, None, C.byref(n))
        out = np.empty(n.value, dtype=np.int32)
        call("xr_rc_camera_model_proj_associations", self._h, n.value, _ptr(out), C.byref(n))
        return out

    def set_proj_cam_model(self, proj_idx: int, cam_idx: int) -> None:
        call("xr_rc_set_proj_cam_model", self._h, int(proj_idx), int(cam_idx))

    def xforms_cam_to_itk_phys(self) -> np.ndarray:
        """Every projection's pose, [num_projs, 4, 4]."""
        n = C.c_int64()
        call("xr_rc_xforms_cam_to_itk_phys", self._h, 0, None, C.byref(n))
        out = np.empty((n.value, 4, 4), dtype=np.float64)
        call("xr_rc_xforms_cam_to_itk_phys", self._h, n.value, _ptr(out), C.byref(n))
        return out

    def pre_multiply_all_xforms(self, pre_xform) -> None:
        m = np.ascontiguousarray(np.asarray(pre_xform, dtype=np.float64).reshape(4, 4))
        call("xr_rc_pre_multiply_all_xforms", self._h, _ptr(m))

    def post_multiply_all_xforms(self, post_xform) -> None:
        m = np.ascontiguousarray(np.asarray(post_xform, dtype=np.float64).reshape(4, 4))
        call("xr_rc_post_multiply_all_xforms", self._h, _ptr(m))

    def num_vols(self) -> int:
        v = C.c_int32()
        call("xr_rc_num_vols", self._h, C.byref(v))
        return v.value

    def num_camera_models(self) -> int:
        v = C.c_int32()
        call("xr_rc_num_camera_models", self._h, C.byref(v))
        return v.value

    def xform_img_center_to_itk_phys(self, vol_idx: int = 0) -> np.ndarray:
        out = np.empty((4, 4), dtype=np.float64)
        call("xr_rc_xform_img_center_to_itk_phys", self._h, int(vol_idx), _ptr(out))
        return out

    def xform_cam_wrt_carm_center_of_rot(self, cam_idx: int = 0) -> np.ndarray:
        out = np.empty((4, 4), dtype=np.float64)
        call("xr_rc_xform_cam_wrt_carm_center_of_rot", self._h, int(cam_idx), _ptr(out))
        return out

    def allocate_resources(self) -> None:
        call("xr_rc_allocate_resources", self._h)

    def max_num_projs_possible(self) -> int:
        v = C.c_int64()
        call("xr_rc_max_num_projs_possible", self._h, C.byref(v))
        return int(v.value)

    def set_count_samples(self, enable: bool) -> None:
        call("xr_rc_set_count_samples", self._h, int(bool(enable)))

    def set_launch_config(self, layout: int = L.XR_LAYOUT_AUTO, block_warps_x: int = 2, unroll: int = 1,
                          warp_rows: int = 4) -> None:
        """DRR launch configuration; warp_rows 4 = 8x4-pixel warps, 8 = 4x8."""
        call("xr_rc_set_launch_config_ex", self._h, int(layout), int(block_warps_x), int(unroll), int(warp_rows))

    def launch_config(self) -> tuple:
        """(layout, block_warps_x, unroll) of the last compute."""
        return self.launch_config_ex()[:3]

    def launch_config_ex(self) -> tuple:
        """(layout, block_warps_x, unroll, warp_rows) of the last compute."""
        a, b, c, d = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        call("xr_rc_get_launch_config_ex", self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d))
        return (a.value, b.value, c.value, d.value)

    def set_build_cell_layout(self, enable: bool) -> None:
        call("xr_rc_set_build_cell_layout", self._h, int(bool(enable)))

    def set_empty_space_skipping(self, enable: bool) -> None:
        call("xr_rc_set_empty_space_skipping", self._h, int(bool(enable)))

    def compute(self, vol_idx: int = 0) -> None:
        call("xr_rc_compute", self._h, int(vol_idx))

    def _shape(self):
        c = self._cams[0]
        return c.num_det_rows, c.num_det_cols

    def proj(self, idx: int) -> np.ndarray:
        r, c = self._shape()
        out = np.empty((r, c), dtype=np.float32)
        call("xr_rc_proj", self._h, int(idx), _ptr(out))
        return out

    def projs(self) -> np.ndarray:
        r, c = self._shape()
        out = np.empty((self.num_projs(), r, c), dtype=np.float32)
        call("xr_rc_copy_projs_to_host", self._h, _ptr(out))
        return out

    def device_pixel_buf(self) -> int:
        p = C.c_void_p()
        call("xr_rc_device_pixel_buf", self._h, C.byref(p))
        return int(p.value or 0)

    def use_other_proj_buf(self, other: "RayCasterLineIntCUDA | None") -> None:
        """RayCaster::use_other_proj_buf: write the images into other's buffer."""
        call("xr_rc_use_other_proj_buf", self._h, other.handle if other is not None else None)
        self._other_ref = other

    def use_external_host_pixel_buf(self, buf: np.ndarray | None) -> None:
        """RayCaster::use_external_host_pixel_buf: a float32 array of
        num_projs x rows x cols that receives the images after each compute
        (read it after synchronize())."""
        if buf is None:
            call("xr_rc_use_external_host_pixel_buf", self._h, None)
        else:
            assert buf.dtype == np.float32 and buf.flags["C_CONTIGUOUS"]
            call("xr_rc_use_external_host_pixel_buf", self._h, _ptr(buf))
        self._ext_ref = buf

    def last_num_samples(self) -> int:
        v = C.c_uint64()
        call("xr_rc_last_num_samples", self._h, C.byref(v))
        return int(v.value)

    def last_num_loaded_samples(self) -> int:
        """Samples the last compute loaded (the others were proven zero and
        skipped); needs set_count_samples(True)."""
        v = C.c_uint64()
        call("xr_rc_last_num_loaded_samples", self._h, C.byref(v))
        return int(v.value)


# -------------------------------------------------------------------- metrics
class ImgSimMetric2DCUDA:
    """Base of the GPU similarity metrics (ImgSimMetric2D, xregImgSimMetric2D.h:42-159)."""

    KIND = -1

    def __init__(self, device: int = -1):
        load()
        h = C.c_void_p()
        call("xr_sm_create", int(self.KIND), int(device), C.byref(h))
        self._h = h
        self._n = 0

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                load().xr_sm_destroy(h)
            except Exception:
                pass
            self._h = None

    def close(self):
        self.__del__()

    def set_stream(self, cuda_stream: int | None) -> None:
        call("xr_sm_set_stream", self._h, C.c_void_p(cuda_stream or 0))

    def set_fixed_image(self, img: np.ndarray) -> None:
        a = np.ascontiguousarray(img, dtype=np.float32)
        call("xr_sm_set_fixed_image", self._h, _ptr(a), a.shape[0], a.shape[1])

    def set_mask(self, mask: np.ndarray | None) -> None:
        if mask is None:
            call("xr_sm_set_mask", self._h, C.c_void_p(0))
        else:
            m = np.ascontiguousarray(mask, dtype=np.uint8)
            call("xr_sm_set_mask", self._h, _ptr(m))

    def set_num_moving_images(self, n: int) -> None:
        call("xr_sm_set_num_moving_images", self._h, int(n))
        self._n = int(n)

    def num_moving_images(self) -> int:
        v = C.c_int64()
        call("xr_sm_num_moving_images", self._h, C.byref(v))
        return v.value

    def num_pix_per_proj(self) -> int:
        v = C.c_int64()
        call("xr_sm_num_pix_per_proj", self._h, C.byref(v))
        return v.value

    def fixed_image(self) -> np.ndarray:
        r, c = C.c_int64(), C.c_int64()
        call("xr_sm_fixed_image", self._h, 0, None, C.byref(r), C.byref(c))
        out = np.empty((r.value, c.value), dtype=np.float32)
        call("xr_sm_fixed_image", self._h, out.size, _ptr(out), C.byref(r), C.byref(c))
        return out

    def mask(self):
        """The mask as set, or None."""
        has = C.c_int32()
        n = self.num_pix_per_proj()
        out = np.empty(n, dtype=np.uint8)
        call("xr_sm_mask", self._h, n, _ptr(out), C.byref(has))
        if not has.value:
            return None
        r, c = C.c_int64(), C.c_int64()
        call("xr_sm_fixed_image", self._h, 0, None, C.byref(r), C.byref(c))
        return out.reshape(r.value, c.value)

    def num_moving_images(self) -> int:
        return self._n

    def set_mov_imgs_buf_from_ray_caster(self, rc: RayCasterLineIntCUDA, proj_offset: int = 0) -> None:
        call("xr_sm_set_mov_imgs_buf_from_ray_caster", self._h, rc.handle, int(proj_offset))
        self._rc_ref = rc  # keep the ray caster alive at least as long as this metric

    def set_mov_imgs_host_buf(self, imgs: np.ndarray) -> None:
        """ImgSimMetric2D::set_mov_imgs_host_buf: float32 images (n x rows x cols),
        copied to the device at every compute."""
        a = np.ascontiguousarray(imgs, dtype=np.float32)
        self._host_ref = a
        call("xr_sm_set_mov_imgs_host_buf", self._h, _ptr(a))

    def set_mov_imgs_device_buf(self, d_ptr: int, proj_offset: int = 0) -> None:
        call("xr_sm_set_mov_imgs_device_buf", self._h, C.c_void_p(int(d_ptr)), int(proj_offset))

    def allocate_resources(self) -> None:
        call("xr_sm_allocate_resources", self._h)

    def compute(self) -> None:
        call("xr_sm_compute", self._h)

    def sim_vals(self) -> np.ndarray:
        out = np.empty(self._n, dtype=np.float32)
        call("xr_sm_sim_vals", self._h, _ptr(out))
        return out

    def sim_val(self, i: int) -> float:
        return float(self.sim_vals()[i])

    def device_sim_vals(self) -> int:
        p = C.c_void_p()
        call("xr_sm_device_sim_vals", self._h, C.byref(p))
        return int(p.value or 0)


class _GradParams:
    def set_smooth_img_before_sobel_kernel_radius(self, r: int) -> None:
        call("xr_sm_set_smooth_img_before_sobel_kernel_radius", self._h, int(r))


class _PatchParams:
    def set_patch_radius(self, r: int) -> None:
        call("xr_sm_set_patch_radius", self._h, int(r))

    def set_patch_stride(self, s: int) -> None:
        call("xr_sm_set_patch_stride", self._h, int(s))

    def patch_options(self) -> dict:
        o = L.xr_patch_options()
        call("xr_sm_get_patch_options", self._h, C.byref(o))
        return {k: getattr(o, k) for k, _ in L.xr_patch_options._fields_}

    def set_patch_options(self, **kw) -> None:
        """ImgSimMetric2DPatchCommon / PatchNCC / PatchGradNCC setters by name
        (use_mask_for_weighting, use_mask_for_patch_stats, normalize_weights_as_prob,
        weight_patch_sims_in_combine, compute_mean_of_patch_sims,
        use_fixed_img_patch_variances_as_wgts, use_mov_img_patch_variances_as_wgts,
        use_variances_in_grad_imgs_as_wgts, choose_rand_patches, mask_only_for_weights,
        num_rand_patches, rand_patch_min_pixels_sep, rand_seed); unnamed ones keep their values."""
        o = L.xr_patch_options()
        call("xr_sm_get_patch_options", self._h, C.byref(o))
        for k, v in kw.items():
            if k not in dict(L.xr_patch_options._fields_):
                raise TypeError(f"unknown patch option {k!r}")
            setattr(o, k, type(getattr(o, k))(v) if not isinstance(getattr(o, k), float) else float(v))
        call("xr_sm_set_patch_options", self._h, C.byref(o))

    def set_wgt_img(self, img: np.ndarray | None) -> None:
        if img is None:
            call("xr_sm_set_patch_wgt_img", self._h, None)
        else:
            a = np.ascontiguousarray(img, dtype=np.float32)
            call("xr_sm_set_patch_wgt_img", self._h, _ptr(a))

    def patch_indices_used(self) -> np.ndarray:
        n = C.c_int64()
        call("xr_sm_patch_indices_used", self._h, 0, None, C.byref(n))
        out = np.empty(n.value, dtype=np.int64)
        call("xr_sm_patch_indices_used", self._h, n.value, _ptr(out), C.byref(n))
        return out

    def set_patches_to_use(self, idx) -> None:
        """set_patches_to_use (grid indices, repeats counted); empty or None = reset_patches_to_use."""
        a = np.ascontiguousarray(np.asarray([] if idx is None else idx, dtype=np.int64).ravel())
        call("xr_sm_set_patches_to_use", self._h, a.size, _ptr(a) if a.size else None)

    def reset_patches_to_use(self) -> None:
        self.set_patches_to_use(None)

    def patch_scores(self, img: int) -> np.ndarray:
        """sim_vals_for_each_patch for moving image img of the last compute (patches
        in use order; needs save_all_per_patch_scores before allocate_resources)."""
        n = C.c_int64()
        call("xr_sm_patch_scores", self._h, int(img), 0, None, C.byref(n))
        out = np.empty(n.value, dtype=np.float32)
        call("xr_sm_patch_scores", self._h, int(img), n.value, _ptr(out), C.byref(n))
        return out


class ImgSimMetric2DNCCCUDA(ImgSimMetric2DCUDA):
    KIND = L.XR_SIM_NCC


class ImgSimMetric2DGradNCCCUDA(ImgSimMetric2DCUDA, _GradParams):
    KIND = L.XR_SIM_GRAD_NCC


class ImgSimMetric2DPatchNCCCUDA(ImgSimMetric2DCUDA, _PatchParams):
    KIND = L.XR_SIM_PATCH_NCC


class ImgSimMetric2DPatchGradNCCCUDA(ImgSimMetric2DCUDA, _GradParams, _PatchParams):
    KIND = L.XR_SIM_PATCH_GRAD_NCC


# ------------------------------------------------------ population objective
class PopulationObjective:
    """Intensity2D3DRegi::obj_fn for one object (xregIntensity2D3DRegi.cpp:571-742):
    poses -> DRR per (view, pose) -> metric per view -> mean over views."""

    def __init__(self, rc: RayCasterLineIntCUDA, metrics, max_pop: int, vol_idx: int = 0):
        hs = (C.c_void_p * len(metrics))(*[m.handle.value for m in metrics])
        h = C.c_void_p()
        call("xr_obj_create", rc.handle, int(vol_idx), len(metrics), hs, int(max_pop), C.byref(h))
        self._h = h
        self.rc = rc
        self.metrics = list(metrics)
        for m in self.metrics:
            m._rc_ref = rc
        self.max_pop = int(max_pop)

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                load().xr_obj_destroy(h)
            except Exception:
                pass
            self._h = None

    def close(self):
        self.__del__()

    def eval(self, xforms) -> np.ndarray:
        x = np.ascontiguousarray(np.asarray(xforms, dtype=np.float64).reshape(-1, 16))
        out = np.empty(x.shape[0], dtype=np.float32)
        call("xr_obj_eval", self._h, x.shape[0], _ptr(x), _ptr(out))
        return out

    def eval_device(self, pop: int, d_xforms: int, d_sims: int) -> None:
        call("xr_obj_eval_device", self._h, int(pop), C.c_void_p(int(d_xforms)), C.c_void_p(int(d_sims)))

    def set_fused(self, enable: bool) -> None:
        """Split (default) or fused evaluation path; identical values (xr_obj_set_fused)."""
        call("xr_obj_set_fused", self._h, int(bool(enable)))


# ------------------------------------------------------------------ job sets
class JobSet:
    """One step of several registrations at once: one geometry launch, one
    DRR launch and one batched grad-NCC launch over every listed objective's
    work (or the fused DRR + grad-NCC launch) (xr_jobset_*)."""

    def __init__(self, device: int = -1):
        load()
        h = C.c_void_p()
        call("xr_jobset_create", int(device), C.byref(h))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                load().xr_jobset_destroy(h)
            except Exception:
                pass
            self._h = None

    def close(self):
        self.__del__()

    def set_stream(self, cuda_stream: int | None) -> None:
        call("xr_jobset_set_stream", self._h, C.c_void_p(cuda_stream or 0))

    def eval(self, objectives, poses_per_job):
        """poses_per_job[i]: [pop_i, 4, 4] for objectives[i]; returns a list of value arrays."""
        n = len(objectives)
        xs = [np.ascontiguousarray(np.asarray(p, dtype=np.float64).reshape(-1, 16)) for p in poses_per_job]
        outs = [np.empty(x.shape[0], dtype=np.float32) for x in xs]
        objs = (C.c_void_p * n)(*[o._h.value for o in objectives])
        pops = (C.c_int64 * n)(*[x.shape[0] for x in xs])
        xp = (C.c_void_p * n)(*[x.ctypes.data for x in xs])
        op = (C.c_void_p * n)(*[o.ctypes.data for o in outs])
        call("xr_jobset_eval", self._h, n, objs, pops, xp, op)
        return outs

    def eval_device(self, objectives, pops, d_xforms, d_sims) -> None:
        n = len(objectives)
        objs = (C.c_void_p * n)(*[o._h.value for o in objectives])
        pp = (C.c_int64 * n)(*[int(p) for p in pops])
        xp = (C.c_void_p * n)(*[int(p) for p in d_xforms])
        sp = (C.c_void_p * n)(*[int(p) for p in d_sims])
        call("xr_jobset_eval_device", self._h, n, objs, pp, xp, sp)

    def regi_step(self, step_jobs) -> tuple:
        """xr_regi_jobset_step: one generation of every job (xr_regi_step_job
        structs); returns (stop codes, poses evaluated) per job."""
        n = len(step_jobs)
        arr = (L.xr_regi_step_job * n)(*step_jobs)
        stop = (C.c_int32 * n)()
        ev = (C.c_int32 * n)()
        call("xr_regi_jobset_step", self._h, n, arr, stop, ev)
        return list(stop), list(ev)

    def last_launch(self):
        a, b = C.c_int64(), C.c_int32()
        call("xr_jobset_last_launch", self._h, C.byref(a), C.byref(b))
        return a.value, b.value

    def set_fused(self, enable: bool) -> None:
        """Batched split (default) or fused evaluation step; identical values (xr_jobset_set_fused)."""
        call("xr_jobset_set_fused", self._h, int(bool(enable)))

    def set_pose_groups(self, mode: int) -> None:
        """DRR items of 4 consecutive projections mapped by their coherence:
        0 never, 1 for jobs whose poses lie within a voxel, 2 for every job
        (xr_jobset_set_pose_groups); identical values in every mode."""
        call("xr_jobset_set_pose_groups", self._h, int(mode))

    def last_pose_grouped(self) -> int:
        """Jobs of the last step that ran pose-grouped DRR items."""
        v = C.c_int32()
        call("xr_jobset_last_pose_grouped", self._h, C.byref(v))
        return int(v.value)

    def last_kernel_launches(self) -> int:
        """Kernel launches of the last step."""
        v = C.c_int32()
        call("xr_jobset_last_kernel_launches", self._h, C.byref(v))
        return int(v.value)


# --------------------------------------------------------- data preparation
def hu_to_lin_att_device(d_hu: int, n: int, d_mu: int, stream: int = 0) -> None:
    """HUToLinAtt on device buffers (xr_hu_to_lin_att); asynchronous on `stream`."""
    call("xr_hu_to_lin_att", C.c_void_p(int(d_hu)), int(n), C.c_void_p(int(d_mu)), C.c_void_p(int(stream)))


def downsample_size(rows: int, cols: int, factor: float) -> tuple:
    r, c = C.c_int64(), C.c_int64()
    call("xr_downsample_image_size", int(rows), int(cols), float(factor), C.byref(r), C.byref(c))
    return r.value, c.value


def downsample_image(img: np.ndarray, factor: float, device: int = -1) -> np.ndarray:
    """DownsampleProjData's image part on the GPU (discrete Gaussian + resampling)."""
    import torch
    dev = torch.device("cuda", device if device >= 0 else torch.cuda.current_device())
    src = torch.from_numpy(np.ascontiguousarray(img, dtype=np.float32)).to(dev)
    rows, cols = src.shape
    orows, ocols = downsample_size(rows, cols, factor)
    scratch = torch.empty(2 * rows * cols, dtype=torch.float64, device=dev)
    dst = torch.empty((orows, ocols), dtype=torch.float32, device=dev)
    s = torch.cuda.current_stream(dev)
    call("xr_downsample_image", C.c_void_p(src.data_ptr()), rows, cols, float(factor),
         C.c_void_p(scratch.data_ptr()), C.c_void_p(dst.data_ptr()), C.c_void_p(s.cuda_stream))
    s.synchronize()
    return dst.cpu().numpy()


def crop_image_boundary(img: np.ndarray, width: int, device: int = -1) -> np.ndarray:
    """CropImage2DBoundary on the GPU (xr_crop_image_boundary)."""
    import torch
    dev = torch.device("cuda", device if device >= 0 else torch.cuda.current_device())
    src = torch.from_numpy(np.ascontiguousarray(img, dtype=np.float32)).to(dev)
    rows, cols = src.shape
    dst = torch.empty((max(rows - 2 * width, 0), max(cols - 2 * width, 0)), dtype=torch.float32, device=dev)
    s = torch.cuda.current_stream(dev)
    call("xr_crop_image_boundary", C.c_void_p(src.data_ptr()), rows, cols, int(width), C.c_void_p(dst.data_ptr()),
         C.c_void_p(s.cuda_stream))
    s.synchronize()
    return dst.cpu().numpy()


def log_remap(img: np.ndarray, use_max_as_i0: bool = True, i0: float = 1.0, device: int = -1) -> np.ndarray:
    """ImageIntensLogTransFilter as ProjPreProc runs it, on the GPU (xr_log_remap)."""
    import torch
    dev = torch.device("cuda", device if device >= 0 else torch.cuda.current_device())
    src = torch.from_numpy(np.ascontiguousarray(img, dtype=np.float32)).to(dev)
    rows, cols = src.shape
    scratch = torch.empty(rows * cols + 1025, dtype=torch.float64, device=dev)
    dst = torch.empty_like(src)
    s = torch.cuda.current_stream(dev)
    call("xr_log_remap", C.c_void_p(src.data_ptr()), rows, cols, int(bool(use_max_as_i0)), float(i0),
         C.c_void_p(scratch.data_ptr()), C.c_void_p(dst.data_ptr()), C.c_void_p(s.cuda_stream))
    s.synchronize()
    return dst.cpu().numpy()


def proj_preproc(img: np.ndarray, cam: CameraModel, crop_width: int = 50, no_log_remap: bool = False,
                 device: int = -1):
    """ProjPreProc::operator() (xregProjPreProc.cpp:31-139) for one projection with
    its defaults (crop 50 pixels from every side, then the log remap with I0 from
    the smoothed maximum; metal auto-masking is not part of it here).  Returns
    (image, camera)."""
    out, c = np.ascontiguousarray(img, dtype=np.float32), cam
    if crop_width > 0:
        c = cam.crop_boundary(crop_width)
        out = crop_image_boundary(out, crop_width, device)
    if not no_log_remap:
        out = log_remap(out, True, 1.0, device)
    return out, c


# ------------------------------------------------------------ poses on disk
def regi_pose_map(centre, start_pose, xs) -> np.ndarray:
    """xr_regi_pose_map: pose = centre @ Exp(x) @ inv(centre) @ start_pose for each row x."""
    c = np.ascontiguousarray(centre, dtype=np.float64)
    s = np.ascontiguousarray(start_pose, dtype=np.float64)
    x = np.ascontiguousarray(xs, dtype=np.float64).reshape(-1, 6)
    out = np.empty((x.shape[0], 4, 4), dtype=np.float64)
    call("xr_regi_pose_map", _ptr(c), _ptr(s), x.shape[0], _ptr(x), _ptr(out))
    return out


def read_itk_affine_transform(path: str) -> np.ndarray:
    """ReadITKAffineTransformFromFile: the 4x4 pose in an ITK text transform file
    (".txt" / ".tfm"; xr_itk_affine_transform_read)."""
    out = np.empty((4, 4), dtype=np.float64)
    call("xr_itk_affine_transform_read", os.fsencode(path), out.ctypes.data_as(C.c_void_p))
    return out


def read_slicer_affine_transform(path: str) -> np.ndarray:
    """ReadSlicerAffineTransformFromFile: the inverse of the file's pose
    (xr_itk_slicer_affine_transform_read)."""
    out = np.empty((4, 4), dtype=np.float64)
    call("xr_itk_slicer_affine_transform_read", os.fsencode(path), out.ctypes.data_as(C.c_void_p))
    return out


def write_itk_affine_transform(path: str, xform) -> None:
    """WriteITKAffineTransform: the pose as an AffineTransform_float_3_3 in an ITK
    text transform file (xr_itk_affine_transform_write)."""
    x = np.ascontiguousarray(np.asarray(xform, dtype=np.float64).reshape(4, 4))
    call("xr_itk_affine_transform_write", os.fsencode(path), x.ctypes.data_as(C.c_void_p))


def simple_ray_cast(rc: RayCasterLineIntCUDA, cam_world_to_vols, inter_frames=None, inter_frames_wrt_vol=None,
                    ref_frames_cam_world_to_vol=None, vols_to_proj=None) -> list:
    """SimpleRayCasterWrapperFn (xregRayCastInterface.cpp:456-533): one projection
    per camera of every volume in vols_to_proj (all when None) at
    cam_world_to_vols[i], the first replacing and the rest accumulating, about
    optional intermediate frames; returns the projection of each camera and
    restores the caster's projection count and camera associations."""
    nv = len(vols_to_proj) if vols_to_proj is not None else rc.num_vols()
    poses = [np.asarray(x, dtype=np.float64).reshape(4, 4) for x in cam_world_to_vols]
    if len(poses) != nv:
        raise ValueError("simple_ray_cast: one pose per volume")
    inter = inter_frames is not None and len(inter_frames) > 0
    if inter and not (len(inter_frames) == nv == len(inter_frames_wrt_vol) == len(ref_frames_cam_world_to_vol)):
        raise ValueError("simple_ray_cast: one intermediate frame per volume")
    ncam = rc.num_camera_models()
    prev_n = rc.num_projs()
    assocs = rc.camera_model_proj_associations()
    rc.set_num_projs(ncam)
    for v in range(nv):
        if v == 0:
            rc.use_proj_store_replace_method()
        else:
            rc.use_proj_store_accum_method()
        rc.distribute_xforms_among_cam_models(poses[v][None])
        if inter:
            F = np.asarray(inter_frames[v], dtype=np.float64).reshape(4, 4)
            R = np.asarray(ref_frames_cam_world_to_vol[v], dtype=np.float64).reshape(4, 4)
            if inter_frames_wrt_vol[v]:
                rc.pre_multiply_all_xforms(F)
                rc.post_multiply_all_xforms(np.linalg.inv(F) @ R)
            else:
                rc.pre_multiply_all_xforms(R @ F)
                rc.post_multiply_all_xforms(np.linalg.inv(F))
        rc.compute(int(vols_to_proj[v]) if vols_to_proj is not None else v)
    projs = [rc.proj(c) for c in range(ncam)]
    rc.set_num_projs(prev_n)
    if prev_n > 0 and assocs.size == prev_n:
        rc.set_camera_model_proj_associations(assocs)
    return projs


def measure_l2_read_bandwidth(device: int = -1, nbytes: int = 48 << 20, reps: int = 40) -> float:
    """Measured L2 read bandwidth of a device in GB/s (xr_measure_l2_read_bandwidth)."""
    v = C.c_double()
    call("xr_measure_l2_read_bandwidth", int(device), int(nbytes), int(reps), C.byref(v))
    return float(v.value)
