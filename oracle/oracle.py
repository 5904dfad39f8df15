"""ctypes wrapper of the CPU oracle (oracle/xr_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The product never imports it.
Parity status: unpinned against the reference binary (it cannot be built here
and ships no golden vectors); pinned by analytic known-answer tests.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libxr_oracle.so"
CMAES_REF = HERE / "_ref" / "libcmaes_ref.so"


class vol_geom(C.Structure):
    _fields_ = [("n", C.c_int64 * 3), ("spacing", C.c_double * 3), ("origin", C.c_double * 3),
                ("direction", C.c_double * 9)]


class camera(C.Structure):
    _fields_ = [("intrins", C.c_double * 9), ("extrins", C.c_double * 16), ("num_det_rows", C.c_int64),
                ("num_det_cols", C.c_int64), ("det_row_spacing", C.c_double), ("det_col_spacing", C.c_double),
                ("focal_len", C.c_double), ("coord_frame_type", C.c_int32), ("pad_", C.c_int32)]


class proj_geom(C.Structure):
    """Per-projection float set-up (xo_proj_geom): 44 floats."""
    _fields_ = [("M", C.c_float * 12), ("pin_idx", C.c_float * 3), ("Ki", C.c_float * 9), ("dz", C.c_float),
                ("zadj", C.c_float), ("Ei", C.c_float * 12), ("pin", C.c_float * 3), ("pad", C.c_float * 3)]


def build(force: bool = False) -> Path:
    if force or not LIB.exists() or LIB.stat().st_mtime < (HERE / "xr_oracle.c").stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE), "_build/libxr_oracle.so"], check=True)
    return LIB


def reference_dir() -> str | None:
    """The xReg source tree named by XREG_REFERENCE_DIR, if it is set and present."""
    d = os.environ.get("XREG_REFERENCE_DIR")
    return d if d and Path(d).is_dir() else None


def build_ref(ref_dir: str | None = None) -> Path | None:
    """Compiles the reference's vendored CMA-ES when its sources are present
    (ref_dir, else XREG_REFERENCE_DIR)."""
    if CMAES_REF.exists():
        return CMAES_REF
    ref_dir = ref_dir or reference_dir()
    if not ref_dir or not Path(ref_dir, "third_party", "cmaes", "cmaes.c").exists():
        return None
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF_DIR={ref_dir}"], check=True)
    return CMAES_REF


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        i64 = C.c_int64
        L.xo_set_num_threads.argtypes = [C.c_int]
        L.xo_get_num_threads.restype = C.c_int
        L.xo_drr_f32.argtypes = [P, C.POINTER(vol_geom), C.POINTER(camera), i64, P, P, i64, C.c_float, C.c_int,
                                 C.c_int, C.c_float, P, P, P]
        L.xo_drr_f64.argtypes = [P, C.POINTER(vol_geom), C.POINTER(camera), i64, P, P, i64, C.c_float, C.c_int,
                                 C.c_double, P, P]
        L.xo_proj_geoms.argtypes = [C.POINTER(vol_geom), C.POINTER(camera), P, P, i64, C.POINTER(proj_geom)]
        L.xo_camera_setup_naive.argtypes = [C.c_double, i64, i64, C.c_double, C.c_double, C.c_int32,
                                            C.POINTER(camera)]
        L.xo_camera_downsample.argtypes = [C.POINTER(camera), C.c_double, C.c_int, C.POINTER(camera)]
        L.xo_camera_crop_boundary.argtypes = [C.POINTER(camera), i64, C.POINTER(camera)]
        L.xo_frame_mul_f32.argtypes = [P, P, P]
        L.xo_ray_setups.argtypes = [C.POINTER(vol_geom), C.POINTER(camera), i64, P, P, i64, C.c_float, P, P, P, P]
        L.xo_grad_images.argtypes = [P, i64, i64, C.c_int, P, P]
        L.xo_ncc.argtypes = [P, P, i64, i64, P, P]
        L.xo_grad_ncc.argtypes = [P, P, i64, i64, i64, C.c_int, P, P]
        L.xo_grad_ncc_par.argtypes = [P, P, i64, i64, i64, C.c_int, P]
        L.xo_patch_ncc.argtypes = [P, P, i64, i64, i64, i64, i64, P]
        L.xo_patch_grad_ncc.argtypes = [P, P, i64, i64, i64, C.c_int, i64, i64, P]
        L.xo_hu_to_lin_att.argtypes = [P, i64, P]
        _lib = L
    return _lib


def set_threads(n: int | None = None) -> int:
    n = n or os.cpu_count() or 1
    lib().xo_set_num_threads(int(n))
    return n


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def vol_geom_of(voxels: np.ndarray, spacing, origin=(0, 0, 0), direction=None) -> vol_geom:
    g = vol_geom()
    nz, ny, nx = voxels.shape
    g.n[0], g.n[1], g.n[2] = nx, ny, nz
    d = np.eye(3) if direction is None else np.asarray(direction, dtype=np.float64)
    for i in range(3):
        g.spacing[i] = float(spacing[i])
        g.origin[i] = float(origin[i])
    for i in range(9):
        g.direction[i] = float(d.reshape(9)[i])
    return g


def camera_from_tuple(t) -> camera:
    """From the product's CameraModel.as_tuple() (same fields)."""
    c = camera()
    intr, extr, nr, nc, rs, cs, f, frame = t
    for i in range(9):
        c.intrins[i] = intr[i]
    for i in range(16):
        c.extrins[i] = extr[i]
    c.num_det_rows, c.num_det_cols = nr, nc
    c.det_row_spacing, c.det_col_spacing, c.focal_len, c.coord_frame_type = rs, cs, f, frame
    return c


def camera_naive(f, nr, nc, rs, cs, frame=1) -> camera:
    c = camera()
    lib().xo_camera_setup_naive(f, nr, nc, rs, cs, frame, C.byref(c))
    return c


def camera_downsample(c: camera, ds: float, force_even: bool = False) -> camera:
    d = camera()
    lib().xo_camera_downsample(C.byref(c), ds, int(force_even), C.byref(d))
    return d


def camera_crop_boundary(c: camera, width: int) -> camera:
    d = camera()
    lib().xo_camera_crop_boundary(C.byref(c), int(width), C.byref(d))
    return d


def camera_fields(c: camera) -> tuple:
    """Every field of a camera, for field-by-field comparisons."""
    return (tuple(c.intrins), tuple(c.extrins), c.num_det_rows, c.num_det_cols, c.det_row_spacing,
            c.det_col_spacing, c.focal_len, c.coord_frame_type)


def frame_mul_f32(a, b) -> np.ndarray:
    """FrameTransform product a * b in xReg's float arithmetic (4x4 in, 4x4 out)."""
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(16)
    b = np.ascontiguousarray(b, dtype=np.float64).reshape(16)
    out = np.zeros(16)
    lib().xo_frame_mul_f32(_p(a), _p(b), _p(out))
    return out.reshape(4, 4)


def ray_setups(geom: vol_geom, cams, poses, cam_idx=None, step=1.0):
    """xReg's per-ray float set-up of every pixel: (hit, samples, start, step vector),
    shapes [n, rows, cols] and [n, rows, cols, 3]."""
    poses = np.ascontiguousarray(np.asarray(poses, dtype=np.float64).reshape(-1, 16))
    n = poses.shape[0]
    cams = list(cams)
    ci = np.zeros(n, dtype=np.int32) if cam_idx is None else np.ascontiguousarray(cam_idx, dtype=np.int32)
    carr = (camera * len(cams))(*cams)
    rows, cols = cams[0].num_det_rows, cams[0].num_det_cols
    hit = np.zeros((n, rows, cols), np.int32)
    ns = np.zeros((n, rows, cols), np.uint64)
    st = np.zeros((n, rows, cols, 3), np.float32)
    sv = np.zeros((n, rows, cols, 3), np.float32)
    assert lib().xo_ray_setups(C.byref(geom), carr, len(cams), _p(poses), _p(ci), n, step, _p(hit), _p(ns), _p(st),
                               _p(sv)) == 0
    return hit, ns, st, sv


def drr_f32(voxels, geom: vol_geom, cams, poses, cam_idx=None, step=1.0, kernel=0, store=0, default_bg=0.0,
            bg_projs=None, out=None, count=False):
    """FP32 xReg-CPU semantics.  poses: [n, 4, 4] cam -> ITK phys. Returns [n, rows, cols]."""
    voxels = np.ascontiguousarray(voxels, dtype=np.float32)
    poses = np.ascontiguousarray(np.asarray(poses, dtype=np.float64).reshape(-1, 16))
    n = poses.shape[0]
    cams = list(cams)
    ci = np.zeros(n, dtype=np.int32) if cam_idx is None else np.ascontiguousarray(cam_idx, dtype=np.int32)
    carr = (camera * len(cams))(*cams)
    rows, cols = cams[0].num_det_rows, cams[0].num_det_cols
    if out is None:
        out = np.zeros((n, rows, cols), dtype=np.float32)
    bg = None if bg_projs is None else np.ascontiguousarray(bg_projs, dtype=np.float32)
    ns = np.zeros((n, rows, cols), dtype=np.uint64) if count else None
    rc = lib().xo_drr_f32(_p(voxels), C.byref(geom), carr, len(cams), _p(poses), _p(ci), n, step, kernel, store,
                          default_bg, None if bg is None else _p(bg), _p(out), None if ns is None else _p(ns))
    assert rc == 0
    return (out, ns) if count else out


def drr_f64(voxels, geom: vol_geom, cams, poses, cam_idx=None, step=1.0, kernel=0, default_bg=0.0, count=False):
    voxels = np.ascontiguousarray(voxels, dtype=np.float32)
    poses = np.ascontiguousarray(np.asarray(poses, dtype=np.float64).reshape(-1, 16))
    n = poses.shape[0]
    cams = list(cams)
    ci = np.zeros(n, dtype=np.int32) if cam_idx is None else np.ascontiguousarray(cam_idx, dtype=np.int32)
    carr = (camera * len(cams))(*cams)
    rows, cols = cams[0].num_det_rows, cams[0].num_det_cols
    out = np.zeros((n, rows, cols), dtype=np.float64)
    ns = np.zeros((n, rows, cols), dtype=np.uint64) if count else None
    rc = lib().xo_drr_f64(_p(voxels), C.byref(geom), carr, len(cams), _p(poses), _p(ci), n, step, kernel,
                          default_bg, _p(out), None if ns is None else _p(ns))
    assert rc == 0
    return (out, ns) if count else out


def proj_geoms(geom: vol_geom, cams, poses, cam_idx=None) -> np.ndarray:
    poses = np.ascontiguousarray(np.asarray(poses, dtype=np.float64).reshape(-1, 16))
    n = poses.shape[0]
    ci = np.zeros(n, dtype=np.int32) if cam_idx is None else np.ascontiguousarray(cam_idx, dtype=np.int32)
    carr = (camera * len(cams))(*cams)
    out = (proj_geom * n)()
    lib().xo_proj_geoms(C.byref(geom), carr, _p(poses), _p(ci), n, out)
    return np.frombuffer(out, dtype=np.float32).reshape(n, 44).copy()


def grad_images(img, smooth_ksize=5):
    img = np.ascontiguousarray(img, dtype=np.float32)
    gx = np.zeros(img.shape, dtype=np.float64)
    gy = np.zeros(img.shape, dtype=np.float64)
    assert lib().xo_grad_images(_p(img), img.shape[0], img.shape[1], smooth_ksize, _p(gx), _p(gy)) == 0
    return gx, gy


def ncc(fixed, movs, mask=None) -> np.ndarray:
    f = np.ascontiguousarray(fixed, dtype=np.float32)
    m = np.ascontiguousarray(movs, dtype=np.float32).reshape(-1, f.size)
    out = np.zeros(m.shape[0], dtype=np.float64)
    mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
    lib().xo_ncc(_p(f), _p(m), f.size, m.shape[0], None if mk is None else _p(mk), _p(out))
    return out


def grad_ncc(fixed, movs, smooth_ksize=5, mask=None) -> np.ndarray:
    f = np.ascontiguousarray(fixed, dtype=np.float32)
    m = np.ascontiguousarray(movs, dtype=np.float32).reshape(-1, *f.shape)
    out = np.zeros(m.shape[0], dtype=np.float64)
    mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
    if mk is None:
        lib().xo_grad_ncc_par(_p(f), _p(m), f.shape[0], f.shape[1], m.shape[0], smooth_ksize, _p(out))
    else:
        assert lib().xo_grad_ncc(_p(f), _p(m), f.shape[0], f.shape[1], m.shape[0], smooth_ksize, _p(mk),
                                 _p(out)) == 0
    return out


def patch_ncc(fixed, movs, radius=5, stride=1) -> np.ndarray:
    f = np.ascontiguousarray(fixed, dtype=np.float32)
    m = np.ascontiguousarray(movs, dtype=np.float32).reshape(-1, *f.shape)
    out = np.zeros(m.shape[0], dtype=np.float64)
    lib().xo_patch_ncc(_p(f), _p(m), f.shape[0], f.shape[1], m.shape[0], radius, stride, _p(out))
    return out


def patch_grad_ncc(fixed, movs, smooth_ksize=5, radius=5, stride=1) -> np.ndarray:
    f = np.ascontiguousarray(fixed, dtype=np.float32)
    m = np.ascontiguousarray(movs, dtype=np.float32).reshape(-1, *f.shape)
    out = np.zeros(m.shape[0], dtype=np.float64)
    assert lib().xo_patch_grad_ncc(_p(f), _p(m), f.shape[0], f.shape[1], m.shape[0], smooth_ksize, radius, stride,
                                   _p(out)) == 0
    return out


class patch_opts(C.Structure):
    """Options of the masked / weighted patch metrics (xReg's defaults)."""
    _fields_ = [("use_mask_for_weighting", C.c_int), ("use_mask_for_patch_stats", C.c_int),
                ("normalize_weights_as_prob", C.c_int), ("weight_patch_sims_in_combine", C.c_int),
                ("compute_mean_of_patch_sims", C.c_int), ("use_fixed_var_wgts", C.c_int),
                ("use_mov_var_wgts", C.c_int), ("use_grad_var_wgts", C.c_int),
                ("wgt_img", C.c_void_p), ("patch_count", C.c_void_p), ("mask_only_for_weights", C.c_int)]


def _patch_opts(opts, shape, keep):
    o = patch_opts(1, 0, 1, 1, 0, 0, 0, 0, None, None, 0)
    for k, v in (opts or {}).items():
        if k == "wgt_img":
            a = np.ascontiguousarray(v, dtype=np.float32).reshape(shape)
            keep.append(a)
            o.wgt_img = a.ctypes.data
        elif k == "patch_count":
            a = np.ascontiguousarray(v, dtype=np.int32)
            keep.append(a)
            o.patch_count = a.ctypes.data
        else:
            setattr(o, k, int(v))
    return o


def patch_ncc_ex(fixed, movs, radius=5, stride=1, mask=None, **opts) -> np.ndarray:
    """Patch NCC with an optional mask and xReg's weighting options (double arithmetic)."""
    f = np.ascontiguousarray(fixed, dtype=np.float32)
    m = np.ascontiguousarray(movs, dtype=np.float32).reshape(-1, *f.shape)
    keep = []
    mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8).reshape(f.shape)
    o = _patch_opts(opts, f.shape, keep)
    out = np.zeros(m.shape[0], dtype=np.float64)
    L = lib()
    L.xo_patch_ncc_ex.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                  C.c_void_p, C.POINTER(patch_opts), C.c_void_p]
    assert L.xo_patch_ncc_ex(_p(f), _p(m), f.shape[0], f.shape[1], m.shape[0], radius, stride,
                             None if mk is None else _p(mk), C.byref(o), _p(out)) == 0
    return out


def patch_grad_ncc_ex(fixed, movs, smooth_ksize=5, radius=5, stride=1, mask=None, **opts) -> np.ndarray:
    """Patch grad-NCC with an optional mask and xReg's weighting options (double arithmetic)."""
    f = np.ascontiguousarray(fixed, dtype=np.float32)
    m = np.ascontiguousarray(movs, dtype=np.float32).reshape(-1, *f.shape)
    keep = []
    mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8).reshape(f.shape)
    o = _patch_opts(opts, f.shape, keep)
    out = np.zeros(m.shape[0], dtype=np.float64)
    L = lib()
    L.xo_patch_grad_ncc_ex.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_int,
                                       C.c_int64, C.c_int64, C.c_void_p, C.POINTER(patch_opts), C.c_void_p]
    assert L.xo_patch_grad_ncc_ex(_p(f), _p(m), f.shape[0], f.shape[1], m.shape[0], smooth_ksize, radius, stride,
                                  None if mk is None else _p(mk), C.byref(o), _p(out)) == 0
    return out


def hu_to_lin_att(hu) -> np.ndarray:
    h = np.ascontiguousarray(hu, dtype=np.float32)
    out = np.empty_like(h)
    lib().xo_hu_to_lin_att(_p(h), h.size, _p(out))
    return out


class RefCMAES:
    """The reference's vendored CMA-ES (cmaes.c) through oracle/_ref (checker only)."""

    _lib = None

    def __init__(self, xstart, stddevs, lam, seed, tol_fun=1e-12, tol_x=1e-11, max_iter=1e6):
        if RefCMAES._lib is None:
            p = build_ref()
            if p is None:
                raise FileNotFoundError("the reference CMA-ES library is not available")
            L = C.CDLL(str(p))
            L.xo_cmaes_new.restype = C.c_void_p
            L.xo_cmaes_new.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_long, C.c_int, C.c_double, C.c_double,
                                       C.c_double]
            for n in ("xo_cmaes_sample", "xo_cmaes_update", "xo_cmaes_mean"):
                getattr(L, n).argtypes = [C.c_void_p, C.c_void_p]
            L.xo_cmaes_stop.argtypes = [C.c_void_p]
            L.xo_cmaes_generation.argtypes = [C.c_void_p]
            L.xo_cmaes_generation.restype = C.c_double
            L.xo_cmaes_free.argtypes = [C.c_void_p]
            RefCMAES._lib = L
        x0 = np.ascontiguousarray(xstart, dtype=np.float64)
        sd = np.ascontiguousarray(stddevs, dtype=np.float64)
        self.n, self.lam = x0.size, int(lam)
        self.h = RefCMAES._lib.xo_cmaes_new(self.n, _p(x0), _p(sd), int(seed), self.lam, tol_fun, tol_x, max_iter)
        self.pop = np.zeros((self.lam, self.n))

    def sample(self):
        RefCMAES._lib.xo_cmaes_sample(self.h, _p(self.pop))
        return self.pop

    def update(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        RefCMAES._lib.xo_cmaes_update(self.h, _p(f))

    def stop(self) -> bool:
        return bool(RefCMAES._lib.xo_cmaes_stop(self.h))

    def mean(self):
        m = np.zeros(self.n)
        RefCMAES._lib.xo_cmaes_mean(self.h, _p(m))
        return m

    def generation(self) -> int:
        return int(RefCMAES._lib.xo_cmaes_generation(self.h))

    def __del__(self):
        if getattr(self, "h", None):
            RefCMAES._lib.xo_cmaes_free(self.h)
            self.h = None


def discrete_gaussian_taps(variance, max_error=0.01, max_width=32):
    out = np.zeros(64)
    L = lib()
    L.xo_discrete_gaussian_taps.argtypes = [C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_int]
    L.xo_discrete_gaussian_taps.restype = C.c_int
    r = L.xo_discrete_gaussian_taps(variance, max_error, max_width, _p(out), 64)
    return out[:r + 1].copy()


def downsample_image(img, factor):
    src = np.ascontiguousarray(img, dtype=np.float32)
    orows, ocols = int(src.shape[0] * factor + 0.5), int(src.shape[1] * factor + 0.5)
    dst = np.zeros((orows, ocols), np.float32)
    L = lib()
    L.xo_downsample_image.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_double, C.c_void_p]
    assert L.xo_downsample_image(_p(src), src.shape[0], src.shape[1], factor, _p(dst)) == 0
    return dst


def log_remap(img, use_max=True, i0=1.0):
    src = np.ascontiguousarray(img, dtype=np.float32)
    dst = np.zeros_like(src)
    L = lib()
    L.xo_log_remap.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int, C.c_float, C.c_void_p]
    assert L.xo_log_remap(_p(src), src.shape[0], src.shape[1], int(use_max), float(i0), _p(dst)) == 0
    return dst
