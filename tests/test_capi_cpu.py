"""The C-ABI library loads on a machine without a GPU, exports every entry point
that include/xreg_gb300.h declares, and its host-only helpers (camera model set-up
and argument validation) behave like xReg's.  No compute calls are made here."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        names |= set(re.findall(r"XR_API\s+[\w\s\*]+?\b(xr_\w+)\s*\(", h.read_text()))
    return names


def test_library_exports_every_declared_symbol(xr):
    from xreg_gb300 import _lib
    lib = _lib.load()
    declared = _declared()
    assert len(declared) >= 40
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding types every declared entry point
    assert declared <= set(_lib.EXPORTED), sorted(declared - set(_lib.EXPORTED))
    assert lib.xr_version().decode().startswith("xreg_gb300")


def test_camera_helpers_match_oracle(xr, oracle):
    """The product's camera set-up (naive, downsample, crop) equals the oracle's
    own restatement of xReg's float CameraModel field for field."""
    from xreg_gb300.api import CameraModel
    for args in [(1020.0, 1536, 1536, 0.194, 0.194), (1000.0, 255, 257, 0.3, 0.31), (900.0, 7, 9, 1.1, 0.9),
                 (1020.0, 256, 256, 1.55, 1.55)]:
        for frame in (0, 1, 2):
            mine = CameraModel.naive(*args, coord_frame_type=frame)
            ref = oracle.camera_naive(*args, frame)
            assert mine.as_tuple() == oracle.camera_fields(ref)
            for ds in (0.25, 0.5, 0.125, 0.33):
                for even in (False, True):
                    b = oracle.camera_downsample(ref, ds, even)
                    if b.num_det_rows < 1 or b.num_det_cols < 1:
                        with pytest.raises(Exception):
                            mine.downsample(ds, even)  # no pixels left: refused
                        continue
                    a = mine.downsample(ds, even)
                    assert a.as_tuple() == oracle.camera_fields(b)
                    if a.num_det_rows > 8 and a.num_det_cols > 8:
                        assert a.crop_boundary(3).as_tuple() == oracle.camera_fields(
                            oracle.camera_crop_boundary(b, 3))


def test_camera_fields_are_xreg_floats(xr, oracle):
    """CameraModel's members are floats in xReg: every field holds a float value,
    the intrinsics are divided in float, and a downsampled camera's focal length
    is FocalLenFromIntrins of its float intrinsics."""
    from xreg_gb300.api import CameraModel
    cam = CameraModel.naive(1020.0, 1536, 1536, 0.194, 0.194)
    for v in cam.as_tuple()[0] + (cam.desc.focal_len, cam.desc.det_row_spacing):
        assert float(np.float32(v)) == v
    assert cam.intrins[0, 0] == float(-(np.float32(1020.0) / np.float32(0.194)))
    ds = cam.downsample(0.25)
    k = np.float32(cam.intrins[0, 0]) * np.float32(0.25)
    cs = np.float32(0.194) / np.float32(0.25)
    assert ds.focal_len == float((abs(k * cs) + abs(k * cs)) / np.float32(2.0))
    # the helpers rebuild the oracle's cameras from its own set-up
    from tests.helpers import oracle_camera
    view = CameraModel.naive(1020.0, 64, 64, 0.5, 0.5).downsample(0.5)
    c, s = np.cos(0.3), np.sin(0.3)
    view.set_extrins(np.array([[c, 0, s, 1.5], [0, 1, 0, -2.0], [-s, 0, c, 3.25], [0, 0, 0, 1.0]]))
    assert oracle.camera_fields(oracle_camera(view)) == view.as_tuple()


def test_invalid_arguments_report_errors(xr):
    from xreg_gb300 import _lib
    from xreg_gb300.api import CameraModel
    with pytest.raises(_lib.XRegError) as e:
        CameraModel.naive(0.0, 10, 10, 1.0, 1.0)
    assert e.value.status == _lib.XR_ERR_INVALID_ARG
    assert "focal" in str(e.value)
    lib = _lib.load()
    d = _lib.xr_camera_desc()
    assert lib.xr_camera_setup_naive(1000.0, 0, 10, 1.0, 1.0, 1, C.byref(d)) == _lib.XR_ERR_INVALID_ARG
    assert lib.xr_camera_downsample(None, 0.5, 0, C.byref(d)) == _lib.XR_ERR_INVALID_ARG
    assert lib.xr_rc_set_num_projs(None, 4) == _lib.XR_ERR_INVALID_ARG
    assert lib.xr_sm_compute(None) == _lib.XR_ERR_INVALID_ARG
    assert lib.xr_obj_eval(None, 1, None, None) == _lib.XR_ERR_INVALID_ARG
    assert b"NULL" in lib.xr_last_error()
    # destroying NULL handles is a no-op
    assert lib.xr_rc_destroy(None) == 0 and lib.xr_sm_destroy(None) == 0 and lib.xr_obj_destroy(None) == 0


def test_volume_geometry_helpers():
    from xreg_gb300.api import Volume
    v = Volume(np.zeros((4, 6, 8), np.float32), spacing=(0.5, 1.0, 2.0), origin=(1.0, 2.0, 3.0))
    assert v.size == (8, 6, 4)
    T = v.xform_img_center_to_itk_phys()
    np.testing.assert_allclose(T[:3, 3], [1.0 + 4 * 0.5, 2.0 + 3 * 1.0, 3.0 + 2 * 2.0])
