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
    from xreg_gb300.api import CameraModel
    from tests.helpers import oracle_cams
    for args in [(1020.0, 1536, 1536, 0.194, 0.194), (1000.0, 255, 257, 0.3, 0.31), (900.0, 7, 9, 1.1, 0.9)]:
        for frame in (0, 1, 2):
            mine = CameraModel.naive(*args, coord_frame_type=frame)
            ref = oracle.camera_naive(*args, frame)
            assert oracle_cams([mine])[0].intrins[:] == ref.intrins[:]
            for ds in (0.25, 0.5, 0.125, 0.33):
                a = mine.downsample(ds)
                b = oracle.camera_downsample(ref, ds)
                assert (a.num_det_rows, a.num_det_cols) == (b.num_det_rows, b.num_det_cols)
                assert a.desc.intrins[:] == b.intrins[:]
                assert a.focal_len == b.focal_len
                assert a.desc.det_row_spacing == b.det_row_spacing


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
