"""Poses in ITK text transform files (xr_itk_affine_transform_read / _write, the
ReadITKAffineTransformFromFile / WriteITKAffineTransform pair of
lib/itk/xregITKIOUtils.cpp): round trips, a hand-written file with a centre
(offset = T + C - A C), the Slicer inverse, and the refusals xReg makes.  Host
code only: runs without a GPU."""
import numpy as np
import pytest

HEADER = "#Insight Transform File V1.0\n#Transform 0\n"


def _pose(seed):
    from xreg_gb300.se3 import exp_se3_batch
    rng = np.random.default_rng(seed)
    x = np.concatenate([rng.normal(0, 0.4, 3), rng.normal(0, 300.0, 3)])
    return exp_se3_batch(x[None])[0]


def test_round_trip_is_the_float_pose(xr, tmp_path):
    for seed, ext in ((1, ".txt"), (2, ".tfm"), (3, ".TXT")):
        pose = _pose(seed)
        path = str(tmp_path / f"pose{seed}{ext}")
        xr.write_itk_affine_transform(path, pose)
        text = open(path).read().splitlines()
        assert text[0] == "#Insight Transform File V1.0"
        assert text[2] == "Transform: AffineTransform_float_3_3"
        assert text[4] == "FixedParameters: 0 0 0"
        got = xr.read_itk_affine_transform(path)
        want = pose.astype(np.float32).astype(np.float64)
        want[3] = [0, 0, 0, 1]
        np.testing.assert_array_equal(got, want)


def test_centre_and_matrix_offset_class(xr, tmp_path):
    A = np.array([[0.9, -0.1, 0.2], [0.15, 1.1, -0.05], [0.0, 0.3, 0.95]])
    T = np.array([10.5, -3.25, 7.0])
    Cc = np.array([1.5, -2.0, 30.0])
    p = tmp_path / "moff.txt"
    p.write_text(HEADER + "Transform: MatrixOffsetTransformBase_double_3_3\n"
                 f"Parameters: {' '.join(repr(float(v)) for v in A.ravel())} {' '.join(repr(float(v)) for v in T)}\n"
                 f"FixedParameters: {' '.join(repr(float(v)) for v in Cc)}\n")
    got = xr.read_itk_affine_transform(str(p))
    np.testing.assert_array_equal(got[:3, :3], A.astype(np.float32).astype(np.float64))
    np.testing.assert_array_equal(got[:3, 3], (T + Cc - A @ Cc).astype(np.float32).astype(np.float64))
    np.testing.assert_array_equal(got[3], [0, 0, 0, 1])
    # no FixedParameters line: centre 0; float class; blank lines and spacing
    q = tmp_path / "aff.tfm"
    q.write_text(HEADER + "\nTransform:   AffineTransform_double_3_3\n"
                 "Parameters: 1 0 0 0 1 0 0 0 1   4 5 6\n")
    np.testing.assert_array_equal(xr.read_itk_affine_transform(str(q))[:3, 3], [4, 5, 6])


def test_slicer_read_is_the_inverse(xr, tmp_path):
    pose = _pose(7)
    path = str(tmp_path / "slicer.txt")
    xr.write_itk_affine_transform(path, pose)
    fwd = xr.read_itk_affine_transform(path)
    inv = xr.read_slicer_affine_transform(path)
    np.testing.assert_allclose(inv @ fwd, np.eye(4), atol=1e-5)


@pytest.mark.parametrize("body,status,msg", [
    ("", "INVALID_ARG", "Transform file is empty!"),
    ("Transform: AffineTransform_double_3_3\nParameters: 1 0 0 0 1 0 0 0 1 0 0 0\n"
     "Transform: AffineTransform_double_3_3\nParameters: 1 0 0 0 1 0 0 0 1 0 0 0\n",
     "INVALID_ARG", "multiple transforms"),
    ("Transform: CompositeTransform_double_3\n", "UNSUPPORTED", "Composite transforms are not supported!"),
    ("Transform: Euler3DTransform_double_3_3\nParameters: 0 0 0 0 0 0\nFixedParameters: 0 0 0 0\n",
     "UNSUPPORTED", "Unsupported ITK transform class!"),
    ("Transform: AffineTransform_double_3_3\nParameters: 1 0 0 0 1 0 0 0 1 0 0\n", "INVALID_ARG", "12 parameters"),
    ("Transform: AffineTransform_double_3_3\nParameters: 1 0 0 0 1 0 0 0 1 0 0 x\n", "INVALID_ARG", "bad number"),
])
def test_refusals(xr, tmp_path, body, status, msg):
    from xreg_gb300 import _lib
    p = tmp_path / "bad.txt"
    p.write_text(HEADER + body)
    with pytest.raises(_lib.XRegError) as e:
        xr.read_itk_affine_transform(str(p))
    assert e.value.status == getattr(_lib, f"XR_ERR_{status}")
    assert msg in str(e.value)


def test_paths(xr, tmp_path):
    from xreg_gb300 import _lib
    for ext in (".h5", ".hdf5", ".mat"):
        with pytest.raises(_lib.XRegError) as e:
            xr.write_itk_affine_transform(str(tmp_path / f"pose{ext}"), np.eye(4))
        assert e.value.status == _lib.XR_ERR_UNSUPPORTED
    with pytest.raises(_lib.XRegError) as e:
        xr.read_itk_affine_transform(str(tmp_path / "missing.txt"))
    assert e.value.status == _lib.XR_ERR_INVALID_ARG
    with pytest.raises(_lib.XRegError):
        xr.write_itk_affine_transform(str(tmp_path / "pose.xyz"), np.eye(4))
    with pytest.raises(_lib.XRegError):
        bad = np.eye(4)
        bad[0, 3] = np.nan
        xr.write_itk_affine_transform(str(tmp_path / "nan.txt"), bad)
