"""Shared set-up for the parity tests: workloads in both the product's and the
oracle's descriptions, and the error measures the tolerances are stated in."""
from __future__ import annotations

import numpy as np

from oracle import oracle as O
from xreg_gb300 import synth


def oracle_camera(cam):
    """The oracle's own camera model built by the same steps as the product's
    (naive set-up, downsampling, crop, extrinsics); every field must agree."""
    assert cam.recipe is not None, "a camera built from a raw descriptor has no set-up steps to repeat"
    c = None
    for step in cam.recipe:
        kind, args = step[0], step[1:]
        if kind == "naive":
            c = O.camera_naive(*args)
        elif kind == "downsample":
            c = O.camera_downsample(c, args[0], args[1])
        elif kind == "crop":
            c = O.camera_crop_boundary(c, args[0])
        elif kind == "extrins":
            for i in range(16):
                c.extrins[i] = args[0][i]
        else:
            raise ValueError(kind)
    assert O.camera_fields(c) == cam.as_tuple(), (O.camera_fields(c), cam.as_tuple())
    return c


def oracle_cams(cams):
    return [oracle_camera(c) for c in cams]


def oracle_geom(vol):
    return O.vol_geom_of(vol.voxels, vol.spacing, vol.origin, vol.direction)


def drr_rel_err(gpu: np.ndarray, ref: np.ndarray, floor: float = 0.0):
    """Max relative error |g - o| / |o| over pixels with o != 0; pixels with
    o == 0 must be 0 on the GPU as well (returned as the second value)."""
    g = np.asarray(gpu, dtype=np.float64)
    o = np.asarray(ref, dtype=np.float64)
    nz = np.abs(o) > floor
    rel = np.abs(g - o)[nz] / np.abs(o[nz]) if nz.any() else np.zeros(1)
    zero_mismatch = float(np.abs(g[~nz]).max()) if (~nz).any() else 0.0
    return float(rel.max()), zero_mismatch


def small_volume(seed=0, size=(40, 36, 32), spacing=(1.5, 1.5, 1.5)):
    return synth.phantom_volume(size, spacing, seed)


def small_camera(det=(48, 40), px=4.0):
    from xreg_gb300.api import CameraModel
    return CameraModel.naive(synth.SDD_MM, det[0], det[1], px, px)
