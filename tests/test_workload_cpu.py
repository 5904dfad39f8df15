"""The checker side's workload generators (oracle/workload.py, used by the
reference arm of bench.py so that it loads nothing of the product) equal the
product's own generators bit for bit: phantom voxels, cameras, poses."""
import numpy as np

from oracle import workload as W
from xreg_gb300 import synth


def test_phantom_equal():
    for size, sp, seed in (((40, 36, 32), (1.5, 1.5, 1.5), 0), ((33, 20, 17), (0.8, 0.8, 1.0), 7)):
        np.testing.assert_array_equal(W.phantom(size, sp, seed), synth.phantom_volume(size, sp, seed).voxels)


def test_poses_and_camera_equal(xr, oracle):
    vol = synth.phantom_volume((24, 22, 20), (1.0, 1.0, 1.0), 3)
    np.testing.assert_array_equal(W.gt_pose(vol.size, vol.spacing), synth.gt_pose(vol))
    a = W.sample_poses(vol.size, vol.spacing, synth.gt_pose(vol), 7, 10.0, 20.0, seed=5)
    b = synth.sample_poses(vol, synth.gt_pose(vol), 7, 10.0, 20.0, seed=5)
    np.testing.assert_array_equal(a, b)
    cam = oracle.camera_downsample(oracle.camera_naive(W.SDD_MM, 1536, 1536, 0.194, 0.194, 1), 0.25)
    assert oracle.camera_fields(cam) == synth.camera_for(1536, 0.194, 0.25).as_tuple()
