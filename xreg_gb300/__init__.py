"""xreg_gb300 -- GB300-native (sm_103a) line-integral DRR ray caster and 2D
similarity metrics with xReg's RayCaster / ImgSimMetric2D operator surface.

All computation runs in libxreg_gb300.so (hand-written CUDA); this package is the
host-side mirror of the reference interface.  There is no CPU fallback: using a
class without the built library raises ImportError.
"""
from ._lib import XRegError, load, lib_path  # noqa: F401
from . import _lib as capi  # noqa: F401
from .api import (  # noqa: F401
    CameraModel,
    ImgSimMetric2DCUDA,
    ImgSimMetric2DGradNCCCUDA,
    ImgSimMetric2DNCCCUDA,
    ImgSimMetric2DPatchGradNCCCUDA,
    ImgSimMetric2DPatchNCCCUDA,
    JobSet,
    PopulationObjective,
    RayCasterLineIntCUDA,
    Volume,
    crop_image_boundary,
    downsample_image,
    downsample_size,
    hu_to_lin_att_device,
    log_remap,
    measure_l2_read_bandwidth,
    proj_preproc,
    read_itk_affine_transform,
    read_slicer_affine_transform,
    simple_ray_cast,
    write_itk_affine_transform,
)

__version__ = "0.1.0"
