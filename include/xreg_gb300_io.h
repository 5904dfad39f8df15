/*
 * xreg_gb300_io.h -- C ABI for poses on disk: ITK's text transform files, the
 * format xReg's pose writer produces for ".txt" / ".tfm" paths.
 * Plain C types, xr_status returns, xr_last_error() for messages.
 * Citations are paths inside the xReg project.
 */
#ifndef XREG_GB300_IO_H_
#define XREG_GB300_IO_H_

#include "xreg_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ReadITKAffineTransformFromFile (lib/itk/xregITKIOUtils.h:53-54,
 * xregITKIOUtils.cpp:157-224): the pose in a transform file holding exactly one
 * AffineTransform or MatrixOffsetTransformBase (double or float, 3 -> 3), as a
 * row-major 4x4 [A offset; 0 0 0 1] with offset = T + C - A C (T the translation
 * parameters, C the centre), rounded to float as xReg's CoordScalar.  Errors
 * (XR_ERR_INVALID_ARG unless noted): a missing or unreadable file, no
 * transform ("Transform file is empty!"), several transforms, a composite
 * transform (XR_ERR_UNSUPPORTED), another class (XR_ERR_UNSUPPORTED), a wrong
 * parameter count.  Paths must end in ".txt" or ".tfm"; ".h5", ".hdf5" and
 * ".mat" (ITK's HDF5 and MATLAB formats) return XR_ERR_UNSUPPORTED. */
XR_API xr_status xr_itk_affine_transform_read(const char* path, double* xform /* [16] */);

/* ReadSlicerAffineTransformFromFile (xregITKIOUtils.h:46-50,
 * xregITKIOUtils.cpp:33-36): the inverse of xr_itk_affine_transform_read's
 * pose (3D Slicer saves the inverse). */
XR_API xr_status xr_itk_slicer_affine_transform_read(const char* path, double* xform /* [16] */);

/* WriteITKAffineTransform (xregITKIOUtils.h:56-57, xregITKIOUtils.cpp:226-241):
 * writes the row-major 4x4 pose as an AffineTransform_float_3_3 (matrix =
 * upper 3x3, translation = last column, centre 0), 9 significant digits so the
 * float values read back exactly.  Same path rules as the reader. */
XR_API xr_status xr_itk_affine_transform_write(const char* path, const double* xform /* [16] */);

#ifdef __cplusplus
}
#endif

#endif /* XREG_GB300_IO_H_ */
