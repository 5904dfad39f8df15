/*
 * xr_oracle.c -- CPU restatement of xReg's CPU line-integral ray caster and its
 * 2D similarity metrics.  TEST INFRASTRUCTURE ONLY: tests/, the smoke check and
 * the CPU-baseline leg of bench.py load this library as the checker; the product
 * (xreg_gb300) never links, loads or calls it.
 *
 * Parity status: the reference cannot be compiled here (ITK, Eigen, OpenCV, TBB
 * are absent) and its repository holds no golden vectors or known-answer tests,
 * so this restatement is "parity unpinned" with respect to the reference binary.
 * It is pinned instead by analytic known-answer tests (uniform-box chords,
 * OpenCV kernel identities, NCC self/negation identities) and by its own FP64
 * twin; see tests/test_oracle_*.py.
 *
 * Followed reference code (paths inside the xReg project):
 *   lib/ray_cast/xregRayCastLineIntCPU.cpp:106-290  per-ray loop (clip, nudge,
 *        floor(len/step)+1 samples, sum*step, replace/accum, sum/max kernels)
 *   lib/ray_cast/xregRayCastBaseCPU.cpp:128-158     pre_compute (bg fill / keep)
 *   lib/spatial/xregSpatialPrimitives.cpp:176-221   RayRectIntersect slab test
 *   lib/itk/xregITKBasicImageUtils.h:56-75,133-165  index bounds, index->phys
 *   lib/transforms/xregPerspectiveXform.cpp:200-254,401-414,654-689 camera model
 *   lib/regi/sim_metrics_2d/xregImgSimMetric2DNCCCPU.cpp:53-63,164-209  NCC
 *   lib/regi/sim_metrics_2d/xregImgSimMetric2DGradImgCPU.cpp:32-102 blur+Sobel
 *   lib/regi/sim_metrics_2d/xregImgSimMetric2DGradNCCCPU.cpp:51-65  grad-NCC
 *   lib/regi/sim_metrics_2d/xregImgSimMetric2DPatchCommon.cpp:256-300 patch grid
 *   lib/regi/sim_metrics_2d/xregImgSimMetric2DPatchNCCCPU.cpp:74-300,332-441,
 *        558-619                                    patch NCC
 *   lib/regi/sim_metrics_2d/xregImgSimMetric2DPatchGradNCCCPU.cpp:34-400
 *   lib/regi/sim_metrics_2d/xregImgSimMetric2DPatchCommon.cpp:306-493 patch
 *        weights (mask / weight image / variances, normalisation), subsets
 *   lib/image/xregHUToLinAtt.cpp:45-69              HU -> linear attenuation
 *   lib/image/xregProjData.cpp:40-53, lib/itk/xregITKResampleUtils.h:51-187
 *                                                    DownsampleImage
 *   lib/image/xregImageIntensLogTrans.cpp:52-146    log remap (ProjPreProc)
 *
 * Third-party arithmetic restated from published descriptions (absent here):
 *   ITK 5.1.1 LinearInterpolateImageFunction: trilinear at a continuous index,
 *     voxel centres at integer indices, a neighbour past the last index is not
 *     used (the in-bounds voxel keeps full weight); computed in double and
 *     rounded to the float pixel type before the float ray sum.
 *   OpenCV 3.4 GaussianBlur(ksize 5x5, sigma 0): separable, the fixed small
 *     kernel [1 4 6 4 1]/16; Sobel(ksize 3): [-1 0 1] x [1 2 1]; both with the
 *     default border BORDER_REFLECT_101 (gfedcb|abcdefgh|gfedcba).
 *   ITK DiscreteGaussianImageFilter / GaussianOperator: Lindeberg's discrete
 *     Gaussian e^-t I_k(t) (I_0, I_1 from their power series; Bessel recurrence
 *     for k >= 2), cut at 1 - max_error or 32 one-sided taps, replicated edges,
 *     double passes, float output.
 *   ITK BSplineDecompositionImageFilter + BSplineInterpolateImageFunction,
 *     order 3 (Unser, "Splines: a perfect fit for signal and image processing",
 *     1999, Box 2): mirror-boundary recursive prefilter, 4 x 4 weights.
 *
 * Geometry precision contract: the FP32 restatement repeats xReg's own float
 * geometry -- camera set-up (MakeNaiveIntrins, DownsampleCameraModel, SE3Inv,
 * Matrix3f::inverse), the index <-> physical inverse, the per-ray
 * phys_to_idx * pose composition, detector point, slab test, nudge, lengths
 * and step count -- in Eigen 3.3's evaluation order (see "xReg's float
 * geometry" below) with no fused multiply-add (compile with -ffp-contract=off).
 * A one-sample difference on a ray moves its pixel by about 1/300, so this is
 * what makes the sample counts xReg's.  The FP64 twin does the same algorithm
 * with every quantity in double and is the error reference.
 */
#include <math.h>
#include <float.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#if defined(__FP_FAST_FMA) && !defined(XO_ALLOW_CONTRACT)
/* nothing: contraction is controlled by -ffp-contract=off */
#endif

#define XO_EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------------- */
/* Shared layouts (mirrored in the product's include/xreg_gb300.h)            */
/* ------------------------------------------------------------------------- */
typedef struct {
  int64_t n[3];           /* size along index x, y, z (x fastest in memory)   */
  double spacing[3];
  double origin[3];
  double direction[9];    /* row-major ITK direction matrix                   */
} xo_vol_geom;

typedef struct {
  double intrins[9];      /* row-major 3x3 K                                  */
  double extrins[16];     /* row-major 4x4 world -> camera                    */
  int64_t num_det_rows;
  int64_t num_det_cols;
  double det_row_spacing;
  double det_col_spacing;
  double focal_len;
  int32_t coord_frame_type; /* 0 focal pt +z, 1 focal pt -z (default), 2 on detector */
  int32_t pad_;
} xo_camera;

/* Per-projection ray set-up in float, as xReg evaluates it for each ray of a
 * projection (the same result for every ray): camera -> index transform M,
 * pinhole in index coordinates, intrins_inv, det_z_val, z_adjust(2),
 * extrins_inv and the pinhole in camera-world coordinates. */
typedef struct {
  float M[12];      /* L row-major, then t */
  float pin_idx[3];
  float Ki[9];
  float dz;
  float zadj;
  float Ei[12];     /* L row-major, then t */
  float pin[3];
  float pad[3];
} xo_proj_geom;

/* ------------------------------------------------------------------------- */
/* Small parallel-for (stands in for TBB parallel_for over a flat range)       */
/* ------------------------------------------------------------------------- */
typedef void (*xo_range_fn)(void* ctx, int64_t begin, int64_t end);

typedef struct {
  xo_range_fn fn;
  void* ctx;
  int64_t n;
  int64_t chunk;
  int64_t next;            /* guarded by mu */
  pthread_mutex_t mu;
} xo_pool_job;

static int g_num_threads = 1;

XO_EXPORT void xo_set_num_threads(int n) { g_num_threads = n < 1 ? 1 : n; }
XO_EXPORT int xo_get_num_threads(void) { return g_num_threads; }

static void* xo_worker(void* arg) {
  xo_pool_job* job = (xo_pool_job*)arg;
  for (;;) {
    int64_t b;
    pthread_mutex_lock(&job->mu);
    b = job->next;
    job->next += job->chunk;
    pthread_mutex_unlock(&job->mu);
    if (b >= job->n) break;
    int64_t e = b + job->chunk;
    if (e > job->n) e = job->n;
    job->fn(job->ctx, b, e);
  }
  return NULL;
}

static void xo_parallel_for(xo_range_fn fn, void* ctx, int64_t n, int64_t chunk) {
  if (n <= 0) return;
  if (g_num_threads <= 1 || n <= chunk) { fn(ctx, 0, n); return; }
  xo_pool_job job;
  job.fn = fn; job.ctx = ctx; job.n = n; job.chunk = chunk; job.next = 0;
  pthread_mutex_init(&job.mu, NULL);
  int nt = g_num_threads;
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nt);
  for (int i = 1; i < nt; ++i) pthread_create(&th[i], NULL, xo_worker, &job);
  xo_worker(&job);
  for (int i = 1; i < nt; ++i) pthread_join(th[i], NULL);
  free(th);
  pthread_mutex_destroy(&job.mu);
}

/* ------------------------------------------------------------------------- */
/* Double helpers with a fixed evaluation order                              */
/* ------------------------------------------------------------------------- */
static void m3_inverse(const double a[9], double out[9]) {
  const double c00 = a[4] * a[8] - a[5] * a[7];
  const double c01 = a[5] * a[6] - a[3] * a[8];
  const double c02 = a[3] * a[7] - a[4] * a[6];
  const double det = (a[0] * c00 + a[1] * c01) + a[2] * c02;
  const double id = 1.0 / det;
  out[0] = c00 * id;
  out[1] = (a[2] * a[7] - a[1] * a[8]) * id;
  out[2] = (a[1] * a[5] - a[2] * a[4]) * id;
  out[3] = c01 * id;
  out[4] = (a[0] * a[8] - a[2] * a[6]) * id;
  out[5] = (a[2] * a[3] - a[0] * a[5]) * id;
  out[6] = c02 * id;
  out[7] = (a[1] * a[6] - a[0] * a[7]) * id;
  out[8] = (a[0] * a[4] - a[1] * a[3]) * id;
}

static void m3_mul(const double a[9], const double b[9], double out[9]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      out[i * 3 + j] = (a[i * 3 + 0] * b[0 * 3 + j] + a[i * 3 + 1] * b[1 * 3 + j]) + a[i * 3 + 2] * b[2 * 3 + j];
}

static void m3_vec(const double a[9], const double v[3], double out[3]) {
  for (int i = 0; i < 3; ++i)
    out[i] = (a[i * 3 + 0] * v[0] + a[i * 3 + 1] * v[1]) + a[i * 3 + 2] * v[2];
}

/* ------------------------------------------------------------------------- */
/* xReg's float geometry in Eigen 3.3's evaluation order                      */
/* ------------------------------------------------------------------------- */
/* xReg keeps poses, cameras and the index <-> physical transform as Eigen float
 * objects and sets up each ray in float (xregRayCastLineIntCPU.cpp:196-259), so
 * the FP32 restatement repeats that arithmetic, in the order Eigen 3.3 (the
 * reference's pinned version, README.md:60-70) evaluates it on x86-64 with its
 * default SSE2 vectorisation and without FMA:
 *   fixed-size 3-element products and norms: a0 + (a1 + a2) (unrolled reduction
 *     split 1 + 2);
 *   Transform * Vector3: 4x4 matrix times [p; 1] summed by columns:
 *     ((a0 + a1) + a2) + t;
 *   products through runtime-sized blocks (block(0,0,3,3) * v and its norm,
 *     SE3Inv): (a0 + a1) + a2;
 *   Matrix3f::inverse: adjugate, determinant from the first column, 1 / det. */
typedef struct { float L[9]; float t[3]; } xo_aff;

static float xf_fix3(float a0, float a1, float a2, float b0, float b1, float b2) {
  return a0 * b0 + (a1 * b1 + a2 * b2);
}
static float xf_loop3(float a0, float a1, float a2, float b0, float b1, float b2) {
  return (a0 * b0 + a1 * b1) + a2 * b2;
}

static void xf_inv3(const float m[9], float out[9]) {
  float cof[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
      cof[i * 3 + j] = m[i1 * 3 + j1] * m[i2 * 3 + j2] - m[i1 * 3 + j2] * m[i2 * 3 + j1];
    }
  const float det = xf_fix3(cof[0], cof[3], cof[6], m[0], m[3], m[6]);
  const float invdet = 1.0f / det;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) out[r * 3 + c] = cof[c * 3 + r] * invdet;
}

/* Transform * Vector3 */
static void xf_apply(const xo_aff* a, const float p[3], float out[3]) {
  float o[3];
  for (int i = 0; i < 3; ++i) o[i] = xf_loop3(a->L[i * 3], a->L[i * 3 + 1], a->L[i * 3 + 2], p[0], p[1], p[2]) + a->t[i];
  memcpy(out, o, sizeof(o));
}

/* Transform * Transform (affine): linear parts, then La tb + ta */
static void xf_compose(const xo_aff* a, const xo_aff* b, xo_aff* out) {
  xo_aff r;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j)
      r.L[i * 3 + j] = xf_fix3(a->L[i * 3], a->L[i * 3 + 1], a->L[i * 3 + 2], b->L[j], b->L[3 + j], b->L[6 + j]);
    r.t[i] = xf_fix3(a->L[i * 3], a->L[i * 3 + 1], a->L[i * 3 + 2], b->t[0], b->t[1], b->t[2]) + a->t[i];
  }
  *out = r;
}

/* Transform::inverse (affine): L^-1, -(L^-1 t) */
static void xf_inverse(const xo_aff* a, xo_aff* out) {
  xo_aff r;
  xf_inv3(a->L, r.L);
  for (int i = 0; i < 3; ++i) r.t[i] = -xf_fix3(r.L[i * 3], r.L[i * 3 + 1], r.L[i * 3 + 2], a->t[0], a->t[1], a->t[2]);
  *out = r;
}

/* SE3Inv (xregRigidUtils.cpp:29-38) */
static void xf_se3_inv(const xo_aff* e, xo_aff* out) {
  xo_aff r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.L[i * 3 + j] = e->L[j * 3 + i];
  for (int i = 0; i < 3; ++i) r.t[i] = -xf_loop3(r.L[i * 3], r.L[i * 3 + 1], r.L[i * 3 + 2], e->t[0], e->t[1], e->t[2]);
  *out = r;
}

/* ITKImagePhysicalPointTransformsAsEigen (xregITKBasicImageUtils.h:133-165),
 * inverted as in RayCasterLineIntCPU::compute (xregRayCastLineIntCPU.cpp:307-309). */
static void xo_phys_to_idx_f32(const xo_vol_geom* vg, xo_aff* out) {
  xo_aff i2p;
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) i2p.L[r * 3 + c] = (float)(vg->direction[r * 3 + c] * vg->spacing[c]);
    i2p.t[r] = (float)vg->origin[r];
  }
  xf_inverse(&i2p, out);
}

/* Per-projection set-up (CameraModel::setup derived members,
 * xregPerspectiveXform.cpp:302-334; xform_cam_to_itk_idx and the pinhole,
 * xregRayCastLineIntCPU.cpp:206-212).  The camera's fields and the pose are the
 * float values xReg holds (double fields rounded to float). */
static void xo_proj_geom_from(const xo_aff* p2i, const xo_camera* cam, const double pose_cam_to_phys[16],
                              xo_proj_geom* out) {
  float K[9];
  for (int k = 0; k < 9; ++k) K[k] = (float)cam->intrins[k];
  float Ki[9];
  xf_inv3(K, Ki);
  xo_aff E, Ei;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) E.L[i * 3 + j] = (float)cam->extrins[i * 4 + j];
    E.t[i] = (float)cam->extrins[i * 4 + 3];
  }
  xf_se3_inv(&E, &Ei);
  const float f = (float)cam->focal_len;
  float pin[3];
  if (cam->coord_frame_type == 2) {
    const float pz[3] = {0.0f, 0.0f, f};
    xf_apply(&Ei, pz, pin);
  } else {
    memcpy(pin, Ei.t, sizeof(pin));
  }
  xo_aff pose, M;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) pose.L[i * 3 + j] = (float)pose_cam_to_phys[i * 4 + j];
    pose.t[i] = (float)pose_cam_to_phys[i * 4 + 3];
  }
  xf_compose(p2i, &pose, &M);
  float pi[3];
  xf_apply(&M, pin, pi);
  memset(out, 0, sizeof(*out));
  memcpy(out->M, M.L, sizeof(M.L));
  memcpy(out->M + 9, M.t, sizeof(M.t));
  memcpy(out->pin_idx, pi, sizeof(pi));
  memcpy(out->Ki, Ki, sizeof(Ki));
  out->dz = (cam->coord_frame_type == 1) ? -f : f;
  out->zadj = (cam->coord_frame_type == 2) ? -f : 0.0f;
  memcpy(out->Ei, Ei.L, sizeof(Ei.L));
  memcpy(out->Ei + 9, Ei.t, sizeof(Ei.t));
  memcpy(out->pin, pin, sizeof(pin));
}

XO_EXPORT void xo_proj_geom_one(const xo_vol_geom* vg, const xo_camera* cam,
                                const double pose_cam_to_phys[16], xo_proj_geom* out) {
  xo_aff p2i;
  xo_phys_to_idx_f32(vg, &p2i);
  xo_proj_geom_from(&p2i, cam, pose_cam_to_phys, out);
}

/* One ray (xregRayCastLineIntCPU.cpp:196-259): returns 1 and the start point,
 * step vector and num_steps quotient when the segment is sampled, 0 otherwise. */
static int xo_ray_setup_f32(const xo_proj_geom* g, float col, float row, const float maxb[3], float step,
                            float start[3], float stepv[3], float* quot) {
  /* ind_pt_to_phys_det_pt (xregPerspectiveXform.cpp:401-414) */
  const float s0 = g->dz * col, s1 = g->dz * row, s2 = g->dz * 1.0f;
  float q[3];
  for (int i = 0; i < 3; ++i) q[i] = xf_fix3(g->Ki[i * 3], g->Ki[i * 3 + 1], g->Ki[i * 3 + 2], s0, s1, s2);
  q[0] = q[0] + 0.0f;
  q[1] = q[1] + 0.0f;
  q[2] = q[2] + g->zadj;
  float det[3];
  for (int i = 0; i < 3; ++i) det[i] = xf_loop3(g->Ei[i * 3], g->Ei[i * 3 + 1], g->Ei[i * 3 + 2], q[0], q[1], q[2]) + g->Ei[9 + i];
  float d[3];
  for (int i = 0; i < 3; ++i)
    d[i] = (xf_loop3(g->M[i * 3], g->M[i * 3 + 1], g->M[i * 3 + 2], det[0], det[1], det[2]) + g->M[9 + i]) - g->pin_idx[i];
  /* RayRectIntersect, limited to the segment (xregSpatialPrimitives.cpp:176-221) */
  float t0 = 0.0f, t1 = 1.0f;
  for (int k = 0; k < 3; ++k) {
    if ((double)fabsf(d[k]) > 1.0e-8) {
      const float inv = 1.0f / d[k];
      float ta = (0.0f - g->pin_idx[k]) * inv;
      float tb = (maxb[k] - g->pin_idx[k]) * inv;
      if (tb < ta) { float tmp = ta; ta = tb; tb = tmp; }
      t0 = (t0 < ta) ? ta : t0;
      t1 = (tb < t1) ? tb : t1;
      if (t0 > t1) return 0;
    } else if (g->pin_idx[k] < 0.0f || g->pin_idx[k] > maxb[k]) {
      return 0;
    }
  }
  if (!((t1 - t0) > 2.0f * 1.0e-3f)) return 0;
  t0 = t0 + 1.0e-3f;
  t1 = t1 - 1.0e-3f;
  for (int i = 0; i < 3; ++i) start[i] = g->pin_idx[i] + t0 * d[i];
  const float dlen = sqrtf(xf_fix3(d[0], d[1], d[2], d[0], d[1], d[2]));
  const float ilen = (t1 - t0) * dlen;
  float u[3];
  for (int i = 0; i < 3; ++i) u[i] = det[i] - g->pin[i];
  const float z = xf_fix3(u[0], u[1], u[2], u[0], u[1], u[2]);
  if (z > 0.0f) {
    const float n = sqrtf(z);
    for (int i = 0; i < 3; ++i) u[i] = u[i] / n;
  }
  for (int i = 0; i < 3; ++i) u[i] = u[i] * step;
  float w[3];
  for (int i = 0; i < 3; ++i) w[i] = xf_loop3(g->M[i * 3], g->M[i * 3 + 1], g->M[i * 3 + 2], u[0], u[1], u[2]);
  const float slen = sqrtf(xf_loop3(w[0], w[1], w[2], w[0], w[1], w[2]));
  *quot = ilen / slen;
  const float sc = slen / dlen;
  for (int i = 0; i < 3; ++i) stepv[i] = d[i] * sc;
  return 1;
}

/* ------------------------------------------------------------------------- */
/* Trilinear interpolation with ITK's boundary rule                           */
/* ------------------------------------------------------------------------- */
static inline double xo_clampd(double x, double hi) {
  return x < 0.0 ? 0.0 : (x > hi ? hi : x);
}

static inline double xo_trilinear(const float* vol, int64_t nx, int64_t ny, int64_t nz,
                                  double x, double y, double z) {
  x = xo_clampd(x, (double)(nx - 1));
  y = xo_clampd(y, (double)(ny - 1));
  z = xo_clampd(z, (double)(nz - 1));
  int64_t ix = (int64_t)floor(x), iy = (int64_t)floor(y), iz = (int64_t)floor(z);
  if (ix > nx - 2) ix = nx - 2;
  if (iy > ny - 2) iy = ny - 2;
  if (iz > nz - 2) iz = nz - 2;
  const double fx = x - (double)ix, fy = y - (double)iy, fz = z - (double)iz;
  const int64_t sy = nx, sz = nx * ny;
  const float* p = vol + iz * sz + iy * sy + ix;
  const double v000 = p[0], v100 = p[1], v010 = p[sy], v110 = p[sy + 1];
  const double v001 = p[sz], v101 = p[sz + 1], v011 = p[sz + sy], v111 = p[sz + sy + 1];
  const double a00 = v000 + (v100 - v000) * fx;
  const double a10 = v010 + (v110 - v010) * fx;
  const double a01 = v001 + (v101 - v001) * fx;
  const double a11 = v011 + (v111 - v011) * fx;
  const double b0 = a00 + (a10 - a00) * fy;
  const double b1 = a01 + (a11 - a01) * fy;
  return b0 + (b1 - b0) * fz;
}

/* ------------------------------------------------------------------------- */
/* Line integrals                                                             */
/* ------------------------------------------------------------------------- */
enum { XO_KERNEL_SUM = 0, XO_KERNEL_MAX = 1 };
enum { XO_STORE_REPLACE = 0, XO_STORE_ACCUM = 1 };

typedef struct {
  const float* vol;
  int64_t n[3];
  const xo_proj_geom* geo;   /* [num_projs] */
  int64_t rows, cols;
  float step;
  int kernel;
  float* out;
  double* out64;             /* FP64 mode output (NULL in FP32 mode) */
  uint64_t* nsamples;        /* optional per-ray sample count */
  const double* geo64;       /* FP64 mode: per projection 21 doubles */
} xo_drr_ctx;

/* FP32 per-ray semantics (the "xReg CPU" target): xReg's float set-up, then
 * the sample loop (xregRayCastLineIntCPU.cpp:253-282). */
static void xo_drr_f32_range(void* vctx, int64_t b, int64_t e) {
  xo_drr_ctx* c = (xo_drr_ctx*)vctx;
  const int64_t npix = c->rows * c->cols;
  const float maxb[3] = {(float)(c->n[0] - 1), (float)(c->n[1] - 1), (float)(c->n[2] - 1)};
  for (int64_t idx = b; idx < e; ++idx) {
    const int64_t p = idx / npix;
    const int64_t off = idx - p * npix;
    const int64_t row = off / c->cols;
    const int64_t col = off - row * c->cols;
    float sum = (c->kernel == XO_KERNEL_MAX) ? -FLT_MAX : 0.0f;
    uint64_t ns = 0;
    float pos[3], stepv[3], quot;
    if (xo_ray_setup_f32(&c->geo[p], (float)col, (float)row, maxb, c->step, pos, stepv, &quot)) {
      const uint64_t nsteps = (uint64_t)quot;
      for (uint64_t s = 0; s <= nsteps; ++s) {
        const float val = (float)xo_trilinear(c->vol, c->n[0], c->n[1], c->n[2], pos[0], pos[1], pos[2]);
        if (c->kernel == XO_KERNEL_MAX) sum = (sum < val) ? val : sum;
        else sum = sum + val;
        pos[0] = pos[0] + stepv[0];
        pos[1] = pos[1] + stepv[1];
        pos[2] = pos[2] + stepv[2];
      }
      sum = sum * c->step;
      ns = nsteps + 1;
    }
    /* aa_sum = 0 + sum * 1 (xregRayCastLineIntCPU.cpp:189,282) */
    const float aa = 0.0f + sum;
    const float prev = c->out[idx];
    c->out[idx] = (c->kernel == XO_KERNEL_MAX) ? ((prev < aa) ? aa : prev) : (prev + aa);
    if (c->nsamples) c->nsamples[idx] = ns;
  }
}

/* FP64 twin: the same algorithm with every quantity in double; geometry from
 * double set-up vectors.  It is the error reference, not the parity target. */
static void xo_drr_f64_range(void* vctx, int64_t b, int64_t e) {
  xo_drr_ctx* c = (xo_drr_ctx*)vctx;
  const int64_t npix = c->rows * c->cols;
  const double maxb[3] = {(double)(c->n[0] - 1), (double)(c->n[1] - 1), (double)(c->n[2] - 1)};
  const double step = (double)c->step;
  for (int64_t idx = b; idx < e; ++idx) {
    const int64_t p = idx / npix;
    const int64_t off = idx - p * npix;
    const int64_t row = off / c->cols;
    const int64_t col = off - row * c->cols;
    const double* g = c->geo64 + p * 21;
    const double* src = g;
    const double* d0 = g + 3; const double* dc = g + 6; const double* dr = g + 9;
    const double* e0 = g + 12; const double* ec = g + 15; const double* er = g + 18;
    double dir[3], v[3];
    for (int k = 0; k < 3; ++k) {
      dir[k] = (d0[k] + (double)col * dc[k]) + (double)row * dr[k];
      v[k] = (e0[k] + (double)col * ec[k]) + (double)row * er[k];
    }
    int hit = 1;
    double t0 = 0.0, t1 = 1.0;
    for (int k = 0; k < 3; ++k) {
      if (fabs(dir[k]) > 1.0e-8) {
        const double inv = 1.0 / dir[k];
        double ta = (0.0 - src[k]) * inv, tb = (maxb[k] - src[k]) * inv;
        if (tb < ta) { double tmp = ta; ta = tb; tb = tmp; }
        t0 = (t0 < ta) ? ta : t0;
        t1 = (tb < t1) ? tb : t1;
        if (t0 > t1) { hit = 0; break; }
      } else if (src[k] < 0.0 || src[k] > maxb[k]) {
        hit = 0; break;
      }
    }
    double sum = (c->kernel == XO_KERNEL_MAX) ? -DBL_MAX : 0.0;
    uint64_t ns = 0;
    if (hit && ((t1 - t0) > 2.0e-3)) {
      t0 += 1.0e-3;
      t1 -= 1.0e-3;
      double pos[3] = {src[0] + t0 * dir[0], src[1] + t0 * dir[1], src[2] + t0 * dir[2]};
      const double lc = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      const uint64_t nsteps = (uint64_t)(((t1 - t0) * lc) / step);
      const double sc = step / lc;
      const double stepv[3] = {dir[0] * sc, dir[1] * sc, dir[2] * sc};
      for (uint64_t s = 0; s <= nsteps; ++s) {
        const double val = xo_trilinear(c->vol, c->n[0], c->n[1], c->n[2], pos[0], pos[1], pos[2]);
        if (c->kernel == XO_KERNEL_MAX) sum = (sum < val) ? val : sum;
        else sum += val;
        pos[0] += stepv[0]; pos[1] += stepv[1]; pos[2] += stepv[2];
      }
      sum *= step;
      ns = nsteps + 1;
    }
    const double prev = c->out64[idx];
    c->out64[idx] = (c->kernel == XO_KERNEL_MAX) ? ((prev < sum) ? sum : prev) : (prev + sum);
    if (c->nsamples) c->nsamples[idx] = ns;
  }
}

/* Double set-up vectors for the FP64 twin (no float rounding). */
static void xo_proj_geom_one_f64(const xo_vol_geom* vg, const xo_camera* cam,
                                 const double pose[16], double out[21]) {
  double A[9], Ai[9], ti[3], Ki[9], ER[9], Et[3], pin[3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) A[i * 3 + j] = vg->direction[i * 3 + j] * vg->spacing[j];
  m3_inverse(A, Ai);
  m3_vec(Ai, vg->origin, ti);
  for (int k = 0; k < 3; ++k) ti[k] = -ti[k];
  m3_inverse(cam->intrins, Ki);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) ER[i * 3 + j] = cam->extrins[j * 4 + i];
  {
    double t[3] = {cam->extrins[3], cam->extrins[7], cam->extrins[11]};
    m3_vec(ER, t, Et);
    for (int k = 0; k < 3; ++k) Et[k] = -Et[k];
  }
  const double f = cam->focal_len;
  if (cam->coord_frame_type == 2) {
    double pz[3] = {0.0, 0.0, f}, tmp[3];
    m3_vec(ER, pz, tmp);
    for (int k = 0; k < 3; ++k) pin[k] = tmp[k] + Et[k];
  } else {
    for (int k = 0; k < 3; ++k) pin[k] = Et[k];
  }
  const double dz = (cam->coord_frame_type == 1) ? -f : f;
  const double zadj = (cam->coord_frame_type == 2) ? -f : 0.0;
  double kc[3] = {Ki[0] * dz, Ki[3] * dz, Ki[6] * dz};
  double kr[3] = {Ki[1] * dz, Ki[4] * dz, Ki[7] * dz};
  double k0[3] = {Ki[2] * dz, Ki[5] * dz, Ki[8] * dz + zadj};
  double dcol[3], drow[3], det0[3], e0[3];
  m3_vec(ER, kc, dcol);
  m3_vec(ER, kr, drow);
  m3_vec(ER, k0, det0);
  for (int k = 0; k < 3; ++k) { det0[k] += Et[k]; e0[k] = det0[k] - pin[k]; }
  double TR[9], Tt[3], MR[9], Mt[3];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) TR[i * 3 + j] = pose[i * 4 + j];
    Tt[i] = pose[i * 4 + 3];
  }
  m3_mul(Ai, TR, MR);
  m3_vec(Ai, Tt, Mt);
  for (int k = 0; k < 3; ++k) Mt[k] += ti[k];
  double src[3];
  m3_vec(MR, pin, src);
  for (int k = 0; k < 3; ++k) src[k] += Mt[k];
  m3_vec(MR, e0, out + 3);
  m3_vec(MR, dcol, out + 6);
  m3_vec(MR, drow, out + 9);
  for (int k = 0; k < 3; ++k) {
    out[k] = src[k];
    out[12 + k] = e0[k];
    out[15 + k] = dcol[k];
    out[18 + k] = drow[k];
  }
}

static int xo_check_cams(const xo_camera* cams, int64_t ncams) {
  for (int64_t i = 1; i < ncams; ++i)
    if (cams[i].num_det_rows != cams[0].num_det_rows || cams[i].num_det_cols != cams[0].num_det_cols) return -1;
  return 0;
}

/* Pre-compute of the projection buffer (xregRayCastBaseCPU.cpp:128-158).
 * bg_projs (optional): one image per camera, used when use_bg_projs. */
static void xo_pre_compute_f32(float* out, int64_t nproj, int64_t npix, int store, float default_bg,
                               const float* bg_projs, const int32_t* cam_idx) {
  if (bg_projs)
    for (int64_t p = 0; p < nproj; ++p)
      memcpy(out + p * npix, bg_projs + (int64_t)cam_idx[p] * npix, sizeof(float) * (size_t)npix);
  if (store == XO_STORE_REPLACE && !bg_projs)
    for (int64_t i = 0; i < nproj * npix; ++i) out[i] = default_bg;
}

/* Line-integral DRRs, FP32 xReg-CPU semantics.
 * poses: [nproj][16] row-major cam -> ITK physical; cam_idx: [nproj].
 * out: [nproj][rows][cols]; nsamples (optional): per-ray sample counts. */
XO_EXPORT int xo_drr_f32(const float* vol, const xo_vol_geom* vg,
                         const xo_camera* cams, int64_t ncams,
                         const double* poses, const int32_t* cam_idx, int64_t nproj,
                         float step, int kernel, int store, float default_bg,
                         const float* bg_projs, float* out, uint64_t* nsamples) {
  if (xo_check_cams(cams, ncams)) return -1;
  xo_proj_geom* geo = (xo_proj_geom*)malloc(sizeof(xo_proj_geom) * (size_t)nproj);
  xo_aff p2i;
  xo_phys_to_idx_f32(vg, &p2i);
  for (int64_t p = 0; p < nproj; ++p) xo_proj_geom_from(&p2i, &cams[cam_idx[p]], poses + 16 * p, &geo[p]);
  const int64_t rows = cams[0].num_det_rows, cols = cams[0].num_det_cols;
  xo_pre_compute_f32(out, nproj, rows * cols, store, default_bg, bg_projs, cam_idx);
  xo_drr_ctx c;
  memset(&c, 0, sizeof(c));
  c.vol = vol; c.n[0] = vg->n[0]; c.n[1] = vg->n[1]; c.n[2] = vg->n[2];
  c.geo = geo; c.rows = rows; c.cols = cols; c.step = step; c.kernel = kernel;
  c.out = out; c.nsamples = nsamples;
  xo_parallel_for(xo_drr_f32_range, &c, nproj * rows * cols, 256);
  free(geo);
  return 0;
}

/* FP64 twin.  out: double[nproj][rows][cols]; replace mode with default_bg. */
XO_EXPORT int xo_drr_f64(const float* vol, const xo_vol_geom* vg,
                         const xo_camera* cams, int64_t ncams,
                         const double* poses, const int32_t* cam_idx, int64_t nproj,
                         float step, int kernel, double default_bg,
                         double* out, uint64_t* nsamples) {
  if (xo_check_cams(cams, ncams)) return -1;
  double* geo = (double*)malloc(sizeof(double) * 21 * (size_t)nproj);
  for (int64_t p = 0; p < nproj; ++p) xo_proj_geom_one_f64(vg, &cams[cam_idx[p]], poses + 16 * p, geo + 21 * p);
  const int64_t rows = cams[0].num_det_rows, cols = cams[0].num_det_cols;
  for (int64_t i = 0; i < nproj * rows * cols; ++i) out[i] = default_bg;
  xo_drr_ctx c;
  memset(&c, 0, sizeof(c));
  c.vol = vol; c.n[0] = vg->n[0]; c.n[1] = vg->n[1]; c.n[2] = vg->n[2];
  c.geo64 = geo; c.rows = rows; c.cols = cols; c.step = step; c.kernel = kernel;
  c.out64 = out; c.nsamples = nsamples;
  xo_parallel_for(xo_drr_f64_range, &c, nproj * rows * cols, 256);
  free(geo);
  return 0;
}

/* Exposes the per-projection float set-up (for tests of the geometry contract). */
XO_EXPORT void xo_proj_geoms(const xo_vol_geom* vg, const xo_camera* cams, const double* poses,
                             const int32_t* cam_idx, int64_t nproj, xo_proj_geom* out) {
  for (int64_t p = 0; p < nproj; ++p) xo_proj_geom_one(vg, &cams[cam_idx[p]], poses + 16 * p, &out[p]);
}

/* ------------------------------------------------------------------------- */
/* Camera model helpers                                                       */
/* ------------------------------------------------------------------------- */
/* CameraModel::setup(f, nr, nc, rs, cs) with MakeNaiveIntrins
 * (xregPerspectiveXform.cpp:200-254): CameraModel's members are floats, so the
 * arguments become floats and K is formed in float; frame type 1 (-z) by
 * default.  The double fields hold those float values. */
XO_EXPORT void xo_camera_setup_naive(double f, int64_t nr, int64_t nc, double rs, double cs,
                                     int32_t frame_type, xo_camera* cam) {
  memset(cam, 0, sizeof(*cam));
  const float ff = (float)f, fr = (float)rs, fc = (float)cs;
  cam->coord_frame_type = frame_type;
  cam->focal_len = ff;
  cam->num_det_rows = nr; cam->num_det_cols = nc;
  cam->det_row_spacing = fr; cam->det_col_spacing = fc;
  float K[9] = {ff / fc, 0, 0, 0, ff / fr, 0, 0, 0, 1};
  if (frame_type == 1) { K[0] *= -1.0f; K[4] *= -1.0f; }
  /* (num_cols - 1) * 0.5 in double, stored into the float matrix */
  K[2] = (float)((double)(nc - 1) * 0.5);
  K[5] = (float)((double)(nr - 1) * 0.5);
  for (int i = 0; i < 9; ++i) cam->intrins[i] = K[i];
  for (int i = 0; i < 16; ++i) cam->extrins[i] = (i % 5 == 0) ? 1.0 : 0.0;
}

/* FocalLenFromIntrins (xregPerspectiveXform.cpp:186-190), float. */
static float xo_focal_from_intrins(const float K[9], float xps, float yps) {
  return (fabsf(K[0] * xps) + fabsf(K[4] * ((yps < 0) ? xps : yps))) / 2.0f;
}

/* DownsampleCameraModel (xregPerspectiveXform.cpp:654-689) in float; the new
 * camera's focal length comes from CameraModel::setup(K, E, ...). */
XO_EXPORT void xo_camera_downsample(const xo_camera* src, double ds, int force_even, xo_camera* dst) {
  const float fds = (float)ds;
  *dst = *src;
  float K[9];
  for (int i = 0; i < 9; ++i) K[i] = (float)src->intrins[i];
  K[0] *= fds; K[4] *= fds; K[2] *= fds; K[5] *= fds;
  long nr = lroundf((float)src->num_det_rows * fds);
  long nc = lroundf((float)src->num_det_cols * fds);
  if (force_even) { if (nr % 2) --nr; if (nc % 2) --nc; }
  for (int i = 0; i < 9; ++i) dst->intrins[i] = K[i];
  for (int i = 0; i < 16; ++i) dst->extrins[i] = (float)src->extrins[i];
  dst->num_det_rows = nr; dst->num_det_cols = nc;
  const float rs = (float)src->det_row_spacing / fds, cs = (float)src->det_col_spacing / fds;
  dst->det_row_spacing = rs;
  dst->det_col_spacing = cs;
  dst->focal_len = xo_focal_from_intrins(K, cs, rs);
}

/* UpdateCameraModelFor2DROI (xregPerspectiveXform.cpp:482-503) for a crop of
 * `width` pixels on every side (CropBoundaryPixels, xregProjData.cpp:543-567). */
XO_EXPORT void xo_camera_crop_boundary(const xo_camera* src, int64_t width, xo_camera* dst) {
  *dst = *src;
  float K[9];
  for (int i = 0; i < 9; ++i) K[i] = (float)src->intrins[i];
  K[2] -= (float)width;
  K[5] -= (float)width;
  for (int i = 0; i < 9; ++i) dst->intrins[i] = K[i];
  for (int i = 0; i < 16; ++i) dst->extrins[i] = (float)src->extrins[i];
  const float rs = (float)src->det_row_spacing, cs = (float)src->det_col_spacing;
  dst->det_row_spacing = rs;
  dst->det_col_spacing = cs;
  dst->focal_len = xo_focal_from_intrins(K, cs, rs);
  dst->num_det_rows = src->num_det_rows - 2 * width;
  dst->num_det_cols = src->num_det_cols - 2 * width;
}

/* FrameTransform * FrameTransform in float (pre_multiply_all_xforms /
 * post_multiply_all_xforms, xregRayCastInterface.cpp:235-261); row-major 4x4
 * doubles holding float values in and out. */
XO_EXPORT void xo_frame_mul_f32(const double* a, const double* b, double* out) {
  xo_aff fa, fb, r;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) { fa.L[i * 3 + j] = (float)a[i * 4 + j]; fb.L[i * 3 + j] = (float)b[i * 4 + j]; }
    fa.t[i] = (float)a[i * 4 + 3];
    fb.t[i] = (float)b[i * 4 + 3];
  }
  xf_compose(&fa, &fb, &r);
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) out[i * 4 + j] = r.L[i * 3 + j];
    out[i * 4 + 3] = r.t[i];
    out[12 + i] = 0.0;
  }
  out[15] = 1.0;
}

/* Per-ray set-up of every pixel (test access to the geometry): hit flag,
 * sample count, start point and step vector, [nproj][rows][cols]. */
XO_EXPORT int xo_ray_setups(const xo_vol_geom* vg, const xo_camera* cams, int64_t ncams, const double* poses,
                            const int32_t* cam_idx, int64_t nproj, float step, int32_t* hit, uint64_t* nsamples,
                            float* start, float* stepv) {
  if (xo_check_cams(cams, ncams)) return -1;
  xo_aff p2i;
  xo_phys_to_idx_f32(vg, &p2i);
  const int64_t rows = cams[0].num_det_rows, cols = cams[0].num_det_cols;
  const float maxb[3] = {(float)(vg->n[0] - 1), (float)(vg->n[1] - 1), (float)(vg->n[2] - 1)};
  for (int64_t p = 0; p < nproj; ++p) {
    xo_proj_geom g;
    xo_proj_geom_from(&p2i, &cams[cam_idx[p]], poses + 16 * p, &g);
    for (int64_t r = 0; r < rows; ++r)
      for (int64_t c = 0; c < cols; ++c) {
        const int64_t i = (p * rows + r) * cols + c;
        float q = 0.0f;
        hit[i] = xo_ray_setup_f32(&g, (float)c, (float)r, maxb, step, start + 3 * i, stepv + 3 * i, &q);
        nsamples[i] = hit[i] ? (uint64_t)q + 1 : 0;
        if (!hit[i]) for (int k = 0; k < 3; ++k) start[3 * i + k] = stepv[3 * i + k] = 0.0f;
      }
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* 2D metrics (double arithmetic; float images in, double values out)         */
/* ------------------------------------------------------------------------- */
static inline int64_t xo_reflect101(int64_t i, int64_t n) {
  if (n == 1) return 0;
  while (i < 0 || i >= n) {
    if (i < 0) i = -i;
    if (i >= n) i = 2 * (n - 1) - i;
  }
  return i;
}

/* cv::GaussianBlur(5x5, sigma 0) then cv::Sobel dx / dy, reflect-101 borders
 * (xregImgSimMetric2DGradImgCPU.cpp:48-65,86-101).  smooth_ksize 0 disables the
 * blur; only 5 (kernel [1 4 6 4 1]/16) and 3 ([1 2 1]/4) are supported. */
XO_EXPORT int xo_grad_images(const float* img, int64_t rows, int64_t cols, int smooth_ksize,
                             double* gx, double* gy) {
  const double k5[5] = {0.0625, 0.25, 0.375, 0.25, 0.0625};
  const double k3[3] = {0.25, 0.5, 0.25};
  const double* k = NULL;
  int kr = 0;
  if (smooth_ksize == 5) { k = k5; kr = 2; }
  else if (smooth_ksize == 3) { k = k3; kr = 1; }
  else if (smooth_ksize != 0) return -1;
  const int64_t n = rows * cols;
  double* src = (double*)malloc(sizeof(double) * (size_t)n);
  for (int64_t i = 0; i < n; ++i) src[i] = img[i];
  if (k) {
    double* tmp = (double*)malloc(sizeof(double) * (size_t)n);
    for (int64_t r = 0; r < rows; ++r)
      for (int64_t c = 0; c < cols; ++c) {
        double s = 0;
        for (int t = -kr; t <= kr; ++t) s += k[t + kr] * src[r * cols + xo_reflect101(c + t, cols)];
        tmp[r * cols + c] = s;
      }
    for (int64_t r = 0; r < rows; ++r)
      for (int64_t c = 0; c < cols; ++c) {
        double s = 0;
        for (int t = -kr; t <= kr; ++t) s += k[t + kr] * tmp[xo_reflect101(r + t, rows) * cols + c];
        src[r * cols + c] = s;
      }
    free(tmp);
  }
  for (int64_t r = 0; r < rows; ++r) {
    const int64_t ru = xo_reflect101(r - 1, rows), rd = xo_reflect101(r + 1, rows);
    for (int64_t c = 0; c < cols; ++c) {
      const int64_t cl = xo_reflect101(c - 1, cols), cr = xo_reflect101(c + 1, cols);
      const double a = src[ru * cols + cl], b = src[ru * cols + c], cc = src[ru * cols + cr];
      const double d = src[r * cols + cl], f = src[r * cols + cr];
      const double g = src[rd * cols + cl], h = src[rd * cols + c], ii = src[rd * cols + cr];
      gx[r * cols + c] = ((cc - a) + 2.0 * (f - d)) + (ii - g);
      gy[r * cols + c] = ((g - a) + 2.0 * (h - b)) + (ii - cc);
    }
  }
  free(src);
  return 0;
}

/* NCC sim value (1 - ncc)/2 of one moving image against one fixed image
 * (xregImgSimMetric2DNCCCPU.cpp:53-63,164-209): sample std dev (n-1) clamped at
 * 1e-6, dot product divided by n.  mask (optional, nonzero = use). */
static double xo_ncc_one_d(const double* f, const double* m, int64_t n, const uint8_t* mask) {
  int64_t len = 0;
  double sf = 0, sm = 0;
  for (int64_t i = 0; i < n; ++i)
    if (!mask || mask[i]) { sf += f[i]; sm += m[i]; ++len; }
  const double mf = sf / (double)len, mm = sm / (double)len;
  double vf = 0, vm = 0, cov = 0;
  for (int64_t i = 0; i < n; ++i)
    if (!mask || mask[i]) {
      const double a = f[i] - mf, b = m[i] - mm;
      vf += a * a; vm += b * b; cov += a * b;
    }
  double sdf = sqrt(vf / (double)(len - 1)); if (sdf < 1.0e-6) sdf = 1.0e-6;
  double sdm = sqrt(vm / (double)(len - 1)); if (sdm < 1.0e-6) sdm = 1.0e-6;
  const double ncc = cov / ((double)len * sdf * sdm);
  return (1.0 - ncc) * 0.5;
}

XO_EXPORT void xo_ncc(const float* fixed, const float* mov, int64_t npix, int64_t nimgs,
                      const uint8_t* mask, double* out) {
  double* f = (double*)malloc(sizeof(double) * (size_t)npix);
  double* m = (double*)malloc(sizeof(double) * (size_t)npix);
  for (int64_t i = 0; i < npix; ++i) f[i] = fixed[i];
  for (int64_t k = 0; k < nimgs; ++k) {
    for (int64_t i = 0; i < npix; ++i) m[i] = mov[k * npix + i];
    out[k] = xo_ncc_one_d(f, m, npix, mask);
  }
  free(f); free(m);
}

/* Grad-NCC: 0.5 * (NCC(gx_f, gx_m) + NCC(gy_f, gy_m)) (xregImgSimMetric2DGradNCCCPU.cpp:51-65). */
XO_EXPORT int xo_grad_ncc(const float* fixed, const float* mov, int64_t rows, int64_t cols, int64_t nimgs,
                          int smooth_ksize, const uint8_t* mask, double* out) {
  const int64_t n = rows * cols;
  double* fgx = (double*)malloc(sizeof(double) * (size_t)n);
  double* fgy = (double*)malloc(sizeof(double) * (size_t)n);
  double* mgx = (double*)malloc(sizeof(double) * (size_t)n);
  double* mgy = (double*)malloc(sizeof(double) * (size_t)n);
  int rc = xo_grad_images(fixed, rows, cols, smooth_ksize, fgx, fgy);
  for (int64_t k = 0; rc == 0 && k < nimgs; ++k) {
    rc = xo_grad_images(mov + k * n, rows, cols, smooth_ksize, mgx, mgy);
    if (rc) break;
    out[k] = 0.5 * (xo_ncc_one_d(fgx, mgx, n, mask) + xo_ncc_one_d(fgy, mgy, n, mask));
  }
  free(fgx); free(fgy); free(mgx); free(mgy);
  return rc;
}

/* Mean and sample std dev of one patch, two passes, std dev clamped at 1e-6
 * (xregImgSimMetric2DPatchNCCCPU.cpp:558-619, no mask). */
static void xo_patch_stats(const double* img, int64_t cols, int64_t r0, int64_t c0, int64_t diam,
                           double* mean, double* sd) {
  const int64_t np = diam * diam;
  double s = 0;
  for (int64_t r = 0; r < diam; ++r)
    for (int64_t c = 0; c < diam; ++c) s += img[(r0 + r) * cols + c0 + c];
  const double mu = s / (double)np;
  double v = 0;
  for (int64_t r = 0; r < diam; ++r)
    for (int64_t c = 0; c < diam; ++c) { const double t = img[(r0 + r) * cols + c0 + c] - mu; v += t * t; }
  v /= (double)(np - 1);
  double d = sqrt(v);
  *mean = mu;
  *sd = d < 1.0e-6 ? 1.0e-6 : d;
}

/* Patch NCC of one moving image: patch centres radius..n-1-radius with stride
 * (xregImgSimMetric2DPatchCommon.cpp:256-300); per patch score 1 - sum(((m-mu_m)/sd_m) * fhat)
 * with fhat = (f - mu_f)/(sd_f * n_patch); unit weights, so the combined value is
 * the mean score (xregImgSimMetric2DPatchNCCCPU.cpp:205-287). */
static double xo_patch_ncc_one(const double* f, const double* m, int64_t rows, int64_t cols,
                               int64_t radius, int64_t stride) {
  const int64_t diam = 2 * radius + 1, np = diam * diam;
  double total = 0;
  int64_t count = 0;
  for (int64_t cr = radius; cr + radius <= rows - 1; cr += stride)
    for (int64_t cc = radius; cc + radius <= cols - 1; cc += stride) {
      double mf, sf, mm, sm;
      xo_patch_stats(f, cols, cr - radius, cc - radius, diam, &mf, &sf);
      xo_patch_stats(m, cols, cr - radius, cc - radius, diam, &mm, &sm);
      double acc = 0;
      for (int64_t r = 0; r < diam; ++r)
        for (int64_t c = 0; c < diam; ++c) {
          const int64_t i = (cr - radius + r) * cols + cc - radius + c;
          const double fh = (f[i] - mf) / (sf * (double)np);
          acc += ((m[i] - mm) / sm) * fh;
        }
      total += 1.0 - acc;
      ++count;
    }
  return total / (double)count;
}

XO_EXPORT void xo_patch_ncc(const float* fixed, const float* mov, int64_t rows, int64_t cols, int64_t nimgs,
                            int64_t radius, int64_t stride, double* out) {
  const int64_t n = rows * cols;
  double* f = (double*)malloc(sizeof(double) * (size_t)n);
  double* m = (double*)malloc(sizeof(double) * (size_t)n);
  for (int64_t i = 0; i < n; ++i) f[i] = fixed[i];
  for (int64_t k = 0; k < nimgs; ++k) {
    for (int64_t i = 0; i < n; ++i) m[i] = mov[k * n + i];
    out[k] = xo_patch_ncc_one(f, m, rows, cols, radius, stride);
  }
  free(f); free(m);
}

typedef struct {
  const double *fgx, *fgy;
  const float* mov;
  int64_t rows, cols, radius, stride;
  int smooth;
  double* out;
} xo_pgncc_ctx;

static void xo_pgncc_range(void* vctx, int64_t b, int64_t e) {
  xo_pgncc_ctx* c = (xo_pgncc_ctx*)vctx;
  const int64_t n = c->rows * c->cols;
  double* mgx = (double*)malloc(sizeof(double) * (size_t)n);
  double* mgy = (double*)malloc(sizeof(double) * (size_t)n);
  for (int64_t k = b; k < e; ++k) {
    xo_grad_images(c->mov + k * n, c->rows, c->cols, c->smooth, mgx, mgy);
    c->out[k] = 0.5 * (xo_patch_ncc_one(c->fgx, mgx, c->rows, c->cols, c->radius, c->stride) +
                       xo_patch_ncc_one(c->fgy, mgy, c->rows, c->cols, c->radius, c->stride));
  }
  free(mgx); free(mgy);
}

/* Patch grad-NCC (xregImgSimMetric2DPatchGradNCCCPU.cpp:104-230): blur + Sobel,
 * patch NCC on gx and on gy with the same patches, 0.5 * (s_x + s_y).
 * Parallel over moving images. */
XO_EXPORT int xo_patch_grad_ncc(const float* fixed, const float* mov, int64_t rows, int64_t cols, int64_t nimgs,
                                int smooth_ksize, int64_t radius, int64_t stride, double* out) {
  const int64_t n = rows * cols;
  double* fgx = (double*)malloc(sizeof(double) * (size_t)n);
  double* fgy = (double*)malloc(sizeof(double) * (size_t)n);
  int rc = xo_grad_images(fixed, rows, cols, smooth_ksize, fgx, fgy);
  if (rc == 0) {
    xo_pgncc_ctx c = {fgx, fgy, mov, rows, cols, radius, stride, smooth_ksize, out};
    xo_parallel_for(xo_pgncc_range, &c, nimgs, 1);
  }
  free(fgx); free(fgy);
  return rc;
}

/* ------------------------------------------------------------------------- */
/* Patch NCC with masks, weights and patch subsets                            */
/* (xregImgSimMetric2DPatchCommon.cpp:256-493, xregImgSimMetric2DPatchNCCCPU.cpp:34-441,558-619,
 *  xregImgSimMetric2DPatchGradNCCCPU.cpp:34-400).  Double arithmetic.          */
/* ------------------------------------------------------------------------- */
typedef struct {
  int use_mask_for_weighting;      /* default 1 */
  int use_mask_for_patch_stats;    /* default 0 */
  int normalize_weights_as_prob;   /* default 1 */
  int weight_patch_sims_in_combine;/* default 1 */
  int compute_mean_of_patch_sims;  /* default 0 */
  int use_fixed_var_wgts;          /* fixed-image patch variances as weights */
  int use_mov_var_wgts;            /* moving-image patch variances as weights */
  int use_grad_var_wgts;           /* patch grad-NCC: variances of the gradient images */
  const float* wgt_img;            /* weight image (rows x cols) or NULL */
  const int32_t* patch_count;      /* times each patch is used (npatch) or NULL = every patch once */
  int mask_only_for_weights;       /* the OpenCL metric: every pixel enters the correlation sums */
} xo_patch_opts;

/* ComputePatchMeanStdDev (xregImgSimMetric2DPatchNCCCPU.cpp:558-619): pixels with
 * (!use_mask_for_stats || !mask || mask) count; the mean is divided and the
 * variance formed only when more than one pixel counts; sd clamped at 1e-6. */
static void xo_patch_stats_m(const double* img, int64_t cols, int64_t r0, int64_t c0, int64_t diam,
                             const uint8_t* mask, int use_mask_for_stats, double* mean, double* sd, int64_t* cnt) {
  int64_t n = 0;
  double mu = 0;
  for (int64_t r = 0; r < diam; ++r)
    for (int64_t c = 0; c < diam; ++c) {
      const int64_t i = (r0 + r) * cols + c0 + c;
      if (!use_mask_for_stats || !mask || mask[i]) { mu += img[i]; ++n; }
    }
  double var = 0;
  if (n > 1) {
    mu /= (double)n;
    for (int64_t r = 0; r < diam; ++r)
      for (int64_t c = 0; c < diam; ++c) {
        const int64_t i = (r0 + r) * cols + c0 + c;
        if (!use_mask_for_stats || !mask || mask[i]) { const double t = img[i] - mu; var += t * t; }
      }
    var /= (double)(n - 1);
  }
  const double d = sqrt(var);
  *mean = mu;
  *sd = d < 1.0e-6 ? 1.0e-6 : d;
  *cnt = n;
}

typedef struct {
  int64_t rows, cols, radius, stride, diam, ncr, ncc, np;
  const uint8_t* mask;
  xo_patch_opts o;
  double* fhat;       /* np * diam * diam scaled fixed patches */
  double* w;          /* np static patch weights */
  int32_t* cnt;       /* np multiplicities */
  int64_t nused;      /* sum of multiplicities */
} xo_pncc;

static int64_t xo_pncc_centre(const xo_pncc* P, int64_t p, int64_t* cr, int64_t* cc) {
  *cr = P->radius + (p / P->ncc) * P->stride;
  *cc = P->radius + (p % P->ncc) * P->stride;
  return *cr * P->cols + *cc;
}

/* compute_weights (xregImgSimMetric2DPatchCommon.cpp:306-410) given a weight image or none. */
static void xo_pncc_weights(xo_pncc* P, const double* wimg) {
  const int use_img = wimg != NULL;
  const int use_mask = P->o.use_mask_for_weighting && P->mask;
  for (int64_t p = 0; p < P->np; ++p) {
    int64_t cr, cc;
    const int64_t ci = xo_pncc_centre(P, p, &cr, &cc);
    double w = 1.0;
    if (use_img) {
      w = wimg[ci];
      if (use_mask && !P->mask[ci]) w = 0.0;
    } else if (use_mask) {
      int64_t k = 0;
      for (int64_t r = 0; r < P->diam; ++r)
        for (int64_t c = 0; c < P->diam; ++c)
          if (P->mask[(cr - P->radius + r) * P->cols + cc - P->radius + c]) ++k;
      w = (double)k / (double)(P->diam * P->diam);
    }
    P->w[p] = w;
  }
  if ((use_img || use_mask) && P->o.normalize_weights_as_prob) {
    double s = 0;
    for (int64_t p = 0; p < P->np; ++p) s += P->w[p];
    for (int64_t p = 0; p < P->np; ++p) P->w[p] /= s;
  }
}

/* Patch grid and fixed side; wimg_override: weight image handed down (patch grad-NCC). */
static void xo_pncc_setup(xo_pncc* P, const double* f, int64_t rows, int64_t cols, int64_t radius, int64_t stride,
                          const uint8_t* mask, const xo_patch_opts* o, const double* wimg_override) {
  P->rows = rows; P->cols = cols; P->radius = radius; P->stride = stride; P->diam = 2 * radius + 1;
  P->ncr = (rows - 1 - 2 * radius) / stride + 1;
  P->ncc = (cols - 1 - 2 * radius) / stride + 1;
  P->np = P->ncr * P->ncc;
  P->mask = mask;
  P->o = *o;
  const int64_t dd = P->diam * P->diam;
  P->fhat = (double*)malloc(sizeof(double) * (size_t)(P->np * dd));
  P->w = (double*)malloc(sizeof(double) * (size_t)P->np);
  P->cnt = (int32_t*)malloc(sizeof(int32_t) * (size_t)P->np);
  double* wimg = NULL;
  if (o->use_fixed_var_wgts && !wimg_override) wimg = (double*)calloc((size_t)(rows * cols), sizeof(double));
  for (int64_t p = 0; p < P->np; ++p) {
    int64_t cr, cc;
    const int64_t ci = xo_pncc_centre(P, p, &cr, &cc);
    double mu, sd;
    int64_t n;
    xo_patch_stats_m(f, cols, cr - radius, cc - radius, P->diam, mask, o->use_mask_for_patch_stats, &mu, &sd, &n);
    for (int64_t r = 0; r < P->diam; ++r)
      for (int64_t c = 0; c < P->diam; ++c)
        P->fhat[p * dd + r * P->diam + c] = (f[(cr - radius + r) * cols + cc - radius + c] - mu) / (sd * (double)n);
    if (wimg) {
      if (mask && !o->use_mask_for_patch_stats)
        xo_patch_stats_m(f, cols, cr - radius, cc - radius, P->diam, mask, 1, &mu, &sd, &n);
      wimg[ci] = sd * sd;
    }
  }
  const double* wsrc = wimg_override ? wimg_override : (wimg ? wimg : NULL);
  if (!wsrc && o->wgt_img) {
    wimg = (double*)malloc(sizeof(double) * (size_t)(rows * cols));
    for (int64_t i = 0; i < rows * cols; ++i) wimg[i] = o->wgt_img[i];
    wsrc = wimg;
  }
  xo_pncc_weights(P, wsrc);
  free(wimg);
  P->nused = 0;
  for (int64_t p = 0; p < P->np; ++p) {
    P->cnt[p] = o->patch_count ? o->patch_count[p] : 1;
    P->nused += P->cnt[p];
  }
}

static void xo_pncc_free(xo_pncc* P) { free(P->fhat); free(P->w); free(P->cnt); }

/* Moving-image patch variances (all pixels, no mask) at unmasked centres, 0
 * elsewhere, for every used patch (with multiplicity); normalised as a
 * probability when asked.  Returns 0 when that normalisation finds a total at
 * or below 1e-6 (the value is then FLT_MAX). */
static int xo_pncc_mov_vars(const xo_pncc* P, const double* m, double* var) {
  double s = 0;
  for (int64_t p = 0; p < P->np; ++p) {
    int64_t cr, cc;
    const int64_t ci = xo_pncc_centre(P, p, &cr, &cc);
    var[p] = 0.0;
    if (!P->cnt[p]) continue;
    if (!P->mask || P->mask[ci]) {
      double mu, sd;
      int64_t n;
      xo_patch_stats_m(m, P->cols, cr - P->radius, cc - P->radius, P->diam, NULL, 0, &mu, &sd, &n);
      var[p] = sd * sd;
    }
    s += P->cnt[p] * var[p];
  }
  if (P->o.normalize_weights_as_prob) {
    if (!(s > 1.0e-6)) return 0;
    for (int64_t p = 0; p < P->np; ++p) var[p] /= s;
  }
  return 1;
}

/* One moving image (ImgSimMetric2DPatchNCCCPU::compute, :74-287); mvar: per patch
 * moving-variance weights (already normalised) or NULL. */
static double xo_pncc_eval(const xo_pncc* P, const double* m, const double* mvar) {
  const int64_t dd = P->diam * P->diam;
  double total = 0;
  for (int64_t p = 0; p < P->np; ++p) {
    if (!P->cnt[p]) continue;
    int64_t cr, cc;
    xo_pncc_centre(P, p, &cr, &cc);
    const double wgt = mvar ? mvar[p] : P->w[p];
    double val = 0.0;
    if (!P->o.weight_patch_sims_in_combine || fabs(wgt) > 1.0e-6) {
      double mu, sd;
      int64_t n;
      xo_patch_stats_m(m, P->cols, cr - P->radius, cc - P->radius, P->diam, P->mask, P->o.use_mask_for_patch_stats,
                       &mu, &sd, &n);
      double acc = 0;
      for (int64_t r = 0; r < P->diam; ++r)
        for (int64_t c = 0; c < P->diam; ++c) {
          const int64_t i = (cr - P->radius + r) * P->cols + cc - P->radius + c;
          if (!P->mask || P->o.mask_only_for_weights || P->mask[i])
            acc += ((m[i] - mu) / sd) * P->fhat[p * dd + r * P->diam + c];
        }
      val = (P->o.weight_patch_sims_in_combine ? wgt : 1.0) * (1.0 - acc);
    }
    total += P->cnt[p] * val;
  }
  if (P->o.compute_mean_of_patch_sims) {
    total /= (double)P->nused;
  } else if (P->o.weight_patch_sims_in_combine) {
    double tw = 0;
    for (int64_t p = 0; p < P->np; ++p) tw += P->cnt[p] * P->w[p];
    total /= tw;
  }
  return total;
}

#define XO_FLT_MAX 3.4028234663852886e38

XO_EXPORT int xo_patch_ncc_ex(const float* fixed, const float* mov, int64_t rows, int64_t cols, int64_t nimgs,
                              int64_t radius, int64_t stride, const uint8_t* mask, const xo_patch_opts* o,
                              double* out) {
  const int64_t n = rows * cols;
  double* f = (double*)malloc(sizeof(double) * (size_t)n);
  double* m = (double*)malloc(sizeof(double) * (size_t)n);
  for (int64_t i = 0; i < n; ++i) f[i] = fixed[i];
  xo_pncc P;
  xo_pncc_setup(&P, f, rows, cols, radius, stride, mask, o, NULL);
  double* var = (double*)malloc(sizeof(double) * (size_t)P.np);
  for (int64_t k = 0; k < nimgs; ++k) {
    for (int64_t i = 0; i < n; ++i) m[i] = mov[k * n + i];
    if (o->use_mov_var_wgts) {
      out[k] = xo_pncc_mov_vars(&P, m, var) ? xo_pncc_eval(&P, m, var) : XO_FLT_MAX;
    } else {
      out[k] = xo_pncc_eval(&P, m, NULL);
    }
  }
  free(var);
  xo_pncc_free(&P);
  free(f); free(m);
  return 0;
}

/* Patch grad-NCC with the same options (xregImgSimMetric2DPatchGradNCCCPU.cpp:34-400):
 * patch NCC on gx and on gy, 0.5 (s_x + s_y).  Without use_grad_var_wgts the
 * variance weights come from the (fixed / moving) images themselves and are
 * shared by both directions; with it each direction uses its gradient image. */
XO_EXPORT int xo_patch_grad_ncc_ex(const float* fixed, const float* mov, int64_t rows, int64_t cols, int64_t nimgs,
                                   int smooth_ksize, int64_t radius, int64_t stride, const uint8_t* mask,
                                   const xo_patch_opts* o, double* out) {
  const int64_t n = rows * cols;
  double* fgx = (double*)malloc(sizeof(double) * (size_t)n);
  double* fgy = (double*)malloc(sizeof(double) * (size_t)n);
  double* mgx = (double*)malloc(sizeof(double) * (size_t)n);
  double* mgy = (double*)malloc(sizeof(double) * (size_t)n);
  double* mimg = (double*)malloc(sizeof(double) * (size_t)n);
  int rc = xo_grad_images(fixed, rows, cols, smooth_ksize, fgx, fgy);
  if (rc) { free(fgx); free(fgy); free(mgx); free(mgy); free(mimg); return rc; }
  xo_patch_opts so = *o;
  double* wimg = NULL;
  if (!o->use_grad_var_wgts) {
    so.use_fixed_var_wgts = 0;
    so.use_mov_var_wgts = 0;
    if (o->use_fixed_var_wgts) {
      /* variances of the fixed image's patches (mask-aware stats when masked) */
      double* f = (double*)malloc(sizeof(double) * (size_t)n);
      for (int64_t i = 0; i < n; ++i) f[i] = fixed[i];
      wimg = (double*)calloc((size_t)n, sizeof(double));
      const int64_t diam = 2 * radius + 1;
      for (int64_t cr = radius; cr + radius <= rows - 1; cr += stride)
        for (int64_t cc = radius; cc + radius <= cols - 1; cc += stride) {
          double mu, sd;
          int64_t k;
          xo_patch_stats_m(f, cols, cr - radius, cc - radius, diam, mask, mask != NULL, &mu, &sd, &k);
          wimg[cr * cols + cc] = sd * sd;
        }
      free(f);
    }
  }
  xo_pncc X, Y;
  xo_pncc_setup(&X, fgx, rows, cols, radius, stride, mask, &so, wimg);
  xo_pncc_setup(&Y, fgy, rows, cols, radius, stride, mask, &so, wimg);
  free(wimg);
  double* vx = (double*)malloc(sizeof(double) * (size_t)X.np);
  double* vy = (double*)malloc(sizeof(double) * (size_t)X.np);
  for (int64_t k = 0; k < nimgs; ++k) {
    xo_grad_images(mov + k * n, rows, cols, smooth_ksize, mgx, mgy);
    if (o->use_mov_var_wgts && !o->use_grad_var_wgts) {
      for (int64_t i = 0; i < n; ++i) mimg[i] = mov[k * n + i];
      xo_pncc Pm = X;  /* same grid, mask, counts and normalisation flag */
      if (!xo_pncc_mov_vars(&Pm, mimg, vx)) { out[k] = XO_FLT_MAX; continue; }
      out[k] = 0.5 * (xo_pncc_eval(&X, mgx, vx) + xo_pncc_eval(&Y, mgy, vx));
    } else if (o->use_mov_var_wgts) {
      const double sx = xo_pncc_mov_vars(&X, mgx, vx) ? xo_pncc_eval(&X, mgx, vx) : XO_FLT_MAX;
      const double sy = xo_pncc_mov_vars(&Y, mgy, vy) ? xo_pncc_eval(&Y, mgy, vy) : XO_FLT_MAX;
      out[k] = 0.5 * (sx + sy);
    } else {
      out[k] = 0.5 * (xo_pncc_eval(&X, mgx, NULL) + xo_pncc_eval(&Y, mgy, NULL));
    }
  }
  free(vx); free(vy);
  xo_pncc_free(&X);
  xo_pncc_free(&Y);
  free(fgx); free(fgy); free(mgx); free(mgy); free(mimg);
  return 0;
}

typedef struct {
  const float* fixed;
  const float* mov;
  int64_t rows, cols;
  int smooth;
  double* out;
} xo_gncc_ctx;

static void xo_gncc_range(void* vctx, int64_t b, int64_t e) {
  xo_gncc_ctx* c = (xo_gncc_ctx*)vctx;
  xo_grad_ncc(c->fixed, c->mov + b * c->rows * c->cols, c->rows, c->cols, e - b, c->smooth, NULL, c->out + b);
}

/* Grad-NCC parallel over moving images (CPU baseline timing path). */
XO_EXPORT void xo_grad_ncc_par(const float* fixed, const float* mov, int64_t rows, int64_t cols, int64_t nimgs,
                               int smooth_ksize, double* out) {
  xo_gncc_ctx c = {fixed, mov, rows, cols, smooth_ksize, out};
  xo_parallel_for(xo_gncc_range, &c, nimgs, 1);
}

/* HU -> linear attenuation (xregHUToLinAtt.cpp:45-69, mu_water 0.02683,
 * mu_air 0.02485e-4, hu_lower -1000), double math, float result. */
XO_EXPORT void xo_hu_to_lin_att(const float* hu, int64_t n, float* out) {
  const double mu_w = 0.02683 * 1.0, mu_a = 0.02485 * 0.0001, hu_lower = -1000.0;
  const double hu_scale = (mu_w - mu_a) * 1.0e-3;
  const double mu_lower = (hu_lower * hu_scale) + mu_w;
  for (int64_t i = 0; i < n; ++i) {
    const double v = ((double)hu[i] * hu_scale) + mu_w - mu_lower;
    out[i] = (float)(v > 0.0 ? v : 0.0);
  }
}

/* ------------------------------------------------------------------------- */
/* Fixed-image downsampling (DownsampleImage, lib/itk/xregITKResampleUtils.h:51-131) */
/* ------------------------------------------------------------------------- */
/* Discrete Gaussian taps as ITK's GaussianOperator builds them: e^{-t} I0(t),
 * e^{-t} I1(t), then the Bessel recurrence c_k = c_{k-2} - 2 (k-1) / t c_{k-1},
 * accumulated until c_0 + 2 sum c_k >= 1 - max_error (or max_width one-sided taps),
 * normalised to sum one.  I0 and I1 are summed from their power series here. */
static double xo_bessel_i_series(int k, double t) {
  double term = 1.0;
  for (int j = 1; j <= k; ++j) term *= (0.5 * t) / j;
  double s = term;
  const double q = 0.25 * t * t;
  for (int m = 1; m < 500; ++m) {
    term *= q / ((double)m * (double)(m + k));
    s += term;
    if (term < 1e-18 * s) break;
  }
  return s;
}

XO_EXPORT int xo_discrete_gaussian_taps(double variance, double max_error, int max_width, double* out, int cap_len) {
  const double et = exp(-variance);
  int n = 0;
  out[n++] = et * xo_bessel_i_series(0, variance);
  double sum = out[0];
  out[n++] = et * xo_bessel_i_series(1, variance);
  sum += 2.0 * out[1];
  for (int i = 2; sum < 1.0 - max_error && n < cap_len; ++i) {
    out[n] = out[i - 2] - 2.0 * (i - 1) * out[i - 1] / variance;
    sum += 2.0 * out[n];
    ++n;
    if (n > max_width) break;
  }
  for (int i = 0; i < n; ++i) out[i] /= sum;
  return n - 1;  /* radius */
}

/* Separable discrete Gaussian, edges replicated, in double: src (float) along x
 * into a, then along y into b. */
static void xo_gauss2d(const float* src, int64_t rows, int64_t cols, const double* taps, int radius, double* a,
                       double* b) {
  for (int64_t r = 0; r < rows; ++r)
    for (int64_t c = 0; c < cols; ++c) {
      double s = taps[0] * src[r * cols + c];
      for (int t = 1; t <= radius; ++t) {
        const int64_t l = c - t < 0 ? 0 : c - t, h = c + t > cols - 1 ? cols - 1 : c + t;
        s += taps[t] * ((double)src[r * cols + l] + (double)src[r * cols + h]);
      }
      a[r * cols + c] = s;
    }
  for (int64_t r = 0; r < rows; ++r)
    for (int64_t c = 0; c < cols; ++c) {
      double s = taps[0] * a[r * cols + c];
      for (int t = 1; t <= radius; ++t) {
        const int64_t l = r - t < 0 ? 0 : r - t, h = r + t > rows - 1 ? rows - 1 : r + t;
        s += taps[t] * (a[l * cols + c] + a[h * cols + c]);
      }
      b[r * cols + c] = s;
    }
}

/* Cubic B-spline prefilter of one line in place (ITK BSplineDecompositionImageFilter
 * with spline order 3, after Unser, "Splines: a perfect fit for signal and image
 * processing", 1999, Box 2): gain (1 - z)(1 - 1/z), causal start with mirror
 * boundaries (summed to the horizon ceil(log 1e-10 / log|z|) when the line is
 * longer, else the closed full sum), causal recursion, anti-causal start
 * z / (z^2 - 1) (z v[N-2] + v[N-1]), anti-causal recursion. */
static void xo_bspline_line(double* v, int64_t len, int64_t stride) {
  if (len < 2) return;
  const double z = sqrt(3.0) - 2.0;
  double c0 = 1.0;
  c0 = c0 * (1.0 - z) * (1.0 - 1.0 / z);
  for (int64_t n = 0; n < len; ++n) v[n * stride] *= c0;
  const int64_t horizon = (int64_t)ceil(log(1.0e-10) / log(fabs(z)));
  double zn = z, sum;
  if (horizon < len) {
    sum = v[0];
    for (int64_t n = 1; n < horizon; ++n) {
      sum += zn * v[n * stride];
      zn *= z;
    }
    v[0] = sum;
  } else {
    const double iz = 1.0 / z;
    double z2n = pow(z, (double)(len - 1));
    sum = v[0] + z2n * v[(len - 1) * stride];
    z2n *= z2n * iz;
    for (int64_t n = 1; n <= len - 2; ++n) {
      sum += (zn + z2n) * v[n * stride];
      zn *= z;
      z2n *= iz;
    }
    v[0] = sum / (1.0 - zn * zn);
  }
  for (int64_t n = 1; n < len; ++n) v[n * stride] += z * v[(n - 1) * stride];
  v[(len - 1) * stride] = (z / (z * z - 1.0)) * (z * v[(len - 2) * stride] + v[(len - 1) * stride]);
  for (int64_t n = len - 2; n >= 0; --n) v[n * stride] = z * (v[(n + 1) * stride] - v[n * stride]);
}

static int64_t xo_mirror(int64_t k, int64_t n) {
  if (n == 1) return 0;
  if (k < 0) k = -k;
  if (k > n - 1) k = (n - 1) - (k - (n - 1));
  return k;
}

/* ITK BSplineInterpolateImageFunction (order 3) at continuous index (x, y):
 * support starts at floor((float)x) - 1, weights of t = x - floor((float)x),
 * indices mirrored, sum over the 4 x 4 points with x fastest. */
static double xo_bspline_eval(const double* coef, int64_t rows, int64_t cols, double x, double y) {
  const double xy[2] = {x, y};
  const int64_t len[2] = {cols, rows};
  double w[2][4];
  int64_t idx[2][4];
  for (int d = 0; d < 2; ++d) {
    const int64_t i1 = (int64_t)floor((float)xy[d]);
    const double t = xy[d] - (double)i1;
    w[d][3] = (1.0 / 6.0) * t * t * t;
    w[d][0] = (1.0 / 6.0) + 0.5 * t * (t - 1.0) - w[d][3];
    w[d][2] = t + w[d][0] - 2.0 * w[d][3];
    w[d][1] = 1.0 - w[d][0] - w[d][2] - w[d][3];
    for (int k = 0; k < 4; ++k) idx[d][k] = xo_mirror(i1 - 1 + k, len[d]);
  }
  double acc = 0.0;
  for (int p = 0; p < 16; ++p) {
    const int a = p % 4, b = p / 4;
    const double wt = w[0][a] * w[1][b];
    acc += wt * coef[idx[1][b] * cols + idx[0][a]];
  }
  return acc;
}

/* DownsampleImage (lib/itk/xregITKResampleUtils.h:51-131, default cubic B-spline
 * interpolator :183-187) as used by DownsampleProjData (lib/image/xregProjData.cpp:40-53).
 * dst: floor(rows*factor+0.5) x floor(cols*factor+0.5) floats. */
XO_EXPORT int xo_downsample_image(const float* src, int64_t rows, int64_t cols, double factor, float* dst) {
  const int64_t orows = (int64_t)((double)rows * factor + 0.5), ocols = (int64_t)((double)cols * factor + 0.5);
  const int64_t n = rows * cols;
  double* a = (double*)malloc(sizeof(double) * (size_t)n);
  double* b = (double*)malloc(sizeof(double) * (size_t)n);
  if (factor < 1.0) {
    double taps[64];
    const double sigma = 0.5 / factor;
    const int radius = xo_discrete_gaussian_taps(sigma * sigma, 0.01, 32, taps, 64);
    xo_gauss2d(src, rows, cols, taps, radius, a, b);
    for (int64_t i = 0; i < n; ++i) b[i] = (double)(float)b[i];  /* the smoothed float image */
  } else {
    for (int64_t i = 0; i < n; ++i) b[i] = (double)src[i];
  }
  for (int64_t r = 0; r < rows; ++r) xo_bspline_line(b + r * cols, cols, 1);
  for (int64_t c = 0; c < cols; ++c) xo_bspline_line(b + c, rows, cols);
  for (int64_t r = 0; r < orows; ++r)
    for (int64_t c = 0; c < ocols; ++c) {
      const double y = (double)r / factor, x = (double)c / factor;
      const int inside = x >= -0.5 && x < cols - 0.5 && y >= -0.5 && y < rows - 0.5;
      dst[r * ocols + c] = inside ? (float)xo_bspline_eval(b, rows, cols, x, y) : 0.0f;
    }
  free(a);
  free(b);
  return 0;
}

/* ImageIntensLogTransFilter::GenerateData with UseMaxIntensityAsI0
 * (lib/image/xregImageIntensLogTrans.cpp:52-146): I0 = max of the image smoothed
 * by a discrete Gaussian of variance 2 (pixel units, max error 0.01, width 32,
 * rounded to float); min_pos = smallest value above 1e-6 (0 if none);
 * out = x > 1e-6 ? -log(x / I0) : -log(min_pos / I0), in float.
 * use_max 0 takes I0 = i0. */
XO_EXPORT int xo_log_remap(const float* src, int64_t rows, int64_t cols, int use_max, float i0, float* dst) {
  const int64_t n = rows * cols;
  const float eps = 1.0e-6f;
  float I0 = i0;
  if (use_max) {
    double* a = (double*)malloc(sizeof(double) * (size_t)n);
    double* b = (double*)malloc(sizeof(double) * (size_t)n);
    double taps[64];
    const int radius = xo_discrete_gaussian_taps(2.0, 0.01, 32, taps, 64);
    xo_gauss2d(src, rows, cols, taps, radius, a, b);
    I0 = (float)b[0];
    for (int64_t i = 1; i < n; ++i)
      if ((float)b[i] > I0) I0 = (float)b[i];
    free(a);
    free(b);
  }
  float min_pos = 0.0f;
  int found = 0;
  for (int64_t i = 0; i < n; ++i)
    if (src[i] > eps) {
      if (!found || min_pos > src[i]) min_pos = src[i];
      found = 1;
    }
  const float out_max = -logf(min_pos / I0);
  for (int64_t i = 0; i < n; ++i) dst[i] = (src[i] > eps) ? -logf(src[i] / I0) : out_max;
  return 0;
}
