"""Patch metrics with masks, weights and patch subsets against the oracle's
restatement of ImgSimMetric2DPatchCommon / PatchNCCCPU / PatchGradNCCCPU
(double arithmetic): mask-derived weights, masked correlation sums, statistics
over masked-in pixels, a user weight image, fixed- and moving-image patch
variances as weights (with the FLT_MAX value of flat moving images), the
combine rules (weighted, unweighted, mean) and random patch subsets.
Tolerance: absolute difference of each value <= 1e-5."""
import numpy as np
import pytest

from tests.test_gpu_metrics import _drrs

pytestmark = pytest.mark.gpu

TOL = 1e-5
FLT_MAX = np.finfo(np.float32).max


def _eval(xr, cls, rc, fixed, n, radius, stride, mask=None, wgt=None, offset=1, **opts):
    m = cls()
    m.set_fixed_image(fixed)
    if mask is not None:
        m.set_mask(mask)
    if wgt is not None:
        m.set_wgt_img(wgt)
    m.set_patch_radius(radius)
    m.set_patch_stride(stride)
    if opts:
        m.set_patch_options(**opts)
    m.set_num_moving_images(n)
    m.set_mov_imgs_buf_from_ray_caster(rc, offset)
    m.allocate_resources()
    m.compute()
    return m, m.sim_vals()


def _mask(shape, seed, frac=0.35):
    rng = np.random.default_rng(seed)
    mk = (rng.random(shape) > frac).astype(np.uint8)
    mk[: shape[0] // 4, : shape[1] // 3] = 0  # a masked-out block: patches with weight 0
    return mk


CASES = [
    dict(),
    dict(use_mask_for_patch_stats=1),
    dict(use_mask_for_weighting=0),
    dict(normalize_weights_as_prob=0),
    dict(weight_patch_sims_in_combine=0),
    dict(compute_mean_of_patch_sims=1),
    dict(use_fixed_img_patch_variances_as_wgts=1),
    dict(use_mov_img_patch_variances_as_wgts=1),
    dict(use_mov_img_patch_variances_as_wgts=1, normalize_weights_as_prob=0),
    dict(mask_only_for_weights=1),
]

ORACLE_KEYS = {"use_fixed_img_patch_variances_as_wgts": "use_fixed_var_wgts",
               "use_mov_img_patch_variances_as_wgts": "use_mov_var_wgts",
               "use_variances_in_grad_imgs_as_wgts": "use_grad_var_wgts"}


def _okw(opts):
    return {ORACLE_KEYS.get(k, k): v for k, v in opts.items()}


@pytest.mark.parametrize("opts", CASES)
def test_patch_ncc_options(xr, oracle, opts):
    rc, imgs, fixed = _drrs(xr, seed=11)
    mask = _mask(fixed.shape, 5)
    _, got = _eval(xr, xr.ImgSimMetric2DPatchNCCCUDA, rc, fixed, 6, 3, 2, mask=mask, **opts)
    ref = oracle.patch_ncc_ex(fixed, imgs[1:], radius=3, stride=2, mask=mask, **_okw(opts))
    np.testing.assert_allclose(got, ref, atol=TOL, rtol=2e-6)


@pytest.mark.parametrize("opts", CASES + [dict(use_fixed_img_patch_variances_as_wgts=1,
                                               use_variances_in_grad_imgs_as_wgts=1),
                                          dict(use_mov_img_patch_variances_as_wgts=1,
                                               use_variances_in_grad_imgs_as_wgts=1)])
def test_patch_grad_ncc_options(xr, oracle, opts):
    rc, imgs, fixed = _drrs(xr, seed=12)
    mask = _mask(fixed.shape, 6)
    _, got = _eval(xr, xr.ImgSimMetric2DPatchGradNCCCUDA, rc, fixed, 6, 3, 2, mask=mask, **opts)
    ref = oracle.patch_grad_ncc_ex(fixed, imgs[1:], smooth_ksize=5, radius=3, stride=2, mask=mask, **_okw(opts))
    np.testing.assert_allclose(got, ref, atol=TOL, rtol=2e-6)


def test_weight_image_and_no_mask(xr, oracle):
    rc, imgs, fixed = _drrs(xr, seed=13)
    wgt = np.random.default_rng(2).random(fixed.shape).astype(np.float32)
    for cls, fn in ((xr.ImgSimMetric2DPatchNCCCUDA, oracle.patch_ncc_ex),
                    (xr.ImgSimMetric2DPatchGradNCCCUDA, oracle.patch_grad_ncc_ex)):
        _, got = _eval(xr, cls, rc, fixed, 6, 5, 1, wgt=wgt)
        np.testing.assert_allclose(got, fn(fixed, imgs[1:], radius=5, stride=1, wgt_img=wgt), atol=TOL, rtol=0)
        # with a mask too: masked centres get weight 0
        mask = _mask(fixed.shape, 7)
        _, got = _eval(xr, cls, rc, fixed, 6, 5, 1, wgt=wgt, mask=mask)
        np.testing.assert_allclose(got, fn(fixed, imgs[1:], radius=5, stride=1, wgt_img=wgt, mask=mask),
                                   atol=TOL, rtol=0)
    # no mask and no options: the plain metric
    _, got = _eval(xr, xr.ImgSimMetric2DPatchNCCCUDA, rc, fixed, 6, 3, 2)
    np.testing.assert_allclose(got, oracle.patch_ncc(fixed, imgs[1:], radius=3, stride=2), atol=TOL, rtol=0)


def test_flat_moving_images_give_flt_max(xr, oracle):
    """Normalised moving-variance weights of an image whose patches are all flat
    sum to at most 1e-6: the value is FLT_MAX, as in xReg."""
    import torch
    rng = np.random.default_rng(4)
    fixed = rng.random((40, 44)).astype(np.float32)
    movs = np.stack([np.full((40, 44), 2.0, np.float32), rng.random((40, 44)).astype(np.float32)])
    d = torch.from_numpy(movs).cuda()
    for cls, fn in ((xr.ImgSimMetric2DPatchNCCCUDA, oracle.patch_ncc_ex),
                    (xr.ImgSimMetric2DPatchGradNCCCUDA, oracle.patch_grad_ncc_ex)):
        m = cls()
        m.set_fixed_image(fixed)
        m.set_patch_radius(3)
        m.set_patch_stride(2)
        m.set_patch_options(use_mov_img_patch_variances_as_wgts=1)
        m.set_num_moving_images(2)
        m.set_mov_imgs_device_buf(d.data_ptr(), 0)
        m.allocate_resources()
        torch.cuda.synchronize()
        m.compute()
        got = m.sim_vals()
        ref = fn(fixed, movs, radius=3, stride=2, use_mov_var_wgts=1)
        assert got[0] == FLT_MAX and ref[0] > 1e38
        assert abs(got[1] - ref[1]) <= TOL


@pytest.mark.parametrize("grad", [0, 1])
def test_random_patch_subsets(xr, oracle, grad):
    rc, imgs, fixed = _drrs(xr, seed=14)
    mask = _mask(fixed.shape, 8)
    cls = xr.ImgSimMetric2DPatchGradNCCCUDA if grad else xr.ImgSimMetric2DPatchNCCCUDA
    fn = oracle.patch_grad_ncc_ex if grad else oracle.patch_ncc_ex
    m, got = _eval(xr, cls, rc, fixed, 6, 3, 1, mask=mask, choose_rand_patches=1, num_rand_patches=40,
                   rand_seed=123)
    idx = m.patch_indices_used()
    assert idx.size == 40
    ncc = fixed.shape[1] - 6
    centres = np.stack([3 + idx // ncc, 3 + idx % ncc], axis=1).astype(np.float64)
    dist = np.sqrt(((centres[:, None, :] - centres[None, :, :]) ** 2).sum(-1)) + np.eye(40) * 1e9
    assert dist.min() >= np.sqrt(2.0 * 9.0) - 1e-9  # the default minimum separation
    count = np.bincount(idx, minlength=(fixed.shape[0] - 6) * ncc).astype(np.int32)
    ref = fn(fixed, imgs[1:], radius=3, stride=1, mask=mask, patch_count=count)
    np.testing.assert_allclose(got, ref, atol=TOL, rtol=2e-6)
    # each compute draws anew; the same seed repeats the draws
    m.compute()
    idx2 = m.patch_indices_used()
    assert not np.array_equal(idx, idx2)
    m2, _ = _eval(xr, cls, rc, fixed, 6, 3, 1, mask=mask, choose_rand_patches=1, num_rand_patches=40,
                  rand_seed=123)
    np.testing.assert_array_equal(m2.patch_indices_used(), idx)
    # zero-weight (fully masked) patches are never drawn
    w_zero = np.array([mask[int(r) - 3:int(r) + 4, int(c) - 3:int(c) + 4].sum() == 0 for r, c in centres])
    assert not w_zero.any()


def test_objective_with_masked_random_patch_metric(xr, oracle):
    """A masked, randomly sampled patch grad-NCC with moving-variance weights
    inside the population objective (run directly, without the captured graph):
    every evaluation equals the oracle on the objective's own DRRs and the
    patches that evaluation drew."""
    from tests.helpers import small_camera, small_volume
    from xreg_gb300 import synth
    vol = small_volume(15, (48, 44, 40), (1.5, 1.5, 1.5))
    cam = small_camera((64, 72), 2.5)
    rc = xr.RayCasterLineIntCUDA()
    rc.set_volume(vol)
    rc.set_camera_model(cam)
    rc.set_ray_step_size(0.5)
    poses = synth.sample_poses(vol, synth.gt_pose(vol), 5, 8.0, 10.0, seed=2)
    fixed = np.random.default_rng(3).random((64, 72)).astype(np.float32)
    mask = _mask((64, 72), 9)
    m = xr.ImgSimMetric2DPatchGradNCCCUDA()
    m.set_fixed_image(fixed)
    m.set_mask(mask)
    m.set_patch_radius(3)
    m.set_patch_options(choose_rand_patches=1, num_rand_patches=30, rand_seed=7,
                        use_mov_img_patch_variances_as_wgts=1)
    obj = xr.PopulationObjective(rc, [m], 5)
    seen = []
    for _ in range(3):
        vals = obj.eval(poses)
        drr = rc.projs()
        idx = m.patch_indices_used()
        seen.append(idx.copy())
        count = np.bincount(idx, minlength=(64 - 6) * (72 - 6)).astype(np.int32)
        ref = oracle.patch_grad_ncc_ex(fixed, drr, radius=3, stride=1, mask=mask, patch_count=count,
                                       use_mov_var_wgts=1)
        np.testing.assert_allclose(vals, ref, atol=TOL, rtol=2e-6)
    assert not np.array_equal(seen[0], seen[1])


def test_unmasked_tiles_and_random_subsets(xr, oracle):
    """Unmasked patches without variance weights run four vertically adjacent
    patches per thread over 16x64-centre tiles: a detector with several tile
    rows and a ragged last one, random subsets (patch counts) through that
    path, and a radius whose tall tile exceeds the shared-memory budget (one
    patch per thread again)."""
    rc, imgs, fixed = _drrs(xr, det=(150, 70), seed=21, px=0.8)
    for cls, fn in ((xr.ImgSimMetric2DPatchNCCCUDA, oracle.patch_ncc_ex),
                    (xr.ImgSimMetric2DPatchGradNCCCUDA, oracle.patch_grad_ncc_ex)):
        _, got = _eval(xr, cls, rc, fixed, 6, 5, 1)
        np.testing.assert_allclose(got, fn(fixed, imgs[1:], radius=5, stride=1), atol=TOL, rtol=2e-6)
        _, got = _eval(xr, cls, rc, fixed, 6, 4, 3)
        np.testing.assert_allclose(got, fn(fixed, imgs[1:], radius=4, stride=3), atol=TOL, rtol=2e-6)
        m, got = _eval(xr, cls, rc, fixed, 6, 3, 1, choose_rand_patches=1, num_rand_patches=60, rand_seed=5)
        idx = m.patch_indices_used()
        ncc = fixed.shape[1] - 6
        count = np.bincount(idx, minlength=(fixed.shape[0] - 6) * ncc).astype(np.int32)
        np.testing.assert_allclose(got, fn(fixed, imgs[1:], radius=3, stride=1, patch_count=count),
                                   atol=TOL, rtol=2e-6)
    _, got = _eval(xr, xr.ImgSimMetric2DPatchGradNCCCUDA, rc, fixed, 6, 16, 1)  # 136 KB tall tile
    np.testing.assert_allclose(got, oracle.patch_grad_ncc_ex(fixed, imgs[1:], radius=16, stride=1),
                               atol=TOL, rtol=2e-6)


def _np_patch_scores(fixed, mov, radius, stride):
    """Each patch's score 1 - sum(((m - mu_m) / sd_m) (f - mu_f) / (sd_f n)) in
    double (sample standard deviations, clamped at 1e-6), in grid order."""
    d = 2 * radius + 1
    n = d * d
    rows, cols = fixed.shape
    out = []
    for r in range(radius, rows - radius, stride):
        for c in range(radius, cols - radius, stride):
            f = fixed[r - radius:r + radius + 1, c - radius:c + radius + 1].astype(np.float64)
            m = mov[r - radius:r + radius + 1, c - radius:c + radius + 1].astype(np.float64)
            sf = max(np.sqrt(((f - f.mean()) ** 2).sum() / (n - 1)), 1e-6)
            sm = max(np.sqrt(((m - m.mean()) ** 2).sum() / (n - 1)), 1e-6)
            out.append(1.0 - (((m - m.mean()) / sm) * (f - f.mean()) / (sf * n)).sum())
    return np.array(out)


@pytest.mark.parametrize("masked", [0, 1])
def test_per_patch_scores(xr, oracle, masked):
    """save_all_per_patch_scores: every patch's score in xReg's order; for patch
    NCC against a direct double computation, for patch grad-NCC 0.5 (s_x + s_y)
    against the same computation on the oracle's gradient images; the weighted
    mean of the kept scores is the metric's value; random subsets list the drawn
    patches in draw order; flat moving images mark every patch FLT_MAX."""
    rc, imgs, fixed = _drrs(xr, det=(40, 46), seed=31)
    mask = _mask(fixed.shape, 12) if masked else None
    r, st = 3, 2
    m, vals = _eval(xr, xr.ImgSimMetric2DPatchNCCCUDA, rc, fixed, 4, r, st, mask=mask,
                    save_all_per_patch_scores=1)
    ncr, ncc = (fixed.shape[0] - 2 * r + st - 1) // st, (fixed.shape[1] - 2 * r + st - 1) // st
    for k in range(4):
        sc = m.patch_scores(k)
        assert sc.shape == (ncr * ncc,)
        if not masked:
            np.testing.assert_allclose(sc, _np_patch_scores(fixed, imgs[1 + k], r, st), atol=2e-5, rtol=0)
        else:
            # patches wholly inside the masked-out block have weight 0: left out, kept as 0
            out = np.array([mask[rr - r:rr + r + 1, cc - r:cc + r + 1].sum() == 0
                            for rr in range(r, fixed.shape[0] - r, st) for cc in range(r, fixed.shape[1] - r, st)])
            assert out.any() and np.all(sc[out] == 0.0)
    if masked:
        # unweighted mean combine: the value is the mean of the kept scores
        mm, mvals = _eval(xr, xr.ImgSimMetric2DPatchNCCCUDA, rc, fixed, 4, r, st, mask=mask,
                          save_all_per_patch_scores=1, weight_patch_sims_in_combine=0, compute_mean_of_patch_sims=1)
        for k in range(4):
            np.testing.assert_allclose(mm.patch_scores(k).mean(), mvals[k], atol=2e-5, rtol=0)
    mg, gvals = _eval(xr, xr.ImgSimMetric2DPatchGradNCCCUDA, rc, fixed, 4, r, st, save_all_per_patch_scores=1)
    fgx, fgy = oracle.grad_images(fixed)
    for k in range(4):
        mgx, mgy = oracle.grad_images(imgs[1 + k])
        ref = 0.5 * (_np_patch_scores(fgx, mgx, r, st) + _np_patch_scores(fgy, mgy, r, st))
        np.testing.assert_allclose(mg.patch_scores(k), ref, atol=2e-5, rtol=0)
        np.testing.assert_allclose(mg.patch_scores(k).mean(), gvals[k], atol=2e-5, rtol=0)
    # random subsets: the drawn patches in draw order
    mr, _ = _eval(xr, xr.ImgSimMetric2DPatchNCCCUDA, rc, fixed, 4, r, 1, choose_rand_patches=1,
                  num_rand_patches=12, rand_seed=3, save_all_per_patch_scores=1)
    idx = mr.patch_indices_used()
    full = _np_patch_scores(fixed, imgs[1], r, 1)
    sc = mr.patch_scores(0)
    assert sc.shape == (12,)
    np.testing.assert_allclose(sc, full[idx], atol=2e-5, rtol=0)


def test_per_patch_scores_flat_image(xr):
    import torch
    rng = np.random.default_rng(4)
    fixed = rng.random((30, 32)).astype(np.float32)
    movs = np.stack([np.full((30, 32), 2.0, np.float32), rng.random((30, 32)).astype(np.float32)])
    d = torch.from_numpy(movs).cuda()
    m = xr.ImgSimMetric2DPatchNCCCUDA()
    m.set_fixed_image(fixed)
    m.set_patch_radius(3)
    m.set_patch_options(use_mov_img_patch_variances_as_wgts=1, save_all_per_patch_scores=1)
    m.set_num_moving_images(2)
    m.set_mov_imgs_device_buf(d.data_ptr(), 0)
    m.allocate_resources()
    torch.cuda.synchronize()
    m.compute()
    assert np.all(m.patch_scores(0) == FLT_MAX)
    assert np.all(m.patch_scores(1) < 2.0)


@pytest.mark.parametrize("grad", [0, 1])
def test_patches_to_use(xr, oracle, grad):
    """set_patches_to_use: a fixed list (repeats counted) instead of the grid or a
    draw; the value equals the oracle with those counts, the indices and the kept
    scores follow the list; reset returns to the whole grid."""
    rc, imgs, fixed = _drrs(xr, det=(44, 50), seed=33)
    mask = _mask(fixed.shape, 13)
    cls = xr.ImgSimMetric2DPatchGradNCCCUDA if grad else xr.ImgSimMetric2DPatchNCCCUDA
    fn = oracle.patch_grad_ncc_ex if grad else oracle.patch_ncc_ex
    np_all = (44 - 6) * (50 - 6)
    lst = np.array([5, 77, 77, 300, 1203, 999, 5, 640, 641, 1500], dtype=np.int64)
    for mk in (None, mask):
        m = cls()
        m.set_fixed_image(fixed)
        if mk is not None:
            m.set_mask(mk)
        m.set_patch_radius(3)
        m.set_patch_options(save_all_per_patch_scores=1, choose_rand_patches=1, num_rand_patches=20)
        m.set_patches_to_use(lst)  # the list wins over random draws
        m.set_num_moving_images(5)
        m.set_mov_imgs_buf_from_ray_caster(rc, 1)
        m.allocate_resources()
        m.compute()
        count = np.bincount(lst, minlength=np_all).astype(np.int32)
        ref = fn(fixed, imgs[1:6], radius=3, stride=1, mask=mk, patch_count=count)
        np.testing.assert_allclose(m.sim_vals(), ref, atol=TOL, rtol=2e-6)
        np.testing.assert_array_equal(m.patch_indices_used(), lst)
        sc = m.patch_scores(2)
        assert sc.shape == lst.shape and sc[0] == sc[6] and sc[1] == sc[2]
        m.reset_patches_to_use()
        m.set_patch_options(choose_rand_patches=0)
        m.allocate_resources()
        m.compute()
        np.testing.assert_allclose(m.sim_vals(), fn(fixed, imgs[1:6], radius=3, stride=1, mask=mk),
                                   atol=TOL, rtol=2e-6)
        assert m.patch_scores(0).shape == (np_all,)
    with pytest.raises(Exception):
        m.set_patches_to_use([np_all])  # outside the grid: refused at allocate_resources
        m.allocate_resources()


@pytest.mark.parametrize("grad", [0, 1])
def test_every_patch_size_launches_and_matches(xr, oracle, grad):
    """Every patch radius the API accepts (1-16) at strides 1 and 3, with and
    without a mask: each tile shape and launch path (four patches per thread,
    the compile-time 11 x 11 scorer, one patch per thread, shared memory above
    48 KB) runs and matches the oracle."""
    rc, imgs, fixed = _drrs(xr, det=(90, 76), seed=41, px=1.2)
    mask = _mask(fixed.shape, 15)
    cls = xr.ImgSimMetric2DPatchGradNCCCUDA if grad else xr.ImgSimMetric2DPatchNCCCUDA
    fn = oracle.patch_grad_ncc_ex if grad else oracle.patch_ncc_ex
    for radius in range(1, 17):
        for stride in (1, 3):
            for mk in (None, mask):
                _, got = _eval(xr, cls, rc, fixed, 3, radius, stride, mask=mk)
                ref = fn(fixed, imgs[1:4], radius=radius, stride=stride, mask=mk)
                np.testing.assert_allclose(got, ref, atol=TOL, rtol=2e-6,
                                           err_msg=f"radius {radius} stride {stride} masked {mk is not None}")
