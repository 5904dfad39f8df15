"""Error bound of the FP16 cell blend (interp8_h16 in xr_raycast.cu), restated
operation by operation in numpy: x blend in half arithmetic on the stored
(z0, z1) half pairs with weights scaled by 2^15 before rounding to half, y blend
as exact products of halves added in float (fma.rn.f32.f16), z blend in float.
The volume stores its maximum in [0.5, 1).  Against float trilinear on the same
stored values the sample error stays within 1.5e-3 (inside the 2e-3 DRR bound
for half-precision volumes) also where a fraction is as small as a float ulp of
a position; unscaled half weights (subnormal below 6.1e-5) would not."""
import numpy as np

H, F, D = np.float16, np.float32, np.float64


def _half(x):
    return np.asarray(x, D).astype(F).astype(H)


def _hmul(a, b):  # exact product in double, one rounding to half
    return (a.astype(D) * b.astype(D)).astype(H)


def _hfma(a, b, c):  # a * b + c rounded once to half (the double sum is exact for halves)
    return (a.astype(D) * b.astype(D) + c.astype(D)).astype(H)


def _blend_h16(v, fx, fy, fz, ws=2.0 ** 15, ys=2.0 ** 15):
    """v[..., 8] stored halves (v000 v001 v100 v101 v010 v011 v110 v111)."""
    FX, GX = _half(F(fx) * F(ws)), _half(D(ws) - D(F(fx) * F(ws)))
    GY, FY = _half(D(ys) - D(F(fy) * F(ys))), _half(F(fy) * F(ys))
    a0 = [_hfma(v[..., 2 + z], FX, _hmul(v[..., 0 + z], GX)) for z in (0, 1)]  # y = 0
    a1 = [_hfma(v[..., 6 + z], FX, _hmul(v[..., 4 + z], GX)) for z in (0, 1)]  # y = 1
    b = [F(F(a0[z].astype(D) * GY.astype(D)).astype(D) + a1[z].astype(D) * FY.astype(D)) for z in (0, 1)]
    gz = F(1.0) - F(fz)
    return (b[1].astype(D) * D(fz) + F(b[0] * gz).astype(D)).astype(F) / (ws * ys)


def _trilinear(v, fx, fy, fz):
    V = v.astype(D)
    gx, gy, gz = 1 - fx, 1 - fy, 1 - fz
    a00, a01 = V[..., 0] * gx + V[..., 2] * fx, V[..., 1] * gx + V[..., 3] * fx
    a10, a11 = V[..., 4] * gx + V[..., 6] * fx, V[..., 5] * gx + V[..., 7] * fx
    return (a00 * gy + a10 * fy) * gz + (a01 * gy + a11 * fy) * fz


def _cells(seed, n=200000):
    rng = np.random.default_rng(seed)
    mu = rng.uniform(0.0, 0.065, (n, 8))
    mu[rng.random((n, 8)) < 0.5] = 0.0  # air corners
    scale = 2.0 ** np.floor(np.log2(1.0 / mu.max()))  # stored maximum in [0.5, 1)
    v = _half(mu * scale)
    f = rng.random((n, 3)).astype(F).astype(D)
    tiny = rng.random(n) < 0.3
    # fractions down to a float ulp of a position (a ray running along a grid plane)
    f[tiny, 0] = 2.0 ** -rng.integers(7, 24, int(tiny.sum())).astype(D)
    return v, f, tiny


def test_fp16_blend_within_bound():
    v, f, tiny = _cells(3)
    got = _blend_h16(v, f[:, 0], f[:, 1], f[:, 2]).astype(D)
    ref = _trilinear(v, f[:, 0], f[:, 1], f[:, 2])
    nz = ref > 0
    rel = np.abs(got - ref)[nz] / ref[nz]
    assert rel.max() <= 1.5e-3, rel.max()
    assert np.mean(rel) <= 3e-4
    t = tiny & nz
    assert (np.abs(got - ref)[t] / ref[t]).max() <= 1.5e-3
    assert np.all(got[~nz] == 0.0)  # all-zero cells stay exactly zero


def test_unscaled_half_weights_fail_on_small_fractions():
    v, f, tiny = _cells(4)
    got = _blend_h16(v, f[:, 0], f[:, 1], f[:, 2], ws=1.0, ys=1.0).astype(D)
    ref = _trilinear(v, f[:, 0], f[:, 1], f[:, 2])
    t = tiny & (ref > 0)
    assert (np.abs(got - ref)[t] / ref[t]).max() > 1e-2
