"""The oracle's texture restatement on the CPU: MIP pyramids built as
SLoadTexture::generateMIPS does (CSTextureProcess.h:352-400), the
anisotropic EWA lookup (STexture2DSamplerAnisotropic, CSTextureProcess.h:
138-239) and the isotropic trilinear one (STexture2DSamplerIsotropic,
CSTextureProcess.h:259-289) on textures whose filtered values are known."""
import numpy as np
import pytest


def _mips_numpy(t):
    """generateMIPS restated in numpy float32: interior texels the 2x2 box
    average, the last column / row the average of the previous level's last
    column / row pair, the corner the previous level's last texel."""
    n = int(np.uint16(np.log2(max(t.shape[0], t.shape[1])) - 1.0))
    n = max(n, 1)
    out = [t]
    for _ in range(1, n):
        p = out[-1]
        h, w = max(1, p.shape[0] // 2), max(1, p.shape[1] // 2)
        c = np.zeros((h, w, 3), np.float32)
        a, b = p[0:2 * (h - 1):2, 0:2 * (w - 1):2], p[0:2 * (h - 1):2, 1:2 * (w - 1):2]
        cc, d = p[1:2 * (h - 1):2, 0:2 * (w - 1):2], p[1:2 * (h - 1):2, 1:2 * (w - 1):2]
        c[:h - 1, :w - 1] = (((a + b) + cc) + d) * np.float32(0.25)
        c[:h - 1, w - 1] = (p[0:2 * (h - 1):2, -1] + p[1:2 * (h - 1):2, -1]) * np.float32(0.5)
        c[h - 1, :w - 1] = (p[-1, 0:2 * (w - 1):2] + p[-1, 1:2 * (w - 1):2]) * np.float32(0.5)
        c[h - 1, w - 1] = p[-1, -1]
        out.append(c)
    return out


@pytest.mark.parametrize("shape", [(60, 100), (256, 256), (16, 32), (4, 4), (7, 13)])
def test_mip_pyramid_matches_generate_mips(O, shape):
    t = np.random.default_rng(shape[0] * 1000 + shape[1]).random(shape + (3,), dtype=np.float32)
    got = O.texture_levels(t)
    want = _mips_numpy(t)
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert g.shape == w.shape
        assert np.array_equal(g.view(np.uint32), w.view(np.uint32))


def test_mip_level_count_rule(O):
    # floor(log2(max side)) - 1 levels, at least one
    for (h, w), n in {(256, 256): 7, (60, 100): 5, (4, 4): 1, (8, 4): 2, (1024, 16): 9}.items():
        assert len(O.texture_levels(np.zeros((h, w, 3), np.float32))) == n


def test_constant_texture_filters_to_itself(O):
    rng = np.random.default_rng(5)
    c = np.empty((64, 48, 3), np.float32)
    c[...] = np.array([0.25, 1.5, 3.0], np.float32)
    for _ in range(200):
        p = rng.uniform(0.05, 0.95, 2)
        d = rng.normal(0, 10 ** rng.uniform(-4, -0.5), 4)
        v = O.texture_eval(c, (p[0], p[1], d[0], d[1], d[2], d[3]))
        np.testing.assert_allclose(v, [0.25, 1.5, 3.0], rtol=1e-5)


def test_zero_footprint_is_bilinear_on_the_finest_level(O):
    rng = np.random.default_rng(7)
    t = rng.random((32, 40, 3), dtype=np.float32)
    H, W = t.shape[:2]
    for _ in range(100):
        st = rng.uniform(0.05, 0.95, 2).astype(np.float32)
        s = st[0] * np.float32(W) - np.float32(0.5)
        u = st[1] * np.float32(H) - np.float32(0.5)
        s0, t0 = int(np.floor(s)), int(np.floor(u))
        ds, dt = s - np.float32(s0), u - np.float32(t0)
        want = (t[t0, s0] * (1 - ds) * (1 - dt) + t[t0 + 1, s0] * (1 - ds) * dt + t[t0, s0 + 1] * ds * (1 - dt)
                + t[t0 + 1, s0 + 1] * ds * dt)
        got = O.texture_eval(t, (st[0], st[1], 0, 0, 0, 0))
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)


def test_wide_footprints_average_out_a_fine_checker(O):
    # one-texel checker of 0 and 1: a footprint of a few texels reads ~0.5, a
    # footprint far below a texel reads the texel (or its bilinear blend)
    y, x = np.mgrid[0:128, 0:128]
    t = np.repeat(((x + y) & 1).astype(np.float32)[..., None], 3, axis=2)
    rng = np.random.default_rng(11)
    for _ in range(50):
        p = rng.uniform(0.2, 0.8, 2)
        wide = O.texture_eval(t, (p[0], p[1], 8.0 / 128, 0.0, 0.0, 8.0 / 128))
        assert abs(wide[0] - 0.5) < 0.05
    centre = (np.float32(10.5) / 128, np.float32(20.5) / 128)
    fine = O.texture_eval(t, (centre[0], centre[1], 1e-4 / 128, 0.0, 0.0, 1e-4 / 128))
    assert abs(fine[0] - t[20, 10, 0]) < 1e-3


def test_anisotropic_footprint_blurs_along_its_major_axis_only(O):
    # stripes along t (value varies with s only); a footprint long in t and
    # narrow in s keeps the stripe value, one long in s averages it away
    x = np.arange(256)
    stripe = ((x // 4) & 1).astype(np.float32)
    t = np.repeat(np.repeat(stripe[None, :, None], 256, axis=0), 3, axis=2)
    s_mid = (np.float32(4 * 10 + 2) + np.float32(0.5)) / 256  # centre of a stripe of value 0
    along = O.texture_eval(t, (s_mid, 0.5, 0.0, 20.0 / 256, 0.5 / 256, 0.0))
    across = O.texture_eval(t, (s_mid, 0.5, 20.0 / 256, 0.0, 0.0, 0.5 / 256))
    assert along[0] < 0.2
    assert abs(across[0] - 0.5) < 0.2


def test_major_axis_is_never_swapped(O):
    # the reference compares dstdx with itself when it picks the major axis,
    # so the level follows |dstdy| even when dstdy is the longer derivative:
    # the same footprint with its derivatives exchanged filters differently
    x = np.arange(256)
    stripe = ((x // 4) & 1).astype(np.float32)
    t = np.repeat(np.repeat(stripe[None, :, None], 256, axis=0), 3, axis=2)
    s_mid = (np.float32(4 * 10 + 2) + np.float32(0.5)) / 256
    dx_long = O.texture_eval(t, (s_mid, 0.5, 0.0, 40.0 / 256, 0.5 / 256, 0.0))
    dy_long = O.texture_eval(t, (s_mid, 0.5, 0.5 / 256, 0.0, 0.0, 40.0 / 256))
    assert dx_long[0] < 0.05
    assert dy_long[0] > 0.45


def test_isotropic_sampler_levels(O):
    rng = np.random.default_rng(13)
    t = rng.random((64, 64, 3), dtype=np.float32)
    lv = O.texture_levels(t)
    p = (0.37, 0.61)
    fine = O.texture_eval(t, (p[0], p[1], 0, 0, 0, 0), isotropic=True)
    assert np.array_equal(fine, O.texture_eval(t, (p[0], p[1], 0, 0, 0, 0)))  # both: bilinear on level 0
    # negative components never widen the footprint: still the finest level
    neg = O.texture_eval(t, (p[0], p[1], -0.3, -0.2, -0.1, -0.4), isotropic=True)
    assert np.array_equal(neg, fine)
    # a footprint at or past the coarsest level reads its texel (0, 0)
    coarse = O.texture_eval(t, (p[0], p[1], 0.5, 0.0, 0.0, 0.0), isotropic=True)
    assert np.array_equal(coarse, lv[-1][0, 0])
    # constant texture: every level blends to the constant
    c = np.full((64, 64, 3), 0.75, np.float32)
    for w in (1e-3, 1e-2, 3e-2, 0.1):
        np.testing.assert_allclose(O.texture_eval(c, (0.5, 0.5, w, 0.0, 0.0, w / 2), isotropic=True), 0.75, rtol=1e-6)


def test_isotropic_sampler_blurs_with_width(O):
    y, x = np.mgrid[0:128, 0:128]
    t = np.repeat(((x + y) & 1).astype(np.float32)[..., None], 3, axis=2)
    vals = [O.texture_eval(t, (0.5 + 0.3 / 128, 0.5 + 0.2 / 128, w, 0.0, 0.0, w), isotropic=True)[0]
            for w in (0.1 / 128, 3.0 / 128, 8.0 / 128)]
    # width 2w: below one texel of level 0 -> level 0; 6/128 -> between levels 0 and 1
    assert abs(vals[0] - 0.5) > abs(vals[1] - 0.5) > abs(vals[2] - 0.5)
    assert abs(vals[2] - 0.5) < 0.05


def test_nan_footprint_gives_nan_without_touching_texels(O):
    t = np.random.default_rng(3).random((32, 32, 3), dtype=np.float32)
    nan = float("nan")
    for fp in [(0.5, 0.5, nan, 0.01, 0.02, 0.0), (nan, 0.5, 0.01, 0.0, 0.0, 0.01), (0.5, 0.5, nan, nan, nan, nan)]:
        v = O.texture_eval(t, fp)
        assert np.all(np.isnan(v)), (fp, v)
