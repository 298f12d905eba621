"""Sampled64 mode (wpbr_set_spectrum): the spectral render pass against the
oracle's spectral restatement, bit for bit, on the plain scene and on the
full-frame scene (environment light, specular material) with quirks."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same_nan_aware(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return bool(np.all((a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))))


@pytest.mark.parametrize("config,res,level,quirks", [(0, (64, 48), 0, 0), (2, (48, 32), 4, 2), (2, (48, 32), 4, 32),
                                                     (0, (37, 23), 0, 0), (2, (70, 41), 4, 0),
                                                     # 2^17 pixels and more: spawn and finish in material order
                                                     (2, (512, 256), 5, 0), (0, (400, 330), 0, 64)])
def test_spectral_film_matches_oracle(W, O, ctx, config, res, level, quirks):
    g = W.SceneGen(config, 0, res, level=level)
    ctx.set_quirks(quirks)
    ctx.set_spectrum(W.SPECTRUM_SAMPLED64)
    ctx.upload(g.desc)
    ctx.build()
    ctx.render_setup(2, seed=3, stream=1)
    ctx.render()
    L, w = ctx.film(*res)
    Lo, wo = O.OracleScene(g.desc, quirks).render_spectral(res[0], res[1], 2, 3, 1)
    assert np.array_equal(w, wo)
    assert _same_nan_aware(L, Lo)
    assert np.isfinite(L).mean() > 0.99 and np.nanmax(L) > 0
    with pytest.raises(W.WpbrError):
        ctx.job("CAMERA_RAYS", 0)  # the staged jobs are RGB only
    ctx.check_device_errors()
    ctx.set_spectrum(W.SPECTRUM_RGB)
    ctx.set_quirks(0)


@pytest.mark.parametrize("spp", [3, 4, 6, 8])
def test_spectral_frame_in_pass_groups(W, O, ctx, spp):
    # wpbr_render runs Sampled64 frames in groups of 4 or 2 sequential passes
    # (whichever divides spp, else one at a time), gathering each group's
    # samples into the film at once, in pass order: the film is the oracle's
    g = W.SceneGen(2, 0, (44, 28), level=4)
    ctx.set_quirks(0)
    ctx.set_spectrum(W.SPECTRUM_SAMPLED64)
    try:
        ctx.upload(g.desc)
        ctx.build()
        ctx.render_setup(spp, seed=5, stream=3)
        ctx.render()
        L, w = ctx.film(44, 28)
        Lo, wo = O.OracleScene(g.desc).render_spectral(44, 28, spp, 5, 3)
        assert np.array_equal(w, wo)
        assert _same_nan_aware(L, Lo)
        # a second frame on the same context reuses the group graph
        ctx.render_setup(spp, seed=5, stream=3)
        ctx.render()
        L2, w2 = ctx.film(44, 28)
        assert np.array_equal(w2, wo) and _same_nan_aware(L2, Lo)
    finally:
        ctx.set_spectrum(W.SPECTRUM_RGB)
    ctx.check_device_errors()


def test_back_to_rgb_after_spectral(W, O, ctx):
    g = W.SceneGen(0, 0, (32, 32))
    ctx.set_quirks(0)
    ctx.set_spectrum(W.SPECTRUM_SAMPLED64)
    ctx.upload(g.desc)
    ctx.build()
    ctx.render_setup(1, seed=0)
    ctx.render()
    ctx.set_spectrum(W.SPECTRUM_RGB)
    ctx.render_setup(2, seed=0)
    ctx.render()
    L, w = ctx.film(32, 32)
    Lo, wo = O.OracleScene(g.desc).render(32, 32, 2)
    assert np.array_equal(L.view(np.uint32), Lo.view(np.uint32)) and np.array_equal(w, wo)


def test_spectral_passes_one_at_a_time(W, O, ctx):
    # wpbr_render_pass leaves the film's toRGB to the next film read
    g = W.SceneGen(0, 0, (40, 24))
    ctx.set_quirks(0)
    ctx.set_spectrum(W.SPECTRUM_SAMPLED64)
    try:
        ctx.upload(g.desc)
        ctx.build()
        ctx.render_setup(3, seed=4, stream=2)
        o = O.OracleScene(g.desc)
        for p in range(3):
            ctx.render_pass(p)
        L, w = ctx.film(40, 24)
        Lo, wo = o.render_spectral(40, 24, 3, 4, 2)
        assert np.array_equal(w, wo)
        assert _same_nan_aware(L, Lo)
        # a film read after each pass sees the film so far
        ctx.render_setup(3, seed=4, stream=2)
        ctx.render_pass(0)
        L1, w1 = ctx.film(40, 24)
        ctx.render_pass(1)
        ctx.render_pass(2)
        L3, w3 = ctx.film(40, 24)
        assert _same_nan_aware(L3, Lo) and not np.array_equal(w1, w3)
    finally:
        ctx.set_spectrum(W.SPECTRUM_RGB)
    ctx.check_device_errors()
