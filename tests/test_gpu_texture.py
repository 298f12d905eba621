"""Textured metal (WPBR_MAT_METAL and WPBR_MAT_METAL_ISOTROPIC,
CMaterialMetal.cpp:8-58) on the GPU against the oracle: camera-ray
differentials at the hit, uv and sphere mappings, MIP-mapped anisotropic EWA
and isotropic trilinear lookups and the conductor built from them, through
the staged jobs (per-pixel records), the fused graph-captured pass, the
Sampled64 pass and a batch. Films are bit-identical up to NaN payloads (the
reference's sphere parameterisation makes a few NaN samples; device and host
NaN payloads differ)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STAGES = ["CAMERA_RAYS", "COLLIDE_PRIMARY", "EMITTED_LIGHT", "BSDF_SETUP", "SAMPLE_LIGHT", "SHADOW_LIGHT",
          "BSDF_COMPUTE", "INTEGRATE_LIGHT", "SAMPLE_BSDF", "SHADOW_BSDF", "LIGHT_COMPUTE", "INTEGRATE_BSDF"]
RES = (96, 64)


def _same_nan_aware(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    if a.dtype != np.float32:
        return bool(np.array_equal(a, b))
    return bool(np.all((a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))))


def _metal_pixels(g, hit_prim):
    """Which pixels hit a textured-metal primitive, which of them use the
    isotropic sampler, and which pixels hit a sphere."""
    d = g.desc.contents
    ns = d.n_spheres
    mat_of = np.zeros(ns + d.n_triangles, np.int64)
    for i in range(ns):
        mat_of[i] = d.spheres[i].material
    for m in range(d.n_meshes):
        me = d.meshes[m]
        mat_of[ns + me.tri_begin: ns + me.tri_begin + me.tri_count] = me.material
    types = np.array([d.materials[i].type for i in range(d.n_materials)])
    hp = np.asarray(hit_prim).astype(np.int64)
    hit = hp != 0xFFFFFFFF
    t = np.full(hp.shape, -1)
    t[hit] = types[mat_of[hp[hit]]]
    return (t == 3) | (t == 4), t == 4, hit & (hp < ns)


@pytest.fixture(scope="module")
def scene(W):
    return W.SceneGen(5, 0, RES)


def test_scene_has_textured_spheres_and_ground(W, scene):
    d = scene.desc.contents
    assert d.n_textures == 4
    assert [(d.textures[i].width, d.textures[i].height) for i in range(4)] == [(256, 256), (64, 64), (100, 60), (32, 16)]
    assert sum(d.materials[i].type == 3 for i in range(d.n_materials)) == 2
    assert sum(d.materials[i].type == 4 for i in range(d.n_materials)) == 1


def test_staged_jobs_match_oracle(W, O, ctx, scene):
    Wd, Hd = RES
    spp = 4
    ctx.set_quirks(0)
    ctx.upload(scene.desc)
    ctx.build()
    ctx.render_setup(spp, seed=0)
    o = O.OracleScene(scene.desc)
    for p in (0, 3):
        for s in STAGES:
            ctx.job(s, p)
        rg = ctx.record(0, 0, Wd, Hd)
        ro = o.render_pass(p, spp, 0, 0, (0, 0, Wd, Hd))
        for k in ro:
            assert _same_nan_aware(rg[k], ro[k]), (k, p)
        metal, iso, sph = _metal_pixels(scene, ro["hit_prim"])
        # both mappings and both samplers are exercised: textured ground,
        # anisotropic and isotropic textured spheres
        assert metal.sum() > 0.2 * Wd * Hd and (metal & sph & ~iso).sum() > 10 and iso.sum() > 10
    ctx.check_device_errors()


def test_fused_film_matches_oracle(W, O, ctx, scene):
    Wd, Hd = RES
    spp = 4
    ctx.set_quirks(0)
    ctx.upload(scene.desc)
    ctx.build()
    ctx.render_setup(spp, seed=0)
    ctx.render()
    Lg, wg = ctx.film(Wd, Hd)
    Lo, wo = O.OracleScene(scene.desc).render(Wd, Hd, spp)
    assert np.array_equal(wg, wo)
    assert _same_nan_aware(Lg, Lo)
    assert np.isfinite(Lg).mean() > 0.99 and np.nanmax(Lg) > 0
    # the staged jobs through the film job give the same film
    ctx.render_setup(spp, seed=0)
    for p in range(spp):
        for s in STAGES + ["FILM_ACCUMULATE"]:
            ctx.job(s, p)
    Ls, ws = ctx.film(Wd, Hd)
    assert _same_nan_aware(Ls, Lo) and np.array_equal(ws, wo)
    ctx.check_device_errors()


def test_textures_change_the_image(W, O, ctx, scene):
    # the same scene with the ground's roughness texture swapped for the
    # sphere one renders differently where the ground is seen: the lookups
    # are live, not constant
    d = scene.desc.contents
    mats = (type(d.materials[0]) * d.n_materials)()
    C.memmove(mats, d.materials, C.sizeof(mats))
    ground = d.meshes[0].material
    mats[ground].tex[1] = 3
    d2 = type(d).from_buffer_copy(d)
    d2.materials = C.cast(mats, type(d.materials))
    ctx.set_quirks(0)
    ctx.upload(C.pointer(d2))
    ctx.build()
    ctx.render_setup(2, seed=0)
    ctx.render()
    L2, _ = ctx.film(*RES)
    Lo2, _ = O.OracleScene(C.pointer(d2)).render(RES[0], RES[1], 2)
    assert _same_nan_aware(L2, Lo2)
    ctx.upload(scene.desc)
    ctx.build()
    ctx.render_setup(2, seed=0)
    ctx.render()
    L1, _ = ctx.film(*RES)
    diff = np.nan_to_num(np.abs(L1 - L2)).sum(-1) > 0
    assert diff.mean() > 0.1
    ctx.check_device_errors()


@pytest.mark.parametrize("spectrum", [0, 1])
def test_material_sorted_films_match_oracle(W, O, ctx, spectrum):
    # a film of 2^17 pixels: the spawn and finish kernels run over the pixels
    # ordered by primitive kind and material type (textured metal, conductor,
    # dielectric, specular on spheres and the ground, misses), RGB and Sampled64
    g = W.SceneGen(5, 0, (512, 256))
    ctx.set_quirks(0)
    ctx.set_spectrum(spectrum)
    try:
        ctx.upload(g.desc)
        ctx.build()
        ctx.render_setup(2, seed=1, stream=2)
        ctx.render()
        L, w = ctx.film(512, 256)
        o = O.OracleScene(g.desc)
        Lo, wo = o.render_spectral(512, 256, 2, 1, 2) if spectrum else o.render(512, 256, 2, 1, 2)
        assert np.array_equal(w, wo)
        assert _same_nan_aware(L, Lo)
    finally:
        ctx.set_spectrum(0)
    ctx.check_device_errors()


def test_spectral_film_matches_oracle(W, O, ctx, scene):
    Wd, Hd = RES
    ctx.set_quirks(0)
    ctx.set_spectrum(W.SPECTRUM_SAMPLED64)
    try:
        ctx.upload(scene.desc)
        ctx.build()
        ctx.render_setup(2, seed=3, stream=1)
        ctx.render()
        L, w = ctx.film(Wd, Hd)
        Lo, wo = O.OracleScene(scene.desc).render_spectral(Wd, Hd, 2, 3, 1)
        assert np.array_equal(w, wo)
        assert _same_nan_aware(L, Lo)
    finally:
        ctx.set_spectrum(W.SPECTRUM_RGB)
    ctx.check_device_errors()


def test_batch_with_a_textured_scene(W, O, ctx, scene):
    g0 = W.SceneGen(0, 0, (64, 48))
    b = W.Batch(0)
    assert b.add(g0.desc) == 0
    assert b.add(scene.desc) == 1
    b.build()
    b.render_setup(2, seed=7, first_stream=4)
    b.render()
    Lb, wb = b.film(1)
    Lo, wo = O.OracleScene(scene.desc).render(RES[0], RES[1], 2, 7, 5)
    assert np.array_equal(wb, wo) and _same_nan_aware(Lb, Lo)
    L0, _ = b.film(0)
    Lo0, _ = O.OracleScene(g0.desc).render(64, 48, 2, 7, 4)
    assert _same_nan_aware(L0, Lo0)
    b.close()


def test_upload_rejects_bad_textures(W, ctx, scene):
    d = scene.desc.contents
    mats = (type(d.materials[0]) * d.n_materials)()
    C.memmove(mats, d.materials, C.sizeof(mats))
    metal = [i for i in range(d.n_materials) if mats[i].type in (3, 4)][0]
    mats[metal].tex[0] = d.n_textures
    bad = type(d).from_buffer_copy(d)
    bad.materials = C.cast(mats, type(d.materials))
    with pytest.raises(W.WpbrError):
        ctx.upload(C.pointer(bad))
    tiny = type(d).from_buffer_copy(d)
    texs = (type(d.textures[0]) * d.n_textures)()
    C.memmove(texs, d.textures, C.sizeof(texs))
    texs[2].width = 3
    tiny.textures = C.cast(texs, type(d.textures))
    with pytest.raises(W.WpbrError):
        ctx.upload(C.pointer(tiny))
    nul = type(d).from_buffer_copy(d)
    nul.textures = None
    with pytest.raises(W.WpbrError):
        ctx.upload(C.pointer(nul))
    ctx.upload(scene.desc)  # the context stays usable


def test_adjoint_rejects_textured_metal(W, ctx, scene):
    ctx.set_quirks(0)
    ctx.upload(scene.desc)
    ctx.build()
    with pytest.raises(W.WpbrError):
        ctx.adjoint_setup(2)
