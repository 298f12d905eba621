"""Batched scenes (wpbr_batch_*): uneven scenes and films from one pooled
traversal arena, one CUDA graph per pass. Every scene's film must be
bit-identical to rendering the scene alone through wpbr_ctx with the same
spp, seed and stream id, whatever traversal queue depth the autotuner picks,
and (spot-checked) to the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_SCENES = 5
SPP = 2
SEED = 5
FIRST_STREAM = 10


def _scenes(W):
    # the batched set's scenes 0..4 at reduced size: films 96^2/128^2, <= 20k prims
    return [W.SceneGen(3, seed=3, res=(128, 20000), level=k) for k in range(N_SCENES)]


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _same_nan_aware(a, b):
    # bit-identical, except that NaNs match any NaN: the reference's sphere
    # parameterisation takes acos(z / r) of an unrefined hit point, which is
    # NaN when rounding puts |z| above r (CSSphere.cpp), and the NaN sample
    # reaches the film; device and host NaN payloads differ
    same = _bits(a) == _bits(b)
    both_nan = np.isnan(a) & np.isnan(b)
    return bool(np.all(same | both_nan))


@pytest.fixture(scope="module")
def singles(W, ctx):
    gens = _scenes(W)
    films = []
    for k, g in enumerate(gens):
        cam = g.desc.contents.camera
        ctx.set_quirks(0)
        ctx.upload(g.desc)
        ctx.build()
        ctx.render_setup(SPP, seed=SEED, stream=FIRST_STREAM + k)
        ctx.render()
        films.append(ctx.film(cam.res_x, cam.res_y))
    ctx.check_device_errors()
    return gens, films


def _batch(W, gens):
    b = W.Batch(0)
    for k, g in enumerate(gens):
        assert b.add(g.desc) == k
    b.build()
    b.render_setup(SPP, seed=SEED, first_stream=FIRST_STREAM)
    return b


def _assert_films(b, films):
    for k, (L, w) in enumerate(films):
        Lb, wb = b.film(k)
        assert Lb.shape == L.shape
        assert np.array_equal(_bits(wb), _bits(w)), k
        assert np.array_equal(_bits(Lb), _bits(L)), k


def test_batch_matches_single_scenes_and_oracle(W, O, singles):
    gens, films = singles
    with _batch(W, gens) as b:
        info = b.info()
        assert info["n_scenes"] == N_SCENES and info["spp"] == SPP
        assert info["total_prims"] == sum(g.desc.contents.n_triangles + g.desc.contents.n_spheres for g in gens)
        assert info["total_pixels"] == sum(g.desc.contents.camera.res_x * g.desc.contents.camera.res_y for g in gens)
        # Node2 (64 B) per record (interior nodes + leaf-split records) + 48 B per primitive, 256-byte aligned blocks
        assert 48 * info["total_prims"] <= info["arena_bytes"] <= 240 * info["total_prims"] + 768 * N_SCENES
        b.render()
        b.check_device_errors()
        _assert_films(b, films)
    # the single-scene films are the oracle's (checked on a mesh and a sphere set)
    for k in (0, 1):
        cam = gens[k].desc.contents.camera
        Lo, wo = O.OracleScene(gens[k].desc).render(cam.res_x, cam.res_y, SPP, SEED, FIRST_STREAM + k)
        L, w = films[k]
        assert np.array_equal(_bits(w), _bits(wo))
        assert _same_nan_aware(L, Lo)


def test_batch_at_full_scene_sizes_matches_oracle(W, O):
    # scenes of the batched set at their specified sizes: scene 3 (1,310,720
    # triangles, 1024x1024 film), scene 29 (26,800 spheres, 1024x1024),
    # scene 21 (47,620 spheres, 512x512) and scene 6 (20,480 triangles,
    # 256x256), 2 passes each, every film against the oracle
    picks = (3, 29, 21, 6)
    gens = [W.SceneGen(3, seed=3, res=(1024, 2000000), level=k) for k in picks]
    d3 = gens[0].desc.contents
    assert d3.n_triangles == 1310720 and (d3.camera.res_x, d3.camera.res_y) == (1024, 1024)
    with W.Batch(0) as b:
        for k, g in enumerate(gens):
            assert b.add(g.desc) == k
        b.build()
        b.render_setup(SPP, seed=SEED, first_stream=FIRST_STREAM)
        b.render()
        b.check_device_errors()
        for k, (g, pick) in enumerate(zip(gens, picks)):
            cam = g.desc.contents.camera
            Lb, wb = b.film(k)
            Lo, wo = O.OracleScene(g.desc).render(cam.res_x, cam.res_y, SPP, SEED, FIRST_STREAM + k)
            assert np.array_equal(_bits(wb), _bits(wo)), pick
            assert _same_nan_aware(Lb, Lo), pick
            # per-pixel radiance within 1e-4 mean / 1e-3 max relative (finite pixels)
            rg, ro = Lb / wb[..., None], Lo / wo[..., None]
            fin = np.isfinite(ro) & np.isfinite(rg)
            rel = np.abs(rg[fin] - ro[fin]) / np.maximum(np.abs(ro[fin]), 1e-12)
            assert rel.mean() <= 1e-4 and rel.max() <= 1e-3, pick


@pytest.mark.parametrize("rpb", [0, 4096, 256, 7])
def test_batch_queue_depth_does_not_change_films(W, singles, rpb):
    gens, films = singles
    with _batch(W, gens) as b:
        b.set_rays_per_block(rpb)
        assert b.info()["rays_per_block"] == rpb and b.info()["autotune_source"] == 3
        b.render()
        b.check_device_errors()
        _assert_films(b, films)


def test_batch_autotune_and_cache(W, singles, tmp_path, monkeypatch):
    gens, films = singles
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("WPBR_AUTOTUNE_CACHE", str(cache))
    with _batch(W, gens) as b:
        info = b.autotune(use_cache=False)
        assert info["autotune_source"] == 1
        assert info["rays_per_block"] in (0, 4096, 1024, 256)
        lines = cache.read_text().splitlines()
        assert len(lines) == 1 and lines[0].split()[1] == str(info["rays_per_block"])
        b.render()  # autotuning cleared the films
        _assert_films(b, films)
        chosen = info["rays_per_block"]
    with _batch(W, gens) as b:
        info = b.autotune(use_cache=True)
        assert info["autotune_source"] == 2 and info["rays_per_block"] == chosen
        b.render()
        _assert_films(b, films)


def test_batch_errors(W, singles):
    gens, _ = singles
    b = W.Batch(0)
    with pytest.raises(W.WpbrError):
        b.build()  # no scenes
    b.add(gens[0].desc)
    with pytest.raises(W.WpbrError):
        b.render_pass(0)  # not set up
    b.build()
    with pytest.raises(W.WpbrError):
        b.add(gens[1].desc)  # after build
    with pytest.raises(W.WpbrError):
        b.render_setup(0)
    b.render_setup(1, seed=0)
    with pytest.raises(W.WpbrError):
        b.render_pass(1)  # pass >= spp
    with pytest.raises(W.WpbrError):
        b.set_stream(None)  # the legacy stream cannot be captured
    b.render_pass(0)
    b.synchronize()
    b.close()
