"""The C-ABI library loads without a GPU, exports every entry point declared
in include/*.h, keeps the documented struct layouts, and its host-only parts
(scene generator, camera setup) agree with the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"WPBR_API\s+[^;(]*?\b(wpbr_\w+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol(W):
    decl = declared_symbols()
    assert len(decl) >= 30
    L = C.CDLL(W.LIB_PATH)
    missing = [n for n in sorted(decl) if not hasattr(L, n)]
    assert not missing, missing
    assert set(W.EXPORTED) <= decl
    assert W.lib().wpbr_version().decode().startswith("wpbr-gb300")


def test_struct_layouts(W):
    A = W._abi
    assert C.sizeof(A.Material) == 64
    assert C.sizeof(A.Sphere) == 144
    assert C.sizeof(A.Mesh) == 16
    assert C.sizeof(A.Light) == 20
    assert C.sizeof(A.PassRecord) == 32 * 8
    assert C.sizeof(A.Texture) == 16
    assert A.Material.tex.offset == 60 and A.SceneDesc.n_textures.offset == A.SceneDesc.textures.offset + 8


def test_host_entry_points_validate_arguments(W):
    h = C.c_void_p()
    assert W.lib().wpbr_scenegen_create(0, 0, 0, 16, 0, 0, C.byref(h)) == W.ERR_INVALID_ARG
    assert W.lib().wpbr_scenegen_create(9, 0, 16, 16, 0, 0, C.byref(h)) == W.ERR_INVALID_ARG
    assert W.lib().wpbr_camera_setup(None, None, None, None) == W.ERR_INVALID_ARG
    assert W.lib().wpbr_create(0, None) == W.ERR_INVALID_ARG


def test_instrumentation_entry_points_validate_arguments(W):
    L = W.lib()
    c = C.c_uint32()
    f = C.c_float()
    assert L.wpbr_collide_launches(None, 1000, C.byref(c)) == W.ERR_INVALID_ARG
    assert L.wpbr_set_kernel_timing(None, 1) == W.ERR_INVALID_ARG
    assert L.wpbr_kernel_timing(None, C.byref(f), C.byref(c)) == W.ERR_INVALID_ARG
    assert L.wpbr_collide(None, None, 0, None, 0) == W.ERR_INVALID_ARG
    keys = (C.c_uint32 * 4)()
    assert L.wpbr_debug_ray_order(None, None, 0, keys, keys) == W.ERR_INVALID_ARG


def test_no_device_is_reported_not_faked(W):
    if W.device_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert W.lib().wpbr_create(0, C.byref(h)) == W.ERR_NO_DEVICE


def test_scenegen_counts_and_determinism(W):
    g = W.SceneGen(1, 0, (8, 8), level=8)
    d = g.desc.contents
    assert d.n_triangles == 1310720 and d.n_vertices == 655362 and d.n_spheres == 0
    pos = np.ctypeslib.as_array(d.positions, shape=(d.n_vertices * 3,)).copy()
    g2 = W.SceneGen(1, 0, (8, 8), level=8)
    d2 = g2.desc.contents
    assert np.array_equal(pos, np.ctypeslib.as_array(d2.positions, shape=(d2.n_vertices * 3,)))
    r = np.linalg.norm(pos.reshape(-1, 3), axis=1)
    assert 0.89 < r.min() and r.max() < 1.11
    # the desc points into its generator: keep each generator alive while it is read
    g0 = W.SceneGen(0, 0, (256, 256))
    c0 = g0.desc.contents
    assert c0.n_spheres == 65 and c0.n_triangles == 2 and c0.n_lights == 1
    g2 = W.SceneGen(2, 0, (64, 36), level=4)
    c2 = g2.desc.contents
    assert c2.n_spheres == 256 and c2.envmap.contents.width == 1024 and c2.envmap.contents.height == 512


def test_c1_ray_set(W):
    g = W.SceneGen(1, 0, (64, 64), level=5, rays=True)
    rays = g.rays()
    assert rays.shape == (2 * 64 * 64, 8)
    d = rays[:, 4:7]
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)
    assert np.all(np.isinf(rays[:, 7]))


@pytest.mark.parametrize("config,res,level", [(0, (256, 256), 0), (2, (1920, 1080), 4)])
def test_camera_setup_matches_oracle(W, O, config, res, level):
    g = W.SceneGen(config, 0, res, level=level)
    rc, dx, dy = W.camera_setup(g.desc.contents.camera)
    o = O.OracleScene(g.desc)
    orc, odx, ody = o.camera()
    assert np.array_equal(rc.view(np.uint32), orc.view(np.uint32))
    assert np.array_equal(dx.view(np.uint32), odx.view(np.uint32))
    assert np.array_equal(dy.view(np.uint32), ody.view(np.uint32))


def test_batched_scene_set(W):
    # 32 scenes: primitive counts log-uniform on [10k, 2M] rounded to an
    # icosphere level (or a sphere set), films from {256, 512, 768, 1024}^2
    films, counts, spheres_sets = set(), [], 0
    for k in range(32):
        gk = W.SceneGen(3, seed=3, res=(1024, 2000000), level=k)
        d = gk.desc.contents
        assert d.camera.res_x == d.camera.res_y
        films.add(d.camera.res_x)
        n = d.n_triangles + d.n_spheres - 1  # the light's sphere
        counts.append(n)
        spheres_sets += d.n_triangles == 0
        assert d.n_lights == 2 and d.envmap and d.envmap.contents.width == 256  # sphere + environment
    assert films <= {256, 512, 768, 1024} and len(films) >= 3
    assert 10000 <= min(counts) and max(counts) <= 2000000 and len(set(counts)) >= 5
    assert 0 < spheres_sets < 32
    ga, gb = (W.SceneGen(3, seed=3, res=(1024, 2000000), level=13) for _ in range(2))
    a, b = ga.desc.contents, gb.desc.contents
    assert a.n_spheres == b.n_spheres and bytes(a.spheres[5]) == bytes(b.spheres[5])
    gs = W.SceneGen(3, seed=3, res=(128, 20000), level=1)
    small = gs.desc.contents
    assert small.camera.res_x in (32, 64, 96, 128) and small.n_spheres + small.n_triangles <= 20001 + 1


def test_batch_entry_points_validate_arguments(W):
    assert W.lib().wpbr_batch_create(0, None) == W.ERR_INVALID_ARG
    assert W.lib().wpbr_batch_add_scene(None, None, 0, None) == W.ERR_INVALID_ARG
    assert W.lib().wpbr_batch_info_get(None, None) == W.ERR_INVALID_ARG
    assert W.lib().wpbr_batch_last_error(None) == b"null batch"


def test_textured_scene_generation(W):
    g = W.SceneGen(5, 3, (64, 48))
    d = g.desc.contents
    assert d.n_textures == 4 and d.n_spheres == 65 and d.n_triangles == 2
    metal = [m for m in range(d.n_materials) if d.materials[m].type in (3, 4)]
    assert len(metal) == 3 and sum(d.materials[m].type == 4 for m in metal) == 1
    for m in metal:
        assert all(t < d.n_textures for t in d.materials[m].tex)
    # ground and every third sphere are textured metal
    assert d.meshes[0].material in metal
    assert sum(d.spheres[i].material in metal for i in range(64)) == 22

    def texels(desc, i):
        t = desc.textures[i]
        return np.ctypeslib.as_array(t.rgb, shape=(t.width * t.height * 3,)).copy()

    g2, g3 = W.SceneGen(5, 3, (64, 48)), W.SceneGen(5, 4, (64, 48))  # keep the generators alive
    d2, d3 = g2.desc.contents, g3.desc.contents
    for i in range(4):
        a = texels(d, i)
        assert np.isfinite(a).all() and (a >= 0).all()
        assert np.array_equal(a, texels(d2, i))
        assert not np.array_equal(a, texels(d3, i))
    rough = texels(d, 1).reshape(64, 64, 3)[..., 0]
    assert 1e-6 < rough.min() and rough.max() <= 1e-2


def _desc_bytes(desc):
    """Every array and struct a scene description points to, as raw bytes."""
    d = desc.contents
    out = [bytes(d.camera)]

    def arr(ptr, n, ctype):
        if n == 0 or not ptr:
            return b""
        return bytes((ctype * n).from_address(C.addressof(ptr.contents)))

    out.append(arr(d.spheres, d.n_spheres, type(d.spheres.contents) if d.n_spheres else C.c_uint8))
    for name in ("positions", "normals", "tangents", "uvs"):
        p = getattr(d, name)
        k = 2 if name == "uvs" else 3
        out.append(arr(p, d.n_vertices * k, C.c_float) if p else b"")
    out.append(arr(d.indices, 3 * d.n_triangles, C.c_uint32))
    for name, n in (("meshes", d.n_meshes), ("materials", d.n_materials), ("lights", d.n_lights)):
        p = getattr(d, name)
        out.append(arr(p, n, type(p.contents)) if n else b"")
    if d.envmap:
        e = d.envmap.contents
        out.append(bytes(e.light_to_world) + bytes(e.world_to_light))
        out.append(arr(e.rgb, 3 * e.width * e.height, C.c_float))
    for i in range(d.n_textures):
        t = d.textures[i]
        out.append(arr(t.rgb, 3 * t.width * t.height, C.c_float))
    return out


@pytest.mark.parametrize("config,level,res,rays", [
    (0, 0, (256, 256), False), (1, 4, (256, 256), True), (2, 3, (64, 36), False), (3, 13, (1024, 2000000), False),
    (3, 2, (128, 20000), False), (4, 1, (64, 64), False), (5, 0, (48, 32), False)])
def test_oracle_copy_of_scene_generator_is_identical(W, O, config, level, res, rays):
    # the CPU baseline and the reference arm of the benchmark take their inputs
    # from the oracle library's copy of the generator: same source, same flags,
    # byte-identical scenes and rays
    a = W.SceneGen(config, 0, res, level=level, rays=rays)
    b = O.SceneGen(config, 0, res, level=level, rays=rays)
    assert _desc_bytes(a.desc) == _desc_bytes(b.desc)
    if rays:
        assert np.array_equal(a.rays().view(np.uint32), b.rays().view(np.uint32))
