"""GPU LBVH build (wpbr_bvh_build) against the oracle: bounds, centroids,
Morton codes, sort permutation, treelets and the flattened tree must be
bit-exact."""
import ctypes as C

import numpy as np
import pytest

import woodenpbrengine_gb300._abi as A

pytestmark = pytest.mark.gpu


def compare_build(W, O, ctx, desc, quirks=0):
    ctx.set_quirks(quirks)
    ctx.upload(desc)
    ctx.build()
    ge = ctx.bvh_export()
    oe = O.OracleScene(desc, quirks).bvh_export()
    for k in ("n_prims", "n_nodes", "n_treelets", "max_depth"):
        assert ge[k] == oe[k], (k, ge[k], oe[k])
    for k in ("prim_bounds", "centroids", "codes", "sorted_codes", "sorted_prims", "treelet_start", "nodes",
              "node_bounds", "shapes"):
        a, b = np.asarray(ge[k]), np.asarray(oe[k])
        if a.dtype == np.float32:
            assert np.array_equal(a, b), k  # == so that -0 equals +0
            assert np.array_equal(a.view(np.uint32)[a != 0], b.view(np.uint32)[b != 0]), k
        else:
            bad = np.nonzero(a != b)[0]
            assert bad.size == 0, (k, bad[:10], a[bad[:10]], b[bad[:10]])
    assert np.array_equal(ge["cbounds"], oe["cbounds"])
    ctx.check_device_errors()
    return ge


@pytest.mark.parametrize("config,level,res", [(0, 0, (64, 64)), (1, 4, (8, 8)), (1, 6, (8, 8)), (2, 4, (64, 36))])
def test_build_parity(W, O, ctx, config, level, res):
    g = W.SceneGen(config, 0, res, level=level)
    compare_build(W, O, ctx, g.desc)


def test_build_parity_full_sort_quirk(W, O, ctx):
    g = W.SceneGen(1, 0, (8, 8), level=6)
    e = compare_build(W, O, ctx, g.desc, quirks=W.Q_FULL_MORTON_SORT)
    assert e["n_treelets"] < 4096
    ctx.set_quirks(0)


def test_build_parity_level8(W, O, ctx):
    g = W.SceneGen(1, 0, (8, 8), level=8)
    compare_build(W, O, ctx, g.desc)


def _spheres_desc(W, centers, radii):
    g = W.SceneGen(0, 0, (16, 16))
    base = g.desc.contents
    n = len(centers)
    sph = (A.Sphere * n)()
    for i, (c, r) in enumerate(zip(centers, radii)):
        for j in range(16):
            sph[i].object_to_world.m[j] = 0.0
            sph[i].world_to_object.m[j] = 0.0
        for j in range(4):
            sph[i].object_to_world.m[5 * j] = 1.0
            sph[i].world_to_object.m[5 * j] = 1.0
        for a in range(3):
            sph[i].object_to_world.m[4 * a + 3] = c[a]
            sph[i].world_to_object.m[4 * a + 3] = -c[a]
        sph[i].radius = r
        sph[i].material = 0
    d = A.SceneDesc()
    d.spheres = C.cast(sph, C.POINTER(A.Sphere))
    d.n_spheres = n
    d.materials = base.materials
    d.n_materials = base.n_materials
    d.camera = base.camera
    return d, (g, sph)


@pytest.mark.parametrize("kind", ["single", "pair", "coincident40", "line100"])
def test_build_edge_cases(W, O, ctx, kind):
    if kind == "single":
        c, r = [(0, 0, 0)], [1.0]
    elif kind == "pair":
        c, r = [(0, 0, 0), (3, 1, 2)], [1.0, 0.5]
    elif kind == "coincident40":  # identical Morton codes: one leaf past the 29-shape limit
        c, r = [(1.0, 2.0, 3.0)] * 40, [0.5] * 40
    else:  # degenerate extent in y and z (0/0 lerp factors)
        c, r = [(float(i), 0.0, 0.0) for i in range(100)], [0.4] * 100
    d, keep = _spheres_desc(W, c, r)
    compare_build(W, O, ctx, C.pointer(d))
