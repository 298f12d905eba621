"""The oracle itself: known-answer checks of its restated formulas, internal
consistency (the pruned traversal equals the reference's prune-free
candidate list; the flattened tree is well formed) and the committed golden
fixtures (regression pins; the reference ships none)."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_fresnel_known_answers(O):
    L = O.lib()
    for et in (1.3, 1.5, 1.7):
        assert L.orc_fresnel_dielectric(1.0, 1.0, et) == pytest.approx(((et - 1) / (et + 1)) ** 2, rel=1e-6)
    # exiting with sin(theta_t) >= 1: total internal reflection
    assert L.orc_fresnel_dielectric(-0.1, 1.0, 1.5) == 1.0
    for eta, k in ((0.2, 3.0), (1.5, 1.0), (3.0, 0.2)):
        ref = ((eta - 1) ** 2 + k * k) / ((eta + 1) ** 2 + k * k)
        assert L.orc_fresnel_conductor(1.0, 1.0, eta, k) == pytest.approx(ref, rel=1e-5)


def test_microfacet_and_mis_known_answers(O):
    L = O.lib()
    for a in (0.05, 0.25, 0.5):
        af = float(np.float32(a))
        # D(n) = 1 / (PI a^2) with PI = 3.14 (pch.h:30), evaluated in double
        assert L.orc_tr_d(af, af, 0.0, 0.0, 1.0) == np.float32(1.0 / (3.14 * af * af))
    assert L.orc_power_heuristic(1.0, 1.0) == 0.5
    assert L.orc_power_heuristic(3.0, 4.0) == pytest.approx(9 / 25, rel=1e-7)
    B = np.float32(1 / 3)
    assert L.orc_mitchell(0.0) == pytest.approx((6 - 2 * B) / 6, rel=1e-6)
    assert abs(L.orc_mitchell(1.0)) < 1e-6  # |2x| = 2: support edge (float rounding of B, C)
    assert L.orc_left_shift3(1) == 1 and L.orc_left_shift3(2) == 8
    assert L.orc_left_shift3(1023) == 0x09249249 and L.orc_left_shift3(1024) == 0x09249249


def test_pruned_traversal_equals_faithful(W, O):
    for config, level in ((1, 5), (1, 6)):
        g = W.SceneGen(config, 0, (128, 128), level=level, rays=True)
        o = O.OracleScene(g.desc)
        rays = g.rays()
        hf = o.trace(rays, mode=0)
        hp = o.trace(rays, mode=1)
        assert np.array_equal(hf.view(np.uint32), hp.view(np.uint32))
        ha = o.trace(rays, mode=2)
        assert np.array_equal(ha[:, 1].view(np.uint32) == 0xFFFFFFFF, hf[:, 1].view(np.uint32) == 0xFFFFFFFF)


@pytest.mark.parametrize("full_sort", [False, True])
def test_pruned_traversal_equals_faithful_on_exact_ties(W, O, full_sort):
    # Rays straight down onto the diagonals of a flat grid's quads hit both
    # triangles of the quad at exactly t = 5: the pruned traversal must pick
    # the same one as the prune-free candidate list, and any-hit must find a
    # hit exactly where the closest-hit does.
    from scenes import grid_desc

    desc, keep = grid_desc()
    q = W.Q_FULL_MORTON_SORT if full_sort else 0
    o = O.OracleScene(desc, q)
    nodes = o.bvh_export()["nodes"].reshape(-1, 3)
    assert nodes[nodes[:, 1] > 0, 1].max() == (18 if full_sort else 2)
    rng = np.random.default_rng(3)
    n = 20000
    s = rng.choice([0.25, 0.5, 0.75], n).astype(np.float32)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0] = rng.integers(-24, 24, n) + s
    rays[:, 2] = rng.integers(-24, 24, n) + s
    rays[:, 1] = 5.0
    rays[:, 5] = -1.0
    rays[:, 7] = np.inf
    hf = o.trace(rays, mode=0)
    hp = o.trace(rays, mode=1)
    assert np.all(hf[:, 0] == 5.0)
    assert np.array_equal(hf.view(np.uint32), hp.view(np.uint32))
    ha = o.trace(rays, mode=2)
    assert np.array_equal(ha[:, 1].view(np.uint32) == 0xFFFFFFFF, hf[:, 1].view(np.uint32) == 0xFFFFFFFF)
    del keep


def test_pruned_traversal_equals_faithful_in_one_large_leaf(W, O):
    # 100 triangles sharing one Morton code form one leaf; rays through the
    # cluster hit many of them
    from scenes import cluster_desc

    desc, keep = cluster_desc(100)
    o = O.OracleScene(desc)
    nodes = o.bvh_export()["nodes"].reshape(-1, 3)
    assert nodes[nodes[:, 1] > 0, 1].max() == 100
    rng = np.random.default_rng(5)
    n = 5000
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, :3] = 0.5 - 2.0 * d + rng.uniform(-0.002, 0.002, (n, 3))
    rays[:, 4:7] = d
    rays[:, 7] = np.inf
    hf = o.trace(rays, mode=0)
    hp = o.trace(rays, mode=1)
    assert np.mean(hf[:, 1].view(np.uint32) != 0xFFFFFFFF) > 0.9
    assert np.array_equal(hf.view(np.uint32), hp.view(np.uint32))
    del keep


def check_tree(e):
    nodes = e["nodes"].reshape(-1, 3)
    nb = e["node_bounds"].reshape(-1, 6)
    N, M = e["n_prims"], e["n_nodes"]
    covered = np.zeros(N, np.int64)
    for i in range(M):
        off, n, axis = nodes[i]
        if n > 0:
            covered[off:off + n] += 1
        else:
            assert axis < 3 and i + 1 < M and i + 1 < off < M
            for c in (i + 1, off):
                assert np.all(nb[c, :3] >= nb[i, :3]) and np.all(nb[c, 3:] <= nb[i, 3:])
    assert np.all(covered == 1)
    assert sorted(e["shapes"].tolist()) == list(range(N))


@pytest.mark.parametrize("quirks", [0, 16])
def test_oracle_tree_well_formed(W, O, quirks):
    g = W.SceneGen(1, 0, (8, 8), level=5)
    o = O.OracleScene(g.desc, quirks)
    e = o.bvh_export()
    check_tree(e)
    sc = e["sorted_codes"]
    key = sc if quirks else (sc & 0xFFFFFF)
    assert np.all(np.diff(key.astype(np.int64)) >= 0)  # sorted by the key the tree uses
    assert np.array_equal(e["codes"][e["sorted_prims"]], sc)


def test_golden_fixtures(W, O):
    from tests.golden.make_golden import compute

    ref = np.load(os.path.join(GOLDEN, "oracle_golden.npz"))
    now = compute(W, O)
    assert set(ref.files) == set(now)
    for k in ref.files:
        assert np.array_equal(ref[k].view(np.uint8), np.asarray(now[k]).view(np.uint8)), k


def test_fp64_estimator_dual_gradient_matches_central_differences(W, O):
    # the oracle's FP64 frozen-direction estimator: its image at the scene's
    # own parameters is the oracle render's, and its dual-number gradient
    # matches central differences of its own loss
    g0 = W.SceneGen(4, 0, (40, 32), level=0)
    g1 = W.SceneGen(4, 0, (40, 32), level=1)

    def params(g):
        d = g.desc.contents
        m = np.array([[x.alpha_x, *x.R, *x.eta_t, *x.k] for x in [d.materials[i] for i in range(d.n_materials)]],
                     np.float64).reshape(-1)
        e = np.ctypeslib.as_array(d.envmap.contents.rgb, shape=(256 * 128 * 3,)).astype(np.float64)
        return m, e

    m0, e0 = params(g0)
    m1, e1 = params(g1)
    o = O.OracleScene(g0.desc)
    _, img0, _ = o.adjoint_eval(40, 32, 2, 0, 0, m0, e0, None, None, image=True)
    L, w = o.render(40, 32, 2, 0, 0)
    I = L / w[..., None]
    ok = np.isfinite(I)
    assert np.max(np.abs(img0 - I)[ok] / np.maximum(np.abs(I[ok]), 1e-6)) < 1e-4
    _, target, _ = O.OracleScene(g1.desc).adjoint_eval(40, 32, 2, 0, 0, m1, e1, None, None, image=True)
    target = target.astype(np.float32)
    rng = np.random.default_rng(4)
    sel = np.concatenate([rng.choice(m0.size, 6, replace=False), m0.size + rng.choice(e0.size, 2000, replace=False)])
    loss, _, grad = o.adjoint_eval(40, 32, 2, 0, 0, m0, e0, target, sel)
    keep = np.concatenate([np.arange(6), 6 + np.nonzero(grad[6:])[0][:4]])
    h = 1e-4
    for k in keep:
        i = sel[k]
        mp, ep, mm, em = m0.copy(), e0.copy(), m0.copy(), e0.copy()
        if i < m0.size:
            mp[i] += h
            mm[i] -= h
        else:
            ep[i - m0.size] += h
            em[i - m0.size] -= h
        fd = (o.adjoint_eval(40, 32, 2, 0, 0, mp, ep, target)[0] - o.adjoint_eval(40, 32, 2, 0, 0, mm, em, target)[0]) / (2 * h)
        assert abs(grad[k] - fd) <= 1e-4 * max(abs(fd), 1e-3 * np.abs(grad).max()), (i, grad[k], fd)
        # the same differences with the frozen state computed once
        fd1 = o.adjoint_fd(2, 0, 0, m0, e0, target, [i], h=h)[0]
        assert abs(fd1 - fd) <= 1e-9 * max(abs(fd), 1e-12), (i, fd, fd1)


def test_spectral_tables_and_conversions(W, O):
    # binned CIE matching functions and RGB-to-spectrum bases of the
    # Sampled64 mode (64 bins over 400-700 nm)
    t = O.spectral_tables()
    X, Y, Z = t[0], t[1], t[2]
    white_refl, white_illum = t[3], t[10]
    assert np.all(Y >= 0) and np.all(X >= 0) and np.all(Z >= 0)
    dl = 300.0 / 64
    # the visible part of the Y integral (106.857 over 360-830 nm)
    assert 100.0 < Y.sum() * dl < 106.857
    assert np.argmax(Y) in range(25, 35)          # peak near 555 nm
    assert abs(white_refl.mean() - 1.0) < 0.1 and abs(white_illum.mean() - 1.0) < 0.1
    # a spectral render of the plain scene is finite and, up to the
    # unnormalised toXYZ scale, close in chromaticity to the RGB render
    g = W.SceneGen(0, 0, (48, 40))
    o = O.OracleScene(g.desc)
    Ls, ws = o.render_spectral(48, 40, 2, 0, 0)
    Lr, wr = o.render(48, 40, 2, 0, 0)
    assert np.array_equal(ws, wr)
    ok = np.isfinite(Ls).all(axis=-1) & (Lr.sum(-1) > 1e-3)
    assert ok.sum() > 100
    lum_s, lum_r = Ls[ok].sum(-1), Lr[ok].sum(-1)
    ratio = lum_s / lum_r
    # toXYZ is not divided by CIE_Y_integral: the spectral film is ~107x the RGB one
    assert 100 < np.median(ratio) < 115 and np.std(np.log(ratio)) < 0.1
