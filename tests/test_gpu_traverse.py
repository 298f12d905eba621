"""GPU collision (wpbr_collide) against the oracle's prune-free reference
traversal: hit primitive ids and t bit-exact, barycentrics bit-exact."""
import numpy as np
import pytest
from scenes import cluster_desc, grid_desc

pytestmark = pytest.mark.gpu


def _check(hg, ho):
    pg, po = hg[:, 1].view(np.uint32), ho[:, 1].view(np.uint32)
    bad = np.nonzero(pg != po)[0]
    assert bad.size == 0, (bad.size, bad[:8], pg[bad[:8]], po[bad[:8]], hg[bad[:4]], ho[bad[:4]])
    assert np.array_equal(hg.view(np.uint32), ho.view(np.uint32))


@pytest.mark.parametrize("level,res", [(5, (128, 128)), (7, (256, 256))])
def test_closest_hit_parity_c1(W, O, ctx, level, res):
    g = W.SceneGen(1, 0, res, level=level, rays=True)
    ctx.set_quirks(0)
    ctx.upload(g.desc)
    ctx.build()
    rays = g.rays()
    hg = ctx.collide(rays)
    ho = O.OracleScene(g.desc).trace(rays, mode=0)
    _check(hg, ho)
    assert 0.3 < np.mean(hg[:, 1].view(np.uint32) != 0xFFFFFFFF) < 1.0
    ha = ctx.collide(rays, mode=W.TRACE_ANY)
    assert np.array_equal(ha[:, 1].view(np.uint32) == 0xFFFFFFFF, hg[:, 1].view(np.uint32) == 0xFFFFFFFF)
    ctx.check_device_errors()


def test_closest_hit_parity_c1_full_size_sample(W, O, ctx):
    g = W.SceneGen(1, 0, (2048, 2048), level=8, rays=True)
    ctx.set_quirks(0)
    ctx.upload(g.desc)
    ctx.build()
    rays = g.rays()
    assert rays.shape[0] == 8 * 1024 * 1024
    hg = ctx.collide(rays)
    idx = np.random.default_rng(5).choice(rays.shape[0], 60000, replace=False)
    ho = O.OracleScene(g.desc).trace(rays[idx], mode=0)
    _check(hg[idx], ho)
    ctx.check_device_errors()


def test_degenerate_rays_and_quirk(W, O, ctx):
    g = W.SceneGen(0, 0, (64, 64))
    rng = np.random.default_rng(7)
    n = 20000
    o = rng.uniform(-15, 15, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d[: n // 4, 1:] = 0.0          # axis-aligned directions (inf reciprocals)
    d[n // 4: n // 2, 0] = 0.0     # one zero component
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[n // 2: n // 2 + 100, 1] = -1.0  # straight down onto the ground quad
    d[n // 2: n // 2 + 100, [0, 2]] = 0.0
    rays = np.zeros((n, 8), np.float32)
    rays[:, :3] = o
    rays[:, 4:7] = d
    rays[:, 7] = np.inf
    for q in (0, W.Q_TRI_PERMUTATION_BUG):
        ctx.set_quirks(q)
        ctx.upload(g.desc)
        ctx.build()
        hg = ctx.collide(rays)
        ho = O.OracleScene(g.desc, q).trace(rays, mode=0)
        _check(hg, ho)
    ctx.set_quirks(0)


@pytest.mark.parametrize("config,level,res", [(1, 6, (128, 128)), (0, 0, (64, 64)), (2, 4, (64, 36))])
def test_split_and_full_leaf_traversals_agree(W, O, ctx, config, level, res):
    # the leaf-split layout visits a split leaf's primitives in their sorted
    # order: identical hits to the reference's leaves as they are, ties included
    g = W.SceneGen(config, 0, res, level=level, rays=(config == 1))
    ctx.set_quirks(0)
    ctx.set_traversal(W.TRAVERSAL_BINARY_FULL_LEAVES)
    ctx.upload(g.desc)
    ctx.build()
    if config == 1:
        rays = g.rays()
    else:
        rng = np.random.default_rng(3)
        n = 30000
        rays = np.zeros((n, 8), np.float32)
        rays[:, :3] = rng.uniform(-12, 12, (n, 3))
        d = rng.normal(size=(n, 3))
        rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
        rays[:, 7] = np.inf
    hw = ctx.collide(rays)
    aw = ctx.collide(rays, mode=W.TRACE_ANY)
    ctx.set_traversal(W.TRAVERSAL_BINARY)
    hb = ctx.collide(rays)
    ab = ctx.collide(rays, mode=W.TRACE_ANY)
    assert np.array_equal(hw.view(np.uint32), hb.view(np.uint32))
    assert np.array_equal(aw[:, 1].view(np.uint32) == 0xFFFFFFFF, ab[:, 1].view(np.uint32) == 0xFFFFFFFF)
    _check(hw, O.OracleScene(g.desc).trace(rays, mode=0))
    ctx.check_device_errors()


def test_ray_reordering_keeps_hits(W, ctx):
    # batches of 256k rays and more are traced in Morton order of their
    # origins; every hit is written back to its input position unchanged
    g = W.SceneGen(1, 0, (512, 512), level=6, rays=True)
    ctx.set_quirks(0)
    ctx.upload(g.desc)
    ctx.build()
    rays = g.rays()
    assert rays.shape[0] >= 1 << 18
    hs = ctx.collide(rays)
    as_ = ctx.collide(rays, mode=W.TRACE_ANY)
    ctx.set_ray_sort(0)
    hu = ctx.collide(rays)
    au = ctx.collide(rays, mode=W.TRACE_ANY)
    assert ctx.collide_launches(rays.shape[0]) == 1  # traversal only
    ctx.set_ray_sort(5)
    h5 = ctx.collide(rays)
    # key kernel + 2 radix passes (15 bits) x (histogram, scan, scatter) + traversal
    assert ctx.collide_launches(rays.shape[0]) > 4
    assert ctx.collide_launches(1000) == 1
    ctx.set_ray_sort(8)
    # traversal launches timed with CUDA events when asked, and only then
    ctx.set_kernel_timing(True)
    ctx.collide(rays)
    ctx.collide(rays, mode=W.TRACE_ANY)
    ms, launches = ctx.kernel_timing()
    assert launches == 2 and ms > 0.0
    assert ctx.kernel_timing() == (0.0, 0)
    ctx.set_kernel_timing(False)
    ctx.collide(rays)
    assert ctx.kernel_timing()[1] == 0
    assert np.array_equal(hs.view(np.uint32), h5.view(np.uint32))
    assert np.array_equal(hs.view(np.uint32), hu.view(np.uint32))
    assert np.array_equal(as_[:, 1].view(np.uint32) == 0xFFFFFFFF, au[:, 1].view(np.uint32) == 0xFFFFFFFF)
    ctx.check_device_errors()


@pytest.mark.parametrize("bits", [8, 5, 10])
def test_ray_order_is_a_stable_sort(W, ctx, bits):
    # the radix sort behind the ray order (one pass per 8-bit digit; 15 bits
    # end on a 7-bit digit, 30 bits take four passes): for
    # whole, ragged, one-tile and tiny batches, in the generator's order and
    # shuffled, the trace order is the stable sort of the origin keys
    g = W.SceneGen(1, 0, (512, 512), level=6, rays=True)
    ctx.set_quirks(0)
    ctx.upload(g.desc)
    ctx.build()
    rays = g.rays()
    shuffled = rays[np.random.default_rng(3).permutation(rays.shape[0])]
    ctx.set_ray_sort(bits)
    try:
        for rs in (rays, shuffled):
            for n in (rs.shape[0], 3 * 2048 + 5, 2048, 2, 1):
                keys, perm = ctx.debug_ray_order(rs[:n])
                assert int(keys.max()) < 1 << (3 * bits)
                assert np.array_equal(perm, np.argsort(keys, kind="stable").astype(np.uint32))
        # identical origins share a key (the coherent half has one origin)
        o = rays[:, :3]
        same = np.all(o == o[0], axis=1)
        keys, _ = ctx.debug_ray_order(rays)
        assert same.sum() > 1 and np.all(keys[same] == keys[0])
    finally:
        ctx.set_ray_sort(8)
    ctx.check_device_errors()


def test_chunked_host_collide_matches_device_collide(W, ctx):
    # host-buffer batches of 2^22 rays and more are copied and traced in
    # chunks whose copies overlap the neighbouring chunks' traversal; the
    # hits must equal one device-resident call over the whole batch (each
    # chunk is reordered on its own, and reordering never changes a hit)
    torch = pytest.importorskip("torch")
    g = W.SceneGen(1, 0, (1024, 1024), level=7, rays=True)
    ctx.set_quirks(0)
    ctx.upload(g.desc)
    ctx.build()
    rays = g.rays()
    rays = np.concatenate([rays, rays, rays])
    n = (1 << 22) + (1 << 21) + 777  # 4 uneven chunks, none a multiple of the others
    rays = np.concatenate([rays, rays[: n - rays.shape[0]]])
    assert rays.shape[0] == n
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()  # the context's stream does not wait for torch's
    for mode in (W.TRACE_CLOSEST, W.TRACE_ANY):
        ctx.collide_device(d_rays.data_ptr(), n, d_hits.data_ptr(), mode)
        ctx.synchronize()
        hd = d_hits.cpu().numpy()
        hh = ctx.collide(rays, mode=mode)
        if mode == W.TRACE_CLOSEST:
            assert np.array_equal(hh.view(np.uint32), hd.view(np.uint32))
        else:
            assert np.array_equal(hh[:, 1].view(np.uint32) == 0xFFFFFFFF, hd[:, 1].view(np.uint32) == 0xFFFFFFFF)
    ctx.check_device_errors()


@pytest.mark.parametrize("full_sort", [False, True])
def test_leaf_split_keeps_ties_and_first_hits(W, O, ctx, full_sort):
    # Leaves of more than eight primitives are subdivided for traversal into
    # small trees over position ranges, visited lowest range first. Rays
    # straight down onto the diagonals of a flat grid's quads hit two
    # triangles at exactly t = 5 (with the full 30-bit sort the grid's leaves
    # hold 18 triangles, so some tied pairs straddle two ranges): the winner
    # must still be the first in the reference's order, and any-hit the first
    # hit of its scan.
    desc, keep = grid_desc()
    q = W.Q_FULL_MORTON_SORT if full_sort else 0
    ctx.set_quirks(q)
    ctx.upload(desc)
    ctx.build()
    rng = np.random.default_rng(11)
    n = 40000
    o = np.zeros((n, 3), np.float32)
    s = rng.choice([0.25, 0.5, 0.75], n).astype(np.float32)
    o[:, 0] = rng.integers(-24, 24, n) + s
    o[:, 2] = rng.integers(-24, 24, n) + s
    o[:, 1] = 5.0
    o[-10000:, [0, 2]] = rng.uniform(-24, 24, (10000, 2))  # off the diagonals
    rays = np.zeros((n, 8), np.float32)
    rays[:, :3] = o
    rays[:, 5] = -1.0
    rays[:, 7] = np.inf
    sl = rng.normal(size=(5000, 3))  # and slanted rays
    sl[:, 1] = -np.abs(sl[:, 1]) - 0.1
    rays[-5000:, 4:7] = sl / np.linalg.norm(sl, axis=1, keepdims=True)
    oracle = O.OracleScene(desc, q)
    ho, ha_o = oracle.trace(rays, mode=0), oracle.trace(rays, mode=2)
    assert np.mean(ho[: n - 10000, 0] == 5.0) > 0.99
    for mode in (W.TRAVERSAL_BINARY, W.TRAVERSAL_BINARY_FULL_LEAVES):
        ctx.set_traversal(mode)
        _check(ctx.collide(rays), ho)
        _check(ctx.collide(rays, mode=W.TRACE_ANY), ha_o)
    ctx.set_traversal(W.TRAVERSAL_BINARY)
    ctx.set_quirks(0)
    ctx.check_device_errors()
    del keep


@pytest.mark.parametrize("config,level,res", [(1, 6, (128, 128)), (0, 0, (64, 64)), (2, 4, (64, 36))])
def test_leaf_split_layout_matches_reference_leaves(W, O, ctx, config, level, res):
    # closest- and any-hit records of the default (leaf-split) layout equal
    # those over the reference's leaves as they are and the oracle's
    g = W.SceneGen(config, 0, res, level=level, rays=(config == 1))
    ctx.set_quirks(0)
    ctx.upload(g.desc)
    ctx.build()
    if config == 1:
        rays = g.rays()
    else:
        rng = np.random.default_rng(4)
        n = 30000
        rays = np.zeros((n, 8), np.float32)
        rays[:, :3] = rng.uniform(-12, 12, (n, 3))
        d = rng.normal(size=(n, 3))
        rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
        rays[:, 7] = np.inf
    oracle = O.OracleScene(g.desc)
    ctx.set_traversal(W.TRAVERSAL_BINARY)
    hs, as_ = ctx.collide(rays), ctx.collide(rays, mode=W.TRACE_ANY)
    ctx.set_traversal(W.TRAVERSAL_BINARY_FULL_LEAVES)
    hf, af = ctx.collide(rays), ctx.collide(rays, mode=W.TRACE_ANY)
    ctx.set_traversal(W.TRAVERSAL_BINARY)
    assert np.array_equal(hs.view(np.uint32), hf.view(np.uint32))
    assert np.array_equal(as_.view(np.uint32), af.view(np.uint32))
    _check(hs, oracle.trace(rays, mode=0))
    _check(as_, oracle.trace(rays, mode=2))
    ctx.check_device_errors()


@pytest.mark.parametrize("k", [100, 5000])
def test_leaf_split_of_one_large_leaf(W, O, ctx, k):
    # k triangles far smaller than one Morton cell share a code, so the
    # reference's tree holds them in one leaf: 100 become a range tree of
    # depth 4, 5000 exceed the split's bound (4096) and stay one leaf. Rays
    # aimed at the cluster hit many of them; closest and any-hit records must
    # equal the oracle's either way.
    desc, keep = cluster_desc(k)
    rng = np.random.default_rng(k + 1)
    ctx.set_quirks(0)
    ctx.upload(desc)
    ctx.build()
    oracle = O.OracleScene(desc)
    nodes = oracle.bvh_export()["nodes"].reshape(-1, 3)
    assert nodes[nodes[:, 1] > 0, 1].max() == k
    n = 4000
    dirs = rng.normal(size=(n, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, :3] = 0.5 - 2.0 * dirs + rng.uniform(-0.002, 0.002, (n, 3))
    rays[:, 4:7] = dirs
    rays[:, 7] = np.inf
    ho, ha_o = oracle.trace(rays, mode=0), oracle.trace(rays, mode=2)
    assert np.mean(ho[:, 1].view(np.uint32) != 0xFFFFFFFF) > 0.9
    for mode in (W.TRAVERSAL_BINARY, W.TRAVERSAL_BINARY_FULL_LEAVES):
        ctx.set_traversal(mode)
        _check(ctx.collide(rays), ho)
        _check(ctx.collide(rays, mode=W.TRACE_ANY), ha_o)
    ctx.set_traversal(W.TRAVERSAL_BINARY)
    ctx.check_device_errors()
    del keep


def test_traversal_modes(W, ctx):
    # two layouts; anything else (the retired four-wide value 1 included) is
    # an invalid argument
    for mode in (W.TRAVERSAL_BINARY, W.TRAVERSAL_BINARY_FULL_LEAVES):
        ctx.set_traversal(mode)
    for bad in (1, 3):
        with pytest.raises(W.WpbrError):
            ctx.set_traversal(bad)
    ctx.set_traversal(W.TRAVERSAL_BINARY)
