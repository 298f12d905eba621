"""Failure paths, exercised without faulting the GPU.

- Traversal bounds: wpbr_set_traversal_limits lowers the lane stack or the
  loop bound; the kernel gives up on its rays, records the bound in the
  device error word and returns (no trap), wpbr_check_device_errors reports
  WPBR_ERR_TRAVERSAL_LIMIT, and the same context traces correctly once the
  bounds are restored. The reference's stack (nodesToVisit[256],
  SLBVH.cpp:101) is unchecked.
- Host-side injections: non-finite geometry and empty scenes at upload, zero
  rays, and device allocations that fail (wpbr_debug_fail_allocations, a
  fake of cudaMalloc's out-of-memory) without leaking device memory."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rays(n, seed=3, span=12.0):
    rng = np.random.default_rng(seed)
    r = np.zeros((n, 8), np.float32)
    r[:, :3] = rng.uniform(-span, span, (n, 3))
    d = rng.normal(size=(n, 3))
    r[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r[:, 7] = np.inf
    return r


def _same_hits(a, b):
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.fixture(scope="module")
def mesh(W, O):
    g = W.SceneGen(1, 0, (128, 128), level=6, rays=True)
    return g, g.rays(), O.OracleScene(g.desc)


@pytest.mark.parametrize("limits", [(1, 0), (0, 2)])
def test_traversal_limit_is_reported_and_the_context_recovers(W, ctx, mesh, limits):
    g, rays, o = mesh
    ctx.set_quirks(0)
    ctx.upload(g.desc)
    ctx.build()
    ref = o.trace(rays, mode=0)
    ctx.check_device_errors()
    ctx.set_traversal_limits(*limits)
    for mode in (W.TRACE_CLOSEST, W.TRACE_ANY):
        ctx.collide(rays, mode=mode)  # returns; the hits of abandoned rays are not valid
        with pytest.raises(W.WpbrError) as ei:
            ctx.check_device_errors()
        assert ei.value.status == W.ERR_TRAVERSAL_LIMIT
    ctx.set_traversal_limits(0, 0)
    assert _same_hits(ctx.collide(rays), ref)
    ctx.check_device_errors()  # cleared, and nothing new


def test_traversal_limit_in_the_render_pass(W, O, ctx):
    g = W.SceneGen(2, 0, (64, 36), level=4)
    ctx.set_quirks(0)
    ctx.upload(g.desc)
    ctx.build()
    ctx.set_traversal_limits(1, 0)
    ctx.render_setup(2, seed=0)
    ctx.render()
    with pytest.raises(W.WpbrError) as ei:
        ctx.check_device_errors()
    assert ei.value.status == W.ERR_TRAVERSAL_LIMIT
    ctx.set_traversal_limits(0, 0)  # the pass graph is recaptured with the default bounds
    ctx.render_setup(2, seed=0)
    ctx.render()
    L, w = ctx.film(64, 36)
    Lo, wo = O.OracleScene(g.desc).render(64, 36, 2)
    assert np.array_equal(L.view(np.uint32), Lo.view(np.uint32)) and np.array_equal(w, wo)
    ctx.check_device_errors()


def test_limit_arguments_are_validated(W, ctx):
    with pytest.raises(W.WpbrError) as ei:
        ctx.set_traversal_limits(257, 0)
    assert ei.value.status == W.ERR_INVALID_ARG
    ctx.set_traversal_limits(0, 0)


def test_non_finite_geometry_is_rejected(W, ctx):
    g = W.SceneGen(2, 0, (32, 18), level=2)
    d = g.desc.contents
    for name, poke in (("vertex", lambda v: d.positions.__setitem__(7, v)),
                       ("radius", lambda v: setattr(d.spheres[3], "radius", v)),
                       ("transform", lambda v: d.spheres[5].object_to_world.m.__setitem__(3, v))):
        for bad in (np.nan, np.inf):
            keep = (d.positions[7], d.spheres[3].radius, d.spheres[5].object_to_world.m[3])
            poke(float(bad))
            with pytest.raises(W.WpbrError) as ei:
                ctx.upload(g.desc)
            assert ei.value.status == W.ERR_INVALID_ARG, name
            d.positions[7], d.spheres[3].radius = keep[0], keep[1]
            d.spheres[5].object_to_world.m[3] = keep[2]
    ctx.upload(g.desc)  # restored: accepted again
    ctx.build()
    ctx.check_device_errors()


def test_empty_scene_and_zero_rays(W, ctx):
    g = W.SceneGen(0, 0, (32, 32))
    d = g.desc.contents
    keep = (d.n_spheres, d.n_triangles, d.n_meshes, d.n_lights)
    d.n_spheres = d.n_triangles = d.n_meshes = d.n_lights = 0
    try:
        ctx.set_quirks(0)
        ctx.upload(g.desc)
        ctx.build()
        info = ctx.bvh_info()
        assert info["n_prims"] == 0
        h = ctx.collide(_rays(1000))
        assert np.all(h[:, 1].view(np.uint32) == 0xFFFFFFFF) and np.all(np.isinf(h[:, 0]))
        # no lights and nothing to hit: an all-black film of full weight
        ctx.render_setup(2, seed=0)
        ctx.render()
        L, w = ctx.film(32, 32)
        assert np.all(L == 0) and np.all(w > 0)
    finally:
        d.n_spheres, d.n_triangles, d.n_meshes, d.n_lights = keep
    # zero rays: nothing to do, through both entry points
    ctx.upload(g.desc)
    ctx.build()
    assert ctx.collide(np.zeros((0, 8), np.float32)).shape == (0, 4)
    assert W.lib().wpbr_collide_device(ctx.handle, None, 0, None, W.TRACE_CLOSEST) == W.OK
    ctx.check_device_errors()


def _free_bytes():
    torch = pytest.importorskip("torch")
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_allocation_failures_return_oom_without_leaking(W, O):
    g = W.SceneGen(2, 0, (64, 36), level=4)
    rays = _rays(4096)
    ref = O.OracleScene(g.desc).trace(rays, mode=0)
    Lo, wo = O.OracleScene(g.desc).render(64, 36, 2)
    before = _free_bytes()
    # context creation itself
    W.debug_fail_allocations(0)
    try:
        with pytest.raises(W.WpbrError) as ei:
            W.Context(0)
        assert ei.value.status == W.ERR_OOM
    finally:
        W.debug_fail_allocations(-1)
    # every allocation point of upload, build, collide and a render in turn
    failures = 0
    for k in range(0, 400):
        c = W.Context(0)
        try:
            W.debug_fail_allocations(k)
            try:
                c.upload(g.desc)
                c.build()
                c.collide(rays)
                c.render_setup(2, seed=0)
                c.render()
                completed = True
            except W.WpbrError as e:
                assert e.status == W.ERR_OOM, (k, e)
                completed = False
                failures += 1
            finally:
                W.debug_fail_allocations(-1)
            # the same context finishes the work once allocations succeed again
            c.upload(g.desc)
            c.build()
            assert _same_hits(c.collide(rays), ref), k
            c.render_setup(2, seed=0)
            c.render()
            L, w = c.film(64, 36)
            assert np.array_equal(L.view(np.uint32), Lo.view(np.uint32)) and np.array_equal(w, wo), k
            c.check_device_errors()
        finally:
            c.close()
        if completed:
            break
    assert completed and failures >= 10
    assert abs(_free_bytes() - before) <= 8 << 20  # everything the contexts held was freed
