"""The differentiable estimator (wpbr_adjoint_*): forward image against the
plain render and the FP64 oracle, gradients against the oracle's dual-number
gradient and against central finite differences of the device forward, on the
differentiable scene (config 4) at reduced film size."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RES = (64, 48)
SPP = 4
N_SEL = 64
TOL = 1e-3


def _params_of(desc):
    d = desc.contents
    mats = [d.materials[i] for i in range(d.n_materials)]
    mat = np.array([[m.alpha_x, *m.R, *m.eta_t, *m.k] for m in mats], np.float32).reshape(-1)
    e = d.envmap.contents
    env = np.ctypeslib.as_array(e.rgb, shape=(e.width * e.height * 3,)).astype(np.float32)
    return mat, env


def _rel_err(g, ref):
    # per-parameter relative error; parameters whose reference gradient is
    # below 1% of the group's largest are compared against that 1% floor
    floor = 1e-2 * np.max(np.abs(ref)) if np.any(ref) else 1.0
    return np.abs(g - ref) / np.maximum(np.abs(ref), floor)


@pytest.fixture(scope="module")
def setup(W, O, ctx):
    g0 = W.SceneGen(4, 0, RES, level=0)
    g1 = W.SceneGen(4, 0, RES, level=1)
    ctx.set_quirks(0)
    ctx.upload(g0.desc)
    ctx.build()
    nm, ne = ctx.adjoint_setup(SPP, seed=0, stream=0)
    assert nm == 640 and ne == 256 * 128 * 3
    m0, e0 = ctx.adjoint_params()
    m0d, e0d = _params_of(g0.desc)
    assert np.array_equal(m0, m0d) and np.array_equal(e0, e0d)
    mh, eh = _params_of(g1.desc)
    ctx.adjoint_set_params(mh, eh)
    ctx.adjoint_freeze()
    target, _ = ctx.adjoint_forward(*RES)
    ctx.adjoint_set_params(m0, e0)
    ctx.adjoint_freeze()
    image, loss = ctx.adjoint_forward(*RES, target)
    gm, ge = ctx.adjoint_backward()
    ctx.check_device_errors()
    rng = np.random.default_rng(4)
    sel_m = rng.choice(nm, N_SEL // 2, replace=False)
    live = np.nonzero(ge)[0]
    sel_e = nm + rng.choice(live, N_SEL // 2, replace=False)
    sel = np.concatenate([sel_m, sel_e]).astype(np.uint32)
    o = O.OracleScene(g0.desc)
    oloss, oimg, ograd = o.adjoint_eval(RES[0], RES[1], SPP, 0, 0, m0, e0, target, sel, image=True)
    return dict(g0=g0, g1=g1, m0=m0, e0=e0, target=target, image=image, loss=loss, gm=gm, ge=ge, sel=sel,
                oloss=oloss, oimg=oimg, ograd=ograd, grad=np.concatenate([gm, ge])[sel])


def test_forward_matches_plain_render(W, ctx, setup):
    ctx.render_setup(SPP, seed=0, stream=0)
    ctx.render()
    L, w = ctx.film(*RES)
    I = L / w[..., None]
    ok = np.isfinite(I)
    rel = np.abs(setup["image"] - I)[ok] / np.maximum(np.abs(I[ok]), 1e-6)
    assert rel.mean() <= 1e-5 and rel.max() <= 1e-3, (rel.mean(), rel.max())


def test_forward_and_loss_match_fp64_oracle(setup):
    img, oimg = setup["image"], setup["oimg"]
    rel = np.abs(img - oimg) / np.maximum(np.abs(oimg), 1e-6)
    assert rel.mean() <= 1e-5 and rel.max() <= 1e-3, (rel.mean(), rel.max())
    assert abs(setup["loss"] - setup["oloss"]) <= 1e-5 * setup["oloss"]


def test_gradient_matches_fp64_oracle(setup):
    g, ref = setup["grad"], setup["ograd"]
    half = N_SEL // 2
    for part in (slice(0, half), slice(half, N_SEL)):
        err = _rel_err(g[part], ref[part])
        assert err.max() <= TOL, (err.max(), setup["sel"][part][np.argmax(err)])
    assert np.linalg.norm(g - ref) <= TOL * np.linalg.norm(ref)


def _central_differences(f, m0, e0, sel, h):
    nm = m0.size
    fd = np.zeros(len(sel))
    for k, i in enumerate(sel):
        vals = []
        for s in (+1, -1):
            m, e = m0.copy(), e0.copy()
            if i < nm:
                m[i] += s * h
            else:
                e[i - nm] += s * h
            vals.append(f(m, e))
        fd[k] = (vals[0] - vals[1]) / (2 * h)
    return fd


def test_gradient_matches_central_differences(O, ctx, setup):
    m0, e0, target, sel, g = setup["m0"], setup["e0"], setup["target"], setup["sel"], setup["grad"]
    h = 1e-3
    # central differences of the FP64 estimator (same frozen sample streams)
    o = O.OracleScene(setup["g0"].desc)
    m64, e64 = m0.astype(np.float64), e0.astype(np.float64)
    fd64 = _central_differences(lambda m, e: o.adjoint_eval(RES[0], RES[1], SPP, 0, 0, m, e, target)[0],
                                m64, e64, sel, h)
    half = N_SEL // 2
    for part in (slice(0, half), slice(half, N_SEL)):
        err = _rel_err(g[part], fd64[part])
        assert err.max() <= TOL, (err.max(), sel[part][np.argmax(err)])
    assert np.linalg.norm(g - fd64) <= TOL * np.linalg.norm(fd64)

    # central differences of the device's own FP32 forward: agreement is
    # bounded by FP32 rounding of the per-sample radiance at h = 1e-3
    def gpu_loss(m, e):
        ctx.adjoint_set_params(m, e)
        return ctx.adjoint_forward(*RES, target)[1]

    fd32 = _central_differences(gpu_loss, m0, e0, sel, h)
    ctx.adjoint_set_params(m0, e0)
    assert np.linalg.norm(g - fd32) <= 5e-2 * np.linalg.norm(fd32), np.linalg.norm(g - fd32) / np.linalg.norm(fd32)


def test_backward_requires_forward_at_current_parameters(W, ctx, setup):
    ctx.adjoint_set_params(setup["m0"], None)
    with pytest.raises(W.WpbrError):
        ctx.adjoint_backward()
    ctx.adjoint_forward(*RES, setup["target"])
    gm, _ = ctx.adjoint_backward()
    assert np.allclose(gm, setup["gm"], rtol=1e-4, atol=1e-7 * np.abs(setup["gm"]).max())


def test_descent_lowers_the_loss(ctx, setup):
    m0, e0, gm, ge = setup["m0"], setup["e0"], setup["gm"], setup["ge"]
    step = 1e-2 / max(np.abs(gm).max(), np.abs(ge).max())
    ctx.adjoint_set_params(m0 - step * gm, e0 - step * ge)
    _, l1 = ctx.adjoint_forward(*RES, setup["target"])
    ctx.adjoint_set_params(m0, e0)
    assert l1 < setup["loss"]
