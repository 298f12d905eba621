"""The C++17 host runner (woodenpbrengine_gb300/host/wpbr_host.cpp): OBJ and
PFM ingestion without a GPU; on the GPU, the fused and staged job orders give
the film of the Python binding bit for bit."""
import json
import os
import subprocess

import numpy as np
import pytest


@pytest.fixture(scope="session")
def host(W):
    from woodenpbrengine_gb300.build import build_host

    return build_host()


def _write_obj(path, pos, idx, uv=None, quads=False):
    with open(path, "w") as f:
        f.write("# test mesh\n")
        for p in pos:
            f.write("v %.9g %.9g %.9g\n" % tuple(p))
        if uv is not None:
            for t in uv:
                f.write("vt %.9g %.9g\n" % tuple(t))
        for t in idx:
            if uv is not None:
                f.write("f %d/%d %d/%d %d/%d\n" % (t[0] + 1, t[0] + 1, t[1] + 1, t[1] + 1, t[2] + 1, t[2] + 1))
            else:
                f.write("f %d %d %d\n" % (t[0] + 1, t[1] + 1, t[2] + 1))
        if quads:  # a quad with negative (relative) indices, fanned into 2 triangles
            f.write("v 0 0 5\nv 1 0 5\nv 1 1 5\nv 0 1 5\nf -4 -3 -2 -1\n")


def _write_pfm(path, rgb):
    H, W, _ = rgb.shape
    with open(path, "wb") as f:
        f.write(b"PF\n%d %d\n-1.0\n" % (W, H))
        f.write(np.ascontiguousarray(rgb[::-1], "<f4").tobytes())


def _read_pfm(path):
    with open(path, "rb") as f:
        assert f.readline().strip() == b"PF"
        W, H = map(int, f.readline().split())
        scale = float(f.readline())
        data = np.frombuffer(f.read(), "<f4" if scale < 0 else ">f4").reshape(H, W, 3)
    return data[::-1].copy()


def _mesh(W):
    g = W.SceneGen(1, 0, (8, 8), level=2)
    d = g.desc.contents
    pos = np.ctypeslib.as_array(d.positions, shape=(d.n_vertices * 3,)).reshape(-1, 3).copy()
    idx = np.ctypeslib.as_array(d.indices, shape=(d.n_triangles * 3,)).reshape(-1, 3).copy()
    return pos, idx


def test_obj_and_pfm_ingestion(W, host, tmp_path):
    pos, idx = _mesh(W)
    uv = np.stack([pos[:, 0] * 0.5 + 0.5, pos[:, 1] * 0.5 + 0.5], 1)
    obj = str(tmp_path / "m.obj")
    _write_obj(obj, pos, idx, uv=uv, quads=True)
    env = np.random.default_rng(0).random((8, 16, 3)).astype(np.float32)
    pfm = str(tmp_path / "e.pfm")
    _write_pfm(pfm, env)
    out = subprocess.run([host, "--obj", obj, "--env", pfm, "--dump-scene"], capture_output=True, text=True,
                         timeout=60)
    assert out.returncode == 0, out.stderr
    info = json.loads(out.stdout)
    assert info["triangles"] == len(idx) + 2 and info["vertices"] == len(pos) + 4
    assert info["uvs"] == 1 and info["env"] == [16, 8] and info["lights"] == 2
    assert abs(info["position_sum"] - (float(pos.astype(np.float64).sum()) + 2 + 2 + 20)) < 1e-3
    bad = subprocess.run([host, "--obj", str(tmp_path / "missing.obj"), "--dump-scene"], capture_output=True,
                         text=True, timeout=60)
    assert bad.returncode == 2 and "cannot open" in bad.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("staged", [False, True])
def test_host_runner_film_matches_binding(W, ctx, host, tmp_path, staged):
    Wd, Hd, spp = 64, 48, 2
    cmd = [host, "--config", "0", "--res", "%dx%d" % (Wd, Hd), "--spp", str(spp), "--out", str(tmp_path / "f")]
    if staged:
        cmd.append("--staged")
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    info = json.loads(out.stdout)
    assert info["mode"] == ("staged" if staged else "fused")
    I = _read_pfm(str(tmp_path / "f.pfm"))
    g = W.SceneGen(0, 0, (Wd, Hd))
    ctx.set_quirks(0)
    ctx.upload(g.desc)
    ctx.build()
    ctx.render_setup(spp, seed=0, stream=0)
    ctx.render()
    L, w = ctx.film(Wd, Hd)
    ref = (L / w[..., None]).astype(np.float32)
    assert np.array_equal(I.view(np.uint32), ref.view(np.uint32))
    assert os.path.getsize(str(tmp_path / "f.ppm")) == Wd * Hd * 3 + len(b"P6\n64 48\n255\n")


@pytest.mark.gpu
def test_host_runner_renders_obj_with_environment(W, host, tmp_path):
    pos, idx = _mesh(W)
    obj = str(tmp_path / "m.obj")
    _write_obj(obj, pos, idx)
    env = np.full((16, 32, 3), 0.5, np.float32)
    pfm = str(tmp_path / "e.pfm")
    _write_pfm(pfm, env)
    out = subprocess.run([host, "--obj", obj, "--env", pfm, "--res", "48x32", "--spp", "2", "--out",
                          str(tmp_path / "o")], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    I = _read_pfm(str(tmp_path / "o.pfm"))
    assert np.isfinite(I).all() and I.max() > 0.0


def test_obj_textured_metal_ingestion(W, host, tmp_path):
    pos, idx = _mesh(W)
    uv = np.stack([pos[:, 0] * 0.5 + 0.5, pos[:, 1] * 0.5 + 0.5], 1)
    rng = np.random.default_rng(1)
    k, r = str(tmp_path / "k.pfm"), str(tmp_path / "r.pfm")
    _write_pfm(k, rng.uniform(0.2, 3.0, (16, 16, 3)).astype(np.float32))
    _write_pfm(r, rng.uniform(0.0, 0.01, (8, 8, 3)).astype(np.float32))
    obj = str(tmp_path / "m.obj")
    _write_obj(obj, pos, idx, uv=uv)
    out = subprocess.run([host, "--obj", obj, "--metal", k, r, "--dump-scene"], capture_output=True, text=True,
                         timeout=60)
    assert out.returncode == 0, out.stderr
    assert json.loads(out.stdout)["textures"] == 2
    plain = str(tmp_path / "p.obj")
    _write_obj(plain, pos, idx)  # no texture coordinates
    bad = subprocess.run([host, "--obj", plain, "--metal", k, r, "--dump-scene"], capture_output=True, text=True,
                         timeout=60)
    assert bad.returncode == 2 and "texture coordinates" in bad.stderr
    both = subprocess.run([host, "--config", "0", "--staged", "--spectral"], capture_output=True, text=True,
                          timeout=60)
    assert both.returncode == 2


@pytest.mark.gpu
def test_host_runner_sampled64_textured_matches_binding(W, ctx, host, tmp_path):
    Wd, Hd, spp = 48, 32, 2
    out = subprocess.run([host, "--config", "5", "--res", "%dx%d" % (Wd, Hd), "--spp", str(spp), "--spectral",
                          "--out", str(tmp_path / "s")], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert json.loads(out.stdout)["mode"] == "fused-sampled64"
    I = _read_pfm(str(tmp_path / "s.pfm"))
    g = W.SceneGen(5, 0, (Wd, Hd))
    ctx.set_quirks(0)
    ctx.set_spectrum(W.SPECTRUM_SAMPLED64)
    try:
        ctx.upload(g.desc)
        ctx.build()
        ctx.render_setup(spp, seed=0, stream=0)
        ctx.render()
        L, w = ctx.film(Wd, Hd)
    finally:
        ctx.set_spectrum(W.SPECTRUM_RGB)
    ref = (L / w[..., None]).astype(np.float32)
    same = (I.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(I) & np.isnan(ref))
    assert same.all()


@pytest.mark.gpu
def test_host_runner_renders_textured_obj(W, host, tmp_path):
    pos, idx = _mesh(W)
    uv = np.stack([pos[:, 0] * 0.5 + 0.5, pos[:, 1] * 0.5 + 0.5], 1)
    obj = str(tmp_path / "m.obj")
    _write_obj(obj, pos, idx, uv=uv)
    rng = np.random.default_rng(2)
    k, r = str(tmp_path / "k.pfm"), str(tmp_path / "r.pfm")
    _write_pfm(k, rng.uniform(0.2, 3.0, (16, 16, 3)).astype(np.float32))
    _write_pfm(r, rng.uniform(0.0, 0.01, (8, 8, 3)).astype(np.float32))
    base = [host, "--obj", obj, "--res", "48x32", "--spp", "2"]
    a = subprocess.run(base + ["--metal", k, r, "--out", str(tmp_path / "a")], capture_output=True, text=True,
                       timeout=300)
    b = subprocess.run(base + ["--out", str(tmp_path / "b")], capture_output=True, text=True, timeout=300)
    assert a.returncode == 0 and b.returncode == 0, (a.stderr, b.stderr)
    Ia, Ib = _read_pfm(str(tmp_path / "a.pfm")), _read_pfm(str(tmp_path / "b.pfm"))
    assert np.isfinite(Ia).mean() > 0.99 and np.nanmax(Ia) > 0.0
    assert not np.array_equal(np.nan_to_num(Ia), np.nan_to_num(Ib))
