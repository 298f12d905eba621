"""ctypes binding of oracle/_build/liboracle.so — TEST INFRASTRUCTURE ONLY."""
import ctypes as C
import os

import numpy as np

from woodenpbrengine_gb300 import _abi as A

from .build import OUT, build_oracle

_FP = C.POINTER(C.c_float)
_UP = C.POINTER(C.c_uint32)
_VP = C.c_void_p
_SIGS = {
    "orc_scene_create": (_VP, [C.POINTER(A.SceneDesc), C.c_uint32]),
    "orc_scene_destroy": (None, [_VP]),
    "orc_num_threads": (C.c_int, []),
    "orc_set_threads": (None, [C.c_int]),
    "orc_bvh_sizes": (None, [_VP, _UP]),
    "orc_bvh_export": (None, [_VP, _FP, _FP, _FP, _UP, _UP, _UP, _UP, _UP, _FP, _UP]),
    "orc_trace": (None, [_VP, _FP, C.c_uint64, C.c_int, _FP, _UP]),
    "orc_camera": (None, [_VP, _FP, _FP, _FP]),
    "orc_env_distribution": (None, [_VP, _FP, _FP, _FP, _FP]),
    "orc_render_pass": (None, [_VP] + [C.c_uint32] * 8 + [C.POINTER(A.PassRecord)]),
    "orc_render": (None, [_VP, C.c_uint32, C.c_uint32, C.c_uint32, _FP, _FP]),
    "orc_render_passes": (None, [_VP, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _UP, _FP, _FP]),
    # the oracle library's own copy of the synthetic scene generator
    "wpbr_scenegen_create": (C.c_int, [C.c_uint32] * 6 + [C.POINTER(_VP)]),
    "wpbr_scenegen_desc": (C.POINTER(A.SceneDesc), [_VP]),
    "wpbr_scenegen_ray_count": (C.c_uint64, [_VP]),
    "wpbr_scenegen_rays": (_FP, [_VP]),
    "wpbr_scenegen_destroy": (None, [_VP]),
    "orc_fresnel_dielectric": (C.c_float, [C.c_float] * 3),
    "orc_fresnel_conductor": (C.c_float, [C.c_float] * 4),
    "orc_tr_d": (C.c_float, [C.c_float] * 5),
    "orc_power_heuristic": (C.c_float, [C.c_float] * 2),
    "orc_mitchell": (C.c_float, [C.c_float]),
    "orc_left_shift3": (C.c_uint32, [C.c_uint32]),
    "orc_roughness_to_alpha": (C.c_float, [C.c_float]),
    "orc_sample2d": (None, [C.c_uint32] * 7 + [_FP]),
    "orc_sample1d": (C.c_float, [C.c_uint32] * 7),
    "orc_philox": (None, [_UP, _UP, _UP]),
    "orc_fmath": (None, [C.c_int, _FP, _FP, _FP, C.c_uint64]),
    "orc_fmath_d": (None, [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_uint64]),
    "orc_render_spectral": (None, [_VP, C.c_uint32, C.c_uint32, C.c_uint32, _FP, _FP]),
    "orc_spectral_tables": (None, [_FP]),
    "orc_texture_level": (C.c_uint32, [C.c_void_p, C.c_uint32, _FP, _UP]),
    "orc_texture_eval": (None, [C.c_void_p, _FP, C.c_uint32, _FP]),
    "orc_adjoint_eval": (C.c_double, [_VP, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_double),
                                      C.POINTER(C.c_double), _FP, C.POINTER(C.c_double), C.c_uint32, _UP,
                                      C.POINTER(C.c_double)]),
    "orc_adjoint_fd": (None, [_VP, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_double),
                              C.POINTER(C.c_double), _FP, C.c_uint32, _UP, C.c_double, C.POINTER(C.c_double)]),
}
_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle() if not os.path.exists(OUT) else OUT
        L = C.CDLL(path)
        for k, (r, a) in _SIGS.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def _fp(a):
    return a.ctypes.data_as(_FP) if a is not None else None


def _up(a):
    return a.ctypes.data_as(_UP) if a is not None else None


class SceneGen:
    """The seeded synthetic scenes and rays, generated by the oracle library's
    copy of the scene generator (the same source and flags as the product's),
    so a CPU-only process never loads the product library."""

    def __init__(self, config, seed=0, res=(256, 256), level=0, rays=False):
        self._h = _VP()
        st = lib().wpbr_scenegen_create(config, seed, res[0], res[1], level, 1 if rays else 0, C.byref(self._h))
        if st != 0:
            raise RuntimeError("scenegen_create(config=%d) failed with status %d" % (config, st))

    @property
    def desc(self):
        return lib().wpbr_scenegen_desc(self._h)

    def rays(self):
        n = lib().wpbr_scenegen_ray_count(self._h)
        if n == 0:
            return np.zeros((0, 8), np.float32)
        p = lib().wpbr_scenegen_rays(self._h)
        return np.ctypeslib.as_array(p, shape=(n * 8,)).reshape(n, 8).copy()

    def close(self):
        if self._h:
            lib().wpbr_scenegen_destroy(self._h)
            self._h = _VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OracleScene:
    def __init__(self, desc, quirks=0):
        self._h = lib().orc_scene_create(desc, quirks)

    def close(self):
        if self._h:
            lib().orc_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sizes(self):
        s = np.zeros(4, np.uint32)
        lib().orc_bvh_sizes(self._h, _up(s))
        return dict(n_prims=int(s[0]), n_nodes=int(s[1]), n_treelets=int(s[2]), max_depth=int(s[3]))

    def bvh_export(self):
        z = self.sizes()
        N, M, T = z["n_prims"], z["n_nodes"], z["n_treelets"]
        r = dict(prim_bounds=np.zeros(N * 6, np.float32), centroids=np.zeros(N * 3, np.float32),
                 cbounds=np.zeros(6, np.float32), codes=np.zeros(N, np.uint32), sorted_codes=np.zeros(N, np.uint32),
                 sorted_prims=np.zeros(N, np.uint32), treelet_start=np.zeros(max(T, 1), np.uint32),
                 nodes=np.zeros(M * 3, np.uint32), node_bounds=np.zeros(M * 6, np.float32),
                 shapes=np.zeros(N, np.uint32))
        lib().orc_bvh_export(self._h, _fp(r["prim_bounds"]), _fp(r["centroids"]), _fp(r["cbounds"]), _up(r["codes"]),
                             _up(r["sorted_codes"]), _up(r["sorted_prims"]), _up(r["treelet_start"]),
                             _up(r["nodes"]), _fp(r["node_bounds"]), _up(r["shapes"]))
        r["treelet_start"] = r["treelet_start"][:T]
        r.update(z)
        return r

    def trace(self, rays, mode=1, stats=False):
        """mode 0 faithful (prune-free candidate list), 1 pruned closest, 2 any-hit."""
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = rays.shape[0]
        hits = np.zeros((n, 4), np.float32)
        st = np.zeros((n, 2), np.uint32) if stats else None
        lib().orc_trace(self._h, _fp(rays), n, mode, _fp(hits), _up(st))
        return (hits, st) if stats else hits

    def camera(self):
        rc = np.zeros(16, np.float32)
        dx = np.zeros(3, np.float32)
        dy = np.zeros(3, np.float32)
        lib().orc_camera(self._h, _fp(rc), _fp(dx), _fp(dy))
        return rc.reshape(4, 4), dx, dy

    def env_distribution(self, W, H):
        cc = np.zeros(H * (W + 1), np.float32)
        ci = np.zeros(H, np.float32)
        mc = np.zeros(H + 1, np.float32)
        mi = np.zeros(1, np.float32)
        lib().orc_env_distribution(self._h, _fp(cc), _fp(ci), _fp(mc), _fp(mi))
        return cc, ci, mc, mi

    def render_pass(self, p, spp, seed, stream, rect, fields=None):
        x0, y0, x1, y1 = rect
        rec, arrays = A.make_record((x1 - x0) * (y1 - y0), fields)
        lib().orc_render_pass(self._h, p, spp, seed, stream, x0, y0, x1, y1, C.byref(rec))
        return arrays

    def adjoint_fd(self, spp, seed, stream, mat, env, target, sel, h=1e-3):
        """FP64 central differences (step h) of the frozen estimator's loss
        at the parameter indices `sel`."""
        dp = C.POINTER(C.c_double)
        mat = np.ascontiguousarray(mat, np.float64)
        env = np.ascontiguousarray(env if env is not None else np.zeros(0), np.float64)
        tgt = np.ascontiguousarray(target, np.float32)
        sel_a = np.ascontiguousarray(sel, np.uint32)
        fd = np.zeros(len(sel_a), np.float64)
        lib().orc_adjoint_fd(self._h, spp, seed, stream, mat.ctypes.data_as(dp), env.ctypes.data_as(dp), _fp(tgt),
                             len(sel_a), _up(sel_a), h, fd.ctypes.data_as(dp))
        return fd

    def adjoint_eval(self, W, H, spp, seed, stream, mat, env, target=None, sel=None, image=False):
        """FP64 frozen-direction estimator at parameters (mat, env): returns
        (loss, image or None, gradient at the indices `sel` or None)."""
        dp = C.POINTER(C.c_double)
        mat = np.ascontiguousarray(mat, np.float64)
        env = np.ascontiguousarray(env if env is not None else np.zeros(0), np.float64)
        tgt = np.ascontiguousarray(target, np.float32) if target is not None else None
        img = np.zeros(W * H * 3, np.float64) if image else None
        sel_a = np.ascontiguousarray(sel, np.uint32) if sel is not None else np.zeros(0, np.uint32)
        g = np.zeros(len(sel_a), np.float64)
        loss = lib().orc_adjoint_eval(self._h, spp, seed, stream, mat.ctypes.data_as(dp), env.ctypes.data_as(dp),
                                      _fp(tgt), img.ctypes.data_as(dp) if img is not None else None, len(sel_a),
                                      _up(sel_a), g.ctypes.data_as(dp))
        return loss, (img.reshape(H, W, 3) if img is not None else None), (g if sel is not None else None)

    def render_spectral(self, W, H, spp, seed=0, stream=0):
        L = np.zeros(W * H * 3, np.float32)
        w = np.zeros(W * H, np.float32)
        lib().orc_render_spectral(self._h, spp, seed, stream, _fp(L), _fp(w))
        return L.reshape(H, W, 3), w.reshape(H, W)

    def render(self, W, H, spp, seed=0, stream=0):
        L = np.zeros(W * H * 3, np.float32)
        w = np.zeros(W * H, np.float32)
        lib().orc_render(self._h, spp, seed, stream, _fp(L), _fp(w))
        return L.reshape(H, W, 3), w.reshape(H, W)

    def render_passes(self, W, H, spp, passes, seed=0, stream=0):
        """Film of the listed passes of an spp-pass render, accumulated in order."""
        p = np.ascontiguousarray(passes, np.uint32)
        L = np.zeros(W * H * 3, np.float32)
        w = np.zeros(W * H, np.float32)
        lib().orc_render_passes(self._h, spp, seed, stream, p.size, _up(p), _fp(L), _fp(w))
        return L.reshape(H, W, 3), w.reshape(H, W)


def spectral_tables():
    t = np.zeros(17 * 64, np.float32)
    lib().orc_spectral_tables(_fp(t))
    return t.reshape(17, 64)


def _texture(rgb):
    """A wpbr_texture over an (h, w, 3) float32 array (kept alive by the caller)."""
    h, w, _ = rgb.shape
    return A.Texture(w, h, rgb.ctypes.data_as(_FP))


def texture_levels(rgb):
    """The MIP pyramid the oracle builds for an (h, w, 3) texture: a list of
    (h_l, w_l, 3) arrays, level 0 first."""
    rgb = np.ascontiguousarray(rgb, np.float32)
    t = _texture(rgb)
    n = lib().orc_texture_level(C.byref(t), 0, None, None)
    out = []
    for lvl in range(n):
        wh = np.zeros(2, np.uint32)
        buf = np.zeros(rgb.size, np.float32)
        lib().orc_texture_level(C.byref(t), lvl, _fp(buf), _up(wh))
        out.append(buf[: wh[0] * wh[1] * 3].reshape(wh[1], wh[0], 3))
    return out


def texture_eval(rgb, fp, isotropic=False):
    """Anisotropic EWA (or, with isotropic, trilinear) lookup of an (h, w, 3)
    texture at the footprint fp = (s, t, ds/dx, dt/dx, ds/dy, dt/dy)."""
    rgb = np.ascontiguousarray(rgb, np.float32)
    t = _texture(rgb)
    f = np.asarray(fp, np.float32)
    o = np.zeros(3, np.float32)
    lib().orc_texture_eval(C.byref(t), _fp(f), 1 if isotropic else 0, _fp(o))
    return o


def philox(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib().orc_philox(_up(c), _up(k), _up(o))
    return o


FM = dict(sin=0, cos=1, atan2=2, acos=3, exp=4, log=5, tan=6)


def fmath(name, x, y=None):
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y if y is not None else np.zeros_like(x), np.float32)
    o = np.zeros_like(x)
    lib().orc_fmath(FM[name], _fp(x), _fp(y), _fp(o), x.size)
    return o


def fmath_d(name, x):
    x = np.ascontiguousarray(x, np.float64)
    o = np.zeros_like(x)
    dp = C.POINTER(C.c_double)
    lib().orc_fmath_d(0 if name == "sin" else 1, x.ctypes.data_as(dp), o.ctypes.data_as(dp), x.size)
    return o


def sample2d(seed, stream, spp, pixel, p, dim, arrays=0):
    u = np.zeros(2, np.float32)
    lib().orc_sample2d(seed, stream, spp, pixel, p, dim, arrays, _fp(u))
    return u


def sample1d(seed, stream, spp, pixel, p, dim, arrays=0):
    return lib().orc_sample1d(seed, stream, spp, pixel, p, dim, arrays)
