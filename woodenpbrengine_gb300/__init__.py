"""GB300 wavefront implementation of WoodenPBREngine's per-sample ray pipeline.

Python binding of the C ABI in include/wpbr_gpu.h (libwpbr_gpu.so, built
in-tree by woodenpbrengine_gb300.build). The library is the product; this
module only marshals numpy arrays through ctypes. There is no CPU fallback:
without the built library the import of `lib()` raises, and without a CUDA
device the context constructor raises.
"""
import ctypes as C
import os

import numpy as np

from . import _abi as A

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libwpbr_gpu.so")

OK, ERR_INVALID_ARG, ERR_OOM, ERR_CUDA, ERR_TRAVERSAL_LIMIT, ERR_NOT_BUILT, ERR_NO_DEVICE = range(7)
TRACE_CLOSEST, TRACE_ANY = 0, 1
TRAVERSAL_BINARY, TRAVERSAL_BINARY_FULL_LEAVES = 0, 2
SPECTRUM_RGB, SPECTRUM_SAMPLED64 = 0, 1
Q_XYZ_MATRIX_FIX = 32
Q_REF_SAMPLER_ARRAYS = 64
Q_TRI_PERMUTATION_BUG, Q_ENV_LI_SAMPLE_FIX, Q_SPHERE_PDF_FIX, Q_ENV_DISTRIB_INDEX_BUG, Q_FULL_MORTON_SORT = (
    1, 2, 4, 8, 16)
MAT_CONDUCTOR, MAT_DIELECTRIC, MAT_SPECULAR = 0, 1, 2
LIGHT_SPHERE, LIGHT_ENV = 0, 1

JOBS = [
    "CAMERA_RAYS", "COLLIDE_PRIMARY", "EMITTED_LIGHT", "BSDF_SETUP", "SAMPLE_LIGHT", "SHADOW_LIGHT",
    "BSDF_COMPUTE", "INTEGRATE_LIGHT", "SAMPLE_BSDF", "SHADOW_BSDF", "LIGHT_COMPUTE", "INTEGRATE_BSDF",
    "FILM_ACCUMULATE",
]
JOB = {name: i for i, name in enumerate(JOBS)}

# exported symbols and their ctypes signatures (restype, argtypes)
_VP = C.c_void_p
_FP = C.POINTER(C.c_float)
_UP = C.POINTER(C.c_uint32)
_SIGS = {
    "wpbr_version": (C.c_char_p, []),
    "wpbr_create": (C.c_int, [C.c_int, C.POINTER(_VP)]),
    "wpbr_destroy": (None, [_VP]),
    "wpbr_last_error": (C.c_char_p, [_VP]),
    "wpbr_set_stream": (C.c_int, [_VP, _VP]),
    "wpbr_get_stream": (_VP, [_VP]),
    "wpbr_set_quirks": (C.c_int, [_VP, C.c_uint32]),
    "wpbr_synchronize": (C.c_int, [_VP]),
    "wpbr_set_traversal": (C.c_int, [_VP, C.c_uint32]),
    "wpbr_set_spectrum": (C.c_int, [_VP, C.c_uint32]),
    "wpbr_set_ray_sort": (C.c_int, [_VP, C.c_uint32]),
    "wpbr_check_device_errors": (C.c_int, [_VP]),
    "wpbr_scene_upload": (C.c_int, [_VP, C.POINTER(A.SceneDesc)]),
    "wpbr_camera_info": (C.c_int, [_VP, _FP, _FP, _FP]),
    "wpbr_env_distribution": (C.c_int, [_VP, _FP, _FP, _FP, _FP]),
    "wpbr_camera_setup": (C.c_int, [C.POINTER(A.Camera), _FP, _FP, _FP]),
    "wpbr_bvh_build": (C.c_int, [_VP]),
    "wpbr_bvh_info": (C.c_int, [_VP, _UP]),
    "wpbr_bvh_export": (C.c_int, [_VP, _FP, _FP, _FP, _UP, _UP, _UP, _UP, _UP, _FP, _UP]),
    "wpbr_collide": (C.c_int, [_VP, _FP, C.c_uint64, _FP, C.c_uint32]),
    "wpbr_collide_device": (C.c_int, [_VP, _VP, C.c_uint64, _VP, C.c_uint32]),
    "wpbr_collide_stats": (C.c_int, [_VP, _FP, C.c_uint64, _FP, _UP, C.c_uint32]),
    "wpbr_collide_launches": (C.c_int, [_VP, C.c_uint64, _UP]),
    "wpbr_set_kernel_timing": (C.c_int, [_VP, C.c_uint32]),
    "wpbr_kernel_timing": (C.c_int, [_VP, C.POINTER(C.c_float), _UP]),
    "wpbr_render_setup": (C.c_int, [_VP, C.c_uint32, C.c_uint32, C.c_uint32]),
    "wpbr_render_pass": (C.c_int, [_VP, C.c_uint32]),
    "wpbr_render": (C.c_int, [_VP]),
    "wpbr_film_read": (C.c_int, [_VP, _FP, _FP]),
    "wpbr_film_tonemap": (C.c_int, [_VP, C.POINTER(C.c_uint8)]),
    "wpbr_job_run": (C.c_int, [_VP, C.c_uint32, C.c_uint32]),
    "wpbr_job_record": (C.c_int, [_VP, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(A.PassRecord)]),
    "wpbr_scenegen_create": (C.c_int, [C.c_uint32] * 6 + [C.POINTER(_VP)]),
    "wpbr_scenegen_desc": (C.POINTER(A.SceneDesc), [_VP]),
    "wpbr_scenegen_ray_count": (C.c_uint64, [_VP]),
    "wpbr_scenegen_rays": (_FP, [_VP]),
    "wpbr_scenegen_destroy": (None, [_VP]),
    "wpbr_sort_morton_noalloc": (C.c_int, [_VP, C.c_uint32, C.c_uint32, _VP, _VP, _VP]),
    "wpbr_sort_morton_noalloc_error": (C.c_char_p, []),
    "wpbr_adjoint_setup": (C.c_int, [_VP, C.c_uint32, C.c_uint32, C.c_uint32]),
    "wpbr_adjoint_param_counts": (C.c_int, [_VP, _UP, _UP]),
    "wpbr_adjoint_get_params": (C.c_int, [_VP, _FP, _FP]),
    "wpbr_adjoint_set_params": (C.c_int, [_VP, _FP, _FP]),
    "wpbr_adjoint_set_params_device": (C.c_int, [_VP, _VP, _VP]),
    "wpbr_adjoint_freeze": (C.c_int, [_VP]),
    "wpbr_adjoint_forward": (C.c_int, [_VP, _FP, _FP, C.POINTER(C.c_double)]),
    "wpbr_adjoint_forward_device": (C.c_int, [_VP, _VP, _VP, C.POINTER(C.c_double)]),
    "wpbr_adjoint_backward": (C.c_int, [_VP, _FP, _FP]),
    "wpbr_adjoint_backward_device": (C.c_int, [_VP, _VP, _VP]),
    "wpbr_batch_create": (C.c_int, [C.c_int, C.POINTER(_VP)]),
    "wpbr_batch_destroy": (None, [_VP]),
    "wpbr_batch_last_error": (C.c_char_p, [_VP]),
    "wpbr_batch_add_scene": (C.c_int, [_VP, C.POINTER(A.SceneDesc), C.c_uint32, _UP]),
    "wpbr_batch_build": (C.c_int, [_VP]),
    "wpbr_batch_render_setup": (C.c_int, [_VP, C.c_uint32, C.c_uint32, C.c_uint32]),
    "wpbr_batch_autotune": (C.c_int, [_VP, C.c_int]),
    "wpbr_batch_set_rays_per_block": (C.c_int, [_VP, C.c_uint32]),
    "wpbr_batch_render_pass": (C.c_int, [_VP, C.c_uint32]),
    "wpbr_batch_render": (C.c_int, [_VP]),
    "wpbr_batch_synchronize": (C.c_int, [_VP]),
    "wpbr_batch_info_get": (C.c_int, [_VP, C.POINTER(A.BatchInfo)]),
    "wpbr_batch_film_size": (C.c_int, [_VP, C.c_uint32, _UP, _UP]),
    "wpbr_batch_film_read": (C.c_int, [_VP, C.c_uint32, _FP, _FP]),
    "wpbr_batch_set_stream": (C.c_int, [_VP, _VP]),
    "wpbr_batch_check_device_errors": (C.c_int, [_VP]),
    "wpbr_set_traversal_limits": (C.c_int, [_VP, C.c_uint32, C.c_uint32]),
    "wpbr_debug_fail_allocations": (None, [C.c_int64]),
    "wpbr_debug_ray_order": (C.c_int, [_VP, _FP, C.c_uint64, _UP, _UP]),
}
SORT_NOALLOC_MAX_KEYS = 1 << 20
EXPORTED = sorted(_SIGS)

_lib = None


class WpbrError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("wpbr status %d: %s" % (status, msg))
        self.status = status


def lib():
    """Load libwpbr_gpu.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libwpbr_gpu.so is not built; run woodenpbrengine_gb300.build.build_library()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _fp(a):
    return a.ctypes.data_as(_FP) if a is not None else None


def _up(a):
    return a.ctypes.data_as(_UP) if a is not None else None


def debug_fail_allocations(n):
    """Testing aid: the library's next n device allocations succeed, later ones
    fail as out-of-memory; n < 0 disables the injection."""
    lib().wpbr_debug_fail_allocations(n)


class SceneGen:
    """Seeded synthetic scene (host-only; see csrc/scene_gen.cpp)."""

    def __init__(self, config, seed=0, res=(256, 256), level=0, rays=False):
        self._h = _VP()
        st = lib().wpbr_scenegen_create(config, seed, res[0], res[1], level, 1 if rays else 0, C.byref(self._h))
        if st != OK:
            raise WpbrError(st, "scenegen_create(config=%d)" % config)
        self.config = config

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


class Context:
    """One wpbr_ctx (one GPU). Thin, checked wrappers over the C ABI."""

    def __init__(self, device=0):
        self._h = _VP()
        st = lib().wpbr_create(device, C.byref(self._h))
        if st != OK:
            raise WpbrError(st, "wpbr_create(device=%d) failed" % device)

    def _check(self, st, what):
        if st != OK:
            raise WpbrError(st, "%s: %s" % (what, lib().wpbr_last_error(self._h).decode()))

    def close(self):
        if self._h:
            lib().wpbr_destroy(self._h)
            self._h = _VP()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr):
        self._check(lib().wpbr_set_stream(self._h, stream_ptr), "set_stream")

    def set_quirks(self, q):
        self._check(lib().wpbr_set_quirks(self._h, q), "set_quirks")

    def set_traversal(self, mode):
        self._check(lib().wpbr_set_traversal(self._h, mode), "set_traversal")

    def set_ray_sort(self, bits_per_axis):
        """Origin-grid bits per axis for reordering large collide batches (0: input order)."""
        self._check(lib().wpbr_set_ray_sort(self._h, int(bits_per_axis)), "set_ray_sort")

    def set_spectrum(self, mode):
        self._check(lib().wpbr_set_spectrum(self._h, mode), "set_spectrum")

    def synchronize(self):
        self._check(lib().wpbr_synchronize(self._h), "synchronize")

    def check_device_errors(self):
        self._check(lib().wpbr_check_device_errors(self._h), "device errors")

    def upload(self, desc):
        self._check(lib().wpbr_scene_upload(self._h, desc), "scene_upload")

    def camera_info(self):
        rc = np.zeros(16, np.float32)
        dx = np.zeros(3, np.float32)
        dy = np.zeros(3, np.float32)
        self._check(lib().wpbr_camera_info(self._h, _fp(rc), _fp(dx), _fp(dy)), "camera_info")
        return rc.reshape(4, 4), dx, dy

    def env_distribution(self, W, H):
        cc = np.zeros(H * (W + 1), np.float32)
        ci = np.zeros(H, np.float32)
        mc = np.zeros(H + 1, np.float32)
        mi = np.zeros(1, np.float32)
        self._check(lib().wpbr_env_distribution(self._h, _fp(cc), _fp(ci), _fp(mc), _fp(mi)), "env_distribution")
        return cc, ci, mc, mi

    def build(self):
        self._check(lib().wpbr_bvh_build(self._h), "bvh_build")

    def bvh_info(self):
        out = np.zeros(4, np.uint32)
        self._check(lib().wpbr_bvh_info(self._h, _up(out)), "bvh_info")
        return dict(n_prims=int(out[0]), n_nodes=int(out[1]), n_treelets=int(out[2]), max_depth=int(out[3]))

    def bvh_export(self):
        info = self.bvh_info()
        N, M, T = info["n_prims"], info["n_nodes"], info["n_treelets"]
        r = dict(prim_bounds=np.zeros(N * 6, np.float32), centroids=np.zeros(N * 3, np.float32),
                 cbounds=np.zeros(6, np.float32), codes=np.zeros(N, np.uint32), sorted_codes=np.zeros(N, np.uint32),
                 sorted_prims=np.zeros(N, np.uint32), treelet_start=np.zeros(max(T, 1), np.uint32),
                 nodes=np.zeros(M * 3, np.uint32), node_bounds=np.zeros(M * 6, np.float32),
                 shapes=np.zeros(N, np.uint32))
        self._check(lib().wpbr_bvh_export(
            self._h, _fp(r["prim_bounds"]), _fp(r["centroids"]), _fp(r["cbounds"]), _up(r["codes"]),
            _up(r["sorted_codes"]), _up(r["sorted_prims"]), _up(r["treelet_start"]), _up(r["nodes"]),
            _fp(r["node_bounds"]), _up(r["shapes"])), "bvh_export")
        r["treelet_start"] = r["treelet_start"][:T]
        r.update(info)
        return r

    def collide(self, rays, mode=TRACE_CLOSEST, stats=False):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = rays.shape[0]
        hits = np.zeros((n, 4), np.float32)
        if stats:
            st = np.zeros((n, 2), np.uint32)
            self._check(lib().wpbr_collide_stats(self._h, _fp(rays), n, _fp(hits), _up(st), mode), "collide_stats")
            return hits, st
        self._check(lib().wpbr_collide(self._h, _fp(rays), n, _fp(hits), mode), "collide")
        return hits

    def set_traversal_limits(self, max_stack_entries=0, max_loop_steps=0):
        """Testing aid: lower the traversal's stack / loop bounds (0: default)."""
        self._check(lib().wpbr_set_traversal_limits(self._h, max_stack_entries, max_loop_steps),
                    "set_traversal_limits")

    def collide_launches(self, n):
        """Kernels one collide_device call of n rays launches."""
        c = C.c_uint32()
        self._check(lib().wpbr_collide_launches(self._h, n, C.byref(c)), "collide_launches")
        return c.value

    def set_kernel_timing(self, enable):
        self._check(lib().wpbr_set_kernel_timing(self._h, 1 if enable else 0), "set_kernel_timing")

    def kernel_timing(self):
        """(summed ms, launches) of the traversal launches timed since the last read."""
        ms, c = C.c_float(), C.c_uint32()
        self._check(lib().wpbr_kernel_timing(self._h, C.byref(ms), C.byref(c)), "kernel_timing")
        return ms.value, c.value

    def debug_ray_order(self, rays):
        """(keys in input order, trace order) of a sorted collide of rays (n, 8)."""
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        keys = np.zeros(n, np.uint32)
        perm = np.zeros(n, np.uint32)
        self._check(lib().wpbr_debug_ray_order(self._h, _fp(rays), n, _up(keys), _up(perm)), "debug_ray_order")
        return keys, perm

    def collide_device(self, d_rays, n, d_hits, mode=TRACE_CLOSEST):
        self._check(lib().wpbr_collide_device(self._h, d_rays, n, d_hits, mode), "collide_device")

    def render_setup(self, spp, seed=0, stream=0):
        self._check(lib().wpbr_render_setup(self._h, spp, seed, stream), "render_setup")

    def render_pass(self, p):
        self._check(lib().wpbr_render_pass(self._h, p), "render_pass")

    def render(self):
        self._check(lib().wpbr_render(self._h), "render")

    def film(self, W, H):
        L = np.zeros(W * H * 3, np.float32)
        w = np.zeros(W * H, np.float32)
        self._check(lib().wpbr_film_read(self._h, _fp(L), _fp(w)), "film_read")
        return L.reshape(H, W, 3), w.reshape(H, W)

    def tonemap(self, W, H):
        out = np.zeros(W * H * 3, np.uint8)
        self._check(lib().wpbr_film_tonemap(self._h, out.ctypes.data_as(C.POINTER(C.c_uint8))), "tonemap")
        return out.reshape(H, W, 3)

    def job(self, name, p):
        self._check(lib().wpbr_job_run(self._h, JOB[name], p), "job " + name)

    def record(self, x0, y0, x1, y1, fields=None):
        rec, arrays = A.make_record((x1 - x0) * (y1 - y0), fields)
        self._check(lib().wpbr_job_record(self._h, x0, y0, x1, y1, C.byref(rec)), "job_record")
        return arrays

    # ---- differentiable estimator (wpbr_adjoint_*) ----
    def adjoint_setup(self, spp, seed=0, stream=0):
        self._check(lib().wpbr_adjoint_setup(self._h, spp, seed, stream), "adjoint_setup")
        nm, ne = C.c_uint32(), C.c_uint32()
        self._check(lib().wpbr_adjoint_param_counts(self._h, C.byref(nm), C.byref(ne)), "adjoint_param_counts")
        self._adj_counts = (nm.value, ne.value)
        return self._adj_counts

    def adjoint_params(self):
        nm, ne = self._adj_counts
        m = np.zeros(nm, np.float32)
        e = np.zeros(ne, np.float32)
        self._check(lib().wpbr_adjoint_get_params(self._h, _fp(m), _fp(e) if ne else None), "adjoint_get_params")
        return m, e

    def adjoint_set_params(self, mat=None, env=None):
        m = np.ascontiguousarray(mat, np.float32) if mat is not None else None
        e = np.ascontiguousarray(env, np.float32) if env is not None else None
        self._check(lib().wpbr_adjoint_set_params(self._h, _fp(m), _fp(e)), "adjoint_set_params")

    def adjoint_set_params_device(self, d_mat=None, d_env=None):
        self._check(lib().wpbr_adjoint_set_params_device(self._h, d_mat, d_env), "adjoint_set_params_device")

    def adjoint_freeze(self):
        self._check(lib().wpbr_adjoint_freeze(self._h), "adjoint_freeze")

    def adjoint_forward(self, W, H, target=None):
        """Returns (image (H, W, 3), loss or None)."""
        img = np.zeros(W * H * 3, np.float32)
        t = np.ascontiguousarray(target, np.float32).reshape(-1) if target is not None else None
        loss = C.c_double(0.0)
        self._check(lib().wpbr_adjoint_forward(self._h, _fp(t), _fp(img), C.byref(loss)), "adjoint_forward")
        return img.reshape(H, W, 3), (loss.value if target is not None else None)

    def adjoint_forward_device(self, d_target, d_image=None):
        loss = C.c_double(0.0)
        self._check(lib().wpbr_adjoint_forward_device(self._h, d_target, d_image, C.byref(loss)),
                    "adjoint_forward_device")
        return loss.value

    def adjoint_backward(self):
        """Returns (material gradient (n_mat_params,), environment gradient (n_env_params,))."""
        nm, ne = self._adj_counts
        gm = np.zeros(nm, np.float32)
        ge = np.zeros(ne, np.float32)
        self._check(lib().wpbr_adjoint_backward(self._h, _fp(gm), _fp(ge) if ne else None), "adjoint_backward")
        return gm, ge

    def adjoint_backward_device(self, d_grad_mat, d_grad_env):
        self._check(lib().wpbr_adjoint_backward_device(self._h, d_grad_mat, d_grad_env), "adjoint_backward_device")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many scenes rendered together (wpbr_batch_*): pooled traversal arena,
    one CUDA graph per sample pass, autotuned traversal queue depth."""

    def __init__(self, device=0):
        self._h = _VP()
        st = lib().wpbr_batch_create(device, C.byref(self._h))
        if st != OK:
            raise WpbrError(st, "batch_create(device=%d)" % device)
        self._keep = []

    def _check(self, st, what):
        if st != OK:
            raise WpbrError(st, "%s: %s" % (what, lib().wpbr_batch_last_error(self._h).decode()))

    def add(self, desc, quirks=0):
        idx = C.c_uint32()
        self._check(lib().wpbr_batch_add_scene(self._h, desc, quirks, C.byref(idx)), "batch_add_scene")
        return idx.value

    def build(self):
        self._check(lib().wpbr_batch_build(self._h), "batch_build")

    def render_setup(self, spp, seed=0, first_stream=0):
        self._check(lib().wpbr_batch_render_setup(self._h, spp, seed, first_stream), "batch_render_setup")

    def autotune(self, use_cache=True):
        self._check(lib().wpbr_batch_autotune(self._h, 1 if use_cache else 0), "batch_autotune")
        return self.info()

    def set_rays_per_block(self, rpb):
        self._check(lib().wpbr_batch_set_rays_per_block(self._h, rpb), "batch_set_rays_per_block")

    def render_pass(self, p):
        self._check(lib().wpbr_batch_render_pass(self._h, p), "batch_render_pass")

    def render(self):
        self._check(lib().wpbr_batch_render(self._h), "batch_render")

    def synchronize(self):
        self._check(lib().wpbr_batch_synchronize(self._h), "batch_synchronize")

    def set_stream(self, stream_ptr):
        self._check(lib().wpbr_batch_set_stream(self._h, stream_ptr), "batch_set_stream")

    def check_device_errors(self):
        self._check(lib().wpbr_batch_check_device_errors(self._h), "batch_check_device_errors")

    def info(self):
        bi = A.BatchInfo()
        self._check(lib().wpbr_batch_info_get(self._h, C.byref(bi)), "batch_info")
        return {f: getattr(bi, f) for f, _ in A.BatchInfo._fields_}

    def film_size(self, k):
        w, h = C.c_uint32(), C.c_uint32()
        self._check(lib().wpbr_batch_film_size(self._h, k, C.byref(w), C.byref(h)), "batch_film_size")
        return w.value, h.value

    def film(self, k):
        W, H = self.film_size(k)
        L = np.zeros(W * H * 3, np.float32)
        w = np.zeros(W * H, np.float32)
        self._check(lib().wpbr_batch_film_read(self._h, k, _fp(L), _fp(w)), "batch_film_read")
        return L.reshape(H, W, 3), w.reshape(H, W)

    def close(self):
        if self._h:
            lib().wpbr_batch_destroy(self._h)
            self._h = _VP()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def camera_setup(camera):
    """A1 on the host: (raster_camera 4x4, dxCamera, dyCamera) for a wpbr_camera."""
    rc = np.zeros(16, np.float32)
    dx = np.zeros(3, np.float32)
    dy = np.zeros(3, np.float32)
    st = lib().wpbr_camera_setup(C.byref(camera), _fp(rc), _fp(dx), _fp(dy))
    if st != OK:
        raise WpbrError(st, "camera_setup")
    return rc.reshape(4, 4), dx, dy


def device_available():
    """True when a CUDA device answers (no exception when there is none)."""
    try:
        c = Context(0)
    except (WpbrError, ImportError, OSError):
        return False
    c.close()
    return True
