"""The allocation-free Morton sort (wpbr_sort_morton_noalloc) against the
sort inside wpbr_bvh_build.

It exists for callers that cannot allocate device memory — hosts that own all
device memory through their own arena, loops that must not take cudaMalloc's
synchronisation — and keeps its temporaries in
a fixed file-scope device array. Two calls in a row must both reproduce the
build's sorted codes and permutation exactly (integer data: bit-exact), and a
size above the fixed capacity must be rejected. Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_sort_matches_build(W):
    torch = pytest.importorskip("torch")
    L = W.lib()
    for quirks, bits in ((0, 24), (W.Q_FULL_MORTON_SORT, 30)):
        g = W.SceneGen(1, 0, (8, 8), level=7)  # 327,680 triangles
        with W.Context(0) as ctx:
            ctx.set_quirks(quirks)
            ctx.upload(g.desc)
            ctx.build()
            e = ctx.bvh_export()
        n = e["n_prims"]
        codes = torch.from_numpy(e["codes"].view(np.int32)).to("cuda")
        out_k = torch.full_like(codes, -1)
        out_p = torch.full_like(codes, -1)
        stream = torch.cuda.current_stream().cuda_stream
        for call in range(2):
            st = L.wpbr_sort_morton_noalloc(C.c_void_p(codes.data_ptr()), n, bits, C.c_void_p(out_k.data_ptr()),
                                            C.c_void_p(out_p.data_ptr()), C.c_void_p(stream))
            assert st == W.OK, L.wpbr_sort_morton_noalloc_error()
            torch.cuda.synchronize()
            assert np.array_equal(out_k.cpu().numpy().view(np.uint32), e["sorted_codes"]), (bits, call)
            assert np.array_equal(out_p.cpu().numpy().view(np.uint32), e["sorted_prims"]), (bits, call)


def test_noalloc_sort_rejects_oversize(W):
    L = W.lib()
    big = W.SORT_NOALLOC_MAX_KEYS + 1
    st = L.wpbr_sort_morton_noalloc(C.c_void_p(16), big, 24, C.c_void_p(32), C.c_void_p(48), None)
    assert st == W.ERR_INVALID_ARG
    assert b"capacity" in L.wpbr_sort_morton_noalloc_error()
