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


@pytest.mark.parametrize("n", [1, 2047, 2049, 16384, 16385, 1 << 20])
@pytest.mark.parametrize("bits", [24, 30])
def test_noalloc_sort_edge_sizes(W, n, bits):
    # partial last tiles (2047, 2049, 16385), exactly one scan tile of block
    # histograms (16384 keys: 8 blocks x 256 digits = 2048 counters), a single
    # key, and the capacity itself (512 blocks, 64 scan tiles), each against
    # numpy's stable argsort of the low `bits` bits; two calls in a row
    torch = pytest.importorskip("torch")
    L = W.lib()
    rng = np.random.default_rng(n * 31 + bits)
    codes_h = rng.integers(0, 1 << 30, n, dtype=np.uint32)
    codes_h[: n // 3] &= 0xFFF  # many equal low digits: stability matters
    perm_ref = np.argsort(codes_h & np.uint32((1 << bits) - 1), kind="stable").astype(np.uint32)
    codes = torch.from_numpy(codes_h.view(np.int32)).to("cuda")
    out_k = torch.full_like(codes, -1)
    out_p = torch.full_like(codes, -1)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        st = L.wpbr_sort_morton_noalloc(C.c_void_p(codes.data_ptr()), n, bits, C.c_void_p(out_k.data_ptr()),
                                        C.c_void_p(out_p.data_ptr()), C.c_void_p(stream))
        assert st == W.OK, L.wpbr_sort_morton_noalloc_error()
        torch.cuda.synchronize()
        assert np.array_equal(out_p.cpu().numpy().view(np.uint32), perm_ref), (n, bits, call)
        assert np.array_equal(out_k.cpu().numpy().view(np.uint32), codes_h[perm_ref]), (n, bits, call)


def test_noalloc_sort_rejects_oversize(W):
    L = W.lib()
    big = W.SORT_NOALLOC_MAX_KEYS + 1
    st = L.wpbr_sort_morton_noalloc(C.c_void_p(16), big, 24, C.c_void_p(32), C.c_void_p(48), None)
    assert st == W.ERR_INVALID_ARG
    assert b"capacity" in L.wpbr_sort_morton_noalloc_error()
