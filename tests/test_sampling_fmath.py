"""Shared definitions the GPU pipeline and the oracle both compile:
Philox-4x32-10 streams (published known-answer vectors) and the portable
elementary functions (error bounds against libm in double precision)."""
import numpy as np
import pytest


def test_philox_known_answers(O):
    # Random123 kat_vectors for philox4x32_10
    assert list(O.philox([0, 0, 0, 0], [0, 0])) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert list(O.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert list(O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_streams_are_stratified(O):
    spp = 16
    for pixel in (0, 7, 12345):
        cells = set()
        for p in range(spp):
            u = O.sample2d(0, 0, spp, pixel, p, 2)
            assert 0.0 <= u[0] < 1.0 and 0.0 <= u[1] < 1.0
            cells.add((int(u[0] * 4), int(u[1] * 4)))
        assert len(cells) == spp
        strata = {int(O.sample1d(0, 0, spp, pixel, p, 1) * spp) for p in range(spp)}
        assert strata == set(range(spp))


def test_reference_sample_arrays(O):
    # WPBR_Q_REF_SAMPLER_ARRAYS: reading every position of a pixel's arrays
    # returns each element of the reference's fill exactly once
    # (CSSamplerStratified.cpp:28-39, 68-87 with the sizes of CSFilm.cpp:22-23)
    inv1, inv2 = np.float32(1.0 / 80), np.float32(1.0 / 272)
    for pixel in (0, 5, 99999):
        v1 = np.array([O.sample1d(7, 0, 64, pixel, p, 1, arrays=1) for p in range(80)], np.float32)
        strata = np.floor(v1 * 80).astype(int)
        assert sorted(strata) == list(range(80))           # one value per stratum
        assert not np.array_equal(strata, np.arange(80))   # shuffled
        # element s = (s + u) * float(1/80): u recovered in [0, 1)
        u = v1 / inv1 - strata
        assert (u >= -1e-4).all() and (u < 1 + 1e-4).all()
        # 2D: pass p reads positions 3p (camera, dim 0), 3p+1 (light, 2), 3p+2 (BSDF, 3)
        pairs = []
        for p in range(91):
            for dim in (0, 2, 3):
                if len(pairs) < 272:
                    pairs.append(O.sample2d(7, 0, 64, pixel, p, dim, arrays=1))
        pairs = np.array(pairs, np.float32)
        assert (pairs < 1.0 / 17 + 1e-7).all()             # the 1/data.size() scale
        zeros = np.all(pairs == 0, axis=1)
        assert zeros.sum() == 16                           # 272 - 16*16 never-written pairs
        cells = {(int(np.floor(a / inv2)), int(np.floor(b / inv2))) for a, b in pairs[~zeros]}
        assert cells == {(i, j) for i in range(16) for j in range(16)}
        # positions wrap after the array (pass 91 reads position 273 = 1)
        assert np.array_equal(O.sample2d(7, 0, 64, pixel, 91, 0, arrays=1), pairs[1])
    # off by default
    assert O.sample1d(7, 0, 64, 3, 0, 1) != O.sample1d(7, 0, 64, 3, 0, 1, arrays=1)


def _ulp(ref32):
    r = np.abs(ref32.astype(np.float32))
    return (np.nextafter(r, np.float32(np.inf)) - r).astype(np.float64)


@pytest.mark.parametrize("name,lo,hi,bound", [
    ("sin", -20, 20, 3), ("cos", -20, 20, 3), ("exp", -80, 80, 3), ("tan", -1.5, 1.5, 6)])
def test_fmath_unary(O, name, lo, hi, bound):
    rng = np.random.default_rng(1)
    x = rng.uniform(lo, hi, 200000).astype(np.float32)
    got = O.fmath(name, x).astype(np.float64)
    ref = getattr(np, name)(x.astype(np.float64))
    err = np.abs(got - ref) / _ulp(ref)
    assert err.max() <= bound, (name, err.max())


def test_fmath_atan2_acos_log(O):
    rng = np.random.default_rng(2)
    y = rng.uniform(-5, 5, 200000).astype(np.float32)
    x = rng.uniform(-5, 5, 200000).astype(np.float32)
    got = O.fmath("atan2", y, x).astype(np.float64)
    ref = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    assert (np.abs(got - ref) / _ulp(ref)).max() <= 3
    z = rng.uniform(-1, 1, 200000).astype(np.float32)
    ref = np.arccos(z.astype(np.float64))
    assert (np.abs(O.fmath("acos", z) - ref) / _ulp(ref)).max() <= 3
    l = np.exp(rng.uniform(-80, 80, 200000)).astype(np.float32)
    ref = np.log(l.astype(np.float64))
    assert (np.abs(O.fmath("log", l) - ref) / _ulp(ref)).max() <= 3
    # C-library conventions on signed zeros and out-of-domain input
    sp = O.fmath("atan2", np.array([0.0, -0.0, 0.0], np.float32), np.array([-0.0, -0.0, 0.0], np.float32))
    assert sp[0] == np.float32(np.pi) and sp[1] == -np.float32(np.pi) and sp[2] == 0.0
    assert np.isnan(O.fmath("acos", np.array([1.0000001], np.float32)))[0]


def test_fmath_double_sin(O):
    x = np.random.default_rng(3).uniform(-8, 8, 100000)
    for name, f in (("sin", np.sin), ("cos", np.cos)):
        got = O.fmath_d(name, x)
        ref = f(x)
        ulp = np.spacing(np.abs(ref))
        assert (np.abs(got - ref) / ulp).max() <= 4
