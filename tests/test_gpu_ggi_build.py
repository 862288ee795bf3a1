"""GGI weights built on the device (mrg_ggi_build) against the oracle's
construction: bit-identical CSR (pointers, source faces, weights) on jittered
non-conformal quads, triangles against quads, sliding (partly uncovered)
patches and the full-size 3:2 interface of the asymmetric configuration;
empty and disjoint patches; rejected faces."""
import numpy as np
import pytest

from test_oracle import jittered_faces

pytestmark = pytest.mark.gpu


def triangles(ptr, xy):
    """Each counter-clockwise quad split into two counter-clockwise triangles."""
    out = []
    for f in range(len(ptr) - 1):
        p = xy[ptr[f]:ptr[f + 1]]
        out += [p[0], p[1], p[2], p[0], p[2], p[3]]
    n = 2 * (len(ptr) - 1)
    return np.arange(0, 3 * n + 1, 3, dtype=np.int32), np.array(out)


def assert_same(mrg, ctx, oracle_mod, fa, fb, tol=1e-15):
    ga, gb = mrg.Ggi.build(ctx, *fa, *fb, tol=tol)
    try:
        ref = oracle_mod.ggi_weights(*fa, *fb, tol=tol)
        for g, (p, s, w) in zip((ga, gb), ref):
            dp, ds, dw = g.csr()
            np.testing.assert_array_equal(dp, p)
            np.testing.assert_array_equal(ds, s)
            assert dw.tobytes() == np.asarray(w, np.float64).tobytes()
        return ga, gb, ref
    except BaseException:
        ga.close()
        gb.close()
        raise


def test_ggi_build_jittered_32(mrg, ctx, oracle_mod):
    fa = jittered_faces(24, 24, 0.2, 1)
    fb = jittered_faces(16, 24, 0.2, 2)
    ga, gb, ref = assert_same(mrg, ctx, oracle_mod, fa, fb)
    # the device weights drive the device gather like uploaded ones
    src = np.random.default_rng(3).standard_normal(ga.n_src)
    np.testing.assert_array_equal(ga.apply(src), oracle_mod.ggi_apply(*ref[0], src, fused=True))
    np.testing.assert_allclose(gb.apply(np.full(gb.n_src, 7.0)), 7.0, rtol=1e-14)
    ga.close()
    gb.close()


def test_ggi_build_triangles(mrg, ctx, oracle_mod):
    fa = triangles(*jittered_faces(20, 20, 0.25, 5))
    fb = jittered_faces(13, 17, 0.2, 6)
    ga, gb, _ = assert_same(mrg, ctx, oracle_mod, fa, fb)
    ga.close()
    gb.close()


def test_ggi_build_sliding(mrg, ctx, oracle_mod):
    # B slid by 2.2 A faces: A's two left columns and B's right column are
    # uncovered (no weights), the faces next to them partly covered
    fa = jittered_faces(18, 12, 0.2, 7)
    pb, xb = jittered_faces(12, 12, 0.2, 8)
    xb = xb + np.array([2.2 / 18, 0.0])
    ga, gb, (wa, wb) = assert_same(mrg, ctx, oracle_mod, fa, (pb, xb))
    assert (np.diff(wa[0]) == 0).sum() == 2 * 12 and (np.diff(wb[0]) == 0).sum() == 12
    ga.close()
    gb.close()


def test_ggi_build_disjoint_and_empty(mrg, ctx, oracle_mod):
    fa = jittered_faces(6, 6, 0.1, 9)
    pb, xb = jittered_faces(4, 4, 0.1, 10)
    ga, gb, _ = assert_same(mrg, ctx, oracle_mod, fa, (pb, xb + 5.0))
    assert ga.csr()[0][-1] == 0 and gb.csr()[0][-1] == 0
    ga.close()
    gb.close()
    empty = (np.zeros(1, np.int32), np.zeros((0, 2)))
    ga, gb = mrg.Ggi.build(ctx, *fa, *empty)
    assert ga.n_dst == 36 and gb.n_dst == 0 and ga.csr()[0][-1] == 0
    ga.close()
    gb.close()


def test_ggi_build_rejects(mrg, ctx):
    fa = jittered_faces(4, 4, 0.1, 11)
    bad = (np.array([0, 2], np.int32), np.array([[0.0, 0.0], [1.0, 1.0]]))
    with pytest.raises(mrg.MrgError, match="3 to 32 vertices"):
        mrg.Ggi.build(ctx, *fa, *bad)
    t = np.linspace(0, 2 * np.pi, 41)[:-1]
    big = (np.array([0, 40], np.int32), np.stack([np.cos(t), np.sin(t)], 1))
    with pytest.raises(mrg.MrgError, match="3 to 32 vertices"):
        mrg.Ggi.build(ctx, *big, *fa)


def test_ggi_build_full_size_c3(mrg, ctx, oracle_mod):
    # the 96x96 : 64x96 interface of the asymmetric configuration (seed 0)
    fa = jittered_faces(96, 96, 0.2, 101)
    fb = jittered_faces(64, 96, 0.2, 102)
    ga, gb, _ = assert_same(mrg, ctx, oracle_mod, fa, fb)
    ga.close()
    gb.close()
