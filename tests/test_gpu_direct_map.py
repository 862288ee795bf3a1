"""directMap on the device (mrg_direct_map_build): the conformal face map by
face-centre match, against the oracle's literal N^2 restatement of
directMapInterfaceToInterfaceMapping.C:147-190, on the reference's tutorial
interface (flowOverHeatedPlate, 200 faces) and on a permuted, shifted
conformal grid; the transfer to[i] = from[map[i]] through mrg_ggi_apply; and
the "not conformal" errors."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _map_of(g):
    ptr, addr, w = g.csr()
    assert np.array_equal(ptr, np.arange(g.n_dst + 1)) and np.all(w == 1.0)
    return addr


def test_tutorial_interface(mrg, ctx, oracle_mod, fohp):
    tol = 1e-3 * min(float(fohp["solid_iface_min_edge"]), float(fohp["fluid_iface_min_edge"]))
    ca, cb = fohp["solid_iface_centres"], fohp["fluid_iface_centres"]
    a_from_b, b_from_a = mrg.Ggi.direct_map(ctx, ca, cb, tol)
    try:
        assert np.array_equal(_map_of(a_from_b), oracle_mod.direct_map(ca, cb, tol))
        assert np.array_equal(_map_of(b_from_a), oracle_mod.direct_map(cb, ca, tol))
        # the transfer of a face field, and the reference's self-check: face
        # centres mapped across are the other side's centres
        f = np.random.default_rng(1).uniform(-1.0, 1.0, len(ca))
        assert np.array_equal(b_from_a.apply(f), f[oracle_mod.direct_map(cb, ca, tol)])
        xyz = np.ascontiguousarray(ca, np.float64).reshape(-1, 3)
        mapped = np.stack([b_from_a.apply(xyz[:, k].copy()) for k in range(3)], axis=1)
        assert np.abs(mapped - np.asarray(cb).reshape(-1, 3)).max() < tol
    finally:
        a_from_b.close()
        b_from_a.close()


def test_permuted_grid_and_first_match(mrg, ctx, oracle_mod):
    rng = np.random.default_rng(4)
    X, Y = np.meshgrid(np.arange(64) + 0.5, np.arange(48) + 0.5, indexing="xy")
    ca = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1)
    perm = rng.permutation(len(ca))
    cb = ca[perm] + rng.uniform(-1e-5, 1e-5, ca.shape)      # conformal up to round-off
    tol = 1e-3 * 1.0
    a_from_b, b_from_a = mrg.Ggi.direct_map(ctx, ca, cb, tol)
    try:
        m = _map_of(a_from_b)
        assert np.array_equal(m, oracle_mod.direct_map(ca, cb, tol))
        assert np.array_equal(cb[m] - ca < 1.0, np.ones_like(ca, bool))
        assert np.array_equal(_map_of(b_from_a), perm)
    finally:
        a_from_b.close()
        b_from_a.close()
    # two candidates within the tolerance: the first in face order wins
    cb2 = np.array([[0.0, 0, 0], [0.0, 0, 0], [1.0, 0, 0]])
    ca2 = np.array([[0.0, 0, 0], [1.0, 0, 0], [0.0, 0, 1e-9]])
    g1, g2 = mrg.Ggi.direct_map(ctx, ca2, cb2, 1e-6)
    try:
        assert _map_of(g1).tolist() == oracle_mod.direct_map(ca2, cb2, 1e-6).tolist() == [0, 2, 0]
    finally:
        g1.close()
        g2.close()


def test_not_conformal(mrg, ctx):
    a = np.array([[0.0, 0, 0], [1.0, 0, 0]])
    with pytest.raises(mrg.MrgError, match="not conformal"):
        mrg.Ggi.direct_map(ctx, a, np.array([[0.0, 0, 0], [0.5, 0, 0]]), 1e-3)
    with pytest.raises(mrg.MrgError, match="not conformal"):
        mrg.Ggi.direct_map(ctx, a, np.array([[0.0, 0, 0]]), 1e-3)
