"""Block-coupled systems as scalar LDU systems (mrg_block_addressing /
mrg_block_coeffs, host-only): the library's expansion equals the oracle's
entry-by-entry restatement exactly, is in upper-triangular face order, and
its scalar product equals the block product; bad sizes and addressing are
rejected.  No GPU needed.
"""
import numpy as np
import pytest

from multiregionfoam_gb300.cases import block_case


@pytest.fixture(scope="module")
def bo():
    import block_oracle
    return block_oracle


@pytest.mark.parametrize("bs,symmetric", [(4, False), (4, True), (3, False), (1, False)])
def test_expansion_matches_oracle(mrg, bo, bs, symmetric):
    c = block_case(5, 4, 3, bs=bs, seed=bs + 10 * symmetric, symmetric=symmetric)
    n_s, s_lo, s_up, s_d, s_uc, s_lc = mrg.block_system(c["n"], c["lower"], c["upper"], bs, c["D"], c["U"], c["L"])
    o_lo, o_up, o_d, o_uc, o_lc = bo.expand(c["n"], c["lower"], c["upper"], bs, c["D"], c["U"], c["L"])
    assert n_s == bs * c["n"]
    assert len(s_lo) == bs * bs * len(c["lower"]) + c["n"] * bs * (bs - 1) // 2
    for got, want in ((s_lo, o_lo), (s_up, o_up)):
        assert np.array_equal(got, want)
    for got, want in ((s_d, o_d), (s_uc, o_uc), (s_lc, o_lc)):
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    # upper-triangular order: owner ascending, neighbour ascending within it
    key = s_lo.astype(np.int64) * n_s + s_up
    assert np.all(s_lo < s_up) and np.all(np.diff(key) > 0)
    if symmetric:
        assert np.array_equal(s_uc, s_lc)


def test_expansion_preserves_amul(mrg, bo):
    c = block_case(6, 5, 4, bs=4, seed=3)
    n, bs = c["n"], 4
    n_s, s_lo, s_up, s_d, s_uc, s_lc = mrg.block_system(n, c["lower"], c["upper"], bs, c["D"], c["U"], c["L"])
    x = np.random.default_rng(0).uniform(-1, 1, (n, bs))
    yb = bo.block_amul(n, c["lower"], c["upper"], c["D"], c["U"], c["L"], x).ravel()
    ys = bo.scalar_amul(n_s, s_lo, s_up, s_d, s_uc, s_lc, x.ravel())
    assert np.allclose(ys, yb, rtol=1e-13, atol=1e-13)


def test_bs1_is_the_scalar_system(mrg):
    c = block_case(4, 4, 4, bs=1, seed=5)
    n_s, s_lo, s_up, s_d, s_uc, s_lc = mrg.block_system(c["n"], c["lower"], c["upper"], 1, c["D"], c["U"], c["L"])
    order = np.lexsort((c["upper"], c["lower"]))
    assert np.array_equal(s_lo, c["lower"][order]) and np.array_equal(s_up, c["upper"][order])
    assert np.array_equal(s_uc, c["U"].ravel()[order]) and np.array_equal(s_lc, c["L"].ravel()[order])


@pytest.mark.parametrize("bs", [0, 9])
def test_bad_block_size(mrg, bs):
    c = block_case(3, 3, 3, bs=2, seed=1)
    with pytest.raises(mrg.MrgError, match="block size"):
        mrg.block_system(c["n"], c["lower"], c["upper"], bs, np.zeros((c["n"], 1)), np.zeros((len(c["lower"]), 1)))


def test_bad_addressing(mrg):
    c = block_case(3, 3, 3, bs=2, seed=1)
    lo = c["lower"].copy()
    lo[0] = c["upper"][0]   # lower == upper: not an internal face
    with pytest.raises(mrg.MrgError, match="block addressing"):
        mrg.block_system(c["n"], lo, c["upper"], 2, c["D"], c["U"], c["L"])


def test_unordered_block_faces(mrg):
    """Block faces out of upper-triangular order are rejected, as for the
    scalar mesh upload (foam's lduAddressing is always in that order)."""
    c = block_case(5, 4, 3, bs=3, seed=8)
    perm = np.random.default_rng(1).permutation(len(c["lower"]))
    with pytest.raises(mrg.MrgError, match="upper-triangular"):
        mrg.block_system(c["n"], c["lower"][perm], c["upper"][perm], 3, c["D"], c["U"][perm], c["L"][perm])


def test_block_preconditioner_oracle_exact_on_chain(bo):
    """The restated block factorisation (oracle/block_oracle.py) is an exact
    LU on a block tridiagonal matrix (a chain of cells: no fill-in to drop),
    and for a symmetric block matrix M^-1 is symmetric."""
    n, bs = 12, 4
    rng = np.random.default_rng(3)
    lower = np.arange(n - 1, dtype=np.int32)
    upper = lower + 1
    U = rng.uniform(-1, 1, (n - 1, bs, bs))
    L = rng.uniform(-1, 1, (n - 1, bs, bs))
    D = rng.uniform(-0.3, 0.3, (n, bs, bs)) + np.eye(bs) * 10.0
    dD = bo.block_factor(n, lower, upper, D, U, L)
    r = rng.standard_normal((n, bs))
    w = bo.block_apply(n, lower, upper, D, U, L, dD, r)
    assert np.abs(bo.block_amul(n, lower, upper, D, U, L, w) - r).max() < 1e-12
    c = block_case(4, 3, 3, bs=3, seed=8, symmetric=True)
    dD = bo.block_factor(c["n"], c["lower"], c["upper"], c["D"], c["U"], None)
    E = np.eye(c["n"] * 3)
    Minv = np.stack([bo.block_apply(c["n"], c["lower"], c["upper"], c["D"], c["U"], None, dD, e).ravel() for e in E])
    assert np.allclose(Minv, Minv.T, rtol=0, atol=1e-12)
