"""mrg_residual_noalloc: the foam residual without any device allocation.

Some callers cannot allocate device memory where they need a residual: code
inside a host application whose own allocator already holds the GPU's memory
(a caching pool, an MPS client under a hard limit), or monitoring code beside
asynchronous solves, where cudaMalloc / cudaFree would synchronise the
device.  mrg_residual_noalloc serves them from a fixed scratch array inside
the library.  These tests call it through the C ABI on matrices held in
device arrays in foam's lduAddressing (lowerAddr, upperAddr, ownerStartAddr,
losortAddr, losortStartAddr) and check it against mrg_residual, the entry
point that uploads the matrix into its own device memory, and against the
CPU oracle's foam-order residual, within the same 1e-12 relative tolerance
the other residual tests use -- on two calls in a row with different x, then
again on the first x, which must repeat the first call's result exactly
although the scratch keeps the previous call's contents.  Free device memory
is the same before and after those calls: the entry point allocates nothing.

The file is named to be collected last, so that it runs both after every
other test in one process and, alone, in a fresh one.
"""
import ctypes

import numpy as np
import pytest

from multiregionfoam_gb300 import cases

from conftest import GOLDEN, gpu_mesh, oracle_matrix

pytestmark = pytest.mark.gpu

REL = 1e-12
MAX_CELLS = 16_777_216   # the scratch array's limit


def _fohp():
    fx = dict(np.load(f"{GOLDEN}/flowOverHeatedPlate_ldu.npz"))
    return cases.flow_over_heated_plate(fx, form="global")


SYSTEMS = {
    "cht": lambda: cases.cht_system(16, 14, 12, 7, seed=1, form="global", k_range=(0.1, 50.0)),
    "cht-perm": lambda: cases.random_permute(
        cases.cht_system(13, 11, 9, 6, seed=3, form="global", k_range=(0.1, 50.0)), seed=4),
    "cd": lambda: cases.convdiff_system(14, 13, 12, seed=2),
    "fohp": _fohp,
    "c1": lambda: cases.c1(form="global"),
}


def lduaddressing(s):
    """ownerStartAddr, losortAddr, losortStartAddr of an upper-triangular LDU
    face list (foam's lduAddressing builds the same arrays)."""
    lower = np.asarray(s.lower, np.int64)
    upper = np.asarray(s.upper, np.int64)
    cells = np.arange(s.n + 1)
    owner_start = np.searchsorted(lower, cells, side="left")
    losort = np.argsort(upper, kind="stable")
    losort_start = np.searchsorted(upper[losort], cells, side="left")
    return [a.astype(np.int32) for a in (owner_start, losort, losort_start)]


class DeviceLdu:
    """The caller's own device arrays (allocated here by the caller, not by
    the entry point under test)."""

    def __init__(self, ctx, s):
        self.ctx = ctx
        owner_start, losort, losort_start = lduaddressing(s)
        arrays = dict(lower_addr=np.asarray(s.lower, np.int32), upper_addr=np.asarray(s.upper, np.int32),
                      owner_start=owner_start, losort=losort, losort_start=losort_start,
                      diag=s.diag, upper=s.upper_c, b=s.b)
        if s.lower_c is not None:
            arrays["lower"] = s.lower_c
        self.p = {k: ctx.to_device(np.ascontiguousarray(v)) for k, v in arrays.items()}
        self.p.setdefault("lower", None)
        self.x = ctx.dev_alloc(8 * s.n)
        self.n, self.nf = s.n, s.nf

    def residual(self, mrg, x, n_cells=None):
        buf = np.ascontiguousarray(x, np.float64)
        mrg._check(mrg.load().mrg_dev_copy(self.ctx.h, ctypes.c_void_p(self.x), buf.ctypes.data_as(ctypes.c_void_p),
                                           buf.nbytes, 0))
        p = self.p
        return mrg.residual_noalloc(self.n if n_cells is None else n_cells, self.nf, p["lower_addr"],
                                    p["upper_addr"], p["owner_start"], p["losort"], p["losort_start"],
                                    p["diag"], p["upper"], p["lower"], p["b"], self.x)

    def close(self):
        for v in list(self.p.values()) + [self.x]:
            if v is not None:
                self.ctx.dev_free(v)


def _close(a, b):
    return abs(a - b) <= REL * abs(b)


def free_device_bytes(mrg):
    """cudaMemGetInfo's free bytes on the current device (the CUDA runtime
    libmrgpu is linked against)."""
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert mrg.load().cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_noalloc_matches_residual(mrg, ctx, oracle_mod, name):
    s = SYSTEMS[name]()
    assert s.iface is None
    x1 = s.x0
    x2 = x1 + 0.25 * np.random.default_rng(11).standard_normal(s.n)
    m = gpu_mesh(mrg, ctx, s)
    want = [m.residual(s.b, x) for x in (x1, x2)]
    m.close()
    A = oracle_matrix(oracle_mod, s)
    foam = [(A.residual(s.b, x), A.norm_factor(x, s.b)) for x in (x1, x2)]
    d = DeviceLdu(ctx, s)
    try:
        d.residual(mrg, x2)                 # warm: device code loaded, scratch holds a previous result
        free0 = free_device_bytes(mrg)
        got1 = d.residual(mrg, x1)
        got2 = d.residual(mrg, x2)
        again = d.residual(mrg, x1)
        free1 = free_device_bytes(mrg)
    finally:
        d.close()
    assert free1 == free0, (free0, free1)
    for (r, nf), (rw, nfw), (ro, nfo) in zip((got1, got2), want, foam):
        assert _close(nf, nfw), (nf, nfw)
        assert _close(r, rw), (r, rw)
        assert _close(nf, nfo), (nf, nfo)
        assert _close(r, ro), (r, ro)
    assert got1 != got2
    assert again == got1


def test_noalloc_rejects_oversize_and_bad_addressing(mrg, ctx):
    s = SYSTEMS["cht"]()
    d = DeviceLdu(ctx, s)
    try:
        # beyond the scratch: refused on the host before anything is queued
        # (the size is checked before the arrays, so NULL arrays suffice)
        with pytest.raises(mrg.MrgError) as e:
            mrg.residual_noalloc(MAX_CELLS + 1, 3 * MAX_CELLS, *[0] * 10)
        assert e.value.code == 1 and str(MAX_CELLS) in str(e.value)
        with pytest.raises(mrg.MrgError):
            mrg.residual_noalloc(0, 0, *[0] * 10)
        # a losortAddr entry past the last face: the kernel checks every
        # index before it reads through it, skips it and reports it
        bad = lduaddressing(s)[1].copy()
        bad[len(bad) // 2] = s.nf + 5
        ctx.dev_free(d.p["losort"])
        d.p["losort"] = ctx.to_device(bad)
        with pytest.raises(mrg.MrgError) as e:
            d.residual(mrg, s.x0)
        assert e.value.code == 1 and "addressing" in str(e.value)
        # the next call starts from a cleared error word
        d.p["losort"], good = ctx.to_device(lduaddressing(s)[1]), d.p["losort"]
        ctx.dev_free(good)
        r, nf = d.residual(mrg, s.x0)
        assert np.isfinite(r) and nf > 0
        # faces out of upper-triangular order (two neighbours of one owner
        # swapped): the summation order foam's Amul gives is undefined, so
        # the call is refused; valid addressing works again afterwards
        upper = np.asarray(s.upper, np.int32).copy()
        lower = np.asarray(s.lower, np.int32)
        f = int(np.flatnonzero((lower[:-1] == lower[1:]) & (upper[:-1] < upper[1:]))[0])
        upper[f], upper[f + 1] = upper[f + 1], upper[f]
        good = d.p["upper_addr"]
        d.p["upper_addr"] = ctx.to_device(upper)
        with pytest.raises(mrg.MrgError) as e:
            d.residual(mrg, s.x0)
        assert e.value.code == 1 and "upper-triangular" in str(e.value)
        ctx.dev_free(d.p["upper_addr"])
        d.p["upper_addr"] = good
        assert d.residual(mrg, s.x0) == (r, nf)
    finally:
        d.close()
