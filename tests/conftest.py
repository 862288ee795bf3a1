import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def mrg():
    """The product library (built in-tree); fails loudly without it."""
    from multiregionfoam_gb300 import _build, mrgpu
    _build.build()
    mrgpu.load()
    return mrgpu


@pytest.fixture(scope="session")
def ctx(mrg):
    c = mrg.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def fohp():
    return dict(np.load(os.path.join(GOLDEN, "flowOverHeatedPlate_ldu.npz")))


@pytest.fixture(scope="session")
def golden_small():
    return dict(np.load(os.path.join(GOLDEN, "oracle_small.npz")))


def golden_system(g, name):
    """Rebuild a golden system from its stored input arrays."""
    from multiregionfoam_gb300 import cases
    iface = None
    if f"{name}_iface_cells" in g:
        iface = {k: g[f"{name}_iface_{k}"] for k in ("cells", "bou", "ptr", "src", "w")}
        iface["int"] = None
    return cases.LduSystem(int(g[f"{name}_n"]), g[f"{name}_lower"], g[f"{name}_upper"], g[f"{name}_diag"],
                           g[f"{name}_upper_c"], g.get(f"{name}_lower_c"), g[f"{name}_b"], g[f"{name}_x0"],
                           iface, name=name)


def oracle_matrix(O, s):
    return O.OracleMatrix(s.n, s.lower, s.upper, s.diag, s.upper_c, s.lower_c, s.iface)


def gpu_mesh(mrg, ctx, s):
    m = mrg.Mesh(ctx, s.n, s.lower, s.upper, s.iface)
    f = s.iface
    m.upload(s.diag, s.upper_c, s.lower_c, None if f is None else f["bou"], None if f is None else f.get("int"))
    return m
