"""The adapters' dictionary reading, on the CPU: foam's fvSolution entry
syntax with the coupled solvers' nested preconditioner dictionary (the
tutorials' Tcoupled entry), flat entries, comments, and malformed input
(FatalError)."""
import json
import subprocess

import pytest

from test_gpu_adapter import TCOUPLED


@pytest.fixture(scope="module")
def exe():
    from multiregionfoam_gb300 import _build
    _build.build()
    return _build.build_adapter()


def read(exe, tmp_path, text, entry):
    f = tmp_path / "fvSolution"
    f.write_text(text)
    r = subprocess.run([exe, "--print-dict", str(f), entry], capture_output=True, text=True, timeout=60)
    return r.returncode, json.loads(r.stdout.strip().splitlines()[-1])


def test_tcoupled_nested_preconditioner(exe, tmp_path):
    rc, d = read(exe, tmp_path, TCOUPLED, "Tcoupled")
    assert rc == 0, d
    assert d == {"solver": "BiCGStab", "preconditioner": "Cholesky", "nested": 1, "tolerance": 1e-15,
                 "relTol": 0.0, "minIter": 0.0, "maxIter": 200.0}


def test_flat_entry_and_comments(exe, tmp_path):
    text = """// solid region
    T
    {
        solver          gpuPCG;   /* the GPU drop-in */
        preconditioner  DIC;
        tolerance       1e-06;
        relTol          0.01;
    }
    """
    rc, d = read(exe, tmp_path, text, "T")
    assert rc == 0 and d["solver"] == "gpuPCG" and d["preconditioner"] == "DIC" and d["nested"] == 0
    assert d["tolerance"] == 1e-6 and d["relTol"] == 0.01 and d["maxIter"] == -1.0


@pytest.mark.parametrize("text", ["T { solver gpuPCG }", "T { solver gpuPCG; ", "T { solver gpuPCG; } }"])
def test_malformed_is_fatal(exe, tmp_path, text):
    rc, d = read(exe, tmp_path, text, "T")
    assert rc == 1 and "dictionary" in d["error"]
