"""libclbm_refshim.a: a program written against the reference's own function
signatures (tests/refshim_harness.cpp: the reference drivers' step sequence
and a spatial-force collision, geometry in the program's globals, host
arrays) linked with the shim instead of the reference's LBM objects gives the
reference's results bit for bit (the golden fixtures recorded from the
reference itself)."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = Path(__file__).resolve().parent
GOLD = HERE / "golden"


@pytest.fixture(scope="module")
def harness(gpu, clbm_lib, tmp_path_factory):
    import build as b
    lib = b.build_shim()
    exe = tmp_path_factory.mktemp("shim") / "refshim_harness"
    cuda = b.CUDA_HOME
    r = subprocess.run([b.CXX, "-std=c++17", "-O2", "-o", str(exe), str(HERE / "refshim_harness.cpp"), str(lib),
                        f"-L{b.BUILD}", "-lclbm", f"-Wl,-rpath,{b.BUILD}", f"-L{cuda / 'lib64'}", "-lcudart",
                        f"-Wl,-rpath,{cuda / 'lib64'}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("i", range(4))
def test_reference_signatures_through_the_shim(harness, tmp_path, i):
    z = np.load(GOLD / "steps.npz")
    nx, ny, x0, x1, y0, y1, tau, beta, _ = z["cases"][i]
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([nx, ny, x0, x1, y0, y1], np.int32).tofile(f)
        np.array([tau, beta, 0.3]).tofile(f)
        z[f"case{i}_f0"].astype(np.float64).tofile(f)
        z[f"case{i}_map"].astype(np.float64).tofile(f)
    r = subprocess.run([str(harness), str(inp), str(out)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    N, n = 9 * int(nx) * int(ny), int(nx) * int(ny)
    o = np.fromfile(out)
    assert o.size == N + 5 + 2 * N + 3 * n
    assert np.array_equal(o[:N], z[f"case{i}_f5"])
    assert np.array_equal(o[N:N + 5], z[f"case{i}_drag"])
    q = N + 5
    assert np.array_equal(o[q:q + N], z[f"case{i}_sp_fin"])
    assert np.array_equal(o[q + N:q + 2 * N], z[f"case{i}_sp_fout"])
    assert np.array_equal(o[q + 2 * N:].reshape(3, n), z[f"case{i}_sp_macro"])
