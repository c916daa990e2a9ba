"""Link-level drop-in: the reference's own pops-perturb driver object
(compiled in place from the reference tree into oracle/_ref by
oracle/Makefile) links against libclbm_refshim.a + libclbm in place of the
reference's LBM and perturbation objects (streamCollCompute, domain_noSlipWalls,
square, force, generatePerturbedState), with only its I/O objects beside it.
Runs where the reference objects exist (this is a link check: running the
program needs a GPU, and the reference objects are host-architecture
builds)."""
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
REF = REPO / "oracle" / "_ref"


def test_reference_driver_links_against_the_shim(tmp_path):
    import build as b
    objs = [REF / "main_popsPerturb.o", REF / "initialize_lattice_arrays.o", REF / "write_vtk.o"]
    if not all(o.exists() for o in objs):
        pytest.skip("reference objects not built here (oracle/Makefile ref needs the reference tree)")
    b.build_library()
    lib = b.build_shim()
    exe = tmp_path / "TLGK_LBM_POPS_PERTURB_on_clbm"
    cuda = b.CUDA_HOME
    r = subprocess.run([b.CXX, "-o", str(exe), *map(str, objs), str(lib), f"-L{b.BUILD}", "-lclbm",
                        f"-L{cuda / 'lib64'}", "-lcudart", "-lm", "-Wl,--no-undefined"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    syms = subprocess.run(["nm", "-C", str(exe)], capture_output=True, text=True).stdout
    for f in ("streamingAndCollisionComputeMacroBodyForce", "computeDomainNoSlipWalls_BB",
              "computeSquareBounceBack_TEST", "computeForceOnSquare", "generatePerturbedState"):
        assert f in syms
