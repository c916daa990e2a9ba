"""Build libclbm.so (sm_103a) and the drop-in driver executables in-tree.

    python cloning-lbm-mpi_gb300/build.py            # library + drivers
    python cloning-lbm-mpi_gb300/build.py --lib-only

Every .cu translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a``; the objects are linked into
``cloning-lbm-mpi_gb300/_build/libclbm.so`` with the CUDA runtime linked
statically, so the library needs nothing but the NVIDIA driver at run time.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
DRIVERS = PKG / "drivers"
BUILD = PKG / "_build"
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUFLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
           "-I", str(REPO / "include")]
CXX = os.environ.get("CXX", "g++")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"build step failed: {cmd[0]} ... {cmd[-1]}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [REPO / "include" / "clbm.h"]
    sources = sorted(CSRC.glob("*.cu"))
    objs = []
    jobs = []
    for src in sources:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([NVCC, *ARCH, *CUFLAGS, "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    lib = BUILD / "libclbm.so"
    if _stale(lib, objs):
        _run([NVCC, *ARCH, "-shared", "-cudart", "static", "-o", str(lib), *map(str, objs)])
    if verbose:
        print(f"built {lib}")
    return lib


CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def build_shim(verbose: bool = False) -> Path:
    """libclbm_refshim.a: the reference's LBM and perturbation functions with
    their own C++ signatures over libclbm (shim/clbm_refshim.cpp).  A program
    links it as  libclbm_refshim.a -lclbm -lcudart  in place of the
    reference's LBM objects."""
    BUILD.mkdir(exist_ok=True)
    src = PKG / "shim" / "clbm_refshim.cpp"
    obj, lib = BUILD / "clbm_refshim.o", BUILD / "libclbm_refshim.a"
    if _stale(lib, [src, REPO / "include" / "clbm.h"]):
        _run([CXX, "-std=c++17", "-O2", "-fPIC", "-I", str(REPO / "include"), "-I", str(CUDA_HOME / "include"),
              "-c", str(src), "-o", str(obj)])
        if lib.exists():
            lib.unlink()
        _run(["ar", "rcs", str(lib), str(obj)])
    if verbose:
        print(f"built {lib}")
    return lib


DRIVER_VARIANTS = (("TLGK_LBM", "plain"), ("TLGK_LBM_POPS_PERTURB", "pops"),
                   ("TLGK_LBM_FORCING", "forcing"))


def build_drivers(verbose: bool = False) -> list[Path]:
    """The drop-in executables (TLGK_LBM, TLGK_LBM_POPS_PERTURB,
    TLGK_LBM_FORCING, LBM_BODYFORCE), C++ host code over libclbm's C ABI."""
    outs = []
    srcs = sorted(DRIVERS.glob("*.cpp"))
    if not srcs:
        return outs
    headers = list(DRIVERS.glob("*.h")) + [REPO / "include" / "clbm.h"]
    lib = BUILD / "libclbm.so"
    mains = {"tlgk_main", "lbm_bodyforce"}
    common = [s for s in srcs if s.stem not in mains]
    link = [f"-L{BUILD}", "-lclbm", "-Wl,-rpath,$ORIGIN", "-lm"]
    jobs = []
    targets = [(name, DRIVERS / "tlgk_main.cpp", [f"-DCLBM_VARIANT_{variant.upper()}"])
               for name, variant in DRIVER_VARIANTS]
    targets.append(("LBM_BODYFORCE", DRIVERS / "lbm_bodyforce.cpp", []))
    for name, main, defs in targets:
        exe = BUILD / name
        outs.append(exe)
        if _stale(exe, srcs + headers + [lib]):
            jobs.append([CXX, "-std=c++17", "-O2", *defs, "-I", str(REPO / "include"), "-o", str(exe),
                         str(main), *map(str, common), *link])
    with ThreadPoolExecutor(max_workers=4) as ex:
        list(ex.map(_run, jobs))
    if verbose:
        print("built drivers:", ", ".join(o.name for o in outs))
    return outs


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--lib-only", action="store_true")
    a = ap.parse_args()
    build_library(verbose=True)
    if not a.lib_only:
        build_drivers(verbose=True)
        build_shim(verbose=True)


if __name__ == "__main__":
    main()
