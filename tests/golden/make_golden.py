"""Regenerate the golden fixtures in tests/golden/ from the REFERENCE itself.

Needs the reference tree ($CLBM_REFERENCE_TREE, else a checkout named
"reference" beside this repository);
it compiles the reference's own objects and its pops-perturb driver in place
(oracle/Makefile -> oracle/_ref/) and records their outputs:

  steps.npz         5 LB steps + drag of random states on small channels
                    (reference functions, src/lbm_src/*.cpp), plus one
                    spatial-forcing collision (streamCollCompute.cpp:50-93)
  perturb.npz       generatePerturbedState on a random state, its drand48
                    prefactors drawn from the never-seeded stream
  pops_driver.npz   the reference pops-perturb driver (mpi_LBM_GK_pops_perturb
                    .cpp, single rank) on two small runs: labels.dat,
                    rvalues.dat and every clone's data_force.datout; the input
                    popfiles are regenerated from the oracle's deterministic
                    initial-state routine and pinned by a SHA-256.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent / "oracle"))
import oracle  # noqa: E402

STEP_CASES = [
    # nx, ny, xmin, xmax, ymin, ymax, tau, beta, seed
    (20, 12, 5, 9, 4, 8, 0.56, 3e-6, 1),
    (24, 10, 10, 13, 3, 6, 0.8, 1e-5, 2),
    (17, 17, 8, 12, 6, 10, 0.6, 5.5e-5, 3),
    (32, 16, 8, 16, 4, 12, 0.53, 2e-6, 4),
]

DRIVER_RUNS = [
    # L, Nc, U0, tau, alpha, eps, T, dT
    dict(L=4, Nc=4, U0=0.05, tau=0.6, alpha=8.0, eps=0.01, T=1.0, dT=0.25),
    dict(L=4, Nc=8, U0=0.05, tau=0.56, alpha=20.0, eps=0.02, T=1.5, dT=0.25),
]


def popfiles(g, n_files: int) -> list[np.ndarray]:
    return [oracle.init_equilibrium(g, 0.05, 2e-2, 7, 0, i) for i in range(n_files)]


def make_steps(R):
    out = {}
    for i, (nx, ny, x0, x1, y0, y1, tau, beta, seed) in enumerate(STEP_CASES):
        rng = np.random.default_rng(seed)
        f = (oracle.W[None, None, :] * (1 + 0.05 * rng.standard_normal((nx, ny, 9)))).ravel()
        R.ref_set_geom(nx, ny, x0, x1, y0, y1)
        st = f.copy()
        drag = np.empty(5)
        R.ref_run_clone(st.ctypes.data_as(C.c_void_p), 5, beta, tau, drag.ctypes.data_as(C.c_void_p))
        out[f"case{i}_f0"] = f
        out[f"case{i}_f5"] = st
        out[f"case{i}_drag"] = drag
        # one spatial-forcing collision with its macroscopic fields
        mp = rng.standard_normal(nx * ny)
        fin = f.copy()
        fout = np.empty_like(f)
        rho, ux, uy = np.empty(nx * ny), np.empty(nx * ny), np.empty(nx * ny)
        R.ref_stream_collide_spatial(*[a.ctypes.data_as(C.c_void_p) for a in (fin, fout, rho, ux, uy)],
                                     beta, mp.ctypes.data_as(C.c_void_p), tau, 0.3)
        out[f"case{i}_map"] = mp
        out[f"case{i}_sp_fin"] = fin
        out[f"case{i}_sp_fout"] = fout
        out[f"case{i}_sp_macro"] = np.stack([rho, ux, uy])
    out["cases"] = np.array(STEP_CASES, dtype=np.float64)
    np.savez_compressed(HERE / "steps.npz", **out)


def make_perturb(R):
    libc = C.CDLL("libc.so.6")
    rng = np.random.default_rng(11)
    n = 9 * 12 * 10
    f = (1 + 0.01 * rng.standard_normal(n)) / 9
    snaps = (1 + 0.01 * rng.standard_normal(10 * n)) / 9
    libc.seed48((C.c_ushort * 3)(0, 0, 0))  # the never-seeded state
    out = f.copy()
    R.ref_perturb(out.ctypes.data_as(C.c_void_p), snaps.ctypes.data_as(C.c_void_p), 10, n, 0.05)
    np.savez_compressed(HERE / "perturb.npz", f=f, snaps=snaps, eps=0.05, out=out)


def make_driver():
    out = {}
    for i, p in enumerate(DRIVER_RUNS):
        g = oracle.reference_square_geom(p["L"])
        files = popfiles(g, max(p["Nc"], 10))
        h = hashlib.sha256(b"".join(a.tobytes() for a in files)).hexdigest()
        wd = Path(tempfile.mkdtemp())
        try:
            (wd / "pops").mkdir()
            for j, a in enumerate(files):
                a.tofile(wd / "pops" / f"p{j}.bin")
            (wd / "pops" / "popfiles_list.dat").write_text("".join(f"p{j}.bin\n" for j in range(len(files))))
            (wd / "input").write_text(f"{p['Nc']}\n{p['T']}\n{p['dT']}\n{p['eps']}\n{p['L']}\n{p['tau']}\n"
                                      f"{p['U0']}\n{p['alpha']}\npops/\nout/\n1000000\n")
            r = subprocess.run([str(oracle.REF_DRIVER), "input"], cwd=wd, capture_output=True, text=True)
            assert r.returncode == 0, r.stderr
            out[f"run{i}_labels"] = np.fromfile(wd / "out" / "labels.dat", np.int32)
            out[f"run{i}_rvalues"] = np.fromfile(wd / "out" / "rvalues.dat")
            out[f"run{i}_force"] = np.stack([np.fromfile(wd / "out" / f"clone_{j}" / "data_force.datout")
                                             for j in range(p["Nc"])])
            out[f"run{i}_sha256"] = np.array(h)
        finally:
            shutil.rmtree(wd)
    out["params"] = np.array([[p["L"], p["Nc"], p["U0"], p["tau"], p["alpha"], p["eps"], p["T"], p["dT"]]
                              for p in DRIVER_RUNS])
    np.savez_compressed(HERE / "pops_driver.npz", **out)


def main():
    oracle.build()
    if not oracle.build_ref():
        sys.exit("reference tree not found; set CLBM_REFERENCE_TREE")
    R = oracle.ref()
    make_steps(R)
    make_perturb(R)
    make_driver()
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
