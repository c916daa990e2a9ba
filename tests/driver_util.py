"""Helpers to stage the reference's input files and popfiles for the
drop-in driver executables."""
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent.parent
BUILD = REPO / "cloning-lbm-mpi_gb300" / "_build"


def stage_pops_run(orc, wd: Path, p: dict, nfiles: int | None = None):
    """Writes popfiles (oracle initial states), popfiles_list.dat and the
    pops-layout input file; returns the list of states."""
    g = orc.reference_square_geom(int(p["L"]))
    nfiles = nfiles or max(int(p["Nc"]), 10)
    files = [orc.init_equilibrium(g, 0.05, 2e-2, 7, 0, j) for j in range(nfiles)]
    (wd / "pops").mkdir(parents=True, exist_ok=True)
    for j, a in enumerate(files):
        a.tofile(wd / "pops" / f"p{j}.bin")
    (wd / "pops" / "popfiles_list.dat").write_text("".join(f"p{j}.bin\n" for j in range(nfiles)))
    (wd / "input").write_text(f"{int(p['Nc'])}\n{p['T']}\n{p['dT']}\n{p['eps']}\n{int(p['L'])}\n"
                              f"{p['tau']}\n{p['U0']}\n{p['alpha']}\npops/\nout/\n1000000\n")
    return g, files
