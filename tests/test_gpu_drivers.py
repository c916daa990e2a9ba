"""The drop-in executables on the GPU, checked at the file level: the
reference pops-perturb driver's labels.dat, rvalues.dat and every clone's
data_force.datout (golden fixtures recorded from the reference), an
emulated 2-rank run against the oracle, and the plain driver."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from driver_util import BUILD, stage_pops_run

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def drivers(gpu):
    import build as b
    b.build_drivers()
    return BUILD


@pytest.mark.parametrize("i", range(2))
def test_pops_driver_files_match_reference(drivers, orc, tmp_path, i):
    """Also --reconstruct: lineage files built from the driver's own labels.dat
    and slot files (what post_processing/reconstruction.cpp does) must equal
    the device-side reconstruction."""
    z = np.load(GOLD / "pops_driver.npz")
    L, Nc, U0, tau, alpha, eps, T, dT = z["params"][i]
    p = dict(L=int(L), Nc=int(Nc), U0=U0, tau=tau, alpha=alpha, eps=eps, T=T, dT=dT)
    stage_pops_run(orc, tmp_path, p)
    r = subprocess.run([str(drivers / "TLGK_LBM_POPS_PERTURB"), "--reconstruct", "input"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = tmp_path / "out"
    assert np.array_equal(np.fromfile(out / "labels.dat", np.int32), z[f"run{i}_labels"])
    np.testing.assert_allclose(np.fromfile(out / "rvalues.dat"), z[f"run{i}_rvalues"], rtol=1e-11)
    steps = orc.reference_scalars(int(L), U0, dT, T)["steps"]
    for j in range(int(Nc)):
        f = np.fromfile(out / f"clone_{j}" / "data_force.datout")
        g = z[f"run{i}_force"][j]
        assert f.shape == g.shape
        assert np.array_equal(f[:steps], g[:steps])
        assert np.abs(f - g).max() <= 1e-12 * np.abs(g).max()
    labels = np.fromfile(out / "labels.dat", np.int32).reshape(-1, int(Nc))
    nint = labels.shape[0]
    slots = [np.fromfile(out / f"clone_{j}" / "data_force.datout").reshape(nint, steps) for j in range(int(Nc))]
    for j in range(int(Nc)):
        slot, expect = j, []
        for t in range(nint - 1, -1, -1):
            expect.append(slots[slot][t])
            if t > 0:
                slot = labels[t - 1][slot]
        lin = np.fromfile(out / "reconstructed" / f"clone_{j}" / "data_force.datout")
        assert np.array_equal(lin, np.concatenate(expect[::-1]))


def test_pops_driver_two_ranks_matches_oracle(drivers, orc, tmp_path):
    p = dict(L=4, Nc=8, U0=0.05, tau=0.56, alpha=20.0, eps=0.02, T=1.5, dT=0.25)
    g, files = stage_pops_run(orc, tmp_path, p)
    r = subprocess.run([str(drivers / "TLGK_LBM_POPS_PERTURB"), "--ranks", "2", "input"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    sc = orc.reference_scalars(4, 0.05, 0.25, 1.5)
    # rank 0 reads names[4..7]... no: with p ranks clone j >= Nc/p reads name j - Nc/p,
    # clone j < Nc/p reads name Nc - Nc/p + j (the master serves the other ranks first)
    local = 4
    order = [(j - local) if j >= local else (8 - local + j) for j in range(8)]
    states = np.concatenate([files[k] for k in order])
    ref = orc.run_sampler(g, states, steps=sc["steps"], intervals=sc["intervals"], tau=0.56, beta=sc["beta"],
                          alpha=20.0, force_scale=sc["force_scale"], force_shift=1.775, dt=sc["dt"],
                          perturb_mode=1, eps=0.02, snaps=np.concatenate(files[:10]), ranks=2)
    assert np.array_equal(np.fromfile(tmp_path / "out" / "labels.dat", np.int32), ref["labels"].ravel())
    np.testing.assert_allclose(np.fromfile(tmp_path / "out" / "rvalues.dat"), ref["rvalues"], rtol=1e-11)


def test_plain_driver(drivers, orc, tmp_path):
    L, tau, Ma, t0 = 4, 0.6, 0.1, 40.0
    (tmp_path / "input_LBM.datin").write_text(f"{L} {tau} {Ma} {t0}\n")
    g = orc.reference_square_geom(L)
    f0 = orc.init_equilibrium(g, 0.03, 1e-2, 3, 0, 0)
    f0.tofile(tmp_path / "pops.datout")
    r = subprocess.run([str(drivers / "TLGK_LBM")], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    import math
    Dy = 4 * L + 1
    nu = 1.0 / 3.0 * (tau - 0.5)
    cs = 1.0 / math.sqrt(3)
    u0 = cs * cs * Ma
    beta0 = 8 * nu * u0 / ((Dy - 1) // 2) / ((Dy - 1) // 2)
    steps = math.floor(1 / (1.0 / t0))
    ref = orc.run_sampler(g, np.concatenate([f0, f0]), steps=steps, intervals=1, tau=tau, beta=beta0,
                          alpha=0.04, force_scale=1.0, force_shift=0.0, dt=1.0 / t0)
    assert np.array_equal(np.fromfile(tmp_path / "labels.dat", np.int32), ref["labels"].ravel())
    np.testing.assert_allclose(np.fromfile(tmp_path / "rvalues.dat"), ref["rvalues"], rtol=1e-13)


def test_bodyforce_warmup_and_snapshots(drivers, orc, tmp_path):
    """LBM_BODYFORCE (main_bodyforce.cpp) from the rest state: final
    populations, raw force every facquForce steps and the ux probe every
    facquU steps against the oracle; snapshot mode writes popfiles and
    popfiles_list.dat that TLGK_LBM_POPS_PERTURB reads."""
    L, steps, tau, Ma = 4, 30, 0.6, 0.15
    (tmp_path / "input.datin").write_text(f"1 {steps} {L} {tau} {Ma} run 0 10 3 5\n")
    r = subprocess.run([str(drivers / "LBM_BODYFORCE"), "--snapshots", "3", "--every", "5"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    import math
    g = orc.reference_square_geom(L)
    Dy = 4 * L + 1
    cs = 1.0 / math.sqrt(3)
    beta = 8 * (1.0 / 3 * (tau - 0.5)) * (cs * cs * Ma) / ((Dy - 1) // 2) / ((Dy - 1) // 2)
    f = np.tile(orc.W, Dy * Dy)
    force, ux = [], []
    for t in range(steps + 15):
        f_new, _, rho, uxf, uyf = orc.lbm_step(g, f, beta, tau)
        if t < steps and t % 5 == 0:
            ux.append(uxf[(Dy // 4) + Dy * (Dy // 4)])
        F = orc.force(g, f_new, 1.0 / tau)
        if t < steps and t % 3 == 0:
            force.append(F)
        f = f_new
        if t == steps - 1:
            assert np.array_equal(np.fromfile(tmp_path / "run" / "pops.datout"), f)
        if t >= steps and (t + 1 - steps) % 5 == 0:
            k = (t + 1 - steps) // 5 - 1
            assert np.array_equal(np.fromfile(tmp_path / "run" / f"pops_{k}.datout"), f)
    assert np.array_equal(np.fromfile(tmp_path / "run" / "data_force.datout"), np.array(force))
    assert np.array_equal(np.fromfile(tmp_path / "run" / "ux_t.datout"), np.array(ux))
    assert len(list((tmp_path / "run" / "vtk_fluid").glob("fluid_t*.vtk"))) == 3
    assert (tmp_path / "run" / "popfiles_list.dat").read_text().split() == [f"pops_{k}.datout" for k in range(3)]


def test_pops_driver_fp32_first_interval(drivers, orc, tmp_path):
    """--fp32 (the driver autotunes the interval kernel): the first interval's
    force series of every clone within 1e-5 of the reference driver's (the
    genealogy may differ later, FP32 rounding can flip a resampling draw)."""
    z = np.load(GOLD / "pops_driver.npz")
    L, Nc, U0, tau, alpha, eps, T, dT = z["params"][0]
    p = dict(L=int(L), Nc=int(Nc), U0=U0, tau=tau, alpha=alpha, eps=eps, T=T, dT=dT)
    stage_pops_run(orc, tmp_path, p)
    r = subprocess.run([str(drivers / "TLGK_LBM_POPS_PERTURB"), "--fp32", "input"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    steps = orc.reference_scalars(int(L), U0, dT, T)["steps"]
    for j in range(int(Nc)):
        f = np.fromfile(tmp_path / "out" / f"clone_{j}" / "data_force.datout")[:steps]
        g = z["run0_force"][j][:steps]
        assert np.abs(f - g).max() <= 1e-5 * np.abs(g).max()
