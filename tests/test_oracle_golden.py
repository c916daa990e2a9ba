"""Pin the oracle against the reference: every committed fixture in
tests/golden/ was produced by the reference's own objects and driver
(tests/golden/make_golden.py); the oracle must reproduce each bit for bit.
Runs on any machine (the fixtures travel; the reference tree does not)."""
import ctypes as C
import hashlib
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def steps():
    return np.load(GOLD / "steps.npz")


@pytest.mark.parametrize("i", range(4))
def test_five_steps_and_drag(orc, steps, i):
    nx, ny, x0, x1, y0, y1, tau, beta, _ = steps["cases"][i]
    g = orc.Geom(int(nx), int(ny), int(x0), int(x1), int(y0), int(y1))
    st, drag = orc.run_clone(g, steps[f"case{i}_f0"], 5, beta, tau)
    assert np.array_equal(st, steps[f"case{i}_f5"])
    assert np.array_equal(drag, steps[f"case{i}_drag"])


@pytest.mark.parametrize("i", range(4))
def test_spatial_forcing_collision(orc, steps, i):
    nx, ny, x0, x1, y0, y1, tau, beta, _ = steps["cases"][i]
    g = orc.Geom(int(nx), int(ny), int(x0), int(x1), int(y0), int(y1))
    fin = steps[f"case{i}_f0"].copy()
    fout = np.empty_like(fin)
    n = g.nx * g.ny
    rho, ux, uy = np.empty(n), np.empty(n), np.empty(n)
    mp = steps[f"case{i}_map"]
    orc.lib().orc_stream_collide_spatial(C.byref(g), *[a.ctypes.data_as(C.c_void_p) for a in (fin, fout, rho, ux, uy)],
                                         C.c_double(beta), mp.ctypes.data_as(C.c_void_p), C.c_double(tau), C.c_double(0.3))
    assert np.array_equal(fin, steps[f"case{i}_sp_fin"])
    assert np.array_equal(fout, steps[f"case{i}_sp_fout"])
    assert np.array_equal(np.stack([rho, ux, uy]), steps[f"case{i}_sp_macro"])


def test_generate_perturbed_state(orc):
    z = np.load(GOLD / "perturb.npz")
    d = orc.D48()
    orc.lib().orc_drand48_init_default(C.byref(d))
    pre = np.array([orc.lib().orc_drand48_next(C.byref(d)) for _ in range(10)])
    out = orc.perturb_mix(z["f"], z["snaps"], float(z["eps"]), pre)
    assert np.array_equal(out, z["out"])


@pytest.mark.parametrize("i", range(2))
def test_pops_driver_run(orc, i):
    z = np.load(GOLD / "pops_driver.npz")
    L, Nc, U0, tau, alpha, eps, T, dT = z["params"][i]
    L, Nc = int(L), int(Nc)
    g = orc.reference_square_geom(L)
    files = [orc.init_equilibrium(g, 0.05, 2e-2, 7, 0, j) for j in range(max(Nc, 10))]
    assert hashlib.sha256(b"".join(a.tobytes() for a in files)).hexdigest() == str(z[f"run{i}_sha256"])
    sc = orc.reference_scalars(L, U0, dT, T)
    res = orc.run_sampler(g, np.concatenate(files[:Nc]), steps=sc["steps"], intervals=sc["intervals"],
                          tau=tau, beta=sc["beta"], alpha=alpha, force_scale=sc["force_scale"],
                          force_shift=1.775, dt=sc["dt"], perturb_mode=1, eps=eps,
                          snaps=np.concatenate(files[:10]))
    assert res["status"] == 0
    assert np.array_equal(res["labels"].ravel(), z[f"run{i}_labels"])
    assert np.array_equal(res["rvalues"], z[f"run{i}_rvalues"])
    force = res["drag"].transpose(1, 0, 2).reshape(Nc, -1)  # slot files: intervals appended
    assert np.array_equal(force, z[f"run{i}_force"])
    # the run actually exercised cloning
    assert (res["labels"] != np.arange(Nc)).any()
