"""Oracle against the reference objects compiled in place (oracle/_ref), on
random channel geometries, states and parameters beyond the fixtures.
Skipped where the reference tree is not available (e.g. on the GPU machine)."""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def R(orc):
    if not orc.build_ref():
        pytest.skip("reference tree not available")
    return orc.ref()


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


@pytest.mark.parametrize("seed", range(10))
def test_random_geometry_bit_exact(orc, R, seed):
    rng = np.random.default_rng(100 + seed)
    nx, ny = int(rng.integers(8, 48)), int(rng.integers(8, 32))
    s = int(rng.integers(1, min(nx - 1, ny - 3)))
    x0, y0 = int(rng.integers(0, nx - s)), int(rng.integers(1, ny - s - 1))
    g = orc.Geom(nx, ny, x0, x0 + s, y0, y0 + s)
    R.ref_set_geom(nx, ny, x0, x0 + s, y0, y0 + s)
    f = (orc.W[None, None, :] * (1 + 0.05 * rng.standard_normal((nx, ny, 9)))).ravel()
    tau, beta = 0.51 + rng.random(), 1e-4 * rng.random()
    a = f.copy()
    drag_r = np.empty(4)
    R.ref_run_clone(_p(a), 4, beta, tau, _p(drag_r))
    b, drag_o = orc.run_clone(g, f, 4, beta, tau)
    assert np.array_equal(a, b)
    assert np.array_equal(drag_r, drag_o)


def test_perturbation_with_libc_stream(orc, R):
    libc = C.CDLL("libc.so.6")
    rng = np.random.default_rng(5)
    n = 9 * 20 * 8
    f = (1 + 0.01 * rng.standard_normal(n)) / 9
    snaps = rng.random(7 * n)
    libc.seed48((C.c_ushort * 3)(3, 4, 5))
    a = f.copy()
    R.ref_perturb(_p(a), _p(snaps), 7, n, 0.2)
    libc.seed48((C.c_ushort * 3)(3, 4, 5))
    libc.drand48.restype = C.c_double
    pre = np.array([libc.drand48() for _ in range(7)])
    assert np.array_equal(a, orc.perturb_mix(f, snaps, 0.2, pre))
