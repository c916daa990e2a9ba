"""ctypes wrapper of the oracle (clbm_oracle.c) and of the reference harness.

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke entry point (as the
checker) and by bench.py's CPU-baseline leg.  The product path never imports
this module.

``build()`` compiles ``oracle/_build/liboracle.so`` with make (gcc,
-ffp-contract=off); ``build_ref()`` compiles the reference's own objects in
place into ``oracle/_ref/`` when the reference tree is present.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref_core.so"
REF_DRIVER = HERE / "_ref" / "TLGK_LBM_POPS_PERTURB"
# the reference checkout: $CLBM_REFERENCE_TREE, else a checkout named
# "reference" beside this repository
REF_TREE = Path(os.environ.get("CLBM_REFERENCE_TREE", str(HERE.parent.parent / "reference")))

W = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])
OPP = np.array([0, 3, 4, 1, 2, 7, 8, 5, 6])


class Geom(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nx", "ny", "xmin", "xmax", "ymin", "ymax")]


class SamplerCfg(C.Structure):
    _fields_ = [("g", Geom), ("nclones", C.c_int), ("steps", C.c_int), ("intervals", C.c_int),
                ("ranks", C.c_int), ("tau", C.c_double), ("beta", C.c_double),
                ("alpha", C.c_double), ("force_scale", C.c_double), ("force_shift", C.c_double),
                ("dt", C.c_double), ("perturb_mode", C.c_int), ("resample_mode", C.c_int),
                ("nsnap", C.c_int), ("eps", C.c_double), ("seed", C.c_uint64), ("run", C.c_uint32),
                ("drag_mode", C.c_int)]


class D48(C.Structure):
    _fields_ = [("x", C.c_uint64)]


class GlibcRand(C.Structure):
    _fields_ = [("r", C.c_uint32 * 34), ("i", C.c_int)]


class CloneResult(C.Structure):
    _fields_ = [("rbar", C.c_double), ("logr", C.c_double), ("ncopies_drawn", C.c_int),
                ("ncomm", C.c_int), ("status", C.c_int)]


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def build_ref() -> bool:
    """Compile the reference objects in place; False when the tree is absent."""
    if not (REF_TREE / "src" / "lbm_src" / "streamCollCompute.cpp").exists():
        return False
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={REF_TREE}"], check=True,
                   capture_output=True)
    return REF_LIB.exists()


_lib = None
_ref = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        L.orc_force_on_square.restype = C.c_double
        L.orc_force_momentum_exchange.restype = C.c_double
        L.orc_drand48_next.restype = C.c_double
        L.orc_glibc_rand_next.restype = C.c_int32
        L.orc_philox_uniform.restype = C.c_double
        L.orc_philox_uniform.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]
        L.orc_bench_lbm.restype = C.c_double
        L.orc_bench_lbm.argtypes = [C.POINTER(Geom), C.c_int, C.c_int, C.c_double, C.c_double,
                                    C.c_int, C.POINTER(C.c_double)]
        L.orc_clone_reference.restype = CloneResult
        L.orc_clone_systematic.restype = CloneResult
        L.orc_clone_systematic.argtypes = [C.c_int, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p,
                                           C.c_void_p]
        L.orc_bounce_mask.restype = C.c_int
        _lib = L
    return _lib


def ref() -> C.CDLL | None:
    """The reference objects (None when they were not built here)."""
    global _ref
    if _ref is None and REF_LIB.exists():
        R = C.CDLL(str(REF_LIB))
        R.ref_force.restype = C.c_double
        R.ref_bench.restype = C.c_double
        for f in ("ref_stream_collide",):
            getattr(R, f).argtypes = [C.c_void_p] * 5 + [C.c_double, C.c_double]
        R.ref_stream_collide_spatial.argtypes = [C.c_void_p] * 5 + [C.c_double, C.c_void_p,
                                                                    C.c_double, C.c_double]
        R.ref_force.argtypes = [C.c_void_p, C.c_double]
        R.ref_perturb.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double]
        R.ref_run_clone.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_void_p]
        R.ref_bench.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double,
                                C.POINTER(C.c_double)]
        _ref = R
    return _ref


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# ---- channel set-ups ----------------------------------------------------
def reference_square_geom(L: int) -> Geom:
    """The reference drivers' square domain Dx = Dy = 4L+1 with the obstacle
    at x in [(Dx-1)/2, +L], y in [(Dy-1)/2 - L/2, +L]
    (src/mpi_LBM_GK_pops_perturb.cpp:131-133)."""
    D = 4 * L + 1
    x0 = (D - 1) // 2
    y0 = (D - 1) // 2 - L // 2
    return Geom(D, D, x0, x0 + L, y0, y0 + L)


def channel_geom(width: int, height: int, side: int, xc: int, yc: int) -> Geom:
    """A W x H channel with a square of side s centred at (xc, yc):
    xmin = xc - floor(s/2), xmax = xmin + s, same in y (perimeter nodes are
    fluid, as in the reference)."""
    x0 = xc - side // 2
    y0 = yc - side // 2
    return Geom(width, height, x0, x0 + side, y0, y0 + side)


def reference_scalars(L: int, U0: float, dT: float, T: float, Dx: int | None = None,
                      Dy: int | None = None) -> dict:
    """beta0, T0, F0, dt and step counts exactly as the pops driver computes
    them (:144-151, :119)."""
    Dx = Dx or 4 * L + 1
    Dy = Dy or 4 * L + 1
    beta0 = (1.0 / (Dx - 1)) * (float(L) / (Dy - 1)) * U0 * U0
    T0 = L / U0
    F0 = (U0 * U0) * L * 0.5
    return {"beta": beta0, "T0": T0, "F0": F0, "force_scale": 1.0 / F0, "dt": 1.0 / T0,
            "steps": math.floor(dT * T0), "intervals": math.floor(T / dT)}


# ---- wrappers ---------------------------------------------------------------
def init_equilibrium(g: Geom, u0: float, noise: float, seed: int, run: int, clone: int) -> np.ndarray:
    f = np.empty(9 * g.nx * g.ny)
    lib().orc_init_equilibrium(_p(f), C.byref(g), C.c_double(u0), C.c_double(noise),
                               C.c_uint64(seed), C.c_uint32(run), C.c_uint32(clone))
    return f


def lbm_step(g: Geom, f: np.ndarray, beta: float, tau: float, map_=None, eps=0.0):
    """One reference LB step (collide, stream, walls, square, reset) on a copy;
    returns (new_state, post_collision_fin, rho, ux, uy)."""
    fin = f.copy()
    fout = np.empty_like(fin)
    n = g.nx * g.ny
    rho, ux, uy = np.empty(n), np.empty(n), np.empty(n)
    if map_ is None:
        lib().orc_stream_collide(C.byref(g), _p(fin), _p(fout), _p(rho), _p(ux), _p(uy),
                                 C.c_double(beta), C.c_double(tau))
    else:
        lib().orc_stream_collide_spatial(C.byref(g), _p(fin), _p(fout), _p(rho), _p(ux), _p(uy),
                                         C.c_double(beta), _p(map_), C.c_double(tau),
                                         C.c_double(eps))
    lib().orc_walls_bb(C.byref(g), _p(fout), _p(fin))
    lib().orc_square_bb(C.byref(g), _p(fout), _p(fin))
    lib().orc_interior_reset(C.byref(g), _p(fout))
    return fout, fin, rho, ux, uy


def force(g: Geom, f: np.ndarray, omega: float) -> float:
    return lib().orc_force_on_square(C.byref(g), _p(f), C.c_double(omega))


def force_momentum_exchange(g: Geom, f: np.ndarray) -> float:
    """Momentum-exchange x-drag of a streamed, bounced AoS state."""
    f = np.ascontiguousarray(f, dtype=np.float64)
    return lib().orc_force_momentum_exchange(C.byref(g), _p(f))


def run_clone(g: Geom, f: np.ndarray, steps: int, beta: float, tau: float) -> tuple[np.ndarray, np.ndarray]:
    """steps reference LB steps of one clone with the drag after each."""
    drag = np.empty(steps)
    cur = f.copy()
    for s in range(steps):
        cur = lbm_step(g, cur, beta, tau)[0]
        drag[s] = force(g, cur, 1.0 / tau)
    return cur, drag


def perturb_mix(f: np.ndarray, snaps: np.ndarray, eps: float, prefactors: np.ndarray) -> np.ndarray:
    out = f.copy()
    pre = np.ascontiguousarray(prefactors, dtype=np.float64)
    s = np.ascontiguousarray(snaps, dtype=np.float64)
    lib().orc_perturb_mix(_p(out), _p(s), C.c_int(len(pre)), C.c_int(f.size), C.c_double(eps), _p(pre))
    return out


def philox_uniform(seed, c0, c1, c2, c3) -> float:
    return lib().orc_philox_uniform(seed, c0, c1, c2, c3)


def run_sampler(g: Geom, states: np.ndarray, *, steps: int, intervals: int, tau: float,
                beta: float, alpha: float, force_scale: float, force_shift: float, dt: float,
                perturb_mode: int = 0, resample_mode: int = 0, eps: float = 0.0,
                snaps: np.ndarray | None = None, seed: int = 0, run: int = 0,
                ranks: int = 1, drag_mode: int = 0) -> dict:
    nc = states.size // (9 * g.nx * g.ny)
    nsnap = 0 if snaps is None else snaps.size // (9 * g.nx * g.ny)
    cfg = SamplerCfg(g, nc, steps, intervals, ranks, tau, beta, alpha, force_scale, force_shift,
                     dt, perturb_mode, resample_mode, nsnap, eps, seed, run, drag_mode)
    st = np.ascontiguousarray(states, dtype=np.float64).copy()
    drag = np.zeros((intervals, nc, steps))
    labels = np.zeros((intervals, nc), np.int32)
    rv = np.zeros(intervals)
    logr = np.zeros(intervals)
    wts = np.zeros((intervals, nc))
    cop = np.zeros((intervals, 2, nc), np.int32)
    sn = None if snaps is None else np.ascontiguousarray(snaps, dtype=np.float64)
    status = lib().orc_run_sampler(C.byref(cfg), _p(st), _p(sn), _p(drag), _p(labels), _p(rv),
                                   _p(logr), _p(wts), _p(cop))
    return {"status": status, "states": st, "drag": drag, "labels": labels, "rvalues": rv,
            "logr": logr, "weights": wts, "copies": cop}


def bench_lbm(g: Geom, nclones: int, steps: int, tau: float, beta: float, nthreads: int) -> tuple[float, float]:
    chk = C.c_double()
    t = lib().orc_bench_lbm(C.byref(g), nclones, steps, tau, beta, nthreads, C.byref(chk))
    return t, chk.value
