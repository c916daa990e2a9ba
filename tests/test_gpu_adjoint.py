"""The hand-written adjoint of the interval-integrated drag against central
finite differences of the FP64 forward (the forward is the sampler's own,
bit-identical to the oracle).

A directional derivative g.d along a random direction d can lie arbitrarily
close to zero (g.d / (|g| |d|) is about N(0, 1/n) for n populations), where
its relative error means nothing; the tolerances are therefore stated on the
error relative to |g| |d| (FP64 adjoint 1e-10, FP32 1e-6, the FP32 forward
recomputation and adjoint), on the relative error of the directions whose
derivative is not near zero (|g.d| >= 0.1 |g| |d| / sqrt(n): FP64 1e-6, FP32
5e-4), and, for FP32, on the whole gradient against the FP64 adjoint's
(relative L2 distance 1e-5)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def case(orc, clbm_lib, W=64, H=24, side=6, nc=3, tau=0.56, u0=0.05):
    g = orc.channel_geom(W, H, side, W // 4, H // 2)
    phys = dict(tau=tau, beta=side * u0 * u0 / ((W - 1) * (H - 1)), alpha=0.5,
                force_scale=2 / (u0 * u0 * side), force_shift=0.0, dt=u0 / side)
    d = clbm_lib.RunDesc(width=g.nx, height=g.ny, xmin=g.xmin, xmax=g.xmax, ymin=g.ymin, ymax=g.ymax,
                         nclones=nc, ranks=1, **phys)
    return g, phys, d


def test_forward_drag_matches_oracle(gpu, clbm_lib, orc):
    g, phys, d = case(orc, clbm_lib)
    nc, T = 3, 25
    states = np.concatenate([orc.init_equilibrium(g, 0.05, 1e-3, 9, 0, j) for j in range(nc)])
    ref = orc.run_sampler(g, states, steps=T, intervals=1, **phys)
    with clbm_lib.Sampler([d], clbm_lib.FP64, max_steps=T) as s:
        s.load_run(0, states)
        J = s.drag_fwd(T, 7)
        assert np.array_equal(s.drag(0), ref["drag"][0])
        np.testing.assert_allclose(np.exp(phys["alpha"] * J), ref["weights"][0], rtol=1e-15)
        assert np.array_equal(s.dump(0, 1), states[g.nx * g.ny * 9:2 * g.nx * g.ny * 9])  # state untouched


@pytest.mark.parametrize("drag_mode", [0, 1])
def test_adjoint_vs_central_differences(gpu, clbm_lib, orc, drag_mode):
    """drag_mode 0: the reference's stress integration; 1: momentum exchange."""
    g, phys, d = case(orc, clbm_lib)
    d.drag_mode = drag_mode
    nc, T, every, eps = 3, 30, 7, 1e-6
    n = 9 * g.nx * g.ny
    rng = np.random.default_rng(5)
    base = np.concatenate([orc.init_equilibrium(g, 0.05, 1e-3, 5, 0, j) for j in range(nc)])
    S0 = base + rng.normal(0.0, 1e-4, base.size)
    grad = {}
    for prec in (clbm_lib.FP64, clbm_lib.FP32):
        with clbm_lib.Sampler([d], prec, max_steps=T) as s:
            s.load_run(0, S0)
            s.drag_fwd(T, every)
            s.drag_bwd()
            grad[prec] = np.concatenate([s.drag_grad(0, j) for j in range(nc)]).reshape(nc, n)
    g64, g32 = grad[clbm_lib.FP64], grad[clbm_lib.FP32]
    gnorm = np.linalg.norm(g64, axis=1)
    assert np.isfinite(g32).all() and (gnorm > 0).all()
    assert (np.linalg.norm(g32 - g64, axis=1) / gnorm < 1e-5).all()
    with clbm_lib.Sampler([d], clbm_lib.FP64, max_steps=T) as f:
        for _ in range(4):
            dirn = rng.normal(0.0, 1.0, base.size)
            f.load_run(0, S0 + eps * dirn)
            jp = f.drag_fwd(T, every)
            f.load_run(0, S0 - eps * dirn)
            jm = f.drag_fwd(T, every)
            fd = (jp - jm) / (2 * eps)
            dn = np.linalg.norm(dirn.reshape(nc, n), axis=1)
            well = np.abs(fd) >= 0.1 * gnorm * dn / np.sqrt(n)
            for gr, tol_norm, tol_rel in ((g64, 1e-10, 1e-6), (g32, 1e-6, 5e-4)):
                ad = (gr * dirn.reshape(nc, n)).sum(axis=1)
                assert (np.abs(ad - fd) / (gnorm * dn) < tol_norm).all(), (ad, fd)
                assert (np.abs(ad - fd)[well] / np.abs(fd)[well] < tol_rel).all(), (ad, fd)


@pytest.mark.parametrize("prec", [0, 1])
def test_adjoint_with_random_field(gpu, clbm_lib, orc, prec):
    """A forcing-variant run: the forward and the adjoint step under the fields
    of the last interval (drawn by one interval first), the field acting on
    the first 12 of 30 steps; FD on the FP64 forward with the same fields."""
    g, phys, d = case(orc, clbm_lib)
    d.field_mode, d.field_steps, d.field_eps, d.field_sigma = 1, 12, 0.3, 4.0
    nc, T, every, eps = 3, 30, 7, 1e-6
    n = 9 * g.nx * g.ny
    rng = np.random.default_rng(9)
    base = np.concatenate([orc.init_equilibrium(g, 0.05, 1e-3, 5, 0, j) for j in range(nc)])
    S0 = base + rng.normal(0.0, 1e-4, base.size)

    def sampler(p):
        s = clbm_lib.Sampler([d], p, max_steps=T)
        s.init_equilibrium(0, 0.05, 1e-3, 1)
        s.run_interval(T)  # draws the fields the forward and adjoint use
        assert np.abs(s.field_map(0, 0)[0]).max() > 0.1
        return s

    with sampler(prec) as s:
        s.load_run(0, S0)
        s.drag_fwd(T, every)
        s.drag_bwd()
        grad = np.concatenate([s.drag_grad(0, j) for j in range(nc)]).reshape(nc, n)
    gnorm = np.linalg.norm(grad, axis=1)
    tol_norm, tol_rel = (1e-10, 1e-6) if prec == clbm_lib.FP64 else (1e-6, 5e-4)
    with sampler(clbm_lib.FP64) as f:
        for _ in range(3):
            dirn = rng.normal(0.0, 1.0, base.size)
            f.load_run(0, S0 + eps * dirn)
            jp = f.drag_fwd(T, every)
            f.load_run(0, S0 - eps * dirn)
            jm = f.drag_fwd(T, every)
            fd = (jp - jm) / (2 * eps)
            dn = np.linalg.norm(dirn.reshape(nc, n), axis=1)
            ad = (grad * dirn.reshape(nc, n)).sum(axis=1)
            assert (np.abs(ad - fd) / (gnorm * dn) < tol_norm).all(), (ad, fd)
            well = np.abs(fd) >= 0.1 * gnorm * dn / np.sqrt(n)
            assert (np.abs(ad - fd)[well] / np.abs(fd)[well] < tol_rel).all(), (ad, fd)
