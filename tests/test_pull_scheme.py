"""The device kernels store POST-collision populations and pull
S(n,k) = P(n - c_k, k), or P(n, opp k) on bounced slots (bounce_mask); this
checks on the CPU that the pull formulation reproduces the reference's
collide / push-stream / wall BB / square BB / interior reset sequence exactly,
and that no fluid node ever pulls a square-interior value."""
import numpy as np
import pytest




@pytest.mark.parametrize("seed", range(12))
def test_pull_equals_reference_push(orc, seed):
    import ctypes as C
    rng = np.random.default_rng(seed)
    nx, ny = int(rng.integers(6, 30)), int(rng.integers(6, 24))
    s = int(rng.integers(1, min(nx - 1, ny - 3)))
    x0 = int(rng.integers(0, nx - s))
    y0 = int(rng.integers(1, ny - s - 1))
    g = orc.Geom(nx, ny, x0, x0 + s, y0, y0 + s)
    f = (orc.W[None, None, :] * (1 + 0.05 * rng.standard_normal((nx, ny, 9)))).ravel()
    tau, beta = 0.55 + rng.random(), 1e-5 * rng.random()
    ref_state, post, *_ = orc.lbm_step(g, f, beta, tau)
    P = post.reshape(nx, ny, 9).copy()
    masks = np.array([[orc.lib().orc_bounce_mask(C.byref(g), x, y) for y in range(ny)] for x in range(nx)])
    interior = (masks >> 9) & 1
    P[interior.astype(bool)] = np.nan  # never read
    S = np.empty_like(P)
    for x in range(nx):
        for y in range(ny):
            m = masks[x, y]
            if m & 512:
                S[x, y] = orc.W
                continue
            for k in range(9):
                if (m >> k) & 1:
                    S[x, y, k] = P[x, y, orc.OPP[k]]
                else:
                    sx = (x - orc.CX[k]) % nx
                    sy = y - orc.CY[k]
                    assert 0 <= sy < ny, "pull across a wall that is not bounced"
                    S[x, y, k] = P[sx, sy, k]
    assert not np.isnan(S).any(), "a fluid node pulled a square-interior value"
    assert np.array_equal(S.ravel(), ref_state)
