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


def _collide(orc, g, S):
    """post-collision populations of state S (the oracle's in-place collision)"""
    import ctypes as C
    fin = S.copy()
    fout = np.empty_like(fin)
    orc.lib().orc_stream_collide(C.byref(g), fin.ctypes.data_as(C.c_void_p), fout.ctypes.data_as(C.c_void_p),
                                 None, None, None, C.c_double(0.0), C.c_double(0.7))
    return fin


@pytest.mark.parametrize("seed", range(8))
def test_in_place_aa_scheme_equals_reference(orc, seed):
    """The on-chip interval kernel's in-place update: after a gather step
    A[m][k] holds the streamed state, after a local step A[n][opp k] holds
    P(n,k); every slot is read and written by one node only."""
    import ctypes as C
    rng = np.random.default_rng(200 + seed)
    nx, ny = int(rng.integers(6, 24)), int(rng.integers(6, 20))
    s = int(rng.integers(1, min(nx - 1, ny - 3)))
    x0, y0 = int(rng.integers(0, nx - s)), int(rng.integers(1, ny - s - 1))
    g = orc.Geom(nx, ny, x0, x0 + s, y0, y0 + s)
    masks = np.array([[orc.lib().orc_bounce_mask(C.byref(g), x, y) for y in range(ny)] for x in range(nx)])
    solid = ((masks >> 9) & 1).astype(bool)
    S = (orc.W[None, None, :] * (1 + 0.05 * rng.standard_normal((nx, ny, 9))))
    S[solid] = orc.W
    ref = [S.ravel().copy()]
    cur = S.ravel().copy()
    for _ in range(4):
        cur = orc.lbm_step(g, cur, 0.0, 0.7)[0]
        ref.append(cur.copy())
    # AA: start from P_0 in the local-step layout
    P0 = _collide(orc, g, S.ravel()).reshape(nx, ny, 9)
    A = np.full((nx, ny, 9), np.nan)
    for k in range(9):
        A[:, :, orc.OPP[k]] = P0[:, :, k]
    for t in range(4):
        gather = t % 2 == 0
        owner = {}
        newA = A.copy()
        states = np.full((nx, ny, 9), np.nan)
        for x in range(nx):
            for y in range(ny):
                if solid[x, y]:
                    continue
                m = masks[x, y]
                for k in range(9):
                    if not gather or (m >> k) & 1:
                        slot = (x, y, k)
                    else:
                        slot = ((x - orc.CX[k]) % nx, y - orc.CY[k], orc.OPP[k])
                    assert 0 <= slot[1] < ny
                    assert owner.setdefault(slot, (x, y)) == (x, y), "slot read by two nodes"
                    states[x, y, k] = A[slot]
        S_t = states.copy()
        S_t[solid] = orc.W
        assert np.array_equal(S_t.ravel(), ref[t + 1]), t
        P = _collide(orc, g, S_t.ravel()).reshape(nx, ny, 9)
        written = set()
        for x in range(nx):
            for y in range(ny):
                if solid[x, y]:
                    continue
                m = masks[x, y]
                for k in range(9):
                    ok = orc.OPP[k]
                    if not gather or (m >> ok) & 1:
                        slot = (x, y, ok)
                    else:
                        tx, ty = (x + orc.CX[k]) % nx, y + orc.CY[k]
                        assert 0 <= ty < ny
                        if solid[tx, ty]:
                            continue
                        slot = (tx, ty, k)
                    assert slot not in written
                    assert owner.get(slot, (x, y)) == (x, y), "slot written by a node that did not read it"
                    written.add(slot)
                    newA[slot] = P[x, y, k]
        A = newA
