"""Band splits of the cluster-resident interval kernel (host-only logic,
clbm_band_rows): the even split, the balanced split against a brute-force
restatement of its cost model, and the argument checks."""
import itertools

import numpy as np
import pytest

SMEM_LIMIT = 227 * 1024


def smem(nb):
    nseg = (nb + 31) // 32
    return 36 * nb + 2 * ((nseg + 7) & ~7) + ((nseg + 15) & ~15) + 32


def rows_limit(W):
    r = 0
    while smem((r + 1) * W) <= SMEM_LIMIT:
        r += 1
    return r


def row_cost(W, H, xmin, xmax, ymin, ymax, y, g):
    gen = 0
    if y in (0, H - 1):
        gen = 0.25 * W
    elif ymin <= y <= ymax:
        x0 = max(0, xmin) // 32 * 32
        x1 = min(W, (min(W - 1, xmax) // 32 + 1) * 32)
        gen = max(0, x1 - x0)
    return W + g * gen


def split_cost(W, H, box, rows, g):
    """(largest band cost, sum of squared band costs) of a split"""
    costs, y = [], 0
    for r in rows:
        c = sum(row_cost(W, H, *box, yy, g) for yy in range(y, y + r))
        c += (0.25 * g * W if y > 0 else 0) + (0.25 * g * W if y + r < H else 0)
        costs.append(c)
        y += r
    return max(costs), sum(c * c for c in costs)


def desc(clbm, W, H, xmin, xmax, ymin, ymax):
    return clbm.RunDesc(width=W, height=H, xmin=xmin, xmax=xmax, ymin=ymin, ymax=ymax, nclones=1, ranks=1,
                        tau=0.55, beta=1e-6, alpha=0.1, force_scale=1.0, dt=0.01)


def test_even_split(clbm_lib):
    d = desc(clbm_lib, 256, 64, 58, 70, 26, 38)
    assert list(clbm_lib.band_rows(d, 3, 0.0)) == [22, 21, 21]
    assert list(clbm_lib.band_rows(d, 4, 0.0)) == [16] * 4
    d = desc(clbm_lib, 64, 25, 13, 19, 9, 15)
    assert list(clbm_lib.band_rows(d, 4, 0.0)) == [7, 6, 6, 6]


def test_square_band_shrinks_with_weight(clbm_lib):
    # the 256x64 channel with a 12-side square at (64, 32): the middle band
    # holds the square's rows and gets fewer rows as their weight grows
    d = desc(clbm_lib, 256, 64, 58, 70, 26, 38)
    assert list(clbm_lib.band_rows(d, 3, 3.0)) == [24, 15, 25]
    mids = [clbm_lib.band_rows(d, 3, g)[1] for g in (0.0, 0.5, 1.0, 2.0, 3.0, 4.0, 8.0)]
    assert mids == sorted(mids, reverse=True) and mids[-1] < mids[0]
    for g in (0.5, 2.0, 8.0):
        r = clbm_lib.band_rows(d, 3, g)
        assert r.sum() == 64 and r.max() <= rows_limit(256) and r.min() >= 1


@pytest.mark.parametrize("W,H,box,cs", [
    (64, 12, (20, 30, 4, 7), 2), (64, 12, (20, 30, 4, 7), 3), (96, 17, (30, 40, 2, 6), 3),
    (128, 14, (0, 127, 5, 9), 4), (256, 15, (58, 70, 9, 14), 3)])
@pytest.mark.parametrize("g", [0.5, 1.5, 4.0])
def test_balanced_split_is_optimal(clbm_lib, W, H, box, cs, g):
    got = list(clbm_lib.band_rows(desc(clbm_lib, W, H, *box), cs, g))
    best = None
    for cut in itertools.combinations(range(1, H), cs - 1):
        rows = np.diff((0,) + cut + (H,)).tolist()
        if max(rows) > rows_limit(W):
            continue
        c = split_cost(W, H, box, rows, g)
        if best is None or c < best[0]:
            best = (c, rows)
    mx, sq = split_cost(W, H, box, got, g)
    assert sum(got) == H and min(got) >= 1
    assert mx == pytest.approx(best[0][0], rel=1e-12)
    assert sq <= best[0][1] * (1 + 1e-12) or mx < best[0][0]


def test_band_rows_argument_checks(clbm_lib):
    d = desc(clbm_lib, 256, 64, 58, 70, 26, 38)
    for cs in (0, 17, 65):
        with pytest.raises(clbm_lib.ClbmError):
            clbm_lib.band_rows(d, cs, 1.0)
    with pytest.raises(clbm_lib.ClbmError):  # one band of 64 rows of 4096 nodes exceeds shared memory
        clbm_lib.band_rows(desc(clbm_lib, 4096, 64, 100, 110, 20, 30), 1, 1.0)
