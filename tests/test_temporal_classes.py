"""CPU check of the cluster-resident interval kernel's segment classes
(cloning-lbm-mpi_gb300/csrc/clbm_temporal.cu): for every node of a band and
every class a segment can fall in -- walls through the bulk update with the
bounce-back built in, band-edge rows, segments spanning two rows at a band
edge, wrap and interior bulk -- the slots a gather step reads for S(n,k)
and writes P(n,k) to are those of the general path (bounce-back masks of
the walls and the square, pushes dropped into the square or beyond a wall),
every slot lies in its band, and the remote slots of a band-edge row are the
adjacent band's edge row.  Slots are (band, band-local node, k); the band
splits include the uneven ones the autotuner balances."""
import pytest

CX = [0, 1, 0, -1, 0, 1, -1, -1, 1]
CY = [0, 0, 1, 0, -1, 1, 1, -1, -1]
OPP = [0, 3, 4, 1, 2, 7, 8, 5, 6]


def bounce_mask(H, box, x, y):
    """bit k: slot k bounces back; bit 9: inside the square
    (src/lbm_src/domain_noSlipWalls.cpp:6-22, src/lbm_src/square.cpp:24-50)"""
    xmin, xmax, ymin, ymax = box
    m = 0
    if y == H - 1:
        m |= (1 << 4) | (1 << 7) | (1 << 8)
    if y == 0:
        m |= (1 << 2) | (1 << 5) | (1 << 6)
    inx, iny = xmin < x < xmax, ymin < y < ymax
    if inx and y == ymin:
        m |= (1 << 7) | (1 << 4) | (1 << 8)
    if inx and y == ymax:
        m |= (1 << 5) | (1 << 2) | (1 << 6)
    if iny and x == xmin:
        m |= (1 << 6) | (1 << 3) | (1 << 7)
    if iny and x == xmax:
        m |= (1 << 8) | (1 << 1) | (1 << 5)
    if x == xmin and y == ymin:
        m |= 1 << 7
    if x == xmin and y == ymax:
        m |= 1 << 6
    if x == xmax and y == ymax:
        m |= 1 << 5
    if x == xmax and y == ymin:
        m |= 1 << 8
    if inx and iny:
        m |= 1 << 9
    return m


def check(W, H, box, rows):
    xmin, xmax, ymin, ymax = box
    cs = len(rows)
    row0 = [sum(rows[:b]) for b in range(cs + 1)]

    def slot(x, y, k):
        b = max(i for i in range(cs) if row0[i] <= y)
        return (b, (y - row0[b]) * W + x, k)

    def general(x, y, plain):
        in_box = not plain and xmin <= x <= xmax and ymin <= y <= ymax
        mask = bounce_mask(H, box, x, y) if (not plain and (in_box or y in (0, H - 1))) else 0
        if mask & 512:
            return None
        rd = {k: slot(x, y, k) if (mask >> k) & 1 else slot((x - CX[k]) % W, y - CY[k], OPP[k]) for k in range(9)}
        wr = {}
        for k in range(9):
            if not plain and not (mask >> OPP[k]) & 1:
                tx, ty = (x + CX[k]) % W, y + CY[k]
                if ty < 0 or ty >= H or (xmin < tx < xmax and ymin < ty < ymax):
                    continue
            wr[k] = rd[OPP[k]]
        return rd, wr

    def fast(x, y, wall):
        rd, wr = {}, {}
        for k in range(9):
            if (wall == 1 and k in (2, 5, 6)) or (wall == 2 and k in (4, 7, 8)):
                rd[k] = slot(x, y, k)
            else:
                rd[k] = slot((x - CX[k]) % W, y - CY[k], OPP[k])
        for k in range(9):
            if (wall == 1 and k in (4, 7, 8)) or (wall == 2 and k in (2, 5, 6)):
                wr[k] = slot(x, y, OPP[k])
            else:
                wr[k] = slot((x + CX[k]) % W, y + CY[k], k)
        return rd, wr

    classes = [0] * 6
    for b in range(cs):
        nb = rows[b] * W
        for sg in range((nb + 31) // 32):
            lanes = []
            for i in range(sg * 32, sg * 32 + 32):
                ly = i // W
                lanes.append((ly, i - ly * W, row0[b] + ly, i >= nb))
            box_ = any(not p and xmin <= x <= xmax and ymin <= y <= ymax for ly, x, y, p in lanes)
            pad = any(p for *_, p in lanes)
            wall = any(not p and y in (0, H - 1) for ly, x, y, p in lanes)
            edge = any(not p and cs > 1 and ly in (0, rows[b] - 1) for ly, x, y, p in lanes)
            one_row = all(not p and ly == lanes[0][0] for ly, x, y, p in lanes) and rows[b] > 1
            if box_ or pad:
                c = 5
            elif wall:
                c = 4 if one_row else 5
            elif edge:
                c = 3 if one_row else 2
            else:
                c = 0 if all(not p and 0 < x < W - 1 for ly, x, y, p in lanes) else 1
            classes[c] += 1
            for ly, x, y, p in lanes:
                if p:
                    continue
                ref = general(x, y, False)
                got = {5: lambda: ref, 4: lambda: fast(x, y, 1 if y == 0 else 2), 2: lambda: general(x, y, True)}.get(
                    c, lambda: fast(x, y, 0))()
                assert got == ref, (rows, b, sg, c, x, y)
                if got is None:
                    continue
                for s in list(got[0].values()) + list(got[1].values()):
                    assert 0 <= s[1] < rows[s[0]] * W
                    if c in (0, 1, 4):
                        assert s[0] == b
                    if c == 3 and s[0] != b:  # the row across the band edge
                        assert (s[0] == b - 1 and ly == 0 and s[1] // W == rows[b - 1] - 1) or \
                               (s[0] == b + 1 and ly == rows[b] - 1 and s[1] // W == 0)
    return classes


def box_of(side, xc, yc):
    xmin, ymin = xc - side // 2, yc - side // 2
    return (xmin, xmin + side, ymin, ymin + side)


@pytest.mark.parametrize("W,H,side,xc,yc,rows", [
    (256, 64, 12, 64, 32, [25, 14, 25]), (256, 64, 12, 64, 32, [16] * 4), (256, 64, 12, 64, 32, [22, 21, 21]),
    (200, 50, 8, 50, 25, [7, 7, 6, 6, 6, 6, 6, 6]), (200, 50, 8, 50, 25, [12, 8, 6, 12, 12]),
    (96, 23, 5, 30, 9, [5, 5, 5, 4, 4]), (96, 23, 5, 30, 9, [20, 3]), (96, 23, 5, 30, 9, [3, 3, 3] + [2] * 7),
    (64, 24, 6, 16, 12, [1, 11, 11, 1]), (64, 24, 6, 16, 12, [24]), (400, 100, 20, 100, 50, [12] + [11] * 8),
    (128, 32, 6, 32, 16, [16, 16]), (320, 80, 16, 80, 40, [20] * 4),
])
def test_segment_classes_match_general_path(W, H, side, xc, yc, rows):
    classes = check(W, H, box_of(side, xc, yc), rows)
    assert sum(classes) == sum((r * W + 31) // 32 for r in rows)
