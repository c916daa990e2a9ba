"""The benchmark workload table against the workload descriptions (CPU)."""
from clbm import configs


def test_uneven_batch_squares_round_down():
    """Eight lattices, square side floor(H/5) centred at (W/4, H/2), k evenly
    spaced in [-0.5, 0.5], 256 clones each, T = 100, 40 cloning steps."""
    sizes = [(128, 32), (192, 48), (256, 64), (320, 80), (384, 96), (448, 112), (512, 128), (256, 128)]
    wl = configs.c4()
    assert (wl.steps, wl.intervals) == (100, 40)
    for i, ((w, h), r) in enumerate(zip(sizes, wl.runs)):
        s = h // 5
        assert (r.width, r.height, r.side, r.nclones) == (w, h, s, 256)
        assert r.xmin == w // 4 - s // 2 and r.ymin == h // 2 - s // 2
        assert abs(r.k - (-0.5 + i / 7)) < 1e-15


def test_benchmark_workloads_as_described():
    r = configs.c3().runs[0]
    assert (r.width, r.height, r.side, r.xc, r.yc, r.nclones) == (256, 64, 12, 64, 32, 4096)
    assert (r.u0, r.tau, r.k, r.noise, r.seed) == (0.04, 0.55, 0.3, 1e-5, 3)
    c2 = configs.c2()
    assert [r.k for r in c2.runs] == [-0.2, 0.2] and (c2.steps, c2.intervals) == (200, 50)
    r = c2.runs[0]
    assert (r.width, r.height, r.side, r.xc, r.yc, r.nclones, r.tau, r.noise) == (400, 100, 20, 100, 50, 512, 0.53, 1e-4)
