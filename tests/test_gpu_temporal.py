"""The cluster-resident FP32 interval kernel (every clone in the shared
memory of one thread-block cluster for a whole interval) must give results
bit-identical to the streaming step kernel: same pull rules, same collision
arithmetic.  Cases cover cluster sizes 1, 2, 4 and 8 with the square across
band edges, heights that the cluster size does not divide (uneven bands), a
width that is not a multiple of 32, copies and perturbations between
intervals, and the random body-force field."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NSTREAM = 8   # streaming launch variants come first in the autotuner's numbering
NTHREAD = 3   # thread configurations of the cluster-resident kernel (1024, 512, 256)


CLUSTER_SIZES = (1, 2, 4, 8, 16, 3, 5, 6, 7, 9, 10)  # the autotuner's order


def temporal_variant(cs, tv=0):
    return NSTREAM + CLUSTER_SIZES.index(cs) * NTHREAD + tv


@pytest.mark.parametrize("W,H,side,xc,yc,cs,tv,field", [
    (64, 24, 6, 16, 12, 1, 0, False),
    (128, 32, 6, 32, 16, 2, 2, False),   # more box/edge segments (15) than warps of a CTA (8)
    (64, 32, 6, 20, 16, 2, 0, False),
    (256, 16, 6, 64, 8, 2, 1, True),
    (64, 32, 6, 20, 16, 4, 2, False),
    (32, 64, 5, 10, 30, 1, 2, False),
    (64, 24, 6, 16, 12, 2, 1, False),
    (64, 24, 6, 16, 12, 4, 2, False),
    (200, 32, 8, 50, 16, 4, 0, True),
    (96, 16, 5, 30, 9, 2, 2, True),
    (64, 25, 6, 16, 12, 4, 0, False),    # H % cs != 0: bands of 7, 6, 6, 6 rows
    (96, 23, 5, 30, 9, 4, 2, True),      # bands of 6, 6, 6, 5 rows, field
    (200, 50, 8, 50, 25, 8, 1, False),   # bands of 7 and 6 rows, square across bands
    (64, 25, 6, 16, 12, 3, 0, False),    # cluster sizes that are not powers of two
    (96, 23, 5, 30, 9, 5, 1, True),
    (200, 50, 8, 50, 25, 6, 2, False),
    (64, 32, 6, 20, 16, 7, 1, False),
    (200, 50, 8, 50, 25, 9, 0, False),      # non-portable cluster sizes
    (96, 23, 5, 30, 9, 10, 2, True),
])
def test_temporal_equals_streaming(gpu, clbm_lib, orc, W, H, side, xc, yc, cs, tv, field):
    g = orc.channel_geom(W, H, side, xc, yc)
    u0, nc, T = 0.05, 5, 21
    d = clbm_lib.RunDesc(width=g.nx, height=g.ny, xmin=g.xmin, xmax=g.xmax, ymin=g.ymin, ymax=g.ymax,
                         nclones=nc, ranks=1, tau=0.57, beta=side * u0 * u0 / ((W - 1) * (H - 1)), alpha=8.0,
                         force_scale=2 / (u0 * u0 * side), dt=u0 / side, perturb_mode=clbm_lib.PERTURB_UNIFORM,
                         eps=1e-4, seed=7)
    if field:
        d.field_mode, d.field_steps, d.field_eps, d.field_sigma = 1, 7, 0.2, 6.0
    out = []
    for variant in (4, temporal_variant(cs, tv)):
        with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=T) as s:
            s.set_step_variant(variant)
            s.init_equilibrium(0, u0, 1e-3, 7)
            res = []
            for t in range(3):
                s.run_interval(T)
                res.append(s.drag(0))
                s.clone_step()
                res.append(s.clone_result(0)["labels"].astype(np.float64))
            s.run_interval(T)
            res.append(s.drag(0))
            res.extend(s.dump(0, j) for j in range(nc))
            assert s.error_word() == 0
            out.append(res)
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_autotune_considers_cluster_resident_kernel(gpu, clbm_lib, orc):
    g = orc.channel_geom(256, 64, 12, 64, 32)
    d = clbm_lib.RunDesc(width=g.nx, height=g.ny, xmin=g.xmin, xmax=g.xmax, ymin=g.ymin, ymax=g.ymax,
                         nclones=64, ranks=1, tau=0.55, beta=1e-6, alpha=0.3, force_scale=100.0, dt=0.003)
    with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=20) as s:
        s.init_equilibrium(0, 0.04, 1e-3, 3)
        before = s.dump(0, 5)
        best, ms = s.autotune(launches=2)
        assert len(ms) == NSTREAM + len(CLUSTER_SIZES) * NTHREAD
        assert (ms[NSTREAM:] > 0).any(), ms
        assert np.array_equal(s.dump(0, 5), before)
        s.run_interval(20)
        assert s.error_word() == 0


def test_graph_replay_with_cluster_resident_kernel(gpu, clbm_lib, orc):
    """Intervals captured in CUDA graphs with the cluster-resident kernel (and
    a switch of variant between captured intervals) equal eager streaming."""
    g = orc.channel_geom(64, 24, 6, 16, 12)
    u0, nc, T = 0.05, 5, 21
    d = clbm_lib.RunDesc(width=g.nx, height=g.ny, xmin=g.xmin, xmax=g.xmax, ymin=g.ymin, ymax=g.ymax,
                         nclones=nc, ranks=1, tau=0.57, beta=6 * u0 * u0 / (63 * 23), alpha=8.0,
                         force_scale=2 / (u0 * u0 * 6), dt=u0 / 6, perturb_mode=clbm_lib.PERTURB_UNIFORM,
                         eps=1e-4, seed=7)
    with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=T) as s:
        s.set_step_variant(4)
        s.init_equilibrium(0, u0, 1e-3, 7)
        ref = s.run_sampler(T, 4)
        ref_state = [s.dump(0, j) for j in range(nc)]
    with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=T, flags=clbm_lib.FLAG_GRAPH) as s:
        s.set_step_variant(temporal_variant(2, 0))
        s.init_equilibrium(0, u0, 1e-3, 7)
        rv = [s.run_sampler(T, 2)]
        s.set_step_variant(4)
        rv.append(s.run_sampler(T, 1))
        s.set_step_variant(temporal_variant(1, 1))
        rv.append(s.run_sampler(T, 1))
        assert s.error_word() == 0
        assert np.array_equal(np.concatenate(rv, axis=1), ref)
        for j in range(nc):
            assert np.array_equal(s.dump(0, j), ref_state[j])


@pytest.mark.parametrize("cs,rows", [(4, None), (3, [24, 16, 24])])
def test_bench_lattice_at_bench_shape(gpu, clbm_lib, orc, cs, rows):
    """The bench's clone lattice (256x64, square 12) at the bench's interval
    length and the shapes the autotuner picks there (cluster size 4, and
    cluster size 3 with the square's band 16 rows high, 1024 threads):
    bit-identical to the streaming kernel, and mass conserved (bounce-back and
    the body force keep sum f; FP32 rounding only)."""
    from clbm import configs
    r = configs.WORKLOADS["c3"]().runs[0]
    g = orc.channel_geom(r.width, r.height, r.side, r.xc, r.yc)
    d = clbm_lib.RunDesc(width=g.nx, height=g.ny, xmin=g.xmin, xmax=g.xmax, ymin=g.ymin, ymax=g.ymax,
                         nclones=8, ranks=1, tau=r.tau, beta=r.beta, alpha=r.k, force_scale=1.0 / r.F0,
                         dt=r.dt, perturb_mode=clbm_lib.PERTURB_UNIFORM, eps=1e-3, seed=5)
    T = 100
    out = []
    for variant in (7, temporal_variant(cs, 0)):
        with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=T) as s:
            s.set_step_variant(variant)
            if rows and variant != 7:
                s.set_band_rows(0, rows)
                assert list(s.band_rows(0)) == rows
            s.init_equilibrium(0, r.u0, 1e-3, 9)
            m0 = [s.dump(0, j).sum() for j in range(8)]
            s.run_interval(T)
            res = [s.drag(0)] + [s.dump(0, j) for j in range(8)]
            for j in range(8):
                assert abs(res[1 + j].sum() - m0[j]) < 1e-6 * m0[j]
            s.clone_step()
            s.run_interval(T)
            res += [s.drag(0)] + [s.dump(0, j) for j in range(8)]
            assert s.error_word() == 0
            out.append(res)
    for a, b in zip(*out):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("W,H,side,xc,yc,cs,tv,rows", [
    (64, 24, 6, 16, 12, 3, 0, [10, 4, 10]),
    (64, 24, 6, 16, 12, 4, 1, [1, 11, 11, 1]),       # one-row bands: both neighbours across CTAs
    (96, 23, 5, 30, 9, 2, 2, [20, 3]),
    (200, 50, 8, 50, 25, 5, 0, [12, 8, 6, 12, 12]),
])
def test_band_split_equals_streaming(gpu, clbm_lib, orc, W, H, side, xc, yc, cs, tv, rows):
    """Uneven band splits (set through clbm_set_band_rows), in eager and
    graph-captured intervals: bit-identical to the streaming kernel."""
    g = orc.channel_geom(W, H, side, xc, yc)
    u0, nc, T = 0.05, 4, 21
    d = clbm_lib.RunDesc(width=g.nx, height=g.ny, xmin=g.xmin, xmax=g.xmax, ymin=g.ymin, ymax=g.ymax,
                         nclones=nc, ranks=1, tau=0.57, beta=side * u0 * u0 / ((W - 1) * (H - 1)), alpha=8.0,
                         force_scale=2 / (u0 * u0 * side), dt=u0 / side, perturb_mode=clbm_lib.PERTURB_UNIFORM,
                         eps=1e-4, seed=7)
    with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=T) as s:
        s.set_step_variant(4)
        s.init_equilibrium(0, u0, 1e-3, 7)
        ref = s.run_sampler(T, 3)
        ref_state = [s.dump(0, j) for j in range(nc)]
    for flags in (0, clbm_lib.FLAG_GRAPH):
        with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=T, flags=flags) as s:
            s.set_step_variant(temporal_variant(cs, tv))
            assert s.band_rows(0).sum() == H and len(s.band_rows(0)) == cs
            s.set_band_rows(0, rows)
            assert list(s.band_rows(0)) == rows
            s.init_equilibrium(0, u0, 1e-3, 7)
            rv = [s.run_sampler(T, 2)]
            s.set_band_rows(0, [])  # back to the even split between captured intervals
            rv.append(s.run_sampler(T, 1))
            assert s.error_word() == 0
            assert np.array_equal(np.concatenate(rv, axis=1), ref)
            for j in range(nc):
                assert np.array_equal(s.dump(0, j), ref_state[j])


def test_band_rows_checks(gpu, clbm_lib, orc):
    g = orc.channel_geom(64, 24, 6, 16, 12)
    d = clbm_lib.RunDesc(width=g.nx, height=g.ny, xmin=g.xmin, xmax=g.xmax, ymin=g.ymin, ymax=g.ymax,
                         nclones=2, ranks=1, tau=0.57, beta=1e-6, alpha=1.0, force_scale=1.0, dt=0.01)
    with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=10) as s:
        s.set_step_variant(4)
        assert len(s.band_rows(0)) == 0  # streaming run: no bands
        with pytest.raises(clbm_lib.ClbmError):  # not cluster-resident
            s.set_band_rows(0, [12, 12])
        s.set_step_variant(temporal_variant(2, 0))
        for bad in ([12, 11], [24, 0], [8, 8, 8], [25, -1]):
            with pytest.raises(clbm_lib.ClbmError):
                s.set_band_rows(0, bad)
        s.set_band_rows(0, [5, 19])
        s.set_step_variant(temporal_variant(2, 0))  # a variant change restores the even split
        assert list(s.band_rows(0)) == [12, 12]


@pytest.mark.parametrize("W,H,side,xc,yc,cs,tv,mode,field,T,flags", [
    (64, 24, 6, 16, 12, 2, 0, "uniform", False, 20, 0),
    (96, 23, 5, 30, 9, 3, 1, "mix", False, 22, 1),
    (64, 24, 6, 16, 12, 4, 2, "uniform", True, 20, 1),
    (200, 50, 8, 50, 25, 8, 1, "none", False, 10, 0),
])
def test_fused_reseed_equals_streaming(gpu, clbm_lib, orc, W, H, side, xc, yc, cs, tv, mode, field, T, flags):
    """Every run cluster-resident and an even interval length: the interval
    kernel forms P_0 itself (parent copy, perturbation -- counter-based or
    snapshot mix --, first collision) while loading its clone, with no reseed
    launch (a random-field run keeps the reseed kernel); bit-identical to the
    streaming path, which runs the reseed kernel, over three intervals with
    cloning steps."""
    g = orc.channel_geom(W, H, side, xc, yc)
    u0, nc = 0.05, 6
    pm = {"uniform": clbm_lib.PERTURB_UNIFORM, "mix": clbm_lib.PERTURB_MIX, "none": clbm_lib.PERTURB_NONE}[mode]
    d = clbm_lib.RunDesc(width=g.nx, height=g.ny, xmin=g.xmin, xmax=g.xmax, ymin=g.ymin, ymax=g.ymax,
                         nclones=nc, ranks=1, tau=0.57, beta=side * u0 * u0 / ((W - 1) * (H - 1)), alpha=12.0,
                         force_scale=2 / (u0 * u0 * side), dt=u0 / side, perturb_mode=pm,
                         eps=1e-3 if mode == "uniform" else 0.01, seed=3, nsnap=4 if mode == "mix" else 0)
    if field:
        d.field_mode, d.field_steps, d.field_eps, d.field_sigma = 1, 7, 0.2, 6.0
    snaps = np.concatenate([orc.init_equilibrium(g, u0, 2e-2, 5, 0, j) for j in range(4)]) if mode == "mix" else None
    out = []
    for variant in (4, temporal_variant(cs, tv)):
        with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=T, flags=flags) as s:
            s.set_step_variant(variant)
            s.init_equilibrium(0, u0, 1e-3, 7)
            if snaps is not None:
                s.set_snapshots(0, snaps)
            res = []
            for t in range(3):
                s.run_interval(T)
                res.append(s.drag(0))
                s.clone_step()
                cr = s.clone_result(0)
                res.append(cr["labels"].astype(np.float64))
                res.append(cr["weights"])
            res.extend(s.dump(0, j) for j in range(nc))
            assert s.error_word() == 0
            out.append(res)
    # some slot took another's state (the copy is exercised)
    assert any(not np.array_equal(out[0][i], np.arange(nc)) for i in (1, 4, 7))
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_fused_reseed_two_runs(gpu, clbm_lib, orc):
    """Two cluster-resident runs of different lattices in one context (each
    interval kernel forms its own run's P_0, run index and clone base
    included): bit-identical to both runs streaming."""
    u0, T = 0.05, 20
    descs = []
    for (W, H, side, xc, yc, nc, seed) in ((64, 24, 6, 16, 12, 5, 3), (96, 23, 5, 30, 9, 4, 4)):
        g = orc.channel_geom(W, H, side, xc, yc)
        descs.append(clbm_lib.RunDesc(width=g.nx, height=g.ny, xmin=g.xmin, xmax=g.xmax, ymin=g.ymin, ymax=g.ymax,
                                      nclones=nc, ranks=1, tau=0.57, beta=side * u0 * u0 / ((W - 1) * (H - 1)),
                                      alpha=12.0, force_scale=2 / (u0 * u0 * side), dt=u0 / side,
                                      perturb_mode=clbm_lib.PERTURB_UNIFORM, eps=1e-3, seed=seed))
    out = []
    for variants in ([4, 4], [temporal_variant(2, 0), temporal_variant(3, 1)]):
        with clbm_lib.Sampler(descs, clbm_lib.FP32, max_steps=T, flags=clbm_lib.FLAG_GRAPH) as s:
            s.set_run_variants(variants)
            for r in range(2):
                s.init_equilibrium(r, u0, 1e-3, 7 + r)
            rv = s.run_sampler(T, 3)
            res = [rv] + [s.dump(r, j) for r in range(2) for j in range(descs[r].nclones)]
            assert s.error_word() == 0
            out.append(res)
    for a, b in zip(*out):
        assert np.array_equal(a, b)
