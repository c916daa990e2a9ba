"""Per-run interval plans on an uneven batch: runs given a cluster-resident
variant run it concurrently, each on its own stream, while the streaming runs
share one step launch per step through their own descriptor table.  Every
plan must give results bit-identical to the uniform streaming kernel (same
pull rules, same explicitly rounded FP32 arithmetic), eagerly and replayed
as CUDA graphs whose intervals hold the runs as parallel branches."""
import numpy as np
import pytest

from test_gpu_temporal import temporal_variant

pytestmark = pytest.mark.gpu

# (W, H, side, xc, yc, cluster size of its cluster-resident variant)
LATTICES = [(64, 24, 6, 16, 12, 1), (128, 32, 6, 32, 16, 2), (200, 50, 8, 50, 25, 0), (96, 23, 5, 30, 9, 4),
            (72, 40, 8, 20, 20, 0)]


def descs(clbm, orc, nc=4):
    out = []
    for r, (W, H, side, xc, yc, _) in enumerate(LATTICES):
        g = orc.channel_geom(W, H, side, xc, yc)
        u0 = 0.05
        out.append(clbm.RunDesc(width=g.nx, height=g.ny, xmin=g.xmin, xmax=g.xmax, ymin=g.ymin, ymax=g.ymax,
                                nclones=nc + r, ranks=1, tau=0.56, beta=side * u0 * u0 / ((W - 1) * (H - 1)),
                                alpha=6.0 - 3.0 * r, force_scale=2 / (u0 * u0 * side), dt=u0 / side,
                                perturb_mode=clbm.PERTURB_UNIFORM, eps=1e-4, seed=11 + r,
                                drag_mode=r % 2))
    return out


def mixed_plan():
    return [temporal_variant(cs, r % 3) if cs else 4 for r, (*_, cs) in enumerate(LATTICES)]


def run(clbm, orc, setup, flags=0, T=21, n=3):
    d = descs(clbm, orc)
    res = []
    with clbm.Sampler(d, clbm.FP32, max_steps=T, flags=flags) as s:
        setup(s)
        for r in range(len(d)):
            s.init_equilibrium(r, 0.05, 1e-3, 7 + r)
        if flags:
            rv = s.run_sampler(T, n)
            res.append(rv)
            for r in range(len(d)):
                res.append(s.drag(r))
                res.append(s.clone_result(r)["labels"].astype(np.float64))
        else:
            for t in range(n):
                s.run_interval(T)
                res.extend(s.drag(r) for r in range(len(d)))
                s.clone_step()
                res.extend(s.clone_result(r)["labels"].astype(np.float64) for r in range(len(d)))
        for r in range(len(d)):
            res.extend(s.dump(r, j) for j in range(d[r].nclones))
        assert s.error_word() == 0
        variants = s.run_variants()
    return res, variants


def test_mixed_plan_equals_streaming(gpu, clbm_lib, orc):
    base, v0 = run(clbm_lib, orc, lambda s: s.set_step_variant(4))
    assert (v0 == 4).all()
    plan = mixed_plan()
    mixed, v1 = run(clbm_lib, orc, lambda s: s.set_run_variants(plan))
    assert list(v1) == plan
    for a, b in zip(base, mixed):
        assert np.array_equal(a, b)


def test_mixed_plan_in_cuda_graphs(gpu, clbm_lib, orc):
    """Graph replay of the mixed plan (parallel branches) equals eager
    streaming replay; so does a plan switch between captured intervals."""
    base, _ = run(clbm_lib, orc, lambda s: s.set_step_variant(4), flags=clbm_lib.FLAG_GRAPH)
    graph, _ = run(clbm_lib, orc, lambda s: s.set_run_variants(mixed_plan()), flags=clbm_lib.FLAG_GRAPH)
    for a, b in zip(base, graph):
        assert np.array_equal(a, b)


def test_autotuned_plan_is_bit_identical(gpu, clbm_lib, orc):
    base, _ = run(clbm_lib, orc, lambda s: s.set_step_variant(4))
    picked = {}

    def tune(s):
        best, ms = s.autotune(launches=3)
        picked["best"] = best
        assert len(ms) == 8 + 33

    tuned, variants = run(clbm_lib, orc, tune)
    if picked["best"] != clbm_lib.VARIANT_PER_RUN:
        assert (variants == picked["best"]).all()
    for a, b in zip(base, tuned):
        assert np.array_equal(a, b)


def test_run_variant_checks(gpu, clbm_lib, orc):
    d = descs(clbm_lib, orc)
    with clbm_lib.Sampler(d, clbm_lib.FP32, max_steps=10) as s:
        with pytest.raises(clbm_lib.ClbmError):  # two streaming launch variants
            s.set_run_variants([4, 5, 4, 4, 4])
        with pytest.raises(clbm_lib.ClbmError):  # no such variant
            s.set_run_variants([4, 4, 4, 8 + 33, 4])
        assert list(s.run_variants()) == [0] * 5
    with clbm_lib.Sampler(d, clbm_lib.FP64, max_steps=10) as s:
        with pytest.raises(clbm_lib.ClbmError):  # cluster-resident intervals are FP32 only
            s.set_run_variants([temporal_variant(1, 0)] + [0] * 4)
