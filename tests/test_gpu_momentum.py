"""Momentum-exchange drag (drag_mode = CLBM_DRAG_MOMENTUM) on the GPU.

The per-node terms are formed inside the step kernels from the populations
the square bounced back, and summed per clone by a warp-shuffle reduction
whose order the oracle restates, so FP64 mode is checked bit for bit against
the oracle (drag series, genealogy, states).  The FP32 streaming and
cluster-resident kernels must agree with each other bit for bit and with the
FP64 oracle within the FP32 drag tolerance of the stress-integration tests
(1e-5 relative over one interval)."""
import numpy as np
import pytest

from test_gpu_sampler import channel_case, desc, rel
from test_gpu_temporal import temporal_variant

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("resample,k", [(0, 3.0), (1, 1000.0)])
def test_fp64_momentum_exchange_matches_oracle(gpu, clbm_lib, orc, resample, k):
    g, phys, T, n, nc, seed = channel_case(orc, W=72, H=40, side=20, k=k, nc=8)
    states = np.concatenate([orc.init_equilibrium(g, 0.05, 1e-3, seed, 0, j) for j in range(nc)])
    ref = orc.run_sampler(g, states, steps=T, intervals=n, perturb_mode=2, resample_mode=resample,
                          eps=1e-4, seed=seed, drag_mode=1, **phys)
    assert ref["status"] == 0
    d = desc(clbm_lib, g, nc, perturb_mode=2, resample_mode=resample, eps=1e-4, seed=seed,
             drag_mode=clbm_lib.DRAG_MOMENTUM, **phys)
    with clbm_lib.Sampler([d], clbm_lib.FP64, max_steps=T) as s:
        s.init_equilibrium(0, 0.05, 1e-3, seed)
        for t in range(n):
            s.run_interval(T)
            assert np.array_equal(s.drag(0), ref["drag"][t]), f"interval {t}"
            s.clone_step()
            assert np.array_equal(s.clone_result(0)["labels"], ref["labels"][t])
        assert (ref["labels"] != np.arange(nc)).any()
        for j in range(nc):
            np.testing.assert_array_equal(s.dump(0, j), ref["states"][j * 9 * g.nx * g.ny:(j + 1) * 9 * g.nx * g.ny])


def test_mixed_drag_modes_in_one_context(gpu, clbm_lib, orc):
    """One run per drag mode in one context (both reductions in one interval);
    the 20-side square gives 84 perimeter terms, more than one lane stride."""
    cases = [channel_case(orc, W=72, H=40, side=20, nc=6, k=2.0, seed=21),
             channel_case(orc, W=64, H=24, side=6, nc=5, k=-3.0, seed=22)]
    modes = [1, 0]
    refs, descs = [], []
    for r, ((g, phys, T, n, nc, seed), m) in enumerate(zip(cases, modes)):
        st = np.concatenate([orc.init_equilibrium(g, 0.05, 1e-3, seed, r, j) for j in range(nc)])
        refs.append(orc.run_sampler(g, st, steps=T, intervals=n, perturb_mode=2, eps=1e-4, seed=seed,
                                    run=r, drag_mode=m, **phys))
        descs.append(desc(clbm_lib, g, nc, perturb_mode=2, eps=1e-4, seed=seed, drag_mode=m, **phys))
    T, n = cases[0][2], cases[0][3]
    with clbm_lib.Sampler(descs, clbm_lib.FP64, max_steps=T) as s:
        for r, c in enumerate(cases):
            s.init_equilibrium(r, 0.05, 1e-3, c[5])
        for t in range(n):
            s.run_interval(T)
            for r in range(2):
                assert np.array_equal(s.drag(r), refs[r]["drag"][t]), (r, t)
            s.clone_step()
            for r in range(2):
                assert np.array_equal(s.clone_result(r)["labels"], refs[r]["labels"][t])


@pytest.mark.parametrize("W,H,side,xc,yc,cs", [(72, 40, 20, 20, 20, 4), (200, 50, 8, 50, 25, 8)])
def test_fp32_momentum_exchange_both_kernels(gpu, clbm_lib, orc, W, H, side, xc, yc, cs):
    g = orc.channel_geom(W, H, side, xc, yc)
    u0, nc, T, seed = 0.05, 4, 30, 5
    phys = dict(tau=0.56, beta=side * u0 * u0 / ((W - 1) * (H - 1)), alpha=0.0,
                force_scale=2 / (u0 * u0 * side), force_shift=0.0, dt=u0 / side)
    states = np.concatenate([orc.init_equilibrium(g, u0, 1e-3, seed, 0, j) for j in range(nc)])
    ref = orc.run_sampler(g, states, steps=T, intervals=1, drag_mode=1, **phys)
    d = desc(clbm_lib, g, nc, drag_mode=clbm_lib.DRAG_MOMENTUM, **phys)
    out = []
    for variant in (4, temporal_variant(cs, 0)):
        with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=T) as s:
            s.set_step_variant(variant)
            s.load_run(0, states)
            s.run_interval(T)
            out.append(s.drag(0))
            assert s.error_word() == 0
    assert np.array_equal(out[0], out[1])
    assert rel(out[0], ref["drag"][0]) < 1e-5


def test_momentum_exchange_needs_a_solid_square(gpu, clbm_lib, orc):
    g = orc.channel_geom(40, 20, 1, 10, 10)
    d = desc(clbm_lib, g, 2, tau=0.6, drag_mode=clbm_lib.DRAG_MOMENTUM)
    with pytest.raises(clbm_lib.ClbmError):
        clbm_lib.Sampler([d], clbm_lib.FP64, max_steps=4)
