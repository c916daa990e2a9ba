"""GPU parity at the benchmark workloads' own sizes, not toy lattices.

* The plain FP64 cloning run (16 clones of a 200x50 channel, square 8 at
  (50,25), u0 = 0.05, tau = 0.56, k = 0.1, T = 100, 20 cloning steps, uniform
  noise 1e-4 at each clone creation, seed 1) against the oracle for all 20
  intervals: the per-step drag bit for bit and the genealogy exactly (the
  reference loop, src/mpi_LBM_GK_pops_perturb.cpp:424-469, and its cloning
  step, :487-624).
* The 512-clone 400x100 pair, the 4096-clone 256x64 run and the uneven batch
  of eight lattices (square side floor(H/5) at x = W/4, y = H/2): every clone
  of every run advances one interval on the GPU at the full size, and a few
  clones of each run are compared with the oracle -- clones are independent
  within an interval.  FP64 mode: bit for bit (the stated bound is 1e-12
  relative).  FP32 populations: within 1e-5 relative of the FP64 oracle.

The workload table itself (sizes, squares, the floor(H/5) rounding for the
uneven batch, physics) is checked against the workload descriptions on the
CPU in tests/test_configs.py."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _geom(orc, r):
    return orc.channel_geom(r.width, r.height, r.side, r.xc, r.yc)


def test_plain_fp64_run_all_intervals_match_oracle(gpu, clbm_lib, orc):
    from clbm import configs
    wl = configs.c1()
    r = wl.runs[0]
    assert (r.width, r.height, r.side, r.xc, r.yc, r.nclones) == (200, 50, 8, 50, 25, 16)
    assert (r.u0, r.tau, r.k, r.noise, r.seed, wl.steps, wl.intervals) == (0.05, 0.56, 0.1, 1e-4, 1, 100, 20)
    g = _geom(orc, r)
    states = np.concatenate([orc.init_equilibrium(g, r.u0, wl.init_noise, r.seed, 0, j)
                             for j in range(r.nclones)])
    ref = orc.run_sampler(g, states, steps=wl.steps, intervals=wl.intervals, tau=r.tau, beta=r.beta,
                          alpha=r.k, force_scale=1 / r.F0, force_shift=0.0, dt=r.dt,
                          perturb_mode=2, resample_mode=0, eps=r.noise, seed=r.seed)
    assert ref["status"] == 0
    with clbm_lib.Sampler(wl.descs(), clbm_lib.FP64, max_steps=wl.steps) as s:
        s.init_equilibrium(0, r.u0, wl.init_noise, r.seed)
        for t in range(wl.intervals):
            s.run_interval(wl.steps)
            d = s.drag(0)
            assert np.abs(d - ref["drag"][t]).max() <= 1e-12 * np.abs(ref["drag"][t]).max()
            assert np.array_equal(d, ref["drag"][t]), f"interval {t}"
            s.clone_step()
            res = s.clone_result(0)
            assert np.array_equal(res["labels"], ref["labels"][t]), f"interval {t}"
            assert res["rvalue"] == ref["rvalues"][t]
        assert s.error_word() == 0


def _first_interval(clbm_lib, orc, wl, precision, probe):
    got, want = [], []
    with clbm_lib.Sampler(wl.descs(), precision, max_steps=wl.steps) as s:
        for i, r in enumerate(wl.runs):
            s.init_equilibrium(i, r.u0, wl.init_noise, r.seed)
        s.run_interval(wl.steps)
        for i, r in enumerate(wl.runs):
            g = _geom(orc, r)
            d = s.drag(i)
            for j in probe(r.nclones):
                st = orc.init_equilibrium(g, r.u0, wl.init_noise, r.seed, i, j)
                ref = orc.run_sampler(g, st, steps=wl.steps, intervals=1, tau=r.tau, beta=r.beta,
                                      alpha=r.k, force_scale=1 / r.F0, force_shift=0.0, dt=r.dt,
                                      run=i)
                got.append(d[j])
                want.append(ref["drag"][0][0])
        assert s.error_word() == 0
    return np.array(got), np.array(want)


WORKLOADS = ["c2", "c3", "c4"]


@pytest.mark.parametrize("name", WORKLOADS)
def test_first_interval_full_size_fp64(gpu, clbm_lib, orc, name):
    from clbm import configs
    wl = configs.WORKLOADS[name]()
    got, want = _first_interval(clbm_lib, orc, wl, clbm_lib.FP64, lambda n: (0, n // 2, n - 1))
    rel = np.abs(got - want).max() / np.abs(want).max()
    assert rel <= 1e-12
    assert np.array_equal(got, want)


@pytest.mark.parametrize("name", WORKLOADS)
def test_first_interval_full_size_fp32(gpu, clbm_lib, orc, name):
    from clbm import configs
    wl = configs.WORKLOADS[name]()
    got, want = _first_interval(clbm_lib, orc, wl, clbm_lib.FP32, lambda n: (0, n - 1))
    rel = np.abs(got - want).max(axis=1) / np.abs(want).max(axis=1)
    print(f"{name}: FP32 first-interval drag max rel. error per probed clone {rel}")
    assert rel.max() < 1e-5
