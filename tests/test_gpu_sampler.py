"""Sampler-level parity on the GPU: the batched device sampler (clbm_ctx)
against the oracle and the reference driver's golden outputs.

Tolerances: FP64 mode follows the reference's operation order, so the
per-step drag must agree to 1e-12 relative (it is bit-identical except after
a snapshot-mix perturbation, whose two norms the device reduces in tree
order) and the genealogy (labels) must be identical.  FP32 mode is compared
with the FP64 oracle at the tolerances written in each test."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def desc(clbm, g, nc, **kw):
    d = clbm.RunDesc(width=g.nx, height=g.ny, xmin=g.xmin, xmax=g.xmax, ymin=g.ymin, ymax=g.ymax,
                     nclones=nc, ranks=kw.pop("ranks", 1))
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("i", range(2))
def test_pops_driver_golden(gpu, clbm_lib, orc, i):
    """The reference pops-perturb driver's labels, R_t and force files."""
    z = np.load(GOLD / "pops_driver.npz")
    L, Nc, U0, tau, alpha, eps, T, dT = z["params"][i]
    L, Nc = int(L), int(Nc)
    g = orc.reference_square_geom(L)
    files = [orc.init_equilibrium(g, 0.05, 2e-2, 7, 0, j) for j in range(max(Nc, 10))]
    sc = orc.reference_scalars(L, U0, dT, T)
    d = desc(clbm_lib, g, Nc, tau=tau, beta=sc["beta"], alpha=alpha, force_scale=sc["force_scale"],
             force_shift=1.775, dt=sc["dt"], perturb_mode=clbm_lib.PERTURB_MIX, eps=eps, nsnap=10)
    with clbm_lib.Sampler([d], clbm_lib.FP64, max_steps=sc["steps"]) as s:
        s.load_run(0, np.concatenate(files[:Nc]))
        s.set_snapshots(0, np.concatenate(files[:10]))
        labels, rv, force = [], [], []
        for t in range(sc["intervals"]):
            s.run_interval(sc["steps"])
            force.append(s.drag(0))
            s.clone_step()
            r = s.clone_result(0)
            labels.append(r["labels"])
            rv.append(r["rvalue"])
    force = np.concatenate(force, axis=1)
    assert np.array_equal(np.concatenate(labels), z[f"run{i}_labels"])
    # R_t = mean exp(alpha s): alpha (up to 20 here) amplifies the ulp-level
    # rounding of the tree-ordered perturbation norms
    np.testing.assert_allclose(rv, z[f"run{i}_rvalues"], rtol=1e-11)
    assert rel(force, z[f"run{i}_force"]) < 1e-12
    # before the first perturbation the series is bit-identical
    assert np.array_equal(force[:, :sc["steps"]], z[f"run{i}_force"][:, :sc["steps"]])


def channel_case(orc, W=64, H=24, side=6, nc=8, u0=0.05, tau=0.56, k=2.0, T=40, n=3, seed=1):
    g = orc.channel_geom(W, H, side, W // 4, H // 2)
    beta = side * u0 * u0 / ((W - 1) * (H - 1))
    F0 = u0 * u0 * side / 2
    return g, dict(tau=tau, beta=beta, alpha=k, force_scale=1 / F0, force_shift=0.0, dt=u0 / side), T, n, nc, seed


@pytest.mark.parametrize("resample,k", [(0, 2.0), (1, 100.0)])
def test_fp64_uniform_perturbation_matches_oracle(gpu, clbm_lib, orc, resample, k):
    g, phys, T, n, nc, seed = channel_case(orc, k=k)
    states = np.concatenate([orc.init_equilibrium(g, 0.05, 1e-3, seed, 0, j) for j in range(nc)])
    ref = orc.run_sampler(g, states, steps=T, intervals=n, perturb_mode=2, resample_mode=resample,
                          eps=1e-4, seed=seed, **phys)
    assert ref["status"] == 0
    d = desc(clbm_lib, g, nc, perturb_mode=2, resample_mode=resample, eps=1e-4, seed=seed, **phys)
    with clbm_lib.Sampler([d], clbm_lib.FP64, max_steps=T) as s:
        s.init_equilibrium(0, 0.05, 1e-3, seed)
        assert np.array_equal(s.dump(0, 3), states[3 * 9 * g.nx * g.ny:4 * 9 * g.nx * g.ny])
        for t in range(n):
            s.run_interval(T)
            drag = s.drag(0)
            assert np.array_equal(drag, ref["drag"][t]), f"interval {t}"
            s.clone_step()
            r = s.clone_result(0)
            assert np.array_equal(r["labels"], ref["labels"][t])
            np.testing.assert_allclose(r["rvalue"], ref["rvalues"][t], rtol=1e-14)
        assert (ref["labels"] != np.arange(nc)).any()
        rv, lr = s.rvalues(0)
        np.testing.assert_allclose(lr, ref["logr"], rtol=1e-14, atol=1e-14)
        for j in range(nc):
            np.testing.assert_array_equal(s.dump(0, j), ref["states"][j * 9 * g.nx * g.ny:(j + 1) * 9 * g.nx * g.ny])


def test_zero_bias_keeps_every_clone(gpu, clbm_lib, orc):
    g, phys, T, n, nc, seed = channel_case(orc, k=0.0)
    d = desc(clbm_lib, g, nc, perturb_mode=2, eps=1e-4, seed=3, **phys)
    with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=T) as s:
        s.init_equilibrium(0, 0.05, 1e-3, 3)
        for t in range(n):
            s.run_interval(T)
            s.clone_step()
            r = s.clone_result(0)
            assert np.array_equal(r["labels"], np.arange(nc))
            assert r["rvalue"] == 1.0


def test_virtual_ranks(gpu, clbm_lib, orc):
    g, phys, T, n, nc, seed = channel_case(orc, nc=8, k=6.0)
    files = [orc.init_equilibrium(g, 0.05, 2e-2, 9, 0, j) for j in range(10)]
    states = np.concatenate(files[:nc])
    snaps = np.concatenate(files[:10])
    ref = orc.run_sampler(g, states, steps=T, intervals=n, perturb_mode=1, eps=0.01, snaps=snaps, ranks=2, **phys)
    d = desc(clbm_lib, g, nc, ranks=2, perturb_mode=1, eps=0.01, nsnap=10, **phys)
    with clbm_lib.Sampler([d], clbm_lib.FP64, max_steps=T) as s:
        s.load_run(0, states)
        s.set_snapshots(0, snaps)
        for t in range(n):
            s.run_interval(T)
            assert rel(s.drag(0), ref["drag"][t]) < 1e-12
            s.clone_step()
            assert np.array_equal(s.clone_result(0)["labels"], ref["labels"][t])


def test_uneven_batch_in_one_context(gpu, clbm_lib, orc):
    cases = [channel_case(orc, W=48, H=16, side=4, nc=4, k=3.0, seed=11),
             channel_case(orc, W=72, H=24, side=6, nc=6, k=-2.0, seed=12),
             channel_case(orc, W=40, H=20, side=5, nc=3, k=5.0, seed=13)]
    refs, descs = [], []
    for r, (g, phys, T, n, nc, seed) in enumerate(cases):
        st = np.concatenate([orc.init_equilibrium(g, 0.05, 1e-3, seed, r, j) for j in range(nc)])
        refs.append(orc.run_sampler(g, st, steps=T, intervals=n, perturb_mode=2, eps=1e-4, seed=seed, run=r, **phys))
        descs.append(desc(clbm_lib, g, nc, perturb_mode=2, eps=1e-4, seed=seed, **phys))
    T, n = cases[0][2], cases[0][3]
    with clbm_lib.Sampler(descs, clbm_lib.FP64, max_steps=T) as s:
        for r, c in enumerate(cases):
            s.init_equilibrium(r, 0.05, 1e-3, c[5])
        for t in range(n):
            s.run_interval(T)
            for r in range(len(cases)):
                assert np.array_equal(s.drag(r), refs[r]["drag"][t]), (r, t)
            s.clone_step()
            for r in range(len(cases)):
                assert np.array_equal(s.clone_result(r)["labels"], refs[r]["labels"][t])


@pytest.mark.parametrize("prec", [0, 1])
def test_graph_replay_equals_eager(gpu, clbm_lib, orc, prec):
    g, phys, T, n, nc, seed = channel_case(orc, T=25, n=4, k=4.0)
    d = desc(clbm_lib, g, nc, perturb_mode=2, eps=1e-4, seed=seed, **phys)
    out = []
    for flags in (0, clbm_lib.FLAG_GRAPH):
        with clbm_lib.Sampler([d], prec, max_steps=T, flags=flags) as s:
            s.init_equilibrium(0, 0.05, 1e-3, seed)
            rv = s.run_sampler(T, n)
            out.append((rv, s.clone_result(0)["labels"], s.dump(0, 1)))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][2], out[1][2])


@pytest.mark.parametrize("prec,flags", [(0, 0), (1, 1)])
def test_run_sampler_outputs_equals_per_interval_reads(gpu, clbm_lib, orc, prec, flags):
    """clbm_run_sampler_outputs (outputs staged while the next interval runs)
    delivers exactly what per-interval clbm_run_sampler + clbm_get_drag +
    clbm_get_clone_result read, on an uneven two-run batch."""
    cases = [channel_case(orc, W=48, H=16, side=4, nc=4, k=3.0, T=30, n=5, seed=21),
             channel_case(orc, W=72, H=24, side=6, nc=6, k=-2.0, T=30, n=5, seed=22)]
    descs = [desc(clbm_lib, g, nc, perturb_mode=2, eps=1e-4, seed=seed, **phys)
             for (g, phys, T, n, nc, seed) in cases]
    T, n = 30, 5
    ref = {"drag": [], "labels": [], "weights": [], "rv": []}
    with clbm_lib.Sampler(descs, prec, max_steps=T, flags=flags) as s:
        for r, c in enumerate(cases):
            s.init_equilibrium(r, 0.05, 1e-3, c[5])
        for t in range(n):
            ref["rv"].append(s.run_sampler(T, 1)[:, 0])
            ref["drag"].append(np.concatenate([s.drag(r) for r in range(2)]))
            crs = [s.clone_result(r) for r in range(2)]
            ref["labels"].append(np.concatenate([c["labels"] for c in crs]))
            ref["weights"].append(np.concatenate([c["weights"] for c in crs]))
        ref_state = s.dump(1, 2)
    with clbm_lib.Sampler(descs, prec, max_steps=T, flags=flags) as s:
        for r, c in enumerate(cases):
            s.init_equilibrium(r, 0.05, 1e-3, c[5])
        first = s.run_sampler_outputs(T, 2)
        rest = s.run_sampler_outputs(T, n - 2)
        assert s.error_word() == 0
        assert np.array_equal(s.dump(1, 2), ref_state)
    for key, k2 in (("drag", "drag"), ("labels", "labels"), ("weights", "weights")):
        got = np.concatenate([first[k2], rest[k2]])
        assert np.array_equal(got, np.stack(ref[key])), key
    assert np.array_equal(np.concatenate([first["rvalues"], rest["rvalues"]], axis=1), np.stack(ref["rv"], axis=1))


def test_fp32_against_fp64_oracle(gpu, clbm_lib, orc):
    """FP32 populations (stored as f - w) with FP64 drag integral: first
    interval drag series within 1e-5 relative of the FP64 oracle."""
    g, phys, T, n, nc, seed = channel_case(orc, W=96, H=32, side=8, T=100, n=1)
    states = np.concatenate([orc.init_equilibrium(g, 0.05, 1e-3, seed, 0, j) for j in range(nc)])
    ref = orc.run_sampler(g, states, steps=T, intervals=1, **phys)
    d = desc(clbm_lib, g, nc, **phys)
    with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=T) as s:
        s.load_run(0, states)
        s.run_interval(T)
        err = rel(s.drag(0), ref["drag"][0])
        assert err < 1e-5, err
        s.clone_step()
        # weights exp(alpha s): relative error about alpha * s * (drag error)
        np.testing.assert_allclose(s.clone_result(0)["weights"], ref["weights"][0], rtol=2e-4)


def test_weight_overflow_is_reported(gpu, clbm_lib, orc):
    g, phys, T, n, nc, seed = channel_case(orc, k=1e6)
    d = desc(clbm_lib, g, nc, **phys)
    with clbm_lib.Sampler([d], clbm_lib.FP64, max_steps=T) as s:
        s.init_equilibrium(0, 0.05, 1e-3, 1)
        s.run_interval(T)
        with pytest.raises(clbm_lib.ClbmError) as e:
            s.clone_step()
        assert e.value.status == clbm_lib.ERR_DEVICE
        assert s.error_word(clear=True) & 0x2
        assert np.array_equal(s.clone_result(0)["labels"], np.arange(nc))


def test_step_variants_are_bit_identical_and_autotune_keeps_state(gpu, clbm_lib, orc):
    g, phys, T, n, nc, seed = channel_case(orc, W=200, H=50, side=8, nc=6, T=30, n=1, k=0.5)
    d = desc(clbm_lib, g, nc, perturb_mode=2, eps=1e-4, seed=seed, **phys)
    drags = []
    with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=T) as s:
        s.init_equilibrium(0, 0.05, 1e-3, seed)
        before = s.dump(0, 2)
        best, ms = s.autotune(launches=2)
        # streaming launch variants always run; cluster-resident ones where
        # the lattice fits (-1 otherwise)
        assert 0 <= best < len(ms) and ms[best] > 0 and (ms[:8] > 0).all()
        assert (ms[8:] > 0).any() and ((ms[8:] > 0) | (ms[8:] == -1)).all()
        assert np.array_equal(s.dump(0, 2), before)
        assert s.error_word() == 0
    for v in np.flatnonzero(ms > 0):
        with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=T) as s:
            s.init_equilibrium(0, 0.05, 1e-3, seed)
            s.set_step_variant(int(v))
            s.run_interval(T)
            drags.append(s.drag(0))
            s.clone_step()
    for v in range(1, len(drags)):
        assert np.array_equal(drags[v], drags[0]), v


def test_scgf_and_genealogy_lock(gpu, clbm_lib, orc):
    g, phys, T, n, nc, seed = channel_case(orc, k=3.0, n=4)
    d = desc(clbm_lib, g, nc, perturb_mode=2, eps=1e-4, seed=seed, **phys)
    states = np.concatenate([orc.init_equilibrium(g, 0.05, 1e-3, seed, 0, j) for j in range(nc)])
    ref = orc.run_sampler(g, states, steps=T, intervals=n, perturb_mode=2, eps=1e-4, seed=seed, **phys)
    dT = T * phys["dt"]
    with clbm_lib.Sampler([d], clbm_lib.FP64, max_steps=T) as a, clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=T) as b:
        a.load_run(0, states)
        b.load_run(0, states)
        for t in range(n):
            a.run_interval(T)
            b.run_interval(T)
            a.clone_step()
            b.clone_step()
            b.set_pending_labels(0, a.clone_result(0)["labels"])   # FP32 follows the FP64 genealogy
        psi = a.scgf(0, dT)
        expect = np.sum(ref["logr"]) / (n * dT)
        assert abs(psi - expect) <= 1e-13 * abs(expect)
        psi32 = b.scgf(0, dT)
        assert abs(psi32 - psi) <= 1e-4 * abs(psi)


@pytest.mark.parametrize("flags", [0, 1])
def test_lineage_reconstruction(gpu, clbm_lib, orc, flags):
    """Each final slot's drag series traced back through its ancestors, as
    post_processing/reconstruction.cpp assembles it from labels.dat and the
    slot files, against the oracle's outputs."""
    g, phys, T, n, nc, seed = channel_case(orc, k=6.0, n=5, T=20)
    d = desc(clbm_lib, g, nc, perturb_mode=2, eps=1e-4, seed=seed, **phys)
    states = np.concatenate([orc.init_equilibrium(g, 0.05, 1e-3, seed, 0, j) for j in range(nc)])
    ref = orc.run_sampler(g, states, steps=T, intervals=n, perturb_mode=2, eps=1e-4, seed=seed, **phys)
    anc_ref = np.zeros((nc, n), np.int32)
    series = np.zeros((nc, n * T))
    for j in range(nc):
        slot = j
        for t in range(n - 1, -1, -1):
            anc_ref[j, t] = slot
            series[j, t * T:(t + 1) * T] = ref["drag"][t, slot]
            if t > 0:
                slot = ref["labels"][t - 1, slot]
    assert (anc_ref[:, 0] != np.arange(nc)).any()
    with clbm_lib.Sampler([d], clbm_lib.FP64, max_steps=T, flags=flags) as s:
        s.enable_history(16)
        s.load_run(0, states)
        s.run_sampler(T, n)
        out, anc = s.reconstruct(0, T)
    assert np.array_equal(anc, anc_ref)
    assert np.array_equal(out, series)
