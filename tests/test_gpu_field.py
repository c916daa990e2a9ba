"""The forcing variant on the GPU: Gaussian random body-force fields and the
TLGK_LBM_FORCING driver.

The reference draws fields from rand() through FFTW
(generate_random_field.cpp), so parity is statistical: the device fields
must have the covariance of the reference's circulant embedding (restated
here with numpy's FFT, generalised to W x H), and, given the device fields,
the FP64 batched spatial-force stepping must match the oracle's
streamingAndCollisionComputeMacroBodyForceSpatial restatement bit for bit."""
import subprocess

import numpy as np
import pytest

from driver_util import BUILD

pytestmark = pytest.mark.gpu


def embedding_spectrum(W, H, sigma):
    """lambda = Re FFT2(G)/(M1 M2), G[a][b] = c(min(a, M1-a), min(b, M2-b)),
    the reference's block-circulant first row (generate_random_field.cpp:41-110)."""
    M1, M2 = 2 * W - 1, 2 * H - 1
    a = np.minimum(np.arange(M1), M1 - np.arange(M1))
    b = np.minimum(np.arange(M2), M2 - np.arange(M2))
    G = np.exp(-(a[:, None] ** 2 + b[None, :] ** 2) / (2 * sigma ** 2)) / (M1 * M2)
    return np.real(np.fft.fft2(G)), M1, M2


def run_desc(clbm_lib, g, nc, **kw):
    d = clbm_lib.RunDesc(width=g.nx, height=g.ny, xmin=g.xmin, xmax=g.xmax, ymin=g.ymin, ymax=g.ymax,
                         nclones=nc, ranks=1)
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def test_field_covariance_and_determinism(gpu, clbm_lib, orc):
    W, H, sig, nc = 40, 24, 3.0, 256
    g = orc.channel_geom(W, H, 4, 10, 12)
    d = run_desc(clbm_lib, g, nc, tau=0.6, beta=1e-6, field_mode=1, field_steps=1, field_eps=0.1,
                 field_sigma=sig, seed=11, force_scale=1.0, dt=1.0)
    maps = []
    for rep in range(2):
        with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=2) as s:
            s.init_equilibrium(0, 0.02, 1e-3, 1)
            s.run_interval(2)
            maps.append(np.stack([s.field_map(0, j)[0].reshape(W, H) for j in range(nc)]))
    assert np.array_equal(maps[0], maps[1])
    f = maps[0]
    lam, M1, M2 = embedding_spectrum(W, H, sig)
    lam = np.maximum(lam, 0.0)
    for dx, dy in [(0, 0), (1, 0), (0, 1), (3, 0), (0, 3), (2, 2), (6, 0)]:
        expect = np.sum(lam * np.cos(2 * np.pi * (np.arange(M1)[:, None] * dx / M1 + np.arange(M2)[None, :] * dy / M2)))
        emp = np.mean(f[:, : W - dx, : H - dy] * f[:, dx:, dy:])
        assert abs(emp - expect) < 0.08 * max(expect, 0.2), (dx, dy, emp, expect)
    assert abs(f.mean()) < 0.03


def philox4x32_10(c0, c1, c2, c3, seed):
    """Philox4x32-10 (Salmon et al., SC'11), vectorised over counter arrays."""
    M = np.uint64(0xFFFFFFFF)
    c = [np.asarray(v, dtype=np.uint64) & M for v in (c0, c1, c2, c3)]
    k0, k1 = np.uint64(seed & 0xFFFFFFFF), np.uint64(seed >> 32)
    for _ in range(10):
        p0 = np.uint64(0xD2511F53) * c[0]
        p1 = np.uint64(0xCD9E8D57) * c[2]
        c = [((p1 >> np.uint64(32)) ^ c[1] ^ k0) & M, p1 & M, ((p0 >> np.uint64(32)) ^ c[3] ^ k1) & M, p0 & M]
        k0 = (k0 + np.uint64(0x9E3779B9)) & M
        k1 = (k1 + np.uint64(0xBB67AE85)) & M
    return c


def field_fp64(W, H, sigma, seed, clone, interval, run=0):
    """The device's field of (clone, interval) recomputed in FP64: the same
    Philox counters and Box-Muller normals, then map = Re(F1 (s Z) F2) over
    the embedding (the two contractions of the device stages)."""
    lam, M1, M2 = embedding_spectrum(W, H, sigma)
    s = np.sqrt(np.maximum(lam, 0.0))
    s = s.astype(np.float32).astype(np.float64)  # the device keeps sqrt(lambda) in FP32
    a, b = np.meshgrid(np.arange(M1), np.arange(M2), indexing="ij")
    c = philox4x32_10(a * M2 + b, np.full(a.shape, clone), np.full(a.shape, interval),
                      np.full(a.shape, (run << 4) | 4), seed)
    u1 = (c[0].astype(np.float64) + 1.0) * 2.0 ** -32
    u2 = c[1].astype(np.float64) * 2.0 ** -32
    rad = s * np.sqrt(-2.0 * np.log(u1))
    Z = np.where(s != 0, rad * np.exp(2j * np.pi * u2), 0)
    F1 = np.exp(-2j * np.pi * np.outer(np.arange(W), np.arange(M1)) / M1)
    F2 = np.exp(-2j * np.pi * np.outer(np.arange(M2), np.arange(H)) / M2)
    return np.real(F1 @ Z @ F2)  # [x][y]


@pytest.mark.parametrize("W,H,sig", [(40, 24, 3.0), (200, 80, 12.0), (300, 20, 32.0)])
def test_field_transform_against_fp64(gpu, clbm_lib, orc, W, H, sig):
    """The tensor-core stage 1 (TF32 operands, FP32 accumulation) and stage 2
    against the same fields in FP64: every value within 4e-3 of the fields'
    RMS (TF32 keeps 11 significant bits of the operands).  The lattices cover
    one 128-row tile, four tiles with two column tiles (M2 = 159), and two
    passes of row tiles (2W = 600)."""
    g = orc.channel_geom(W, H, 4, W // 4, H // 2)
    nc, seed = 3, 17
    d = run_desc(clbm_lib, g, nc, tau=0.6, beta=1e-6, field_mode=1, field_steps=1, field_eps=0.1,
                 field_sigma=sig, seed=seed, force_scale=1.0, dt=1.0)
    with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=2) as s:
        s.init_equilibrium(0, 0.02, 1e-3, 1)
        for t in range(2):
            s.run_interval(2)
            for j in range(nc):
                got = s.field_map(0, j)[0].reshape(W, H)
                ref = field_fp64(W, H, sig, seed, j, t)
                rms = np.sqrt(np.mean(ref ** 2))
                assert rms > 0.1
                assert np.abs(got - ref).max() < 4e-3 * rms, (t, j, np.abs(got - ref).max() / rms)
            s.clone_step()
        assert s.error_word() == 0


def test_spatial_force_stepping_matches_oracle(gpu, clbm_lib, orc):
    W, H, side, nc, T1, T2 = 48, 20, 5, 3, 6, 5
    g = orc.channel_geom(W, H, side, 12, 10)
    u0 = 0.05
    phys = dict(tau=0.58, beta=side * u0 * u0 / ((W - 1) * (H - 1)), alpha=1.0, force_scale=2 / (u0 * u0 * side),
                force_shift=0.0, dt=u0 / side)
    d = run_desc(clbm_lib, g, nc, field_mode=1, field_steps=T1, field_eps=0.3, field_sigma=8.0, seed=3, **phys)
    states = [orc.init_equilibrium(g, u0, 1e-3, 4, 0, j) for j in range(nc)]
    with clbm_lib.Sampler([d], clbm_lib.FP64, max_steps=T1 + T2) as s:
        s.load_run(0, np.concatenate(states))
        s.run_interval(T1 + T2)
        drag = s.drag(0)
        maps = [s.field_map(0, j)[0] for j in range(nc)]
    for j in range(nc):
        f = states[j]
        for t in range(T1 + T2):
            f = orc.lbm_step(g, f, phys["beta"], phys["tau"], map_=maps[j] if t < T1 else None, eps=0.3)[0]
            F = orc.force(g, f, 1.0 / phys["tau"]) * phys["force_scale"] - 0.0
            assert drag[j, t] == F, (j, t)


def test_forcing_driver_outputs(gpu, clbm_lib, orc, tmp_path):
    import build as b
    b.build_drivers()
    L, Nc, U0, tau, alpha, eps, T, dT, dT0 = 4, 4, 0.05, 0.6, 5.0, 0.2, 1.0, 0.25, 0.1
    g = orc.reference_square_geom(L)
    (tmp_path / "pops").mkdir()
    for j in range(Nc):
        orc.init_equilibrium(g, 0.05, 2e-2, 7, 0, j).tofile(tmp_path / "pops" / f"p{j}.bin")
    (tmp_path / "pops" / "popfiles_list.dat").write_text("".join(f"p{j}.bin\n" for j in range(Nc)))
    (tmp_path / "input").write_text(f"{Nc}\n{T}\n{dT}\n{dT0}\n{eps}\n{L}\n{tau}\n{U0}\n{alpha}\npops/\nout/\n")
    r = subprocess.run([str(BUILD / "TLGK_LBM_FORCING"), "input"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    import math
    T0 = L / U0
    steps = math.floor(dT0 * T0) + math.floor((dT - dT0) * T0)
    nint = math.floor(T / dT)
    out = tmp_path / "out"
    assert np.fromfile(out / "rvalues.dat").size == nint
    for t in range(nint):
        w = np.fromfile(out / f"weights_evolution_{t}")
        cp = np.fromfile(out / f"copies_evolution_{t}", np.int32)
        assert w.size == Nc and cp.size == 2 * Nc and cp[Nc:].sum() == Nc
        for j in range(Nc):
            F = np.fromfile(out / f"clone_{j}" / f"evolution_{t}_clone_{j}")
            assert F.size == steps
            np.testing.assert_allclose(w[j], math.exp(alpha * (F.sum() * (1.0 / T0))), rtol=1e-12)


def test_function_level_random_field(gpu, clbm_lib, orc):
    """clbm_ref_random_field (generate_random_field's drop-in): the field of
    draw t is the sampler's clone-0 field of interval t (same seed and
    lattice), and over many draws it has the embedding's covariance."""
    W, H, sig, seed = 40, 24, 3.0, 11
    g = orc.channel_geom(W, H, 4, 10, 12)
    d = run_desc(clbm_lib, g, 1, tau=0.6, beta=1e-6, field_mode=1, field_steps=1, field_eps=0.1,
                 field_sigma=sig, seed=seed, force_scale=1.0, dt=1.0)
    with clbm_lib.Sampler([d], clbm_lib.FP32, max_steps=2) as s:
        s.init_equilibrium(0, 0.02, 1e-3, 1)
        for t in range(2):
            s.run_interval(2)
            m, neg = clbm_lib.ref_random_field(W, H, sig, seed, t)
            assert np.array_equal(m, s.field_map(0, 0)[0])
            assert neg == s.field_map(0, 0)[1]
            s.clone_step()
    f = np.stack([clbm_lib.ref_random_field(W, H, sig, 5, t)[0].reshape(W, H) for t in range(200)])
    lam, M1, M2 = embedding_spectrum(W, H, sig)
    lam = np.maximum(lam, 0.0)
    for dx, dy in [(0, 0), (1, 0), (0, 1), (3, 0), (2, 2)]:
        expect = np.sum(lam * np.cos(2 * np.pi * (np.arange(M1)[:, None] * dx / M1 + np.arange(M2)[None, :] * dy / M2)))
        emp = np.mean(f[:, : W - dx, : H - dy] * f[:, dx:, dy:])
        assert abs(emp - expect) < 0.1 * max(expect, 0.2), (dx, dy, emp, expect)
    with pytest.raises(clbm_lib.ClbmError):
        clbm_lib.ref_random_field(2000, 24, sig, 1, 0)
