"""The oracle's momentum-exchange drag (CLBM_DRAG_MOMENTUM), on the CPU.

The reference integrates the stress over the square's perimeter
(src/lbm_src/force.cpp:8-144); momentum exchange over the bounced links is
the other usual estimator of the force on a bounce-back body, and libclbm
offers it as a run option.  The oracle restates it in libclbm's
order (per-node terms in the stress integration's West/East/North/South node
order, 32 strided lane partials, xor butterfly) so the GPU can be checked bit
for bit in FP64.  Here: that restatement against a plain-Python one, its
rest-state cancellation, and its agreement with the stress integration on a
developing channel flow."""
import ctypes as C

import numpy as np
import pytest

CX = [0, 1, 0, -1, 0, 1, -1, -1, 1]


def me_python(orc, g, f):
    """Momentum exchange written out in Python floats (IEEE double)."""
    H = g.ny

    def node(x, y):
        m = orc.lib().orc_bounce_mask(C.byref(g), x, y)
        v = 0.0
        for k in range(1, 9):
            if CX[k] == 0 or not (m >> k) & 1:
                continue
            fk = float(f[k + 9 * (y + H * x)])
            v = v + (fk + fk) if CX[k] < 0 else v - (fk + fk)
        return v

    terms = [node(g.xmin, y) for y in range(g.ymin, g.ymax + 1)]
    terms += [node(g.xmax, y) for y in range(g.ymin, g.ymax + 1)]
    for yy in (g.ymax, g.ymin):
        terms += [0.0 if x in (g.xmin, g.xmax) else node(x, yy) for x in range(g.xmin, g.xmax + 1)]
    lane = [0.0] * 32
    for l in range(32):
        for j in range(l, len(terms), 32):
            lane[l] = lane[l] + terms[j]
    o = 16
    while o:
        lane = [lane[l] + lane[l ^ o] for l in range(32)]
        o >>= 1
    return lane[0]


@pytest.mark.parametrize("geom", [(40, 24, 8, 12, 12), (61, 37, 20, 25, 18), (33, 17, 3, 10, 8)])
def test_oracle_matches_python_restatement(orc, geom):
    W, H, s, xc, yc = geom
    g = orc.channel_geom(W, H, s, xc, yc)
    rng = np.random.default_rng(W * H)
    f = (np.tile(orc.W, W * H) * (1 + 0.05 * rng.standard_normal(9 * W * H)))
    assert orc.force_momentum_exchange(g, f) == me_python(orc, g, f)


def test_rest_state_carries_no_momentum(orc):
    g = orc.channel_geom(64, 32, 10, 20, 16)
    f = np.tile(orc.W, 64 * 32)
    assert abs(orc.force_momentum_exchange(g, f)) < 1e-15


def test_agrees_with_stress_integration_on_a_developing_flow(orc):
    """The 16-clone plain run's channel (200 x 50, square 8 at (50, 25),
    u0 = 0.05, tau = 0.56), one clone from the synthetic equilibrium: over
    steps 3000-4000 the two estimators' mean drags agree within 10 %."""
    W, H, s, u0, tau = 200, 50, 8, 0.05, 0.56
    g = orc.channel_geom(W, H, s, 50, 25)
    beta = s * u0 * u0 / ((W - 1) * (H - 1))
    F0 = u0 * u0 * s / 2
    st = orc.init_equilibrium(g, u0, 1e-4, 1, 0, 0)
    drag = {}
    for mode in (0, 1):
        o = orc.run_sampler(g, st, steps=4000, intervals=1, tau=tau, beta=beta, alpha=0.0,
                            force_scale=1 / F0, force_shift=0.0, dt=u0 / s, drag_mode=mode)
        assert o["status"] == 0
        drag[mode] = o["drag"][0, 0]
    a, b = drag[0][3000:].mean(), drag[1][3000:].mean()
    assert a > 1.0 and b > 1.0
    assert abs(b - a) / a < 0.1


def test_sampler_uses_the_mode(orc):
    """drag_mode = 1 in the sampler is orc_force_momentum_exchange of each
    streamed state (checked on the first step of one clone)."""
    g = orc.channel_geom(48, 20, 6, 14, 10)
    st = orc.init_equilibrium(g, 0.05, 1e-3, 3, 0, 0)
    o = orc.run_sampler(g, st, steps=1, intervals=1, tau=0.6, beta=1e-5, alpha=0.0,
                        force_scale=1.0, force_shift=0.0, dt=1.0, drag_mode=1)
    new, *_ = orc.lbm_step(g, st, 1e-5, 0.6)
    assert o["drag"][0, 0, 0] == orc.force_momentum_exchange(g, new)
