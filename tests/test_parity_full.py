"""FP64 CUDA path against the oracle on the workloads at their full sizes (GPU).

The smaller cases of test_parity_fp64.py exercise every code path; these run
the workloads themselves -- the two-level 128^3 + 128^3 Gaussian pulse, the
three-level 256 x 128 x 128 sphere and sampled batch domains at their own
cell counts -- for a few coarse steps, and compare f, g, rho, u and T at
1e-12 relative (the FP64 form is normally bit-identical to the oracle).

Step counts: the literal parameters (RT = 1/3 with nu = 0.002 ... 0.02) are
linearly unstable in the reference scheme (growth 2.1 - 2.4 per step,
test_stability.py), so they run the few steps before round-off grows past
the tolerance; the stable variants (RT = 0.1 for the pulse, RT = 0.03 for
the sphere) run longer.
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _ctx_from_oracle(o, p, levels):
    import marbles_gb300 as M
    ctx = M.Context(cases.mbg_params_from(p, 0))
    for lev, b in enumerate(levels):
        ctx.define_level(lev, b, o.get_grown_flags(lev))
    for lev in range(len(levels)):
        f, g = o.get_state(lev)
        ctx.set_state(lev, f, g)
    return ctx


def _rel(a, b):
    scale = float(np.max(np.abs(b)))
    d = float(np.max(np.abs(a - b)))
    return d / scale if scale > 0 else d


def _compare(ctx, o, nlev):
    worst = 0.0
    for lev in range(nlev):
        fg, gg = ctx.get_state(lev)
        fo, go = o.get_state(lev)
        assert np.isfinite(fg).all() and np.isfinite(gg).all()
        worst = max(worst, _rel(fg, fo), _rel(gg, go))
        del fg, gg, fo, go
        mg = ctx.get_macro(lev).reshape(-1)
        mo = o.get_macro(lev).reshape(-1)
        off = 0
        for b in o.levels[lev]:
            vol = int(np.prod(b[3:] - b[:3] + 1))
            a = mg[off:off + 19 * vol].reshape(19, vol)
            r = mo[off:off + 19 * vol].reshape(19, vol)
            for c in (0, 1, 2, 3, 18):
                worst = max(worst, _rel(a[c], r[c]))
            off += 19 * vol
    return worst


@pytest.mark.parametrize("t0,steps", [(1.0 / 3.0, 5), (0.1, 20)])
def test_two_level_pulse_full_size(t0, steps):
    """Coarse 128^3 periodic + fine 128^3 over the central 64^3 coarse cells,
    max_grid_size 32 (64 + 64 boxes), nu = 0.01: explosion, subcycling and
    coalescence on the workload's own hierarchy."""
    p, levels = cases.gaussian_pulse(t0=t0)
    o = cases.run_oracle(p, levels, 0)
    ctx = _ctx_from_oracle(o, p, levels)
    ctx.step(steps)
    o.step(steps)
    w = _compare(ctx, o, 2)
    assert w <= RTOL, w


def test_sphere_three_levels_full_size():
    """256 x 128 x 128 with the EB sphere (radius 16 at (64, 64, 64)),
    velocity inflow at x-low, outflow at x-high, periodic y and z, nu =
    0.016, three levels refining the cells within 8 of the sphere (the drop-in
    driver's grids from the workload's inputs), at RT = 0.03."""
    import inputs
    import marbles_gb300 as M
    text = inputs.sphere()
    text += "\nic_constant.initial_temperature = 0.03\nvelocity_bc_constant.initial_temperature = 0.03\n"
    d = M.LBM(text)
    d.prepare()
    levels = [d.boxes(lev) for lev in range(d.num_levels())]
    assert len(levels) == 3
    d.close()
    p, _ = cases.sphere_channel(256, 128, 128, radius=16.0, center=(64.0, 64.0, 64.0), mgs=32, t0=0.03)
    o = cases.run_oracle(p, levels, 0)
    ctx = _ctx_from_oracle(o, p, levels)
    ctx.step(3)
    o.step(3)
    w = _compare(ctx, o, 3)
    assert w <= RTOL, w


def test_batch_domains_literal_sizes():
    """16 of the 256 batched Taylor-Green domains (every 16th seed) at their
    own cell counts, velocities and viscosities, one FP64 context each."""
    doms = cases.batch_domains(256)[::16]
    worst = 0.0
    for n, nu, v0 in doms:
        p, levels = cases.tg_domain(*n, nu=nu, v0=v0)
        o = cases.run_oracle(p, levels, 0)
        ctx = _ctx_from_oracle(o, p, levels)
        ctx.step(3)
        o.step(3)
        worst = max(worst, _compare(ctx, o, 1))
        ctx.close()
        o.close()
    assert worst <= RTOL, worst
