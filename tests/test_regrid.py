"""Regrid on the GPU against the oracle's restatement (GPU).

* mbg_tag_cells (ErrorEst with AMReX's AMRErrorTag: value_greater /
  value_less on a macro field or is_fluid, boxes, time windows, max_level)
  gives the oracle's tags bit for bit, before any step (moments of the
  stored state) and after steps (the moments the last collision started
  from, the reference's m_macrodata).
* mbg_regrid (RemakeLevel / MakeNewLevelFromCoarse / ClearLevel: old values
  where an old box held the cell, conservative linear interpolation from the
  coarse level elsewhere) matches the oracle's regrid at 1e-12 right after
  the regrid and after further steps, for a moved fine level, an added third
  level and dropped fine levels; the 16-bit forms stay within their storage
  tolerance of FP64.
* The drop-in driver's regrid (tags on the GPU, grids rebuilt, levels
  remade) continues bit-identically to the oracle fed the same grids.
All on the two-level 32^3 Gaussian pulse at RT = 0.1 (stable).
"""
import numpy as np
import pytest

import cases
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _case():
    return cases.gaussian_pulse(nc=32, fine_lo=8, fine_hi=23, mgs=16, width=3.0, t0=0.1)


def _ctx(o, p, levels, prec=0):
    import marbles_gb300 as M
    c = M.Context(cases.mbg_params_from(p, prec))
    for lev, b in enumerate(levels):
        c.define_level(lev, b, o.get_grown_flags(lev))
        f, g = o.get_state(lev)
        c.set_state(lev, f, g)
    return c


def _rel(a, b):
    s = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) / s if s > 0 else float(np.max(np.abs(a - b)))


def _compare_states(c, o, nlev, rtol=RTOL):
    worst = 0.0
    for lev in range(nlev):
        fg, gg = c.get_state(lev)
        fo, go = o.get_state(lev)
        assert fg.shape == fo.shape, lev
        assert np.isfinite(fg).all() and np.isfinite(gg).all()
        worst = max(worst, _rel(fg, fo), _rel(gg, go))
    assert worst <= rtol, worst


def _tag_pairs():
    import marbles_gb300 as M
    crit = [("rho", "greater", 1.0005, None, -1e300, 1e300, 1000),
            ("temperature", "less", 0.09999, None, -1e300, 1e300, 1000),
            ("vel_mag", "greater", 1e-5, ((10.0, 10.0, 10.0), (22.0, 22.0, 22.0)), -1e300, 1e300, 1000),
            ("rho", "box", 0.0, ((2.0, 2.0, 2.0), (5.5, 5.0, 4.0)), 0.0, 100.0, 1),
            ("pxx", "greater", 0.1, None, 50.0, 100.0, 1000)]
    gpu = [M.make_tag(f, k, v, box, t0, t1, ml) for f, k, v, box, t0, t1, ml in crit]
    orc = [O.make_tag(M.FIELDS.index(f), {"box": 0, "greater": 1, "less": 2}[k], v, box, t0, t1, ml)
           for f, k, v, box, t0, t1, ml in crit]
    return gpu, orc


def test_tags_match_oracle():
    p, levels = _case()
    o = cases.run_oracle(p, levels, 0)
    c = _ctx(o, p, levels)
    gt, ot = _tag_pairs()
    for steps, time in ((0, 0.0), (3, 3.0)):
        if steps:
            c.step(steps)
            o.step(steps)
        for lev in range(2):
            a = c.tag_cells(lev, gt, time)
            b = o.tag_cells(lev, ot, time)
            assert a.sum() > 0, (lev, steps)
            assert np.array_equal(a, b), (lev, steps, int(a.sum()), int(b.sum()))


def test_regrid_moves_adds_and_drops_levels():
    p, levels = _case()
    o = cases.run_oracle(p, levels, 0)
    c = _ctx(o, p, levels)
    c.step(3)
    o.step(3)
    # the fine level moved (overlapping the old one) and a third level added
    new1 = cases.chop([2 * 6, 2 * 10, 2 * 8], [2 * 21 + 1, 2 * 25 + 1, 2 * 23 + 1], 16)
    new2 = cases.chop([2 * 24, 2 * 28, 2 * 24], [2 * 36 - 1, 2 * 40 - 1, 2 * 36 - 1], 16)
    c.regrid(1, [new1, new2])
    o.regrid(1, [new1, new2])
    _compare_states(c, o, 3)
    c.step(4)
    o.step(4)
    _compare_states(c, o, 3)
    # back to one level
    c.regrid(1, [])
    o.regrid(1, [])
    c.step(2)
    o.step(2)
    _compare_states(c, o, 1)


@pytest.mark.parametrize("prec", [1, 2])
def test_regrid_16bit_forms(prec):
    p, levels = _case()
    o = cases.run_oracle(p, levels, 0)
    c64 = _ctx(o, p, levels)
    c16 = _ctx(o, p, levels, prec)
    new1 = cases.chop([2 * 6, 2 * 10, 2 * 8], [2 * 21 + 1, 2 * 25 + 1, 2 * 23 + 1], 16)
    for c in (c64, c16):
        c.step(3)
        c.regrid(1, [new1])
        c.step(3)
    tol = {1: 1e-4, 2: 1e-3}[prec]
    for lev in range(2):
        a = c16.get_macro(lev).reshape(-1)
        r = c64.get_macro(lev).reshape(-1)
        off = 0
        for b in (levels[0] if lev == 0 else new1):
            vol = int(np.prod(b[3:] - b[:3] + 1))
            A, R = a[off:off + 19 * vol].reshape(19, vol), r[off:off + 19 * vol].reshape(19, vol)
            assert np.max(np.abs(A[0] - R[0]) / R[0]) <= tol, lev
            off += 19 * vol


def _moving_inputs():
    """The 32^3 pulse with tagging on state fields and time windows: rho >
    1.0015 until t = 2 (the fine level around the pulse, tagged on the initial
    state), then rho > 1.0005 and a box towards the low corner from t = 3:
    the fine level must move and grow at a regrid after step 3."""
    import inputs
    text = inputs.pulse(nc=32, lo=8, hi=24, mgs=16, width=3.0, t0=0.1)
    return text.replace("tagging.refinement_indicators = centre",
                        "tagging.refinement_indicators = early late corner\n"
                        "tagging.early.field_name = rho\ntagging.early.value_greater = 1.0015\n"
                        "tagging.early.end_time = 2.0\n"
                        "tagging.late.field_name = rho\ntagging.late.value_greater = 1.0005\n"
                        "tagging.late.start_time = 3.0\n"
                        "tagging.corner.in_box_lo = 6.0 6.0 8.0\ntagging.corner.in_box_hi = 10.0 9.0 12.0\n"
                        "tagging.corner.start_time = 3.0")


def test_driver_regrid_continues_like_the_oracle():
    """Field tagging picks the fine level from the initial state; after 3
    steps an explicit regrid moves it; the oracle, given the driver's grids at
    the same points, ends in the same state."""
    import marbles_gb300 as M
    d = M.LBM(_moving_inputs())
    ctx = d.init()
    g0 = [d.boxes(l) for l in range(d.num_levels())]
    assert len(g0) == 2
    p, _ = _case()
    o = O.Oracle(p, g0)
    o.init()
    d.evolve(3)
    o.step(3)
    d.regrid()
    g1 = [d.boxes(l) for l in range(d.num_levels())]
    moved = len(g1) != len(g0) or any(a.shape != b.shape or (a != b).any() for a, b in zip(g0[1:], g1[1:]))
    assert moved, "the pulse spread but the fine level did not change"
    o.regrid(1, g1[1:])
    d.evolve(3)
    o.step(3)
    _compare_states(ctx, o, len(g1))


def test_driver_regrid_interval():
    import marbles_gb300 as M
    text = _moving_inputs().replace("amr.regrid_int = 1000000", "amr.regrid_int = 2")
    d = M.LBM(text)
    ctx = d.init()
    n0 = sum(int(np.prod(b[3:] - b[:3] + 1)) for b in d.boxes(1))
    d.evolve(8)
    n1 = sum(int(np.prod(b[3:] - b[:3] + 1)) for b in d.boxes(1)) if d.num_levels() > 1 else 0
    assert n1 != n0
    for lev in range(d.num_levels()):
        f, g = ctx.get_state(lev)
        assert np.isfinite(f).all() and np.isfinite(g).all()
