"""The drop-in driver's host work against the oracle (CPU only): box
bookkeeping, is_fluid flags and initial states must be bit-identical."""
import math

import numpy as np
import pytest

import cases
import inputs
from oracle import oracle as O


def _driver(text):
    import marbles_gb300 as M
    d = M.LBM(text)
    d.prepare()
    return d


def test_taylor_green_boxes_and_initial_state():
    d = _driver(inputs.tg(64, 32))
    p, levels = cases.taylor_green(64, 32)
    assert np.array_equal(d.boxes(0), levels[0])
    o = O.Oracle(p, levels)
    o.init()
    fd, gd = d.initial_state(0)
    fo, go = o.get_state(0)
    assert np.array_equal(fd, fo) and np.array_equal(gd, go)


def test_uneven_chop_matches_max_size_restatement():
    d = _driver(inputs.tg(40, 16))
    assert np.array_equal(d.boxes(0), O.chop_domain([40, 40, 40], 16))


def test_pulse_grids_and_fine_initial_state():
    d = _driver(inputs.pulse(nc=32, lo=8, hi=24, mgs=16, width=3.0))
    p, levels = cases.gaussian_pulse(nc=32, fine_lo=8, fine_hi=23, mgs=16, width=3.0)
    assert d.num_levels() if hasattr(d, "num_levels") else True
    assert np.array_equal(d.boxes(0), levels[0])
    assert np.array_equal(d.boxes(1), levels[1])
    o = O.Oracle(p, levels)
    o.init()
    fd, gd = d.initial_state(1)
    fo, go = o.get_state(1)
    assert np.array_equal(fd, fo) and np.array_equal(gd, go)


@pytest.mark.parametrize("maxlev", [0, 1, 2])
def test_sphere_flags_match_oracle(maxlev):
    text = inputs.sphere(nx=64, ny=32, nz=32, r=5.0, c=(24.0, 16.0, 16.0), maxlev=maxlev, mgs=16, buf=2)
    d = _driver(text)
    levels = [d.boxes(l) for l in range(d.num_levels())]
    assert len(levels) == maxlev + 1
    p, _ = cases.sphere_channel(64, 32, 32, radius=5.0, center=(24.0, 16.0, 16.0), mgs=16)
    o = O.Oracle(p, levels)
    o.init()
    for lev in range(len(levels)):
        assert np.array_equal(d.flags(lev), o.get_grown_flags(lev)), lev
    fd, gd = d.initial_state(len(levels) - 1)
    fo, go = o.get_state(len(levels) - 1)
    assert np.array_equal(fd, fo) and np.array_equal(gd, go)


def test_fine_levels_nest_and_contain_the_sphere():
    d = _driver(inputs.sphere(nx=64, ny=32, nz=32, r=5.0, c=(24.0, 16.0, 16.0), maxlev=2, mgs=16, buf=2))
    for lev in (1, 2):
        b = d.boxes(lev)
        assert (b[:, 0:3] % 8 == 0).all() and ((b[:, 3:6] + 1) % 8 == 0).all()   # blocking factor
        assert (b[:, 3:6] - b[:, 0:3] + 1 <= 16).all()                          # max_grid_size
        # every solid cell of level lev-1 is covered by level lev
        fl = d.flags(lev - 1)
        crse = d.boxes(lev - 1)
        off = 0
        for cb in crse:
            n = cb[3:6] - cb[0:3] + 7
            a = fl[off:off + int(np.prod(n))].reshape(n[2], n[1], n[0])
            off += int(np.prod(n))
            solid = np.argwhere((a[3:-3, 3:-3, 3:-3] & 1) == 0)
            for k, j, i in solid:
                c = np.array([i, j, k]) + cb[0:3]
                inside = ((b[:, 0:3] <= 2 * c) & (2 * c <= b[:, 3:6])).all(axis=1)
                assert inside.any()


def test_inputs_overrides_and_errors():
    import marbles_gb300 as M
    d = M.LBM(inputs.tg(16, 8), ["amr.max_grid_size=16"])
    d.prepare()
    assert len(d.boxes(0)) == 1
    with pytest.raises(M.MbgError, match="ic_type"):
        M.LBM(inputs.tg(16, 8).replace('lbm.ic_type = "taylorgreen"', ""))
    with pytest.raises(M.MbgError, match="velocity BC"):
        M.LBM(inputs.sphere().replace('lbm.velocity_bc_type = "constant"', ""))
    with pytest.raises(M.MbgError, match="periodic"):
        M.LBM(inputs.tg(16, 8).replace("lbm.bc_lo = 0 0 0", "lbm.bc_lo = 1 0 0"))
