"""Boundary conditions of Source/BC.H and Source/VelocityBC.H on the GPU
against the oracle (FP64 at 1e-12; the 16-bit forms within tolerance of
FP64): the pressure outlet (code 3, BC.H:222-321, the energy lattice at the
fixed outlet density 1) and the Channel and Parabolic velocity profiles
(VelocityBC.H:90-199).  All at RT = 0.03, a stable temperature of the scheme
(tests/test_stability.py)."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

RTOL = 1e-12

BC_CASES = {
    # velocity inflow, pressure outlet, periodic y and z, sphere in the flow
    "velocity_pressure": dict(bc_lo=(2, 0, 0), bc_hi=(3, 0, 0)),
    # pressure on both x faces, constant velocity functor (rho_bc, T)
    "pressure_pressure": dict(bc_lo=(3, 0, 0), bc_hi=(3, 0, 0)),
    # pressure outlet across y, velocity inflow across x, z periodic... the
    # pressure faces need periodic tangential directions, so x is periodic here
    "pressure_y": dict(bc_lo=(0, 2, 0), bc_hi=(0, 3, 0)),
    # Channel profile inflow between no-slip walls in y and z
    "channel_profile": dict(bc_lo=(2, 1, 1), bc_hi=(5, 1, 1), velbc="channel"),
    # Parabolic profile (normal y, tangential x) between y walls, z periodic
    "parabolic_profile": dict(bc_lo=(2, 1, 0), bc_hi=(5, 1, 0), velbc="parabolic", normal_dir=1,
                              tangential_dir=0),
}


def _case(name, levels=1):
    kw = dict(BC_CASES[name])
    return cases.sphere_channel(32, 24, 16, radius=4.0, center=(12.0, 12.0, 8.0), mgs=16, t0=0.03, levels=levels,
                                **kw)


def _pair(p, levels, o, prec):
    import marbles_gb300 as M
    c = M.Context(cases.mbg_params_from(p, prec))
    for lev, b in enumerate(levels):
        c.define_level(lev, b, o.get_grown_flags(lev))
        f, g = o.get_state(lev)
        c.set_state(lev, f, g)
    return c


def _rel(a, b):
    s = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / s) if s > 0 else float(np.max(np.abs(a - b)))


@pytest.mark.parametrize("name", sorted(BC_CASES))
def test_boundary_condition_matches_oracle(name):
    p, levels = _case(name)
    o = cases.run_oracle(p, levels, 0)
    c = _pair(p, levels, o, 0)
    c.step(8)
    o.step(8)
    fg, gg = c.get_state(0)
    fo, go = o.get_state(0)
    assert np.isfinite(fg).all()
    assert _rel(fg, fo) <= RTOL and _rel(gg, go) <= RTOL, (_rel(fg, fo), _rel(gg, go))


def test_pressure_outlet_two_levels():
    p, levels = cases.sphere_channel(48, 32, 32, radius=5.0, center=(16.0, 16.0, 16.0), mgs=16, levels=2, t0=0.03,
                                     bc_lo=(2, 0, 0), bc_hi=(3, 0, 0))
    o = cases.run_oracle(p, levels, 0)
    c = _pair(p, levels, o, 0)
    c.step(4)
    o.step(4)
    for lev in range(2):
        fg, gg = c.get_state(lev)
        fo, go = o.get_state(lev)
        assert _rel(fg, fo) <= RTOL and _rel(gg, go) <= RTOL, lev


@pytest.mark.parametrize("prec", [1, 2])
def test_pressure_outlet_16bit_forms(prec):
    p, levels = _case("velocity_pressure")
    o = cases.run_oracle(p, levels, 0)
    c64 = _pair(p, levels, o, 0)
    c16 = _pair(p, levels, o, prec)
    c64.step(8)
    c16.step(8)
    a = c16.get_macro(0).reshape(-1)
    r = c64.get_macro(0).reshape(-1)
    off = 0
    worst = 0.0
    for b in levels[0]:
        vol = int(np.prod(b[3:] - b[:3] + 1))
        A, R = a[off:off + 19 * vol].reshape(19, vol), r[off:off + 19 * vol].reshape(19, vol)
        fl = R[0] != 0
        worst = max(worst, float(np.max(np.abs(A[0] - R[0])[fl] / R[0][fl])))
        off += 19 * vol
    assert worst <= {1: 2.5e-4, 2: 2e-3}[prec], worst


def test_pressure_with_wall_tangential_sides_is_rejected():
    import marbles_gb300 as M
    p, _ = cases.sphere_channel(32, 24, 16, radius=4.0, center=(12.0, 12.0, 8.0), mgs=16, t0=0.03,
                                bc_lo=(2, 1, 0), bc_hi=(3, 1, 0))
    with pytest.raises(M.MbgError, match="periodic tangential"):
        M.Context(cases.mbg_params_from(p, 0))
