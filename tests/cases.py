"""Workload definitions shared by the tests and the benchmark.

Each case gives the oracle's parameter block, the box lists of every level
and the matching mbg_params of the CUDA library.  Inputs are synthetic (the
reference's analytic initial conditions or the seeded ones of the workloads).
"""
import math

import numpy as np

from oracle import oracle as O

R_U = 28.96


def chop(lo, hi, mgs):
    """Chop the box [lo, hi] like BoxArray::maxSize (oracle restatement)."""
    n = [hi[d] - lo[d] + 1 for d in range(3)]
    b = O.chop_domain(n, mgs).copy()
    b[:, 0:3] += lo
    b[:, 3:6] += lo
    return b


def mbg_params_from(p, precision=0):
    import marbles_gb300 as M
    q = M.default_params()
    q.n_cell[:] = list(p.n_cell)
    q.prob_lo[:] = list(p.prob_lo)
    q.prob_hi[:] = list(p.prob_hi)
    q.is_periodic[:] = list(p.is_periodic)
    q.bc_lo[:] = list(p.bc_lo)
    q.bc_hi[:] = list(p.bc_hi)
    q.nu, q.alpha = p.nu, p.alpha
    q.dx_outer, q.dt_outer = p.dx_outer, p.dt_outer
    q.adiabatic_exponent, q.m_bar = p.adiabatic_exponent, p.m_bar
    q.precision = precision
    q.velbc_type = p.velbc_type
    q.vbc_dir, q.vbc_normal_dir, q.vbc_tangential_dir = p.vbc_dir, p.vbc_normal_dir, p.vbc_tangential_dir
    sos = math.sqrt(p.vbc_adiabatic_exponent * (R_U / p.vbc_m_bar) * p.vbc_initial_temperature)
    q.vbc_u_ref = p.vbc_mach_ref * sos
    q.vbc_initial_density = p.vbc_initial_density
    q.vbc_initial_temperature = p.vbc_initial_temperature
    q.vbc_adiabatic_exponent = p.vbc_adiabatic_exponent
    q.vbc_m_bar = p.vbc_m_bar
    q.rho_ref = 1.0
    q.t_ref = p.initial_temperature
    if p.ic_type == O.IC_TYPES["constant"]:
        sos = math.sqrt(p.ic_adiabatic_exponent * (R_U / p.ic_m_bar) * p.ic_initial_temperature)
        q.u_ref[:] = [p.ic_mach[d] * sos for d in range(3)]
    return q


def taylor_green(n=64, mgs=32, nu=0.005, v0=0.05):
    """3D Taylor-Green on [0, 2 pi)^3, periodic, u0 = 0.05, nu = 0.005."""
    p = O.default_params()
    p.n_cell[:] = [n, n, n]
    p.prob_lo[:] = [0.0, 0.0, 0.0]
    p.prob_hi[:] = [2 * math.pi] * 3
    p.is_periodic[:] = [1, 1, 1]
    p.max_grid_size = mgs
    p.nu = nu
    p.alpha = nu
    p.ic_type = O.IC_TYPES["taylorgreen"]
    p.ic_rho0 = 1.0
    p.ic_v0 = v0
    p.ic_omega[:] = [1.0 / math.pi] * 3
    return p, [chop([0, 0, 0], [n - 1] * 3, mgs)]


def gaussian_pulse(nc=128, fine_lo=32, fine_hi=95, mgs=32, nu=0.01, amp=0.01, width=8.0, t0=1.0 / 3.0):
    """Two-level pulse: coarse nc^3 periodic, fine level (ratio 2) over the
    coarse cells [fine_lo, fine_hi]^3; rho = 1 + amp exp(-r^2 / (2 width^2))."""
    p = O.default_params()
    p.n_cell[:] = [nc] * 3
    p.prob_lo[:] = [0.0] * 3
    p.prob_hi[:] = [float(nc)] * 3
    p.is_periodic[:] = [1, 1, 1]
    p.max_grid_size = mgs
    p.nu = nu
    p.alpha = nu
    p.ic_type = O.IC_TYPES["gaussian_pulse"]
    p.ic_density = 1.0
    p.ic_pulse_amplitude = amp
    p.ic_pulse_width = width
    p.ic_pulse_center[:] = [nc / 2.0] * 3
    p.ic_initial_temperature = t0
    p.initial_temperature = t0
    lev0 = chop([0, 0, 0], [nc - 1] * 3, mgs)
    lev1 = chop([2 * fine_lo] * 3, [2 * fine_hi + 1] * 3, mgs)
    return p, [lev0, lev1]


def sphere_channel(nx=64, ny=32, nz=32, radius=6.0, center=(20.0, 16.0, 16.0), mgs=16, nu=0.016,
                   mach=0.0670820, levels=1, bc_lo=(2, 0, 0), bc_hi=(5, 0, 0), t0=1.0 / 3.0, velbc="constant",
                   normal_dir=1, tangential_dir=0):
    """Flow past a sphere: velocity inflow at x-lo, outflow at x-hi,
    periodic in y and z, constant velocity BC with u = Mach * c_s (or the
    Channel / Parabolic profiles of Source/VelocityBC.H)."""
    p = O.default_params()
    p.n_cell[:] = [nx, ny, nz]
    p.prob_lo[:] = [0.0] * 3
    p.prob_hi[:] = [float(nx), float(ny), float(nz)]
    p.is_periodic[:] = [0 if (bc_lo[d] or bc_hi[d]) else 1 for d in range(3)]
    p.bc_lo[:] = list(bc_lo)
    p.bc_hi[:] = list(bc_hi)
    p.max_grid_size = mgs
    p.nu = nu
    p.alpha = nu
    p.velbc_type = O.VBC_TYPES[velbc]
    p.vbc_dir = 0
    p.vbc_normal_dir = normal_dir
    p.vbc_tangential_dir = tangential_dir
    p.vbc_mach_ref = mach
    p.vbc_initial_temperature = t0
    p.ic_initial_temperature = t0
    p.initial_temperature = t0
    p.ic_type = O.IC_TYPES["constant"]
    p.ic_density = 1.0
    p.ic_mach[:] = [mach, 0.0, 0.0]
    p.eb_type = O.EB_TYPES["sphere"]
    p.sphere_radius = radius
    p.sphere_center[:] = list(center)
    p.sphere_has_fluid_inside = 0
    boxes = [chop([0, 0, 0], [nx - 1, ny - 1, nz - 1], mgs)]
    # static refinement around the sphere: each level covers the sphere's
    # bounding box plus a buffer, in units of the level above
    lo = np.floor(np.array(center) - radius).astype(int)
    hi = np.ceil(np.array(center) + radius).astype(int) - 1
    for lev in range(1, levels):
        buf = 4 if lev == 1 else 3
        r = 2 ** lev
        flo = (lo * r - buf * r) // 8 * 8
        fhi = ((hi + 1) * r + buf * r + 7) // 8 * 8 - 1
        boxes.append(chop(list(flo), list(fhi), mgs))
    return p, boxes


def run_oracle(p, levels, nsteps):
    o = O.Oracle(p, levels)
    o.init()
    if nsteps:
        o.step(nsteps)
    return o


def tg_domain(nx, ny, nz, nu, v0):
    """One Taylor-Green domain on [0, 2 pi)^3 with nx x ny x nz cells (one box)."""
    p, _ = taylor_green(max(nx, ny, nz), max(nx, ny, nz), nu=nu, v0=v0)
    p.n_cell[:] = [nx, ny, nz]
    return p, [chop([0, 0, 0], [nx - 1, ny - 1, nz - 1], max(nx, ny, nz))]


from inputs import batch_domains  # noqa: E402  (the batched Taylor-Green instances)
