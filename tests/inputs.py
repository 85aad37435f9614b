"""Inputs files (reference keys) for the workloads, as text."""
import math

TG64 = """
max_step = 200
geometry.prob_lo = 0.0 0.0 0.0
geometry.prob_hi = {L} {L} {L}
geometry.is_periodic = 1 1 1
amr.n_cell = {n} {n} {n}
amr.max_level = 0
amr.max_grid_size = {mgs}
lbm.bc_lo = 0 0 0
lbm.bc_hi = 0 0 0
lbm.nu = 0.005
lbm.ic_type = "taylorgreen"
ic_taylorgreen.rho0 = 1.0
ic_taylorgreen.v0 = 0.05
ic_taylorgreen.omega = {w} {w} {w}
eb2.geom_type = "all_regular"
"""


def tg(n=64, mgs=32):
    return TG64.format(L=repr(2 * math.pi), n=n, mgs=mgs, w=repr(1.0 / math.pi))


PULSE = """
max_step = 500
geometry.prob_lo = 0.0 0.0 0.0
geometry.prob_hi = {nc}.0 {nc}.0 {nc}.0
geometry.is_periodic = 1 1 1
amr.n_cell = {nc} {nc} {nc}
amr.max_level = 1
amr.max_grid_size = {mgs}
amr.blocking_factor = 8
amr.n_error_buf = 0
amr.regrid_int = 1000000
lbm.bc_lo = 0 0 0
lbm.bc_hi = 0 0 0
lbm.nu = 0.01
lbm.ic_type = "gaussian_pulse"
ic_gaussian_pulse.density = 1.0
ic_gaussian_pulse.amplitude = 0.01
ic_gaussian_pulse.width = {width}
ic_gaussian_pulse.initial_temperature = {t0!r}
tagging.refinement_indicators = centre
tagging.centre.in_box_lo = {lo}.0 {lo}.0 {lo}.0
tagging.centre.in_box_hi = {hi}.0 {hi}.0 {hi}.0
eb2.geom_type = "all_regular"
"""


def pulse(nc=128, lo=32, hi=96, mgs=32, width=8.0, t0=1.0 / 3.0):
    return PULSE.format(nc=nc, lo=lo, hi=hi, mgs=mgs, width=width, t0=t0)


SPHERE = """
max_step = 2000
geometry.prob_lo = 0.0 0.0 0.0
geometry.prob_hi = {nx}.0 {ny}.0 {nz}.0
geometry.is_periodic = 0 1 1
amr.n_cell = {nx} {ny} {nz}
amr.max_level = {maxlev}
amr.max_grid_size = {mgs}
amr.blocking_factor = 8
amr.n_error_buf = {buf}
amr.regrid_int = 1000000
lbm.bc_lo = 2 0 0
lbm.bc_hi = 5 0 0
lbm.nu = {nu}
lbm.velocity_bc_type = "constant"
velocity_bc_constant.dir = 0
velocity_bc_constant.Mach_ref = {mach}
lbm.ic_type = "constant"
ic_constant.density = 1.0
ic_constant.mach_components = {mach} 0.0 0.0
eb2.geom_type = "sphere"
eb2.sphere_radius = {r}
eb2.sphere_center = {cx} {cy} {cz}
eb2.sphere_has_fluid_inside = 0
tagging.refinement_indicators = solid
tagging.solid.field_name = is_fluid
tagging.solid.value_less = 0.5
"""


def sphere(nx=256, ny=128, nz=128, r=16.0, c=(64.0, 64.0, 64.0), maxlev=2, mgs=32, buf=8, nu=0.016,
           mach=0.0670820):
    return SPHERE.format(nx=nx, ny=ny, nz=nz, r=r, cx=c[0], cy=c[1], cz=c[2], maxlev=maxlev, mgs=mgs, buf=buf,
                         nu=nu, mach=mach)


def tg_domain(nx, ny, nz, nu, v0):
    """One Taylor-Green domain on [0, 2 pi)^3, nx x ny x nz cells in one box."""
    return (TG64.format(L=repr(2 * math.pi), n=nx, mgs=max(nx, ny, nz), w=repr(1.0 / math.pi))
            .replace("amr.n_cell = %d %d %d" % (nx, nx, nx), "amr.n_cell = %d %d %d" % (nx, ny, nz))
            .replace("lbm.nu = 0.005", "lbm.nu = %r" % nu)
            .replace("ic_taylorgreen.v0 = 0.05", "ic_taylorgreen.v0 = %r" % v0))


def batch_domains(count=256, seed0=0, sizes=tuple(range(16, 97, 8)), nu_range=(0.002, 0.02),
                  v0_range=(0.01, 0.08)):
    """Batched Taylor-Green instances: instance s draws, from
    numpy.random.default_rng(seed0 + s), its three cell counts from `sizes`,
    v0 and nu uniformly from the ranges.  Returns [(n_cell, nu, v0)]."""
    import numpy as np
    out = []
    for s in range(count):
        rng = np.random.default_rng(seed0 + s)
        n = [int(v) for v in rng.choice(np.asarray(sizes), size=3)]
        v0 = float(rng.uniform(*v0_range))
        nu = float(rng.uniform(*nu_range))
        out.append((n, nu, v0))
    return out


def gaussian_field(n, seed, corr=8.0):
    """Seeded unit-variance Gaussian random field on a periodic grid n = (nx,
    ny, nz), correlation length `corr` cells (white noise filtered by
    exp(-k^2 corr^2 / 2) in Fourier space); returned x-fastest, flat."""
    import numpy as np
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((n[2], n[1], n[0]))
    kz = np.fft.fftfreq(n[2])[:, None, None] * 2 * np.pi
    ky = np.fft.fftfreq(n[1])[None, :, None] * 2 * np.pi
    kx = np.fft.rfftfreq(n[0])[None, None, :] * 2 * np.pi
    filt = np.exp(-(kx ** 2 + ky ** 2 + kz ** 2) * corr ** 2 / 2)
    gfield = np.fft.irfftn(np.fft.rfftn(w) * filt, s=w.shape, axes=(0, 1, 2))
    gfield -= gfield.mean()
    gfield /= gfield.std()
    return gfield.reshape(-1)
