"""Linear stability of the reference scheme, from the oracle's own collision
(CPU only).

The oracle's collision of one cell (orc_collide_cell: f_to_macrodata,
macrodata_to_equilibrium and relax of Source/LBM.cpp:621-906 with the
q-correction gradient supplied) is linearised around the rest equilibrium
(rho = 1, u = 0, T) by central differences with Richardson extrapolation:

    A = d(f', g') / d(f, g)      54 x 54   (post-stream in, post-collision out)
    B = d(f', g') / d(dQ)        54 x 3
    G = d(Q_corr) / d(f, g)      3 x 54

On an unbounded lattice a Fourier mode exp(i k.x) of the post-collision
state streams to exp(-i k.e_q) times itself (pull of x - e_q), and the
q-correction gradient of Source/Utilities.H:279-312 (central in the
interior, 1/2 (Q(x+e) - Q(x-e)) / dx) becomes i sin(k_a) / dx_a times Q_a.
One step is therefore the 54 x 54 amplification matrix

    M(k) = (A + B diag(i sin(k) / dx) G) diag(exp(-i k.e_q)),

and the scheme is linearly unstable where its spectral radius exceeds 1.

Findings, asserted below:
  * RT = 1/3 at the workloads' viscosities (nu = 0.002 ... 0.02) is unstable:
    the largest growth factor per step is 2.1 - 2.4, at three-dimensional
    wave vectors such as k = (pi, 0.55 pi, 0.18 pi).  At RT = 1/3 the scheme
    is stable only for nu >= about 0.125.
  * The same viscosities at RT = 0.1 (and the sphere's nu = 0.016 at
    RT = 0.03) are stable; at nu = 0.01 the bound is RT <= about 0.22.
  * The reference's recorded viscosity run (Tests/test_files/viscosity_test,
    nu = 1e-4, RT = 0.3333, Tools/viscosity_test/viscosity_tester.ipynb) is
    unstable for three-dimensional modes (growth 2.4 per step) but neutral
    (spectral radius 1) for every mode along y alone, which is all its
    x- and z-uniform initial condition excites: that is why it survives
    5000 steps in the reference and in the oracle alike.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O

EV = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1], [1, 1, 0],
               [-1, -1, 0], [1, -1, 0], [-1, 1, 0], [1, 0, 1], [-1, 0, -1], [1, 0, -1], [-1, 0, 1], [0, 1, 1],
               [0, -1, -1], [0, 1, -1], [0, -1, 1], [1, 1, 1], [-1, -1, -1], [1, -1, 1], [-1, 1, -1],
               [1, -1, -1], [-1, 1, 1], [1, 1, -1], [-1, -1, 1]])
E54 = np.concatenate([EV, EV]).astype(float)

# spectral radius of the conserved (k = 0) modes is exactly 1; the
# linearisation is accurate to about 1e-12
NEUTRAL = 1.0 + 1e-9


def linearise(nu, alpha, temp, dt=1.0, h=1e-4):
    """A, B, G of the oracle's one-cell collision around the rest state."""
    p = O.default_params()
    p.nu, p.alpha = nu, alpha
    o = O.Oracle(p, [O.chop_domain([4, 4, 4], 4)])
    f0, g0 = o.equilibrium_cell(1.0, [0.0, 0.0, 0.0], temp)
    x0 = np.concatenate([f0, g0])
    z = np.zeros(3)

    def out(x, dq):
        fo, go, qc = o.collide_cell(x[:27], x[27:], dq, dt)
        return np.concatenate([fo, go, qc])

    y0 = out(x0, z)
    assert np.max(np.abs(y0[:54] - x0)) < 1e-14   # the rest state is a fixed point

    def deriv(fun):
        d1 = (fun(h) - fun(-h)) / (2 * h)
        d2 = (fun(h / 2) - fun(-h / 2)) / h
        return (4 * d2 - d1) / 3

    A = np.zeros((54, 54))
    G = np.zeros((3, 54))
    B = np.zeros((54, 3))
    for i in range(54):
        def fx(e, i=i):
            x = x0.copy()
            x[i] += e
            return out(x, z)
        d = deriv(fx)
        A[:, i], G[:, i] = d[:54], d[54:]
    for a in range(3):
        def fq(e, a=a):
            dq = z.copy()
            dq[a] += e
            return out(x0, dq)[:54]
        B[:, a] = deriv(fq)
    o.close()
    return A, B, G


def spectral_radius(lin, inv_dx, ks):
    A, B, G = lin
    r = np.empty(len(ks))
    for n, k in enumerate(ks):
        C = A + B @ np.diag(1j * np.sin(k) * inv_dx) @ G
        M = C * np.exp(-1j * (E54 @ k))[None, :]
        r[n] = np.max(np.abs(np.linalg.eigvals(M)))
    return r


def grid3(n):
    """Wave vectors on [0, pi]^3 (the growth factors are even in each k_a)."""
    g = np.linspace(0.0, math.pi, n)
    return np.array([[a, b, c] for a in g for b in g for c in g])


def max_growth(nu, temp, inv_dx=(1.0, 1.0, 1.0), dt=1.0, n=9):
    return float(spectral_radius(linearise(nu, nu, temp, dt), np.array(inv_dx), grid3(n)).max())


TG_INV_DX = 64 / (2 * math.pi)   # Taylor-Green 64^3 on [0, 2 pi)^3


@pytest.mark.parametrize("name,nu,temp,inv_dx,dt", [
    ("two-level pulse, level 0", 0.01, 1.0 / 3.0, 1.0, 1.0),
    ("two-level pulse, fine level", 0.01, 1.0 / 3.0, 2.0, 0.5),
    ("Taylor-Green 64^3", 0.005, 1.0 / 3.0, TG_INV_DX, 1.0),
    ("sphere", 0.016, 1.0 / 3.0, 1.0, 1.0),
    ("batch, lowest nu on the finest domain", 0.002, 1.0 / 3.0, 96 / (2 * math.pi), 1.0),
    ("batch, highest nu on the coarsest domain", 0.02, 1.0 / 3.0, 16 / (2 * math.pi), 1.0),
])
def test_literal_workload_parameters_are_unstable(name, nu, temp, inv_dx, dt):
    r = max_growth(nu, temp, (inv_dx,) * 3, dt)
    assert r > 1.8, (name, r)


@pytest.mark.parametrize("name,nu,temp,inv_dx,dt", [
    ("two-level pulse at RT = 0.1, level 0", 0.01, 0.1, 1.0, 1.0),
    ("two-level pulse at RT = 0.1, fine level", 0.01, 0.1, 2.0, 0.5),
    ("sphere at RT = 0.03", 0.016, 0.03, 1.0, 1.0),
    ("Taylor-Green at the reference's own nu = 0.1733", 0.1733, 1.0 / 3.0, TG_INV_DX, 1.0),
    ("batch parity cases, nu = 0.15", 0.15, 1.0 / 3.0, 1.0, 1.0),
    ("batch parity cases, nu = 0.2", 0.2, 1.0 / 3.0, 1.0, 1.0),
])
def test_parity_and_bench_parameters_are_stable(name, nu, temp, inv_dx, dt):
    r = max_growth(nu, temp, (inv_dx,) * 3, dt)
    assert r <= NEUTRAL, (name, r)


def test_recorded_viscosity_run_is_neutral_in_y_and_unstable_in_3d():
    """Tests/test_files/viscosity_test: nu = 1e-4, T0 = 0.3333, R = 1,
    6 x 200 x 2 cells, the IC varying along y only."""
    lin = linearise(1e-4, 1e-4, 0.3333)
    ky = 2 * math.pi * np.arange(0, 101) / 200.0          # every mode of the 200-cell period
    r1 = spectral_radius(lin, np.ones(3), np.array([[0.0, k, 0.0] for k in ky]))
    assert r1.max() <= NEUTRAL, r1.max()
    r3 = spectral_radius(lin, np.ones(3), grid3(9))
    assert r3.max() > 2.0, r3.max()


def test_stability_bounds_in_nu_and_temperature():
    """At RT = 1/3 the scheme turns stable near nu = 0.125; at nu = 0.01
    near RT = 0.22."""
    assert max_growth(0.12, 1.0 / 3.0, n=7) > NEUTRAL
    assert max_growth(0.13, 1.0 / 3.0, n=7) <= NEUTRAL
    assert max_growth(0.01, 0.23, n=7) > NEUTRAL
    assert max_growth(0.01, 0.21, n=7) <= NEUTRAL
