"""FP64 PyTorch restatement of the periodic-box step the adjoint differentiates
(test infrastructure: autograd over it is the reference gradient).

Follows the reference's algorithm as the library's FP64 step does: pull
stream on a periodic box (Source/LBM.cpp:558-604), moments and macro fields
(LBM.cpp:810-906, Utilities.H:187-210), the q-correction gradient one-sided at
the box faces with physical 1/dx (LBM.cpp:959-991, Utilities.H:279-312), the
product-form f_eq and the Grad-expansion g_eq with the omega1/omega heat-flux
mix (LBM.cpp:621-762, Utilities.H:42-277), BGK relaxation with one omega for
both lattices (LBM.cpp:765-807); initial state = equilibria of (rho0, 0, T0)
(IC.H:474-519).  Arrays are (27, nz, ny, nx), x fastest.
"""
import torch

# D3Q27 directions in the reference's order (Source/Stencil.H)
EX = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1]
EY = [0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1, -1, 1, 1, -1]
EZ = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 1, -1, 1, -1, -1, 1, -1, 1]
NQ = 27


def _weights():
    wsc, wfcc, wbcc = 2.0 / 27.0, 1.0 / 54.0, 1.0 / 216.0
    w0 = 1.0 - (6.0 * wsc + 12.0 * wfcc + 8.0 * wbcc)
    out = []
    for q in range(NQ):
        s = abs(EX[q]) + abs(EY[q]) + abs(EZ[q])
        out.append(w0 if s == 0 else wsc if s == 1 else wfcc if s == 2 else wbcc)
    return out


W = _weights()
TH = 1.0 / 3.0
K = 1.0 / TH
CTH = (0.0 - TH, 1.0 - TH)


class Params:
    def __init__(self, nu, alpha, gamma=5.0 / 3.0, m_bar=28.96, ms=1.0, dt=1.0, idx=(1.0, 1.0, 1.0), rho0=1.0):
        self.nu, self.alpha, self.dt, self.ms, self.rho0 = nu, alpha, dt, ms, rho0
        self.Rg = 28.96 / m_bar
        self.gamma = gamma
        self.cv = self.Rg / (gamma - 1.0)
        self.idx = idx


def _e(shape_like):
    d = dict(dtype=shape_like.dtype, device=shape_like.device)
    ex = torch.tensor(EX, **d).view(NQ, 1, 1, 1)
    ey = torch.tensor(EY, **d).view(NQ, 1, 1, 1)
    ez = torch.tensor(EZ, **d).view(NQ, 1, 1, 1)
    return ex, ey, ez


def moments(f, g):
    ex, ey, ez = _e(f)
    m = {"rho": f.sum(0), "j": [(ex * f).sum(0), (ey * f).sum(0), (ez * f).sum(0)],
         "P": [[(ex * ex * f).sum(0), (ex * ey * f).sum(0), (ex * ez * f).sum(0)],
               [(ey * ex * f).sum(0), (ey * ey * f).sum(0), (ey * ez * f).sum(0)],
               [(ez * ex * f).sum(0), (ez * ey * f).sum(0), (ez * ez * f).sum(0)]],
         "tre": g.sum(0), "q": [(ex * g).sum(0), (ey * g).sum(0), (ez * g).sum(0)]}
    return m


def macro(m, p):
    rho = m["rho"]
    U = [j * (p.ms / rho) for j in m["j"]]
    T = (0.5 / p.cv) * ((m["tre"] / rho) - (U[0] * U[0] + U[1] * U[1] + U[2] * U[2]))
    Qc = [rho * U[a] * ((1.0 - 3.0 * p.Rg * T) - U[a] * U[a]) for a in range(3)]
    return U, T, Qc


def gradient(Q, axis, idx):
    """d/dx_axis with one-sided differences at the box faces; axis 0 = x."""
    dim = 2 - axis
    n = Q.shape[dim]
    a = Q.narrow(dim, 0, 1)
    b = Q.narrow(dim, 1, 1)
    y = Q.narrow(dim, n - 2, 1)
    z = Q.narrow(dim, n - 1, 1)
    mid = 0.5 * Q.narrow(dim, 2, n - 2) - 0.5 * Q.narrow(dim, 0, n - 2)
    return torch.cat([b - a, mid, z - y], dim=dim) * idx


def phi(e, U, P):
    if e == 0:
        return -P + 1.0
    return (0.5 if e == 1 else -0.5) * U + ((1.50 * P - 1.0) - P + 1.0)


def equilibria(m, U, T, dq, p):
    rho, tre = m["rho"], m["tre"]
    omega = 1.0 / (p.nu / (p.Rg * T * p.dt) + 0.5)
    omega1 = 1.0 / (p.alpha / (p.Rg * T * p.dt) + 0.5)
    r = omega1 / omega
    wc = (2.0 - omega) / (2.0 * omega * rho)
    P = [U[a] * U[a] + p.Rg * T + p.dt * wc * dq[a] for a in range(3)]
    ph = [{e: phi(e, U[a], P[a]) for e in (-1, 0, 1)} for a in range(3)]
    feq = torch.stack([rho * ph[0][EX[q]] * ph[1][EY[q]] * ph[2][EZ[q]] for q in range(NQ)])
    energy = tre / (2.0 * rho)
    tmp = (0.5 / p.cv) * ((tre / rho) - (U[0] * U[0] + U[1] * U[1] + U[2] * U[2]))
    pr = rho * p.Rg * tmp
    h = energy + pr / rho
    G = h + pr / rho
    qf = []
    for a in range(3):
        qeq = 2.0 * rho * U[a] * h
        B = m["q"][a] - 2.0 * U[0] * m["P"][a][0] - 2.0 * U[1] * m["P"][a][1] - 2.0 * U[2] * m["P"][a][2] \
            - U[a] * p.dt * dq[a]
        qf.append(qeq * r + (1.0 - r) * B)
    a1 = [qf[a] * K for a in range(3)]
    a2d = [(2.0 * rho * U[a] * U[a] * G + 2.0 * pr * h - tre * TH) * K * K for a in range(3)]
    a2o = {(0, 1): 2.0 * rho * U[0] * U[1] * G * K * K, (0, 2): 2.0 * rho * U[0] * U[2] * G * K * K,
           (1, 2): 2.0 * rho * U[1] * U[2] * G * K * K}
    geq = []
    for q in range(NQ):
        e = (EX[q], EY[q], EZ[q])
        v = tre + e[0] * a1[0] + e[1] * a1[1] + e[2] * a1[2]
        s = CTH[e[0] * e[0]] * a2d[0] + CTH[e[1] * e[1]] * a2d[1] + CTH[e[2] * e[2]] * a2d[2]
        s = s + 2.0 * (e[0] * e[1] * a2o[(0, 1)] + e[0] * e[2] * a2o[(0, 2)] + e[1] * e[2] * a2o[(1, 2)])
        geq.append(W[q] * (v + 0.5 * s))
    return omega, feq, torch.stack(geq)


def pull(s):
    return torch.stack([torch.roll(s[q], shifts=(EZ[q], EY[q], EX[q]), dims=(0, 1, 2)) for q in range(NQ)])


def step(f, g, p):
    pf, pg = pull(f), pull(g)
    m = moments(pf, pg)
    U, T, Qc = macro(m, p)
    dq = [gradient(Qc[a], a, p.idx[a]) for a in range(3)]
    omega, feq, geq = equilibria(m, U, T, dq, p)
    return pf + omega * (feq - pf), pg + omega * (geq - pg)


def initial_state(T0, p):
    rho = torch.full_like(T0, p.rho0)
    zero = torch.zeros_like(T0)
    Pd = p.Rg * T0
    ph = {e: phi(e, zero, Pd) for e in (-1, 0, 1)}
    f = torch.stack([rho * ph[EX[q]] * ph[EY[q]] * ph[EZ[q]] for q in range(NQ)])
    tre = rho * (2.0 * p.cv * T0)
    energy = tre / (2.0 * rho)
    tmp = (0.5 / p.cv) * (tre / rho)
    pr = rho * p.Rg * tmp
    h = energy + pr / rho
    a2d = (2.0 * pr * h - tre * TH) * K * K
    g = torch.stack([W[q] * (tre + 0.5 * (CTH[EX[q] ** 2] + CTH[EY[q] ** 2] + CTH[EZ[q] ** 2]) * a2d)
                     for q in range(NQ)])
    return f, g


def final_temperature(T0, nsteps, p):
    f, g = initial_state(T0, p)
    for _ in range(nsteps):
        f, g = step(f, g, p)
    return macro(moments(f, g), p)[1]
