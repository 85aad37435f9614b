"""The allocation-free step (mbg_step_box_noalloc) against the context's
level advance (GPU).

mbg_step_box_noalloc serves callers that cannot let the library allocate
device memory -- a host code that owns the GPU through its own memory arena,
or one that cannot afford the device synchronisation cudaMalloc / cudaFree may
cause inside its time loop.  It takes the caller's device buffers and keeps its
scratch in a fixed array of the library image.  Two calls in a row must
reproduce two mbg_advance_level calls on a context holding the same box and
the oracle's two steps of that box, and further calls must leave the device's
free memory unchanged.
"""
import ctypes as C

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

RTOL = 1e-12

INPUTS = """
geometry.prob_lo = 0.0 0.0 0.0
geometry.prob_hi = 24.0 16.0 20.0
geometry.is_periodic = 1 1 1
amr.n_cell = 24 16 20
amr.max_level = 0
amr.max_grid_size = 64
lbm.bc_lo = 0 0 0
lbm.bc_hi = 0 0 0
lbm.nu = 0.1733333333333333
lbm.ic_type = "taylorgreen"
ic_taylorgreen.rho0 = 1.0
ic_taylorgreen.v0 = 0.05
ic_taylorgreen.omega = 0.0833333333333333 0.125 0.1
"""


def _params(M):
    p = M.default_params()
    p.n_cell[:] = [24, 16, 20]
    p.prob_lo[:] = [0.0, 0.0, 0.0]
    p.prob_hi[:] = [24.0, 16.0, 20.0]
    p.is_periodic[:] = [1, 1, 1]
    p.nu = 0.1733333333333333
    p.alpha = p.nu
    return p


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _oracle_case():
    p, levels = cases.tg_domain(24, 16, 20, 0.1733333333333333, 0.05)
    p.prob_hi[:] = [24.0, 16.0, 20.0]
    p.ic_omega[:] = [0.0833333333333333, 0.125, 0.1]
    return p, levels


def test_noalloc_step_matches_level_advance_on_two_calls():
    import torch
    import marbles_gb300 as M

    d = M.LBM(INPUTS)
    d.prepare()
    f0, g0 = d.initial_state(0)
    boxes = d.boxes(0)
    assert len(boxes) == 1

    p = _params(M)
    ctx = M.Context(p)
    ctx.define_level(0, boxes)
    ctx.set_state(0, f0, g0)

    # the oracle on the same box and initial state
    op, olev = _oracle_case()
    o = cases.run_oracle(op, olev, 0)
    o.set_state(0, f0, g0)

    fa = torch.tensor(f0, device="cuda")
    ga = torch.tensor(g0, device="cuda")
    fb = torch.empty_like(fa)
    gb = torch.empty_like(ga)
    lib = M.lib()
    for call in range(2):
        ctx.advance_level(0)
        fr, gr = ctx.get_state(0)
        o.advance_level(0)
        fo, go = o.get_state(0)
        st = lib.mbg_step_box_noalloc(C.byref(p), fa.data_ptr(), ga.data_ptr(), fb.data_ptr(), gb.data_ptr(),
                                      None)
        assert st == 0, lib.mbg_last_error(None).decode()
        torch.cuda.synchronize()
        fn, gn = fb.cpu().numpy(), gb.cpu().numpy()
        assert np.isfinite(fn).all() and np.isfinite(gn).all()
        assert _rel(fn, fr) <= RTOL and _rel(gn, gr) <= RTOL, (call, _rel(fn, fr), _rel(gn, gr))
        assert _rel(fn, fo) <= RTOL and _rel(gn, go) <= RTOL, (call, _rel(fn, fo), _rel(gn, go))
        fa, fb = fb, fa
        ga, gb = gb, ga

    # the property the entry point exists for: later calls take no device memory
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        st = lib.mbg_step_box_noalloc(C.byref(p), fa.data_ptr(), ga.data_ptr(), fb.data_ptr(), gb.data_ptr(),
                                      None)
        assert st == 0, lib.mbg_last_error(None).decode()
        fa, fb = fb, fa
        ga, gb = gb, ga
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_oversized_box():
    import marbles_gb300 as M

    p = _params(M)
    p.n_cell[:] = [64, 64, 64]
    x = C.c_void_p(16)
    y = C.c_void_p(32)
    st = M.lib().mbg_step_box_noalloc(C.byref(p), x, y, C.c_void_p(48), C.c_void_p(64), None)
    assert st == 1
    assert b"exceeds the maximum" in M.lib().mbg_last_error(None)


def test_noalloc_rejects_axis_whose_product_would_overflow():
    import marbles_gb300 as M

    p = _params(M)
    p.n_cell[:] = [2 ** 30, 2 ** 30, 2 ** 30]
    st = M.lib().mbg_step_box_noalloc(C.byref(p), C.c_void_p(16), C.c_void_p(32), C.c_void_p(48),
                                      C.c_void_p(64), None)
    assert st == 1
    assert b"exceeds the maximum" in M.lib().mbg_last_error(None)
