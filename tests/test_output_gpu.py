"""Output paths on the GPU: derived fields, EB forces, the drop-in driver's
plotfile and checkpoint/restart.

* mbg_get_derived (vorticity and q-correction gradients of the stored state)
  against the oracle's compute_derived / compute_q_corrections after
  f_to_macrodata, at 1e-12 in FP64; the 16-bit forms within their storage
  tolerance of the FP64 result.
* mbg_eb_forces: the same bits on every call and in a second context run
  the same way (fixed-order reductions, no atomics), 1e-12 of the oracle in
  FP64, within tolerance in the 16-bit forms.
* The driver's plotfile read back by an independent parser (tests/plotfile.py)
  equals mbg_get_macro / mbg_get_state / mbg_get_derived and the flags, with
  the reference's variable names; a run restarted from a checkpoint
  continues bit-identically.
"""
import numpy as np
import pytest

import cases
import plotfile

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _ctx(o, p, levels, prec=0):
    import marbles_gb300 as M
    ctx = M.Context(cases.mbg_params_from(p, prec))
    for lev, b in enumerate(levels):
        ctx.define_level(lev, b, o.get_grown_flags(lev))
    for lev in range(len(levels)):
        f, g = o.get_state(lev)
        ctx.set_state(lev, f, g)
    return ctx


def _oracle_derived(o, lev):
    import ctypes as C
    n = o.ncells(lev)
    out = np.empty(n * 7)
    o.L.orc_get_derived(o.h, lev, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def _per_comp_rel(a, b, levels_boxes, ncomp):
    """worst |a - b| / max |b| per component over the boxes ([box][comp][cell])"""
    worst = np.zeros(ncomp)
    scale = np.zeros(ncomp)
    off = 0
    diffs = []
    for bx in levels_boxes:
        vol = int(np.prod(bx[3:] - bx[:3] + 1))
        A = a[off:off + ncomp * vol].reshape(ncomp, vol)
        B = b[off:off + ncomp * vol].reshape(ncomp, vol)
        diffs.append(np.max(np.abs(A - B), axis=1))
        scale = np.maximum(scale, np.max(np.abs(B), axis=1))
        off += ncomp * vol
    worst = np.max(np.array(diffs), axis=0)
    return worst / np.where(scale > 0, scale, 1.0)


CASES = {
    "pulse2": lambda: cases.gaussian_pulse(nc=32, fine_lo=8, fine_hi=23, mgs=16, width=3.0, t0=0.1),
    "sphere": lambda: cases.sphere_channel(48, 32, 32, radius=5.0, center=(16.0, 16.0, 16.0), mgs=16, levels=2,
                                           t0=0.03),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_derived_fields_match_oracle(case):
    p, levels = CASES[case]()
    o = cases.run_oracle(p, levels, 0)
    ctx = _ctx(o, p, levels)
    ctx.step(3)
    o.step(3)
    for lev in range(len(levels)):
        d = ctx.get_derived(lev)
        r = _oracle_derived(o, lev)
        assert np.isfinite(d).all()
        rel = _per_comp_rel(d, r, levels[lev], 7)
        assert rel.max() <= RTOL, (lev, rel)


@pytest.mark.parametrize("prec", [1, 2])
def test_derived_fields_16bit_forms(prec):
    p, levels = CASES["sphere"]()
    o = cases.run_oracle(p, levels, 0)
    c64 = _ctx(o, p, levels)
    c16 = _ctx(o, p, levels, prec)
    c64.step(3)
    c16.step(3)
    tol = {1: 2e-2, 2: 1.5e-1}[prec]
    for lev in range(len(levels)):
        rel = _per_comp_rel(c16.get_derived(lev), c64.get_derived(lev), levels[lev], 7)
        print("16-bit derived", prec, lev, rel)
        assert rel.max() <= tol, (lev, rel)


def test_eb_forces_deterministic_and_match_oracle():
    p, levels = CASES["sphere"]()
    o = cases.run_oracle(p, levels, 0)
    a = _ctx(o, p, levels)
    b = _ctx(o, p, levels)
    a.step(4)
    b.step(4)
    o.step(4)
    fa = [a.eb_forces() for _ in range(3)] + [b.eb_forces()]
    for f in fa[1:]:
        assert np.array_equal(f, fa[0]), (f, fa[0])
    ref = o.eb_forces()
    assert np.max(np.abs(fa[0] - ref)) <= RTOL * np.max(np.abs(ref)), (fa[0], ref)


@pytest.mark.parametrize("prec", [1, 2])
def test_eb_forces_16bit_forms(prec):
    p, levels = CASES["sphere"]()
    o = cases.run_oracle(p, levels, 0)
    c64 = _ctx(o, p, levels)
    c16 = _ctx(o, p, levels, prec)
    c64.step(4)
    c16.step(4)
    f64 = c64.eb_forces()
    f16 = [c16.eb_forces() for _ in range(2)]
    assert np.array_equal(f16[0], f16[1])
    rel = np.max(np.abs(f16[0] - f64)) / np.max(np.abs(f64))
    print("16-bit force", prec, f16[0], f64, rel)
    assert rel <= {1: 1e-2, 2: 5e-2}[prec], (f16[0], f64)


def _driver_inputs(tmp, extra=""):
    import inputs
    text = inputs.sphere(nx=48, ny=32, nz=32, r=5.0, c=(16.0, 16.0, 16.0), maxlev=1, mgs=16, buf=2)
    text += ("\nic_constant.initial_temperature = 0.03\nvelocity_bc_constant.initial_temperature = 0.03\n"
             "amr.plot_file = %s/plt\namr.chk_file = %s/chk\n" % (tmp, tmp)) + extra
    return text


def test_driver_plotfile_matches_state(tmp_path):
    import marbles_gb300 as M
    d = M.LBM(_driver_inputs(str(tmp_path)))
    ctx = d.init()
    d.evolve(3)
    d.write_plotfile(str(tmp_path / "out"))
    pf = plotfile.read_plotfile(str(tmp_path / "out"))
    names = pf["names"]
    assert names[:19] == ["rho", "vel_x", "vel_y", "vel_z", "vel_mag", "two_rho_e", "QCorrX", "QCorrY", "QCorrZ",
                          "pxx", "pyy", "pzz", "pxy", "pxz", "pyz", "qx", "qy", "qz", "temperature"]
    assert names[19] == "f_00" and names[45] == "f_26" and names[46] == "g_00" and names[72] == "g_26"
    assert names[73:] == ["vort_x", "vort_y", "vort_z", "vort_mag", "dQCorrX", "dQCorrY", "dQCorrZ",
                          "is_fluid", "eb_boundary"]
    assert pf["time"] == 3.0 and pf["level_steps"] == [3, 6]
    for lev in range(d.num_levels()):
        boxes = d.boxes(lev)
        mac, der = ctx.get_macro(lev), ctx.get_derived(lev)
        f, g = ctx.get_state(lev)
        fl = d.flags(lev)
        moff = soff = doff = foff = 0
        for n, b in enumerate(boxes):
            nx, ny, nz = (int(v) for v in b[3:] - b[:3] + 1)
            vol = nx * ny * nz
            got = pf["levels"][lev]["data"][n].reshape(len(names), vol)
            assert np.array_equal(got[:19], mac[moff:moff + 19 * vol].reshape(19, vol))
            assert np.array_equal(got[19:46], f[soff:soff + 27 * vol].reshape(27, vol))
            assert np.array_equal(got[46:73], g[soff:soff + 27 * vol].reshape(27, vol))
            assert np.array_equal(got[73:80], der[doff:doff + 7 * vol].reshape(7, vol))
            gf = fl[foff:foff + (nx + 6) * (ny + 6) * (nz + 6)].reshape(nz + 6, ny + 6, nx + 6)[3:-3, 3:-3, 3:-3]
            assert np.array_equal(got[80], (gf.reshape(-1) & 1).astype(float))
            assert np.array_equal(got[81], ((gf.reshape(-1) >> 1) & 1).astype(float))
            moff += 19 * vol
            soff += 27 * vol
            doff += 7 * vol
            foff += (nx + 6) * (ny + 6) * (nz + 6)


def test_checkpoint_restart_is_bit_identical(tmp_path):
    import marbles_gb300 as M
    a = M.LBM(_driver_inputs(str(tmp_path)))
    ca = a.init()
    a.evolve(3)
    a.write_checkpoint(str(tmp_path / "chk_a"))
    a.evolve(4)
    b = M.LBM(_driver_inputs(str(tmp_path)), ["amr.restart=%s" % (tmp_path / "chk_a")])
    cb = b.init()
    assert b.step_time() == (3, 3.0)
    b.evolve(4)
    assert b.step_time() == a.step_time() == (7, 7.0)
    for lev in range(a.num_levels()):
        fa, ga = ca.get_state(lev)
        fb, gb = cb.get_state(lev)
        assert np.array_equal(fa, fb) and np.array_equal(ga, gb), lev


def test_evolve_writes_plotfiles_and_checkpoints_at_their_intervals(tmp_path):
    import os
    import marbles_gb300 as M
    d = M.LBM(_driver_inputs(str(tmp_path), "amr.plot_int = 2\namr.chk_int = 3\nmax_step = 5\n"))
    d.init()
    d.evolve(0)
    names = sorted(os.listdir(tmp_path))
    # plotfiles at 0, 2, 4 and the last step 5; checkpoints at 0 and 3
    assert names == ["chk00000", "chk00003", "plt00000", "plt00002", "plt00004", "plt00005"], names
    assert open(tmp_path / "chk00003" / "Header").readline().strip() == "Checkpoint file for LBM"


@pytest.mark.parametrize("prec", [0, 1])
def test_state_check_counts_a_planted_nan(prec):
    """mbg_check_state: the state after a few steps of an inflow/outflow
    sphere scans clean (fluid values finite, solid cells at the sentinel);
    a NaN planted at one direction of one fluid cell is counted once and
    located (level 0, box 0, cell 0, direction 5 of f)."""
    import marbles_gb300 as M
    p, levels = cases.sphere_channel(32, 16, 16, radius=4.0, center=(12.0, 8.0, 8.0), mgs=16, t0=0.03)
    o = cases.run_oracle(p, levels, 0)
    flags = o.get_grown_flags(0)
    b0 = levels[0][0]
    n = b0[3:] - b0[:3] + 1
    assert flags[(3 * (n[1] + 6) + 3) * (n[0] + 6) + 3] & 1        # cell 0 of box 0 is fluid
    c = M.Context(cases.mbg_params_from(p, prec))
    c.define_level(0, levels[0], flags)
    c.set_state(0, *o.get_state(0))
    c.step(3)
    counts, first = c.check_state()
    assert counts == (0, 0) and first == (-1, -1, -1, -1)
    f, g = c.get_state(0)
    vol = int(np.prod(n))
    f = f.copy()
    f[5 * vol + 0] = np.nan
    c.set_state(0, f, g)
    counts, first = c.check_state()
    assert counts == (1, 0) and first == (0, 0, 0, 10), (counts, first)
