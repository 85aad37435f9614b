"""ctypes front-end of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm use this module.  It loads oracle/_build/libmarbles_oracle.so, the FP64
restatement of the MARBLES level step in marbles_oracle.cpp, building it with
`make` when the library is missing.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmarbles_oracle.so")

NQ = 27
NMAC = 19

IC_TYPES = {"constant": 0, "taylorgreen": 1, "viscosity_test": 2,
            "thermaldiffusivity_test": 3, "sod": 4, "gaussian_pulse": 5,
            "temperature_field": 6}
VBC_TYPES = {"noop": 0, "constant": 1, "channel": 2, "parabolic": 3}
EB_TYPES = {"all_regular": 0, "sphere": 1}


class OrcParams(C.Structure):
    _fields_ = [
        ("n_cell", C.c_int * 3),
        ("prob_lo", C.c_double * 3), ("prob_hi", C.c_double * 3),
        ("is_periodic", C.c_int * 3),
        ("max_grid_size", C.c_int),
        ("bc_lo", C.c_int * 3), ("bc_hi", C.c_int * 3),
        ("nu", C.c_double), ("alpha", C.c_double),
        ("dx_outer", C.c_double), ("dt_outer", C.c_double),
        ("initial_temperature", C.c_double), ("adiabatic_exponent", C.c_double),
        ("m_bar", C.c_double),
        ("ic_type", C.c_int),
        ("ic_density", C.c_double), ("ic_velocity", C.c_double * 3),
        ("ic_mach", C.c_double * 3), ("ic_initial_temperature", C.c_double),
        ("ic_adiabatic_exponent", C.c_double), ("ic_m_bar", C.c_double),
        ("ic_wave_length", C.c_double),
        ("ic_rho0", C.c_double), ("ic_v0", C.c_double), ("ic_omega", C.c_double * 3),
        ("ic_density_ratio", C.c_double), ("ic_temperature_ratio", C.c_double),
        ("ic_x_discontinuity", C.c_double),
        ("ic_pulse_amplitude", C.c_double), ("ic_pulse_width", C.c_double),
        ("ic_pulse_center", C.c_double * 3),
        ("velbc_type", C.c_int),
        ("vbc_dir", C.c_int), ("vbc_normal_dir", C.c_int), ("vbc_tangential_dir", C.c_int),
        ("vbc_mach_ref", C.c_double), ("vbc_initial_density", C.c_double),
        ("vbc_initial_temperature", C.c_double),
        ("vbc_adiabatic_exponent", C.c_double), ("vbc_m_bar", C.c_double),
        ("eb_type", C.c_int),
        ("sphere_radius", C.c_double), ("sphere_center", C.c_double * 3),
        ("sphere_has_fluid_inside", C.c_int),
        ("nthreads", C.c_int),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.POINTER(OrcParams)]
        L.orc_destroy.argtypes = [vp]
        L.orc_chop_domain.argtypes = [C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int), C.c_int]
        L.orc_define_level.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_int)]
        L.orc_set_temperature_field.argtypes = [vp, C.POINTER(C.c_double), C.c_longlong]
        L.orc_init.argtypes = [vp]
        L.orc_step.argtypes = [vp, C.c_int]
        L.orc_advance_level.argtypes = [vp, C.c_int]
        L.orc_fillpatch.argtypes = [vp, C.c_int]
        L.orc_average_down.argtypes = [vp, C.c_int, C.c_int]
        L.orc_level_cells.restype = C.c_longlong
        L.orc_level_cells.argtypes = [vp, C.c_int]
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        L.orc_get_state.argtypes = [vp, C.c_int, dp, dp]
        L.orc_set_state.argtypes = [vp, C.c_int, dp, dp]
        L.orc_get_macro.argtypes = [vp, C.c_int, dp]
        L.orc_get_derived.argtypes = [vp, C.c_int, dp]
        L.orc_get_flags.argtypes = [vp, C.c_int, ip]
        L.orc_stencil.argtypes = [ip, dp, ip, ip, ip, ip]
        L.orc_get_grown_flags.argtypes = [vp, C.c_int, C.POINTER(C.c_uint8)]
        L.orc_eb_forces.argtypes = [vp, dp]
        L.orc_tag_cells.argtypes = [vp, C.c_int, C.POINTER(OrcTag), C.c_int, C.c_double, C.POINTER(C.c_uint8)]
        L.orc_regrid.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.orc_equilibrium_cell.argtypes = [vp, C.c_double, dp, C.c_double, dp, dp]
        L.orc_collide_cell.argtypes = [vp, dp, dp, dp, C.c_double, dp, dp, dp]
        _lib = L
    return _lib


def build():
    subprocess.check_call(["make", "-s", "-C", HERE])


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def default_params():
    """Defaults of the reference's member initialisers (LBM.H, IC.H, VelocityBC.H)."""
    p = OrcParams()
    p.n_cell[:] = [8, 8, 8]
    p.prob_lo[:] = [0.0, 0.0, 0.0]
    p.prob_hi[:] = [8.0, 8.0, 8.0]
    p.is_periodic[:] = [1, 1, 1]
    p.max_grid_size = 32
    p.nu = 1.0
    p.alpha = 1.0
    p.dx_outer = 1.0
    p.dt_outer = 1.0
    p.initial_temperature = 1.0 / 3.0
    p.adiabatic_exponent = 5.0 / 3.0
    p.m_bar = 28.96
    p.ic_type = 0
    p.ic_density = 1.0
    p.ic_initial_temperature = 1.0 / 3.0
    p.ic_adiabatic_exponent = 5.0 / 3.0
    p.ic_m_bar = 28.96
    p.ic_wave_length = 1.0
    p.ic_rho0 = 1.0
    p.ic_v0 = 1.0
    p.ic_omega[:] = [1.0, 1.0, 1.0]
    p.ic_density_ratio = 1.0
    p.ic_temperature_ratio = 1.0
    p.ic_x_discontinuity = 10.0
    p.ic_pulse_amplitude = 0.01
    p.ic_pulse_width = 8.0
    p.velbc_type = 0
    p.vbc_dir = 1
    p.vbc_normal_dir = 0
    p.vbc_tangential_dir = 1
    p.vbc_mach_ref = 0.005
    p.vbc_initial_density = 1.0
    p.vbc_initial_temperature = 1.0 / 3.0
    p.vbc_adiabatic_exponent = 5.0 / 3.0
    p.vbc_m_bar = 28.96
    p.eb_type = 0
    p.nthreads = 0
    return p


def chop_domain(n_cell, max_grid_size):
    L = lib()
    nc = (C.c_int * 3)(*n_cell)
    n = L.orc_chop_domain(nc, max_grid_size, None, 0)
    out = np.zeros(6 * n, dtype=np.int32)
    L.orc_chop_domain(nc, max_grid_size, _ip(out), n)
    return out.reshape(n, 6)


class OrcTag(C.Structure):
    """One refinement criterion (field: macro component 0..18 or 19 = is_fluid;
    kind 0 box only, 1 value_greater, 2 value_less)."""
    _fields_ = [("field", C.c_int), ("kind", C.c_int), ("value", C.c_double), ("has_box", C.c_int),
                ("box_lo", C.c_double * 3), ("box_hi", C.c_double * 3), ("start_time", C.c_double),
                ("end_time", C.c_double), ("max_level", C.c_int)]


def make_tag(field=0, kind=1, value=0.0, box=None, start_time=-1.0e300, end_time=1.0e300, max_level=1000):
    t = OrcTag()
    t.field, t.kind, t.value = field, kind, value
    t.has_box = 1 if box is not None else 0
    if box is not None:
        t.box_lo[:] = list(box[0])
        t.box_hi[:] = list(box[1])
    t.start_time, t.end_time, t.max_level = start_time, end_time, max_level
    return t


class Oracle:
    """One simulation: levels of boxes, FP64 f and g, the reference's step."""

    def __init__(self, params, levels):
        """params: OrcParams; levels: list of (nbox, 6) int arrays of lo/hi."""
        self.L = lib()
        self.p = params
        self.h = self.L.orc_create(C.byref(params))
        self.levels = [np.ascontiguousarray(b, dtype=np.int32) for b in levels]
        for lev, b in enumerate(self.levels):
            self.L.orc_define_level(self.h, lev, b.shape[0], _ip(b))

    def set_temperature_field(self, t):
        t = np.ascontiguousarray(t, dtype=np.float64).ravel()
        self.L.orc_set_temperature_field(self.h, _dp(t), t.size)

    def init(self):
        self.L.orc_init(self.h)

    def step(self, n=1):
        self.L.orc_step(self.h, n)

    def advance_level(self, lev):
        """One advance of level lev in isolation (stream f, g + collide)."""
        self.L.orc_advance_level(self.h, lev)

    def average_down(self, crse_lev, ng):
        self.L.orc_average_down(self.h, crse_lev, ng)

    def ncells(self, lev):
        return self.L.orc_level_cells(self.h, lev)

    def get_state(self, lev):
        n = self.ncells(lev)
        f = np.empty(n * NQ)
        g = np.empty(n * NQ)
        self.L.orc_get_state(self.h, lev, _dp(f), _dp(g))
        return f, g

    def set_state(self, lev, f, g):
        f = np.ascontiguousarray(f, dtype=np.float64)
        g = np.ascontiguousarray(g, dtype=np.float64)
        self.L.orc_set_state(self.h, lev, _dp(f), _dp(g))

    def get_macro(self, lev):
        n = self.ncells(lev)
        m = np.empty(n * NMAC)
        self.L.orc_get_macro(self.h, lev, _dp(m))
        return m

    def get_flags(self, lev):
        n = self.ncells(lev)
        fl = np.empty(n * 2, dtype=np.int32)
        self.L.orc_get_flags(self.h, lev, _ip(fl))
        return fl

    def get_grown_flags(self, lev):
        b = self.levels[lev]
        n = int(np.sum((b[:, 3] - b[:, 0] + 7) * (b[:, 4] - b[:, 1] + 7) * (b[:, 5] - b[:, 2] + 7)))
        out = np.zeros(n, dtype=np.uint8)
        self.L.orc_get_grown_flags(self.h, lev, out.ctypes.data_as(C.POINTER(C.c_uint8)))
        return out

    def eb_forces(self):
        out = np.zeros(3)
        self.L.orc_eb_forces(self.h, _dp(out))
        return out

    def tag_cells(self, lev, tags, time):
        """ErrorEst tags (0/1 per valid cell of level lev, [box][cell])."""
        arr = (OrcTag * len(tags))(*tags)
        out = np.zeros(self.ncells(lev), dtype=np.uint8)
        self.L.orc_tag_cells(self.h, lev, arr, len(tags), time, out.ctypes.data_as(C.POINTER(C.c_uint8)))
        return out

    def regrid(self, first_lev, new_levels):
        """Replace levels first_lev.. with the box arrays new_levels (RemakeLevel)."""
        nbox = np.array([len(b) for b in new_levels] or [0], dtype=np.int32)
        parts = [np.asarray(b, dtype=np.int32).reshape(-1) for b in new_levels]
        lohi = np.ascontiguousarray(np.concatenate(parts) if parts else np.zeros(6, dtype=np.int32))
        st = self.L.orc_regrid(self.h, first_lev, len(new_levels), _ip(nbox), _ip(lohi))
        assert st == 0
        self.levels = self.levels[:first_lev] + [np.ascontiguousarray(b, dtype=np.int32) for b in new_levels]

    def equilibrium_cell(self, rho, vel, temp):
        """f_eq, g_eq of one cell at (rho, vel, T) (the initializer's)."""
        v = np.ascontiguousarray(vel, dtype=np.float64)
        f = np.empty(NQ)
        g = np.empty(NQ)
        self.L.orc_equilibrium_cell(self.h, rho, _dp(v), temp, _dp(f), _dp(g))
        return f, g

    def collide_cell(self, f, g, dq, dt=1.0):
        """One cell's collision with the q-correction gradient dq supplied:
        returns post-collision f, g and the cell's Q_corr (3 values)."""
        f = np.ascontiguousarray(f, dtype=np.float64)
        g = np.ascontiguousarray(g, dtype=np.float64)
        d = np.ascontiguousarray(dq, dtype=np.float64)
        fo = np.empty(NQ)
        go = np.empty(NQ)
        qc = np.empty(3)
        self.L.orc_collide_cell(self.h, _dp(f), _dp(g), _dp(d), dt, _dp(fo), _dp(go), _dp(qc))
        return fo, go, qc

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def per_box_fields(arr, boxes, ncomp):
    """Split a valid-only [box][comp][k][j][i] array into per-box views."""
    out = []
    off = 0
    for b in boxes:
        nx, ny, nz = b[3] - b[0] + 1, b[4] - b[1] + 1, b[5] - b[2] + 1
        n = nx * ny * nz * ncomp
        out.append(arr[off:off + n].reshape(ncomp, nz, ny, nx))
        off += n
    return out


def stencil_tables():
    ev = np.zeros(81, dtype=np.int32)
    w = np.zeros(27)
    b = [np.zeros(27, dtype=np.int32) for _ in range(4)]
    lib().orc_stencil(_ip(ev), _dp(w), *[_ip(x) for x in b])
    return ev.reshape(27, 3), w, b[0], b[1], b[2], b[3]
