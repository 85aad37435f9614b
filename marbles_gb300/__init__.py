"""GB300-native MARBLES level step: Python binding of libmarbles_gpu.so.

The compute path is the CUDA library built from marbles_gb300/csrc; this
module only marshals arguments through ctypes.  There is no CPU fallback:
if the library is missing or cannot be loaded, every call raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmarbles_gpu.so")

NQ = 27
NMACRO = 19

FP64, FP32C_F16S, FP32C_BF16S = 0, 1, 2
STATUS = {0: "MBG_OK", 1: "MBG_EINVAL", 2: "MBG_ENOMEM", 3: "MBG_ECUDA", 4: "MBG_ETIMEOUT", 5: "MBG_ESTATE"}

# every entry point declared in include/marbles_gb300.h
EXPORTS = [
    "mbg_create", "mbg_destroy", "mbg_last_error", "mbg_define_level", "mbg_level_cells",
    "mbg_set_state", "mbg_get_state", "mbg_get_macro", "mbg_step", "mbg_advance_level",
    "mbg_fillpatch", "mbg_average_down", "mbg_eb_forces", "mbg_synchronize", "mbg_launch_count",
    "mbg_stream", "mbg_set_timing", "mbg_timing_count", "mbg_timing", "mbg_step_box_noalloc",
    "mbg_lbm_create", "mbg_lbm_prepare", "mbg_lbm_initial_state", "mbg_lbm_init", "mbg_lbm_evolve", "mbg_lbm_context", "mbg_lbm_num_levels",
    "mbg_lbm_level_boxes", "mbg_lbm_level_flags", "mbg_lbm_write_plotfile", "mbg_lbm_last_error",
    "mbg_lbm_destroy", "mbg_lbm_write_checkpoint", "mbg_lbm_step_time", "mbg_tag_cells", "mbg_regrid", "mbg_lbm_regrid",
    "mbg_geometry_flags",
    "mbg_get_derived", "mbg_conserved", "mbg_check_state", "mbg_autotune", "mbg_tuning", "mbg_set_variant",
    "mbg_write_plotfile", "mbg_write_multifab", "mbg_read_multifab",
    "mbg_batch_create", "mbg_batch_cells", "mbg_batch_set_state", "mbg_batch_get_state", "mbg_batch_get_macro",
    "mbg_batch_step", "mbg_batch_autotune", "mbg_batch_tuning", "mbg_batch_synchronize", "mbg_batch_launch_count",
    "mbg_batch_stream", "mbg_batch_last_error", "mbg_batch_destroy",
    "mbg_adj_create", "mbg_adj_forward", "mbg_adj_backward", "mbg_adj_launch_count", "mbg_adj_stream",
    "mbg_adj_last_error", "mbg_adj_destroy",
]


class MbgError(RuntimeError):
    pass


class MbgParams(C.Structure):
    """Mirror of struct mbg_params (include/marbles_gb300.h)."""
    _fields_ = [
        ("n_cell", C.c_int * 3),
        ("prob_lo", C.c_double * 3), ("prob_hi", C.c_double * 3),
        ("is_periodic", C.c_int * 3),
        ("bc_lo", C.c_int * 3), ("bc_hi", C.c_int * 3),
        ("nu", C.c_double), ("alpha", C.c_double),
        ("dx_outer", C.c_double), ("dt_outer", C.c_double),
        ("adiabatic_exponent", C.c_double), ("m_bar", C.c_double),
        ("precision", C.c_int),
        ("rho_ref", C.c_double), ("t_ref", C.c_double),
        ("velbc_type", C.c_int),
        ("vbc_dir", C.c_int), ("vbc_normal_dir", C.c_int), ("vbc_tangential_dir", C.c_int),
        ("vbc_u_ref", C.c_double), ("vbc_initial_density", C.c_double),
        ("vbc_initial_temperature", C.c_double), ("vbc_adiabatic_exponent", C.c_double),
        ("vbc_m_bar", C.c_double),
        ("u_ref", C.c_double * 3),
    ]


class MbgTag(C.Structure):
    """mirror of mbg_tag (one refinement criterion)"""
    _fields_ = [("field", C.c_int), ("kind", C.c_int), ("value", C.c_double), ("has_box", C.c_int),
                ("box_lo", C.c_double * 3), ("box_hi", C.c_double * 3), ("start_time", C.c_double),
                ("end_time", C.c_double), ("max_level", C.c_int)]


# macro field names of mbg_get_macro (Source/Constants.H order) and is_fluid
FIELDS = ["rho", "vel_x", "vel_y", "vel_z", "vel_mag", "two_rho_e", "QCorrX", "QCorrY", "QCorrZ", "pxx", "pyy",
          "pzz", "pxy", "pxz", "pyz", "qx", "qy", "qz", "temperature", "is_fluid"]


def make_tag(field="rho", kind="greater", value=0.0, box=None, start_time=-1.0e300, end_time=1.0e300,
             max_level=1000):
    t = MbgTag()
    t.field = FIELDS.index(field) if isinstance(field, str) else field
    t.kind = {"box": 0, "greater": 1, "less": 2}[kind]
    t.value = value
    t.has_box = 1 if box is not None else 0
    if box is not None:
        t.box_lo[:] = list(box[0])
        t.box_hi[:] = list(box[1])
    t.start_time, t.end_time, t.max_level = start_time, end_time, max_level
    return t


class MbgDomain(C.Structure):
    """mirror of mbg_domain (one domain of a batch)"""
    _fields_ = [("n_cell", C.c_int * 3), ("prob_lo", C.c_double * 3), ("prob_hi", C.c_double * 3),
                ("nu", C.c_double), ("alpha", C.c_double)]


_lib = None


def lib():
    """Load the CUDA library (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise MbgError("libmarbles_gpu.so is not built (run __graft_entry__.build())")
        L = C.CDLL(LIB_PATH)
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.mbg_create.argtypes = [C.POINTER(MbgParams), vp, C.POINTER(vp)]
        L.mbg_destroy.argtypes = [vp]
        L.mbg_destroy.restype = None
        L.mbg_last_error.argtypes = [vp]
        L.mbg_last_error.restype = C.c_char_p
        L.mbg_define_level.argtypes = [vp, C.c_int, C.c_int, ip, C.POINTER(C.c_uint8)]
        L.mbg_level_cells.argtypes = [vp, C.c_int, C.POINTER(C.c_longlong)]
        L.mbg_set_state.argtypes = [vp, C.c_int, dp, dp]
        L.mbg_get_state.argtypes = [vp, C.c_int, dp, dp]
        L.mbg_get_macro.argtypes = [vp, C.c_int, dp]
        L.mbg_tag_cells.argtypes = [vp, C.c_int, C.POINTER(MbgTag), C.c_int, C.c_double, C.POINTER(C.c_uint8)]
        L.mbg_regrid.argtypes = [vp, C.c_int, C.c_int, ip, ip, C.POINTER(C.c_uint8)]
        L.mbg_lbm_regrid.argtypes = [vp]
        L.mbg_get_derived.argtypes = [vp, C.c_int, dp]
        L.mbg_write_plotfile.argtypes = [C.c_char_p, C.c_int, ip, ip, ip, dp, dp, C.c_int,
                                         C.POINTER(C.c_char_p), C.POINTER(dp), C.c_double, ip]
        L.mbg_write_multifab.argtypes = [C.c_char_p, C.c_int, ip, C.c_int, dp]
        L.mbg_read_multifab.argtypes = [C.c_char_p, C.c_int, ip, C.c_int, dp]
        L.mbg_lbm_write_checkpoint.argtypes = [vp, C.c_char_p]
        L.mbg_lbm_step_time.argtypes = [vp, ip, dp]
        L.mbg_step.argtypes = [vp, C.c_int]
        L.mbg_advance_level.argtypes = [vp, C.c_int]
        L.mbg_fillpatch.argtypes = [vp, C.c_int]
        L.mbg_average_down.argtypes = [vp, C.c_int, C.c_int]
        L.mbg_autotune.argtypes = [vp, C.c_int]
        L.mbg_adj_create.argtypes = [C.POINTER(MbgParams), C.c_double, dp, vp, C.POINTER(vp)]
        L.mbg_adj_forward.argtypes = [vp, dp, C.c_int, C.c_int, dp]
        L.mbg_adj_backward.argtypes = [vp, dp, dp]
        L.mbg_adj_launch_count.argtypes = [vp]
        L.mbg_adj_launch_count.restype = C.c_longlong
        L.mbg_adj_stream.argtypes = [vp]
        L.mbg_adj_stream.restype = vp
        L.mbg_adj_last_error.argtypes = [vp]
        L.mbg_adj_last_error.restype = C.c_char_p
        L.mbg_adj_destroy.argtypes = [vp]
        L.mbg_adj_destroy.restype = None
        L.mbg_batch_create.argtypes = [C.POINTER(MbgParams), C.c_int, C.POINTER(MbgDomain), vp, C.POINTER(vp)]
        L.mbg_batch_cells.argtypes = [vp, C.POINTER(C.c_longlong)]
        L.mbg_batch_set_state.argtypes = [vp, dp, dp]
        L.mbg_batch_get_state.argtypes = [vp, dp, dp]
        L.mbg_batch_get_macro.argtypes = [vp, dp]
        L.mbg_batch_step.argtypes = [vp, C.c_int]
        L.mbg_batch_autotune.argtypes = [vp, C.c_int]
        L.mbg_batch_tuning.argtypes = [vp, C.POINTER(C.c_int), dp]
        L.mbg_batch_synchronize.argtypes = [vp]
        L.mbg_batch_launch_count.argtypes = [vp]
        L.mbg_batch_launch_count.restype = C.c_longlong
        L.mbg_batch_stream.argtypes = [vp]
        L.mbg_batch_stream.restype = vp
        L.mbg_batch_last_error.argtypes = [vp]
        L.mbg_batch_last_error.restype = C.c_char_p
        L.mbg_batch_destroy.argtypes = [vp]
        L.mbg_batch_destroy.restype = None
        L.mbg_tuning.argtypes = [vp, C.c_int, C.POINTER(C.c_int), dp]
        L.mbg_eb_forces.argtypes = [vp, dp]
        L.mbg_conserved.argtypes = [vp, dp]
        L.mbg_synchronize.argtypes = [vp]
        L.mbg_launch_count.argtypes = [vp]
        L.mbg_launch_count.restype = C.c_longlong
        L.mbg_step_box_noalloc.argtypes = [C.POINTER(MbgParams), vp, vp, vp, vp, vp]
        L.mbg_stream.argtypes = [vp]
        L.mbg_stream.restype = vp
        L.mbg_set_timing.argtypes = [vp, C.c_int]
        L.mbg_timing_count.argtypes = []
        L.mbg_timing.argtypes = [vp, C.c_int, C.POINTER(C.c_char_p), C.POINTER(C.c_longlong),
                                 C.POINTER(C.c_double)]
        L.mbg_lbm_create.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_char_p), C.POINTER(vp)]
        L.mbg_lbm_init.argtypes = [vp]
        L.mbg_lbm_prepare.argtypes = [vp]
        L.mbg_lbm_initial_state.argtypes = [vp, C.c_int, dp, dp]
        L.mbg_lbm_evolve.argtypes = [vp, C.c_int]
        L.mbg_lbm_context.argtypes = [vp]
        L.mbg_lbm_context.restype = vp
        L.mbg_lbm_num_levels.argtypes = [vp]
        L.mbg_lbm_level_boxes.argtypes = [vp, C.c_int, ip, C.c_int, ip]
        L.mbg_lbm_level_flags.argtypes = [vp, C.c_int, C.POINTER(C.c_uint8), C.c_longlong,
                                          C.POINTER(C.c_longlong)]
        L.mbg_lbm_write_plotfile.argtypes = [vp, C.c_char_p]
        L.mbg_lbm_last_error.argtypes = [vp]
        L.mbg_lbm_last_error.restype = C.c_char_p
        L.mbg_lbm_destroy.argtypes = [vp]
        L.mbg_lbm_destroy.restype = None
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def default_params():
    p = MbgParams()
    p.n_cell[:] = [8, 8, 8]
    p.prob_lo[:] = [0.0, 0.0, 0.0]
    p.prob_hi[:] = [8.0, 8.0, 8.0]
    p.is_periodic[:] = [1, 1, 1]
    p.nu = 1.0
    p.alpha = 1.0
    p.dx_outer = 1.0
    p.dt_outer = 1.0
    p.adiabatic_exponent = 5.0 / 3.0
    p.m_bar = 28.96
    p.precision = FP64
    p.rho_ref = 1.0
    p.t_ref = 1.0 / 3.0
    p.velbc_type = 0
    p.vbc_dir = 1
    p.vbc_normal_dir = 0
    p.vbc_tangential_dir = 1
    p.vbc_initial_density = 1.0
    p.vbc_initial_temperature = 1.0 / 3.0
    p.vbc_adiabatic_exponent = 5.0 / 3.0
    p.vbc_m_bar = 28.96
    return p


class Context:
    """One simulation on the GPU (all levels), through the C ABI."""

    def __init__(self, params, stream=None):
        self.L = lib()
        self.p = params
        h = C.c_void_p()
        st = self.L.mbg_create(C.byref(params), stream, C.byref(h))
        if st != 0:
            raise MbgError("mbg_create: %s: %s" % (STATUS.get(st, st), self.L.mbg_last_error(None).decode()))
        self.h = h
        self.boxes = []

    def _check(self, st, what):
        if st != 0:
            raise MbgError("%s: %s: %s" % (what, STATUS.get(st, st), self.L.mbg_last_error(self.h).decode()))

    def define_level(self, lev, boxes, flags=None):
        """boxes: (nbox, 6) lo/hi; flags: uint8 per grown-box cell or None."""
        b = np.ascontiguousarray(boxes, dtype=np.int32)
        fl = None
        if flags is not None:
            flags = np.ascontiguousarray(flags, dtype=np.uint8)
            fl = flags.ctypes.data_as(C.POINTER(C.c_uint8))
        self._check(self.L.mbg_define_level(self.h, lev, b.shape[0], b.ctypes.data_as(C.POINTER(C.c_int)), fl),
                    "mbg_define_level")
        self.boxes.append(b)

    def ncells(self, lev):
        n = C.c_longlong()
        self._check(self.L.mbg_level_cells(self.h, lev, C.byref(n)), "mbg_level_cells")
        return n.value

    def set_state(self, lev, f, g):
        f = np.ascontiguousarray(f, dtype=np.float64)
        g = np.ascontiguousarray(g, dtype=np.float64)
        self._check(self.L.mbg_set_state(self.h, lev, _dp(f), _dp(g)), "mbg_set_state")

    def get_state(self, lev):
        n = self.ncells(lev)
        f = np.empty(n * NQ)
        g = np.empty(n * NQ)
        self._check(self.L.mbg_get_state(self.h, lev, _dp(f), _dp(g)), "mbg_get_state")
        return f, g

    def get_macro(self, lev):
        m = np.empty(self.ncells(lev) * NMACRO)
        self._check(self.L.mbg_get_macro(self.h, lev, _dp(m)), "mbg_get_macro")
        return m

    def get_derived(self, lev):
        """vort_x, vort_y, vort_z, vort_mag, dQCorrX..Z of the stored state, [box][7][cell]."""
        m = np.empty(self.ncells(lev) * 7)
        self._check(self.L.mbg_get_derived(self.h, lev, _dp(m)), "mbg_get_derived")
        return m

    def tag_cells(self, lev, tags, time):
        """ErrorEst tags (0/1 per valid cell of level lev, [box][cell])."""
        arr = (MbgTag * len(tags))(*tags)
        out = np.zeros(self.ncells(lev), dtype=np.uint8)
        self._check(self.L.mbg_tag_cells(self.h, lev, arr, len(tags), time,
                                         out.ctypes.data_as(C.POINTER(C.c_uint8))), "mbg_tag_cells")
        return out

    def regrid(self, first_lev, levels, flags=None):
        """Replace levels first_lev.. by the box arrays `levels` (flags per
        level in the layout of define_level, None: all fluid)."""
        nbox = np.array([len(b) for b in levels] or [0], dtype=np.int32)
        parts = [np.asarray(b, dtype=np.int32).reshape(-1) for b in levels]
        lohi = np.ascontiguousarray(np.concatenate(parts) if parts else np.zeros(6, dtype=np.int32))
        if flags is None:
            flags = [np.ones(int(np.prod(np.asarray(b)[:, 3:] - np.asarray(b)[:, :3] + 7, axis=1).sum()),
                             dtype=np.uint8) for b in levels]
        fparts = [np.asarray(f, dtype=np.uint8) for f in flags]
        fl = np.ascontiguousarray(np.concatenate(fparts) if fparts else np.zeros(1, dtype=np.uint8))
        ipt = C.POINTER(C.c_int)
        self._check(self.L.mbg_regrid(self.h, first_lev, len(levels), nbox.ctypes.data_as(ipt),
                                      lohi.ctypes.data_as(ipt), fl.ctypes.data_as(C.POINTER(C.c_uint8))),
                    "mbg_regrid")
        if getattr(self, "boxes", None) is not None:
            self.boxes = self.boxes[:first_lev] + [np.asarray(b) for b in levels]

    def step(self, n=1):
        self._check(self.L.mbg_step(self.h, n), "mbg_step")

    def advance_level(self, lev):
        self._check(self.L.mbg_advance_level(self.h, lev), "mbg_advance_level")

    def fillpatch(self, lev):
        self._check(self.L.mbg_fillpatch(self.h, lev), "mbg_fillpatch")

    def average_down(self, crse_lev, ng):
        self._check(self.L.mbg_average_down(self.h, crse_lev, ng), "mbg_average_down")

    def autotune(self, reps=3):
        """Time the step variants of every level and keep the fastest (16-bit forms)."""
        self._check(self.L.mbg_autotune(self.h, reps), "mbg_autotune")

    def set_variant(self, variant, lev=-1):
        """Run step variant `variant` on level lev (every level for lev = -1)."""
        self._check(self.L.mbg_set_variant(self.h, lev, variant), "mbg_set_variant")

    def tuning(self, lev):
        """(chosen variant, [ms per step of variants 0..3]) of level lev."""
        v = C.c_int()
        ms = np.zeros(4)
        self._check(self.L.mbg_tuning(self.h, lev, C.byref(v), _dp(ms)), "mbg_tuning")
        return v.value, ms.tolist()

    def conserved(self):
        """[mass, momentum x, y, z, sum of 2 rho E] over the hierarchy (FP64)."""
        out = np.zeros(5)
        self._check(self.L.mbg_conserved(self.h, _dp(out)), "mbg_conserved")
        return out

    def check_state(self):
        """((bad values at fluid cells, at solid cells), (level, box, cell,
        2 q + lattice) of the first, or -1s): the state scan of
        mbg_check_state."""
        counts = (C.c_longlong * 2)()
        first = (C.c_longlong * 4)()
        self._check(self.L.mbg_check_state(self.h, counts, first), "mbg_check_state")
        return (counts[0], counts[1]), tuple(first)

    def eb_forces(self):
        out = np.zeros(3)
        self._check(self.L.mbg_eb_forces(self.h, _dp(out)), "mbg_eb_forces")
        return out

    def synchronize(self):
        self._check(self.L.mbg_synchronize(self.h), "mbg_synchronize")

    def launch_count(self):
        return self.L.mbg_launch_count(self.h)

    def stream(self):
        return self.L.mbg_stream(self.h)

    def set_timing(self, on):
        self._check(self.L.mbg_set_timing(self.h, 1 if on else 0), "mbg_set_timing")

    def timing(self):
        """{kernel class: (launches, total device ms)} since timing was enabled."""
        out = {}
        for k in range(self.L.mbg_timing_count()):
            name, n, ms = C.c_char_p(), C.c_longlong(), C.c_double()
            self._check(self.L.mbg_timing(self.h, k, C.byref(name), C.byref(n), C.byref(ms)), "mbg_timing")
            out[name.value.decode()] = (n.value, ms.value)
        return out

    def close(self):
        if getattr(self, "h", None):
            self.L.mbg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent periodic domains stepped together (mbg_batch_*).

    domains: sequence of (n_cell[3], prob_lo[3], prob_hi[3], nu, alpha)."""

    def __init__(self, common, domains, stream=None):
        self.L = lib()
        arr = (MbgDomain * len(domains))()
        for i, (n, lo, hi, nu, alpha) in enumerate(domains):
            arr[i].n_cell[:] = [int(v) for v in n]
            arr[i].prob_lo[:] = [float(v) for v in lo]
            arr[i].prob_hi[:] = [float(v) for v in hi]
            arr[i].nu, arr[i].alpha = float(nu), float(alpha)
        h = C.c_void_p()
        st = self.L.mbg_batch_create(C.byref(common), len(domains), arr, stream, C.byref(h))
        if st != 0:
            raise MbgError("mbg_batch_create: %s: %s" % (STATUS.get(st, st), self.L.mbg_last_error(None).decode()))
        self.h = h
        n = C.c_longlong()
        self._check(self.L.mbg_batch_cells(self.h, C.byref(n)), "mbg_batch_cells")
        self.n = n.value

    def _check(self, st, what):
        if st != 0:
            raise MbgError("%s: %s: %s" % (what, STATUS.get(st, st), self.L.mbg_batch_last_error(self.h).decode()))

    def ncells(self):
        return self.n

    def set_state(self, f, g):
        f = np.ascontiguousarray(f, dtype=np.float64)
        g = np.ascontiguousarray(g, dtype=np.float64)
        assert f.size == g.size == self.n * NQ
        self._check(self.L.mbg_batch_set_state(self.h, _dp(f), _dp(g)), "mbg_batch_set_state")

    def get_state(self):
        f = np.empty(self.n * NQ)
        g = np.empty(self.n * NQ)
        self._check(self.L.mbg_batch_get_state(self.h, _dp(f), _dp(g)), "mbg_batch_get_state")
        return f, g

    def get_macro(self):
        out = np.empty(self.n * 19)
        self._check(self.L.mbg_batch_get_macro(self.h, _dp(out)), "mbg_batch_get_macro")
        return out

    def step(self, n=1):
        self._check(self.L.mbg_batch_step(self.h, n), "mbg_batch_step")

    def autotune(self, reps=3):
        self._check(self.L.mbg_batch_autotune(self.h, reps), "mbg_batch_autotune")

    def tuning(self):
        v = C.c_int()
        ms = np.zeros(4)
        self._check(self.L.mbg_batch_tuning(self.h, C.byref(v), _dp(ms)), "mbg_batch_tuning")
        return v.value, ms.tolist()

    def synchronize(self):
        self._check(self.L.mbg_batch_synchronize(self.h), "mbg_batch_synchronize")

    def launch_count(self):
        return self.L.mbg_batch_launch_count(self.h)

    def stream(self):
        return self.L.mbg_batch_stream(self.h)

    def close(self):
        if getattr(self, "h", None):
            self.L.mbg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Adjoint:
    """FP64 forward run and its discrete adjoint on one periodic box
    (mbg_adj_*): T0 -> T_final, and dL/dT_final -> dL/dT0."""

    def __init__(self, params, rho0=1.0, u0=(0.0, 0.0, 0.0), stream=None):
        self.L = lib()
        h = C.c_void_p()
        u = np.ascontiguousarray(u0, dtype=np.float64)
        st = self.L.mbg_adj_create(C.byref(params), float(rho0), _dp(u), stream, C.byref(h))
        if st != 0:
            raise MbgError("mbg_adj_create: %s: %s" % (STATUS.get(st, st), self.L.mbg_last_error(None).decode()))
        self.h = h
        self.n = int(params.n_cell[0]) * int(params.n_cell[1]) * int(params.n_cell[2])

    def _check(self, st, what):
        if st != 0:
            raise MbgError("%s: %s: %s" % (what, STATUS.get(st, st), self.L.mbg_adj_last_error(self.h).decode()))

    def forward(self, T0, nsteps, K):
        T0 = np.ascontiguousarray(T0, dtype=np.float64).reshape(-1)
        assert T0.size == self.n
        out = np.empty(self.n)
        self._check(self.L.mbg_adj_forward(self.h, _dp(T0), int(nsteps), int(K), _dp(out)), "mbg_adj_forward")
        return out

    def backward(self, dL_dTfinal):
        g = np.ascontiguousarray(dL_dTfinal, dtype=np.float64).reshape(-1)
        out = np.empty(self.n)
        self._check(self.L.mbg_adj_backward(self.h, _dp(g), _dp(out)), "mbg_adj_backward")
        return out

    def launch_count(self):
        return self.L.mbg_adj_launch_count(self.h)

    def stream(self):
        return self.L.mbg_adj_stream(self.h)

    def close(self):
        if getattr(self, "h", None):
            self.L.mbg_adj_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def temperature_evolution(adj, nsteps, K):
    """A torch.autograd.Function over the C ABI: T0 (FP64 tensor, one value per
    cell) -> T_final after nsteps steps; its backward is the library's
    hand-written adjoint (mbg_adj_backward)."""
    import torch

    class _Evolve(torch.autograd.Function):
        @staticmethod
        def forward(ctx, T0):
            out = adj.forward(T0.detach().cpu().numpy(), nsteps, K)
            return torch.from_numpy(out).to(T0.device)

        @staticmethod
        def backward(ctx, grad):
            g = adj.backward(grad.detach().cpu().numpy())
            return torch.from_numpy(g).to(grad.device)

    return _Evolve.apply


class LBM:
    """The host drop-in driver: inputs text with the reference's keys."""

    def __init__(self, inputs_text, overrides=()):
        self.L = lib()
        h = C.c_void_p()
        ov = (C.c_char_p * max(1, len(overrides)))(*[o.encode() for o in overrides])
        st = self.L.mbg_lbm_create(inputs_text.encode(), len(overrides), ov, C.byref(h))
        if st != 0:
            raise MbgError("mbg_lbm_create: %s: %s" % (STATUS.get(st, st), self.L.mbg_lbm_last_error(None).decode()))
        self.h = h
        self.ctx = None

    def _check(self, st, what):
        if st != 0:
            raise MbgError("%s: %s: %s" % (what, STATUS.get(st, st), self.L.mbg_lbm_last_error(self.h).decode()))

    def init(self):
        self._check(self.L.mbg_lbm_init(self.h), "mbg_lbm_init")
        ctx = Context.__new__(Context)
        ctx.L = self.L
        ctx.h = C.c_void_p(self.L.mbg_lbm_context(self.h))
        ctx.p = None
        ctx.boxes = [self.boxes(l) for l in range(self.num_levels())]
        ctx.close = lambda: None        # owned by the driver
        self.ctx = ctx
        return ctx

    def evolve(self, nsteps):
        self._check(self.L.mbg_lbm_evolve(self.h, nsteps), "mbg_lbm_evolve")

    def prepare(self):
        """Grids and flags on the host (no GPU work)."""
        self._check(self.L.mbg_lbm_prepare(self.h), "mbg_lbm_prepare")

    def initial_state(self, lev):
        b = self.boxes(lev)
        n = int(np.prod(b[:, 3:] - b[:, :3] + 1, axis=1).sum())
        f = np.empty(n * NQ)
        g = np.empty(n * NQ)
        self._check(self.L.mbg_lbm_initial_state(self.h, lev, _dp(f), _dp(g)), "mbg_lbm_initial_state")
        return f, g

    def num_levels(self):
        return self.L.mbg_lbm_num_levels(self.h)

    def boxes(self, lev):
        n = C.c_int()
        self._check(self.L.mbg_lbm_level_boxes(self.h, lev, None, 0, C.byref(n)), "mbg_lbm_level_boxes")
        out = np.zeros(6 * n.value, dtype=np.int32)
        self._check(self.L.mbg_lbm_level_boxes(self.h, lev, out.ctypes.data_as(C.POINTER(C.c_int)), n.value,
                                               C.byref(n)), "mbg_lbm_level_boxes")
        return out.reshape(-1, 6)

    def flags(self, lev):
        n = C.c_longlong()
        self._check(self.L.mbg_lbm_level_flags(self.h, lev, None, 0, C.byref(n)), "mbg_lbm_level_flags")
        out = np.zeros(n.value, dtype=np.uint8)
        self._check(self.L.mbg_lbm_level_flags(self.h, lev, out.ctypes.data_as(C.POINTER(C.c_uint8)), n.value,
                                               C.byref(n)), "mbg_lbm_level_flags")
        return out

    def write_plotfile(self, name):
        self._check(self.L.mbg_lbm_write_plotfile(self.h, name.encode()), "mbg_lbm_write_plotfile")

    def regrid(self):
        """Tag on the GPU, rebuild the fine grids, remake the changed levels."""
        self._check(self.L.mbg_lbm_regrid(self.h), "mbg_lbm_regrid")
        if self.ctx is not None:
            self.ctx.boxes = [self.boxes(l) for l in range(self.num_levels())]

    def write_checkpoint(self, name):
        self._check(self.L.mbg_lbm_write_checkpoint(self.h, name.encode()), "mbg_lbm_write_checkpoint")

    def step_time(self):
        """(coarse steps taken, simulated time)"""
        n, t = C.c_int(), C.c_double()
        self._check(self.L.mbg_lbm_step_time(self.h, C.byref(n), C.byref(t)), "mbg_lbm_step_time")
        return n.value, t.value

    def close(self):
        if getattr(self, "h", None):
            self.L.mbg_lbm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _io_check(st, what):
    if st != 0:
        raise MbgError("%s: %s: %s" % (what, STATUS.get(st, st), lib().mbg_last_error(None).decode()))


def write_plotfile(path, levels, data, varnames, n_cell, prob_lo, prob_hi, time=0.0, level_steps=None):
    """AMReX plotfile of host data (no GPU work): levels = [(nbox, 6) lo/hi],
    data = [array [box][comp][cell] per level], varnames one per component."""
    L = lib()
    nlev = len(levels)
    nbox = np.array([len(b) for b in levels], dtype=np.int32)
    lohi = np.ascontiguousarray(np.concatenate([np.asarray(b, dtype=np.int32).reshape(-1) for b in levels]))
    arrs = [np.ascontiguousarray(d, dtype=np.float64) for d in data]
    ptrs = (C.POINTER(C.c_double) * nlev)(*[_dp(a) for a in arrs])
    names = (C.c_char_p * len(varnames))(*[v.encode() for v in varnames])
    steps = np.asarray(level_steps if level_steps is not None else [0] * nlev, dtype=np.int32)
    nc = np.asarray(n_cell, dtype=np.int32)
    lo = np.asarray(prob_lo, dtype=np.float64)
    hi = np.asarray(prob_hi, dtype=np.float64)
    ipt = C.POINTER(C.c_int)
    _io_check(L.mbg_write_plotfile(path.encode(), nlev, nbox.ctypes.data_as(ipt), lohi.ctypes.data_as(ipt),
                                   nc.ctypes.data_as(ipt), _dp(lo), _dp(hi), len(varnames), names, ptrs,
                                   float(time), steps.ctypes.data_as(ipt)), "mbg_write_plotfile")


def write_multifab(prefix, boxes, ncomp, data):
    """VisMF multifab <prefix>_H / <prefix>_D_00000 of host data [box][comp][cell]."""
    b = np.ascontiguousarray(np.asarray(boxes, dtype=np.int32).reshape(-1))
    d = np.ascontiguousarray(data, dtype=np.float64)
    _io_check(lib().mbg_write_multifab(prefix.encode(), len(b) // 6, b.ctypes.data_as(C.POINTER(C.c_int)), ncomp,
                                       _dp(d)), "mbg_write_multifab")


def read_multifab(prefix, boxes, ncomp):
    b = np.ascontiguousarray(np.asarray(boxes, dtype=np.int32).reshape(-1))
    bb = b.reshape(-1, 6)
    n = int(np.prod(bb[:, 3:] - bb[:, :3] + 1, axis=1).sum())
    out = np.empty(n * ncomp)
    _io_check(lib().mbg_read_multifab(prefix.encode(), len(bb), b.ctypes.data_as(C.POINTER(C.c_int)), ncomp,
                                      _dp(out)), "mbg_read_multifab")
    return out
