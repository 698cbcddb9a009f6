"""ctypes bindings for the oracle (TEST INFRASTRUCTURE ONLY).

Loaded by tests/, by ``__graft_entry__.smoke()`` and by the CPU-baseline leg of ``bench.py`` -- never by
the product package.  Two back ends share one Python interface:

* ``OracleRVE``  -- the C restatement ``oracle/liboracle.so`` (built by ``make -C oracle``), available on
  every machine;
* ``RefRVE``     -- the compiled reference CPU library ``oracle/_ref/libref_{stock,cg1e8}.so`` (built by
  ``oracle/build_ref.sh`` from the reference sources), available only where the reference tree exists.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

FE_LINEAR, FE_ONE_WAY, FE_FULL, MIX_RULE_CHAMIS = 0, 1, 2, 3
MAT_ELASTIC, MAT_PLASTIC, MAT_DAMAGE = 0, 1, 2


class Material(C.Structure):
    """``struct material_base`` (material_base.h:40-45)."""

    _fields_ = [("E", C.c_double), ("nu", C.c_double), ("Ka", C.c_double), ("Sy", C.c_double),
                ("k", C.c_double), ("mu", C.c_double), ("lam", C.c_double), ("Xt", C.c_double),
                ("type", C.c_int)]


class Config(C.Structure):
    """``struct orc_config`` == ``struct micropp3_config`` (same layout)."""

    _fields_ = [("ngp", C.c_int), ("size", C.c_int * 3), ("micro_type", C.c_int),
                ("geo_params", C.c_double * 4), ("materials", Material * 3),
                ("coupling", C.POINTER(C.c_int)), ("subiterations", C.c_int), ("nsubiterations", C.c_int),
                ("mpi_rank", C.c_int), ("nr_max_its", C.c_int), ("nr_max_tol", C.c_double),
                ("nr_rel_tol", C.c_double), ("cg_max_its", C.c_int), ("cg_abs_tol", C.c_double),
                ("cg_rel_tol", C.c_double), ("calc_ctan_lin", C.c_int), ("use_A0", C.c_int),
                ("its_with_A0", C.c_int), ("lin_stress", C.c_int), ("write_log", C.c_int),
                ("elem_type", C.POINTER(C.c_int)), ("precision", C.c_int), ("ctan_mode", C.c_int),
                ("reserved", C.c_int * 4)]


def material(type_, E, nu, Ka=0.0, Sy=0.0, Xt=0.0):
    """``material_set`` (material.c:26-38), computed in Python with the same expressions."""
    m = Material()
    m.E, m.nu, m.Ka, m.Sy, m.Xt, m.type = E, nu, Ka, Sy, Xt, type_
    m.k = E / (3. * (1. - 2. * nu))
    m.mu = E / (2. * (1. + nu))
    m.lam = nu * E / ((1. + nu) * (1. - 2. * nu))
    return m


def make_config(n, ngp=1, micro_type=0, geo=(0.1, 0.1, 0.1, 0.1), mats=None, coupling=None,
                elem_type=None, **kw):
    """A Config with the reference defaults (types.hpp:43-63) and the given overrides.

    ``n`` is the number of elements per axis (nodes = n + 1).  The returned object keeps the coupling and
    element-type arrays alive.
    """
    c = Config()
    c.ngp = ngp
    c.size[:] = [n + 1] * 3 if isinstance(n, int) else [x + 1 for x in n]
    c.micro_type = micro_type
    c.geo_params[:] = list(geo)
    mats = mats or [material(0, 1e7, 0.25)] * 3
    for i in range(3):
        c.materials[i] = mats[i]
    c.subiterations, c.nsubiterations, c.mpi_rank = 0, 10, 0
    c.nr_max_its, c.nr_max_tol, c.nr_rel_tol = 4, 1e-10, 1e-3
    c.cg_max_its, c.cg_abs_tol, c.cg_rel_tol = 1000, 1e-50, 1e-5
    c.calc_ctan_lin, c.use_A0, c.its_with_A0, c.lin_stress, c.write_log = 1, 0, 1, 1, 0
    c.precision, c.ctan_mode = 0, 0
    keep = []
    if coupling is not None:
        arr = (C.c_int * ngp)(*coupling)
        keep.append(arr)
        c.coupling = C.cast(arr, C.POINTER(C.c_int))
    if elem_type is not None:
        et = np.ascontiguousarray(elem_type, dtype=np.int32)
        keep.append(et)
        c.elem_type = et.ctypes.data_as(C.POINTER(C.c_int))
    for k, v in kw.items():
        setattr(c, k, v)
    c._keep = keep
    return c


def _load(path):
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is not built")
    return C.CDLL(path)


class _Base:
    prefix = ""

    def _f(self, name):
        return getattr(self.lib, self.prefix + name)

    def _setup(self):
        L, p = self.lib, self.prefix
        vp = C.c_void_p
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        getattr(L, p + "new").restype = vp
        getattr(L, p + "new").argtypes = [C.POINTER(Config)]
        for n in ("free", "homogenize", "homogenize_linear", "update_vars"):
            getattr(L, p + n).argtypes = [vp]
            getattr(L, p + n).restype = None
        for n in ("set_strain", "get_stress", "get_ctan"):
            getattr(L, p + n).argtypes = [vp, C.c_int, dp]
            getattr(L, p + n).restype = None
        for n in ("is_non_linear", "has_converged", "has_subiterated"):
            getattr(L, p + n).argtypes = [vp, C.c_int]
            getattr(L, p + n).restype = C.c_int
        getattr(L, p + "get_cost").argtypes = [vp, C.c_int]
        getattr(L, p + "get_cost").restype = C.c_long
        getattr(L, p + "get_non_linear_gps").argtypes = [vp]
        getattr(L, p + "get_non_linear_gps").restype = C.c_int
        for n in ("nelem", "nndim"):
            getattr(L, p + n).argtypes = [vp]
            getattr(L, p + n).restype = C.c_int
        getattr(L, p + "get_elem_type").argtypes = [vp, ip]
        for n in ("get_ctan_lin", "get_vol_fractions"):
            getattr(L, p + n).argtypes = [vp, dp]
        for n in ("get_vars", "get_u"):
            getattr(L, p + n).argtypes = [vp, C.c_int, C.c_int, dp]

    def __init__(self, cfg):
        self.cfg = cfg
        self.h = self._f("new")(C.byref(cfg))
        self.ngp = cfg.ngp
        self.nelem = self._f("nelem")(self.h)
        self.nndim = self._f("nndim")(self.h)

    def close(self):
        if self.h:
            self._f("free")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _dp(a):
        return a.ctypes.data_as(C.POINTER(C.c_double))

    def set_strain(self, gp, eps):
        e = np.ascontiguousarray(eps, dtype=np.float64)
        self._f("set_strain")(self.h, gp, self._dp(e))

    def get_stress(self, gp):
        s = np.zeros(6)
        self._f("get_stress")(self.h, gp, self._dp(s))
        return s

    def get_ctan(self, gp):
        c = np.zeros(36)
        self._f("get_ctan")(self.h, gp, self._dp(c))
        return c.reshape(6, 6)

    def homogenize(self):
        self._f("homogenize")(self.h)

    def homogenize_linear(self):
        self._f("homogenize_linear")(self.h)

    def update_vars(self):
        self._f("update_vars")(self.h)

    def is_non_linear(self, gp):
        return bool(self._f("is_non_linear")(self.h, gp))

    def get_non_linear_gps(self):
        return self._f("get_non_linear_gps")(self.h)

    def get_cost(self, gp):
        return self._f("get_cost")(self.h, gp)

    def has_converged(self, gp):
        return bool(self._f("has_converged")(self.h, gp))

    def has_subiterated(self, gp):
        return bool(self._f("has_subiterated")(self.h, gp))

    def elem_type(self):
        a = np.zeros(self.nelem, dtype=np.int32)
        self._f("get_elem_type")(self.h, a.ctypes.data_as(C.POINTER(C.c_int)))
        return a

    def ctan_lin(self):
        a = np.zeros(36)
        self._f("get_ctan_lin")(self.h, self._dp(a))
        return a.reshape(6, 6)

    def vol_fractions(self):
        a = np.zeros(2)
        self._f("get_vol_fractions")(self.h, self._dp(a))
        return a

    def vars(self, gp, which=0):
        a = np.zeros(self.nelem * 8 * 7)
        self._f("get_vars")(self.h, gp, which, self._dp(a))
        return a

    def u(self, gp, which=0):
        a = np.zeros(self.nndim)
        self._f("get_u")(self.h, gp, which, self._dp(a))
        return a


class OracleRVE(_Base):
    """The C restatement (oracle/micropp_oracle.c)."""

    prefix = "orc_"
    lib = None

    def __init__(self, cfg):
        if OracleRVE.lib is None:
            OracleRVE.lib = _load(os.path.join(HERE, "liboracle.so"))
            self._setup()
            L = OracleRVE.lib
            L.orc_get_newton.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                         C.POINTER(C.c_int)]
            L.orc_write_restart.argtypes = [C.c_void_p, C.c_char_p]
            L.orc_write_restart.restype = C.c_int
            L.orc_read_restart.argtypes = [C.c_void_p, C.c_char_p]
            L.orc_read_restart.restype = C.c_int
            L.orc_calc_bmat.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_double)]
            L.orc_get_ops.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
            L.orc_reset_ops.argtypes = [C.c_void_p]
        super().__init__(cfg)

    OPS = ("residual", "assembly", "cg_setup", "cg_iter", "ave_stress", "vars", "homogenize")

    def ops(self, gp):
        """{op: (count, seconds)} of the FE homogenizations of `gp` since construction or reset_ops()."""
        cnt, sec = (C.c_double * 7)(), (C.c_double * 7)()
        self.lib.orc_get_ops(self.h, gp, cnt, sec)
        return {k: (cnt[i], sec[i]) for i, k in enumerate(self.OPS)}

    def reset_ops(self):
        self.lib.orc_reset_ops(self.h)

    def newton(self, gp):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        self.lib.orc_get_newton(self.h, gp, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, bool(c.value)

    def write_restart(self, path):
        return self.lib.orc_write_restart(self.h, path.encode())

    def read_restart(self, path):
        return self.lib.orc_read_restart(self.h, path.encode())


def oracle_available():
    return os.path.exists(os.path.join(HERE, "liboracle.so"))


class RefRVE(_Base):
    """The compiled reference (oracle/_ref/libref_<variant>.so); ``variant`` is 'stock' or 'cg1e8'."""

    prefix = "ref_"
    libs = {}

    def __init__(self, cfg, variant="stock"):
        if variant not in RefRVE.libs:
            lib = _load(os.path.join(HERE, "_ref", f"libref_{variant}.so"))
            RefRVE.libs[variant] = lib
            self.lib = lib
            self._setup()
            lib.ref_write_restart.argtypes = [C.c_void_p, C.c_int]
            lib.ref_read_restart.argtypes = [C.c_void_p, C.c_int]
            lib.ref_output.argtypes = [C.c_void_p, C.c_int, C.c_char_p]
        self.lib = RefRVE.libs[variant]
        super().__init__(cfg)

    def write_restart(self, restart_id):
        self.lib.ref_write_restart(self.h, restart_id)

    def read_restart(self, restart_id):
        self.lib.ref_read_restart(self.h, restart_id)

    def output(self, gp, filename):
        self.lib.ref_output(self.h, gp, filename.encode())


def ref_available(variant="stock"):
    return os.path.exists(os.path.join(HERE, "_ref", f"libref_{variant}.so"))
