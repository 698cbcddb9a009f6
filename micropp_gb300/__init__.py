"""micropp_gb300 -- GB300-native RVE homogenization behind Micropp's micropp3 C ABI.

The product is the shared library ``libmicropp_gb300.so`` (C ABI: ``include/micropp_c.h`` for the drop-in
entry points, ``include/micropp_gb300.h`` for the extensions; C++ API: ``include/micropp.hpp``).  This
module is its Python mirror: ``Micropp`` exposes the methods of the reference's ``micropp<3>`` class
(micropp.hpp:176-217) through ctypes, with the same names and argument meaning.  There is no CPU path:
constructing a ``Micropp`` without the library, or without a CUDA device, raises.
"""
import ctypes as C
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "libmicropp_gb300.so")

FE_LINEAR, FE_ONE_WAY, FE_FULL, MIX_RULE_CHAMIS = 0, 1, 2, 3
MATERIAL_ELASTIC, MATERIAL_PLASTIC, MATERIAL_DAMAGE = 0, 1, 2
(MIC_HOMOGENEOUS, MIC_SPHERE, MIC_LAYER_Y, MIC_CILI_FIB_X, MIC_CILI_FIB_Z, MIC_CILI_FIB_XZ, MIC_QUAD_FIB_XYZ,
 MIC_QUAD_FIB_XZ, MIC_QUAD_FIB_XZ_BROKEN_X, MIC3D_SPHERES, MIC3D_8, MIC3D_FIBS_20_ORDER,
 MIC3D_FIBS_20_DISORDER) = range(13)
FP64, MIXED = 0, 1
CTAN_PERTURB, CTAN_IMPLICIT = 0, 1
PRECOND_JACOBI, PRECOND_MG, PRECOND_MG_HALF = 0, 1, 2
STATUS_OK, STATUS_NEWTON_MAX_ITS, STATUS_CG_MAX_ITS, STATUS_NONFINITE = 0, 1, 2, 4


class MaterialBase(C.Structure):
    """``struct material_base`` (include/material_base.h)."""

    _fields_ = [("E", C.c_double), ("nu", C.c_double), ("Ka", C.c_double), ("Sy", C.c_double),
                ("k", C.c_double), ("mu", C.c_double), ("lam", C.c_double), ("Xt", C.c_double),
                ("type", C.c_int)]


class Config(C.Structure):
    """``struct micropp3_config`` (include/micropp_gb300.h)."""

    _fields_ = [("ngp", C.c_int), ("size", C.c_int * 3), ("micro_type", C.c_int),
                ("geo_params", C.c_double * 4), ("materials", MaterialBase * 3),
                ("coupling", C.POINTER(C.c_int)), ("subiterations", C.c_int), ("nsubiterations", C.c_int),
                ("mpi_rank", C.c_int), ("nr_max_its", C.c_int), ("nr_max_tol", C.c_double),
                ("nr_rel_tol", C.c_double), ("cg_max_its", C.c_int), ("cg_abs_tol", C.c_double),
                ("cg_rel_tol", C.c_double), ("calc_ctan_lin", C.c_int), ("use_A0", C.c_int),
                ("its_with_A0", C.c_int), ("lin_stress", C.c_int), ("write_log", C.c_int),
                ("elem_type", C.POINTER(C.c_int)), ("precision", C.c_int), ("ctan_mode", C.c_int),
                ("precond", C.c_int), ("reserved", C.c_int * 3)]


class Handle(C.Structure):
    """``struct micropp3`` (include/micropp_c.h)."""

    _fields_ = [("ptr", C.c_void_p)]


_lib = None


def library_available():
    return os.path.exists(LIB_PATH)


def load():
    """Load the library (once).  Raises if it was not built: there is no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing; build it with `python -m micropp_gb300.build` "
                           "(the GB300 library has no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    H = C.POINTER(Handle)
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    sig = {
        "material_set": (None, [C.POINTER(MaterialBase), C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                C.c_double]),
        "micropp3_config_default": (None, [C.POINTER(Config)]),
        "micropp3_new_ext": (None, [H, C.POINTER(Config)]),
        "micropp3_new": (None, [H, C.c_int, ip, C.c_int, dp, C.POINTER(MaterialBase), ip, C.c_int, C.c_int]),
        "micropp3_free": (None, [H]),
        "micropp3_last_error": (C.c_char_p, []),
        "micropp3_clear_error": (None, []),
        "micropp3_set_strain": (None, [H, C.c_int, dp]),
        "micropp3_get_stress": (None, [H, C.c_int, dp]),
        "micropp3_get_ctan": (None, [H, C.c_int, dp]),
        "micropp3_homogenize": (None, [H]),
        "micropp3_homogenize_linear": (None, [H]),
        "micropp3_update_vars": (None, [H]),
        "micropp3_is_non_linear": (C.c_bool, [H, C.c_int]),
        "micropp3_get_cost": (C.c_int, [H, C.c_int]),
        "micropp3_has_converged": (C.c_bool, [H, C.c_int]),
        "micropp3_has_subiterated": (C.c_bool, [H, C.c_int]),
        "micropp3_get_non_linear_gps": (C.c_int, [H]),
        "micropp3_write_restart": (None, [H, C.c_int]),
        "micropp3_read_restart": (None, [H, C.c_int]),
        "micropp3_print_info": (None, [H]),
        "micropp3_output": (None, [H, C.c_int, C.c_char_p]),
        "micropp3_get_status": (C.c_int, [H, C.c_int]),
        "micropp3_get_newton": (None, [H, C.c_int, ip, ip, ip]),
        "micropp3_get_nelem": (C.c_int, [H]),
        "micropp3_get_nndim": (C.c_int, [H]),
        "micropp3_get_vars": (None, [H, C.c_int, C.c_int, dp]),
        "micropp3_get_u": (None, [H, C.c_int, C.c_int, dp]),
        "micropp3_get_elem_type": (None, [H, ip]),
        "micropp3_get_ctan_lin": (None, [H, dp]),
        "micropp3_last_homogenize_ms": (C.c_double, [H]),
        "micropp3_set_kernel_timing": (None, [H, C.c_int]),
        "micropp3_kernel_stats": (C.c_int, [H, C.c_char_p, C.POINTER(C.c_long), dp, dp]),
        "micropp3_total_cg_its": (C.c_long, [H]),
        "micropp3_get_mg_levels": (C.c_int, [H]),
        "micropp3_kernel_launches": (C.c_long, [H]),
        "micropp3_path_forward": (C.c_int, [H, C.c_int, dp, dp, C.c_int, dp]),
        "micropp3_path_vjp": (C.c_int, [H, dp, dp, dp]),
        "micropp3_path_newton": (None, [H, C.c_int, ip, ip, ip, dp]),
        "micropp3_set_cuda_graphs": (None, [H, C.c_int]),
        "micropp3_homogenize_many": (None, [C.POINTER(H), C.c_int]),
        "micropp3_ell_solve_cgpd": (C.c_int, [ip, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                             C.c_int, ip, C.c_void_p]),
        "micropp3_ell_solve_cgpd_noalloc": (C.c_int, [ip, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                                     C.c_double, C.c_int, ip, C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def declared_symbols():
    """Function names declared by the public headers include/*.h (the C-ABI contract)."""
    names = set()
    for h in ("material_base.h", "micropp_c.h", "micropp_gb300.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(\w+)\s*\(", text, flags=re.M):
            if m.group(1) not in ("defined",):
                names.add(m.group(1))
    return sorted(n for n in names if n.startswith(("micropp3_", "material_")))


def material(type_, E, nu, Ka=0.0, Sy=0.0, Xt=0.0):
    """A material record filled by the library's ``material_set`` (material_base.h)."""
    m = MaterialBase()
    load().material_set(C.byref(m), type_, E, nu, Ka, Sy, Xt)
    return m


def config(n, ngp=1, micro_type=MIC_HOMOGENEOUS, geo=(0.1, 0.1, 0.1, 0.1), mats=None, coupling=None,
           elem_type=None, **kw):
    """A ``micropp3_config`` with the reference defaults and the given overrides; ``n`` = elements per axis."""
    L = load()
    c = Config()
    L.micropp3_config_default(C.byref(c))
    c.ngp = ngp
    c.size[:] = [n + 1] * 3 if isinstance(n, int) else [x + 1 for x in n]
    c.micro_type = micro_type
    c.geo_params[:] = list(geo)
    mats = mats or [material(0, 1e7, 0.25)] * 3
    for i in range(3):
        c.materials[i] = mats[i]
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


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Micropp:
    """``micropp<3>`` through the C ABI.  Errors of the library raise RuntimeError."""

    def __init__(self, cfg):
        self.lib = load()
        self.cfg = cfg
        self.h = Handle()
        self.lib.micropp3_new_ext(C.byref(self.h), C.byref(cfg))
        if not self.h.ptr:
            raise RuntimeError("micropp3_new_ext failed: " + self.lib.micropp3_last_error().decode())
        self.ngp = cfg.ngp
        self.nelem = self.lib.micropp3_get_nelem(C.byref(self.h))
        self.nndim = self.lib.micropp3_get_nndim(C.byref(self.h))

    def _check(self, what):
        msg = self.lib.micropp3_last_error().decode()
        if msg:
            self.lib.micropp3_clear_error()
            raise RuntimeError(f"{what}: {msg}")

    def _call(self, name, *args):
        self.lib.micropp3_clear_error()
        r = getattr(self.lib, name)(C.byref(self.h), *args)
        self._check(name)
        return r

    def close(self):
        if self.h is not None and self.h.ptr:
            self.lib.micropp3_free(C.byref(self.h))
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # micropp<3> API (micropp.hpp:176-217)
    def set_strain(self, gp, eps):
        e = np.ascontiguousarray(eps, dtype=np.float64)
        self._call("micropp3_set_strain", gp, _dp(e))

    def get_stress(self, gp):
        s = np.zeros(6)
        self._call("micropp3_get_stress", gp, _dp(s))
        return s

    def get_ctan(self, gp):
        c = np.zeros(36)
        self._call("micropp3_get_ctan", gp, _dp(c))
        return c.reshape(6, 6)

    def homogenize(self):
        self._call("micropp3_homogenize")

    def homogenize_linear(self):
        self._call("micropp3_homogenize_linear")

    def update_vars(self):
        self._call("micropp3_update_vars")

    def is_non_linear(self, gp):
        return bool(self._call("micropp3_is_non_linear", gp))

    def get_non_linear_gps(self):
        return self._call("micropp3_get_non_linear_gps")

    def get_cost(self, gp):
        return self._call("micropp3_get_cost", gp)

    def has_converged(self, gp):
        return bool(self._call("micropp3_has_converged", gp))

    def has_subiterated(self, gp):
        return bool(self._call("micropp3_has_subiterated", gp))

    def write_restart(self, restart_id):
        self._call("micropp3_write_restart", restart_id)

    def read_restart(self, restart_id):
        self._call("micropp3_read_restart", restart_id)

    def print_info(self):
        self._call("micropp3_print_info")

    # extensions (micropp_gb300.h)
    def status(self, gp):
        return self._call("micropp3_get_status", gp)

    def newton(self, gp):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        self._call("micropp3_get_newton", gp, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, bool(c.value)

    def vars(self, gp, which=0):
        a = np.zeros(self.nelem * 8 * 7)
        self._call("micropp3_get_vars", gp, which, _dp(a))
        return a

    def u(self, gp, which=0):
        a = np.zeros(self.nndim)
        self._call("micropp3_get_u", gp, which, _dp(a))
        return a

    def elem_type(self):
        a = np.zeros(self.nelem, dtype=np.int32)
        self._call("micropp3_get_elem_type", a.ctypes.data_as(C.POINTER(C.c_int)))
        return a

    def ctan_lin(self):
        a = np.zeros(36)
        self._call("micropp3_get_ctan_lin", _dp(a))
        return a.reshape(6, 6)

    def last_homogenize_ms(self):
        return self._call("micropp3_last_homogenize_ms")

    def set_kernel_timing(self, on):
        self._call("micropp3_set_kernel_timing", 1 if on else 0)

    def kernel_stats(self, family):
        n, ms, by = C.c_long(), C.c_double(), C.c_double()
        ok = self._call("micropp3_kernel_stats", family.encode(), C.byref(n), C.byref(ms), C.byref(by))
        if not ok:
            raise KeyError(family)
        return n.value, ms.value, by.value

    def total_cg_its(self):
        return self._call("micropp3_total_cg_its")

    def mg_levels(self):
        return self._call("micropp3_get_mg_levels")

    def kernel_launches(self):
        return self._call("micropp3_kernel_launches")

    def path_forward(self, strains, params, checkpoint_every=5):
        """Average stress of every step of a load path from the undeformed state (micropp3_path_forward).
        strains: (nsteps, 6); params: (3, 5) = (E, nu, Xt, Sy, Ka) per phase.  Returns (sigma, status)."""
        e = np.ascontiguousarray(strains, dtype=np.float64).reshape(-1, 6)
        p = np.ascontiguousarray(params, dtype=np.float64).reshape(3, 5)
        sig = np.zeros_like(e)
        rc = self._call("micropp3_path_forward", e.shape[0], _dp(e), _dp(p), int(checkpoint_every), _dp(sig))
        return sig, rc

    def set_cuda_graphs(self, on):
        self._call("micropp3_set_cuda_graphs", 1 if on else 0)

    def path_newton(self, step):
        """(Newton its, CG its, status bits, |b|/|b0|) of a step of the last path."""
        a, b, c, d = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        self._call("micropp3_path_newton", step, C.byref(a), C.byref(b), C.byref(c), C.byref(d))
        return a.value, b.value, c.value, d.value

    def path_vjp(self, gsigma):
        """dL/dparams (3, 5) and dL/dstrains (nsteps, 6) for L = sum gsigma . sigma of the last path."""
        g = np.ascontiguousarray(gsigma, dtype=np.float64).reshape(-1, 6)
        gp = np.zeros((3, 5))
        gs = np.zeros_like(g)
        rc = self._call("micropp3_path_vjp", _dp(g), _dp(gp), _dp(gs))
        return gp, gs, rc
