"""Test harness: the oracle (CPU restatement of the reference) behind ctypes,
and the reference's error metric.

The oracle is the checker: tests build it from oracle/ with its Makefile and
compare the CUDA library against it on identical inputs.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from wrf_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle.so")

_OLIB = None


def oracle_lib():
    global _OLIB
    if _OLIB is not None:
        return _OLIB
    srcs = [os.path.join(ORACLE_DIR, f) for f in os.listdir(ORACLE_DIR) if f.endswith((".cpp", ".hpp", ".h"))]
    if not os.path.exists(ORACLE_LIB) or any(os.path.getmtime(s) > os.path.getmtime(ORACLE_LIB) for s in srcs):
        subprocess.run(["make", "-C", ORACLE_DIR], check=True, capture_output=True)
    L = C.CDLL(ORACLE_LIB)
    for pfx in ("oracle_f32_", "oracle_f64_"):
        getattr(L, pfx + "domain_create").argtypes = [C.POINTER(abi.WrfGpuDomainDesc), C.c_int, C.POINTER(C.c_void_p)]
        getattr(L, pfx + "domain_destroy").argtypes = [C.c_void_p]
        getattr(L, pfx + "field_size").argtypes = [C.c_void_p, C.c_int]
        getattr(L, pfx + "field_size").restype = C.c_long
        getattr(L, pfx + "set_field").argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_long]
        getattr(L, pfx + "set_field_f32").argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_long]
        getattr(L, pfx + "get_field").argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_long]
        getattr(L, pfx + "step").argtypes = [C.c_void_p, C.c_int]
        getattr(L, pfx + "run_routine").argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
        getattr(L, pfx + "fill_halo").argtypes = [C.c_void_p, C.c_int, C.c_char]
        getattr(L, pfx + "num_sound_steps").argtypes = [C.c_void_p]
        getattr(L, pfx + "cfl").argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        getattr(L, pfx + "tophat_feeder").argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p]
    _OLIB = L
    return L


class OracleDomain:
    """One domain of the CPU restatement (precision 'f32' or 'f64')."""

    def __init__(self, case, precision="f32", nthreads=1, load=True):
        self.L = oracle_lib()
        self.p = "oracle_%s_" % precision
        self.case = case
        h = C.c_void_p()
        rc = getattr(self.L, self.p + "domain_create")(C.byref(case.desc), nthreads, C.byref(h))
        assert rc == 0, "oracle domain_create failed: %d" % rc
        self.h = h
        if load:
            for fid, arr in case.field_items():
                self.set(fid, arr)

    def __del__(self):
        try:
            getattr(self.L, self.p + "domain_destroy")(self.h)
        except Exception:
            pass

    def set(self, fid, arr, as_f32=False):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        if as_f32:
            a = a.astype(np.float32).astype(np.float64)
        rc = getattr(self.L, self.p + "set_field")(self.h, fid, a.ctypes.data, a.size)
        assert rc == 0, "oracle set_field %d failed" % fid

    def get(self, fid):
        n = getattr(self.L, self.p + "field_size")(self.h, fid)
        a = np.empty(n, dtype=np.float64)
        rc = getattr(self.L, self.p + "get_field")(self.h, fid, a.ctypes.data, n)
        assert rc == 0
        return a

    def step(self, n=1):
        rc = getattr(self.L, self.p + "step")(self.h, n)
        assert rc == 0, "oracle step failed"

    def run(self, name, rk_step=1, iteration=1, species=0):
        rc = getattr(self.L, self.p + "run_routine")(self.h, abi.ROUTINES[name], rk_step, iteration, species)
        assert rc == 0, "oracle routine %s failed" % name

    def fill_halo(self, fid, var):
        rc = getattr(self.L, self.p + "fill_halo")(self.h, fid, var.encode())
        assert rc == 0

    def num_sound_steps(self):
        return getattr(self.L, self.p + "num_sound_steps")(self.h)

    def cfl(self):
        v = C.c_double()
        h = C.c_double()
        getattr(self.L, self.p + "cfl")(self.h, C.byref(v), C.byref(h))
        return v.value, h.value


def tophat_feeder(adv_opt, nloops=2000, every=200, precision="f32"):
    L = oracle_lib()
    out = np.zeros((nloops // every + 1, 91))
    rc = getattr(L, "oracle_%s_tophat_feeder" % precision)(adv_opt, nloops, every, out.ctypes.data)
    assert rc == 0
    return out


# ---------------------------------------------------------------------------
# regions and the reference's error metric
# ---------------------------------------------------------------------------
def shape3(case):
    h = abi.HALO
    return (case.jde + 2 * h, case.kde, case.ide + 2 * h)


def shape2(case):
    h = abi.HALO
    return (case.jde + 2 * h, case.ide + 2 * h)


def field_shape(case, fid):
    k = abi.field_kind(fid)
    if k == 3:
        return shape3(case)
    if k == 2:
        return shape2(case)
    return (case.kde,)


def interior(case, fid, arr, halo=0):
    """The points the model computes (plus `halo` halo points), as an array.

    3-D: i in [1-halo, ide+halo], j in [1-halo, jde+halo], all k.  The
    never-read column ime of non-x-staggered fields is excluded by using at
    most halo 3 on the high side.
    """
    h = abi.HALO
    a = np.asarray(arr).reshape(field_shape(case, fid))
    k = abi.field_kind(fid)
    if k == 1:
        return a
    lo = h - halo
    hi_i = h + case.ide + min(halo, 3)
    hi_j = h + case.jde + min(halo, 3)
    if k == 3:
        return a[lo:hi_j, :, lo:hi_i]
    return a[lo:hi_j, lo:hi_i]


def serr(a, b):
    """diffwrf's relative L2 error sqrt(sum (a-b)^2 / sum b^2)
    (external/io_netcdf/diffwrf.F90:491-497); 0 when both are zero."""
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    den = float(np.sum(b * b))
    num = float(np.sum((a - b) ** 2))
    if den == 0.0:
        return 0.0 if num == 0.0 else float("inf")
    return float(np.sqrt(num / den))


def max_abs(a, b):
    return float(np.max(np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64)))) if np.size(a) else 0.0


STATE_FIELDS = ["u_2", "v_2", "w_2", "t_2", "ph_2", "mu_2", "p", "al"]
