"""ctypes front end of the in-tree CUDA library (libwrfgpu.so).

This is plumbing for Python callers (tests, bench.py); the product is the C
ABI of include/wrfgpu.h.  There is no CPU fallback: if the library is not
built, or no CUDA device is present, every entry point raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi

_LIB = None
_HERE = os.path.dirname(os.path.abspath(__file__))


class WrfGpuError(RuntimeError):
    pass


def lib_path():
    return os.path.join(_HERE, "libwrfgpu.so")


def load():
    """Load libwrfgpu.so (raises if it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = lib_path()
    if not os.path.exists(p):
        raise WrfGpuError("libwrfgpu.so is not built; run `python -c \"import __graft_entry__ as g; g.build()\"`")
    L = C.CDLL(p)
    P = C.POINTER
    vp = C.c_void_p
    L.wrfgpu_ensemble_create.argtypes = [P(abi.WrfGpuDomainDesc), C.c_int, C.c_int, P(vp)]
    L.wrfgpu_ensemble_destroy.argtypes = [vp]
    L.wrfgpu_field_size.argtypes = [vp, C.c_int, C.c_int]
    L.wrfgpu_field_size.restype = C.c_longlong
    for nm in ("wrfgpu_set_field_f32", "wrfgpu_get_field_f32", "wrfgpu_set_field", "wrfgpu_get_field"):
        getattr(L, nm).argtypes = [vp, C.c_int, C.c_int, vp, C.c_longlong]
    L.wrfgpu_step.argtypes = [vp, C.c_int]
    L.wrfgpu_bind_host_state.argtypes = [vp, C.c_int, C.c_int, P(C.c_int), P(vp), P(vp), P(C.c_longlong)]
    L.wrfgpu_unbind_host_state.argtypes = [vp]
    L.wrfgpu_step_host.argtypes = [vp, C.c_int]
    L.wrfgpu_sync.argtypes = [vp]
    L.wrfgpu_time_steps.argtypes = [vp, C.c_int, P(C.c_float)]
    L.wrfgpu_run_routine.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
    L.wrfgpu_fill_halo.argtypes = [vp, C.c_int, C.c_char]
    L.wrfgpu_status.argtypes = [vp, C.c_int, P(C.c_uint), P(C.c_double), P(C.c_double)]
    L.wrfgpu_clear_status.argtypes = [vp]
    L.wrfgpu_set_cfl_limit.argtypes = [vp, C.c_double]
    L.wrfgpu_num_sound_steps.argtypes = [vp, C.c_int]
    L.wrfgpu_device_bytes.argtypes = [vp]
    L.wrfgpu_device_bytes.restype = C.c_longlong
    L.wrfgpu_kernel_launches_per_step.argtypes = [vp]
    L.wrfgpu_profile_phases.argtypes = [vp, C.c_int, P(C.c_double), P(C.c_int), C.c_int]
    L.wrfgpu_autotune.argtypes = [vp, C.c_int]
    L.wrfgpu_tuning.argtypes = [vp, P(C.c_int), P(C.c_int), P(C.c_float), C.c_int]
    L.wrfgpu_phase_name.argtypes = [C.c_int]
    L.wrfgpu_phase_name.restype = C.c_char_p
    L.wrfgpu_version.restype = C.c_char_p
    _LIB = L
    return L


def _check(rc, what):
    if rc != 0:
        raise WrfGpuError("%s failed: %d (%s)" % (what, rc, abi.ERRORS.get(rc, "?")))


FLAG_MIXED = 1
FLAG_NO_GRAPH = 2
FLAG_NO_CHECKS = 4


class Ensemble:
    """Device-resident members advanced together (one member = plain domain)."""

    def __init__(self, descs, flags=0):
        self.L = load()
        self.n = len(descs)
        arr = (abi.WrfGpuDomainDesc * self.n)(*descs)
        self._descs = arr
        h = C.c_void_p()
        _check(self.L.wrfgpu_ensemble_create(arr, self.n, flags, C.byref(h)), "wrfgpu_ensemble_create")
        self.h = h
        self.flags = flags

    @classmethod
    def from_cases(cls, cases, flags=0):
        e = cls([c.desc for c in cases], flags=flags)
        for m, c in enumerate(cases):
            e.load_case(m, c)
        return e

    def close(self):
        if self.h:
            self.L.wrfgpu_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def field_size(self, member, fid):
        return int(self.L.wrfgpu_field_size(self.h, member, fid))

    def set(self, member, fid, arr):
        a = np.ascontiguousarray(arr, dtype=np.float32)
        _check(self.L.wrfgpu_set_field_f32(self.h, member, fid, a.ctypes.data, a.size), "set_field %d" % fid)

    def get(self, member, fid, shape=None):
        n = self.field_size(member, fid)
        a = np.empty(n, dtype=np.float32)
        _check(self.L.wrfgpu_get_field_f32(self.h, member, fid, a.ctypes.data, n), "get_field %d" % fid)
        return a.reshape(shape) if shape is not None else a

    def load_case(self, member, case):
        for fid, arr in case.field_items():
            self.set(member, fid, arr)

    def step(self, n=1):
        _check(self.L.wrfgpu_step(self.h, n), "wrfgpu_step")

    def bind_host_state(self, member, fids, inputs, outputs=None):
        """Bind page-locked float32 numpy arrays (one per field id; outputs
        default to the inputs) to wrfgpu_step_host."""
        outputs = inputs if outputs is None else outputs
        n = len(fids)
        ids = (C.c_int * n)(*fids)
        vin = (C.c_void_p * n)(*[None if a is None else a.ctypes.data for a in inputs])
        vout = (C.c_void_p * n)(*[None if a is None else a.ctypes.data for a in outputs])
        cnt = (C.c_longlong * n)(*[(a if a is not None else b).size for a, b in zip(inputs, outputs)])
        self._host_bufs = (list(inputs), list(outputs))
        _check(self.L.wrfgpu_bind_host_state(self.h, member, n, ids, vin, vout, cnt), "bind_host_state")

    def step_host(self, n=1):
        _check(self.L.wrfgpu_step_host(self.h, n), "step_host")

    def unbind_host_state(self):
        _check(self.L.wrfgpu_unbind_host_state(self.h), "unbind_host_state")
        self._host_bufs = None

    def sync(self):
        _check(self.L.wrfgpu_sync(self.h), "wrfgpu_sync")

    def time_steps(self, n):
        ms = C.c_float()
        _check(self.L.wrfgpu_time_steps(self.h, n, C.byref(ms)), "wrfgpu_time_steps")
        return float(ms.value)

    def run_routine(self, name, rk_step=1, iteration=1, species=0):
        rid = abi.ROUTINES[name] if isinstance(name, str) else int(name)
        _check(self.L.wrfgpu_run_routine(self.h, rid, rk_step, iteration, species), "run_routine " + str(name))

    def fill_halo(self, fid, var):
        _check(self.L.wrfgpu_fill_halo(self.h, fid, var.encode() if isinstance(var, str) else var), "fill_halo")

    def status(self, member=0):
        bits = C.c_uint()
        v = C.c_double()
        hz = C.c_double()
        rc = self.L.wrfgpu_status(self.h, member, C.byref(bits), C.byref(v), C.byref(hz))
        return rc, int(bits.value), float(v.value), float(hz.value)

    def clear_status(self):
        _check(self.L.wrfgpu_clear_status(self.h), "clear_status")

    def set_cfl_limit(self, limit):
        _check(self.L.wrfgpu_set_cfl_limit(self.h, limit), "set_cfl_limit")

    def num_sound_steps(self, member=0):
        return int(self.L.wrfgpu_num_sound_steps(self.h, member))

    def device_bytes(self):
        return int(self.L.wrfgpu_device_bytes(self.h))

    def profile_phases(self, nsteps=1):
        """{phase name: (ms over nsteps, launches)} from events between kernel launches."""
        n = 32
        ms = (C.c_double * n)()
        cnt = (C.c_int * n)()
        got = self.L.wrfgpu_profile_phases(self.h, nsteps, ms, cnt, n)
        if got < 0:
            _check(got, "profile_phases")
        return {self.L.wrfgpu_phase_name(p).decode(): (ms[p], cnt[p]) for p in range(got)}

    TUNE_FAMILIES = ["scalar_pd_update", "scalar_adv_update", "advance_w", "advance_uv", "sumflux_calc_p_rho",
                     "step_prep", "small_step_finish", "small_step_prep", "cfl_check", "rk_tend_w", "rk_tend_u",
                     "rk_tend_v", "calc_p_rho_phi", "advance_mu_t"]

    def autotune(self, rounds=2):
        """Online autotuning (advances the model rounds x 4 steps); returns tuning()."""
        _check(self.L.wrfgpu_autotune(self.h, rounds), "wrfgpu_autotune")
        return self.tuning()

    def tuning(self):
        """{family: {"variant", "param", "ms": [per-variant ms per step]}}."""
        n = len(self.TUNE_FAMILIES)
        var = (C.c_int * n)()
        par = (C.c_int * n)()
        ms = (C.c_float * (4 * n))()
        got = self.L.wrfgpu_tuning(self.h, var, par, ms, n)
        if got < 0:
            _check(got, "wrfgpu_tuning")
        return {f: {"variant": var[q], "param": par[q], "ms": [round(ms[4 * q + v], 4) for v in range(4) if ms[4 * q + v] >= 0]}
                for q, f in enumerate(self.TUNE_FAMILIES)}

    def launches_per_step(self):
        return int(self.L.wrfgpu_kernel_launches_per_step(self.h))


def Domain(case, flags=0):
    """A plain single-domain state loaded from a Case."""
    return Ensemble.from_cases([case], flags=flags)
