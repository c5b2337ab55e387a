"""wrfgpu_advect_scalar_pd_noalloc: the PD advection on device arrays with
the limiter-factor scratch in a static device array (no allocation).

Checked against the routine-level entry point wrfgpu_advect_scalar_pd (host
arrays, its own device domain) on the same developed state: two calls in a
row, the tendency accumulating from the same seeded start.  The two run the
same kernels on the same member layout, so the tendency must agree bit for
bit.  This file is collected last and passes alone as well."""
import ctypes as C

import numpy as np
import pytest

from wrf_gb300 import abi, cases

from _harness import interior
from test_fortran_abi import _fid, _scalars, _state

NAMES = ["qv", "qv_old", "ru_m", "rv_m", "ww_m", "c1h", "c2h", "muts", "mub", "mu_1", "msfux", "msfuy", "msfvx",
         "msfvy", "msftx", "msfty", "fnm", "fnp", "rdnw"]


def _dims(case):
    h = abi.HALO
    return [1, case.ide, 1, case.jde, 1, case.kde, 1 - h, case.ide + h, 1 - h, case.jde + h, 1, case.kde,
            1, case.ide, 1, case.jde, 1, case.kde]


class _Args:
    """ctypes argument builder that keeps every referenced object alive."""

    def __init__(self):
        self.keep = []
        self.args = []

    def ptr(self, p):
        self.args.append(C.c_void_p(p))

    def arr(self, a):
        self.keep.append(a)
        self.args.append(a.ctypes.data_as(C.c_void_p))

    def f32(self, v):
        x = C.c_float(v)
        self.keep.append(x)
        self.args.append(C.cast(C.pointer(x), C.c_void_p))

    def i32(self, v):
        x = C.c_int(v)
        self.keep.append(x)
        self.args.append(C.cast(C.pointer(x), C.c_void_p))

    def cfg(self, cf):
        p = C.pointer(cf)
        self.keep.append(p)
        self.args.append(C.cast(p, C.c_void_p))


def _routine_call(lib, case, host, tend, scal):
    a = _Args()
    a.arr(host["qv"]); a.arr(host["qv_old"]); a.arr(tend)
    z = np.zeros(1, np.float32)
    a.arr(z); a.arr(z)
    for nm in ("ru_m", "rv_m", "ww_m", "c1h", "c2h", "muts", "mub", "mu_1"):
        a.arr(host[nm])
    a.i32(1); a.cfg(case.desc.config); a.i32(0)
    for nm in ("msfux", "msfuy", "msfvx", "msfvy", "msftx", "msfty", "fnm", "fnp"):
        a.arr(host[nm])
    a.f32(scal["rdx"]); a.f32(scal["rdy"]); a.arr(host["rdnw"]); a.f32(scal["dtrk"])
    for d in _dims(case):
        a.i32(d)
    fn = lib.wrfgpu_advect_scalar_pd
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p] * len(a.args)
    return fn(*a.args)


def _noalloc_call(lib, case, dev, tend_dev, scal, dims=None):
    a = _Args()
    a.ptr(dev["qv"].data_ptr()); a.ptr(dev["qv_old"].data_ptr()); a.ptr(tend_dev.data_ptr())
    for nm in ("ru_m", "rv_m", "ww_m", "c1h", "c2h", "muts", "mub", "mu_1"):
        a.ptr(dev[nm].data_ptr())
    a.cfg(case.desc.config)
    for nm in ("msftx", "msfty", "fnm", "fnp"):
        a.ptr(dev[nm].data_ptr())
    a.f32(scal["rdx"]); a.f32(scal["rdy"]); a.ptr(dev["rdnw"].data_ptr()); a.f32(scal["dtrk"])
    for d in (dims or _dims(case)):
        a.i32(d)
    a.args.append(C.c_void_p(None))  # default stream
    fn = lib.wrfgpu_advect_scalar_pd_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p] * len(a.args)
    return fn(*a.args)


@pytest.mark.gpu
def test_noalloc_matches_routine_entry_two_calls(gpulib):
    torch = pytest.importorskip("torch")
    case = cases.small_case(nx=16, ny=12, kde=14, n_scalar=1, seed=21)
    od = _state(case)
    scal = _scalars(case, 3, 1)
    host = {nm: np.ascontiguousarray(od.get(_fid(nm)), dtype=np.float32) for nm in NAMES}
    n_tend = np.asarray(od.get(abi.FIELD_ID["advect_tend"])).size
    rng = np.random.Generator(np.random.PCG64(5))
    t0 = (1e-7 * rng.standard_normal(n_tend)).astype(np.float32)

    ref = t0.copy()
    ref_after = []
    for _ in range(2):
        assert _routine_call(gpulib, case, host, ref, scal) == 0
        ref_after.append(ref.copy())

    dev = {nm: torch.from_numpy(host[nm].copy()).cuda() for nm in NAMES}
    tend_dev = torch.from_numpy(t0.copy()).cuda()
    got_after = []
    for _ in range(2):
        assert _noalloc_call(gpulib, case, dev, tend_dev, scal) == 0
        torch.cuda.synchronize()
        got_after.append(tend_dev.cpu().numpy().copy())

    fid = abi.FIELD_ID["advect_tend"]
    for n in range(2):
        a = interior(case, fid, got_after[n])
        b = interior(case, fid, ref_after[n])
        assert float(np.max(np.abs(b))) > 0.0
        assert np.array_equal(a, b), "call %d: max|diff| %.3e" % (n + 1, float(np.max(np.abs(a - b))))
    # the second call accumulated onto the first
    assert not np.array_equal(got_after[0], got_after[1])


@pytest.mark.gpu
def test_noalloc_rejects_oversize(gpulib):
    """A memory shape above the static scratch's 8 Mi points returns
    WRFGPU_E_SIZE before anything is copied or launched."""
    torch = pytest.importorskip("torch")
    case = cases.small_case(nx=16, ny=12, kde=14, n_scalar=1, seed=21)
    scal = {"rdx": 1e-3, "rdy": 1e-3, "dtrk": 6.0}
    dummy = torch.zeros(16, device="cuda")
    dev = {nm: dummy for nm in NAMES}
    h = abi.HALO
    ide = jde = 401
    kde = 60
    dims = [1, ide, 1, jde, 1, kde, 1 - h, ide + h, 1 - h, jde + h, 1, kde, 1, ide, 1, jde, 1, kde]
    assert (ide + 2 * h) * kde * (jde + 2 * h) > 8 * 1024 * 1024
    assert _noalloc_call(gpulib, case, dev, dummy, scal, dims=dims) == abi.WRFGPU_E_SIZE


def test_noalloc_rejects_unsupported_options():
    """Options a device domain does not accept (open or specified lateral
    boundaries, other advection orders) return WRFGPU_E_ARG before any device
    work, so this runs without a GPU."""
    import os
    from wrf_gb300 import gpu as G
    if not os.path.exists(G.lib_path()):
        import __graft_entry__ as g
        g.build()
    lib = C.CDLL(G.lib_path())
    case = cases.small_case(nx=16, ny=12, kde=14, n_scalar=1, seed=21)
    scal = {"rdx": 1e-3, "rdy": 1e-3, "dtrk": 6.0}

    class _P:  # a stand-in device pointer; never dereferenced
        def data_ptr(self):
            return 256

    dev = {nm: _P() for nm in NAMES}
    for field, value in (("open_xs", 1), ("specified", 1), ("h_sca_adv_order", 3), ("periodic_x", 0)):
        cf = abi.WrfDynConfig.from_buffer_copy(case.desc.config)
        setattr(cf, field, value)
        case.desc.config, saved = cf, case.desc.config
        try:
            assert _noalloc_call(lib, case, dev, _P(), scal) == abi.WRFGPU_E_ARG, field
        finally:
            case.desc.config = saved
