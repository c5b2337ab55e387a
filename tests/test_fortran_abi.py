"""The routine-level C ABI (include/wrfgpu_fortran.h), called the way a
Fortran shim would call it (every argument by reference, arrays in the
reference's memory layout), against the oracle running the same routine on
the same state: outputs bit for bit."""
import ctypes as C

import numpy as np
import pytest

from wrf_gb300 import abi, cases
from wrf_gb300 import gpu as G

from _harness import OracleDomain, interior, max_abs

pytestmark = pytest.mark.gpu

F = lambda name: ("a", name)          # array argument bound to a state field
S = lambda name: ("s", name)          # float scalar by reference
I = lambda value: ("i", value)        # int scalar by reference
Z = lambda name: ("z", name)          # array passed as zeros (an accumulated tendency)
CFG = ("cfg",)
NUL = ("null",)                       # array the physics-off path ignores
DIMS = ("dims",)

ROUTINES = {
    "rk_step_prep": (
        [CFG, I("rk"), F("u_2"), F("v_2"), F("w_2"), F("t_2"), F("ph_2"), F("mu_2"), F("c1h"), F("c2h"),
         F("c1f"), F("c2f"), F("qv"), F("ru"), F("rv"), F("rw"), F("ww"), F("php"), F("alt"), F("muu"),
         F("muv"), F("mub"), F("mut"), F("phb"), F("pb"), F("p"), F("al"), F("alb"), F("cqu"), F("cqv"),
         F("cqw"), F("msfux"), F("msfuy"), F("msfvx"), F("msfvx_inv"), F("msfvy"), F("msftx"), F("msfty"),
         F("fnm"), F("fnp"), F("dnw"), S("rdx"), S("rdy"), I(1), DIMS],
        ["ru", "rv", "rw", "ww", "php", "alt", "muu", "muv", "mut", "cqu", "cqv", "cqw"]),
    "advance_uv": (
        [F("u_2"), F("ru_tend"), F("v_2"), F("rv_tend"), F("p"), F("pb"), F("ph_2"), F("php"), F("alt"),
         F("al"), F("mu_2"), F("muu"), F("cqu"), F("muv"), F("cqv"), F("mudf"), F("c1h"), F("c2h"), F("c1f"),
         F("c2f"), F("c3h"), F("c4h"), F("c3f"), F("c4f"), F("msfux"), F("msfuy"), F("msfvx"), F("msfvx_inv"),
         F("msfvy"), S("rdx"), S("rdy"), S("dts"), S("cf1"), S("cf2"), S("cf3"), F("fnm"), F("fnp"), S("emdiv"),
         F("rdnw"), CFG, I(0), I(1), I(0), DIMS],
        ["u_2", "v_2"]),
    "advance_mu_t": (
        [F("ww"), F("ww1"), F("u_2"), F("u_save"), F("v_2"), F("v_save"), F("mu_2"), F("mut"), F("muave"),
         F("muts"), F("muu"), F("muv"), F("mudf"), F("c1h"), F("c2h"), F("c1f"), F("c2f"), F("c3h"), F("c4h"),
         F("c3f"), F("c4f"), NUL, NUL, NUL, F("t_2"), F("t_save"), F("t_2save"), F("t_tend"), F("mu_tend"),
         S("rdx"), S("rdy"), S("dts"), S("epssm"), F("dnw"), F("fnm"), F("fnp"), F("rdnw"), F("msfux"),
         F("msfuy"), F("msfvx"), F("msfvx_inv"), F("msfvy"), F("msftx"), F("msfty"), I("it"), CFG, DIMS],
        ["ww", "ww1", "mu_2", "muave", "muts", "mudf", "t_2", "t_2save"]),
    "advance_w": (
        [F("w_2"), F("rw_tend"), F("ww"), F("w_save"), F("u_2"), F("v_2"), F("mu_2"), F("mut"), F("muave"),
         F("muts"), F("c1h"), F("c2h"), F("c1f"), F("c2f"), F("c3h"), F("c4h"), F("c3f"), F("c4f"),
         F("t_2save"), F("t_2"), F("t_save"), F("ph_2"), F("ph_save"), F("phb"), F("ph_tend"), F("ht"),
         F("c2a"), F("cqw"), F("alt"), F("alb"), F("a"), F("alpha"), F("gamma"), S("rdx"), S("rdy"), S("dts"),
         S("t0"), S("epssm"), F("dnw"), F("fnm"), F("fnp"), F("rdnw"), F("rdn"), S("cf1"), S("cf2"), S("cf3"),
         F("msftx"), F("msfty"), CFG, I(0), DIMS],
        ["w_2", "t_2save", "ph_2"]),
    "calc_p_rho": (
        [F("al"), F("p"), F("ph_2"), F("alt"), F("t_2"), F("t_save"), F("c2a"), F("pm1"), F("mu_2"), F("muts"),
         F("c1h"), F("c2h"), F("c1f"), F("c2f"), F("c3h"), F("c4h"), F("c3f"), F("c4f"), F("znu"), S("t0"),
         F("rdnw"), F("dnw"), S("smdiv"), I(1), I("it"), DIMS],
        ["al", "p", "pm1"]),
    "calc_coef_w": (
        [F("a"), F("alpha"), F("gamma"), F("mut"), F("c1h"), F("c2h"), F("c1f"), F("c2f"), F("c3h"), F("c4h"),
         F("c3f"), F("c4f"), F("cqw"), F("rdn"), F("rdnw"), F("c2a"), S("dts"), S("g"), S("epssm"), I(0), DIMS],
        ["a", "alpha", "gamma"]),
    "sumflux": (
        [F("u_2"), F("v_2"), F("ww"), F("u_save"), F("v_save"), F("ww1"), F("muu"), F("muv"), F("c1h"), F("c2h"),
         F("c1f"), F("c2f"), F("c3h"), F("c4h"), F("c3f"), F("c4f"), F("ru_m"), F("rv_m"), F("ww_m"),
         S("epssm"), F("msfux"), F("msfuy"), F("msfvx"), F("msfvx_inv"), F("msfvy"), I("it"), I("nsmall"), DIMS],
        ["ru_m", "rv_m", "ww_m"]),
    "small_step_prep": (
        [F("u_1"), F("u_2"), F("v_1"), F("v_2"), F("w_1"), F("w_2"), F("t_1"), F("t_2"), F("ph_1"), F("ph_2"),
         F("mub"), F("mu_1"), F("mu_2"), F("muu"), F("muus"), F("muv"), F("muvs"), F("mut"), F("muts"),
         F("mudf"), F("c1h"), F("c2h"), F("c1f"), F("c2f"), F("c3h"), F("c4h"), F("c3f"), F("c4f"),
         F("u_save"), F("v_save"), F("w_save"), F("t_save"), F("ph_save"), F("mu_save"), F("ww"), F("ww1"),
         F("c2a"), F("pb"), F("p"), F("alt"), F("msfux"), F("msfuy"), F("msfvx"), F("msfvx_inv"), F("msfvy"),
         F("msftx"), F("msfty"), S("rdx"), S("rdy"), I("rk"), DIMS],
        ["u_1", "u_2", "v_1", "v_2", "w_1", "w_2", "t_1", "t_2", "ph_1", "ph_2", "mu_1", "mu_2", "muus", "muvs",
         "muts", "mudf", "u_save", "v_save", "w_save", "t_save", "ph_save", "mu_save", "ww1", "c2a"]),
    "small_step_finish": (
        [F("u_2"), F("u_1"), F("v_2"), F("v_1"), F("w_2"), F("w_1"), F("t_2"), F("t_1"), F("ph_2"), F("ph_1"),
         F("ww"), F("ww1"), F("mu_2"), F("mu_1"), F("mut"), F("muts"), F("muu"), F("muus"), F("muv"), F("muvs"),
         F("c1h"), F("c2h"), F("c1f"), F("c2f"), F("c3h"), F("c4h"), F("c3f"), F("c4f"), F("u_save"),
         F("v_save"), F("w_save"), F("t_save"), F("ph_save"), F("mu_save"), F("msfux"), F("msfuy"), F("msfvx"),
         F("msfvy"), F("msftx"), F("msfty"), NUL, I("nsmall"), S("dts"), I("rk"), I(3), DIMS],
        ["u_2", "v_2", "w_2", "t_2", "ph_2", "ww", "mu_2", "muus", "muvs"]),
    "calc_p_rho_phi": (
        [F("qv"), I(1), I(2), F("al"), F("alb"), F("mu_2"), F("muts"), F("c1h"), F("c2h"), F("c3h"), F("c4h"),
         F("c3f"), F("c4f"), F("ph_2"), F("phb"), F("p"), F("pb"), F("t_2"), S("p0"), S("t0"), S("p_top"),
         F("znu"), F("znw"), F("dnw"), F("rdnw"), F("rdn"), I(1), I(1), DIMS],
        ["al", "p"]),
}

_ADV = lambda fld, tend, rdz: (
    [F(fld), F(fld), F(tend), F("ru"), F("rv"), F("ww"), F("c1h"), F("c2h"), F("mut"), I(1), CFG, F("msfux"),
     F("msfuy"), F("msfvx"), F("msfvy"), F("msftx"), F("msfty"), F("fnm"), F("fnp"), S("rdx"), S("rdy"), F(rdz),
     DIMS], [tend])
ROUTINES["advect_u"] = _ADV("u_2", "ru_tend", "rdnw")
ROUTINES["advect_v"] = _ADV("v_2", "rv_tend", "rdnw")
ROUTINES["advect_w"] = _ADV("w_2", "rw_tend", "rdn")

_MSF = [F("msfux"), F("msfuy"), F("msfvx"), F("msfvy"), F("msftx"), F("msfty")]
ROUTINES["advect_scalar"] = (
    [F("qv"), F("qv"), Z("advect_tend"), F("ru_m"), F("rv_m"), F("ww_m"), F("c1h"), F("c2h"), F("muts"), I(1), CFG]
    + _MSF + [F("fnm"), F("fnp"), S("rdx"), S("rdy"), F("rdnw"), DIMS], ["advect_tend"])
ROUTINES["advect_scalar_pd"] = (
    [F("qv"), F("qv_old"), Z("advect_tend"), NUL, NUL, F("ru_m"), F("rv_m"), F("ww_m"), F("c1h"), F("c2h"),
     F("muts"), F("mub"), F("mu_1"), I(1), CFG, I(0)] + _MSF
    + [F("fnm"), F("fnp"), S("rdx"), S("rdy"), F("rdnw"), S("dtrk"), DIMS], ["advect_tend"])
ROUTINES["rk_update_scalar"] = (
    [I(1), I(1), F("qv_old"), F("qv"), NUL, NUL, NUL, F("advect_tend"), NUL, NUL, F("msftx"), F("msfty"),
     F("c1h"), F("c2h"), F("mu_1"), F("mu_2"), F("mub"), I("rk"), S("dtrk"), I(0), CFG, I(0), DIMS],
    ["qv_old", "qv"])
STAGE = {"advect_scalar_pd": 3}

ORACLE_NAME = {"advect_u": "advect_u", "advect_v": "advect_v", "advect_w": "advect_w"}


# routines that read the full (uncoupled) state rather than the acoustic
# perturbation variables: called right after a large step
FULL_STATE = {"rk_step_prep", "calc_p_rho_phi"}


def _state(case, full=False):
    """A developed state: one large step, then (unless full) rk_step_prep of
    stage 2, the boundary fills the tendencies need, small_step_prep,
    calc_p_rho and calc_coef_w."""
    od = OracleDomain(case, "f32")
    od.step(1)
    if full:
        return od
    od.run("rk_step_prep", 2)
    for nm, var in [("ru", "u"), ("rv", "v"), ("rw", "w"), ("ww", "w"), ("php", "w"), ("alt", "t"), ("p", "p"),
                    ("muu", "u"), ("muv", "v"), ("mut", "t"), ("al", "p"), ("ph_2", "w")]:
        od.fill_halo(abi.FIELD_ID[nm], var)
    od.run("small_step_prep", 2)
    od.run("calc_p_rho", 2, 0)
    od.run("calc_coef_w", 2)
    return od


def _fid(name):
    if name == "qv":
        return abi.species_id(0)
    if name == "qv_old":
        return abi.species_id(0, True)
    return abi.FIELD_ID[name]


def _call(lib, routine, spec, od, case, scal):
    keep = []
    args = []
    arrays = {}
    h = abi.HALO
    dims = [1, case.ide, 1, case.jde, 1, case.kde, 1 - h, case.ide + h, 1 - h, case.jde + h, 1, case.kde,
            1, case.ide, 1, case.jde, 1, case.kde]
    cfg = C.pointer(case.desc.config)
    keep.append(cfg)
    for a in spec:
        if a[0] == "a":
            arr = np.ascontiguousarray(od.get(_fid(a[1])), dtype=np.float32)
            keep.append(arr)
            arrays[a[1]] = arr
            args.append(arr.ctypes.data_as(C.c_void_p))
        elif a[0] == "z":
            arr = np.zeros_like(np.asarray(od.get(_fid(a[1])), dtype=np.float32))
            keep.append(arr)
            arrays[a[1]] = arr
            args.append(arr.ctypes.data_as(C.c_void_p))
        elif a[0] == "null":
            z = np.zeros(1, np.float32)
            keep.append(z)
            args.append(z.ctypes.data_as(C.c_void_p))
        elif a[0] == "s":
            v = C.c_float(scal[a[1]])
            keep.append(v)
            args.append(C.cast(C.pointer(v), C.c_void_p))
        elif a[0] == "i":
            v = C.c_int(scal[a[1]] if isinstance(a[1], str) else a[1])
            keep.append(v)
            args.append(C.cast(C.pointer(v), C.c_void_p))
        elif a[0] == "cfg":
            args.append(C.cast(cfg, C.c_void_p))
        elif a[0] == "dims":
            for d in dims:
                v = C.c_int(d)
                keep.append(v)
                args.append(C.cast(C.pointer(v), C.c_void_p))
    fn = getattr(lib, "wrfgpu_" + routine)
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p] * len(args)
    rc = fn(*args)
    return rc, arrays


def _scalars(case, rk, it):
    s = case.desc.scalars
    f32 = np.float32
    nsound = max(2 * (int(f32(300.0) * f32(s.dt) / f32(min(s.dx, s.dy)) - f32(0.01)) + 1), 4)
    dt = f32(s.dt)
    dts = dt / f32(nsound) if rk > 1 else dt / f32(3.0)
    nsmall = 1 if rk == 1 else (nsound // 2 if rk == 2 else nsound)
    dtrk = dt / f32(3.0) if rk == 1 else (f32(0.5) * dt if rk == 2 else dt)
    return {"dtrk": dtrk,"rdx": f32(s.rdx), "rdy": f32(s.rdy), "dts": dts, "cf1": f32(s.cf1), "cf2": f32(s.cf2),
            "cf3": f32(s.cf3), "emdiv": f32(s.emdiv), "epssm": f32(s.epssm), "smdiv": f32(s.smdiv),
            "t0": f32(300.0), "g": f32(9.81), "p0": f32(100000.0), "p_top": f32(s.p_top),
            "rk": rk, "it": it, "nsmall": nsmall}


@pytest.fixture(scope="module")
def case():
    return cases.small_case(nx=16, ny=12, kde=14, n_scalar=1, seed=21)


@pytest.mark.parametrize("routine", sorted(ROUTINES))
def test_routine_abi_bitwise(gpulib, case, routine):
    spec, outs = ROUTINES[routine]
    rk, it = STAGE.get(routine, 2), 1
    if routine == "small_step_finish":
        it = 0
    od = _state(case, full=routine in FULL_STATE)
    scal = _scalars(case, rk, it)
    rc, arrays = _call(gpulib, routine, spec, od, case, scal)
    assert rc == 0, "%s returned %d" % (routine, rc)
    od.run(ORACLE_NAME.get(routine, routine), rk, it, 0)
    bad = []
    for nm in outs:
        fid = _fid(nm)
        a = interior(case, fid, arrays[nm], halo=0)
        b = interior(case, fid, od.get(fid), halo=0)
        d = max_abs(a, b)
        if d != 0.0:
            bad.append("%s: max|diff| %.3e" % (nm, d))
    assert not bad, "%s: %s" % (routine, "; ".join(bad))


def test_routine_abi_rejects_tiles(gpulib, case):
    """A tile smaller than the patch (num_tiles > 1) is refused, not run."""
    spec, _ = ROUTINES["calc_coef_w"]
    od = _state(case)
    scal = _scalars(case, 2, 1)
    h = abi.HALO
    fn = gpulib.wrfgpu_calc_coef_w
    fn.restype = C.c_int
    # same call with ite = ide - 4
    keep = []
    args = []
    for a in spec:
        if a[0] == "a":
            arr = np.ascontiguousarray(od.get(_fid(a[1])), dtype=np.float32)
            keep.append(arr)
            args.append(arr.ctypes.data_as(C.c_void_p))
        elif a[0] == "s":
            v = C.c_float(scal[a[1]]); keep.append(v); args.append(C.cast(C.pointer(v), C.c_void_p))
        elif a[0] == "i":
            v = C.c_int(a[1]); keep.append(v); args.append(C.cast(C.pointer(v), C.c_void_p))
        elif a[0] == "dims":
            for d in [1, case.ide, 1, case.jde, 1, case.kde, 1 - h, case.ide + h, 1 - h, case.jde + h, 1, case.kde,
                      1, case.ide - 4, 1, case.jde, 1, case.kde]:
                v = C.c_int(d); keep.append(v); args.append(C.cast(C.pointer(v), C.c_void_p))
    fn.argtypes = [C.c_void_p] * len(args)
    assert fn(*args) == abi.WRFGPU_E_ARG
