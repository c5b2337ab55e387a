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
    [I(1), I(1), F("qv_old"), F("qv"), Z("h_diabatic"), NUL, NUL, F("advect_tend"), NUL, NUL, F("msftx"), F("msfty"),
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


def _calc_mu_uv_1(case, od):
    """muus, muvs from muts as solve_em's calc_mu_uv_1 forms them before
    small_step_finish (module_big_step_utilities_em.F:184-326: the
    boundary point one-sided where the direction is not periodic), set into
    the oracle state so that the entry point receives them."""
    h = abi.HALO
    cf = case.desc.config
    ni, nj = case.ide + 2 * h, case.jde + 2 * h
    mu = np.asarray(od.get(abi.FIELD_ID["muts"]), dtype=np.float32).reshape(nj, ni)
    half = np.float32(0.5)
    muus = np.asarray(od.get(abi.FIELD_ID["muus"]), dtype=np.float32).reshape(nj, ni).copy()
    muvs = np.asarray(od.get(abi.FIELD_ID["muvs"]), dtype=np.float32).reshape(nj, ni).copy()
    for jj in range(1, case.jde):
        for ii in range(1, case.ide + 1):
            a, b = ii, ii - 1
            if ii == 1 and not cf.periodic_x:
                b = ii
            if ii == case.ide and not cf.periodic_x:
                a = ii - 1
            muus[jj + h - 1, ii + h - 1] = half * (mu[jj + h - 1, a + h - 1] + mu[jj + h - 1, b + h - 1])
    for jj in range(1, case.jde + 1):
        for ii in range(1, case.ide):
            a, b = jj, jj - 1
            if jj == 1 and not cf.periodic_y:
                b = jj
            if jj == case.jde and not cf.periodic_y:
                a = jj - 1
            muvs[jj + h - 1, ii + h - 1] = half * (mu[a + h - 1, ii + h - 1] + mu[b + h - 1, ii + h - 1])
    od.set(abi.FIELD_ID["muus"], muus.astype(np.float64))
    od.set(abi.FIELD_ID["muvs"], muvs.astype(np.float64))


def _fid(name):
    if name == "qv":
        return abi.species_id(0)
    if name == "qv_old":
        return abi.species_id(0, True)
    return abi.FIELD_ID[name]


def _widen(case, fid, arr, extra, fill=7777.0):
    """A memory-layout array with `extra` more halo points on each side in i
    and j (filled with `fill`), and the index slices of the standard window."""
    h = abi.HALO
    k = abi.field_kind(fid)
    if k == 1 or extra == 0:
        return np.ascontiguousarray(arr, dtype=np.float32), None
    ni, nj = case.ide + 2 * h, case.jde + 2 * h
    if k == 3:
        a = np.asarray(arr, dtype=np.float32).reshape(nj, case.kde, ni)
        w = np.full((nj + 2 * extra, case.kde, ni + 2 * extra), fill, np.float32)
        win = (slice(extra, extra + nj), slice(None), slice(extra, extra + ni))
    else:
        a = np.asarray(arr, dtype=np.float32).reshape(nj, ni)
        w = np.full((nj + 2 * extra, ni + 2 * extra), fill, np.float32)
        win = (slice(extra, extra + nj), slice(extra, extra + ni))
    w[win] = a
    return np.ascontiguousarray(w.ravel()), (w.shape, win)


def _call(lib, routine, spec, od, case, scal, extra=0, tile=None, arrays=None):
    """Call wrfgpu_<routine> as Fortran would; `extra`: memory halo beyond 4,
    `tile`: (its, ite, jts, jte); `arrays`: the (widened) arrays of a
    previous call to pass again (a tile loop over shared arrays)."""
    keep = []
    args = []
    arrays = {} if arrays is None else arrays
    h = abi.HALO + extra
    its, ite, jts, jte = tile if tile else (1, case.ide, 1, case.jde)
    dims = [1, case.ide, 1, case.jde, 1, case.kde, 1 - h, case.ide + h, 1 - h, case.jde + h, 1, case.kde,
            its, ite, jts, jte, 1, case.kde]
    cfg = C.pointer(case.desc.config)
    keep.append(cfg)
    for a in spec:
        if a[0] in ("a", "z"):
            if a[1] not in arrays:
                src = od.get(_fid(a[1])) if a[0] == "a" else np.zeros_like(np.asarray(od.get(_fid(a[1]))))
                arrays[a[1]] = _widen(case, _fid(a[1]), src, extra)
            arr = arrays[a[1]][0]
            keep.append(arr)
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


def _window(arrays, nm):
    """The standard (halo 4) view of a possibly widened array."""
    arr, shp = arrays[nm]
    if shp is None:
        return arr
    shape, win = shp
    return np.ascontiguousarray(arr.reshape(shape)[win]).ravel()


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
    if routine == "small_step_finish":
        _calc_mu_uv_1(case, od)
    scal = _scalars(case, rk, it)
    rc, arrays = _call(gpulib, routine, spec, od, case, scal)
    assert rc == 0, "%s returned %d" % (routine, rc)
    od.run(ORACLE_NAME.get(routine, routine), rk, it, 0)
    bad = []
    for nm in outs:
        fid = _fid(nm)
        a = interior(case, fid, _window(arrays, nm), halo=0)
        b = interior(case, fid, od.get(fid), halo=0)
        d = max_abs(a, b)
        if d != 0.0:
            bad.append("%s: max|diff| %.3e" % (nm, d))
    assert not bad, "%s: %s" % (routine, "; ".join(bad))


@pytest.fixture(scope="module")
def case_open():
    return cases.open_boundaries(cases.small_case(nx=24, ny=20, kde=14, n_scalar=1, seed=22))


@pytest.mark.parametrize("routine", sorted(ROUTINES))
def test_routine_abi_open_boundaries_bitwise(gpulib, case_open, routine):
    """Every routine-level entry point with open lateral boundaries on all
    four sides (the em_quarter_ss namelist): the degraded fluxes, radiation
    terms and boundary limits of the reference routines, bit for bit."""
    test_routine_abi_bitwise(gpulib, case_open, routine)


@pytest.mark.parametrize("routine", ["advance_uv", "calc_p_rho", "rk_step_prep", "advance_w", "small_step_finish"])
def test_routine_abi_tiles_and_wide_halo(gpulib, case, routine):
    """The routine-level entry points take the memory dims of a wider halo
    (ims = ids-6: the window ids-4 .. ide+4 is used and the extra halo is
    left alone) and any tile of the patch (num_tiles > 1: only the tile's
    points of the outputs come back, as the reference's tile loops write
    them).  A loop over 2 x 3 tiles on shared arrays, with the wider halo,
    gives the whole-patch call's outputs bit for bit on every point of the
    patch; a tile outside the patch is refused."""
    spec, outs = ROUTINES[routine]
    rk, it = STAGE.get(routine, 2), 1
    if routine == "small_step_finish":
        it = 0
    od = _state(case, full=routine in FULL_STATE)
    if routine == "small_step_finish":
        _calc_mu_uv_1(case, od)
    scal = _scalars(case, rk, it)
    rc, ref = _call(gpulib, routine, spec, od, case, scal)
    assert rc == 0
    ib = [1, case.ide // 2, case.ide]
    jb = [1, case.jde // 3, 2 * case.jde // 3, case.jde]
    arrays = None
    for a in range(2):
        for b in range(3):
            tile = (ib[a] + (a > 0), ib[a + 1], jb[b] + (b > 0), jb[b + 1])
            rc, arrays = _call(gpulib, routine, spec, od, case, scal, extra=2, tile=tile, arrays=arrays)
            assert rc == 0, tile
    h = abi.HALO

    def patch(nm, arrs):  # the union of the tiles: i in 1..ide, j in 1..jde, every level
        a = _window(arrs, nm)
        if abi.field_kind(_fid(nm)) == 3:
            return a.reshape(case.jde + 2 * h, case.kde, -1)[h:h + case.jde, :, h:h + case.ide]
        return a.reshape(case.jde + 2 * h, -1)[h:h + case.jde, h:h + case.ide]

    bad = []
    for nm in outs:
        if not np.array_equal(patch(nm, arrays), patch(nm, ref)):
            bad.append(nm)
        arr, shp = arrays[nm]
        if shp is not None:
            shape, win = shp
            outer = np.ones(shape, bool)
            outer[win] = False
            if not np.all(arr.reshape(shape)[outer] == 7777.0):
                bad.append(nm + " (extra halo)")
    assert not bad, bad
    rc, _ = _call(gpulib, routine, spec, od, case, scal, tile=(1, case.ide + 1, 1, case.jde))
    assert rc == abi.WRFGPU_E_ARG


# --------------------------------------------------------------------------
# Scalar entry points over several species: 4-D (ims:ime,kms:kme,jms:jme,
# scs:sce) arrays, sc_tend carried through, rk_scalar_tend's dispatch.
# --------------------------------------------------------------------------
class _Argv:
    """ctypes arguments by reference, kept alive for the call."""

    def __init__(self):
        self.keep, self.args = [], []

    def arr(self, a):
        a = np.ascontiguousarray(a, dtype=np.float32)
        self.keep.append(a)
        self.args.append(a.ctypes.data_as(C.c_void_p))
        return a

    def ptr(self, a, offset_elems=0):
        self.keep.append(a)
        self.args.append(C.c_void_p(a.ctypes.data + 4 * offset_elems))

    def null(self):
        self.args.append(C.c_void_p(None))

    def f32(self, v):
        x = C.c_float(v); self.keep.append(x); self.args.append(C.cast(C.pointer(x), C.c_void_p))

    def i32(self, v):
        x = C.c_int(v); self.keep.append(x); self.args.append(C.cast(C.pointer(x), C.c_void_p))

    def cfg(self, cf):
        p = C.pointer(cf); self.keep.append(p); self.args.append(C.cast(p, C.c_void_p))

    def dims(self, case):
        h = abi.HALO
        for d in [1, case.ide, 1, case.jde, 1, case.kde, 1 - h, case.ide + h, 1 - h, case.jde + h, 1, case.kde,
                  1, case.ide, 1, case.jde, 1, case.kde]:
            self.i32(d)

    def call(self, lib, name):
        fn = getattr(lib, name)
        fn.restype = C.c_int
        fn.argtypes = [C.c_void_p] * len(self.args)
        return fn(*self.args)


def _stack(od, ids):
    return np.ascontiguousarray(np.concatenate([np.asarray(od.get(f), dtype=np.float32) for f in ids]))


@pytest.fixture(scope="module")
def case3():
    """Three species (qv + 2 PD scalars), sixth-order diffusion on."""
    c = cases.small_case(nx=16, ny=12, kde=14, n_scalar=2, seed=27)
    c.desc.config.diff_6th_opt = 2
    c.desc.config.diff_6th_factor = 0.12
    c.desc.config.diff_6th_thresh = 0.10
    return c


def _f(od, nm):
    return np.asarray(od.get(_fid(nm)), dtype=np.float32)


def test_rk_update_scalar_pd_abi_bitwise(gpulib, case3):
    """wrfgpu_rk_update_scalar_pd (module_em.F:1803) over species 1..3 with a
    non-zero sc_tend and mu_new != mu_old: each old species bit for bit with
    the oracle's rk_update_scalar_pd; sc_tend zeroed over the update region
    and untouched elsewhere."""
    case = case3
    od = _state(case)
    nsp = 3
    n3 = od.get(abi.species_id(0)).size
    rng = np.random.Generator(np.random.PCG64(9))
    sct = (1e-9 * rng.standard_normal(nsp * n3)).astype(np.float32)
    mu_new = _f(od, "mu_2") + np.float32(3.0)
    scal = _scalars(case, 3, 1)
    a = _Argv()
    a.i32(1); a.i32(nsp)
    q = a.arr(_stack(od, [abi.species_id(s, True) for s in range(nsp)]))
    sct_gpu = a.arr(sct.copy())
    a.arr(_f(od, "c1h")); a.arr(_f(od, "c2h")); a.arr(_f(od, "mu_1")); a.arr(mu_new); a.arr(_f(od, "mub"))
    a.i32(3); a.f32(scal["dtrk"]); a.i32(0); a.cfg(case.desc.config); a.dims(case)
    assert a.call(gpulib, "wrfgpu_rk_update_scalar_pd") == 0
    od.set(abi.FIELD_ID["mu_2"], mu_new)
    bad = []
    for s in range(nsp):
        od.set(abi.FIELD_ID["h_diabatic"], sct[s * n3:(s + 1) * n3])
        od.run("rk_update_scalar_pd_args", 3, 0, s)
        fid = abi.species_id(s, True)
        d = max_abs(interior(case, fid, q[s * n3:(s + 1) * n3], halo=0), interior(case, fid, od.get(fid), halo=0))
        if d != 0.0:
            bad.append("species %d: max|diff| %.3e" % (s, d))
    assert not bad, bad
    # sc_tend: zero over the update region i < ide, k < kde, j < jde, else untouched
    h = abi.HALO
    shape = (case.jde + 2 * h, case.kde, -1)
    for s in range(nsp):
        got = sct_gpu[s * n3:(s + 1) * n3].reshape(shape)
        ref = sct[s * n3:(s + 1) * n3].reshape(shape).copy()
        ref[h:h + case.jde - 1, 0:case.kde - 1, h:h + case.ide - 1] = 0.0
        assert np.array_equal(got, ref), s


@pytest.mark.parametrize("rk", [1, 2])
def test_rk_update_scalar_abi_offset_species_bitwise(gpulib, case3, rk):
    """wrfgpu_rk_update_scalar over species 2..3 only (arrays dimensioned
    scs:sce, the way solve_em passes moist(ims,kms,jms,im)), with sc_tend:
    bit for bit with the oracle's rk_update_scalar."""
    case = case3
    od = _state(case)
    n3 = od.get(abi.species_id(0)).size
    rng = np.random.Generator(np.random.PCG64(10 + rk))
    sct = (1e-9 * rng.standard_normal(2 * n3)).astype(np.float32)
    adv = (1e-7 * rng.standard_normal(n3)).astype(np.float32)
    scal = _scalars(case, rk, 1)
    a = _Argv()
    a.i32(2); a.i32(3)
    q1 = a.arr(_stack(od, [abi.species_id(s, True) for s in (1, 2)]))
    q2 = a.arr(_stack(od, [abi.species_id(s) for s in (1, 2)]))
    a.arr(sct); a.null(); a.null(); a.arr(adv); a.null(); a.null()
    for nm in ("msftx", "msfty", "c1h", "c2h", "mu_1", "mu_2", "mub"):
        a.arr(_f(od, nm))
    a.i32(rk); a.f32(scal["dtrk"]); a.i32(0); a.cfg(case.desc.config); a.i32(0); a.dims(case)
    assert a.call(gpulib, "wrfgpu_rk_update_scalar") == 0
    od.set(abi.FIELD_ID["advect_tend"], adv)
    bad = []
    for n, s in enumerate((1, 2)):
        od.set(abi.FIELD_ID["h_diabatic"], sct[n * n3:(n + 1) * n3])
        od.run("rk_update_scalar_args", rk, 0, s)
        for fid, got in ((abi.species_id(s, True), q1), (abi.species_id(s), q2)):
            d = max_abs(interior(case, fid, got[n * n3:(n + 1) * n3], halo=0), interior(case, fid, od.get(fid), halo=0))
            if d != 0.0:
                bad.append("species %d field %d: max|diff| %.3e" % (s, fid, d))
    assert not bad, bad


@pytest.mark.parametrize("rk", [1, 3])
def test_rk_scalar_tend_abi_bitwise(gpulib, case3, rk):
    """wrfgpu_rk_scalar_tend (module_em.F:1096) over species 1..3: advect_tend
    zeroed over the tile and left holding the last species' tendency
    (advect_scalar at stage 1, advect_scalar_pd at the last stage with
    adv_opt = 1), and at stage 1 every species' sixth-order diffusion added
    to its scalar_tends; bit for bit with the oracle's routines."""
    case = case3
    od = _state(case)
    nsp = 3
    n3 = od.get(abi.species_id(0)).size
    rng = np.random.Generator(np.random.PCG64(20 + rk))
    tends0 = (1e-9 * rng.standard_normal(nsp * n3)).astype(np.float32)
    scal = _scalars(case, rk, 1)
    a = _Argv()
    a.i32(1); a.i32(nsp); a.cfg(case.desc.config); a.i32(0); a.i32(rk); a.f32(scal["dtrk"])
    for nm in ("ru_m", "rv_m", "ww_m", "ww_m"):
        a.arr(_f(od, nm))
    a.null(); a.null(); a.null()                        # wwI, u_old, v_old
    for nm in ("muts", "mub", "mu_1", "c1h", "c2h", "c1f", "c2f", "alt"):
        a.arr(_f(od, nm))
    a.arr(_stack(od, [abi.species_id(s, True) for s in range(nsp)]))
    a.arr(_stack(od, [abi.species_id(s) for s in range(nsp)]))
    tends = a.arr(tends0.copy())
    adv = a.arr((1e3 * np.ones(n3)).astype(np.float32))  # garbage the call must zero
    a.null(); a.null(); a.null(); a.null(); a.i32(1)     # h_, z_tendency, RQVFTEN, base, moist_step
    for nm in ("fnm", "fnp", "msfux", "msfuy", "msfvx", "msfvx_inv", "msfvy", "msftx", "msfty"):
        a.arr(_f(od, nm))
    a.f32(scal["rdx"]); a.f32(scal["rdy"]); a.arr(_f(od, "rdn")); a.arr(_f(od, "rdnw"))
    a.f32(0.0); a.f32(0.0); a.null()                    # khdif, kvdif, xkmhd
    a.i32(2); a.f32(0.12); a.i32(1); a.arr(_f(od, "phb")); a.arr(_f(od, "ph_2")); a.i32(0); a.i32(0)
    a.dims(case)
    assert a.call(gpulib, "wrfgpu_rk_scalar_tend") == 0
    bad = []
    # advect_tend: the last species' advection
    od.run("advect_scalar_pd" if rk == 3 else "advect_scalar", rk, 0, nsp - 1)
    fid = abi.FIELD_ID["advect_tend"]
    d = max_abs(interior(case, fid, adv, halo=0), interior(case, fid, od.get(fid), halo=0))
    if d != 0.0:
        bad.append("advect_tend: max|diff| %.3e" % d)
    for s in range(nsp):
        got = tends[s * n3:(s + 1) * n3]
        if rk == 1:
            od.set(abi.FIELD_ID["h_diabatic"], tends0[s * n3:(s + 1) * n3])
            od.run("sixth_diff_species", 1, 0, s)
            ref = od.get(abi.FIELD_ID["h_diabatic"])
        else:
            ref = tends0[s * n3:(s + 1) * n3]
        d = max_abs(interior(case, fid, got, halo=0), interior(case, fid, ref, halo=0))
        if d != 0.0:
            bad.append("scalar_tends %d: max|diff| %.3e" % (s, d))
    assert not bad, bad
    if rk == 1:  # the diffusion was active
        assert max_abs(interior(case, fid, tends[:n3], halo=0), interior(case, fid, tends0[:n3], halo=0)) > 0.0



@pytest.fixture(scope="module")
def case3x():
    """Three species (qv + 2 PD scalars), explicit diffusion (diff_opt = 1,
    km_opt = 1) and sixth-order diffusion on."""
    c = cases.small_case(nx=16, ny=12, kde=14, n_scalar=2, seed=29)
    cf = c.desc.config
    cf.diff_6th_opt = 2
    cf.diff_6th_factor = 0.12
    cf.diff_6th_thresh = 0.10
    cf.diff_opt = 1
    cf.km_opt = 1
    cf.khdif = 800.0
    cf.kvdif = 30.0
    return c


def test_rk_scalar_tend_abi_explicit_diffusion_bitwise(gpulib, case3x):
    """wrfgpu_rk_scalar_tend at stage 1 with diff_opt = 1 over moist species
    P_QV..P_QV+2 (module_em.F:1378-1435): every species' horizontal and
    vertical explicit diffusion (qv's against qv_base) and then its
    sixth-order diffusion added to scalar_tends, bit for bit with the
    oracle's; a coefficient array that is not khdif / prandtl is refused."""
    case = case3x
    od = _state(case)
    nsp = 3
    n3 = od.get(abi.species_id(0)).size
    cf = case.desc.config
    rng = np.random.Generator(np.random.PCG64(41))
    tends0 = (1e-9 * rng.standard_normal(nsp * n3)).astype(np.float32)
    scal = _scalars(case, 1, 1)
    xk = np.full(n3, np.float32(cf.khdif) / (np.float32(1.0) / np.float32(3.0)), dtype=np.float32)

    def call(xkmhd):
        a = _Argv()
        a.i32(2); a.i32(1 + nsp); a.cfg(cf); a.i32(0); a.i32(1); a.f32(scal["dtrk"])
        for nm in ("ru_m", "rv_m", "ww_m", "ww_m"):
            a.arr(_f(od, nm))
        a.null(); a.null(); a.null()                        # wwI, u_old, v_old
        for nm in ("muts", "mub", "mu_1", "c1h", "c2h", "c1f", "c2f", "alt"):
            a.arr(_f(od, nm))
        a.arr(_stack(od, [abi.species_id(s, True) for s in range(nsp)]))
        a.arr(_stack(od, [abi.species_id(s) for s in range(nsp)]))
        tends = a.arr(tends0.copy())
        a.arr(np.zeros(n3, np.float32))
        a.null(); a.null(); a.null()                        # h_, z_tendency, RQVFTEN
        a.arr(_f(od, "qv_base")); a.i32(1)                  # base, moist_step
        for nm in ("fnm", "fnp", "msfux", "msfuy", "msfvx", "msfvx_inv", "msfvy", "msftx", "msfty"):
            a.arr(_f(od, nm))
        a.f32(scal["rdx"]); a.f32(scal["rdy"]); a.arr(_f(od, "rdn")); a.arr(_f(od, "rdnw"))
        a.f32(cf.khdif); a.f32(cf.kvdif); a.arr(xkmhd)
        a.i32(2); a.f32(0.12); a.i32(1); a.arr(_f(od, "phb")); a.arr(_f(od, "ph_2")); a.i32(0); a.i32(0)
        a.dims(case)
        return a.call(gpulib, "wrfgpu_rk_scalar_tend"), tends

    rc, tends = call(xk)
    assert rc == 0
    fid = abi.FIELD_ID["h_diabatic"]
    bad = []
    for s in range(nsp):
        od.set(fid, tends0[s * n3:(s + 1) * n3])
        od.run("sixth_diff_species", 1, 1 if s == 0 else 0, s)
        got = tends[s * n3:(s + 1) * n3]
        d = max_abs(interior(case, fid, got, halo=0), interior(case, fid, od.get(fid), halo=0))
        if d != 0.0:
            bad.append("scalar_tends %d: max|diff| %.3e" % (s, d))
    assert not bad, bad
    rc, _ = call(xk * np.float32(2.0))
    assert rc == abi.WRFGPU_E_ARG


@pytest.fixture(scope="module")
def case_fwd():
    """Explicit and sixth-order diffusion and the Rayleigh damping all on:
    rk_tendency's stage-1 forward step adds three terms to each *_tendf."""
    c = cases.small_case(nx=16, ny=12, kde=14, n_scalar=1, seed=31)
    cf = c.desc.config
    cf.diff_opt = 1
    cf.km_opt = 1
    cf.khdif = 900.0
    cf.kvdif = 35.0
    cf.diff_6th_opt = 2
    cf.diff_6th_factor = 0.12
    cf.damp_opt = 2
    cf.dampcoef = 0.01
    cf.zdamp = 5000.0
    return c


def test_rk_tendency_abi_forward_step_bitwise(gpulib, case_fwd):
    """wrfgpu_rk_tendency (module_em.F:190) at stage 1 with diff_opt = 1,
    diff_6th_opt = 2 and damp_opt = 2: the large-step tendencies bit for bit
    the oracle's rk_tendency, and ru_tendf, rv_tendf, rw_tendf, t_tendf,
    which arrive holding (physics) tendencies, gain the forward step's
    explicit diffusion, sixth-order diffusion and Rayleigh damping
    (:801-944) bit for bit as the oracle adds them; a coefficient array
    that is not khdif is refused."""
    case = case_fwd
    od = _state(case)
    cf = case.desc.config
    s = case.desc.scalars
    n3 = od.get(abi.FIELD_ID["u_2"]).size
    rng = np.random.Generator(np.random.PCG64(43))
    tf_names = ["ru_tendf", "rv_tendf", "rw_tendf", "t_tendf"]
    tf0 = {nm: (1e-3 * rng.standard_normal(n3)).astype(np.float32) for nm in tf_names}
    xk = np.full(n3, np.float32(cf.khdif), dtype=np.float32)

    def call(xkmhd):
        a = _Argv()
        a.cfg(cf); a.i32(1)
        outs = {}
        for nm in ("ru_tend", "rv_tend", "rw_tend", "ph_tend", "t_tend"):
            outs[nm] = a.arr(np.zeros(n3, np.float32))
        for nm in ("ru_tendf", "rv_tendf", "rw_tendf"):
            outs[nm] = a.arr(tf0[nm].copy())
        a.arr(np.zeros(n3, np.float32))                    # ph_tendf
        outs["t_tendf"] = a.arr(tf0["t_tendf"].copy())
        outs["mu_tend"] = a.arr(np.zeros(od.get(abi.FIELD_ID["mu_2"]).size, np.float32))
        for nm in ("u_save", "v_save", "w_save", "ph_save", "t_save"):
            outs[nm] = a.arr(np.zeros(n3, np.float32))
        outs["mu_save"] = a.arr(np.zeros(od.get(abi.FIELD_ID["mu_2"]).size, np.float32))
        a.null()                                            # RTHFTEN
        for nm in ("ru", "rv", "rw", "ww", "ww"):
            a.arr(_f(od, nm))
        a.arr(_f(od, "ww"))                                 # wwI
        for nm in ("u_2", "v_2", "w_2", "t_2", "ph_2"):
            a.arr(_f(od, nm))
        for _ in range(5):
            a.null()                                        # u_old .. ph_old
        a.null()                                            # h_diabatic
        for nm in ("phb", "t_init"):
            a.arr(_f(od, nm))
        a.null()                                            # mu_old
        for nm in ("mu_2", "mut", "muu", "muv", "mub", "c1h", "c2h", "c1f", "c2f", "al", "ht", "alt", "p", "pb",
                   "php", "cqu", "cqv"):
            a.arr(_f(od, nm))
        outs["cqw"] = a.arr(_f(od, "cqw"))
        for nm in ("u_base", "v_base", "t_base", "qv_base", "z_base", "msfux", "msfuy", "msfvx", "msfvx_inv",
                   "msfvy", "msftx", "msfty"):
            a.arr(_f(od, nm))
        a.null()                                            # clat
        for nm in ("f", "e", "sina", "cosa", "fnm", "fnp", "rdn", "rdnw"):
            a.arr(_f(od, nm))
        a.f32(s.dt); a.f32(np.float32(s.rdx)); a.f32(np.float32(s.rdy))
        a.f32(cf.khdif); a.f32(cf.kvdif); a.arr(xkmhd); a.null()   # khdif, kvdif, xkmhd, xkhh
        a.i32(cf.diff_6th_opt); a.f32(cf.diff_6th_factor); a.i32(1)
        a.f32(cf.dampcoef); a.f32(cf.zdamp); a.i32(cf.damp_opt); a.i32(0)
        for v in (s.cf1, s.cf2, s.cf3, s.cfn, s.cfn1):
            a.f32(np.float32(v))
        a.i32(1); a.i32(1); a.i32(0); a.f32(0.0); a.f32(0.0)
        a.dims(case)
        a.null(); a.null()                                  # max_vert_cfl, max_horiz_cfl
        return a.call(gpulib, "wrfgpu_rk_tendency"), outs

    rc, outs = call(xk)
    assert rc == 0
    bad = []
    for nm, v in tf0.items():
        od.set(abi.FIELD_ID[nm], v)
    od.run("forward_terms", 1)
    for nm in tf_names:
        fid = abi.FIELD_ID[nm]
        d = max_abs(interior(case, fid, outs[nm], halo=0), interior(case, fid, od.get(fid), halo=0))
        if d != 0.0:
            bad.append("%s: max|diff| %.3e" % (nm, d))
        if np.array_equal(outs[nm], tf0[nm]):
            bad.append("%s unchanged" % nm)
    od.run("rk_tendency", 1)
    for nm in ("ru_tend", "rv_tend", "rw_tend", "ph_tend", "t_tend"):
        fid = abi.FIELD_ID[nm]
        d = max_abs(interior(case, fid, outs[nm], halo=0), interior(case, fid, od.get(fid), halo=0))
        if d != 0.0:
            bad.append("%s: max|diff| %.3e" % (nm, d))
    assert not bad, bad
    rc, _ = call(xk * np.float32(2.0))
    assert rc == abi.WRFGPU_E_ARG


@pytest.mark.parametrize("rk", [1, 2])
def test_rk_addtend_dry_abi_bitwise(gpulib, case_fwd, rk):
    """wrfgpu_rk_addtend_dry (module_em.F:959-1092) with random tendencies,
    forward tendencies, saves, h_diabatic and mu tendencies: at stage 1 the
    saves join the forward tendencies, and every stage adds those to the
    large-step ones; every output bit for bit the oracle's restatement, and a
    patch smaller than the domain is refused."""
    case = case_fwd
    od = _state(case)
    n3 = od.get(abi.FIELD_ID["u_2"]).size
    n2 = od.get(abi.FIELD_ID["mu_2"]).size
    rng = np.random.Generator(np.random.PCG64(50 + rk))
    r3 = lambda sc=1e-3: (sc * rng.standard_normal(n3)).astype(np.float32)
    r2 = lambda sc=1e-3: (sc * rng.standard_normal(n2)).astype(np.float32)
    ins = {nm: r3() for nm in ("ru_tend", "rv_tend", "rw_tend", "ph_tend", "t_tend", "ru_tendf", "rv_tendf",
                               "rw_tendf", "ph_tendf", "t_tendf", "u_save", "v_save", "w_save", "ph_save",
                               "t_save", "h_diabatic")}
    ins["mu_tend"] = r2(); ins["mu_tendf"] = r2()

    def call(patch_off=0):
        a = _Argv()
        outs = {}
        for nm in ("ru_tend", "rv_tend", "rw_tend", "ph_tend", "t_tend", "ru_tendf", "rv_tendf", "rw_tendf",
                   "ph_tendf", "t_tendf"):
            outs[nm] = a.arr(ins[nm].copy())
        for nm in ("u_save", "v_save", "w_save", "ph_save", "t_save"):
            a.arr(ins[nm])
        outs["mu_tend"] = a.arr(ins["mu_tend"].copy()); outs["mu_tendf"] = a.arr(ins["mu_tendf"].copy())
        a.i32(rk); a.arr(_f(od, "c1h")); a.arr(_f(od, "c2h")); a.arr(ins["h_diabatic"])
        for nm in ("mut", "msftx", "msfty", "msfux", "msfuy", "msfvx", "msfvx_inv", "msfvy"):
            a.arr(_f(od, nm))
        h = abi.HALO
        for d in [1, case.ide, 1, case.jde, 1, case.kde, 1 - h, case.ide + h, 1 - h, case.jde + h, 1, case.kde,
                  1, case.ide - patch_off, 1, case.jde, 1, case.kde, 1, case.ide, 1, case.jde, 1, case.kde]:
            a.i32(d)
        return a.call(gpulib, "wrfgpu_rk_addtend_dry"), outs

    rc, outs = call()
    assert rc == 0
    carriers = {"ph_tendf": "advect_tend", "mu_tendf": "mudf"}
    for nm, v in ins.items():
        od.set(abi.FIELD_ID[carriers.get(nm, nm)], v)
    od.run("addtend_dry_args", rk)
    bad = []
    for nm, got in outs.items():
        fid = abi.FIELD_ID[carriers.get(nm, nm)]
        d = max_abs(interior(case, fid, got, halo=0), interior(case, fid, od.get(fid), halo=0))
        if d != 0.0:
            bad.append("%s: max|diff| %.3e" % (nm, d))
    assert not bad, bad
    assert not np.array_equal(outs["ru_tend"], ins["ru_tend"])
    rc, _ = call(patch_off=4)
    assert rc == abi.WRFGPU_E_ARG
