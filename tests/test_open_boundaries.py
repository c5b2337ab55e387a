"""Open lateral boundaries (open_xs/xe/ys/ye, the em_quarter_ss namelist) on
the GPU against the oracle.

Next to an open boundary the reference lowers the horizontal flux order
(module_advect_em.F degrade_xs/xe/ys/ye), adds radiation terms on the
boundary rows (advect_u/v/w/scalar/scalar_pd, rhs_ph), leaves the boundary
velocities out of the pressure gradient, Coriolis and curvature, narrows the
positive-definite limiter, and fills the halo with copies of the edge value
(share/module_bc.F).  The large step evaluates the interior stencils in its
tile kernels and recomputes the points within three of an open edge with
the routine-level point functions; every test here is bit for bit.
"""
import numpy as np
import pytest

from wrf_gb300 import abi, cases
from wrf_gb300 import gpu as G

from _harness import OracleDomain, interior, max_abs, STATE_FIELDS
from test_gpu_parity import (BC1, BC2, BC3, BC4, BC5, compare, fills, sync, _bitwise_diffs)

pytestmark = pytest.mark.gpu

SIDES = {"xy": (True, True), "x": (True, False), "y": (False, True)}


def open_case(sides, nx=26, ny=22, kde=14, n_scalar=2, seed=23):
    x, y = SIDES[sides]
    return cases.open_boundaries(cases.small_case(nx=nx, ny=ny, kde=kde, n_scalar=n_scalar, seed=seed), x=x, y=y)


@pytest.mark.parametrize("sides", list(SIDES))
def test_halo_fill_open_bitwise(gpulib, sides):
    """The open-boundary copies of set_physical_bc3d / set_physical_bc2d
    (three halo points take the edge value; u and v copy their boundary
    point) for every variable kind, on random fields."""
    case = open_case(sides)
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    rng = np.random.default_rng(7)
    jobs = [("u_2", "u"), ("v_2", "v"), ("w_2", "w"), ("t_2", "t"), ("p", "p"), ("ph_2", "w"),
            ("mu_2", "t"), ("muu", "u"), ("muv", "v"), ("mudf", "t")]
    bad = []
    for nm, var in jobs:
        fid = abi.FIELD_ID[nm]
        v = rng.standard_normal(od.get(fid).size).astype(np.float32)
        od.set(fid, v)
        ge.set(0, fid, v)
        od.fill_halo(fid, var)
        ge.fill_halo(fid, var)
        a = interior(case, fid, ge.get(0, fid), halo=3)
        b = interior(case, fid, od.get(fid), halo=3)
        if max_abs(a, b) != 0.0:
            bad.append("%s (%s): max|diff| %.3e" % (nm, var, max_abs(a, b)))
    assert not bad, "\n".join(bad)


@pytest.mark.parametrize("sides", list(SIDES))
def test_open_routine_sequence_bitwise(gpulib, sides):
    """Every routine of one large step on an open domain, bit for bit: the
    routine-level kernels carry the open branches themselves."""
    case = open_case(sides)
    od = OracleDomain(case, "f32")
    od.step(1)
    ge = G.Ensemble([case.desc], flags=G.FLAG_NO_GRAPH)
    nsp = case.desc.n_moist + case.desc.n_scalar
    ns = od.num_sound_steps()

    def rc(name, rk, it=1, sp=0, exclude=()):
        sync(od, ge, case)
        od.run(name, rk, it, sp)
        ge.run_routine(name, rk, it, sp)
        compare(od, ge, case, "%s(rk=%d,it=%d,sp=%d)" % (name, rk, it, sp), exclude=exclude)

    def fill_cmp(jobs, label, **kw):
        sync(od, ge, case)
        fills(od, ge, case, jobs, **kw)
        compare(od, ge, case, "fill " + label)

    for rk in (1, 3):
        nsmall = 1 if rk == 1 else ns
        rc("rk_step_prep", rk)
        fill_cmp(BC1, "BC1")
        for piece in ("advect_u", "advect_v", "advect_w", "advect_t", "rhs_ph", "horizontal_pressure_gradient",
                      "coriolis", "curvature"):
            rc(piece, rk)
        rc("rk_tendency", rk, exclude=("u_save", "v_save", "w_save", "t_save", "ph_save", "mu_save"))
        sync(od, ge, case)
        od.run("rk_tendency", rk)
        ge.run_routine("rk_tendency", rk)
        od.run("small_step_prep", rk)
        ge.run_routine("small_step_prep", rk)
        compare(od, ge, case, "rk_tendency+small_step_prep rk=%d" % rk)
        rc("calc_p_rho", rk, 0)
        rc("calc_coef_w", rk)
        fill_cmp(BC2, "BC2")
        for it in range(1, min(nsmall, 2) + 1):
            rc("advance_uv", rk, it)
            rc("advance_mu_t", rk, it)
            rc("advance_w", rk, it)
            rc("sumflux", rk, it)
            rc("calc_p_rho", rk, it)
            fill_cmp(BC3, "BC3")
        rc("small_step_finish", rk)
        if rk == 3:
            fill_cmp(BC4, "BC4")
            fill_cmp([], "species old", species_old=True)
        for s in range(nsp):
            rc("advect_scalar_pd" if rk == 3 else "advect_scalar", rk, 0, s)
            rc("rk_update_scalar", rk, 0, s)
        if rk < 3:
            fill_cmp(BC5, "BC5", species_cur=True)


@pytest.mark.parametrize("nsteps", [1, 3])
@pytest.mark.parametrize("sides", list(SIDES))
def test_open_full_step_bitwise(gpulib, sides, nsteps):
    """Whole large steps (graph-captured; the tile kernels plus the edge-strip
    recomputation): every state field and species, current and old, bit for
    bit with the FP32 oracle."""
    case = open_case(sides)
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    od.step(nsteps)
    ge.step(nsteps)
    ge.sync()
    bad = _bitwise_diffs(case, ge, od)
    assert not bad, "\n".join(bad)


def test_open_multitile_bitwise(gpulib):
    """70 x 46 x 20 with qv and 3 PD scalars, open on all four sides (3 x 6
    tiles, strips crossing tile edges), with the em_quarter_ss damping
    (damp_opt = 2) and w_damping: 3 large steps bit for bit."""
    case = open_case("xy", nx=70, ny=46, kde=20, n_scalar=3, seed=29)
    c = case.desc.config
    c.damp_opt = 2
    c.zdamp = 5000.0
    c.dampcoef = 0.003
    c.w_damping = 1
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    od.step(3)
    ge.step(3)
    ge.sync()
    bad = _bitwise_diffs(case, ge, od)
    assert not bad, "\n".join(bad)


def test_batched_open_and_periodic_members_equal_plain(gpulib):
    """An ensemble mixing open, periodic and half-open members: each
    member's bits equal its own single-domain run's and the oracle's."""
    members = [open_case("xy", nx=30, ny=24, kde=12, n_scalar=1, seed=51),
               cases.small_case(nx=20, ny=16, kde=14, n_scalar=2, seed=52),
               open_case("y", nx=40, ny=28, kde=10, n_scalar=2, seed=53)]
    ens = G.Ensemble.from_cases(members)
    ens.step(2)
    ens.sync()
    for m, c in enumerate(members):
        d = G.Domain(c)
        d.step(2)
        d.sync()
        nsp = c.desc.n_moist + c.desc.n_scalar
        for fid in [abi.FIELD_ID[nm] for nm in STATE_FIELDS] + [abi.species_id(s) for s in range(nsp)]:
            assert np.array_equal(ens.get(m, fid), d.get(0, fid)), (m, fid)
        od = OracleDomain(c, "f32")
        od.step(2)
        bad = _bitwise_diffs(c, ens, od, member=m, old_too=False)
        assert not bad, "member %d:\n" % m + "\n".join(bad)


def test_open_domain_needs_room_for_the_strips(gpulib):
    """Open sides closer than the two edge strips are refused (E_ARG)."""
    small = open_case("x", nx=10, ny=16)
    with pytest.raises(G.WrfGpuError):
        G.Domain(small)


def _with_diffusion(case, explicit, sixth):
    c = case.desc.config
    if sixth:
        c.diff_6th_opt = 2
        c.diff_6th_factor = 0.12
    if explicit:
        c.diff_opt = 1
        c.km_opt = 1
        c.khdif = 300.0
        c.kvdif = 10.0
    return case


@pytest.mark.parametrize("explicit,sixth", [(True, False), (False, True), (True, True)])
@pytest.mark.parametrize("sides", ["xy", "x", "y"])
def test_open_full_step_bitwise_with_diffusion(gpulib, sides, explicit, sixth):
    """Explicit (diff_opt = 1, km_opt = 1) and sixth-order diffusion with open
    boundaries: each term keeps its own loop limits next to the open edges
    (horizontal_diffusion, vertical_diffusion_u / _v, sixth_order_diffusion,
    including the latter's v limits on open_xs), the species' stored
    tendencies reach the edge strips' scalar update; 2 steps bit for bit."""
    case = _with_diffusion(open_case(sides, seed=61), explicit, sixth)
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    od.step(2)
    ge.step(2)
    ge.sync()
    bad = _bitwise_diffs(case, ge, od)
    assert not bad, "\n".join(bad)
