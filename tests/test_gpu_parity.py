"""GPU parity against the oracle (CPU restatement of the reference).

* Routine level: the oracle's state is copied into the GPU before every
  routine of one solve_em large step, both run the routine, and every field
  is compared.  The plain form is built with --fmad=false and IEEE division,
  so all routines agree bit for bit; the log and pow of calc_p_rho_phi are
  correctly rounded on both sides (float-float with Ziv's rounding test and
  an FP64 fallback on the GPU, FP64 libm rounded once in the oracle).
* Step level: the fused, graph-captured solver bit for bit with the oracle
  on the 41x41x41 supercell after 1 and 60 large steps, on a 100x70x30
  domain with 11 species (many tiles, partial edge tiles), and on small
  cases with every option the solver accepts.
* Batched == plain and graph == no-graph, bit for bit.
* Failure detection: a non-finite value injected on the host is reported by
  the device health check as an error status (no device trap).
"""
import numpy as np
import pytest

from wrf_gb300 import abi, cases
from wrf_gb300 import gpu as G

from _harness import OracleDomain, field_shape, interior, serr, max_abs, STATE_FIELDS

pytestmark = pytest.mark.gpu

ALL3 = list(abi.F3D)
ALL2 = list(abi.F2D)
ALL1 = list(abi.F1D)


def all_ids(case):
    ids = [abi.FIELD_ID[n] for n in ALL3 + ALL2 + ALL1]
    nsp = case.desc.n_moist + case.desc.n_scalar
    for s in range(nsp):
        ids += [abi.species_id(s), abi.species_id(s, True)]
    return ids


def id_name(fid):
    for k, v in abi.FIELD_ID.items():
        if v == fid:
            return k
    s = (fid - abi.SPECIES_BASE) // 2
    return "species%d%s" % (s, "_old" if (fid - abi.SPECIES_BASE) % 2 else "")


def sync(od, ge, case):
    for fid in all_ids(case):
        ge.set(0, fid, od.get(fid))


def compare(od, ge, case, label, exclude=(), tol=None):
    bad = []
    for fid in all_ids(case):
        nm = id_name(fid)
        if nm in exclude:
            continue
        a = interior(case, fid, ge.get(0, fid), halo=3)
        b = interior(case, fid, od.get(fid), halo=3)
        if tol is None:
            d = max_abs(a, b)
            if d != 0.0:
                bad.append("%s: max|diff| %.3e (serr %.2e)" % (nm, d, serr(a, b)))
        else:
            e = serr(a, b)
            if e > tol:
                bad.append("%s: serr %.3e > %.1e" % (nm, e, tol))
    assert not bad, "%s differs:\n  " % label + "\n  ".join(bad)


BC1 = [("ru", "u"), ("rv", "v"), ("rw", "w"), ("ww", "w"), ("php", "w"), ("alt", "t"), ("p", "p"),
       ("muu", "u"), ("muv", "v"), ("mut", "t"), ("al", "p"), ("ph_2", "w")]
BC2 = [("ru_tend", "u"), ("rv_tend", "v"), ("ph_2", "w"), ("al", "p"), ("p", "p"), ("t_1", "p"),
       ("t_save", "t"), ("mu_1", "t"), ("mu_2", "t"), ("mudf", "t")]
BC3 = [("ph_2", "w"), ("al", "p"), ("p", "p"), ("muts", "t"), ("mu_2", "t"), ("mudf", "t")]
BC4 = [("ru_m", "u"), ("rv_m", "v"), ("ww_m", "w"), ("mut", "t"), ("muts", "t")]
BC5 = [("u_2", "u"), ("v_2", "v"), ("w_2", "w"), ("t_2", "p"), ("ph_2", "w"), ("mu_2", "t")]


def fills(od, ge, case, jobs, species_old=None, species_cur=False):
    for nm, var in jobs:
        od.fill_halo(abi.FIELD_ID[nm], var)
        ge.fill_halo(abi.FIELD_ID[nm], var)
    nsp = case.desc.n_moist + case.desc.n_scalar
    for s in range(nsp):
        if species_old:
            od.fill_halo(abi.species_id(s, True), "p")
            ge.fill_halo(abi.species_id(s, True), "p")
        if species_cur:
            od.fill_halo(abi.species_id(s), "p")
            ge.fill_halo(abi.species_id(s), "p")


@pytest.fixture(scope="module")
def small():
    return cases.small_case(nx=16, ny=12, kde=14, n_scalar=2, seed=11)


def test_routine_sequence_bitwise(gpulib, small):
    """Every routine of one large step, bit for bit against the oracle."""
    case = small
    od = OracleDomain(case, "f32")
    od.step(1)  # a developed state (bubble, winds, scalars)
    ge = G.Ensemble([case.desc], flags=G.FLAG_NO_GRAPH)
    nsp = case.desc.n_moist + case.desc.n_scalar
    ns = od.num_sound_steps()
    assert ns == ge.num_sound_steps()

    def rc(name, rk, it=1, sp=0, exclude=(), tol=None, label=None):
        sync(od, ge, case)
        od.run(name, rk, it, sp)
        ge.run_routine(name, rk, it, sp)
        compare(od, ge, case, label or "%s(rk=%d,it=%d,sp=%d)" % (name, rk, it, sp), exclude=exclude, tol=tol)

    def fill_cmp(jobs, label, **kw):
        sync(od, ge, case)
        fills(od, ge, case, jobs, **kw)
        compare(od, ge, case, "fill " + label)

    for rk in (1, 2, 3):
        nsmall = 1 if rk == 1 else (ns // 2 if rk == 2 else ns)
        rc("rk_step_prep", rk)
        fill_cmp(BC1, "BC1")
        # the GPU zeroes only the *_save points small_step_prep will not overwrite
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
        for it in range(1, nsmall + 1):
            rc("advance_uv", rk, it)
            rc("advance_mu_t", rk, it)
            rc("advance_w", rk, it)
            rc("sumflux", rk, it)
            rc("calc_p_rho", rk, it)
            fill_cmp(BC3, "BC3")
        rc("small_step_finish", rk)
        if rk == 3:
            fill_cmp(BC4, "BC4")
            sync(od, ge, case)
            for s in range(nsp):
                od.run("rk_update_scalar_pd", rk, 0, s)
            ge.run_routine("rk_update_scalar_pd", rk, 0, 0)
            compare(od, ge, case, "rk_update_scalar_pd")
            fill_cmp([], "species old", species_old=True)
        for s in range(nsp):
            adv = "advect_scalar_pd" if rk == 3 else "advect_scalar"
            rc(adv, rk, 0, s)
            rc("rk_update_scalar", rk, 0, s)
        rc("calc_p_rho_phi", rk, label="calc_p_rho_phi rk=%d" % rk)
        if rk < 3:
            fill_cmp(BC5, "BC5", species_cur=True)
    rc("set_w_surface", 3)


@pytest.mark.parametrize("piece", ["advect_u", "advect_v", "advect_w", "advect_t", "rhs_ph",
                                   "horizontal_pressure_gradient", "pg_buoy_w", "coriolis", "curvature"])
def test_rk_tendency_pieces_bitwise(gpulib, small, piece):
    """Each rk_tendency sub-routine alone (accumulating into the tendencies)."""
    case = small
    od = OracleDomain(case, "f32")
    od.step(1)
    od.run("rk_step_prep", 1)
    for nm, var in BC1:
        od.fill_halo(abi.FIELD_ID[nm], var)
    ge = G.Ensemble([case.desc], flags=G.FLAG_NO_GRAPH)
    sync(od, ge, case)
    od.run(piece, 2)
    ge.run_routine(piece, 2)
    compare(od, ge, case, piece)


def _step_errors(case, nsteps, flags=0):
    od = OracleDomain(case, "f32")
    ge = G.Domain(case, flags=flags)
    od.step(nsteps)
    ge.step(nsteps)
    ge.sync()
    out = {}
    for nm in STATE_FIELDS:
        fid = abi.FIELD_ID[nm]
        out[nm] = serr(interior(case, fid, ge.get(0, fid)), interior(case, fid, od.get(fid)))
    fid = abi.species_id(0)
    out["qv"] = serr(interior(case, fid, ge.get(0, fid)), interior(case, fid, od.get(fid)))
    return out


def _bitwise_diffs(case, ge, od, member=0, old_too=True):
    """Fields (state, *_1 copies, every species current and old) where the
    GPU and the oracle differ, compared over the interior plus 3 halo points."""
    names = STATE_FIELDS + (["t_1", "ph_1", "mu_1", "u_1", "v_1", "w_1"] if old_too else [])
    ids = [abi.FIELD_ID[nm] for nm in names]
    nsp = case.desc.n_moist + case.desc.n_scalar
    ids += [abi.species_id(s) for s in range(nsp)]
    if old_too:
        ids += [abi.species_id(s, True) for s in range(nsp)]
    bad = []
    for fid in ids:
        a = interior(case, fid, ge.get(member, fid), halo=3)
        b = interior(case, fid, od.get(fid), halo=3)
        d = max_abs(a, b)
        if d != 0.0:
            bad.append("%s: max|diff| %.3e serr %.2e" % (id_name(fid), d, serr(a, b)))
    return bad


def test_c1_bitwise_1_and_60_steps(gpulib):
    """The 41x41 x 41-level supercell (2 x 6 tiles of 32 x 8 with partial
    edge tiles, periodic wrap inside the TMA halo planes): every state field
    and qv, current and old, bit for bit with the FP32 oracle after 1 and
    after 60 large steps."""
    case = cases.config1()
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    done = 0
    for n in (1, 60):
        od.step(n - done)
        ge.step(n - done)
        done = n
        ge.sync()
        bad = _bitwise_diffs(case, ge, od)
        assert not bad, "after %d steps:\n" % n + "\n".join(bad)


@pytest.mark.parametrize("nsteps", [1, 3])
def test_multitile_11_species_bitwise(gpulib, nsteps):
    """100 x 70 x 30 levels with qv and 10 PD scalars: 4 x 9 tiles of
    32 x 8 with partial edge tiles in both directions, so the halo planes
    wrap around the periodic boundary in the middle of a tile row; every
    field and all 11 species, current and old, bit for bit."""
    case = cases.small_case(nx=100, ny=70, kde=30, n_scalar=10, seed=31)
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    od.step(nsteps)
    ge.step(nsteps)
    ge.sync()
    bad = _bitwise_diffs(case, ge, od)
    assert not bad, "\n".join(bad)


@pytest.mark.parametrize("nsteps", [1, 3])
def test_full_step_bitwise(gpulib, small, nsteps):
    """The fused solver (graph-captured, scalar transport fused with the RK
    update, species buffers swapped) gives the oracle's bits: every state
    field and every species, current and old, after 1 and 3 large steps."""
    case = small
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    od.step(nsteps)
    ge.step(nsteps)
    ge.sync()
    bad = []
    ids = [abi.FIELD_ID[nm] for nm in STATE_FIELDS + ["t_1", "ph_1", "mu_1", "u_1", "v_1", "w_1"]]
    nsp = case.desc.n_moist + case.desc.n_scalar
    ids += [abi.species_id(s) for s in range(nsp)] + [abi.species_id(s, True) for s in range(nsp)]
    for fid in ids:
        a = interior(case, fid, ge.get(0, fid), halo=3)
        b = interior(case, fid, od.get(fid), halo=3)
        d = max_abs(a, b)
        if d != 0.0:
            bad.append("%s: max|diff| %.3e serr %.2e" % (id_name(fid), d, serr(a, b)))
    assert not bad, "\n".join(bad)


def rotating_case():
    """The small case with non-uniform map factors and a Coriolis parameter,
    so that the map-factor ratios, the Coriolis and the curvature terms of the
    momentum tendencies carry non-trivial values (the idealized cases have
    unit map factors and f = e = 0)."""
    case = cases.small_case(nx=16, ny=12, kde=14, n_scalar=1, seed=13)
    F = case.fields
    nj, ni = F["msfux"].shape
    jj, ii = np.meshgrid(np.arange(nj), np.arange(ni), indexing="ij")
    for n, nm in enumerate(("msfux", "msfuy", "msfvx", "msfvy", "msftx", "msfty")):
        F[nm][...] = 1.0 + 0.03 * np.sin(0.4 * ii + 0.3 * jj + n)
    F["msfvx_inv"][...] = 1.0 / F["msfvx"]
    ang = 0.2 * np.sin(0.25 * ii - 0.35 * jj)
    F["sina"][...] = np.sin(ang)
    F["cosa"][...] = np.cos(ang)
    F["f"][...] = 1.0e-4 * (1.0 + 0.3 * np.cos(0.2 * jj))
    F["e"][...] = 1.2e-4 * (1.0 + 0.2 * np.sin(0.3 * ii))
    return case


@pytest.mark.parametrize("nsteps", [1, 2])
def test_full_step_bitwise_rotating(gpulib, nsteps):
    """Bit for bit with the oracle with map factors, Coriolis and curvature
    terms active (the column tendency kernels form their column-invariant
    products once; the rounding must stay the reference's)."""
    case = rotating_case()
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    od.step(nsteps)
    ge.step(nsteps)
    ge.sync()
    bad = []
    for nm in STATE_FIELDS:
        fid = abi.FIELD_ID[nm]
        a = interior(case, fid, ge.get(0, fid), halo=3)
        b = interior(case, fid, od.get(fid), halo=3)
        d = max_abs(a, b)
        if d != 0.0:
            bad.append("%s: max|diff| %.3e serr %.2e" % (nm, d, serr(a, b)))
    assert not bad, "\n".join(bad)


def test_autotune_keeps_bits(gpulib, small):
    """The autotuner's variants compute the same bits: 4 tuning steps (every
    variant of every family in turn) plus 1 graph step with the choice equal
    the oracle's 5 steps."""
    case = small
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    tun = ge.autotune(1)
    assert set(tun) == set(G.Ensemble.TUNE_FAMILIES)
    for f, t in tun.items():
        assert 0 <= t["variant"] < 4 and t["param"] > 0 and len(t["ms"]) >= 2, (f, t)
    ge.step(1)
    ge.sync()
    od.step(5)
    bad = []
    nsp = case.desc.n_moist + case.desc.n_scalar
    ids = [abi.FIELD_ID[nm] for nm in STATE_FIELDS] + [abi.species_id(s) for s in range(nsp)]
    for fid in ids:
        a = interior(case, fid, ge.get(0, fid), halo=3)
        b = interior(case, fid, od.get(fid), halo=3)
        if max_abs(a, b) != 0.0:
            bad.append(id_name(fid))
    assert not bad, bad


def test_graph_equals_direct(gpulib, small):
    a = G.Domain(small, flags=G.FLAG_NO_GRAPH)
    b = G.Domain(small, flags=0)
    a.step(3)
    b.step(3)
    a.sync()
    b.sync()
    for nm in STATE_FIELDS:
        fid = abi.FIELD_ID[nm]
        assert np.array_equal(a.get(0, fid), b.get(0, fid)), nm


def test_batched_equals_plain_wide_members(gpulib):
    """Members three or more tiles wide in both directions, of different
    level counts and species counts, in one launch: each member's bits equal
    its own single-domain run's and the FP32 oracle's."""
    members = [cases.small_case(nx=72, ny=20, kde=16, n_scalar=2, seed=41),
               cases.small_case(nx=100, ny=30, kde=12, n_scalar=1, seed=42),
               cases.small_case(nx=66, ny=40, kde=20, n_scalar=3, seed=43)]
    ens = G.Ensemble.from_cases(members)
    ens.step(2)
    ens.sync()
    for m, c in enumerate(members):
        d = G.Domain(c)
        d.step(2)
        d.sync()
        nsp = c.desc.n_moist + c.desc.n_scalar
        ids = [abi.FIELD_ID[nm] for nm in STATE_FIELDS] + [abi.species_id(s) for s in range(nsp)]
        for fid in ids:
            assert np.array_equal(ens.get(m, fid), d.get(0, fid)), (m, id_name(fid))
        od = OracleDomain(c, "f32")
        od.step(2)
        bad = _bitwise_diffs(c, ens, od, member=m, old_too=False)
        assert not bad, "member %d:\n" % m + "\n".join(bad)


def test_batched_equals_plain(gpulib):
    """Uneven members in one launch give the same bits as each member alone."""
    members = [cases.small_case(nx=16, ny=12, kde=14, n_scalar=2, seed=3),
               cases.small_case(nx=24, ny=10, kde=12, n_scalar=1, seed=4),
               cases.small_case(nx=12, ny=20, kde=16, n_scalar=3, seed=5)]
    ens = G.Ensemble.from_cases(members)
    ens.step(2)
    ens.sync()
    for m, c in enumerate(members):
        d = G.Domain(c)
        d.step(2)
        d.sync()
        for nm in STATE_FIELDS:
            fid = abi.FIELD_ID[nm]
            assert np.array_equal(ens.get(m, fid), d.get(0, fid)), (m, nm)
        nsp = c.desc.n_moist + c.desc.n_scalar
        for s in range(nsp):
            assert np.array_equal(ens.get(m, abi.species_id(s)), d.get(0, abi.species_id(s))), (m, s)


def test_nonfinite_detected_without_fault(gpulib, small):
    d = G.Domain(small)
    t = small.fields["t_2"].copy()
    t[6, 3, 7] = np.nan
    d.set(0, abi.FIELD_ID["t_2"], t)
    d.clear_status()
    d.step(1)
    rc, bits, vc, hc = d.status(0)
    assert rc == abi.WRFGPU_E_NONFINITE and bits & 1
    # the context stays usable: a clean state steps and reports OK
    d2 = G.Domain(small)
    d2.step(1)
    rc2, bits2, vc2, hc2 = d2.status(0)
    assert rc2 == 0 and bits2 == 0 and vc2 > 0 and hc2 > 0


def test_cfl_limit_reported(gpulib, small):
    d = G.Domain(small)
    d.set_cfl_limit(1e-9)
    d.step(1)
    rc, bits, vc, hc = d.status(0)
    assert rc == abi.WRFGPU_E_CFL and bits & 2


def test_mixed_precision_close_to_fp64(gpulib):
    """The mixed form (FP64 column sums / Thomas) tracks the FP64 oracle at
    least as well as the plain FP32 form does, within 1e-4 after 10 steps
    for u, v, theta, ph and mu (the FP32 oracle itself is 1e-5..6e-5 off
    there; w, p and al, whose FP32 error is 2e-4..2e-3, are reported by
    the bench instead)."""
    case = cases.config1()
    o64 = OracleDomain(case, "f64")
    o64.step(10)
    plain = G.Domain(case)
    mixed = G.Domain(case, flags=G.FLAG_MIXED)
    plain.step(10)
    mixed.step(10)
    plain.sync()
    mixed.sync()
    for nm in ("u_2", "v_2", "t_2", "ph_2", "mu_2"):
        fid = abi.FIELD_ID[nm]
        ref = interior(case, fid, o64.get(fid))
        ep = serr(interior(case, fid, plain.get(0, fid)), ref)
        em = serr(interior(case, fid, mixed.get(0, fid)), ref)
        assert em <= 1e-4, (nm, em, ep)
        assert em <= 3 * ep + 1e-7, (nm, em, ep)


@pytest.mark.parametrize("bc", ["periodic", "symmetric_y"])
def test_halo_fill_bitwise(gpulib, bc):
    """The halo fill of every variable kind against the oracle's restatement
    of set_physical_bc3d / set_physical_bc2d (periodic x; periodic or
    symmetric y, where the normal velocity changes sign), on random fields."""
    case = cases.small_case(nx=16, ny=12, kde=14, n_scalar=1, seed=5)
    if bc == "symmetric_y":
        c = case.desc.config
        c.periodic_y = 0
        c.symmetric_ys = 1
        c.symmetric_ye = 1
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    rng = np.random.default_rng(3)
    jobs = [("u_2", "u"), ("v_2", "v"), ("w_2", "w"), ("t_2", "t"), ("p", "p"), ("ph_2", "w"),
            ("mu_2", "t"), ("muu", "u"), ("muv", "v")]
    bad = []
    for nm, var in jobs:
        fid = abi.FIELD_ID[nm]
        x = rng.standard_normal(od.get(fid).size).astype(np.float32)
        od.set(fid, x)
        ge.set(0, fid, x)
        od.fill_halo(fid, var)
        ge.fill_halo(fid, var)
        a = interior(case, fid, ge.get(0, fid), halo=3)
        b = interior(case, fid, od.get(fid), halo=3)
        if max_abs(a, b) != 0.0:
            bad.append("%s (%s): max|diff| %.3e" % (nm, var, max_abs(a, b)))
    assert not bad, "\n".join(bad)


@pytest.mark.parametrize("nsteps", [1, 2])
def test_full_step_bitwise_symmetric_y(gpulib, nsteps):
    """Whole large steps with symmetric (free-slip) boundaries in y: the
    acoustic kernels skip the v pressure gradient and the tendency on the
    boundary rows, and the halo fill mirrors with a sign change for v."""
    case = cases.small_case(nx=16, ny=12, kde=14, n_scalar=1, seed=17)
    c = case.desc.config
    c.periodic_y = 0
    c.symmetric_ys = 1
    c.symmetric_ye = 1
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    od.step(nsteps)
    ge.step(nsteps)
    ge.sync()
    bad = []
    for nm in STATE_FIELDS:
        fid = abi.FIELD_ID[nm]
        a = interior(case, fid, ge.get(0, fid), halo=3)
        b = interior(case, fid, od.get(fid), halo=3)
        d = max_abs(a, b)
        if d != 0.0:
            bad.append("%s: max|diff| %.3e serr %.2e" % (nm, d, serr(a, b)))
    assert not bad, "\n".join(bad)


def damping_case():
    """Strong convergence (a 60 m/s wave in u over 8 points) on 40 levels
    with dt = 30 s: vertical Courant numbers reach ~2, so w_damp's term is
    active at many points (measured on the oracle)."""
    case = cases.small_case(nx=16, ny=12, kde=40, n_scalar=1, seed=17, dt=30.0)
    F = case.fields
    ni = F["u_2"].shape[-1]
    pert = (60.0 * np.sin(2 * np.pi * np.arange(ni) / 8.0)).astype(F["u_2"].dtype)
    for nm in ("u_1", "u_2"):
        F[nm][...] = F[nm] + pert
    c = case.desc.config
    c.w_damping = 1
    c.w_crit_cfl = 1.2
    return case


@pytest.mark.parametrize("nsteps", [1, 2])
def test_full_step_bitwise_w_damping(gpulib, nsteps):
    """w_damping = 1 (module_big_step_utilities_em.F:2687-2691): rw_tend
    loses sign(w) w_alpha (cfl - w_crit_cfl) mu wherever the vertical Courant
    number passes w_beta; bit for bit with the oracle, and the term is
    active (the oracle's state differs from its w_damping = 0 run)."""
    case = damping_case()
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    od.step(nsteps)
    ge.step(nsteps)
    ge.sync()
    bad = []
    for nm in STATE_FIELDS:
        fid = abi.FIELD_ID[nm]
        a = interior(case, fid, ge.get(0, fid), halo=3)
        b = interior(case, fid, od.get(fid), halo=3)
        d = max_abs(a, b)
        if d != 0.0:
            bad.append("%s: max|diff| %.3e serr %.2e" % (nm, d, serr(a, b)))
    assert not bad, "\n".join(bad)
    case.desc.config.w_damping = 0
    o0 = OracleDomain(case, "f32")
    o0.step(nsteps)
    fid = abi.FIELD_ID["w_2"]
    assert max_abs(o0.get(fid), od.get(fid)) > 0.0


def test_field_copies_pinned_and_pageable(gpulib, small):
    """wrfgpu_set_field_f32 / wrfgpu_get_field_f32 move the same bits whether
    the host array is pageable (staged copy) or page-locked (read and written
    in place by the copy kernels)."""
    torch = pytest.importorskip("torch")
    ge = G.Domain(small)
    rng = np.random.default_rng(1)
    for fid in (abi.FIELD_ID["u_2"], abi.FIELD_ID["w_2"], abi.FIELD_ID["mu_2"], abi.FIELD_ID["c1h"],
                abi.species_id(0)):
        n = ge.field_size(0, fid)
        x = rng.standard_normal(n).astype(np.float32)
        pin = torch.empty(n, dtype=torch.float32, pin_memory=True).numpy()
        pin[:] = x
        ge.set(0, fid, pin)
        assert np.array_equal(ge.get(0, fid), x)
        out = torch.empty(n, dtype=torch.float32, pin_memory=True).numpy()
        assert ge.L.wrfgpu_get_field_f32(ge.h, 0, fid, out.ctypes.data, n) == 0
        assert np.array_equal(out, x)
        y = (x + 1.0).astype(np.float32)
        ge.set(0, fid, y)
        assert ge.L.wrfgpu_get_field_f32(ge.h, 0, fid, out.ctypes.data, n) == 0
        assert np.array_equal(out, y)


def rayleigh_case():
    """damp_opt = 3 with the Registry's dampcoef 0.2 and zdamp 5000 m under
    the 20 km lid of the small case: the top levels are damped."""
    case = cases.small_case(nx=16, ny=12, kde=20, n_scalar=1, seed=19)
    c = case.desc.config
    c.damp_opt = 3
    c.dampcoef = 0.2
    c.zdamp = 5000.0
    return case


@pytest.mark.parametrize("nsteps", [1, 2])
def test_full_step_bitwise_damp_opt_3(gpulib, nsteps):
    """The implicit Rayleigh damping of w in advance_w
    (module_small_step_em.F:1445-1458), whose weight takes a correctly rounded
    sine: bit for bit with the oracle, and active (the oracle's state differs
    from its damp_opt = 0 run)."""
    case = rayleigh_case()
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    od.step(nsteps)
    ge.step(nsteps)
    ge.sync()
    bad = []
    for nm in STATE_FIELDS:
        fid = abi.FIELD_ID[nm]
        a = interior(case, fid, ge.get(0, fid), halo=3)
        b = interior(case, fid, od.get(fid), halo=3)
        d = max_abs(a, b)
        if d != 0.0:
            bad.append("%s: max|diff| %.3e serr %.2e" % (nm, d, serr(a, b)))
    assert not bad, "\n".join(bad)
    case.desc.config.damp_opt = 0
    o0 = OracleDomain(case, "f32")
    o0.step(nsteps)
    fid = abi.FIELD_ID["w_2"]
    assert max_abs(o0.get(fid), od.get(fid)) > 0.0


def test_routine_advance_w_damp_opt_3(gpulib):
    """The routine-level advance_w with damp_opt = 3 against the oracle's,
    after the routines that precede it in the first acoustic step."""
    case = rayleigh_case()
    od = OracleDomain(case, "f32")
    od.step(1)
    ge = G.Ensemble([case.desc], flags=G.FLAG_NO_GRAPH)
    sync(od, ge, case)
    for name, it in (("rk_step_prep", 1), ("rk_tendency", 1), ("small_step_prep", 1), ("calc_p_rho", 0),
                     ("calc_coef_w", 1), ("advance_uv", 1), ("advance_mu_t", 1)):
        od.run(name, 1, it, 0)
    sync(od, ge, case)
    od.run("advance_w", 1, 1, 0)
    ge.run_routine("advance_w", 1, 1, 0)
    compare(od, ge, case, "advance_w with damp_opt = 3")


def test_batched_mixed_options_equals_plain(gpulib):
    """An ensemble whose members differ in the damping options (w_damping = 1,
    damp_opt = 3, symmetric y) gives each member the bits it gets alone: the
    launches compile the options in when any member uses them and each member
    applies its own."""
    a = damping_case()
    b = rayleigh_case()
    c = cases.small_case(nx=12, ny=20, kde=16, n_scalar=1, seed=5)
    cf = c.desc.config
    cf.periodic_y = 0
    cf.symmetric_ys = 1
    cf.symmetric_ye = 1
    members = [a, b, c]
    ens = G.Ensemble.from_cases(members)
    ens.step(2)
    ens.sync()
    for m, cs in enumerate(members):
        d = G.Domain(cs)
        d.step(2)
        d.sync()
        for nm in STATE_FIELDS:
            fid = abi.FIELD_ID[nm]
            assert np.array_equal(ens.get(m, fid), d.get(0, fid)), (m, nm)


def diffusion_case(opt, slopeopt, species=True):
    """Sixth-order diffusion on the small case with a 60 m/s wave in u over
    8 points; the moist and passive species diffused too unless species is
    False."""
    case = cases.small_case(nx=16, ny=12, kde=20, n_scalar=2, seed=23)
    F = case.fields
    ni = F["u_2"].shape[-1]
    pert = (60.0 * np.sin(2 * np.pi * np.arange(ni) / 8.0)).astype(F["u_2"].dtype)
    for nm in ("u_1", "u_2"):
        F[nm][...] = F[nm] + pert
    c = case.desc.config
    c.diff_6th_opt = opt
    c.diff_6th_slopeopt = slopeopt
    c.diff_6th_factor = 0.12
    c.diff_6th_thresh = 0.10
    c.moist_mix6_off = 0 if species else 1
    c.scalar_mix6_off = 0 if species else 1
    return case


@pytest.mark.parametrize("opt,slopeopt,species", [(1, 0, False), (1, 0, True), (2, 0, True), (2, 1, True)])
def test_full_step_bitwise_diff_6th(gpulib, opt, slopeopt, species):
    """Sixth-order diffusion of u, v, w and theta at stage 1
    (module_big_step_utilities_em.F:6220-6636) added at every stage by
    rk_addtend_dry (module_em.F:959-1092), and of the species at stage 1
    into sc_tend (module_em.F:1421-1435) added by rk_update_scalar and the
    positive-definite pre-update: bit for bit with the oracle over two steps
    (state and species), and active (the oracle's state differs from its
    diff_6th_opt = 0 run)."""
    case = diffusion_case(opt, slopeopt, species)
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    od.step(2)
    ge.step(2)
    ge.sync()
    bad = []
    nsp = case.desc.n_moist + case.desc.n_scalar
    for nm, fid in [(n, abi.FIELD_ID[n]) for n in STATE_FIELDS] + [("q%d" % s, abi.species_id(s)) for s in range(nsp)]:
        a = interior(case, fid, ge.get(0, fid), halo=3)
        b = interior(case, fid, od.get(fid), halo=3)
        d = max_abs(a, b)
        if d != 0.0:
            bad.append("%s: max|diff| %.3e serr %.2e" % (nm, d, serr(a, b)))
    assert not bad, "\n".join(bad)
    case.desc.config.diff_6th_opt = 0
    o0 = OracleDomain(case, "f32")
    o0.step(2)
    if species:
        fid = abi.species_id(0)
        assert max_abs(interior(case, fid, o0.get(fid), halo=3), interior(case, fid, od.get(fid), halo=3)) > 0
    fid = abi.FIELD_ID["u_2"]
    assert max_abs(interior(case, fid, o0.get(fid), halo=3), interior(case, fid, od.get(fid), halo=3)) > 0


def sloped_diffusion_case():
    """diffusion_case(2, 1) over terrain-following base-state geopotential:
    phb gains g h(x, y) znw(k) for a smooth periodic terrain h of a few
    metres, and diff_6th_thresh is lowered to 0.001 (a 2 m height step per
    2 km grid length), so that the slope taper of sixth_order_diffusion lies
    strictly between 0 and 1 at some faces and is clamped to 0 at others."""
    case = diffusion_case(2, 1)
    case.desc.config.diff_6th_thresh = 0.001
    F = case.fields
    h = abi.HALO
    nj, nk, ni = F["phb"].shape
    nx, ny = case.ide - 1, case.jde - 1
    xi = (np.arange(ni) - h) % nx
    yj = (np.arange(nj) - h) % ny
    hgt = 5.0 * (1.0 + np.sin(4.0 * np.pi * xi / nx)[None, :] * np.cos(2.0 * np.pi * yj / ny)[:, None])
    znw = np.asarray(F["znw"], dtype=np.float64)[:nk]
    F["phb"] = F["phb"] + cases.G * hgt[:, None, :] * znw[None, :, None]
    return case


def test_full_step_bitwise_diff_6th_slope_taper(gpulib):
    """diff_6th_slopeopt = 1 with a base-state geopotential that varies in x
    and y: the taper max(1 - |dphb| msf / (thresh g dx), 0) of every face
    (module_big_step_utilities_em.F:6487-6590) takes values strictly inside
    (0, 1) and clamps to 0 elsewhere; the state after two steps is bit for
    bit the oracle's, and differs from the untapered run's."""
    case = sloped_diffusion_case()
    phb = case.fields["phb"]
    dx = 1.0 / case.desc.scalars.rdx
    thresh = case.desc.config.diff_6th_thresh * 9.81 * dx
    z = np.abs(np.diff(phb, axis=2))
    sd = np.maximum(1.0 - z / thresh, 0.0)
    assert np.count_nonzero((sd > 0.0) & (sd < 1.0)) > 100 and np.count_nonzero(sd == 0.0) > 100
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    od.step(2)
    ge.step(2)
    ge.sync()
    bad = []
    nsp = case.desc.n_moist + case.desc.n_scalar
    for nm, fid in [(n, abi.FIELD_ID[n]) for n in STATE_FIELDS] + [("q%d" % s, abi.species_id(s)) for s in range(nsp)]:
        a = interior(case, fid, ge.get(0, fid), halo=3)
        b = interior(case, fid, od.get(fid), halo=3)
        d = max_abs(a, b)
        if d != 0.0:
            bad.append("%s: max|diff| %.3e serr %.2e" % (nm, d, serr(a, b)))
    assert not bad, "\n".join(bad)
    case.desc.config.diff_6th_slopeopt = 0
    o0 = OracleDomain(case, "f32")
    o0.step(2)
    for nm in ("u_2", "t_2"):
        fid = abi.FIELD_ID[nm]
        assert max_abs(interior(case, fid, o0.get(fid), halo=3), interior(case, fid, od.get(fid), halo=3)) > 0, nm


def test_bounded_wait_times_out_without_fault(gpulib):
    """The bounded mbarrier wait of the TMA-ring kernels: a phase that
    nothing completes makes the wait give up after its poll limit, the
    timeout bit is recorded and WRFGPU_E_TIMEOUT returned; the positive
    control (the phase completed first) returns 0; and the context stays
    usable: a domain steps and reports a clean status afterwards."""
    import ctypes as C
    lib = gpulib
    lib.wrfgpu_selftest_bounded_wait.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_uint)]
    lib.wrfgpu_selftest_bounded_wait.restype = C.c_int
    bits = C.c_uint(0)
    assert lib.wrfgpu_selftest_bounded_wait(4096, 1, C.byref(bits)) == 0 and bits.value == 0
    assert lib.wrfgpu_selftest_bounded_wait(4096, 0, C.byref(bits)) == abi.WRFGPU_E_TIMEOUT
    assert bits.value & 4
    case = cases.small_case(nx=16, ny=12, kde=14, n_scalar=1, seed=5)
    d = G.Domain(case)
    d.step(1)
    rc, b, vc, hc = d.status(0)
    assert rc == 0 and b == 0


def rayleigh2_case(diff6=False):
    """damp_opt = 2 over the top 5 km of the small case's 20 km column,
    dampcoef 0.01 s-1; with diff6 the sixth-order diffusion is on too, so
    the damping accumulates onto the stored diffusion tendencies."""
    case = diffusion_case(2, 0) if diff6 else cases.small_case(nx=16, ny=12, kde=20, n_scalar=1, seed=19)
    c = case.desc.config
    c.damp_opt = 2
    c.dampcoef = 0.01
    c.zdamp = 5000.0
    return case


@pytest.mark.parametrize("diff6", [False, True])
def test_full_step_bitwise_damp_opt_2(gpulib, diff6):
    """rk_rayleigh_damp (module_big_step_utilities_em.F:5836-6110) at stage 1
    into ru_tendf .. t_tendf, added at every stage by rk_addtend_dry: the
    state after two steps bit for bit the oracle's (alone and on top of the
    sixth-order diffusion), and the term is active (the oracle's state
    differs from its damp_opt = 0 run)."""
    case = rayleigh2_case(diff6)
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    od.step(2)
    ge.step(2)
    ge.sync()
    bad = _bitwise_diffs(case, ge, od, old_too=False)
    assert not bad, "\n".join(bad)
    case.desc.config.damp_opt = 0
    o0 = OracleDomain(case, "f32")
    o0.step(2)
    for nm in ("u_2", "w_2", "t_2"):
        fid = abi.FIELD_ID[nm]
        assert max_abs(interior(case, fid, o0.get(fid), halo=3), interior(case, fid, od.get(fid), halo=3)) > 0, nm


def explicit_case(variant):
    """Explicit diffusion with constant coefficients (diff_opt = 1, km_opt = 1,
    khdif 1500 m2/s, kvdif 40 m2/s) on the small case.  "with_diff6": on
    top of the sixth-order diffusion's wave case, with damp_opt = 2 too, so
    every stored tendency accumulates three terms; "mix2_off": the moist
    species left out of the explicit diffusion."""
    if variant == "with_diff6":
        case = diffusion_case(2, 0)
        case.desc.config.damp_opt = 2
        case.desc.config.dampcoef = 0.01
        case.desc.config.zdamp = 5000.0
    else:
        case = cases.small_case(nx=16, ny=12, kde=20, n_scalar=2, seed=31)
    c = case.desc.config
    c.diff_opt = 1
    c.km_opt = 1
    c.khdif = 1500.0
    c.kvdif = 40.0
    c.moist_mix2_off = 1 if variant == "mix2_off" else 0
    return case


def test_full_step_bitwise_explicit_diffusion_symmetric_y(gpulib):
    """diff_opt = 1 with mirrored y boundaries: the diffusion stencils read
    the symmetric halo rows (v changes sign across the boundary); every
    state field and species after two steps bit for bit the oracle's."""
    case = cases.small_case(nx=16, ny=12, kde=16, n_scalar=2, seed=17)
    c = case.desc.config
    c.periodic_y = 0
    c.symmetric_ys = 1
    c.symmetric_ye = 1
    c.diff_opt = 1
    c.km_opt = 1
    c.khdif = 1500.0
    c.kvdif = 40.0
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    od.step(2)
    ge.step(2)
    ge.sync()
    bad = _bitwise_diffs(case, ge, od, old_too=False)
    assert not bad, "\n".join(bad)


@pytest.mark.parametrize("variant", ["alone", "with_diff6", "mix2_off"])
def test_full_step_bitwise_explicit_diffusion(gpulib, variant):
    """diff_opt = 1 (module_em.F:801-877 in rk_tendency's forward step and
    1378-1419 in rk_scalar_tend): horizontal and vertical diffusion of u, v,
    w, theta (against t_init) and the species (qv against qv_base) into the
    stored tendencies at stage 1, ahead of the sixth-order diffusion and the
    Rayleigh damping: every state field and species after two steps bit for
    bit the oracle's, and the term is active (the oracle's state differs from
    its diff_opt = 0 run)."""
    case = explicit_case(variant)
    od = OracleDomain(case, "f32")
    ge = G.Domain(case)
    od.step(2)
    ge.step(2)
    ge.sync()
    bad = _bitwise_diffs(case, ge, od, old_too=False)
    assert not bad, "\n".join(bad)
    case.desc.config.diff_opt = 0
    o0 = OracleDomain(case, "f32")
    o0.step(2)
    for fid in [abi.FIELD_ID[nm] for nm in ("u_2", "v_2", "w_2", "t_2")] + [abi.species_id(0), abi.species_id(2)]:
        d = max_abs(interior(case, fid, o0.get(fid), halo=3), interior(case, fid, od.get(fid), halo=3))
        if fid == abi.species_id(0) and variant == "mix2_off":
            continue  # qv still feels the diffused winds; only its own term is off
        assert d > 0, id_name(fid)


def test_batched_damp_opt_2_with_other_options(gpulib):
    """An ensemble of a damp_opt = 2 member, a member with the sixth-order
    diffusion, one with the explicit diffusion and a plain one: each member
    gets the bits it gets alone."""
    members = [rayleigh2_case(False), diffusion_case(1, 0), explicit_case("alone"),
               cases.small_case(nx=20, ny=12, kde=16, n_scalar=2, seed=6)]
    ens = G.Ensemble.from_cases(members)
    ens.step(2)
    ens.sync()
    for m, cs in enumerate(members):
        d = G.Domain(cs)
        d.step(2)
        d.sync()
        nsp = cs.desc.n_moist + cs.desc.n_scalar
        for fid in [abi.FIELD_ID[nm] for nm in STATE_FIELDS] + [abi.species_id(s) for s in range(nsp)]:
            assert np.array_equal(ens.get(m, fid), d.get(0, fid)), (m, id_name(fid))
