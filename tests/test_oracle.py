"""The oracle against known answers and the properties the reference's
equations guarantee (CPU only).

The reference ships no golden output for this path, so the restatement is
pinned by:
* known answers of the advection stencils derived from their mathematics
  (exactness on polynomials, the 2-dx damping rate of the 5th-order upwind
  flux);
* the reference's own advection fixture (module_advect_em.F:10564-10871,
  a top-hat carried around a periodic 90-point channel): mass conserved,
  positivity with the PD limiter, return to the starting position;
* conservation and balance: a windless, bubble-free state stays at rest; dry
  mass and coupled scalar mass are conserved with periodic boundaries;
  positive-definite scalars stay non-negative;
* determinism: the tile decomposition (OpenMP j-slabs) does not change a bit,
  and FP32 stays close to FP64.
"""
import numpy as np
import pytest

from wrf_gb300 import abi, cases

from _harness import OracleDomain, interior, tophat_feeder, serr

H = abi.HALO


def mass_interior(case, a, kind=3):
    """Mass points i in [1, ide-1], j in [1, jde-1], k in [1, kde-1]."""
    a = np.asarray(a)
    if kind == 3:
        a = a.reshape(case.jde + 2 * H, case.kde, case.ide + 2 * H)
        return a[H:H + case.jde - 1, :case.kde - 1, H:H + case.ide - 1]
    a = a.reshape(case.jde + 2 * H, case.ide + 2 * H)
    return a[H:H + case.jde - 1, H:H + case.ide - 1]


def rest_case(kde=20, hyps=1):
    rng = np.random.Generator(np.random.PCG64(0))
    return cases.supercell_state(12, 10, kde, 2000.0, 12.0, 20000.0, [], rng, n_scalar=1, noise=0.0,
                                 hodo_radius=0.0, name="rest", hypsometric_opt=hyps)


@pytest.fixture(scope="module")
def small():
    return cases.small_case(nx=12, ny=10, kde=12, n_scalar=2, seed=11)


# ---------------------------------------------------------------------------
# known answers of the flux-divergence stencils
# ---------------------------------------------------------------------------
def _advect_species(case, q, ru=0.0, rv=0.0, ww=0.0):
    od = OracleDomain(case, "f64")
    shp = (case.jde + 2 * H, case.kde, case.ide + 2 * H)
    od.set(abi.FIELD_ID["ru_m"], np.full(shp, ru))
    od.set(abi.FIELD_ID["rv_m"], np.full(shp, rv))
    od.set(abi.FIELD_ID["ww_m"], np.full(shp, ww))
    od.set(abi.species_id(0), q)
    od.set(abi.species_id(0, True), q)
    od.run("advect_scalar", 1, 0, 0)
    return od.get(abi.FIELD_ID["advect_tend"]).reshape(shp)


def _coords(case):
    shp = (case.jde + 2 * H, case.kde, case.ide + 2 * H)
    j, k, i = np.meshgrid(np.arange(shp[0]) + 1 - H, np.arange(shp[1]) + 1, np.arange(shp[2]) + 1 - H, indexing="ij")
    return i.astype(float), j.astype(float), k.astype(float)


@pytest.mark.parametrize("vel", [7.5, -7.5])
def test_flux5_exact_on_quintic_x(small, vel):
    """module_advect_em.F:3102-3119 flux5: the difference of the centred
    6-point fluxes is the 6th-order central derivative (exact to degree 6)
    and the upwind part is a 5th difference (constant for a quintic), so the
    x divergence is exactly -U rdx P'(i)."""
    case = small
    i, _, _ = _coords(case)
    P = lambda x: 0.3 + 0.2 * x - 0.05 * x ** 2 + 0.004 * x ** 3 - 1e-4 * x ** 4 + 2e-6 * x ** 5
    dP = lambda x: 0.2 - 0.1 * x + 0.012 * x ** 2 - 4e-4 * x ** 3 + 1e-5 * x ** 4
    tend = _advect_species(case, P(i), ru=vel)
    rdx = case.desc.scalars.rdx
    want = -vel * rdx * dP(i)
    got = mass_interior(case, tend)
    ref = mass_interior(case, want)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("vel", [4.0, -4.0])
def test_flux5_exact_on_quartic_y(small, vel):
    case = small
    _, j, _ = _coords(case)
    P = lambda y: 1.0 - 0.1 * y + 0.03 * y ** 2 - 0.002 * y ** 3 + 5e-5 * y ** 4
    dP = lambda y: -0.1 + 0.06 * y - 0.006 * y ** 2 + 2e-4 * y ** 3
    tend = _advect_species(case, P(j), rv=vel)
    want = -vel * case.desc.scalars.rdy * dP(j)
    got, ref = mass_interior(case, tend), mass_interior(case, want)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("vel", [3.0, -3.0])
def test_flux5_damps_2dx_wave_at_16_15(small, vel):
    """For q = (-1)^i the centred part vanishes and the upwind part gives a
    tendency of -(16/15) |U| rdx q: the 5th-order scheme's 2-dx damping."""
    case = small
    i, _, _ = _coords(case)
    q = np.where(i % 2 == 0, 1.0, -1.0)
    tend = _advect_species(case, q, ru=vel)
    want = -(16.0 / 15.0) * abs(vel) * case.desc.scalars.rdx * q
    got, ref = mass_interior(case, tend), mass_interior(case, want)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("vel", [0.02, -0.02])
def test_flux3_vertical_exact(small, vel):
    """module_advect_em.F:4306-4333: 3rd-order vertical flux (4-point centred,
    whose differences are the 4th-order central derivative, + a 3rd
    difference) is exact for a quadratic away from the 2nd-order faces k = 2
    and kde-1; with a linear profile every level is exact, including the
    zero-flux top and bottom faces."""
    case = small
    _, _, k = _coords(case)
    rdnw = case.fields["rdnw"]
    kd = case.kde
    # quadratic, levels 3..kde-3
    P = lambda z: 2.0 + 0.3 * z - 0.02 * z ** 2
    tend = _advect_species(case, P(k), ww=vel)
    want = -rdnw[None, :, None] * vel * (P(k + 0.5) - P(k - 0.5))
    got, ref = mass_interior(case, tend), mass_interior(case, want)
    sl = slice(2, kd - 3)
    assert np.max(np.abs(got[:, sl] - ref[:, sl])) <= 1e-12 * np.max(np.abs(ref[:, sl]))
    # linear, all levels (vflux = 0 at k = 1 and kde)
    L = lambda z: 1.0 + 0.25 * z
    tend = _advect_species(case, L(k), ww=vel)
    up = np.where(k + 1 <= kd - 1, L(k + 0.5), 0.0)
    dn = np.where(k >= 2, L(k - 0.5), 0.0)
    want = -rdnw[None, :, None] * vel * (up - dn)
    got, ref = mass_interior(case, tend), mass_interior(case, want)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


# ---------------------------------------------------------------------------
# the reference's advection fixture (top-hat feeder)
# ---------------------------------------------------------------------------
def test_feeder_tophat_pd():
    """ru = 90, dx = 1 km, dt = 5 s: one revolution of the 90-point periodic
    channel every 200 loops.  The PD limiter keeps the top-hat non-negative
    and it comes back to where it started.  The fixture refreshes its
    periodic halo only after the third RK stage, so the first two stages see
    a stale halo and mass drifts slightly (+0.05% per revolution)."""
    rows = tophat_feeder(1, nloops=2000, every=200, precision="f64")
    q = rows[:, :90]
    m0 = q[0].sum()
    x = np.arange(1, 91)
    c0 = (q[0] * x).sum() / m0
    for r in q[1:]:
        assert r.min() >= -1e-12
        assert abs(r.sum() - m0) <= 1e-2 * m0
        assert abs((r * x).sum() / r.sum() - c0) < 1.0
        assert 0.8 < r.max() < 1.2


def test_feeder_tophat_original_undershoots():
    """Without the limiter the 5th-order scheme undershoots below zero at the
    discontinuities, which is what the PD option removes."""
    rows = tophat_feeder(0, nloops=400, every=200, precision="f64")
    q = rows[:, :90]
    assert q[1:].min() < -1e-3
    pd = tophat_feeder(1, nloops=400, every=200, precision="f64")[:, :90]
    assert pd[1:].min() >= -1e-12


def test_feeder_f32_close_to_f64():
    a = tophat_feeder(1, nloops=400, every=200, precision="f32")
    b = tophat_feeder(1, nloops=400, every=200, precision="f64")
    assert serr(a, b) < 1e-5


# ---------------------------------------------------------------------------
# balance and conservation of the full large step
# ---------------------------------------------------------------------------
def test_rest_state_stays_at_rest():
    """No wind, no bubble, hypsometric_opt 1 (the re-diagnosis inverts the
    init's hydrostatic integration): u and v stay exactly 0, theta and mu do
    not move, w stays below 5 mm/s over 20 steps."""
    case = rest_case()
    od = OracleDomain(case, "f64")
    for n in range(4):
        od.step(5)
        for nm in ("u_2", "v_2"):
            assert np.max(np.abs(mass_interior(case, od.get(abi.FIELD_ID[nm])))) == 0.0
        w = od.get(abi.FIELD_ID["w_2"]).reshape(case.jde + 2 * H, case.kde, case.ide + 2 * H)
        assert np.max(np.abs(w[H:H + case.jde - 1, :, H:H + case.ide - 1])) < 5e-3
        t = mass_interior(case, od.get(abi.FIELD_ID["t_2"]))
        assert np.max(np.abs(t - mass_interior(case, case.fields["t_2"]))) < 1e-9
        mu = mass_interior(case, od.get(abi.FIELD_ID["mu_2"]), 2)
        assert np.max(np.abs(mu - mass_interior(case, case.fields["mu_2"], 2))) < 1e-9


def test_rest_state_default_hypsometric_top_adjustment():
    """With the reference's default hypsometric_opt = 2 the init leaves the
    top layer out of balance (log-form al against the linear ph integration):
    a w of O(10 m/s) appears at the lid in the first step, ten times more than
    anywhere in the lower half of the column."""
    case = rest_case(hyps=2)
    od = OracleDomain(case, "f64")
    od.step(1)
    w = od.get(abi.FIELD_ID["w_2"]).reshape(case.jde + 2 * H, case.kde, case.ide + 2 * H)
    w = w[H:H + case.jde - 1, :, H:H + case.ide - 1]
    assert np.max(np.abs(w[:, -1])) > 1.0
    assert np.max(np.abs(w[:, : case.kde // 2])) < 0.1 * np.max(np.abs(w[:, -1]))


def _column_masses(case, od):
    mub = mass_interior(case, case.fields["mub"], 2)
    mu = mass_interior(case, od.get(abi.FIELD_ID["mu_2"]), 2)
    c1h = case.fields["c1h"][:case.kde - 1]
    c2h = case.fields["c2h"][:case.kde - 1]
    dnw = case.fields["dnw"][:case.kde - 1]
    mut = mub + mu
    dry = mu.sum()
    nsp = case.desc.n_moist + case.desc.n_scalar
    sc = []
    for s in range(nsp):
        q = mass_interior(case, od.get(abi.species_id(s)))
        w = (c1h[None, :, None] * mut[:, None, :] + c2h[None, :, None]) * (-dnw)[None, :, None]
        sc.append(float((w * q).sum()))
    return dry, sc


@pytest.mark.parametrize("prec,tol", [("f64", 1e-12), ("f32", 3e-6)])
def test_dry_and_scalar_mass_conserved(small, prec, tol):
    """Flux form with periodic boundaries: sum(mu) and sum((c1 mut + c2) q dnw)
    are invariants of the large step."""
    case = small
    od = OracleDomain(case, prec)
    mub_sum = mass_interior(case, case.fields["mub"], 2).sum()
    d0, s0 = _column_masses(case, od)
    od.step(4)
    d1, s1 = _column_masses(case, od)
    assert abs(d1 - d0) <= tol * (mub_sum + abs(d0))
    for a, b in zip(s0, s1):
        assert abs(b - a) <= 10 * tol * abs(a)


def test_pd_scalars_stay_nonnegative(small):
    """Positive definite up to round-off: the limiter's eps and the final
    mass-weighted update can leave negatives of a few ulp of the field."""
    case = small
    od = OracleDomain(case, "f32")
    for _ in range(3):
        od.step(2)
        for s in range(1 + case.desc.n_scalar):
            q = mass_interior(case, od.get(abi.species_id(s)))
            assert q.min() >= -1e-7 * q.max()


def test_tiling_does_not_change_bits(small):
    a = OracleDomain(small, "f32", nthreads=1)
    b = OracleDomain(small, "f32", nthreads=4)
    a.step(2)
    b.step(2)
    for nm in ("u_2", "v_2", "w_2", "t_2", "ph_2", "mu_2", "p", "al"):
        fid = abi.FIELD_ID[nm]
        assert np.array_equal(a.get(fid), b.get(fid)), nm


def test_f32_tracks_f64():
    """The FP32 restatement against the FP64 one: small after 1 step and
    growing without a jump over 20 steps."""
    case = cases.config1()
    a = OracleDomain(case, "f32", nthreads=4)
    b = OracleDomain(case, "f64", nthreads=4)
    prev = 0.0
    for n in (1, 4, 15):
        a.step(n)
        b.step(n)
        e = max(serr(mass_interior(case, a.get(abi.FIELD_ID[nm])), mass_interior(case, b.get(abi.FIELD_ID[nm])))
                for nm in ("u_2", "v_2", "t_2", "ph_2"))
        assert e < 1e-3
        assert e >= 0.2 * prev
        prev = e


# ---------------------------------------------------------------------------
# sixth-order numerical diffusion (diff_6th_opt)
# ---------------------------------------------------------------------------
def _theta_wave_case(opt, amp=0.5):
    """The rest state plus a 2 dx wave of theta along x (12 columns, periodic)."""
    case = rest_case()
    F = case.fields
    ni = F["t_2"].shape[-1]
    wave = (amp * (-1.0) ** np.arange(ni)).astype(F["t_2"].dtype)
    for nm in ("t_1", "t_2"):
        F[nm][...] = F[nm] + wave
    c = case.desc.config
    c.diff_6th_opt = opt
    c.diff_6th_factor = 0.12
    c.moist_mix6_off = 1
    c.scalar_mix6_off = 1
    return case


@pytest.mark.parametrize("opt", [1, 2])
def test_sixth_order_diffusion_damps_2dx_wave(opt):
    """For a 2 dx wave of amplitude A the sixth-order flux is +-32 A at every
    face (module_big_step_utilities_em.F:6455-6461) and runs down-gradient
    (diff_6th_opt = 2 keeps it), so the stage-1 tendency is
    -(diff_6th_factor / (2 dt)) (c1 mut + c2) A and one large step scales the
    wave by 1 - diff_6th_factor / 2 relative to the undiffused step."""
    amp = {}
    for o in (0, opt):
        case = _theta_wave_case(o)
        od = OracleDomain(case, "f64")
        od.step(1)
        t = mass_interior(case, od.get(abi.FIELD_ID["t_2"]))
        sign = (-1.0) ** np.arange(t.shape[-1])
        amp[o] = abs(float(np.mean(t * sign)))
    assert amp[0] > 0.45
    assert abs(amp[opt] / amp[0] - (1.0 - 0.12 / 2)) < 0.01


@pytest.mark.parametrize("adv", [0, 1])
def test_sixth_order_diffusion_damps_2dx_wave_of_qv(adv):
    """The species' diffusion is formed at stage 1 with the stage's dt (dt / 3,
    module_em.F:1421-1435) and muts, and added at every stage (the
    positive-definite form spends it in the last stage's pre-update), so a
    2 dx wave of qv loses about 3 diff_6th_factor / 2 of its amplitude in one
    step relative to the undiffused step."""
    amp = {}
    for mix_off in (1, 0):
        case = _theta_wave_case(1, amp=0.0)
        cur, old = case.species[0]
        fac = 1.0 + 0.2 * (-1.0) ** np.arange(cur.shape[-1])
        cur[...] = cur * fac
        old[...] = old * fac
        c = case.desc.config
        c.moist_adv_opt = adv
        c.moist_mix6_off = mix_off
        od = OracleDomain(case, "f64")
        od.step(1)
        qv = mass_interior(case, od.get(abi.species_id(0)))
        sign = (-1.0) ** np.arange(qv.shape[-1])
        amp[mix_off] = abs(float(np.mean(qv * sign)))
    assert amp[1] > 0
    assert abs(amp[0] / amp[1] - (1.0 - 1.5 * 0.12)) < 0.02


def test_rayleigh_damping_relaxes_top_layer():
    """damp_opt = 2 (module_big_step_utilities_em.F:5836-6110): the Rayleigh
    relaxation toward the base state lowers the rms w of the top 5 km (where
    the initial state's lid adjustment lives) and leaves the lower levels as
    they were after 3 steps; dampcoef 0.01 s-1 keeps the explicit term
    stable at dt = 12 s."""
    from wrf_gb300 import abi

    def run(damp):
        c = cases.small_case(nx=16, ny=12, kde=20, n_scalar=1, seed=19)
        if damp:
            c.desc.config.damp_opt = 2
            c.desc.config.dampcoef = 0.01
            c.desc.config.zdamp = 5000.0
        od = OracleDomain(c, "f32")
        od.step(3)
        w = interior(c, abi.FIELD_ID["w_2"], od.get(abi.FIELD_ID["w_2"]))
        return float(np.sqrt(np.mean(w[:, -6:, :] ** 2))), float(np.sqrt(np.mean(w[:, :8, :] ** 2)))

    top0, low0 = run(False)
    top1, low1 = run(True)
    assert top1 < 0.97 * top0, (top0, top1)
    assert abs(low1 - low0) <= 1e-3 * low0, (low0, low1)


def _level_deviation_rms(c, od, name):
    """rms over the interior of a field's deviation from its level means."""
    x = interior(c, abi.FIELD_ID[name], od.get(abi.FIELD_ID[name]))
    return float(np.sqrt(np.mean((x - x.mean(axis=(0, 2), keepdims=True)) ** 2)))


def test_explicit_diffusion_smooths_the_bubble():
    """diff_opt = 1, km_opt = 1 (module_em.F:801-877 and 1378-1419): constant
    khdif / kvdif diffusion lowers the horizontal deviation of theta and of
    the species from their level means after 3 steps, against the same run
    without it; with khdif = kvdif = 0 the step equals the undiffused one
    bit for bit (the tendencies are exact zeros added)."""
    def run(khdif, kvdif, on=True):
        c = cases.small_case(nx=16, ny=12, kde=16, n_scalar=1, seed=23)
        if on:
            c.desc.config.diff_opt = 1
            c.desc.config.km_opt = 1
            c.desc.config.khdif = khdif
            c.desc.config.kvdif = kvdif
        od = OracleDomain(c, "f32")
        od.step(3)
        return c, od

    c0, od0 = run(0.0, 0.0, on=False)
    c1, od1 = run(2000.0, 50.0)
    t0, t1 = _level_deviation_rms(c0, od0, "t_2"), _level_deviation_rms(c1, od1, "t_2")
    assert t1 < 0.98 * t0, (t0, t1)
    q0 = interior(c0, abi.species_id(1), od0.get(abi.species_id(1)))
    q1 = interior(c1, abi.species_id(1), od1.get(abi.species_id(1)))
    assert np.std(q1) < np.std(q0), (np.std(q0), np.std(q1))
    cz, odz = run(0.0, 0.0)
    for name in ("u_2", "v_2", "w_2", "t_2", "ph_2"):
        a = od0.get(abi.FIELD_ID[name]); b = odz.get(abi.FIELD_ID[name])
        assert np.array_equal(np.asarray(a), np.asarray(b)), name


def test_explicit_diffusion_of_uniform_fields_is_zero():
    """horizontal_diffusion 'm' / vertical_diffusion 'm' of a species that is
    uniform in x, y and k add exactly zero (every difference is 0)."""
    c = cases.small_case(nx=12, ny=10, kde=12, n_scalar=1, seed=5)
    c.desc.config.diff_opt = 1
    c.desc.config.km_opt = 1
    c.desc.config.khdif = 500.0
    c.desc.config.kvdif = 20.0
    od = OracleDomain(c, "f32")
    od.set(abi.FIELD_ID["muts"], np.asarray(od.get(abi.FIELD_ID["mub"])))  # a column mass, as after a stage
    q = np.asarray(od.get(abi.species_id(1)))
    od.set(abi.species_id(1), np.full_like(q, 1e-3))
    fid = abi.FIELD_ID["h_diabatic"]
    z = np.zeros_like(np.asarray(od.get(fid)))
    od.set(fid, z)
    od.run("sixth_diff_species", 1, 0, 1)
    got = interior(c, fid, od.get(fid))[:, :-1, :]  # mass levels 1..kde-1
    assert np.all(got == 0.0), np.abs(got).max()


# ---------------------------------------------------------------------------
# open lateral boundaries (em_quarter_ss: open_xs/xe/ys/ye)
# ---------------------------------------------------------------------------
OPEN_SIDES = [(True, True), (True, False), (False, True)]


@pytest.mark.parametrize("x,y", OPEN_SIDES)
def test_open_boundaries_tiling_does_not_change_bits(x, y):
    """The degrade flags and the radiation rows depend on the tile's own
    bounds (module_advect_em.F:500-516, its/jts against ids/jds); j-slab tiles
    must reproduce the one-tile result bit for bit."""
    case = cases.open_boundaries(cases.small_case(nx=20, ny=18, kde=12, n_scalar=2, seed=12), x=x, y=y)
    a = OracleDomain(case, "f32", nthreads=1)
    b = OracleDomain(case, "f32", nthreads=4)
    a.step(3)
    b.step(3)
    for nm in ("u_2", "v_2", "w_2", "t_2", "ph_2", "mu_2", "p", "al"):
        fid = abi.FIELD_ID[nm]
        va = a.get(fid)
        assert np.all(np.isfinite(va)), nm
        assert np.array_equal(va, b.get(fid)), nm
    for s in range(3):
        assert np.array_equal(a.get(abi.species_id(s)), b.get(abi.species_id(s)))


@pytest.mark.parametrize("x,y", OPEN_SIDES)
def test_open_boundaries_with_diffusion_tiling_does_not_change_bits(x, y):
    """Explicit and sixth-order diffusion with open boundaries: the loop
    limits of each diffusion term depend on the tile's own bounds; j-slab
    tiles reproduce the one-tile bits."""
    case = cases.open_boundaries(cases.small_case(nx=22, ny=20, kde=12, n_scalar=1, seed=13), x=x, y=y)
    c = case.desc.config
    c.diff_6th_opt = 2
    c.diff_6th_factor = 0.12
    c.diff_opt = 1
    c.km_opt = 1
    c.khdif = 300.0
    c.kvdif = 10.0
    a = OracleDomain(case, "f32", nthreads=1)
    b = OracleDomain(case, "f32", nthreads=4)
    a.step(2)
    b.step(2)
    for nm in ("u_2", "v_2", "w_2", "t_2", "ph_2", "mu_2"):
        fid = abi.FIELD_ID[nm]
        va = a.get(fid)
        assert np.all(np.isfinite(va)), nm
        assert np.array_equal(va, b.get(fid)), nm


def test_open_boundaries_rest_state_stays_at_rest():
    """At rest every radiation term multiplies a zero difference and every
    degraded flux is zero: the open domain stays at rest like the periodic
    one."""
    case = cases.open_boundaries(rest_case())
    od = OracleDomain(case, "f64")
    for n in range(2):
        od.step(5)
        for nm in ("u_2", "v_2"):
            assert np.max(np.abs(mass_interior(case, od.get(abi.FIELD_ID[nm])))) == 0.0
        t = mass_interior(case, od.get(abi.FIELD_ID["t_2"]))
        assert np.max(np.abs(t - mass_interior(case, case.fields["t_2"]))) < 1e-9
        mu = mass_interior(case, od.get(abi.FIELD_ID["mu_2"]), 2)
        assert np.max(np.abs(mu - mass_interior(case, case.fields["mu_2"], 2))) < 1e-9


@pytest.mark.parametrize("x,y", OPEN_SIDES)
def test_open_boundaries_keep_a_uniform_flow_uniform(x, y):
    """A balanced state (hypsometric_opt 1) moving with a uniform wind
    (u = 10, v = -5 m/s at every level): the degraded stencils next to the
    open edges and the radiation terms see no horizontal gradient, so every
    column stays equal to the others up to rounding (the 3rd- and 5th-order
    faces of a uniform field differ in the last bit, and the acoustic steps
    carry that difference into the domain: about 1e-10 of each field after
    four steps).  (A sheared flow with
    vertical motion would not: next to open_ys / open_ye the reference leaves
    u's vertical advection out at i = ids, ide, module_advect_em.F:1350-1351,
    and curvature leaves the boundary u out, :4292-4295.)"""
    base = rest_case(kde=14)
    base.fields["u_1"][:] = 10.0
    base.fields["u_2"][:] = 10.0
    base.fields["v_1"][:] = -5.0
    base.fields["v_2"][:] = -5.0
    case = cases.open_boundaries(base, x=x, y=y)
    od = OracleDomain(case, "f64")
    od.step(4)
    for nm, tol in (("u_2", 1e-8), ("v_2", 1e-8), ("t_2", 1e-8), ("ph_2", 1e-6), ("p", 1e-6)):
        a = mass_interior(case, od.get(abi.FIELD_ID[nm]))
        ref = a[:1, :, :1]
        scale = max(np.max(np.abs(a)), 1.0)
        assert np.max(np.abs(a - ref)) <= tol * scale, (nm, np.max(np.abs(a - ref)) / scale)
    q = mass_interior(case, od.get(abi.species_id(0)))
    assert np.max(np.abs(q - q[:1, :, :1])) <= 1e-8 * np.max(np.abs(q))


def _advect_open(case, q, scheme, ru=0.0, rv=0.0):
    od = OracleDomain(case, "f64")
    shp = (case.jde + 2 * H, case.kde, case.ide + 2 * H)
    od.set(abi.FIELD_ID["ru_m"], np.full(shp, ru))
    od.set(abi.FIELD_ID["rv_m"], np.full(shp, rv))
    od.set(abi.FIELD_ID["ww_m"], np.zeros(shp))
    od.set(abi.FIELD_ID["muts"], case.fields["mub"] + case.fields["mu_1"])
    od.set(abi.species_id(0), q)
    od.set(abi.species_id(0, True), q)
    od.run(scheme, 3, 0, 0)
    return od.get(abi.FIELD_ID["advect_tend"]).reshape(shp)


@pytest.mark.parametrize("scheme", ["advect_scalar", "advect_scalar_pd"])
@pytest.mark.parametrize("axis", ["x", "y"])
@pytest.mark.parametrize("vel", [7.5, -7.5])
def test_open_boundary_fluxes_exact_on_linear_fields(scheme, axis, vel):
    """Next to an open boundary the reference degrades the face fluxes to
    3rd and 2nd order (module_advect_em.F:3554-3632, PD :6560-6779) and the
    boundary cell takes the radiation term instead (:4104-4175, PD
    :7254-7328).  Every one of those fluxes is exact for a linear field, and
    the radiation term gives the upwind difference at an outflow boundary and
    nothing at an inflow one: so with a uniform wind every cell has the
    tendency -U rdx dq, except the inflow boundary cell, which has 0."""
    case = cases.open_boundaries(cases.small_case(nx=14, ny=12, kde=10, n_scalar=0, seed=3),
                                 x=axis == "x", y=axis == "y")
    i, j, _ = _coords(case)
    c = i if axis == "x" else j
    b = 0.02
    q = 1.0 + b * c
    tend = _advect_open(case, q, scheme, ru=vel if axis == "x" else 0.0, rv=vel if axis == "y" else 0.0)
    rd = case.desc.scalars.rdx if axis == "x" else case.desc.scalars.rdy
    got = mass_interior(case, tend)
    want = np.full(got.shape, -vel * rd * b)
    inflow = 0 if vel > 0 else -1
    if axis == "x":
        want[:, :, inflow] = 0.0
    else:
        want[inflow, :, :] = 0.0
    assert np.max(np.abs(got - want)) <= 1e-12 * abs(vel * rd * b), np.max(np.abs(got - want))
