"""Seeded synthetic initial states for the benchmark workloads.

The initial state of an idealised WRF-ARW run is produced by the reference's
dyn_em/module_initialize_ideal.F (init_domain_rk) followed by
dyn_em/start_em.F.  This module restates that arithmetic in numpy (float64)
for the physics-off configurations the bench and tests use:

* vertical coordinate: uniform eta levels (module_initialize_ideal.F:626) and
  the derived 1-D metrics dnw, rdnw, znu, dn, rdn, fnm, fnp, cf1..cf3, cfn,
  cfn1 (:697-731); hybrid_opt = 0 coefficients c1..c4 (:786-880);
* base state mub, pb, t_init, alb, phb by hydrostatic integration of a dry
  sounding (:963-985);
* full state mu_1, qv, t_1, p, alt, al, ph_1 from the moist sounding
  (:991-1060), warm bubbles of cos^2 shape (:1089-1133), conversion to moist
  potential temperature (:1726-1733), and start_em's rediagnosis of al, p,
  alt (start_em.F:790-841, hypsometric_opt = 2).

The sounding is the analytic Weisman-Klemp (1982) profile (theta_0 = 300 K,
tropopause 12 km / 343 K / 213 K, surface qv capped at 14 g/kg) with a
quarter-circle hodograph; random draws use numpy Generator(PCG64(seed)).
Arrays are returned in the Fortran memory layout (i fastest), shaped
(jme-jms+1, kme-kms+1, ime-ims+1), halos filled as the reference's periodic
or symmetric boundary fills would leave them.
"""
import math
import numpy as np

from . import abi

G = 9.81
R_D = 287.0
CP = 7.0 * R_D / 2.0
R_V = 461.6
CV = CP - R_D
CVPM = -CV / CP
P1000 = 1.0e5
T0 = 300.0
CPOVCV = CP / (CP - R_D)
RVOVRD = R_V / R_D


class Case:
    """An initial state: domain description plus named float64 fields."""

    def __init__(self, name, desc, fields, species, meta):
        self.name = name
        self.desc = desc
        self.fields = fields          # name -> ndarray (memory layout)
        self.species = species        # list of (current, old) ndarrays
        self.meta = meta

    @property
    def ide(self):
        return self.desc.ide

    @property
    def jde(self):
        return self.desc.jde

    @property
    def kde(self):
        return self.desc.kde

    def cells(self):
        """Mass cells (ide-1)(jde-1)(kde-1)."""
        return (self.ide - 1) * (self.jde - 1) * (self.kde - 1)

    def field_items(self):
        """(field id, array) for every input field, species included."""
        for name, arr in self.fields.items():
            yield abi.FIELD_ID[name], arr
        for s, (cur, old) in enumerate(self.species):
            yield abi.species_id(s), cur
            yield abi.species_id(s, old=True), old


# ---------------------------------------------------------------------------
# sounding
# ---------------------------------------------------------------------------
def _qvs(p, t):
    es = 611.2 * np.exp(17.67 * (t - 273.15) / (t - 29.65))
    return 0.622 * es / np.maximum(p - es, 1.0)


def wk_sounding(ztop, theta0=300.0, z_tr=12000.0, theta_tr=343.0, t_tr=213.0,
                qv0=0.014, hodo_radius=15.0, dz=20.0, dry=False):
    """Weisman-Klemp (1982) analytic sounding on a fine height grid.

    Returns heights, full pressure, dry pressure, theta, qv, u, v.
    """
    z = np.arange(0.0, ztop + 4000.0 + dz, dz)
    theta = np.where(z <= z_tr, theta0 + (theta_tr - theta0) * (z / z_tr) ** 1.25,
                     theta_tr * np.exp(G / (CP * t_tr) * (z - z_tr)))
    rh = np.where(z <= z_tr, 1.0 - 0.75 * (z / z_tr) ** 1.25, 0.25)
    qv = np.zeros_like(z)
    p = np.zeros_like(z)
    for _ in range(4):
        pi = np.empty_like(z)
        pi[0] = 1.0
        thv = theta * (1.0 + 0.61 * qv)
        for k in range(1, len(z)):
            pi[k] = pi[k - 1] - G * dz / (CP * 0.5 * (thv[k] + thv[k - 1]))
        p = P1000 * pi ** (CP / R_D)
        if dry:
            break
        t = theta * pi
        qv = np.minimum(rh * _qvs(p, t), qv0)
    # dry-air pressure: integrate the dry-air density down from the top
    t = theta * (p / P1000) ** (R_D / CP)
    rho = p / (R_D * t * (1.0 + 0.61 * qv))
    rho_d = rho / (1.0 + qv)
    pd = np.empty_like(z)
    pd[-1] = p[-1] / (1.0 + qv[-1] * RVOVRD)
    for k in range(len(z) - 2, -1, -1):
        pd[k] = pd[k + 1] + G * dz * 0.5 * (rho_d[k] + rho_d[k + 1])
    # quarter-circle hodograph below 2 km, then straight to 6 km
    zh = np.minimum(z, 2000.0) / 2000.0 * (0.5 * math.pi)
    u = hodo_radius * (1.0 - np.cos(zh)) + np.clip(z - 2000.0, 0.0, 4000.0) / 4000.0 * hodo_radius
    v = hodo_radius * np.sin(zh)
    u = u - 0.5 * hodo_radius
    v = v - 0.5 * hodo_radius
    return z, p, pd, theta, qv, u, v


# ---------------------------------------------------------------------------
# vertical coordinate
# ---------------------------------------------------------------------------
def eta_metrics(kde):
    k = np.arange(1, kde + 1, dtype=np.float64)
    znw = 1.0 - (k - 1.0) / (kde - 1.0)
    n = kde + 1  # 1-based storage, index 0 unused
    dnw = np.zeros(n); rdnw = np.zeros(n); znu = np.zeros(n)
    dn = np.zeros(n); rdn = np.zeros(n); fnp = np.zeros(n); fnm = np.zeros(n)
    zw = np.zeros(n); zw[1:] = znw
    for kk in range(1, kde):
        dnw[kk] = zw[kk + 1] - zw[kk]
        rdnw[kk] = 1.0 / dnw[kk]
        znu[kk] = 0.5 * (zw[kk + 1] + zw[kk])
    for kk in range(2, kde):
        dn[kk] = 0.5 * (dnw[kk] + dnw[kk - 1])
        rdn[kk] = 1.0 / dn[kk]
        fnp[kk] = 0.5 * dnw[kk] / dn[kk]
        fnm[kk] = 0.5 * dnw[kk - 1] / dn[kk]
    cof1 = (2.0 * dn[2] + dn[3]) / (dn[2] + dn[3]) * dnw[1] / dn[2]
    cof2 = dn[2] / (dn[2] + dn[3]) * dnw[1] / dn[3]
    cf1 = fnp[2] + cof1
    cf2 = fnm[2] - cof1 - cof2
    cf3 = cof2
    cfn = (0.5 * dnw[kde - 1] + dn[kde - 1]) / dn[kde - 1]
    cfn1 = -0.5 * dnw[kde - 1] / dn[kde - 1]
    return dict(znw=zw, dnw=dnw, rdnw=rdnw, znu=znu, dn=dn, rdn=rdn, fnp=fnp, fnm=fnm,
                cf1=cf1, cf2=cf2, cf3=cf3, cfn=cfn, cfn1=cfn1)


def hybrid_coefs(m, kde, p_top):
    """hybrid_opt = 0 (module_initialize_ideal.F:786-880)."""
    n = kde + 1
    c3f = m["znw"].copy()
    c4f = np.zeros(n); c3h = np.zeros(n); c4h = np.zeros(n)
    c1f = np.zeros(n); c2f = np.zeros(n); c1h = np.zeros(n); c2h = np.zeros(n)
    for k in range(1, kde + 1):
        c4f[k] = (m["znw"][k] - c3f[k]) * (P1000 - p_top)
    for k in range(1, kde):
        c3h[k] = (c3f[k + 1] + c3f[k]) * 0.5
        c4h[k] = (m["znu"][k] - c3h[k]) * (P1000 - p_top)
    for k in range(2, kde):
        c1f[k] = (c3h[k] - c3h[k - 1]) / (m["znu"][k] - m["znu"][k - 1])
    c1f[1] = 1.0
    c1f[kde] = 1.0
    for k in range(1, kde + 1):
        c2f[k] = (1.0 - c1f[k]) * (P1000 - p_top)
    for k in range(1, kde):
        c1h[k] = (c3f[k + 1] - c3f[k]) / (m["znw"][k + 1] - m["znw"][k])
        c2h[k] = (1.0 - c1h[k]) * (P1000 - p_top)
    return dict(c1h=c1h, c2h=c2h, c1f=c1f, c2f=c2f, c3h=c3h, c4h=c4h, c3f=c3f, c4f=c4f)


# ---------------------------------------------------------------------------
# halo fills in numpy (initial state only; the solver does its own)
# ---------------------------------------------------------------------------
def _src_index(n_mem_lo, n_mem_hi, nper, periodic, sym_stag, stag):
    """Source index for every memory index in [lo, hi] (1-based domain)."""
    idx = np.arange(n_mem_lo, n_mem_hi + 1)
    if periodic:
        return (idx - 1) % nper + 1
    # symmetric: mass points mirror about 0.5 / ide-0.5; staggered about 1 / ide
    out = idx.copy()
    if not stag:
        out = np.where(idx < 1, 1 - idx, out)
        out = np.where(idx > nper, 2 * nper + 1 - idx, out)
    else:
        out = np.where(idx < 1, 2 - idx, out)
        out = np.where(idx > nper + 1, 2 * (nper + 1) - idx, out)
    return out


def fill_halo(arr, kind, stag, ide, jde, cfg):
    """Periodic / symmetric image of the interior in the memory halo."""
    h = abi.HALO
    nx, ny = ide - 1, jde - 1
    ix = _src_index(1 - h, ide + h, nx, bool(cfg.periodic_x), 0, stag == "u") + h - 1
    jy = _src_index(1 - h, jde + h, ny, bool(cfg.periodic_y), 0, stag == "v") + h - 1
    sign_y = np.ones(len(jy))
    if not cfg.periodic_y and stag == "v":
        j = np.arange(1 - h, jde + h + 1)
        sign_y = np.where((j < 1) | (j > jde), -1.0, 1.0)
    if kind == 3:
        out = arr[:, :, ix][jy, :, :]
        return out * sign_y[:, None, None]
    out = arr[:, ix][jy, :]
    return out * sign_y[:, None]


def _column_p_al(t1, qv3, mu1_2d, mub, pb, alb, c1f, c2f, rdnw, rdn, kde):
    """module_initialize_ideal.F:1035-1060: p, alt, al by downward integration
    of every column (arrays (j, k, i); mub a scalar or an (j, i) array)."""
    p = np.zeros_like(t1); alt = np.zeros_like(t1); al = np.zeros_like(t1)
    kk = kde - 1; k = kk + 1
    qvf1 = 0.5 * (qv3[:, kk - 1] + qv3[:, kk - 1]); qvf2 = 1.0 / (1.0 + qvf1); qvf1 = qvf1 * qvf2
    p[:, kk - 1] = -0.5 * ((c1f[k] * mu1_2d) + qvf1 * (c1f[k] * mub + c2f[k])) / rdnw[kk] / qvf2
    qvf = 1.0 + RVOVRD * qv3[:, kk - 1]
    alt[:, kk - 1] = (R_D / P1000) * (t1[:, kk - 1] + T0) * qvf * (((p[:, kk - 1] + pb[kk]) / P1000) ** CVPM)
    al[:, kk - 1] = alt[:, kk - 1] - alb[kk]
    for kk in range(kde - 2, 0, -1):
        k = kk + 1
        qvf1 = 0.5 * (qv3[:, kk - 1] + qv3[:, kk]); qvf2 = 1.0 / (1.0 + qvf1); qvf1 = qvf1 * qvf2
        p[:, kk - 1] = p[:, kk] - ((c1f[k] * mu1_2d) + qvf1 * (c1f[k] * mub + c2f[k])) / qvf2 / rdn[kk + 1]
        qvf = 1.0 + RVOVRD * qv3[:, kk - 1]
        alt[:, kk - 1] = (R_D / P1000) * (t1[:, kk - 1] + T0) * qvf * (((p[:, kk - 1] + pb[kk]) / P1000) ** CVPM)
        al[:, kk - 1] = alt[:, kk - 1] - alb[kk]
    return p, alt, al


def _column_ph(al, mu1_2d, mub, alb, c1h, c2h, dnw, kde, ni):
    """module_initialize_ideal.F:1063-1075: perturbation geopotential by
    upward integration of every column."""
    nj = al.shape[0]
    ph = np.zeros((nj, kde, ni))
    for kk in range(2, kde + 1):
        k = kk - 1
        ph[:, kk - 1] = ph[:, kk - 2] - dnw[kk - 1] * (((c1h[k] * mub + c2h[k]) + (c1h[k] * mu1_2d)) * al[:, kk - 2]
                                                      + (c1h[k] * mu1_2d) * alb[kk - 1])
    return ph


# ---------------------------------------------------------------------------
# ideal supercell-type state
# ---------------------------------------------------------------------------
def _interp(x, xp, fp):
    """Linear interpolation for a monotonic table (increasing or decreasing)."""
    if xp[0] > xp[-1]:
        return np.interp(x, xp[::-1], fp[::-1])
    return np.interp(x, xp, fp)


def supercell_state(nx, ny, kde, dx, dt, ztop, bubbles, rng, n_scalar=0,
                    scalar_median=1.0e-6, scalar_sigma=1.0, noise=0.01,
                    hodo_radius=15.0, name="supercell", hypsometric_opt=2):
    """Weisman-Klemp sounding + cos^2 warm bubbles, doubly periodic.

    bubbles: list of (xc [m], yc [m], zc [m], rx [m], ry [m], rz [m], dtheta [K]).
    hypsometric_opt 2 (the reference's default) re-diagnoses al from ph with
    the log form after the linear hydrostatic integration of the init, which
    leaves the top layers slightly out of balance; with 1 the re-diagnosis
    inverts the integration, so a windless, bubble-free state is at rest.
    """
    ide, jde = nx + 1, ny + 1
    cfg = abi.default_config(periodic_x=True, periodic_y=True)
    cfg.hypsometric_opt = hypsometric_opt
    h = abi.HALO
    nim, njm, nk = ide + 2 * h, jde + 2 * h, kde
    m = eta_metrics(kde)
    zd, pdry, _, thd, _, _, _ = wk_sounding(ztop, hodo_radius=hodo_radius, dry=True)
    p_top = float(_interp(ztop, zd, pdry))
    hc = hybrid_coefs(m, kde, p_top)
    c1h, c2h, c1f, c2f = hc["c1h"], hc["c2h"], hc["c1f"], hc["c2f"]
    c3h, c4h, c3f, c4f = hc["c3h"], hc["c4h"], hc["c3f"], hc["c4f"]
    dnw, rdnw, rdn = m["dnw"], m["rdnw"], m["rdn"]

    # base state (horizontally uniform, flat terrain)
    p_surf = float(pdry[0])
    mub = p_surf - p_top
    pb = np.zeros(kde + 1); t_init = np.zeros(kde + 1); alb = np.zeros(kde + 1); phb = np.zeros(kde + 1)
    for k in range(1, kde):
        pl = c3h[k] * (p_surf - p_top) + c4h[k] + p_top
        pb[k] = pl
        t_init[k] = _interp(pl, pdry, thd) - T0
        alb[k] = (R_D / P1000) * (t_init[k] + T0) * (pb[k] / P1000) ** CVPM
    for kk in range(2, kde + 1):
        k = kk - 1
        phb[kk] = phb[kk - 1] - dnw[kk - 1] * (c1h[k] * mub + c2h[k]) * alb[kk - 1]

    # moist sounding and the full column (identical in every column before bubbles)
    zm, pm, pdm, thm, qvm, um, vm = wk_sounding(ztop, hodo_radius=hodo_radius)
    pd_surf = float(pdm[0])
    mu1 = pd_surf - p_top - mub
    qv = np.zeros(kde + 1); th = np.zeros(kde + 1)
    for k in range(1, kde):
        pl = c3h[k] * (pd_surf - p_top) + c4h[k] + p_top
        qv[k] = _interp(pl, pdm, qvm)
        th[k] = _interp(pl, pdm, thm) - T0
    zhalf = np.array([0.5 * (phb[k] + phb[k + 1]) / G if 1 <= k < kde else 0.0 for k in range(kde + 1)])
    u_col = np.zeros(kde + 1); v_col = np.zeros(kde + 1)
    for k in range(1, kde):
        u_col[k] = _interp(zhalf[k], zm, um)
        v_col[k] = _interp(zhalf[k], zm, vm)

    # 3-D arrays on the interior (j, k, i) with 1-based k -> index k-1
    ni, nj, nkm = nx, ny, kde - 1
    t1 = np.broadcast_to(th[1:kde][None, :, None], (nj, nkm, ni)).copy()
    qv3 = np.broadcast_to(qv[1:kde][None, :, None], (nj, nkm, ni)).copy()
    mu1_2d = np.full((nj, ni), mu1)

    def column_p_al(t1, qv3, mu1_2d):
        return _column_p_al(t1, qv3, mu1_2d, mub, pb, alb, c1f, c2f, rdnw, rdn, kde)

    def column_ph(al, mu1_2d):
        return _column_ph(al, mu1_2d, mub, alb, c1h, c2h, dnw, kde, ni)

    p3, alt3, al3 = column_p_al(t1, qv3, mu1_2d)
    ph1 = column_ph(al3, mu1_2d)
    # bubbles (module_initialize_ideal.F:1089-1133 form)
    xi = (np.arange(1, ni + 1) - 0.5) * dx
    yj = (np.arange(1, nj + 1) - 0.5) * dx
    zmass = 0.5 * (ph1[:, :-1] + ph1[:, 1:] + (phb[1:kde] + phb[2:kde + 1])[None, :, None]) / G
    for (xc, yc, zc, rx, ry, rz, dth) in bubbles:
        xr = (xi - xc) / rx
        yr = (yj - yc) / ry
        # only the columns within the bubble's horizontal radius change
        iw = np.nonzero(np.abs(xr) <= 1.0)[0]
        jw = np.nonzero(np.abs(yr) <= 1.0)[0]
        if iw.size == 0 or jw.size == 0:
            continue
        i0, i1, j0, j1 = iw[0], iw[-1] + 1, jw[0], jw[-1] + 1
        rad = np.sqrt(xr[None, None, i0:i1] ** 2 + yr[j0:j1, None, None] ** 2 +
                      ((zmass[j0:j1, :, i0:i1] - zc) / rz) ** 2)
        t1[j0:j1, :, i0:i1] = t1[j0:j1, :, i0:i1] + np.where(rad <= 1.0, dth * np.cos(0.5 * math.pi * rad) ** 2, 0.0)
    if noise > 0:
        t1 = t1 + rng.uniform(-noise, noise, size=t1.shape)
    p3, alt3, al3 = column_p_al(t1, qv3, mu1_2d)
    ph1 = column_ph(al3, mu1_2d)
    # theta -> moist theta (module_initialize_ideal.F:1726-1733)
    tm = (t1 + T0) * (1.0 + (R_V / R_D) * qv3) - T0
    # start_em.F:790-841: al from ph (hypsometric_opt 1 or 2), p from the EOS
    mut = mub + mu1_2d
    al3 = np.zeros_like(tm)
    for k in range(1, kde):
        if hypsometric_opt == 1:
            al3[:, k - 1] = -1.0 / ((c1h[k] * mub + c2h[k]) + c1h[k] * mu1_2d) * (
                alb[k] * (c1h[k] * mu1_2d) + rdnw[k] * (ph1[:, k] - ph1[:, k - 1]))
            continue
        pfu = c3f[k + 1] * mut + c4f[k + 1] + p_top
        pfd = c3f[k] * mut + c4f[k] + p_top
        phm = c3h[k] * mut + c4h[k] + p_top
        al3[:, k - 1] = (ph1[:, k] - ph1[:, k - 1] + phb[k + 1] - phb[k]) / phm / np.log(pfd / pfu) - alb[k]
    p3 = P1000 * ((R_D * (T0 + tm)) / (P1000 * (al3 + alb[1:kde][None, :, None]))) ** CPOVCV - pb[1:kde][None, :, None]
    alt3 = al3 + alb[1:kde][None, :, None]

    # assemble memory-layout arrays
    def mem3(interior, nkk, stag=None):
        a = np.zeros((njm, nk, nim))
        a[h:h + interior.shape[0], :nkk, h:h + interior.shape[2]] = interior
        if stag == "u":
            a[h:h + interior.shape[0], :nkk, h + nx] = interior[:, :, 0]
        if stag == "v":
            a[h + ny, :nkk, h:h + interior.shape[2]] = interior[0, :, :]
        return fill_halo(a, 3, stag, ide, jde, cfg)

    def mem2(interior):
        a = np.zeros((njm, nim))
        a[h:h + nj, h:h + ni] = interior
        return fill_halo(a, 2, None, ide, jde, cfg)

    def col(v1d, nkk):
        return np.broadcast_to(v1d[1:nkk + 1][None, :, None], (nj, nkk, ni))

    f = {}
    f["u_1"] = mem3(np.broadcast_to(u_col[1:kde][None, :, None], (nj, nkm, ni)), nkm, "u")
    f["v_1"] = mem3(np.broadcast_to(v_col[1:kde][None, :, None], (nj, nkm, ni)), nkm, "v")
    f["u_2"] = f["u_1"].copy(); f["v_2"] = f["v_1"].copy()
    f["w_1"] = np.zeros((njm, nk, nim)); f["w_2"] = np.zeros((njm, nk, nim))
    f["t_1"] = mem3(tm, nkm); f["t_2"] = f["t_1"].copy()
    f["ph_1"] = mem3(ph1, kde); f["ph_2"] = f["ph_1"].copy()
    f["phb"] = mem3(col(phb, kde), kde)
    f["pb"] = mem3(col(pb, nkm), nkm)
    f["alb"] = mem3(col(alb, nkm), nkm)
    f["p"] = mem3(p3, nkm)
    f["al"] = mem3(al3, nkm)
    f["alt"] = mem3(alt3, nkm)
    f["mu_1"] = mem2(mu1_2d); f["mu_2"] = f["mu_1"].copy()
    f["mub"] = mem2(np.full((nj, ni), mub))
    for nm in ("msfux", "msfuy", "msfvx", "msfvx_inv", "msfvy", "msftx", "msfty", "cosa"):
        f[nm] = np.ones((njm, nim))
    for nm in ("ht", "f", "e", "sina"):
        f[nm] = np.zeros((njm, nim))
    for nm in ("znw", "znu", "dnw", "rdnw", "dn", "rdn", "fnm", "fnp"):
        f[nm] = m[nm][1:].copy()
    for nm in ("c1h", "c2h", "c1f", "c2f", "c3h", "c4h", "c3f", "c4f"):
        f[nm] = hc[nm][1:].copy()

    _base_profiles(f, t1, qv3, ph1, phb, kde)
    f["t_init"] = mem3(col(t_init, nkm), nkm)
    species = []
    qv_mem = mem3(qv3, nkm)
    species.append((qv_mem, qv_mem.copy()))
    for _ in range(n_scalar):
        qs = scalar_median * np.exp(scalar_sigma * rng.standard_normal(size=(nj, nkm, ni)))
        qm = mem3(qs, nkm)
        species.append((qm, qm.copy()))

    desc = _make_desc(ide, jde, kde, n_scalar, cfg, dt, dx, m, p_top)
    meta = dict(dx=dx, dt=dt, ztop=ztop, bubbles=bubbles, n_scalar=n_scalar)
    return Case(name, desc, f, species, meta)


def _column_sounding(z, theta, rh, dz, p_surf=P1000):
    """Hydrostatic moist sounding on the height grid z (spacing dz) for a
    potential-temperature profile theta and a relative-humidity profile rh:
    full pressure p (integrated up from p_surf with the virtual potential
    temperature, the water vapour iterated to the given humidity), dry-air
    pressure pd (the dry-air density integrated down from the top, as
    get_sounding_b_wave does, module_initialize_ideal.F:2072-2080) and qv."""
    qv = np.zeros_like(z)
    p = np.zeros_like(z)
    for _ in range(4):
        pi = np.empty_like(z)
        pi[0] = (p_surf / P1000) ** (R_D / CP)
        thv = theta * (1.0 + 0.61 * qv)
        for k in range(1, len(z)):
            pi[k] = pi[k - 1] - G * dz / (CP * 0.5 * (thv[k] + thv[k - 1]))
        p = P1000 * pi ** (CP / R_D)
        t = theta * pi
        qv = rh * _qvs(p, t)
    t = theta * (p / P1000) ** (R_D / CP)
    rho = p / (R_D * t * (1.0 + 0.61 * qv))
    rho_d = rho / (1.0 + qv)
    pd = np.empty_like(z)
    pd[-1] = p[-1] / (1.0 + qv[-1] * RVOVRD)
    for k in range(len(z) - 2, -1, -1):
        pd[k] = pd[k + 1] + G * dz * 0.5 * (rho_d[k] + rho_d[k + 1])
    return p, pd, qv


def _channel_profiles(ny, dx, ztop, f, u_max, z_jet, dz):
    """The jet channel's height grid, row coordinates, the theta profile of
    a row (thermal-wind balance) and the base state's dry sounding (the
    middle row's) with the model-top pressure."""
    Ly = ny * dx
    z = np.arange(0.0, ztop + 4000.0 + dz, dz)
    theta_ref = np.where(z <= 12000.0, 300.0 + 43.0 * (z / 12000.0) ** 1.25,
                         343.0 * np.exp(G / (CP * 213.0) * (z - 12000.0)))
    yj = (np.arange(1, ny + 1) - 0.5) * dx
    Y = yj / 2.0 - Ly / (4.0 * math.pi) * np.sin(2.0 * math.pi * yj / Ly)
    below = z <= z_jet

    def row_theta(y_int):
        return theta_ref - np.where(below, f * theta_ref / G * (u_max / z_jet) * y_int, 0.0)

    p_mid, _, _ = _column_sounding(z, row_theta(Y[ny // 2]), np.zeros_like(z), dz)
    p_top = float(_interp(ztop, z, p_mid))
    return z, yj, Y, row_theta, p_mid, p_top


def channel_state(nx, ny, kde, dx, dt, ztop, rng, f=1.0e-4, u_max=30.0, z_jet=10000.0, noise=1.0,
                  z_noise=2000.0, rh=0.8, z_moist=8000.0, n_scalar=0, name="channel", dz=20.0):
    """Zonally periodic channel on an f-plane with a balanced zonal jet
    (the idealised baroclinic-wave case of module_initialize_ideal.F, b_wave,
    :240-260, :344-360, :738-760, :992-1090, restated with an analytic jet
    instead of the tabulated input_jet):

    * u(y, z) = u_max sin^2(pi y / Ly) min(z, z_jet) / z_jet;
    * theta(y, z) = theta_ref(z) - (f theta_ref(z) / g) (u_max / z_jet) Y(y)
      below z_jet, theta_ref(z) above, with Y(y) = y / 2 - Ly / (4 pi)
      sin(2 pi y / Ly): thermal-wind balance f du/dz = -(g / theta) dtheta/dy
      (cold to the north; the jump at z_jet is stable everywhere); theta_ref is
      the Weisman-Klemp dry profile (300 K surface, 12 km / 343 K tropopause);
    * qv from rh relative humidity below z_moist (0 above);
    * a seeded uniform +-noise K perturbation of theta below z_noise;
    * every row's column in hydrostatic balance from a uniform surface
      pressure; the base state is the middle row's dry sounding (as b_wave
      takes the middle column of its jet), flat terrain;
    * periodic in x, symmetric (free-slip walls) in y, Coriolis f, e = 0.
    """
    ide, jde = nx + 1, ny + 1
    cfg = abi.default_config(periodic_x=True, periodic_y=False, symmetric_y=True)
    h = abi.HALO
    nim, njm, nk = ide + 2 * h, jde + 2 * h, kde
    m = eta_metrics(kde)
    Ly = ny * dx
    z, yj, Y, row_theta, p_mid, p_top = _channel_profiles(ny, dx, ztop, f, u_max, z_jet, dz)
    rh_prof = np.where(z <= z_moist, rh, 0.0)
    jmid = ny // 2
    hc = hybrid_coefs(m, kde, p_top)
    c1h, c2h, c1f, c2f = hc["c1h"], hc["c2h"], hc["c1f"], hc["c2f"]
    c3h, c4h, c3f, c4f = hc["c3h"], hc["c4h"], hc["c3f"], hc["c4f"]
    dnw, rdnw, rdn = m["dnw"], m["rdnw"], m["rdn"]
    th_mid = row_theta(Y[jmid])
    p_surf = float(p_mid[0])
    mub = p_surf - p_top
    pb = np.zeros(kde + 1); t_init = np.zeros(kde + 1); alb = np.zeros(kde + 1); phb = np.zeros(kde + 1)
    for k in range(1, kde):
        pl = c3h[k] * (p_surf - p_top) + c4h[k] + p_top
        pb[k] = pl
        t_init[k] = _interp(pl, p_mid, th_mid) - T0
        alb[k] = (R_D / P1000) * (t_init[k] + T0) * (pb[k] / P1000) ** CVPM
    for kk in range(2, kde + 1):
        k = kk - 1
        phb[kk] = phb[kk - 1] - dnw[kk - 1] * (c1h[k] * mub + c2h[k]) * alb[kk - 1]
    zhalf = np.array([0.5 * (phb[k] + phb[k + 1]) / G if 1 <= k < kde else 0.0 for k in range(kde + 1)])

    # full state, row by row (columns of a row are identical before the noise)
    ni, nj, nkm = nx, ny, kde - 1
    t1 = np.zeros((nj, nkm, ni)); qv3 = np.zeros((nj, nkm, ni)); u3 = np.zeros((nj, nkm, ni))
    mu1_2d = np.zeros((nj, ni))
    for j in range(nj):
        th_j = row_theta(Y[j])
        _, pd_j, qv_j = _column_sounding(z, th_j, rh_prof, dz)
        pd_surf = float(pd_j[0])
        mu1_2d[j, :] = pd_surf - p_top - mub
        for k in range(1, kde):
            pl = c3h[k] * (pd_surf - p_top) + c4h[k] + p_top
            qv3[j, k - 1, :] = _interp(pl, pd_j, qv_j)
            t1[j, k - 1, :] = _interp(pl, pd_j, th_j) - T0
            u3[j, k - 1, :] = u_max * math.sin(math.pi * yj[j] / Ly) ** 2 * min(zhalf[k], z_jet) / z_jet

    p3, alt3, al3 = _column_p_al(t1, qv3, mu1_2d, mub, pb, alb, c1f, c2f, rdnw, rdn, kde)
    ph1 = _column_ph(al3, mu1_2d, mub, alb, c1h, c2h, dnw, kde, ni)
    if noise > 0:
        zmass = 0.5 * (ph1[:, :-1] + ph1[:, 1:] + (phb[1:kde] + phb[2:kde + 1])[None, :, None]) / G
        t1 = t1 + np.where(zmass < z_noise, rng.uniform(-noise, noise, size=t1.shape), 0.0)
    p3, alt3, al3 = _column_p_al(t1, qv3, mu1_2d, mub, pb, alb, c1f, c2f, rdnw, rdn, kde)
    ph1 = _column_ph(al3, mu1_2d, mub, alb, c1h, c2h, dnw, kde, ni)
    tm = (t1 + T0) * (1.0 + (R_V / R_D) * qv3) - T0
    mut = mub + mu1_2d
    al3 = np.zeros_like(tm)
    for k in range(1, kde):
        pfu = c3f[k + 1] * mut + c4f[k + 1] + p_top
        pfd = c3f[k] * mut + c4f[k] + p_top
        phm = c3h[k] * mut + c4h[k] + p_top
        al3[:, k - 1] = (ph1[:, k] - ph1[:, k - 1] + phb[k + 1] - phb[k]) / phm / np.log(pfd / pfu) - alb[k]
    p3 = P1000 * ((R_D * (T0 + tm)) / (P1000 * (al3 + alb[1:kde][None, :, None]))) ** CPOVCV - pb[1:kde][None, :, None]
    alt3 = al3 + alb[1:kde][None, :, None]

    def mem3(interior, nkk, stag=None):
        a = np.zeros((njm, nk, nim))
        a[h:h + interior.shape[0], :nkk, h:h + interior.shape[2]] = interior
        if stag == "u":
            a[h:h + interior.shape[0], :nkk, h + nx] = interior[:, :, 0]
        return fill_halo(a, 3, stag, ide, jde, cfg)

    def mem2(interior):
        a = np.zeros((njm, nim))
        a[h:h + nj, h:h + ni] = interior
        return fill_halo(a, 2, None, ide, jde, cfg)

    def col(v1d, nkk):
        return np.broadcast_to(v1d[1:nkk + 1][None, :, None], (nj, nkk, ni))

    fl = {}
    fl["u_1"] = mem3(u3, nkm, "u"); fl["u_2"] = fl["u_1"].copy()
    fl["v_1"] = np.zeros((njm, nk, nim)); fl["v_2"] = np.zeros((njm, nk, nim))
    fl["w_1"] = np.zeros((njm, nk, nim)); fl["w_2"] = np.zeros((njm, nk, nim))
    fl["t_1"] = mem3(tm, nkm); fl["t_2"] = fl["t_1"].copy()
    fl["ph_1"] = mem3(ph1, kde); fl["ph_2"] = fl["ph_1"].copy()
    fl["phb"] = mem3(col(phb, kde), kde)
    fl["pb"] = mem3(col(pb, nkm), nkm)
    fl["alb"] = mem3(col(alb, nkm), nkm)
    fl["p"] = mem3(p3, nkm)
    fl["al"] = mem3(al3, nkm)
    fl["alt"] = mem3(alt3, nkm)
    fl["mu_1"] = mem2(mu1_2d); fl["mu_2"] = fl["mu_1"].copy()
    fl["mub"] = mem2(np.full((nj, ni), mub))
    for nm in ("msfux", "msfuy", "msfvx", "msfvx_inv", "msfvy", "msftx", "msfty", "cosa"):
        fl[nm] = np.ones((njm, nim))
    for nm in ("ht", "e", "sina"):
        fl[nm] = np.zeros((njm, nim))
    fl["f"] = np.full((njm, nim), f)
    for nm in ("znw", "znu", "dnw", "rdnw", "dn", "rdn", "fnm", "fnp"):
        fl[nm] = m[nm][1:].copy()
    for nm in ("c1h", "c2h", "c1f", "c2f", "c3h", "c4h", "c3f", "c4f"):
        fl[nm] = hc[nm][1:].copy()
    _base_profiles(fl, t1, qv3, ph1, phb, kde)
    fl["t_init"] = mem3(col(t_init, nkm), nkm)
    qv_mem = mem3(qv3, nkm)
    species = [(qv_mem, qv_mem.copy())]
    for _ in range(n_scalar):
        qs = 1.0e-6 * np.exp(rng.standard_normal(size=(nj, nkm, ni)))
        qm = mem3(qs, nkm)
        species.append((qm, qm.copy()))
    desc = _make_desc(ide, jde, kde, n_scalar, cfg, dt, dx, m, p_top)
    meta = dict(dx=dx, dt=dt, ztop=ztop, f=f, u_max=u_max, z_jet=z_jet, n_scalar=n_scalar)
    return Case(name, desc, fl, species, meta)


def _base_profiles(f, t1, qv3, ph1, phb, kde):
    """u_base, v_base, t_base, qv_base, z_base of column (1,1) of the initial
    state (module_initialize_ideal.F:1578-1586): theta before the moist
    conversion, the winds, qv, and the mass-level heights from phb + ph_1
    (1-D, kms:kme)."""
    h = abi.HALO
    nkm = kde - 1
    for nm, col in (("u_base", f["u_1"][h, :nkm, h]), ("v_base", f["v_1"][h, :nkm, h]), ("t_base", t1[0, :, 0]),
                    ("qv_base", qv3[0, :, 0])):
        a = np.zeros(kde)
        a[:nkm] = col
        f[nm] = a
    z = np.zeros(kde)
    z[:nkm] = 0.5 * (phb[1:kde] + phb[2:kde + 1] + ph1[0, :nkm, 0] + ph1[0, 1:kde, 0]) / G
    f["z_base"] = z


def _make_desc(ide, jde, kde, n_scalar, cfg, dt, dx, m, p_top):
    desc = abi.WrfGpuDomainDesc()
    desc.ide, desc.jde, desc.kde = ide, jde, kde
    desc.n_moist, desc.n_scalar = 1, n_scalar
    desc.config = cfg
    s = desc.scalars
    s.dt, s.dx, s.dy = dt, dx, dx
    s.rdx, s.rdy = 1.0 / dx, 1.0 / dx
    s.cf1, s.cf2, s.cf3, s.cfn, s.cfn1 = m["cf1"], m["cf2"], m["cf3"], m["cfn"], m["cfn1"]
    s.epssm, s.smdiv, s.emdiv = 0.1, 0.1, 0.01
    s.p_top = p_top
    return desc


def supercell_desc(nx, ny, kde, dx, dt, ztop, n_scalar=0, hypsometric_opt=2, hodo_radius=15.0):
    """The domain description supercell_state gives, without building the
    fields (so that an ensemble can be created before its members' states
    are built and streamed in one at a time)."""
    cfg = abi.default_config(periodic_x=True, periodic_y=True)
    cfg.hypsometric_opt = hypsometric_opt
    m = eta_metrics(kde)
    zd, pdry, _, _, _, _, _ = wk_sounding(ztop, hodo_radius=hodo_radius, dry=True)
    p_top = float(_interp(ztop, zd, pdry))
    return _make_desc(nx + 1, ny + 1, kde, n_scalar, cfg, dt, dx, m, p_top)


# ---------------------------------------------------------------------------
# the benchmark workloads
# ---------------------------------------------------------------------------
def config1(seed=1, scale=1):
    """41x41 x 41 eta levels, dx = 2 km, top 20 km, dt = 12 s, one +3 K bubble
    (10 km / 1.5 km radii at 1.5 km), +-0.01 K noise, qv only."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nx = 41 * scale
    dx = 2000.0
    xc = 0.5 * nx * dx
    return supercell_state(nx, nx, 41, dx, 12.0, 20000.0,
                           [(xc, xc, 1500.0, 10000.0, 10000.0, 1500.0, 3.0)], rng,
                           n_scalar=0, name="c1_41x41x41")


def config2(seed=2, nx=512, kde=80, n_scalar=10):
    """512x512 x 80 levels, dx = 1 km, top 20 km, dt = 6 s, 16 +3 K bubbles at
    seeded positions, 10 positive-definite log-normal scalars (median 1e-6,
    sigma 1) plus qv."""
    rng = np.random.Generator(np.random.PCG64(seed))
    dx = 1000.0
    L = nx * dx
    bubbles = []
    for _ in range(16):
        xc, yc = rng.uniform(0.0, L, size=2)
        bubbles.append((float(xc), float(yc), 1500.0, 10000.0, 10000.0, 1500.0, 3.0))
    return supercell_state(nx, nx, kde, dx, 6.0, 20000.0, bubbles, rng, n_scalar=n_scalar,
                           name="c2_%dx%dx%d" % (nx, nx, kde))


def config3(seed=3, nx=1024, ny=None, kde=96, dx=4000.0, dt=20.0, ztop=25000.0):
    """1024 x 1024 x 96 levels, dx = 4 km, top 25 km, dt = 20 s: the zonally
    periodic f-plane channel (f = 1e-4) with the balanced jet
    u = 30 sin^2(pi y / Ly) (z / 10 km), capped above 10 km, theta in
    thermal-wind balance, +-1 K seeded noise below 2 km, qv at 80 % RH below
    8 km; qv is the one (positive-definite) species.  nx, ny give the
    same channel at other sizes (same dx, so a narrower channel)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ny = nx if ny is None else ny
    return channel_state(nx, ny, kde, dx, dt, ztop, rng, name="c3_%dx%dx%d" % (nx, ny, kde))


def ensemble_members(seed=4, n=64, nmin=64, nmax=256, kmin=41, kmax=80, n_scalar=3, dx=2000.0, dt=12.0):
    """Uneven ensemble: nx, ny ~ U[nmin, nmax], levels ~ U[kmin, kmax], seeded
    bubble position and amplitude in [1, 4] K, 3 PD scalars per member."""
    rng = np.random.Generator(np.random.PCG64(seed))
    specs = []
    for _ in range(n):
        nx = int(rng.integers(nmin, nmax + 1))
        ny = int(rng.integers(nmin, nmax + 1))
        kde = int(rng.integers(kmin, kmax + 1))
        amp = float(rng.uniform(1.0, 4.0))
        xc = float(rng.uniform(0.25, 0.75)) * nx * dx
        yc = float(rng.uniform(0.25, 0.75)) * ny * dx
        specs.append((nx, ny, kde, amp, xc, yc, int(rng.integers(0, 2 ** 31))))
    return specs


def ensemble_member(spec, dx=2000.0, dt=12.0, n_scalar=3):
    nx, ny, kde, amp, xc, yc, mseed = spec
    rng = np.random.Generator(np.random.PCG64(mseed))
    return supercell_state(nx, ny, kde, dx, dt, 20000.0,
                           [(xc, yc, 1500.0, 10000.0, 10000.0, 1500.0, amp)], rng,
                           n_scalar=n_scalar, name="member_%dx%dx%d" % (nx, ny, kde))


def ensemble_member_desc(spec, dx=2000.0, dt=12.0, n_scalar=3):
    nx, ny, kde = spec[0], spec[1], spec[2]
    return supercell_desc(nx, ny, kde, dx, dt, 20000.0, n_scalar=n_scalar)


def channel_desc(nx, ny, kde, dx, dt, ztop, n_scalar=0, f=1.0e-4, u_max=30.0, z_jet=10000.0, dz=20.0):
    """The domain description channel_state gives, without building the
    fields (the base state's sounding alone fixes the model-top pressure)."""
    cfg = abi.default_config(periodic_x=True, periodic_y=False, symmetric_y=True)
    m = eta_metrics(kde)
    p_top = _channel_profiles(ny, dx, ztop, f, u_max, z_jet, dz)[5]
    return _make_desc(nx + 1, ny + 1, kde, n_scalar, cfg, dt, dx, m, p_top)


def c5_members(seed=5, n=256, nmin=96, nmax=384, kmin=41, kmax=96, n_scalar=7):
    """The large mixed ensemble: n members, nx, ny ~ U[nmin, nmax], levels
    ~ U[kmin, kmax], each a supercell (dx = 2 km, dt = 12 s, top 20 km, one
    bubble of seeded position and amplitude in [1, 4] K) or an f-plane jet
    channel (dx = 4 km, dt = 20 s, top 25 km) with even odds, qv plus
    n_scalar positive-definite scalars."""
    rng = np.random.Generator(np.random.PCG64(seed))
    specs = []
    for _ in range(n):
        kind = "channel" if rng.uniform() < 0.5 else "supercell"
        nx = int(rng.integers(nmin, nmax + 1))
        ny = int(rng.integers(nmin, nmax + 1))
        kde = int(rng.integers(kmin, kmax + 1))
        amp = float(rng.uniform(1.0, 4.0))
        fx, fy = float(rng.uniform(0.25, 0.75)), float(rng.uniform(0.25, 0.75))
        specs.append((kind, nx, ny, kde, amp, fx, fy, int(rng.integers(0, 2 ** 31)), n_scalar))
    return specs


def c5_member(spec):
    kind, nx, ny, kde, amp, fx, fy, mseed, n_scalar = spec
    rng = np.random.Generator(np.random.PCG64(mseed))
    if kind == "channel":
        return channel_state(nx, ny, kde, 4000.0, 20.0, 25000.0, rng, n_scalar=n_scalar,
                             name="channel_%dx%dx%d" % (nx, ny, kde))
    dx = 2000.0
    return supercell_state(nx, ny, kde, dx, 12.0, 20000.0,
                           [(fx * nx * dx, fy * ny * dx, 1500.0, 10000.0, 10000.0, 1500.0, amp)], rng,
                           n_scalar=n_scalar, name="supercell_%dx%dx%d" % (nx, ny, kde))


def c5_member_desc(spec):
    kind, nx, ny, kde = spec[0], spec[1], spec[2], spec[3]
    if kind == "channel":
        return channel_desc(nx, ny, kde, 4000.0, 20.0, 25000.0, n_scalar=spec[8])
    return supercell_desc(nx, ny, kde, 2000.0, 12.0, 20000.0, n_scalar=spec[8])


def open_boundaries(case, x=True, y=True):
    """The same initial state with open lateral boundaries in x and/or y (the
    em_quarter_ss namelist: open_xs/xe, open_ys/ye = .true.): the options
    changed, and the memory halo of every field holding its nearest edge
    value, as the open-boundary copy of share/module_bc.F:864-1107 leaves
    it (mass points and w levels copy column ids / ide-1, u copies ids /
    ide; likewise in y)."""
    import copy
    desc = copy.deepcopy(case.desc)
    c = desc.config
    if x:
        c.periodic_x = c.symmetric_xs = c.symmetric_xe = 0
        c.open_xs = c.open_xe = 1
    if y:
        c.periodic_y = c.symmetric_ys = c.symmetric_ye = 0
        c.open_ys = c.open_ye = 1
    h = abi.HALO
    ide, jde = case.ide, case.jde

    def clamp(a, kind, stag):
        # memory index p holds point p + 1 - h; points beyond 1 .. hi take
        # the value of the nearest of the two (x first, then y)
        if a.ndim != kind:
            return a
        out = np.array(a, copy=True, order="C")
        if x:
            hi = ide if stag == "u" else ide - 1
            out[..., :h] = out[..., h:h + 1]
            out[..., hi + h:] = out[..., hi + h - 1:hi + h]
        if y:
            hi = jde if stag == "v" else jde - 1
            out[:h] = out[h:h + 1]
            out[hi + h:] = out[hi + h - 1:hi + h]
        return out

    fields = {}
    for nm, a in case.fields.items():
        stag = "u" if nm in ("u_1", "u_2") else ("v" if nm in ("v_1", "v_2") else None)
        fields[nm] = clamp(a, a.ndim, stag) if a.ndim in (2, 3) else a.copy()
    species = [(clamp(q, 3, None), clamp(qo, 3, None)) for q, qo in case.species]
    name = case.name + ("_openx" if x else "") + ("_openy" if y else "")
    return Case(name, desc, fields, species, dict(case.meta))


def small_case(nx=12, ny=10, kde=12, n_scalar=1, seed=7, dx=2000.0, dt=12.0):
    """A tiny domain for fast parity tests (one bubble, noise, scalars)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    L = nx * dx
    return supercell_state(nx, ny, kde, dx, dt, 20000.0,
                           [(0.5 * L, 0.5 * ny * dx, 1500.0, 6000.0, 6000.0, 1500.0, 3.0)], rng,
                           n_scalar=n_scalar, name="small_%dx%dx%d" % (nx, ny, kde))
