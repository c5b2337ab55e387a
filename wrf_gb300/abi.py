"""ctypes mirror of include/wrfgpu.h (structs, field ids, routine ids).

The C header is the boundary; this module only restates its layout for
Python callers (tests, bench.py) and is kept in step with it by
tests/test_abi.py, which compiles a small probe against the header.
"""
import ctypes as C

HALO = 4

WRFGPU_OK = 0
WRFGPU_E_ARG = -1
WRFGPU_E_CUDA = -2
WRFGPU_E_NONFINITE = -3
WRFGPU_E_CFL = -4
WRFGPU_E_TIMEOUT = -5
WRFGPU_E_NOMEM = -6
WRFGPU_E_SIZE = -7

ERRORS = {
    WRFGPU_E_ARG: "bad argument or unsupported option",
    WRFGPU_E_CUDA: "CUDA runtime error",
    WRFGPU_E_NONFINITE: "non-finite value in the state",
    WRFGPU_E_CFL: "vertical CFL above limit",
    WRFGPU_E_TIMEOUT: "bounded device wait gave up",
    WRFGPU_E_NOMEM: "device allocation failed",
    WRFGPU_E_SIZE: "request larger than a fixed capacity",
}


class WrfDynConfig(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "periodic_x", "periodic_y",
        "symmetric_xs", "symmetric_xe", "symmetric_ys", "symmetric_ye",
        "open_xs", "open_xe", "open_ys", "open_ye",
        "specified", "nested", "polar",
        "rk_ord",
        "h_mom_adv_order", "v_mom_adv_order", "h_sca_adv_order", "v_sca_adv_order",
        "moist_adv_opt", "scalar_adv_opt",
        "non_hydrostatic", "top_lid", "use_theta_m", "hypsometric_opt", "phi_adv_z",
        "w_damping", "damp_opt", "diff_opt", "zadvect_implicit", "map_proj",
        "time_step_sound")] + [("w_crit_cfl", C.c_float), ("dampcoef", C.c_float), ("zdamp", C.c_float),
                               ("diff_6th_opt", C.c_int32), ("diff_6th_slopeopt", C.c_int32),
                               ("diff_6th_factor", C.c_float), ("diff_6th_thresh", C.c_float),
                               ("moist_mix6_off", C.c_int32), ("scalar_mix6_off", C.c_int32),
                               ("km_opt", C.c_int32), ("moist_mix2_off", C.c_int32),
                               ("scalar_mix2_off", C.c_int32), ("pad_cfg", C.c_int32),
                               ("khdif", C.c_float), ("kvdif", C.c_float)]


class WrfGpuScalars(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "dt", "dx", "dy", "rdx", "rdy", "cf1", "cf2", "cf3", "cfn", "cfn1",
        "epssm", "smdiv", "emdiv", "p_top")]


class WrfGpuDomainDesc(C.Structure):
    _fields_ = [("ide", C.c_int32), ("jde", C.c_int32), ("kde", C.c_int32),
                ("n_moist", C.c_int32), ("n_scalar", C.c_int32), ("pad0", C.c_int32),
                ("config", WrfDynConfig), ("scalars", WrfGpuScalars)]


F3D = ["u_1", "u_2", "v_1", "v_2", "w_1", "w_2", "t_1", "t_2", "ph_1", "ph_2",
       "phb", "pb", "alb", "p", "al", "alt", "php",
       "ru", "rv", "rw", "ww", "ww1", "cqu", "cqv", "cqw",
       "ru_tend", "rv_tend", "rw_tend", "t_tend", "ph_tend",
       "u_save", "v_save", "w_save", "t_save", "ph_save",
       "c2a", "pm1", "a", "alpha", "gamma", "t_2save",
       "ru_m", "rv_m", "ww_m", "advect_tend", "h_diabatic", "t_init"]
F2D = ["mu_1", "mu_2", "mub", "mut", "muu", "muv", "muts", "muus", "muvs", "mudf",
       "mu_save", "muave", "mu_tend", "msfux", "msfuy", "msfvx", "msfvx_inv", "msfvy",
       "msftx", "msfty", "ht", "f", "e", "sina", "cosa"]
F1D = ["znw", "znu", "dnw", "rdnw", "dn", "rdn", "fnm", "fnp", "c1h", "c2h", "c1f", "c2f",
       "c3h", "c4h", "c3f", "c4f", "u_base", "v_base", "t_base", "z_base", "qv_base"]
TENDF = ["ru_tendf", "rv_tendf", "rw_tendf", "t_tendf"]
TENDF_BASE = 90
F2D_BASE = 100
F1D_BASE = 200
SPECIES_BASE = 300

FIELD_ID = {}
for _i, _n in enumerate(F3D):
    FIELD_ID[_n] = _i
for _i, _n in enumerate(F2D):
    FIELD_ID[_n] = F2D_BASE + _i
for _i, _n in enumerate(F1D):
    FIELD_ID[_n] = F1D_BASE + _i
for _i, _n in enumerate(TENDF):
    FIELD_ID[_n] = TENDF_BASE + _i


def species_id(s, old=False):
    """Field id of species s (moist species first, then passive scalars)."""
    return SPECIES_BASE + 2 * s + (1 if old else 0)


def field_kind(fid):
    if 0 <= fid < len(F3D) or fid >= SPECIES_BASE or TENDF_BASE <= fid < TENDF_BASE + len(TENDF):
        return 3
    if F2D_BASE <= fid < F2D_BASE + len(F2D):
        return 2
    if F1D_BASE <= fid < F1D_BASE + len(F1D):
        return 1
    raise KeyError(fid)


# Routine ids of the per-routine runner (same values in the oracle).
ROUTINES = {
    "rk_step_prep": 1, "zero_tend": 2, "advect_u": 3, "advect_v": 4, "advect_w": 5,
    "advect_t": 6, "rhs_ph": 7, "horizontal_pressure_gradient": 8, "pg_buoy_w": 9,
    "coriolis": 10, "curvature": 11, "small_step_prep": 12, "calc_p_rho": 13,
    "calc_coef_w": 14, "advance_uv": 15, "advance_mu_t": 16, "advance_w": 17,
    "sumflux": 18, "small_step_finish": 19, "rk_update_scalar_pd": 20,
    "advect_scalar": 21, "advect_scalar_pd": 22, "rk_update_scalar": 23,
    "calc_p_rho_phi": 24, "set_w_surface": 25, "rk_tendency": 26,
    # oracle-only forms checked against the routine-level C entry points
    "rk_update_scalar_pd_args": 30, "rk_update_scalar_args": 31, "sixth_diff_species": 32,
    # rk_tendency's stage-1 forward terms (diffusion, damping) added to the *_tendf fields
    "forward_terms": 33, "addtend_dry_args": 34,
}


def default_config(periodic_x=True, periodic_y=True, symmetric_y=False):
    """The Registry defaults on the physics-off path (Registry.EM_COMMON:2840-2938)."""
    c = WrfDynConfig()
    c.periodic_x = 1 if periodic_x else 0
    c.periodic_y = 1 if periodic_y else 0
    if not periodic_x:
        c.symmetric_xs = c.symmetric_xe = 1
    if symmetric_y:
        c.periodic_y = 0
        c.symmetric_ys = c.symmetric_ye = 1
    c.rk_ord = 3
    c.h_mom_adv_order = 5
    c.v_mom_adv_order = 3
    c.h_sca_adv_order = 5
    c.v_sca_adv_order = 3
    c.moist_adv_opt = 1
    c.scalar_adv_opt = 1
    c.non_hydrostatic = 1
    c.top_lid = 0
    c.use_theta_m = 1
    c.hypsometric_opt = 2
    c.phi_adv_z = 1
    c.w_damping = 0
    c.damp_opt = 0
    c.diff_opt = 0
    c.zadvect_implicit = 0
    c.map_proj = 0
    c.time_step_sound = 0
    c.w_crit_cfl = 1.0
    c.dampcoef = 0.2
    c.zdamp = 5000.0
    c.diff_6th_opt = 0
    c.diff_6th_slopeopt = 0
    c.diff_6th_factor = 0.12
    c.diff_6th_thresh = 0.10
    c.moist_mix6_off = 0
    c.scalar_mix6_off = 0
    c.km_opt = 1
    c.moist_mix2_off = 0
    c.scalar_mix2_off = 0
    c.khdif = 0.0
    c.kvdif = 0.0
    return c
