// ORACLE — test infrastructure only.
//
// A CPU restatement of WRF-ARW's physics-off solve_em large step (RK3 with
// split-explicit acoustic sub-steps, 5th/3rd-order flux-form advection,
// positive-definite scalars) in plain C++, templated on the floating-point
// type: float restates the reference's default REAL (RWORDSIZE=4); double
// restates the `configure -r8` (real*8) build that serves as the FP64
// accuracy oracle.  Every routine follows one Fortran subroutine of the
// reference, keeps its argument meaning and index triples
// (ids:ide / ims:ime / its:ite, x3 for j and k) and cites the file:line it
// restates.  Loop bounds and the left-to-right evaluation order of each
// expression are kept, so that a build with -ffp-contract=off reproduces the
// reference's rounding sequence.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
// this code, and only as the checker or the timed CPU baseline; the product
// path (wrf_gb300/csrc) never links or calls it.
//
// Parity status: the reference's Fortran cannot be compiled where this was
// written (no Fortran compiler), and the reference ships no golden vectors for
// this path, so parity is pinned by the reference's own known-behaviour
// fixture (module_advect_em.F:3-115, the ADVECT_KERNEL top-hat feeder) and by
// conservation / positivity / rest-state properties; see tests/.
//
// Supported option subset (anything else is rejected, like wrf_error_fatal):
//   rk_ord=3, h_*_adv_order=5, v_*_adv_order=3, non_hydrostatic=.true.,
//   periodic_x/periodic_y, symmetric_xs/xe/ys/ye or open_xs/xe/ys/ye lateral
//   boundaries,
//   moist_adv_opt/scalar_adv_opt in {0 (ORIGINAL), 1 (POSITIVEDEF)},
//   hypsometric_opt in {1,2}, phi_adv_z in {1,2}, IEVA off, physics off.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <stdexcept>
#include <algorithm>
#include "../include/wrfgpu.h"

namespace wrforacle {

// ---------------------------------------------------------------------------
// Fortran-style array views.  3-D arrays are (ims:ime, kms:kme, jms:jme),
// i fastest (Registry dims "ikj"); 2-D arrays are (ims:ime, jms:jme); 1-D
// column arrays are (kms:kme).
// ---------------------------------------------------------------------------
struct Dims {
  int ids, ide, jds, jde, kds, kde;
  int ims, ime, jms, jme, kms, kme;
  int its, ite, jts, jte, kts, kte;
};

template <typename R> struct A3 {
  R* p = nullptr; int ims = 0, kms = 0, jms = 0; long sk = 0, sj = 0;
  A3() {}
  A3(R* ptr, const Dims& d) : p(ptr), ims(d.ims), kms(d.kms), jms(d.jms) {
    sk = (long)(d.ime - d.ims + 1); sj = sk * (long)(d.kme - d.kms + 1);
  }
  inline R& operator()(int i, int k, int j) const {
    return p[(long)(i - ims) + (long)(k - kms) * sk + (long)(j - jms) * sj];
  }
};
template <typename R> struct A2 {
  R* p = nullptr; int ims = 0, jms = 0; long sj = 0;
  A2() {}
  A2(R* ptr, const Dims& d) : p(ptr), ims(d.ims), jms(d.jms) { sj = (long)(d.ime - d.ims + 1); }
  inline R& operator()(int i, int j) const { return p[(long)(i - ims) + (long)(j - jms) * sj]; }
};
template <typename R> struct A1 {
  R* p = nullptr; int kms = 0;
  A1() {}
  A1(R* ptr, const Dims& d) : p(ptr), kms(d.kms) {}
  inline R& operator()(int k) const { return p[k - kms]; }
};

// share/module_model_constants.F:17-43, evaluated in the working precision as
// the reference does for REAL PARAMETERs (promoted with -r8).
template <typename R> struct K {
  static constexpr R g = R(9.81);
  static constexpr R r_d = R(287.);
  static constexpr R cp = R(7.) * r_d / R(2.);
  static constexpr R r_v = R(461.6);
  static constexpr R cv = cp - r_d;
  static constexpr R cvpm = -cv / cp;
  static constexpr R p1000mb = R(100000.);
  static constexpr R t0 = R(300.);
  static constexpr R p0 = p1000mb;
  static constexpr R cpovcv = cp / (cp - r_d);
  static constexpr R rvovrd = r_v / r_d;
  static constexpr R reradius = R(1.) / R(6370.0e03);
};

template <typename R> static inline R fsign1(R a) { return std::copysign(R(1), a); }
template <typename R> static inline R fmaxr(R a, R b) { return a > b ? a : b; }   // Fortran MAX(a,b)
template <typename R> static inline R fminr(R a, R b) { return a < b ? a : b; }   // Fortran MIN(a,b)

// Flux operators of advect_u/v/w/scalar (module_advect_em.F:172-186, :3102-3119).
// time_step > 0 in every supported run, so sign(1,time_step) == 1.
template <typename R> static inline R flux4(R qm2, R qm1, R q, R qp1) {
  return (R(7.) * (q + qm1) - (qp1 + qm2)) / R(12.0);
}
template <typename R> static inline R flux3(R qm2, R qm1, R q, R qp1, R ua) {
  return flux4(qm2, qm1, q, qp1) + R(1) * fsign1(ua) * ((qp1 - qm2) - R(3.) * (q - qm1)) / R(12.0);
}
template <typename R> static inline R flux6(R qm3, R qm2, R qm1, R q, R qp1, R qp2) {
  return (R(37.) * (q + qm1) - R(8.) * (qp1 + qm2) + (qp2 + qm3)) / R(60.0);
}
template <typename R> static inline R flux5(R qm3, R qm2, R qm1, R q, R qp1, R qp2, R ua) {
  return flux6(qm3, qm2, qm1, q, qp1, qp2) -
         R(1) * fsign1(ua) * ((qp2 - qm3) - R(5.) * (qp1 - qm2) + R(10.) * (q - qm1)) / R(60.0);
}
// advect_scalar_pd uses pre-divided coefficients (module_advect_em.F:6165-6185).
template <typename R> static inline R pflux4(R qm2, R qm1, R q, R qp1) {
  return (R(7.) / R(12.)) * (q + qm1) - (R(1.) / R(12.)) * (qp1 + qm2);
}
template <typename R> static inline R pflux3(R qm2, R qm1, R q, R qp1, R ua) {
  return pflux4(qm2, qm1, q, qp1) + R(1) * fsign1(ua) * (R(1.) / R(12.)) * ((qp1 - qm2) - R(3.) * (q - qm1));
}
template <typename R> static inline R pflux6(R qm3, R qm2, R qm1, R q, R qp1, R qp2) {
  return (R(37.) / R(60.)) * (q + qm1) - (R(2.) / R(15.)) * (qp1 + qm2) + (R(1.) / R(60.)) * (qp2 + qm3);
}
template <typename R> static inline R pflux5(R qm3, R qm2, R qm1, R q, R qp1, R qp2, R ua) {
  return pflux6(qm3, qm2, qm1, q, qp1, qp2) -
         R(1) * fsign1(ua) * (R(1.) / R(60.)) * ((qp2 - qm3) - R(5.) * (qp1 - qm2) + R(10.) * (q - qm1));
}
template <typename R> static inline R flux_upwind(R qm1, R q, R cr) {
  return R(0.5) * fminr(R(1.0), (cr + std::fabs(cr))) * qm1 + R(0.5) * fmaxr(R(-1.0), (cr - std::fabs(cr))) * q;
}

// Supported-option check (the reference stops in wrf_error_fatal otherwise).
inline void check_config(const WrfDynConfig& c) {
  if (c.rk_ord != 3) throw std::runtime_error("rk_ord must be 3");
  if (c.h_mom_adv_order != 5 || c.h_sca_adv_order != 5) throw std::runtime_error("horizontal advection order must be 5");
  if (c.v_mom_adv_order != 3 || c.v_sca_adv_order != 3) throw std::runtime_error("vertical advection order must be 3");
  if (!c.non_hydrostatic) throw std::runtime_error("hydrostatic option not supported");
  if (c.specified || c.nested || c.polar) throw std::runtime_error("specified/nested/polar boundaries not supported");
  // share/module_bc.F:60-133 boundary_condition_check: one condition per side.
  auto one = [](int a, int b, int e) { return (a != 0) + (b != 0) + (e != 0) == 1; };
  if (!one(c.periodic_x, c.symmetric_xs, c.open_xs) || !one(c.periodic_x, c.symmetric_xe, c.open_xe) ||
      !one(c.periodic_y, c.symmetric_ys, c.open_ys) || !one(c.periodic_y, c.symmetric_ye, c.open_ye))
    throw std::runtime_error("each lateral boundary needs exactly one condition");
  if (c.zadvect_implicit != 0) throw std::runtime_error("IEVA not supported");
  if (c.diff_6th_opt < 0 || c.diff_6th_opt > 2) throw std::runtime_error("diff_6th_opt must be 0, 1 or 2");
}

// ===========================================================================
// share/module_bc.F — set_physical_bc2d (:202-649) and set_physical_bc3d
// (:651-1000), restricted to periodic, symmetric and open boundaries
// (bdyzone = 4, :33).  The serial build has one patch (ips=ids, ipe=ide).
// ===========================================================================
static const int BDYZONE = 4;

// open_bc_copy: the variables whose halo takes the open-boundary copy,
// set_physical_bc2d (module_bc.F:242-251) and set_physical_bc3d (:692-704).
inline bool open_bc_copy2(char v) {
  return v == 'u' || v == 'v' || v == 'w' || v == 't' || v == 'x' || v == 'y' || v == 'r' || v == 'p';
}
inline bool open_bc_copy3(char v) { return open_bc_copy2(v) || v == 'd' || v == 'e' || v == 'f'; }

template <typename R>
void set_physical_bc3d(R* dat_p, char variable_in, const WrfDynConfig& cf, const Dims& d) {
  A3<R> dat(dat_p, d);
  char variable = variable_in;
  if (variable_in >= 'A' && variable_in <= 'Z') variable = (char)(variable_in - 'A' + 'a');
  int istag = -1, jstag = -1;
  int k_end = std::max(1, std::min(d.kde - 1, d.kte));
  if (variable == 'u' || variable == 'x') istag = 0;
  if (variable == 'v' || variable == 'y') jstag = 0;
  if (variable == 'd') { istag = 0; jstag = 0; }
  if (variable == 'e') { istag = 0; k_end = std::min(d.kde, d.kte); }
  if (variable == 'f') { jstag = 0; k_end = std::min(d.kde, d.kte); }
  if (variable == 'w') k_end = std::min(d.kde, d.kte);
  const int ids = d.ids, ide = d.ide, jds = d.jds, jde = d.jde;
  if (cf.periodic_x) {
    if (d.its == ids) {
      for (int j = std::max(jds, d.jts - 1); j <= std::min(d.jte + 1, jde + jstag); ++j)
        for (int k = d.kts; k <= k_end; ++k)
          for (int i = 0; i >= -(BDYZONE - 1); --i) dat(ids + i - 1, k, j) = dat(ide + i - 1, k, j);
    }
    if (d.ite == ide) {
      for (int j = std::max(jds, d.jts - 1); j <= std::min(d.jte + 1, jde + jstag); ++j)
        for (int k = d.kts; k <= k_end; ++k)
          for (int i = -istag; i <= BDYZONE; ++i) dat(ide + i + istag, k, j) = dat(ids + i + istag, k, j);
    }
  } else {
    if (cf.symmetric_xs && d.its == ids) {
      for (int j = std::max(jds, d.jts - 1); j <= std::min(d.jte + 1, jde + jstag); ++j)
        for (int k = d.kts; k <= k_end; ++k)
          for (int i = 1; i <= BDYZONE; ++i) {
            if (istag == -1) dat(ids - i, k, j) = dat(ids + i - 1, k, j);
            else if (variable == 'u') dat(ids - i, k, j) = -dat(ids + i, k, j);
            else dat(ids - i, k, j) = dat(ids + i, k, j);
          }
    }
    if (cf.symmetric_xe && d.ite == ide) {
      for (int j = std::max(jds, d.jts - 1); j <= std::min(d.jte + 1, jde + jstag); ++j)
        for (int k = d.kts; k <= k_end; ++k)
          for (int i = 1; i <= BDYZONE; ++i) {
            if (istag == -1) dat(ide + i - 1, k, j) = dat(ide - i, k, j);
            else if (variable == 'u') dat(ide + i, k, j) = -dat(ide - i, k, j);
            else dat(ide + i, k, j) = dat(ide - i, k, j);
          }
    }
    // module_bc.F:864-925: open boundaries copy the edge value into three
    // halo points, for the variables of open_bc_copy (:692-704).
    if (cf.open_xs && d.its == ids && open_bc_copy3(variable)) {
      for (int j = d.jts - BDYZONE; j <= std::min(d.jte, jde + jstag) + BDYZONE; ++j)
        for (int k = d.kts; k <= k_end; ++k) {
          dat(ids - 1, k, j) = dat(ids, k, j);
          dat(ids - 2, k, j) = dat(ids, k, j);
          dat(ids - 3, k, j) = dat(ids, k, j);
        }
    }
    if (cf.open_xe && d.ite == ide && open_bc_copy3(variable)) {
      if (variable != 'u' && variable != 'x') {
        for (int j = d.jts - BDYZONE; j <= std::min(d.jte, jde + jstag) + BDYZONE; ++j)
          for (int k = d.kts; k <= k_end; ++k) {
            dat(ide, k, j) = dat(ide - 1, k, j);
            dat(ide + 1, k, j) = dat(ide - 1, k, j);
            dat(ide + 2, k, j) = dat(ide - 1, k, j);
          }
      } else {
        for (int j = std::max(jds, d.jts - 1) - BDYZONE; j <= std::min(d.jte + 1, jde + jstag) + BDYZONE; ++j)
          for (int k = d.kts; k <= k_end; ++k) {
            dat(ide + 1, k, j) = dat(ide, k, j);
            dat(ide + 2, k, j) = dat(ide, k, j);
            dat(ide + 3, k, j) = dat(ide, k, j);
          }
      }
    }
  }
  int i_start = std::max(ids, d.its - 1), i_end = std::min(d.ite + 1, ide + istag);
  if (d.its == ids) i_start = d.ims;
  if (d.ite == ide) i_end = d.ime;
  if (cf.periodic_y) {
    if (d.jts == jds) {
      for (int j = 0; j >= -(BDYZONE - 1); --j)
        for (int k = d.kts; k <= k_end; ++k)
          for (int i = i_start; i <= i_end; ++i) dat(i, k, jds + j - 1) = dat(i, k, jde + j - 1);
    }
    if (d.jte == jde) {
      for (int j = -jstag; j <= BDYZONE; ++j)
        for (int k = d.kts; k <= k_end; ++k)
          for (int i = i_start; i <= i_end; ++i) dat(i, k, jde + j + jstag) = dat(i, k, jds + j + jstag);
    }
  } else {
    if (cf.symmetric_ys && d.jts == jds) {
      for (int j = 1; j <= BDYZONE; ++j)
        for (int k = d.kts; k <= k_end; ++k)
          for (int i = i_start; i <= i_end; ++i) {
            if (jstag == -1) dat(i, k, jds - j) = dat(i, k, jds + j - 1);
            else if (variable == 'v') dat(i, k, jds - j) = -dat(i, k, jds + j);
            else dat(i, k, jds - j) = dat(i, k, jds + j);
          }
    }
    if (cf.symmetric_ye && d.jte == jde) {
      for (int j = 1; j <= BDYZONE; ++j)
        for (int k = d.kts; k <= k_end; ++k)
          for (int i = i_start; i <= i_end; ++i) {
            if (jstag == -1) dat(i, k, jde + j - 1) = dat(i, k, jde - j);
            else if (variable == 'v') dat(i, k, jde + j) = -dat(i, k, jde - j);
            else dat(i, k, jde + j) = dat(i, k, jde - j);
          }
    }
    // module_bc.F:1059-1107
    if (cf.open_ys && d.jts == jds && open_bc_copy3(variable)) {
      for (int k = d.kts; k <= k_end; ++k)
        for (int i = i_start; i <= i_end; ++i) {
          dat(i, k, jds - 1) = dat(i, k, jds);
          dat(i, k, jds - 2) = dat(i, k, jds);
          dat(i, k, jds - 3) = dat(i, k, jds);
        }
    }
    if (cf.open_ye && d.jte == jde && open_bc_copy3(variable)) {
      if (variable != 'v' && variable != 'y') {
        for (int k = d.kts; k <= k_end; ++k)
          for (int i = i_start; i <= i_end; ++i) {
            dat(i, k, jde) = dat(i, k, jde - 1);
            dat(i, k, jde + 1) = dat(i, k, jde - 1);
            dat(i, k, jde + 2) = dat(i, k, jde - 1);
          }
      } else {
        for (int k = d.kts; k <= k_end; ++k)
          for (int i = i_start; i <= i_end; ++i) {
            dat(i, k, jde + 1) = dat(i, k, jde);
            dat(i, k, jde + 2) = dat(i, k, jde);
            dat(i, k, jde + 3) = dat(i, k, jde);
          }
      }
    }
  }
  // (The 3-D fill has no separate corner pass: the y pass above copies whole
  //  rows i = ims..ime, x-halo included.)
}

template <typename R>
void set_physical_bc2d(R* dat_p, char variable_in, const WrfDynConfig& cf, const Dims& d) {
  A2<R> dat(dat_p, d);
  char variable = variable_in;
  if (variable_in >= 'A' && variable_in <= 'Z') variable = (char)(variable_in - 'A' + 'a');
  int istag = -1, jstag = -1;
  if (variable == 'u' || variable == 'x') istag = 0;
  if (variable == 'v' || variable == 'y') jstag = 0;
  if (variable == 'd') { istag = 0; jstag = 0; }
  if (variable == 'e') istag = 0;
  if (variable == 'f') jstag = 0;
  const int ids = d.ids, ide = d.ide, jds = d.jds, jde = d.jde;
  if (cf.periodic_x) {
    if (d.its == ids)
      for (int j = std::max(jds, d.jts - 1); j <= std::min(d.jte + 1, jde + jstag); ++j)
        for (int i = 0; i >= -(BDYZONE - 1); --i) dat(ids + i - 1, j) = dat(ide + i - 1, j);
    if (d.ite == ide)
      for (int j = std::max(jds, d.jts - 1); j <= std::min(d.jte + 1, jde + jstag); ++j)
        for (int i = -istag; i <= BDYZONE; ++i) dat(ide + i + istag, j) = dat(ids + i + istag, j);
  } else {
    // module_bc.F:276-314: note the 2-D 'u' branch loops i = 0..bdyzone-1.
    if (cf.symmetric_xs && d.its == ids) {
      for (int j = std::max(jds, d.jts - 1); j <= std::min(d.jte + 1, jde + jstag); ++j) {
        if (variable != 'u' && variable != 'x') {
          for (int i = 1; i <= BDYZONE; ++i) dat(ids - i, j) = dat(ids + i - 1, j);
        } else if (variable == 'u') {
          for (int i = 0; i <= BDYZONE - 1; ++i) dat(ids - i, j) = -dat(ids + i, j);
        } else {
          for (int i = 0; i <= BDYZONE - 1; ++i) dat(ids - i, j) = dat(ids + i, j);
        }
      }
    }
    if (cf.symmetric_xe && d.ite == ide) {
      for (int j = std::max(jds, d.jts - 1); j <= std::min(d.jte + 1, jde + jstag); ++j) {
        if (variable != 'u' && variable != 'x') {
          for (int i = 1; i <= BDYZONE; ++i) dat(ide + i - 1, j) = dat(ide - i, j);
        } else if (variable == 'u') {
          for (int i = 0; i <= BDYZONE - 1; ++i) dat(ide + i, j) = -dat(ide - i, j);
        } else {
          for (int i = 0; i <= BDYZONE - 1; ++i) dat(ide + i, j) = dat(ide - i, j);
        }
      }
    }
    // module_bc.F:386-427
    if (cf.open_xs && d.its == ids && open_bc_copy2(variable))
      for (int j = std::max(jds, d.jts - 1); j <= std::min(d.jte + 1, jde + jstag); ++j) {
        dat(ids - 1, j) = dat(ids, j);
        dat(ids - 2, j) = dat(ids, j);
        dat(ids - 3, j) = dat(ids, j);
      }
    if (cf.open_xe && d.ite == ide && open_bc_copy2(variable)) {
      for (int j = std::max(jds, d.jts - 1); j <= std::min(d.jte + 1, jde + jstag); ++j) {
        if (variable != 'u' && variable != 'x') {
          dat(ide, j) = dat(ide - 1, j);
          dat(ide + 1, j) = dat(ide - 1, j);
          dat(ide + 2, j) = dat(ide - 1, j);
        } else {
          dat(ide + 1, j) = dat(ide, j);
          dat(ide + 2, j) = dat(ide, j);
          dat(ide + 3, j) = dat(ide, j);
        }
      }
    }
  }
  int istart = std::max(ids, d.its - 1), iend = std::min(d.ite + 1, ide + istag);
  if (d.its == ids) istart = d.ims;
  if (d.ite == ide) iend = d.ime;
  if (cf.periodic_y) {
    if (d.jts == jds)
      for (int j = 0; j >= -(BDYZONE - 1); --j)
        for (int i = istart; i <= iend; ++i) dat(i, jds + j - 1) = dat(i, jde + j - 1);
    if (d.jte == jde)
      for (int j = -jstag; j <= BDYZONE; ++j)
        for (int i = istart; i <= iend; ++i) dat(i, jde + j + jstag) = dat(i, jds + j + jstag);
  } else {
    if (cf.symmetric_ys && d.jts == jds)
      for (int j = 1; j <= BDYZONE; ++j)
        for (int i = istart; i <= iend; ++i) {
          if (variable != 'v' && variable != 'y') dat(i, jds - j) = dat(i, jds + j - 1);
          else if (variable == 'v') dat(i, jds - j) = -dat(i, jds + j);
          else dat(i, jds - j) = dat(i, jds + j);
        }
    if (cf.symmetric_ye && d.jte == jde)
      for (int j = 1; j <= BDYZONE; ++j)
        for (int i = istart; i <= iend; ++i) {
          if (variable != 'v' && variable != 'y') dat(i, jde + j - 1) = dat(i, jde - j);
          else if (variable == 'v') dat(i, jde + j) = -dat(i, jde - j);
          else dat(i, jde + j) = dat(i, jde - j);
        }
    // module_bc.F:558-601
    if (cf.open_ys && d.jts == jds && open_bc_copy2(variable))
      for (int i = istart; i <= iend; ++i) {
        dat(i, jds - 1) = dat(i, jds);
        dat(i, jds - 2) = dat(i, jds);
        dat(i, jds - 3) = dat(i, jds);
      }
    if (cf.open_ye && d.jte == jde && open_bc_copy2(variable))
      for (int i = istart; i <= iend; ++i) {
        if (variable != 'v' && variable != 'y') {
          dat(i, jde) = dat(i, jde - 1);
          dat(i, jde + 1) = dat(i, jde - 1);
          dat(i, jde + 2) = dat(i, jde - 1);
        } else {
          dat(i, jde + 1) = dat(i, jde);
          dat(i, jde + 2) = dat(i, jde);
          dat(i, jde + 3) = dat(i, jde);
        }
      }
  }
  if (cf.periodic_x && cf.periodic_y) {
    if (d.its == ids && d.jts == jds)
      for (int j = 0; j >= -(BDYZONE - 1); --j)
        for (int i = 0; i >= -(BDYZONE - 1); --i) dat(ids + i - 1, jds + j - 1) = dat(ide + i - 1, jde + j - 1);
    if (d.ite == ide && d.jts == jds)
      for (int j = 0; j >= -(BDYZONE - 1); --j)
        for (int i = 1; i <= BDYZONE; ++i) dat(ide + i + istag, jds + j - 1) = dat(ids + i + istag, jde + j - 1);
    if (d.ite == ide && d.jte == jde)
      for (int j = 1; j <= BDYZONE; ++j)
        for (int i = 1; i <= BDYZONE; ++i) dat(ide + i + istag, jde + j + jstag) = dat(ids + i + istag, jds + j + jstag);
    if (d.its == ids && d.jte == jde)
      for (int j = 1; j <= BDYZONE; ++j)
        for (int i = 0; i >= -(BDYZONE - 1); --i) dat(ids + i - 1, jde + j + jstag) = dat(ide + i - 1, jds + j + jstag);
  }
}

}  // namespace wrforacle
