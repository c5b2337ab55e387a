// Internal interface between the routine-level C ABI (fortran_abi.cu) and
// the device runtime (driver.cu): one model-layer call in parity mode.
#pragma once
#include <vector>
#include "../../include/wrfgpu.h"

namespace wrfgpu {

// One array argument: the device field it is bound to, the caller's array
// (uploaded before the call if `in`, downloaded after it if `out`).
struct FBind {
  int id;           // field id (WRFGPU_*), species ids included
  float* host;
  bool in, out;
};

struct FCall {
  int routine = 0;                  // WRFGPU_R_*
  int rk_step = 1, iteration = 0, species = 0;
  const int* dims[18] = {};         // ids..kde, ims..kme, its..kte
  WrfDynConfig cfg{};
  int nsp = 1;                      // species of the scratch domain
  // scalars given by the caller (NaN / <= 0: not given)
  float rdx = -1.f, rdy = -1.f, dt = -1.f, dts = -1.f, dtrk = -1.f;
  float epssm = -1.f, smdiv = -1.f, emdiv = -1.f, cf1 = 0.f, cf2 = 0.f, cf3 = 0.f, cfn = 0.f, cfn1 = 0.f;
  bool have_cf = false, have_cfn = false;
  float p_top = -1.f;
  int nsmall = 0;
  bool zero_saves = false;          // rk_tendency: zero the *_save / mu_tend outputs
  std::vector<int> zero_ids;        // fields set to zero before the routine (unbound inputs read as 0)
  float* max_vert_cfl = nullptr;    // rk_tendency diagnostics
  float* max_horiz_cfl = nullptr;
  std::vector<FBind> binds;
  void bind(int id, const float* p, bool in, bool out) {
    if (p) binds.push_back(FBind{id, const_cast<float*>(p), in, out});
  }
};

int fortran_call(const FCall& c);
// The options a domain (or a routine-level call) may use: 0 or WRFGPU_E_ARG.
int check_desc(const WrfGpuDomainDesc& d);
int fortran_release();

}  // namespace wrfgpu
