// advect_scalar_pd on the caller's device arrays, with no device allocation.
//
// Who needs it: a caller whose arrays already live on the GPU (a driver that
// keeps its state device-resident, e.g. a CUDA Fortran or OpenACC port of
// solve_em) and that cannot allocate at this point — its device memory is
// budgeted up front for the resident state, and cudaMalloc / cudaFree would
// also synchronize the device under its other streams.  The routine-level
// entry point wrfgpu_advect_scalar_pd copies host arrays into a cached device
// domain, which it allocates on first use; this variant runs the same two
// kernels (limiter factors, then the limited flux divergence; k_scalar.cu) on
// the caller's pointers and keeps the one scratch array they need, the
// per-cell limiter factor, in a fixed static device array.
//
// Limits and rules:
//   * the memory shape (ime-ims+1)(kme-kms+1)(jme-jms+1) may hold at most
//     NOALLOC_MAX_POINTS points (8 Mi: a 256 x 256 x 120 patch); larger
//     requests return WRFGPU_E_SIZE and launch nothing;
//   * the options are those a device domain accepts (periodic x, periodic or
//     symmetric y, 5th/3rd-order advection, ...): anything else returns
//     WRFGPU_E_ARG before any device work;
//   * nothing in the static arrays has to start at zero except the block
//     prefix's first entry, which the one-time setup writes: the factor pass
//     writes every factor the divergence pass reads, within the same call;
//   * the first call on a device (and the first after that device's primary
//     context was replaced, e.g. after cudaDeviceReset) does the setup —
//     symbol addresses through cudaGetSymbolAddress and one blocking copy —
//     so it should come before any stream capture; every call then enqueues
//     two things on the caller's stream: a one-thread kernel that writes the
//     member descriptor (passed by value as a kernel parameter, so no host
//     memory is read after the call returns) and the two PD kernels;
//   * the two PD kernels have no device-side failure (no bounded wait, no
//     health check): the return code reports argument and launch errors, and
//     there is no device status word to read back;
//   * the static arrays are shared: calls that overlap in time (two host
//     threads, or two streams without ordering between them) race on them.
//     Serialize calls on one stream or synchronize between them.
#include <cstring>
#include <mutex>
#include <cudaTypedefs.h>
#include "common.cuh"
#include "kernels.h"
#include "fcall.h"
#include "../../include/wrfgpu_fortran.h"

namespace wrfgpu {
namespace {

constexpr long long NOALLOC_MAX_POINTS = 8ll * 1024 * 1024;  // 32 MiB of FP32 factors

static __device__ __align__(256) float g_pd_factor[NOALLOC_MAX_POINTS];
static __device__ __align__(16) Mem g_member;
static __device__ int g_block_start[2];
static __device__ float* g_factor_table[1];

constexpr int MAX_DEVICES = 64;
struct DeviceSetup {
  bool done = false;
  CUcontext ctx = nullptr;  // the context the addresses below belong to
  float* factor = nullptr;
  Mem* member = nullptr;
  int* block_start = nullptr;
  float** factor_table = nullptr;
};
static DeviceSetup g_setup[MAX_DEVICES];
static std::mutex g_setup_mu;

// cuCtxGetCurrent from the driver (no link against libcuda): a device's
// static arrays move when its primary context is destroyed and re-created.
static PFN_cuCtxGetCurrent_v4000 g_ctx_current = nullptr;
static int current_context(CUcontext* ctx) {
  if (!g_ctx_current) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 4000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return WRFGPU_E_CUDA;
    g_ctx_current = (PFN_cuCtxGetCurrent_v4000)fn;
  }
  *ctx = nullptr;
  return g_ctx_current(ctx) == CUDA_SUCCESS && *ctx ? WRFGPU_OK : WRFGPU_E_CUDA;
}

// Once per device and context, with that device current: the addresses of
// the static arrays, and the two table entries the kernels read (no
// allocation).
int setup_current_device(DeviceSetup** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return WRFGPU_E_CUDA;
  // make the device's primary context current (initialised if need be)
  if (cudaSetDevice(dev) != cudaSuccess) return WRFGPU_E_CUDA;
  CUcontext ctx = nullptr;
  if (current_context(&ctx)) return WRFGPU_E_CUDA;
  std::lock_guard<std::mutex> lock(g_setup_mu);
  DeviceSetup& s = g_setup[dev];
  if (!s.done || s.ctx != ctx) {
    s.done = false;
    if (cudaGetSymbolAddress((void**)&s.factor, g_pd_factor) != cudaSuccess) return WRFGPU_E_CUDA;
    if (cudaGetSymbolAddress((void**)&s.member, g_member) != cudaSuccess) return WRFGPU_E_CUDA;
    if (cudaGetSymbolAddress((void**)&s.block_start, g_block_start) != cudaSuccess) return WRFGPU_E_CUDA;
    if (cudaGetSymbolAddress((void**)&s.factor_table, g_factor_table) != cudaSuccess) return WRFGPU_E_CUDA;
    if (cudaMemcpyToSymbol(g_factor_table, &s.factor, sizeof(float*)) != cudaSuccess) return WRFGPU_E_CUDA;
    const int zero = 0;
    if (cudaMemcpyToSymbol(g_block_start, &zero, sizeof(int)) != cudaSuccess) return WRFGPU_E_CUDA;
    s.ctx = ctx;
    s.done = true;
  }
  *out = &s;
  return WRFGPU_OK;
}

// The member descriptor, written on the stream from a kernel parameter.
__global__ void k_noalloc_set_member(Mem M, Mem* dst) { *dst = M; }

}  // namespace
}  // namespace wrfgpu

using namespace wrfgpu;

extern "C" int wrfgpu_advect_scalar_pd_noalloc(
    const float* field, const float* field_old, float* tendency, const float* ru, const float* rv, const float* rom,
    const float* c1, const float* c2, const float* mut, const float* mub, const float* mu_old,
    const WrfDynConfig* config_flags, const float* msftx, const float* msfty, const float* fzm, const float* fzp,
    const float* rdx, const float* rdy, const float* rdzw, const float* dt, WRFGPU_DIMS_ARGS, void* stream) {
  const int* d[18] = {ids, ide, jds, jde, kds, kde, ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte};
  for (int q = 0; q < 18; ++q)
    if (!d[q]) return WRFGPU_E_ARG;
  if (!field || !field_old || !tendency || !ru || !rv || !rom || !c1 || !c2 || !mut || !mub || !mu_old ||
      !config_flags || !msftx || !msfty || !fzm || !fzp || !rdx || !rdy || !rdzw || !dt)
    return WRFGPU_E_ARG;
  // the serial build's index space, one tile covering the patch (as the
  // routine-level entry points require)
  if (*ids != 1 || *jds != 1 || *kds != 1) return WRFGPU_E_ARG;
  if (*ims != 1 - WRFGPU_HALO || *ime != *ide + WRFGPU_HALO || *jms != 1 - WRFGPU_HALO ||
      *jme != *jde + WRFGPU_HALO || *kms != 1 || *kme != *kde)
    return WRFGPU_E_ARG;
  if (*its != 1 || *ite != *ide || *jts != 1 || *jte != *jde || *kts != 1 || *kte != *kde) return WRFGPU_E_ARG;
  if (*ide < 8 || *jde < 8 || *kde < 6 || *kde > 128) return WRFGPU_E_ARG;  // the limits of a member
  const long long ni = *ime - *ims + 1, nk = *kme - *kms + 1, nj = *jme - *jms + 1;
  if (ni * nk * nj > NOALLOC_MAX_POINTS) return WRFGPU_E_SIZE;
  if (!(*dt > 0.f) || !(*rdx > 0.f) || !(*rdy > 0.f)) return WRFGPU_E_ARG;
  {  // the options a device domain accepts
    WrfGpuDomainDesc d{};
    d.ide = *ide; d.jde = *jde; d.kde = *kde; d.n_moist = 1; d.n_scalar = 0;
    d.config = *config_flags;
    d.scalars.dt = *dt; d.scalars.dx = 1.0 / *rdx; d.scalars.dy = 1.0 / *rdy;
    d.scalars.rdx = *rdx; d.scalars.rdy = *rdy;
    if (check_desc(d)) return WRFGPU_E_ARG;
  }

  DeviceSetup* s = nullptr;
  int rc = setup_current_device(&s);
  if (rc) return rc;

  Mem M;
  std::memset(&M, 0, sizeof(Mem));
  M.ids = *ids; M.ide = *ide; M.jds = *jds; M.jde = *jde; M.kds = *kds; M.kde = *kde;
  M.ims = *ims; M.ime = *ime; M.jms = *jms; M.jme = *jme; M.kms = *kms; M.kme = *kme;
  M.its = *its; M.ite = *ite; M.jts = *jts; M.jte = *jte; M.kts = *kts; M.kte = *kte;
  M.sk = ni; M.sj = ni * nk; M.s2 = ni;
  M.f3[WRFGPU_RU_M] = const_cast<float*>(ru);
  M.f3[WRFGPU_RV_M] = const_cast<float*>(rv);
  M.f3[WRFGPU_WW_M] = const_cast<float*>(rom);
  M.f3[WRFGPU_ADVECT_TEND] = tendency;
  M.f2[WRFGPU_MUTS - WRFGPU_F2D_BASE] = const_cast<float*>(mut);
  M.f2[WRFGPU_MUB - WRFGPU_F2D_BASE] = const_cast<float*>(mub);
  M.f2[WRFGPU_MU_1 - WRFGPU_F2D_BASE] = const_cast<float*>(mu_old);
  M.f2[WRFGPU_MSFTX - WRFGPU_F2D_BASE] = const_cast<float*>(msftx);
  M.f2[WRFGPU_MSFTY - WRFGPU_F2D_BASE] = const_cast<float*>(msfty);
  M.f1[WRFGPU_C1H - WRFGPU_F1D_BASE] = const_cast<float*>(c1);
  M.f1[WRFGPU_C2H - WRFGPU_F1D_BASE] = const_cast<float*>(c2);
  M.f1[WRFGPU_FNM - WRFGPU_F1D_BASE] = const_cast<float*>(fzm);
  M.f1[WRFGPU_FNP - WRFGPU_F1D_BASE] = const_cast<float*>(fzp);
  M.f1[WRFGPU_RDNW - WRFGPU_F1D_BASE] = const_cast<float*>(rdzw);
  M.q[0] = const_cast<float*>(field);
  M.qo[0] = const_cast<float*>(field_old);
  M.nsp = 1; M.n_moist = 1;
  M.ns_total = 1;
  M.dt = *dt; M.dtrk_fix = *dt;
  M.rdx = *rdx; M.rdy = *rdy;
  M.cf = *config_flags;
  M.err = nullptr;  // the PD kernels raise no device status

  cudaStream_t st = (cudaStream_t)stream;
  k_noalloc_set_member<<<1, 1, 0, st>>>(M, s->member);
  if (cudaGetLastError() != cudaSuccess) return WRFGPU_E_CUDA;
  const int nb = blocks_for(M.ims, M.ime, M.jms, M.jme, (int)nk, 3);
  const Launch L{s->member, s->block_start, 1, 3};
  // rk_step 3 (the last stage, where the reference applies the PD scheme);
  // flags 2 | 4: limiter on regardless of the configuration's scheme, and
  // the tendency accumulates into the caller's array, as advect_scalar_pd does
  launch_advect_scalar_pd2(L, nb, StepArgs{3, 0, 0, 6}, s->factor_table, st);
  if (cudaGetLastError() != cudaSuccess) return WRFGPU_E_CUDA;
  return WRFGPU_OK;
}
