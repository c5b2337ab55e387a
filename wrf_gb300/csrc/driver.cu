// Host runtime: device-resident domains/ensembles, the solve_em large-step
// sequence, CUDA-graph capture and the coarse C ABI of include/wrfgpu.h.
//
// The step sequence follows dyn_em/solve_em.F:578-4750 for the physics-off
// options, with each of the reference's halo-exchange / boundary-fill sync
// sites (HALO_EM_A/B/C/C2/D*, PERIOD_BDY_*, set_physical_bc*) mapped to a
// kernel boundary plus one batched on-device halo-fill launch.  A plain
// domain is an ensemble of one member; an ensemble of uneven members runs
// the same launches with every kernel covering all members' blocks.
//
// Two calls of the reference that provably leave the state unchanged are not
// issued: rk_addtend_dry adds physics tendencies that are identically zero
// with physics off unless a diffusion or the Rayleigh damping stores
// tendencies (module_em.F:959-1092; k_diff.cu issues it then), and the post-RK calc_p_rho_phi
// (solve_em.F:4180-4203) recomputes al and p from the same inputs as the
// stage-3 call.  initialize_moist_old (solve_em.F:517-527) is also skipped:
// moist_old is overwritten by rk_update_scalar before any read.
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <vector>
#include <string>
#include <algorithm>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include "common.cuh"
#include "kernels.h"
#include "open_adv.cuh"
#include "fcall.h"
#include <map>
#include <mutex>
#include <tuple>
#include "../../include/wrfgpu.h"

namespace wrfgpu {

#define CK(x)                                                                                  \
  do {                                                                                         \
    cudaError_t e_ = (x);                                                                      \
    if (e_ != cudaSuccess) {                                                                   \
      std::fprintf(stderr, "wrfgpu: CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
      return WRFGPU_E_CUDA;                                                                    \
    }                                                                                          \
  } while (0)

// Profiling phases (the reference's BENCH timer vocabulary, inc/bench_solve_em_def.h,
// refined to one entry per kernel family).
enum Phase {
  PH_PREP = 0, PH_FILL, PH_TEND_U, PH_TEND_V, PH_TEND_W, PH_TEND_T, PH_TEND_PH, PH_CFL, PH_SSP, PH_CPR0,
  PH_COEFW, PH_AUV, PH_AMUT, PH_AW, PH_SUMF, PH_SSF, PH_USPD, PH_PD, PH_ADVS, PH_UPDS, PH_CPRP, PH_WSURF,
  PH_DIFF, PH_END, NPHASE
};
static const char* PHASE_NAMES[NPHASE] = {
    "step_prep", "bc_fill", "rk_tend_u", "rk_tend_v", "rk_tend_w", "rk_tend_t", "rk_tend_ph", "cfl_check",
    "small_step_prep", "calc_p_rho_0", "calc_coef_w", "advance_uv", "advance_mu_t", "advance_w",
    "sumflux_calc_p_rho", "small_step_finish", "rk_update_scalar_pd", "scalar_pd_update", "scalar_adv_update",
    "rk_update_scalar", "calc_p_rho_phi", "set_w_surface", "sixth_order_diffusion", "end"};

int check_desc(const WrfGpuDomainDesc& d) {
  const WrfDynConfig& c = d.config;
  if (d.ide < 8 || d.jde < 8 || d.kde < 6 || d.kde > 128) return WRFGPU_E_ARG;
  if (d.n_moist != 1 || d.n_scalar < 0 || d.n_moist + d.n_scalar > NSPMAX) return WRFGPU_E_ARG;
  if (c.rk_ord != 3 || c.h_mom_adv_order != 5 || c.h_sca_adv_order != 5 || c.v_mom_adv_order != 3 ||
      c.v_sca_adv_order != 3)
    return WRFGPU_E_ARG;
  if (!c.non_hydrostatic || c.zadvect_implicit != 0 || (c.damp_opt != 0 && c.damp_opt != 2 && c.damp_opt != 3) ||
      (c.w_damping != 0 && c.w_damping != 1) || (c.diff_opt != 0 && c.diff_opt != 1))
    return WRFGPU_E_ARG;
  // explicit diffusion with the constant coefficients of km_opt = 1
  if (c.diff_opt == 1 && (c.km_opt != 1 || !(c.khdif >= 0.f) || !(c.kvdif >= 0.f))) return WRFGPU_E_ARG;
  if (c.damp_opt == 2 && !(c.zdamp > 0.f)) return WRFGPU_E_ARG;
  if (c.diff_6th_opt < 0 || c.diff_6th_opt > 2) return WRFGPU_E_ARG;
  // lateral boundaries, one condition per side (share/module_bc.F:60-133):
  // x periodic or open on both sides, y periodic, symmetric or open on both
  if (c.specified || c.nested || c.polar || c.symmetric_xs || c.symmetric_xe) return WRFGPU_E_ARG;
  const bool ox = c.open_xs && c.open_xe, oy = c.open_ys && c.open_ye;
  const bool sy = c.symmetric_ys && c.symmetric_ye;
  if (c.open_xs != c.open_xe || c.open_ys != c.open_ye || c.symmetric_ys != c.symmetric_ye) return WRFGPU_E_ARG;
  if ((c.periodic_x != 0) == ox) return WRFGPU_E_ARG;
  if ((c.periodic_y != 0) + sy + oy != 1) return WRFGPU_E_ARG;
  // the edge strips of the two open sides of a direction do not overlap
  if ((ox && d.ide < 12) || (oy && d.jde < 12)) return WRFGPU_E_ARG;
  if (c.hypsometric_opt != 1 && c.hypsometric_opt != 2) return WRFGPU_E_ARG;
  if (d.scalars.dt <= 0 || d.scalars.dx <= 0 || d.scalars.dy <= 0) return WRFGPU_E_ARG;
  // the kernels index a field with 32-bit offsets
  const long long pts = (long long)(d.ide + 2 * WRFGPU_HALO + 4) * d.kde * (d.jde + 2 * WRFGPU_HALO);
  if (pts >= (1ll << 31)) return WRFGPU_E_ARG;
  return WRFGPU_OK;
}

// cuTensorMapEncodeTiled from the driver (no link against libcuda).
static PFN_cuTensorMapEncodeTiled_v12000 g_encode_tiled = nullptr;
static int get_tensor_map_encoder() {
  if (g_encode_tiled) return WRFGPU_OK;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return WRFGPU_E_CUDA;
  g_encode_tiled = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  return WRFGPU_OK;
}
// 3-D FP32 field (i fastest, row pitch `pitch` elements), box bx x 1 x by.
static int encode_field_map(CUtensorMap* out, float* base, size_t ni, size_t pitch, size_t nk, size_t nj, int bx,
                            int by) {
  cuuint64_t dims[3] = {(cuuint64_t)ni, (cuuint64_t)nk, (cuuint64_t)nj};
  cuuint64_t strides[2] = {(cuuint64_t)(pitch * 4), (cuuint64_t)(pitch * nk * 4)};
  cuuint32_t box[3] = {(cuuint32_t)bx, 1u, (cuuint32_t)by};
  cuuint32_t es[3] = {1u, 1u, 1u};
  CUresult r = g_encode_tiled(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, es,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? WRFGPU_OK : WRFGPU_E_CUDA;
}

static int num_sound_steps(const WrfGpuDomainDesc& d) {
  if (d.config.time_step_sound != 0) return d.config.time_step_sound;
  float spacing = std::min((float)d.scalars.dx, (float)d.scalars.dy);
  return std::max(2 * ((int)(300.f * (float)d.scalars.dt / spacing - 0.01f) + 1), 4);
}

struct Ensemble {
  int nmem = 0;
  int flags = 0;
  bool fp64 = false;
  std::vector<WrfGpuDomainDesc> descs;
  std::vector<Mem> hm;                 // host copies of the member descriptors
  Mem* d_mems = nullptr;
  int *d_bs2 = nullptr, *d_bs3 = nullptr, *d_bs_st = nullptr, *d_bs_tm = nullptr;
  int* d_bs_pr = nullptr;  // mass tiles x pairs of species (the scalar transport)
  int nb2 = 0, nb3 = 0, nb_st = 0, nb_tm = 0, nb_pr = 0;
  // edge strips of members with open lateral boundaries (strip columns x
  // levels): the tendencies and the 5th/3rd-order transport, the PD
  // transport, and its limiter factors (one wider, halo included)
  int *d_bs_s3 = nullptr, *d_bs_s4 = nullptr, *d_bs_s5 = nullptr;
  int nb_s3 = 0, nb_s4 = 0, nb_s5 = 0;
  bool any_open = false;
  bool capturing = false;
  int capture_swaps = 0;               // species-buffer swaps in one captured step
  int nsp_max = 0, ns_max = 0, nlev_max = 0;
  bool damp3 = false;  // some member uses damp_opt = 3
  bool diff6 = false;  // some member stores diffusion tendencies (diff_6th_opt != 0 or diff_opt = 1)
  bool damp2 = false;  // some member uses damp_opt = 2 (Rayleigh damping toward the base state)
  std::vector<size_t> n3, n2, n1;      // element counts per member (padded rows)
  std::vector<size_t> ni_, nk_, nj_, pitch_;  // Fortran extents and the padded row pitch
  CUtensorMap* d_tmaps = nullptr;      // [nmem][NMAPSLOT][2]
  char* pool = nullptr;                // one device allocation for all fields
  size_t pool_bytes = 0;
  float** d_pd_scratch = nullptr;      // per-member limiter scratch pointers
  unsigned* d_err = nullptr;
  float* d_cfl = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool cfl_check = true;
  int halo_blocks = 64;
  // launch variant of each tuned kernel family (kernels.h), and what the
  // autotuner measured: ms per step of family f with variant v (-1: not timed)
  int tune[NTUNE];
  float tune_ms[NTUNE][TUNE_MAXVAR];
  Ensemble() {
    for (int f = 0; f < NTUNE; ++f) {
      tune[f] = TUNE_DEFAULT[f];
      for (int v = 0; v < TUNE_MAXVAR; ++v) tune_ms[f][v] = -1.f;
    }
  }
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<std::pair<int, cudaEvent_t>>* prof = nullptr;  // per-launch marks when profiling

  void mark(int ph) {
    if (!prof) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, stream);
    prof->push_back({ph, e});
  }

  Launch L2() const { return Launch{d_mems, d_bs2, nmem, 2}; }
  Launch L3() const { return Launch{d_mems, d_bs3, nmem, 3}; }
  TileLaunch LP() const { return TileLaunch{d_mems, d_bs_pr, nmem}; }  // tiles x species pairs
  TileLaunch LST() const { return TileLaunch{d_mems, d_bs_st, nmem}; }  // staggered-extent tiles
  TileLaunch LTM() const { return TileLaunch{d_mems, d_bs_tm, nmem}; }  // mass-extent tiles
  StripLaunch LS3() const { return StripLaunch{d_mems, d_bs_s3, nmem, STRIP_W_TEND, 0}; }
  StripLaunch LS4() const { return StripLaunch{d_mems, d_bs_s4, nmem, STRIP_W_PD, 0}; }
  StripLaunch LS5() const { return StripLaunch{d_mems, d_bs_s5, nmem, STRIP_W_PD + 1, 1}; }

  // The fused scalar update writes the new value into the spare buffer; the
  // swap kernel exchanges (q, qa) in the device member table and the host
  // mirror follows, so field access always sees the current buffer.
  void host_flip() {
    for (int m = 0; m < nmem; ++m)
      for (int s = 0; s < hm[m].nsp; ++s) {
        std::swap(hm[m].q[s], hm[m].qa[s]);
        std::swap(hm[m].qmap[s], hm[m].qamap[s]);
      }
  }
  void swap_species() {
    launch_swap_species(d_mems, nmem, stream);
    host_flip();
    if (capturing) ++capture_swaps;
  }

  // Contiguous device staging buffer of the host <-> device field copies
  // (allocated on first use, sized to the largest field): a field crosses the
  // host link as one contiguous copy, and a kernel moves it between the
  // caller's contiguous rows and the device's padded rows.
  float* d_stage = nullptr;
  size_t stage_n = 0;
  int ensure_stage(size_t n) {
    if (n <= stage_n) return WRFGPU_OK;
    if (d_stage) cudaFree(d_stage);
    d_stage = nullptr;
    stage_n = 0;
    if (cudaMalloc(&d_stage, n * 4) != cudaSuccess) return WRFGPU_E_CUDA;
    stage_n = n;
    return WRFGPU_OK;
  }

  // ---------------------------------------------------------------- host I/O step
  // Host buffers bound to the step (wrfgpu_bind_host_state).  Every
  // step_host() step copies each `in` buffer into its field before the
  // solver's kernels and each field into its `out` buffer after them, all in
  // one captured graph: the passive scalars, first read by stage 1's scalar
  // transport, cross the host link on a second stream while stage 1's
  // dynamics run; everything else (the dry state and the moist species, read
  // from the first kernel on) before the step, and the downloads after it.
  struct HostIO {
    int member = 0, id = 0;
    int species = -1;        // >= 0: the current value of that species (buffers looked up on the device)
    bool late = false;       // a passive scalar: may arrive while stage 1's dynamics run
    const float* in = nullptr;
    float* out = nullptr;
    float* dev = nullptr;    // a fixed field buffer (species < 0)
    size_t count = 0, cols = 0, rows = 0, pitch = 0;
    float* stage = nullptr;  // contiguous device copy
    bool prefetch = false;   // the next step's input may cross during this step's last stage
    bool tail = false;       // the next step's input may cross right behind this step's final downloads
  };
  std::vector<HostIO> hio;
  cudaStream_t cstream = nullptr;  // downloads of the host I/O step that overlap its kernels
  cudaStream_t ustream = nullptr;  // uploads of the host I/O step that overlap its kernels
  std::vector<cudaEvent_t> ev_dn;  // per bound field: its overlapped download is complete
  cudaEvent_t ev_head = nullptr, ev_ojoin2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // [head][prefetch]: head = the previous step's deferred downloads come
  // first; prefetch = the next step's early inputs cross during this one
  cudaGraph_t graph_io[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  cudaGraphExec_t gexec_io[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  bool io_prefetch = false;  // enqueue_step: the dry downloads are followed by the next step's uploads
  int io_swaps = 0;  // species-buffer swaps in one captured I/O step
  bool io_pending = false;  // enqueue_step: the copy-in branch is still to be joined
  bool io_step = false;     // enqueue_step runs inside a host I/O step
  bool io_out_pending = false;
  cudaEvent_t ev_ofork = nullptr, ev_ojoin = nullptr, ev_dryin = nullptr;
  cudaEvent_t ev_tfork = nullptr, ev_tjoin = nullptr, ev_tjoin2 = nullptr;
  // stage 1's transport of a host I/O step in two launches: the pairs whose
  // passive scalars cross in the first three quarters of the uploads (after
  // ev_upA), then the rest (after every upload)
  bool io_split = false;
  unsigned io_pairs_early = ~0u;
  cudaEvent_t ev_upA = nullptr;
  // moist species downloaded right after the last stage's transport (their
  // halo fill issued first), while calc_p_rho_phi runs
  std::vector<char> io_moist_done;
  cudaEvent_t ev_mfork = nullptr;
  bool io_moist_out() {
    bool any = false;
    for (const HostIO& b : hio) any = any || (b.out && b.species >= 0 && !b.late);
    if (!any) return false;
    cudaEventRecord(ev_mfork, stream);
    cudaStreamWaitEvent(cstream, ev_mfork, 0);
    io_moist_done.assign(hio.size(), 0);
    for (size_t q = 0; q < hio.size(); ++q)
      if (hio[q].out && hio[q].species >= 0 && !hio[q].late) {
        copy_out(hio[q], cstream);
        cudaEventRecord(ev_dn[q], cstream);
        io_moist_done[q] = 1;
      }
    return true;
  }

  void io_join() {
    if (!io_pending) return;
    cudaStreamWaitEvent(stream, ev_join, 0);
    cudaStreamWaitEvent(stream, ev_head, 0);
    io_pending = false;
  }
  // Upload of field q on ustream after the downloads of this phase that use
  // its staging buffer or write its host input (dn[g]: g's download is in
  // this phase).
  void upload_after(size_t q, const std::vector<char>& dn) {
    const HostIO& b = hio[q];
    const char* lo = (const char*)b.in;
    const char* hi = lo + b.count * 4;
    for (size_t g = 0; g < hio.size(); ++g) {
      if (!dn[g]) continue;
      const char* glo = (const char*)hio[g].out;
      const char* ghi = glo + hio[g].count * 4;
      if (g == q || (lo < ghi && glo < hi)) cudaStreamWaitEvent(ustream, ev_dn[g], 0);
    }
    cudaMemcpyAsync(b.stage, b.in, b.count * 4, cudaMemcpyHostToDevice, ustream);
  }
  // the _2 dry state is final once the last stage's fills and set_w_surface
  // are done (enqueue_step): its bound outputs cross the link on the copy
  // stream while the scalars advance
  static bool early_out(const HostIO& b) {
    return b.species < 0 && (b.id == WRFGPU_U_2 || b.id == WRFGPU_V_2 || b.id == WRFGPU_W_2 ||
                             b.id == WRFGPU_T_2 || b.id == WRFGPU_PH_2 || b.id == WRFGPU_MU_2);
  }
  void copy_out(const HostIO& b, cudaStream_t st) {
    if (b.species >= 0)
      launch_pack_species(d_mems, b.member, b.species, b.stage, (int)b.cols, (int)b.rows, (int)b.pitch, st);
    else
      launch_pack_rows(b.dev, b.stage, (int)b.cols, (int)b.rows, (int)b.pitch, st);
    cudaMemcpyAsync(b.out, b.stage, b.count * 4, cudaMemcpyDeviceToHost, st);
  }
  void io_dry_out() {
    if (!io_step) return;
    bool any = false;
    for (const HostIO& b : hio) any = any || (b.out && early_out(b)) || (io_prefetch && b.prefetch);
    if (!any) return;
    cudaEventRecord(ev_ofork, stream);
    cudaStreamWaitEvent(cstream, ev_ofork, 0);
    cudaStreamWaitEvent(ustream, ev_ofork, 0);
    std::vector<char> dn(hio.size(), 0);
    for (size_t q = 0; q < hio.size(); ++q)
      if (hio[q].out && early_out(hio[q])) {
        copy_out(hio[q], cstream);
        cudaEventRecord(ev_dn[q], cstream);
        dn[q] = 1;
      }
    // the next step's inputs that no later download of this step can change,
    // on the other copy engine direction, each after the downloads it waits for
    if (io_prefetch)
      for (size_t q = 0; q < hio.size(); ++q)
        if (hio[q].prefetch) upload_after(q, dn);
    cudaEventRecord(ev_ojoin, cstream);
    cudaEventRecord(ev_ojoin2, ustream);
    io_out_pending = true;
  }
  // An early input (the dry state, moist species) may be uploaded during the
  // previous step's last stage when its staging buffer is free then (no
  // output, or an output downloaded at that same point) and its host array
  // overlaps no output downloaded later in the step.
  // Every other early input may cross at the end of the previous step, each
  // behind the final downloads that free its staging buffer or write its host
  // input, unless a passive scalar's download (left for the next step's
  // head) writes part of its host input.
  void set_prefetch() {
    for (HostIO& b : hio) {
      b.prefetch = b.in && !b.late && (!b.out || early_out(b));
      b.tail = false;
      if (!b.prefetch) continue;
      const char* lo = (const char*)b.in;
      const char* hi = lo + b.count * 4;
      for (const HostIO& g : hio) {
        if (!g.out || early_out(g)) continue;
        const char* glo = (const char*)g.out;
        const char* ghi = glo + g.count * 4;
        if (lo < ghi && glo < hi) { b.prefetch = false; break; }
      }
    }
    for (HostIO& b : hio) {
      if (!b.in || b.late || b.prefetch) continue;
      b.tail = true;
      const char* lo = (const char*)b.in;
      const char* hi = lo + b.count * 4;
      for (const HostIO& g : hio) {
        if (!g.out || !deferrable(g)) continue;
        const char* glo = (const char*)g.out;
        const char* ghi = glo + g.count * 4;
        if (lo < ghi && glo < hi) { b.tail = false; break; }
      }
    }
  }
  void drop_io_graph() {
    for (int h = 0; h < 2; ++h)
      for (int v = 0; v < 2; ++v) {
        if (gexec_io[h][v]) { cudaGraphExecDestroy(gexec_io[h][v]); gexec_io[h][v] = nullptr; }
        if (graph_io[h][v]) { cudaGraphDestroy(graph_io[h][v]); graph_io[h][v] = nullptr; }
      }
  }
  void unbind_host() {
    drop_io_graph();
    for (HostIO& b : hio) if (b.stage) cudaFree(b.stage);
    hio.clear();
  }
  int bind_host(int member, int nfield, const int* ids, const float* const* in, float* const* out,
                const long long* n) {
    if (member < 0 || member >= nmem || nfield <= 0 || !ids || !n || (!in && !out)) return WRFGPU_E_ARG;
    std::vector<HostIO> add;
    for (int f = 0; f < nfield; ++f) {
      HostIO b;
      b.member = member; b.id = ids[f];
      b.in = in ? in[f] : nullptr;
      b.out = out ? out[f] : nullptr;
      b.dev = field_ptr(member, b.id, &b.count, &b.cols, &b.rows, &b.pitch);
      if (!b.dev || (long long)b.count != n[f] || (!b.in && !b.out)) return WRFGPU_E_ARG;
      // the copies are graph nodes: the host buffers must be page-locked
      for (const void* hp : {(const void*)b.in, (const void*)b.out}) {
        if (!hp) continue;
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, hp) != cudaSuccess || at.type != cudaMemoryTypeHost) {
          cudaGetLastError();
          return WRFGPU_E_ARG;
        }
      }
      const int sid = b.id - WRFGPU_SPECIES_BASE;
      if (sid >= 0 && sid % 2 == 0) {
        b.species = sid / 2;
        b.late = b.species >= hm[member].n_moist;
        b.dev = nullptr;
      }
      add.push_back(b);
    }
    for (HostIO& b : add) {
      if (cudaMalloc(&b.stage, b.count * 4) != cudaSuccess) {
        for (HostIO& c : add) if (c.stage) cudaFree(c.stage);
        return WRFGPU_E_NOMEM;
      }
    }
    drop_io_graph();
    for (HostIO& b : add) {  // a later binding of the same field replaces the earlier one
      for (size_t q = 0; q < hio.size(); ++q)
        if (hio[q].member == b.member && hio[q].id == b.id) {
          cudaFree(hio[q].stage);
          hio.erase(hio.begin() + q);
          break;
        }
      hio.push_back(b);
    }
    set_prefetch();
    return WRFGPU_OK;
  }
  // one step with its copies, enqueued on `stream` (and `cstream`)
  int io_streams() {
    while (ev_dn.size() < hio.size()) {
      cudaEvent_t e;
      CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      ev_dn.push_back(e);
    }
    if (cstream) return WRFGPU_OK;
    // the copy streams' pack / unpack kernels take SM slots ahead of the
    // step's waiting blocks, so a copy does not wait for a long kernel to drain
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CK(cudaStreamCreateWithPriority(&cstream, cudaStreamNonBlocking, greatest));
    CK(cudaStreamCreateWithPriority(&ustream, cudaStreamNonBlocking, greatest));
    for (cudaEvent_t* e : {&ev_fork, &ev_join, &ev_ofork, &ev_ojoin, &ev_dryin, &ev_head, &ev_ojoin2, &ev_tfork,
                           &ev_tjoin, &ev_tjoin2, &ev_upA, &ev_mfork})
      CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    return WRFGPU_OK;
  }
  // A passive scalar's download may wait for the head of the next step of the
  // same call: it then crosses the link while that step uploads the dry state
  // and runs stage 1's dynamics (the device buffers are not touched before
  // stage 1's scalar transport, and the same copy stream uploads the scalar's
  // next input only after it).
  static bool deferrable(const HostIO& b) { return b.species >= 0 && b.late; }
  // One step with its copies, enqueued on `stream` and `cstream`.  head: the
  // previous step's deferred downloads first; defer: this step's passive
  // scalars left for the next step's head (or flush_deferred).
  int enqueue_io_step(bool head, bool defer, bool pre) {
    if (int rc = io_streams()) return rc;
    auto unpack = [&](const HostIO& b, cudaStream_t st) {
      if (b.species >= 0)
        launch_unpack_species(d_mems, b.member, b.species, b.stage, (int)b.cols, (int)b.rows, (int)b.pitch, st);
      else
        launch_unpack_rows(b.stage, b.dev, nullptr, (int)b.cols, (int)b.rows, (int)b.pitch, st);
    };
    bool late = false;
    for (const HostIO& b : hio) late = late || (b.in && b.late);
    CK(cudaEventRecord(ev_fork, stream));
    CK(cudaStreamWaitEvent(cstream, ev_fork, 0));
    CK(cudaStreamWaitEvent(ustream, ev_fork, 0));
    // the previous step's deferred downloads on one copy direction ...
    std::vector<char> dn(hio.size(), 0);
    if (head)
      for (size_t q = 0; q < hio.size(); ++q)
        if (hio[q].out && deferrable(hio[q])) {
          copy_out(hio[q], cstream);
          CK(cudaEventRecord(ev_dn[q], cstream));
          dn[q] = 1;
        }
    CK(cudaEventRecord(ev_head, cstream));
    // ... the dry state and the moist species first on the other, at the
    // link's full rate (those prefetched during the previous step are across)
    for (const HostIO& b : hio)
      if (b.in && !b.late && !(head && (b.prefetch || b.tail)))
        CK(cudaMemcpyAsync(b.stage, b.in, b.count * 4, cudaMemcpyHostToDevice, stream));
    CK(cudaEventRecord(ev_dryin, stream));
    for (const HostIO& b : hio)
      if (b.in && !b.late) unpack(b, stream);
    // then the passive scalars, each after its own deferred download
    CK(cudaStreamWaitEvent(ustream, ev_dryin, 0));
    std::vector<size_t> lq;  // late inputs in upload order
    for (size_t q = 0; q < hio.size(); ++q)
      if (hio[q].in && hio[q].late) lq.push_back(q);
    // the pairs none of whose passive scalars is among the last quarter of
    // the uploads are transported as soon as their own uploads are in
    // (the stage-1 diffusion of the species reads them all: no split then)
    io_split = false;
    io_pairs_early = ~0u;
    size_t na = 0;
    if (lq.size() >= 4 && !diff6) {
      const size_t thr = (3 * lq.size() + 3) / 4;
      unsigned late_b = 0;
      for (size_t r = thr; r < lq.size(); ++r) late_b |= 1u << (hio[lq[r]].species / 2);
      for (size_t r = 0; r < lq.size(); ++r)
        if (!((late_b >> (hio[lq[r]].species / 2)) & 1u)) na = r + 1;
      io_pairs_early = ~late_b;
      io_split = late_b != 0 && na > 0;
    }
    for (size_t r = 0; r < lq.size(); ++r) {
      upload_after(lq[r], dn);
      unpack(hio[lq[r]], ustream);
      if (io_split && r + 1 == na) CK(cudaEventRecord(ev_upA, ustream));
    }
    CK(cudaEventRecord(ev_join, ustream));
    io_pending = true;
    io_step = true;
    io_prefetch = pre;
    io_out_pending = false;
    io_moist_done.assign(hio.size(), 0);
    enqueue_step();
    io_step = false;
    io_prefetch = false;
    io_join();
    (void)late;
    if (io_out_pending) {
      CK(cudaStreamWaitEvent(stream, ev_ojoin, 0));
      CK(cudaStreamWaitEvent(stream, ev_ojoin2, 0));
      io_out_pending = false;
    }
    if (!pre) {
      for (const HostIO& b : hio)
        if (b.out && !early_out(b) && !(defer && deferrable(b))) copy_out(b, stream);
    } else {
      // the final downloads on one link direction and, behind each, the next
      // step's inputs that wait for it on the other
      CK(cudaEventRecord(ev_tfork, stream));
      CK(cudaStreamWaitEvent(cstream, ev_tfork, 0));
      CK(cudaStreamWaitEvent(ustream, ev_tfork, 0));
      std::vector<char> tdn(hio.size(), 0);
      for (size_t q = 0; q < hio.size(); ++q) {
        const HostIO& b = hio[q];
        if (!b.out || early_out(b) || (defer && deferrable(b))) continue;
        tdn[q] = 1;
        if (io_moist_done[q]) continue;  // downloaded after the last transport
        copy_out(b, cstream);
        CK(cudaEventRecord(ev_dn[q], cstream));
        tdn[q] = 1;
      }
      for (size_t q = 0; q < hio.size(); ++q)
        if (hio[q].tail) upload_after(q, tdn);
      CK(cudaEventRecord(ev_tjoin, cstream));
      CK(cudaEventRecord(ev_tjoin2, ustream));
      CK(cudaStreamWaitEvent(stream, ev_tjoin, 0));
      CK(cudaStreamWaitEvent(stream, ev_tjoin2, 0));
    }
    CK(cudaGetLastError());
    return WRFGPU_OK;
  }
  int flush_deferred() {
    for (const HostIO& b : hio)
      if (b.out && deferrable(b)) copy_out(b, stream);
    CK(cudaGetLastError());
    return WRFGPU_OK;
  }
  // gexec_io[h][p]: h = a later step of a call (the previous step's deferred
  // downloads at its head, its prefetched inputs already across), p = not
  // the call's last step (the next step's inputs prefetched)
  int build_io_graph(int h, int v) {
    if (gexec_io[h][v]) return WRFGPU_OK;
    if (int rc = io_streams()) return rc;  // created outside the capture
    capturing = true;
    capture_swaps = 0;
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue_io_step(h == 1, true, v == 1);
    capturing = false;
    io_swaps = capture_swaps;
    for (int q = 0; q < capture_swaps; ++q) host_flip();
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(stream, &g);
    if (rc || ec != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      return rc ? rc : WRFGPU_E_CUDA;
    }
    graph_io[h][v] = g;
    CK(cudaGraphInstantiateWithFlags(&gexec_io[h][v], graph_io[h][v], cudaGraphInstantiateFlagUseNodePriority));
    return WRFGPU_OK;
  }
  int step_host(int nsteps) {
    if (hio.empty() || nsteps < 0) return WRFGPU_E_ARG;
    if (nsteps == 0) return WRFGPU_OK;
    if (flags & WRFGPU_FLAG_NO_GRAPH) {
      for (int s = 0; s < nsteps; ++s) {
        int rc = enqueue_io_step(s > 0, true, s + 1 < nsteps);
        if (rc) return rc;
      }
    } else {
      // the variants this call needs, captured before the first launch
      const int need[3][2] = {{0, nsteps > 1 ? 1 : 0}, {1, 1}, {1, 0}};
      for (int q = 0; q < 3; ++q) {
        if (q == 1 && nsteps < 3) continue;
        if (q == 2 && nsteps < 2) continue;
        int rc = build_io_graph(need[q][0], need[q][1]);
        if (rc) return rc;
      }
      for (int s = 0; s < nsteps; ++s) {
        const int h = s > 0 ? 1 : 0, v = s + 1 < nsteps ? 1 : 0;
        CK(cudaGraphLaunch(gexec_io[h][v], stream));
        for (int q = 0; q < io_swaps; ++q) host_flip();
      }
    }
    if (int rc = flush_deferred()) return rc;
    CK(cudaStreamSynchronize(stream));
    return WRFGPU_OK;
  }

  ~Ensemble() {
    unbind_host();
    if (cstream) cudaStreamDestroy(cstream);
    if (ustream) cudaStreamDestroy(ustream);
    for (cudaEvent_t e : ev_dn) cudaEventDestroy(e);
    for (cudaEvent_t e : {ev_head, ev_ojoin2})
      if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : {ev_fork, ev_join, ev_ofork, ev_ojoin, ev_dryin})
      if (e) cudaEventDestroy(e);
    if (d_stage) cudaFree(d_stage);
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    if (pool) cudaFree(pool);
    if (d_mems) cudaFree(d_mems);
    if (d_bs2) cudaFree(d_bs2);
    if (d_bs3) cudaFree(d_bs3);
    if (d_bs_pr) cudaFree(d_bs_pr);
    if (d_bs_st) cudaFree(d_bs_st);
    if (d_bs_tm) cudaFree(d_bs_tm);
    if (d_bs_s3) cudaFree(d_bs_s3);
    if (d_bs_s4) cudaFree(d_bs_s4);
    if (d_bs_s5) cudaFree(d_bs_s5);
    if (d_tmaps) cudaFree(d_tmaps);
    if (d_pd_scratch) cudaFree(d_pd_scratch);
    if (d_err) cudaFree(d_err);
    if (d_cfl) cudaFree(d_cfl);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }

  static size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

  int init(const WrfGpuDomainDesc* ds, int n, int fl) {
    nmem = n; flags = fl; fp64 = (fl & WRFGPU_FLAG_MIXED) != 0;
    cfl_check = (fl & WRFGPU_FLAG_NO_CHECKS) == 0;
    descs.assign(ds, ds + n);
    for (int m = 0; m < n; ++m) {
      int rc = check_desc(ds[m]);
      if (rc) return rc;
    }
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&ev0));
    CK(cudaEventCreate(&ev1));
    hm.resize(n); n3.resize(n); n2.resize(n); n1.resize(n);
    ni_.resize(n); nk_.resize(n); nj_.resize(n); pitch_.resize(n);
    // sizes
    std::vector<size_t> off(n);
    size_t total = 0;
    for (int m = 0; m < n; ++m) {
      const WrfGpuDomainDesc& d = ds[m];
      size_t ni = d.ide + 2 * WRFGPU_HALO, nj = d.jde + 2 * WRFGPU_HALO, nk = d.kde;  // ims..ime, jms..jme
      // rows padded to a multiple of 4 elements: 16-byte strides for TMA tile loads
      size_t pitch = (ni + 3) & ~size_t(3);
      ni_[m] = ni; nk_[m] = nk; nj_[m] = nj; pitch_[m] = pitch;
      n3[m] = pitch * nk * nj; n2[m] = pitch * nj; n1[m] = nk;
      int nsp = d.n_moist + d.n_scalar;
      size_t b = 0;
      b += (size_t)WRFGPU_N3D * al256(n3[m] * 4);
      b += (size_t)3 * nsp * al256(n3[m] * 4);  // current, old, spare
      b += (size_t)WRFGPU_N2D * al256(n2[m] * 4);
      b += (size_t)WRFGPU_N1D * al256(n1[m] * 4);
      b += al256(n3[m] * 4);  // limiter scratch
      b += 6 * al256(n3[m] * 4);  // face Courant numbers and low-order factors of the PD transport
      if (fp64) b += 3 * al256(n3[m] * 8);
      const bool sct = d.config.diff_6th_opt != 0 || d.config.diff_opt == 1;  // stored diffusion tendencies
      if (sct || d.config.damp_opt == 2) b += 4 * al256(n3[m] * 4);                   // ru_tendf .. t_tendf
      if (sct) b += nsp * al256(n3[m] * 4);                                           // sc_tend
      off[m] = total;
      total += b;
    }
    pool_bytes = total;
    if (cudaMalloc(&pool, total) != cudaSuccess) { pool = nullptr; return WRFGPU_E_NOMEM; }
    CK(cudaMemsetAsync(pool, 0, total, stream));
    CK(cudaMalloc(&d_err, sizeof(unsigned) * n));
    CK(cudaMemsetAsync(d_err, 0, sizeof(unsigned) * n, stream));
    CK(cudaMalloc(&d_cfl, sizeof(float) * 2 * n));
    CK(cudaMemsetAsync(d_cfl, 0, sizeof(float) * 2 * n, stream));
    std::vector<float*> scr(n);
    std::vector<int> bs2(n + 1, 0), bs3(n + 1, 0), bst(n + 1, 0), btm(n + 1, 0), bpr(n + 1, 0), bs_s3(n + 1, 0),
        bs_s4(n + 1, 0), bs_s5(n + 1, 0);
    for (int m = 0; m < n; ++m) {
      const WrfGpuDomainDesc& d = ds[m];
      Mem& M = hm[m];
      std::memset(&M, 0, sizeof(Mem));
      M.ids = 1; M.ide = d.ide; M.jds = 1; M.jde = d.jde; M.kds = 1; M.kde = d.kde;
      M.ims = 1 - WRFGPU_HALO; M.ime = d.ide + WRFGPU_HALO; M.jms = 1 - WRFGPU_HALO; M.jme = d.jde + WRFGPU_HALO;
      M.kms = 1; M.kme = d.kde;
      M.its = M.ids; M.ite = M.ide; M.jts = M.jds; M.jte = M.jde; M.kts = M.kds; M.kte = M.kde;
      M.sk = (long long)pitch_[m]; M.sj = M.sk * (M.kme - M.kms + 1); M.s2 = M.sk;
      char* p = pool + off[m];
      for (int f = 0; f < WRFGPU_N3D; ++f) { M.f3[f] = (float*)p; p += al256(n3[m] * 4); }
      M.nsp = d.n_moist + d.n_scalar; M.n_moist = d.n_moist;
      for (int s = 0; s < M.nsp; ++s) {
        M.q[s] = (float*)p; p += al256(n3[m] * 4);
        M.qo[s] = (float*)p; p += al256(n3[m] * 4);
        M.qa[s] = (float*)p; p += al256(n3[m] * 4);
        M.qmap[s] = WRFGPU_N3D + 3 * s;
        M.qamap[s] = WRFGPU_N3D + 3 * s + 2;
      }
      for (int f = 0; f < WRFGPU_N2D; ++f) { M.f2[f] = (float*)p; p += al256(n2[m] * 4); }
      for (int f = 0; f < WRFGPU_N1D; ++f) { M.f1[f] = (float*)p; p += al256(n1[m] * 4); }
      scr[m] = (float*)p; p += al256(n3[m] * 4);
      for (int q = 0; q < 6; ++q) { M.pdc[q] = (float*)p; p += al256(n3[m] * 4); }
      if (fp64) for (int q = 0; q < 3; ++q) { M.wd[q] = (double*)p; p += al256(n3[m] * 8); }
      const bool sct = d.config.diff_6th_opt != 0 || d.config.diff_opt == 1;
      if (sct || d.config.damp_opt == 2)  // zero outside the loop limits (the pool is cleared)
        for (int q = 0; q < 4; ++q) { M.tendf[q] = (float*)p; p += al256(n3[m] * 4); }
      if (sct) {
        M.sctend = (float*)p; M.sct_n = (long long)(al256(n3[m] * 4) / 4); p += M.nsp * al256(n3[m] * 4);
      }
      M.ns_total = num_sound_steps(d);
      const WrfGpuScalars& s = d.scalars;
      M.dt = (float)s.dt; M.rdx = (float)s.rdx; M.rdy = (float)s.rdy;
      M.cf1 = (float)s.cf1; M.cf2 = (float)s.cf2; M.cf3 = (float)s.cf3; M.cfn = (float)s.cfn; M.cfn1 = (float)s.cfn1;
      M.epssm = (float)s.epssm; M.smdiv = (float)s.smdiv; M.emdiv = (float)s.emdiv; M.p_top = (float)s.p_top;
      M.cf = d.config;
      M.err = d_err + m;
      M.cfl_out = d_cfl + 2 * m;
      M.cfl_limit = 0.f;
      nsp_max = std::max(nsp_max, M.nsp);
      ns_max = std::max(ns_max, M.ns_total);
      nlev_max = std::max(nlev_max, M.kme - M.kms + 1);
      damp3 = damp3 || M.cf.damp_opt == 3;
      diff6 = diff6 || M.cf.diff_6th_opt != 0 || M.cf.diff_opt == 1;
      damp2 = damp2 || M.cf.damp_opt == 2;
      bs2[m + 1] = bs2[m] + blocks_for(M.ims, M.ime, M.jms, M.jme, M.kme - M.kms + 1, 2);
      bs3[m + 1] = bs3[m] + blocks_for(M.ims, M.ime, M.jms, M.jme, M.kme - M.kms + 1, 3);
      bpr[m + 1] = bpr[m] + tiles_x(M) * tiles_y(M) * blocks_per_tile(M.nsp, TILE_PER_PAIR);
      bst[m + 1] = bst[m] + tiles_x(M, true) * tiles_y(M, true);
      btm[m + 1] = btm[m] + tiles_x(M) * tiles_y(M);
      auto strip_blocks = [&](int w, int h) {
        const int nc = strip_cols(M.ide, M.jde, M.cf.open_xs, M.cf.open_ys, w, h);
        return (nc * (M.kme - M.kms + 1) + STRIP_THREADS - 1) / STRIP_THREADS;
      };
      any_open = any_open || M.cf.open_xs || M.cf.open_ys;
      bs_s3[m + 1] = bs_s3[m] + strip_blocks(STRIP_W_TEND, 0);
      bs_s4[m + 1] = bs_s4[m] + strip_blocks(STRIP_W_PD, 0);
      bs_s5[m + 1] = bs_s5[m] + strip_blocks(STRIP_W_PD + 1, 1);
    }
    nb2 = bs2[n]; nb3 = bs3[n]; nb_st = bst[n]; nb_tm = btm[n]; nb_pr = bpr[n];
    nb_s3 = bs_s3[n]; nb_s4 = bs_s4[n]; nb_s5 = bs_s5[n];
    {  // tensor maps of every 3-D buffer: halo and tile boxes
      int rc = get_tensor_map_encoder();
      if (rc) return rc;
      std::vector<CUtensorMap> maps((size_t)n * NMAPSLOT * NBOX);
      std::memset(maps.data(), 0, maps.size() * sizeof(CUtensorMap));
      for (int m = 0; m < n; ++m) {
        Mem& M = hm[m];
        CUtensorMap* mm = maps.data() + (size_t)m * NMAPSLOT * NBOX;
        auto enc = [&](int slot, float* base) -> int {
          int r1 = encode_field_map(&mm[NBOX * slot + BOX_HALO], base, ni_[m], pitch_[m], nk_[m], nj_[m],
                                    TX + 2 * TMA_HALO, TY + 2 * TMA_HALO);
          int r2 = encode_field_map(&mm[NBOX * slot + BOX_TILE], base, ni_[m], pitch_[m], nk_[m], nj_[m], TX, TY);
          return r1 ? r1 : r2;
        };
        for (int f = 0; f < WRFGPU_N3D; ++f) { rc = enc(f, M.f3[f]); if (rc) return rc; }
        for (int sp = 0; sp < M.nsp; ++sp) {
          if ((rc = enc(WRFGPU_N3D + 3 * sp, M.q[sp]))) return rc;
          if ((rc = enc(WRFGPU_N3D + 3 * sp + 1, M.qo[sp]))) return rc;
          if ((rc = enc(WRFGPU_N3D + 3 * sp + 2, M.qa[sp]))) return rc;
        }
        for (int q = 0; q < 6; ++q)
          if ((rc = enc(PDC_SLOT + q, M.pdc[q]))) return rc;
      }
      CK(cudaMalloc(&d_tmaps, maps.size() * sizeof(CUtensorMap)));
      CK(cudaMemcpy(d_tmaps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice));
      for (int m = 0; m < n; ++m) hm[m].tmap = d_tmaps + (size_t)m * NMAPSLOT * NBOX;
    }
    CK(cudaMalloc(&d_mems, sizeof(Mem) * n));
    CK(cudaMemcpyAsync(d_mems, hm.data(), sizeof(Mem) * n, cudaMemcpyHostToDevice, stream));
    CK(cudaMalloc(&d_bs2, sizeof(int) * (n + 1)));
    CK(cudaMalloc(&d_bs3, sizeof(int) * (n + 1)));
    CK(cudaMemcpyAsync(d_bs2, bs2.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_bs3, bs3.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, stream));
    CK(cudaMalloc(&d_bs_pr, sizeof(int) * (n + 1)));
    CK(cudaMemcpyAsync(d_bs_pr, bpr.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, stream));
    CK(cudaMalloc(&d_bs_st, sizeof(int) * (n + 1)));
    CK(cudaMemcpyAsync(d_bs_st, bst.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, stream));
    CK(cudaMalloc(&d_bs_tm, sizeof(int) * (n + 1)));
    CK(cudaMemcpyAsync(d_bs_tm, btm.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, stream));
    for (auto& pr : {std::make_pair(&d_bs_s3, &bs_s3), std::make_pair(&d_bs_s4, &bs_s4),
                     std::make_pair(&d_bs_s5, &bs_s5)}) {
      CK(cudaMalloc(pr.first, sizeof(int) * (n + 1)));
      CK(cudaMemcpyAsync(*pr.first, pr.second->data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, stream));
    }
    CK(cudaMalloc(&d_pd_scratch, sizeof(float*) * n));
    CK(cudaMemcpyAsync(d_pd_scratch, scr.data(), sizeof(float*) * n, cudaMemcpyHostToDevice, stream));
    // map factors default to 1, cosa to 1 (ideal cases); callers overwrite via set_field
    for (int m = 0; m < n; ++m) {
      std::vector<float> ones(n2[m], 1.f);
      for (int f : {WRFGPU_MSFUX, WRFGPU_MSFUY, WRFGPU_MSFVX, WRFGPU_MSFVX_INV, WRFGPU_MSFVY, WRFGPU_MSFTX,
                    WRFGPU_MSFTY, WRFGPU_COSA})
        CK(cudaMemcpy(hm[m].f2[f - WRFGPU_F2D_BASE], ones.data(), n2[m] * 4, cudaMemcpyHostToDevice));
    }
    CK(cudaStreamSynchronize(stream));
    halo_blocks = std::max(8, std::min(256, (int)(n3[0] / 20000)));
    return WRFGPU_OK;
  }

  // Device buffer of a field and its Fortran shape: `cols` contiguous
  // elements per row (ime-ims+1, or kme-kms+1 for 1-D), `rows` rows, rows
  // `pitch` elements apart on the device.  *count = cols * rows (the caller's
  // contiguous array).
  float* field_ptr(int m, int id, size_t* count, size_t* cols = nullptr, size_t* rows = nullptr,
                   size_t* pitch = nullptr) {
    const Mem& M = hm[m];
    size_t c = 0, r = 0, pt = 0;
    float* p = nullptr;
    if (id >= 0 && id < WRFGPU_N3D) { p = M.f3[id]; c = ni_[m]; r = nk_[m] * nj_[m]; pt = pitch_[m]; }
    else if (id >= WRFGPU_F2D_BASE && id < WRFGPU_F2D_END) { p = M.f2[id - WRFGPU_F2D_BASE]; c = ni_[m]; r = nj_[m]; pt = pitch_[m]; }
    else if (id >= WRFGPU_F1D_BASE && id < WRFGPU_F1D_END) { p = M.f1[id - WRFGPU_F1D_BASE]; c = nk_[m]; r = 1; pt = c; }
    else if (id >= WRFGPU_RU_TENDF && id <= WRFGPU_T_TENDF && M.tendf[id - WRFGPU_RU_TENDF]) {  // when allocated
      p = M.tendf[id - WRFGPU_RU_TENDF]; c = ni_[m]; r = nk_[m] * nj_[m]; pt = pitch_[m];
    }
    else if (id >= WRFGPU_SPECIES_BASE && id < WRFGPU_SPECIES_BASE + 2 * M.nsp) {
      int s = (id - WRFGPU_SPECIES_BASE) / 2, old = (id - WRFGPU_SPECIES_BASE) % 2;
      p = old ? M.qo[s] : M.q[s]; c = ni_[m]; r = nk_[m] * nj_[m]; pt = pitch_[m];
    }
    *count = c * r;
    if (cols) *cols = c;
    if (rows) *rows = r;
    if (pitch) *pitch = pt;
    return p;
  }

  // Spare buffer of a species' current value (null for any other field).
  float* spare_ptr(int m, int id) {
    const Mem& M = hm[m];
    if (id >= WRFGPU_SPECIES_BASE && id < WRFGPU_SPECIES_BASE + 2 * M.nsp && (id - WRFGPU_SPECIES_BASE) % 2 == 0)
      return M.qa[(id - WRFGPU_SPECIES_BASE) / 2];
    return nullptr;
  }

  // ---------------------------------------------------------------- halo
  struct JobList {
    std::vector<HaloJob> v;
    void f3(int id, char var) { HaloJob j{id, 3, -1, 0, var, {0, 0, 0}}; v.push_back(j); }
    void f2(int id, char var) { HaloJob j{id, 2, -1, 0, var, {0, 0, 0}}; v.push_back(j); }
    void sp(int s, int old, char var) { HaloJob j{0, 3, s, old, var, {0, 0, 0}}; v.push_back(j); }
  };
  void fill(const JobList& jl) {
    mark(PH_FILL);
    for (size_t b = 0; b < jl.v.size(); b += MAX_HALO_JOBS) {
      HaloJobs hj;
      hj.n = (int)std::min(jl.v.size() - b, (size_t)MAX_HALO_JOBS);
      for (int q = 0; q < hj.n; ++q) hj.job[q] = jl.v[b + q];
      launch_fill_halo(d_mems, nmem, hj, halo_blocks, stream);
    }
  }

  // ---------------------------------------------------------------- one large step
  void enqueue_step() {
    const Launch l2 = L2(), l3 = L3();
    bool species_filled = false;  // the end-of-step species fill was issued early
    for (int rk_step = 1; rk_step <= 3; ++rk_step) {
      StepArgs a{rk_step, 0, 0, 0};
      mark(PH_PREP);
      launch_rk_step_prep(l2, nb2, stream, tune[TU_PREP]);
      {  // rk_phys_bc_dry_1 + al, ph_2 (solve_em.F:726-754)
        JobList j;
        j.f3(WRFGPU_RU, 'u'); j.f3(WRFGPU_RV, 'v'); j.f3(WRFGPU_RW, 'w'); j.f3(WRFGPU_WW, 'w');
        j.f3(WRFGPU_PHP, 'w'); j.f3(WRFGPU_ALT, 't'); j.f3(WRFGPU_P, 'p');
        j.f2(WRFGPU_MUU, 'u'); j.f2(WRFGPU_MUV, 'v'); j.f2(WRFGPU_MUT, 't');
        j.f3(WRFGPU_AL, 'p'); j.f3(WRFGPU_PH_2, 'w');
        fill(j);
      }
      // rk_tendency (module_em.F:370-781)
      mark(PH_TEND_U); launch_tend_u_col(LST(), nb_st, TF_ALL, stream, tune[TU_TENDU]);
      mark(PH_TEND_V); launch_tend_v_col(LST(), nb_st, TF_ALL, stream, tune[TU_TENDV]);
      mark(PH_TEND_W);
      // open boundaries: rw_tend next to them from the cqw the tile kernel overwrites
      if (any_open) launch_strip_tend_w(LS3(), nb_s3, stream);
      launch_tend_w_col(LST(), nb_st, tune[TU_TENDW], stream);
      mark(PH_TEND_T); launch_tend_t_col(LST(), nb_st, TF_ZERO | TF_ADV, stream);
      mark(PH_TEND_PH); launch_tend_ph_col(LST(), nb_st, TF_ZERO | TF_ADV, stream);
      // open boundaries: the lower-order fluxes and radiation terms next to them
      if (any_open) launch_strip_tend(LS3(), nb_s3, stream);
      if (diff6 || damp2) {  // module_em.F:801-944 (stage 1), then rk_addtend_dry (solve_em.F:967)
        mark(PH_DIFF);
        if (rk_step == 1 && diff6) launch_forward_diff(l3, nb3, 0, stream);
        if (rk_step == 1 && damp2) launch_rayleigh_damp(l2, nb2, stream);
        launch_addtend_dry(l3, nb3, stream);
      }
      if (cfl_check) { mark(PH_CFL); launch_cfl_check_col(LTM(), nb_tm, stream, tune[TU_CFL]); }
      // small_step_prep, calc_p_rho(step 0), calc_coef_w (solve_em.F:1089-1140)
      mark(PH_SSP); launch_small_step_prep(l2, nb2, LST(), nb_st, a, stream, tune[TU_SSP]);
      mark(PH_CPR0); launch_calc_p_rho_col(LTM(), nb_tm, StepArgs{rk_step, 0, 0, 0}, stream);
      mark(PH_COEFW); launch_calc_coef_w_col(LTM(), nb_tm, a, fp64, stream);
      {  // solve_em.F:1176-1264
        JobList j;
        j.f3(WRFGPU_RU_TEND, 'u'); j.f3(WRFGPU_RV_TEND, 'v'); j.f3(WRFGPU_PH_2, 'w'); j.f3(WRFGPU_AL, 'p');
        j.f3(WRFGPU_P, 'p'); j.f3(WRFGPU_T_1, 'p'); j.f3(WRFGPU_T_SAVE, 't');
        j.f2(WRFGPU_MU_1, 't'); j.f2(WRFGPU_MU_2, 't'); j.f2(WRFGPU_MUDF, 't');
        fill(j);
      }
      int nsmall_max = 0;
      for (int m = 0; m < nmem; ++m) nsmall_max = std::max(nsmall_max, stage_of(hm[m], rk_step).nsmall);
      for (int it = 1; it <= nsmall_max; ++it) {
        StepArgs ai{rk_step, it, 0, 0};
        mark(PH_AUV); launch_advance_uv_col(LST(), nb_st, rk_step, it, stream, tune[TU_AUV]);
        mark(PH_AMUT); launch_advance_mu_t_col(LTM(), nb_tm, rk_step, it, fp64, stream, tune[TU_AMUT]);
        mark(PH_AW); launch_advance_w_col(LTM(), nb_tm, rk_step, it, fp64, stream, tune[TU_AW], damp3);
        mark(PH_SUMF); launch_sumflux_p_rho_col(LST(), nb_st, rk_step, it, stream, tune[TU_SUMF]);
        // the fills of solve_em.F:1659-1716 (ph_2, al, p, muts, mu_2, mudf) are
        // the producers' own halo stores (MassImages): advance_mu_t,
        // advance_w and calc_p_rho write each halo image with its interior
        // point, and nothing in the acoustic step reads these halos before
        // the next step's advance_uv; open boundaries' copies are the fill's
        if (any_open) {
          JobList j;
          j.f3(WRFGPU_PH_2, 'w'); j.f3(WRFGPU_AL, 'p'); j.f3(WRFGPU_P, 'p');
          j.f2(WRFGPU_MUTS, 't'); j.f2(WRFGPU_MU_2, 't'); j.f2(WRFGPU_MUDF, 't');
          fill(j);
        }
      }
      mark(PH_SSF); launch_small_step_finish(l2, nb2, a, stream, tune[TU_SSF]);
      if (rk_step == 3) {
        // solve_em.F:1754-1800, and the end-of-step fills of the _2 dry state
        // (set_phys_bc_dry_2, :4439-4535) followed by set_w_surface (:4700-4750),
        // both issued here: the dry state is final after small_step_finish,
        // and nothing until the end of the step reads these fields' halos or
        // w (the scalar transport reads mass fluxes and column masses,
        // calc_p_rho_phi mass columns), so the result is the same and a host
        // I/O step can copy the dry state out while the scalars advance
        JobList j;
        j.f3(WRFGPU_RU_M, 'u'); j.f3(WRFGPU_RV_M, 'v'); j.f3(WRFGPU_WW_M, 'w');
        j.f2(WRFGPU_MUT, 't'); j.f2(WRFGPU_MUTS, 't');
        j.f3(WRFGPU_U_2, 'u'); j.f3(WRFGPU_V_2, 'v'); j.f3(WRFGPU_W_2, 'w'); j.f3(WRFGPU_T_2, 'p');
        j.f3(WRFGPU_PH_2, 'w'); j.f2(WRFGPU_MU_2, 't');
        fill(j);
        mark(PH_WSURF); launch_set_w_surface(l2, nb2, stream);
        io_dry_out();
        mark(PH_USPD); launch_update_scalar_pd_col(LTM(), nb_tm, a, stream, diff6);
        JobList jo;
        for (int s = 0; s < nsp_max; ++s) jo.sp(s, 1, 'p');
        fill(jo);
      }
      // scalar loop (solve_em.F:1815-2160): rk_scalar_tend + rk_update_scalar of every
      // species, fused; the positive-definite scheme at the last stage
      if (io_pending && io_split) {
        // a host I/O step's stage 1: the pairs whose passive scalars are
        // across, then (after every upload) the others
        cudaStreamWaitEvent(stream, ev_upA, 0);
        mark(PH_ADVS); launch_scalar_adv_update(LP(), nb_pr, rk_step, stream, tune[TU_ADV], diff6, io_pairs_early);
        io_join();
        launch_scalar_adv_update(LP(), nb_pr, rk_step, stream, tune[TU_ADV], diff6, ~io_pairs_early);
      } else {
        io_join();  // passive scalars copied in by a host I/O step are read from here on
        if (diff6 && rk_step == 1) { mark(PH_DIFF); launch_forward_diff(l3, nb3, 1, stream); }  // module_em.F:1378-1435
        mark(PH_ADVS); launch_scalar_adv_update(LP(), nb_pr, rk_step, stream, tune[TU_ADV], diff6);
      }
      if (rk_step == 3) {
        mark(PH_PD);
        launch_pd_courant(l2, nb2, rk_step, stream);
        launch_scalar_pd_update(LP(), nb_pr, nlev_max, rk_step, stream, tune[TU_PD]);
      }
      if (any_open) {
        launch_strip_scalar(LS3(), nb_s3, rk_step, stream);
        if (rk_step == 3) launch_strip_pd(LS5(), nb_s5, LS4(), nb_s4, rk_step, nsp_max, d_pd_scratch, stream);
      }
      swap_species();
      // a host I/O step with a next step: the species' final halo values
      // (the end-of-step fill, issued here: calc_p_rho_phi reads qv at its
      // own points only) and the moist species' downloads, beside calc_p_rho_phi
      if (rk_step == 3 && io_step && io_prefetch) {
        JobList js;
        for (int s = 0; s < nsp_max; ++s) js.sp(s, 0, 'p');
        fill(js);
        species_filled = true;
        io_moist_out();
      }
      mark(PH_CPRP); launch_calc_p_rho_phi_col(LTM(), nb_tm, stream, tune[TU_CPRP]);
      if (rk_step < 3) {
        JobList j;  // rk_phys_bc_dry_2 + species (solve_em.F:3240-3330)
        j.f3(WRFGPU_U_2, 'u'); j.f3(WRFGPU_V_2, 'v'); j.f3(WRFGPU_W_2, 'w'); j.f3(WRFGPU_T_2, 'p');
        j.f3(WRFGPU_PH_2, 'w'); j.f2(WRFGPU_MU_2, 't');
        for (int s = 0; s < nsp_max; ++s) j.sp(s, 0, 'p');
        fill(j);
      }
    }
    {  // set_phys_bc_dry_2 of the _1 state + species (solve_em.F:4439-4535); the
       // _2 state's fills and set_w_surface ran after the last small_step_finish
      JobList j;
      j.f3(WRFGPU_U_1, 'u'); j.f3(WRFGPU_V_1, 'v'); j.f3(WRFGPU_W_1, 'w'); j.f3(WRFGPU_T_1, 'p');
      j.f3(WRFGPU_PH_1, 'w'); j.f2(WRFGPU_MU_1, 't');
      if (!species_filled)
        for (int s = 0; s < nsp_max; ++s) j.sp(s, 0, 'p');
      fill(j);
    }
    mark(PH_END);
  }

  int build_graph() {
    if (gexec) return WRFGPU_OK;
    capturing = true;
    capture_swaps = 0;
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    enqueue_step();
    capturing = false;
    // nothing ran during capture: undo the host mirror's swaps
    for (int q = 0; q < capture_swaps; ++q) host_flip();
    CK(cudaStreamEndCapture(stream, &graph));
    CK(cudaGraphInstantiate(&gexec, graph, 0));
    return WRFGPU_OK;
  }

  int step(int nsteps) {
    if (flags & WRFGPU_FLAG_NO_GRAPH) {
      for (int s = 0; s < nsteps; ++s) enqueue_step();
    } else {
      int rc = build_graph();
      if (rc) return rc;
      for (int s = 0; s < nsteps; ++s) {
        CK(cudaGraphLaunch(gexec, stream));
        for (int q = 0; q < capture_swaps; ++q) host_flip();
      }
    }
    CK(cudaGetLastError());
    return WRFGPU_OK;
  }

  // Online autotuning: `rounds` x TUNE_MAXVAR real large steps, launched
  // directly with event marks; step q runs variant q % nvar of every family.
  // Each family keeps the variant with the least time, taking for each
  // variant the minimum over rounds (the first use of a variant also pays
  // its module load).  Variants compute the same bits, so the model
  // advances exactly as it would untuned.  The graph is rebuilt afterwards.
  int autotune(int rounds) {
    static const int fam_phase[NTUNE] = {PH_PD, PH_ADVS, PH_AW, PH_AUV, PH_SUMF, PH_PREP, PH_SSF, PH_SSP, PH_CFL,
                                         PH_TEND_W, PH_TEND_U, PH_TEND_V, PH_CPRP, PH_AMUT};
    for (int f = 0; f < NTUNE; ++f)
      for (int v = 0; v < TUNE_MAXVAR; ++v) tune_ms[f][v] = -1.f;
    for (int r = 0; r < rounds; ++r) {
      for (int q = 0; q < TUNE_MAXVAR; ++q) {
        for (int f = 0; f < NTUNE; ++f) tune[f] = q % TUNE_NVAR[f];
        std::vector<std::pair<int, cudaEvent_t>> marks;
        prof = &marks;
        enqueue_step();
        prof = nullptr;
        CK(cudaStreamSynchronize(stream));
        float ph_ms[NPHASE] = {0.f};
        for (size_t k = 0; k + 1 < marks.size(); ++k) {
          float ms = 0.f;
          cudaEventElapsedTime(&ms, marks[k].second, marks[k + 1].second);
          ph_ms[marks[k].first] += ms;
        }
        for (auto& mk : marks) cudaEventDestroy(mk.second);
        for (int f = 0; f < NTUNE; ++f) {
          const int v = q % TUNE_NVAR[f];
          const float t = ph_ms[fam_phase[f]];
          if (tune_ms[f][v] < 0.f || t < tune_ms[f][v]) tune_ms[f][v] = t;
        }
      }
    }
    for (int f = 0; f < NTUNE; ++f) {
      int best = TUNE_DEFAULT[f];
      for (int v = 0; v < TUNE_NVAR[f]; ++v)
        if (tune_ms[f][v] >= 0.f && tune_ms[f][v] < tune_ms[f][best]) best = v;
      tune[f] = best;
    }
    if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
    if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
    drop_io_graph();
    CK(cudaGetLastError());
    return WRFGPU_OK;
  }

  int run_routine(int routine, int rk_step, int iteration, int species) {
    const Launch l2 = L2(), l3 = L3();
    StepArgs a{rk_step, iteration, species, 0};
    switch (routine) {
      case 1: launch_rk_step_prep(l2, nb2, stream); break;
      case 2:
        launch_tend_u(l3, nb3, TF_ZERO, stream); launch_tend_v(l3, nb3, TF_ZERO, stream);
        launch_tend_w(l2, nb2, TF_ZERO, stream); launch_tend_t(l3, nb3, TF_ZERO, stream);
        launch_tend_ph(l3, nb3, TF_ZERO, stream);
        break;
      case 3: launch_tend_u(l3, nb3, TF_ADV, stream); break;
      case 4: launch_tend_v(l3, nb3, TF_ADV, stream); break;
      case 5: launch_tend_w(l2, nb2, TF_ADV, stream); break;
      case 6: launch_tend_t(l3, nb3, TF_ADV, stream); break;
      case 7: launch_tend_ph(l3, nb3, TF_ADV, stream); break;
      case 8: launch_tend_u(l3, nb3, TF_PG, stream); launch_tend_v(l3, nb3, TF_PG, stream); break;
      case 9: launch_tend_w(l2, nb2, TF_PG, stream); break;
      case 10:
        launch_tend_u(l3, nb3, TF_COR, stream); launch_tend_v(l3, nb3, TF_COR, stream);
        launch_tend_w(l2, nb2, TF_COR, stream);
        break;
      case 11:
        launch_tend_u(l3, nb3, TF_CURV, stream); launch_tend_v(l3, nb3, TF_CURV, stream);
        launch_tend_w(l2, nb2, TF_CURV, stream);
        break;
      case 12: launch_small_step_prep(l2, nb2, LST(), nb_st, a, stream); break;
      case 13: launch_calc_p_rho(l3, nb3, a, stream); break;
      case 14: launch_calc_coef_w(l2, nb2, a, fp64, stream); break;
      case 15: launch_advance_uv(l3, nb3, a, stream); break;
      case 16: launch_advance_mu_t(l2, nb2, a, fp64, stream); break;
      case 17: launch_advance_w(l2, nb2, a, fp64, stream); break;
      case 18: launch_sumflux(l3, nb3, a, stream); break;
      case 19: launch_small_step_finish(l2, nb2, a, stream); break;
      case 119: launch_small_step_finish(l2, nb2, a, stream, TUNE_DEFAULT[TU_SSF], false); break;  // muus, muvs given
      case 20: launch_update_scalar_pd(l3, nb3, a, stream); break;
      case 21: launch_advect_scalar(l3, nb3, StepArgs{rk_step, 0, species, 0}, stream); break;
      case 22: launch_advect_scalar_pd2(l3, nb3, StepArgs{rk_step, 0, species, 2}, d_pd_scratch, stream); break;
      // accumulating forms (tendency += ...) for the routine-level C ABI
      case 121: launch_advect_scalar(l3, nb3, StepArgs{rk_step, 0, species, 4}, stream); break;
      case 122: launch_advect_scalar_pd2(l3, nb3, StepArgs{rk_step, 0, species, 6}, d_pd_scratch, stream); break;
      case 23: launch_update_scalar(l3, nb3, a, stream); break;
      // routine-level C ABI forms of the scalar updates (sc_tend in H_DIABATIC)
      // and of rk_scalar_tend's sixth-order diffusion of one species
      case 130: launch_update_scalar_routine(l3, nb3, rk_step, 0, stream); break;
      case 131: launch_update_scalar_routine(l3, nb3, rk_step, 1, stream); break;
      case 132: launch_species_diff_routine(l3, nb3, iteration, stream); break;
      // rk_tendency's forward terms at stage 1 added to the caller's *_tendf
      case 133: launch_forward_diff(l3, nb3, 2, stream); launch_rayleigh_damp(l2, nb2, stream, true); break;
      case 134: launch_addtend_dry_routine(l3, nb3, rk_step, stream); break;  // rk_addtend_dry
      case 24: launch_calc_p_rho_phi(l3, nb3, stream); break;
      case 25: launch_set_w_surface(l2, nb2, stream); break;
      case 26:
        launch_tend_u(l3, nb3, TF_ALL, stream); launch_tend_v(l3, nb3, TF_ALL, stream);
        launch_tend_w(l2, nb2, TF_ALL, stream); launch_tend_t(l3, nb3, TF_ZERO | TF_ADV, stream);
        launch_tend_ph(l3, nb3, TF_ZERO | TF_ADV, stream);
        break;
      default: return WRFGPU_E_ARG;
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(stream));
    return WRFGPU_OK;
  }
};

// ---------------------------------------------------------------------------
// Self-test of the bounded device wait: one block waits on an mbarrier phase
// with a poll limit.  With `arrive` thread 0 completes the phase first (the
// wait succeeds); without it nothing ever arrives, the wait runs out after
// `polls` polls and the block records ERR_TIMEOUT, exactly as the TMA-ring
// kernels do when a copy never lands, and returns normally.
// ---------------------------------------------------------------------------
__global__ void k_selftest_bounded_wait(int polls, int arrive, unsigned* status) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (arrive && threadIdx.x == 0)
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(&bar)) : "memory");
  const bool ok = mbar_wait(&bar, 0, polls);
  if (!ok) atomicOr(status, ERR_TIMEOUT);
}

// ---------------------------------------------------------------------------
// Routine-level calls in parity mode: a cached single-member scratch domain
// per (ide, jde, kde, species); copy in, run one routine, copy out.
// ---------------------------------------------------------------------------
static std::mutex g_fmu;
static std::map<std::tuple<int, int, int, int, int>, Ensemble*> g_fcache;

int fortran_call(const FCall& c) {
  for (int q = 0; q < 18; ++q)
    if (!c.dims[q]) return WRFGPU_E_ARG;
  const int ids = *c.dims[0], ide = *c.dims[1], jds = *c.dims[2], jde = *c.dims[3], kds = *c.dims[4],
            kde = *c.dims[5];
  const int ims = *c.dims[6], ime = *c.dims[7], jms = *c.dims[8], jme = *c.dims[9], kms = *c.dims[10],
            kme = *c.dims[11];
  const int its = *c.dims[12], ite = *c.dims[13], jts = *c.dims[14], jte = *c.dims[15], kts = *c.dims[16],
            kte = *c.dims[17];
  if (ids != 1 || jds != 1 || kds != 1) return WRFGPU_E_ARG;
  // memory dims: a halo of at least WRFGPU_HALO in i and j (the window
  // ids-4 .. ide+4 of a wider one is used), the full column in k
  if (ims > ids - WRFGPU_HALO || ime < ide + WRFGPU_HALO || jms > jds - WRFGPU_HALO || jme < jde + WRFGPU_HALO ||
      kms != kds || kme != kde)
    return WRFGPU_E_ARG;
  // tile dims: any tile of the patch (the routine runs over the whole patch
  // and only the tile's points of the outputs are copied back), full columns
  if (its < ids || ite > ide || its > ite || jts < jds || jte > jde || jts > jte || kts != kds || kte != kde)
    return WRFGPU_E_ARG;
  const bool whole = its == ids && ite == ide && jts == jds && jte == jde;
  const size_t cni = (size_t)(ime - ims + 1), cnk = (size_t)(kme - kms + 1);
  // the caller's element of (ids - 4, kms, jds - 4) and row length of field id
  auto host_window = [&](int id, size_t* hcols) -> size_t {
    const int kind = (id >= WRFGPU_F1D_BASE && id < WRFGPU_F1D_END) ? 1
                     : (id >= WRFGPU_F2D_BASE && id < WRFGPU_F2D_END) ? 2 : 3;
    if (kind == 1) { *hcols = 0; return 0; }
    *hcols = cni;
    const size_t di = (size_t)(ids - WRFGPU_HALO - ims), dj = (size_t)(jds - WRFGPU_HALO - jms);
    return di + cni * (kind == 3 ? cnk * dj : dj);
  };
  if (c.nsp < 1 || c.nsp > NSPMAX) return WRFGPU_E_ARG;
  std::lock_guard<std::mutex> lock(g_fmu);
  // the diffusions' stored tendencies are allocated with the domain
  const bool sct = c.cfg.diff_6th_opt != 0 || c.cfg.diff_opt == 1;
  const int bufs = (sct || c.cfg.damp_opt == 2 ? 1 : 0) | (sct ? 2 : 0);  // tendf, sc_tend
  const auto key = std::make_tuple(ide, jde, kde, c.nsp, bufs);
  Ensemble* e = nullptr;
  auto it = g_fcache.find(key);
  if (it != g_fcache.end()) e = it->second;
  else {
    WrfGpuDomainDesc d{};
    d.ide = ide; d.jde = jde; d.kde = kde; d.n_moist = 1; d.n_scalar = c.nsp - 1;
    d.config = c.cfg;
    d.config.rk_ord = 3;
    d.scalars.dt = 1.0; d.scalars.dx = d.scalars.dy = 1.0; d.scalars.rdx = d.scalars.rdy = 1.0;
    e = new Ensemble();
    int rc = e->init(&d, 1, WRFGPU_FLAG_NO_GRAPH | WRFGPU_FLAG_NO_CHECKS);
    if (rc) { delete e; return rc; }
    g_fcache[key] = e;
  }
  Mem& M = e->hm[0];
  {
    WrfGpuDomainDesc d = e->descs[0];
    d.config = c.cfg;
    int rc = check_desc(d);
    if (rc) return rc;
  }
  M.cf = c.cfg;
  if (c.rdx > 0.f) M.rdx = c.rdx;
  if (c.rdy > 0.f) M.rdy = c.rdy;
  if (c.dt > 0.f) M.dt = c.dt;
  if (c.epssm >= 0.f) M.epssm = c.epssm;
  if (c.smdiv >= 0.f) M.smdiv = c.smdiv;
  if (c.emdiv >= 0.f) M.emdiv = c.emdiv;
  if (c.have_cf) { M.cf1 = c.cf1; M.cf2 = c.cf2; M.cf3 = c.cf3; }
  if (c.have_cfn) { M.cfn = c.cfn; M.cfn1 = c.cfn1; }
  if (c.p_top >= 0.f) M.p_top = c.p_top;
  M.dts_fix = c.dts > 0.f ? c.dts : 0.f;
  M.dtrk_fix = c.dtrk > 0.f ? c.dtrk : 0.f;
  M.nsmall_fix = c.nsmall > 0 ? c.nsmall : 0;
  CK(cudaMemcpyAsync(e->d_mems, &M, sizeof(Mem), cudaMemcpyHostToDevice, e->stream));
  // every bound array is copied in, outputs too: points a routine does not
  // write keep the caller's values, as they would in the caller's array
  for (const FBind& b : c.binds) {
    size_t cnt = 0, cols = 0, rows = 0, pitch = 0;
    float* p = e->field_ptr(0, b.id, &cnt, &cols, &rows, &pitch);
    if (!p) return WRFGPU_E_ARG;
    size_t hcols = 0;
    const size_t off = host_window(b.id, &hcols);
    if (!hcols) hcols = cols;
    CK(cudaMemcpy2DAsync(p, pitch * 4, b.host + off, hcols * 4, cols * 4, rows, cudaMemcpyHostToDevice, e->stream));
  }
  if (c.zero_saves) {
    for (int f : {WRFGPU_U_SAVE, WRFGPU_V_SAVE, WRFGPU_W_SAVE, WRFGPU_PH_SAVE, WRFGPU_T_SAVE})
      CK(cudaMemsetAsync(M.f3[f], 0, e->n3[0] * 4, e->stream));
    for (int f : {WRFGPU_MU_SAVE, WRFGPU_MU_TEND})
      CK(cudaMemsetAsync(M.f2[f - WRFGPU_F2D_BASE], 0, e->n2[0] * 4, e->stream));
  }
  for (int id : c.zero_ids) {
    size_t cnt = 0, cols = 0, rows = 0, pitch = 0;
    float* p = e->field_ptr(0, id, &cnt, &cols, &rows, &pitch);
    if (!p) return WRFGPU_E_ARG;
    CK(cudaMemsetAsync(p, 0, pitch * rows * 4, e->stream));
  }
  if (c.max_vert_cfl || c.max_horiz_cfl) CK(cudaMemsetAsync(e->d_cfl, 0, sizeof(float) * 2, e->stream));
  int rc = e->run_routine(c.routine, c.rk_step, c.iteration, c.species);
  if (rc) return rc;
  if (c.max_vert_cfl || c.max_horiz_cfl) {
    launch_cfl_check_col(e->LTM(), e->nb_tm, e->stream);
    float cfl[2] = {0.f, 0.f};
    CK(cudaMemcpyAsync(cfl, e->d_cfl, sizeof(cfl), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    if (c.max_vert_cfl) *c.max_vert_cfl = cfl[0];
    if (c.max_horiz_cfl) *c.max_horiz_cfl = cfl[1];
  }
  for (const FBind& b : c.binds) {
    if (!b.out) continue;
    size_t cnt = 0, cols = 0, rows = 0, pitch = 0;
    float* p = e->field_ptr(0, b.id, &cnt, &cols, &rows, &pitch);
    if (!p) return WRFGPU_E_ARG;
    size_t hcols = 0;
    const size_t off = host_window(b.id, &hcols);
    if (!hcols || whole) {  // the whole window (what the routine leaves alone comes back as it went in)
      if (!hcols) hcols = cols;
      CK(cudaMemcpy2DAsync(b.host + off, hcols * 4, p, pitch * 4, cols * 4, rows, cudaMemcpyDeviceToHost,
                           e->stream));
      continue;
    }
    // only the tile's box its..ite x jts..jte (every level): the points this
    // tile's call of the reference routine may write
    const bool f3d = !(b.id >= WRFGPU_F2D_BASE && b.id < WRFGPU_F2D_END);
    const size_t per_j = f3d ? cnk : 1;  // rows per j, the same on both sides
    const size_t i0 = (size_t)(its - (ids - WRFGPU_HALO)), j0 = (size_t)(jts - (jds - WRFGPU_HALO));
    const size_t w = (size_t)(ite - its + 1), h = per_j * (size_t)(jte - jts + 1);
    CK(cudaMemcpy2DAsync(b.host + off + i0 + hcols * per_j * j0, hcols * 4, p + i0 + pitch * per_j * j0, pitch * 4,
                         w * 4, h, cudaMemcpyDeviceToHost, e->stream));
  }
  CK(cudaStreamSynchronize(e->stream));
  return WRFGPU_OK;
}

int fortran_release() {
  std::lock_guard<std::mutex> lock(g_fmu);
  for (auto& kv : g_fcache) delete kv.second;
  g_fcache.clear();
  return WRFGPU_OK;
}

}  // namespace wrfgpu

using wrfgpu::Ensemble;

struct WrfGpuEnsemble { Ensemble e; };

extern "C" {

int wrfgpu_selftest_bounded_wait(int polls, int arrive, unsigned* status_bits) {
  if (polls <= 0 || polls > (1 << 22) || !status_bits) return WRFGPU_E_ARG;
  unsigned* d = nullptr;
  CK(cudaMalloc(&d, sizeof(unsigned)));
  CK(cudaMemset(d, 0, sizeof(unsigned)));
  wrfgpu::k_selftest_bounded_wait<<<1, 32>>>(polls, arrive, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  unsigned bits = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&bits, d, sizeof(unsigned), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return WRFGPU_E_CUDA;
  *status_bits = bits;
  return (bits & wrfgpu::ERR_TIMEOUT) ? WRFGPU_E_TIMEOUT : WRFGPU_OK;
}

int wrfgpu_ensemble_create(const WrfGpuDomainDesc* descs, int n, int flags, WrfGpuEnsemble** out) {
  if (!descs || n <= 0 || !out) return WRFGPU_E_ARG;
  auto* h = new WrfGpuEnsemble();
  int rc = h->e.init(descs, n, flags);
  if (rc) { delete h; *out = nullptr; return rc; }
  *out = h;
  return WRFGPU_OK;
}

int wrfgpu_ensemble_destroy(WrfGpuEnsemble* h) {
  if (!h) return WRFGPU_E_ARG;
  cudaStreamSynchronize(h->e.stream);
  delete h;
  return WRFGPU_OK;
}

long long wrfgpu_field_size(WrfGpuEnsemble* h, int member, int id) {
  if (!h || member < 0 || member >= h->e.nmem) return 0;
  size_t n = 0;
  h->e.field_ptr(member, id, &n);
  return (long long)n;
}

int wrfgpu_set_field_f32(WrfGpuEnsemble* h, int member, int id, const float* src, long long n) {
  if (!h || member < 0 || member >= h->e.nmem || !src) return WRFGPU_E_ARG;
  size_t cnt = 0, cols = 0, rows = 0, pitch = 0;
  float* p = h->e.field_ptr(member, id, &cnt, &cols, &rows, &pitch);
  if (!p || (long long)cnt != n) return WRFGPU_E_ARG;
  // a species' spare buffer gets the same values, so points the solver never
  // writes (halo corners, level kde) agree whichever buffer is current
  float* q = h->e.spare_ptr(member, id);
  cudaStream_t s = h->e.stream;
  if (pitch == cols) {
    if (cudaMemcpyAsync(p, src, cnt * 4, cudaMemcpyHostToDevice, s) != cudaSuccess) return WRFGPU_E_CUDA;
    if (q && cudaMemcpyAsync(q, p, cnt * 4, cudaMemcpyDeviceToDevice, s) != cudaSuccess) return WRFGPU_E_CUDA;
  } else {
    if (int rc = h->e.ensure_stage(cnt)) return rc;
    if (cudaMemcpyAsync(h->e.d_stage, src, cnt * 4, cudaMemcpyHostToDevice, s) != cudaSuccess) return WRFGPU_E_CUDA;
    wrfgpu::launch_unpack_rows(h->e.d_stage, p, q, (int)cols, (int)rows, (int)pitch, s);
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return WRFGPU_E_CUDA;
  return WRFGPU_OK;
}

int wrfgpu_get_field_f32(WrfGpuEnsemble* h, int member, int id, float* dst, long long n) {
  if (!h || member < 0 || member >= h->e.nmem || !dst) return WRFGPU_E_ARG;
  size_t cnt = 0, cols = 0, rows = 0, pitch = 0;
  float* p = h->e.field_ptr(member, id, &cnt, &cols, &rows, &pitch);
  if (!p || (long long)cnt != n) return WRFGPU_E_ARG;
  cudaStream_t s = h->e.stream;
  if (pitch == cols) {
    if (cudaMemcpyAsync(dst, p, cnt * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) return WRFGPU_E_CUDA;
  } else {
    if (int rc = h->e.ensure_stage(cnt)) return rc;
    wrfgpu::launch_pack_rows(p, h->e.d_stage, (int)cols, (int)rows, (int)pitch, s);
    if (cudaMemcpyAsync(dst, h->e.d_stage, cnt * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) return WRFGPU_E_CUDA;
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return WRFGPU_E_CUDA;
  return WRFGPU_OK;
}

int wrfgpu_set_field(WrfGpuEnsemble* h, int member, int id, const double* src, long long n) {
  if (!src || n < 0) return WRFGPU_E_ARG;
  std::vector<float> tmp((size_t)n);
  for (long long i = 0; i < n; ++i) tmp[(size_t)i] = (float)src[i];
  return wrfgpu_set_field_f32(h, member, id, tmp.data(), n);
}

int wrfgpu_get_field(WrfGpuEnsemble* h, int member, int id, double* dst, long long n) {
  if (!dst || n < 0) return WRFGPU_E_ARG;
  std::vector<float> tmp((size_t)n);
  int rc = wrfgpu_get_field_f32(h, member, id, tmp.data(), n);
  if (rc) return rc;
  for (long long i = 0; i < n; ++i) dst[i] = (double)tmp[(size_t)i];
  return WRFGPU_OK;
}

int wrfgpu_step(WrfGpuEnsemble* h, int nsteps) {
  if (!h || nsteps < 0) return WRFGPU_E_ARG;
  return h->e.step(nsteps);
}

int wrfgpu_bind_host_state(WrfGpuEnsemble* h, int member, int nfield, const int* ids, const float* const* in,
                           float* const* out, const long long* n) {
  if (!h) return WRFGPU_E_ARG;
  return h->e.bind_host(member, nfield, ids, in, out, n);
}

int wrfgpu_unbind_host_state(WrfGpuEnsemble* h) {
  if (!h) return WRFGPU_E_ARG;
  h->e.unbind_host();
  return WRFGPU_OK;
}

int wrfgpu_step_host(WrfGpuEnsemble* h, int nsteps) {
  if (!h) return WRFGPU_E_ARG;
  return h->e.step_host(nsteps);
}

int wrfgpu_sync(WrfGpuEnsemble* h) {
  if (!h) return WRFGPU_E_ARG;
  return cudaStreamSynchronize(h->e.stream) == cudaSuccess ? WRFGPU_OK : WRFGPU_E_CUDA;
}

int wrfgpu_time_steps(WrfGpuEnsemble* h, int nsteps, float* ms) {
  if (!h || nsteps < 0 || !ms) return WRFGPU_E_ARG;
  Ensemble& e = h->e;
  if (!(e.flags & WRFGPU_FLAG_NO_GRAPH)) { int rc = e.build_graph(); if (rc) return rc; }
  if (cudaEventRecord(e.ev0, e.stream) != cudaSuccess) return WRFGPU_E_CUDA;
  int rc = e.step(nsteps);
  if (rc) return rc;
  if (cudaEventRecord(e.ev1, e.stream) != cudaSuccess) return WRFGPU_E_CUDA;
  if (cudaEventSynchronize(e.ev1) != cudaSuccess) return WRFGPU_E_CUDA;
  if (cudaEventElapsedTime(ms, e.ev0, e.ev1) != cudaSuccess) return WRFGPU_E_CUDA;
  return WRFGPU_OK;
}

int wrfgpu_run_routine(WrfGpuEnsemble* h, int routine, int rk_step, int iteration, int species) {
  if (!h || rk_step < 1 || rk_step > 3) return WRFGPU_E_ARG;
  return h->e.run_routine(routine, rk_step, iteration, species);
}

int wrfgpu_fill_halo(WrfGpuEnsemble* h, int id, char var) {
  if (!h) return WRFGPU_E_ARG;
  Ensemble::JobList j;
  if (id >= 0 && id < WRFGPU_N3D) j.f3(id, var);
  else if (id >= WRFGPU_F2D_BASE && id < WRFGPU_F2D_END) j.f2(id, var);
  else if (id >= WRFGPU_SPECIES_BASE) j.sp((id - WRFGPU_SPECIES_BASE) / 2, (id - WRFGPU_SPECIES_BASE) % 2, var);
  else return WRFGPU_E_ARG;
  h->e.fill(j);
  if (cudaStreamSynchronize(h->e.stream) != cudaSuccess) return WRFGPU_E_CUDA;
  return WRFGPU_OK;
}

int wrfgpu_status(WrfGpuEnsemble* h, int member, unsigned* err_bits, double* max_vert_cfl, double* max_horiz_cfl) {
  if (!h || member < 0 || member >= h->e.nmem) return WRFGPU_E_ARG;
  Ensemble& e = h->e;
  unsigned eb = 0;
  float c[2] = {0, 0};
  if (cudaStreamSynchronize(e.stream) != cudaSuccess) return WRFGPU_E_CUDA;
  if (cudaMemcpy(&eb, e.d_err + member, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) return WRFGPU_E_CUDA;
  if (cudaMemcpy(c, e.d_cfl + 2 * member, sizeof(float) * 2, cudaMemcpyDeviceToHost) != cudaSuccess) return WRFGPU_E_CUDA;
  if (err_bits) *err_bits = eb;
  if (max_vert_cfl) *max_vert_cfl = c[0];
  if (max_horiz_cfl) *max_horiz_cfl = c[1];
  if (eb & wrfgpu::ERR_NONFINITE) return WRFGPU_E_NONFINITE;
  if (eb & wrfgpu::ERR_CFL) return WRFGPU_E_CFL;
  if (eb & wrfgpu::ERR_TIMEOUT) return WRFGPU_E_TIMEOUT;
  return WRFGPU_OK;
}

int wrfgpu_clear_status(WrfGpuEnsemble* h) {
  if (!h) return WRFGPU_E_ARG;
  Ensemble& e = h->e;
  if (cudaMemsetAsync(e.d_err, 0, sizeof(unsigned) * e.nmem, e.stream) != cudaSuccess) return WRFGPU_E_CUDA;
  if (cudaMemsetAsync(e.d_cfl, 0, sizeof(float) * 2 * e.nmem, e.stream) != cudaSuccess) return WRFGPU_E_CUDA;
  return cudaStreamSynchronize(e.stream) == cudaSuccess ? WRFGPU_OK : WRFGPU_E_CUDA;
}

int wrfgpu_set_cfl_limit(WrfGpuEnsemble* h, double limit) {
  if (!h) return WRFGPU_E_ARG;
  Ensemble& e = h->e;
  for (auto& M : e.hm) M.cfl_limit = (float)limit;
  if (cudaMemcpy(e.d_mems, e.hm.data(), sizeof(wrfgpu::Mem) * e.nmem, cudaMemcpyHostToDevice) != cudaSuccess)
    return WRFGPU_E_CUDA;
  return WRFGPU_OK;
}

int wrfgpu_num_sound_steps(WrfGpuEnsemble* h, int member) {
  if (!h || member < 0 || member >= h->e.nmem) return WRFGPU_E_ARG;
  return h->e.hm[member].ns_total;
}

long long wrfgpu_device_bytes(WrfGpuEnsemble* h) { return h ? (long long)h->e.pool_bytes : 0; }

int wrfgpu_kernel_launches_per_step(WrfGpuEnsemble* h) {
  if (!h) return WRFGPU_E_ARG;
  cudaGraph_t g = nullptr;
  Ensemble& e = h->e;
  if (e.build_graph()) return WRFGPU_E_CUDA;
  size_t n = 0;
  if (cudaGraphGetNodes(e.graph, nullptr, &n) != cudaSuccess) return WRFGPU_E_CUDA;
  (void)g;
  return (int)n;
}

int wrfgpu_autotune(WrfGpuEnsemble* h, int rounds) {
  if (!h || rounds < 1 || rounds > 16) return WRFGPU_E_ARG;
  return h->e.autotune(rounds);
}

int wrfgpu_tuning(WrfGpuEnsemble* h, int* variant, int* param, float* ms, int nfamily) {
  if (!h || !variant || nfamily < (int)wrfgpu::NTUNE) return WRFGPU_E_ARG;
  Ensemble& e = h->e;
  for (int f = 0; f < (int)wrfgpu::NTUNE; ++f) {
    variant[f] = e.tune[f];
    if (param) param[f] = wrfgpu::TUNE_PARAM[f][e.tune[f]];
    if (ms)
      for (int v = 0; v < wrfgpu::TUNE_MAXVAR; ++v) ms[f * wrfgpu::TUNE_MAXVAR + v] = e.tune_ms[f][v];
  }
  return (int)wrfgpu::NTUNE;
}

int wrfgpu_profile_phases(WrfGpuEnsemble* h, int nsteps, double* ms_out, int* launches_out, int nphase) {
  if (!h || nsteps <= 0 || !ms_out || nphase < (int)wrfgpu::NPHASE - 1) return WRFGPU_E_ARG;
  Ensemble& e = h->e;
  std::vector<std::pair<int, cudaEvent_t>> marks;
  for (int p = 0; p < nphase; ++p) { ms_out[p] = 0.0; if (launches_out) launches_out[p] = 0; }
  e.prof = &marks;
  for (int s = 0; s < nsteps; ++s) e.enqueue_step();
  e.prof = nullptr;
  if (cudaStreamSynchronize(e.stream) != cudaSuccess) return WRFGPU_E_CUDA;
  for (size_t q = 0; q + 1 < marks.size(); ++q) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, marks[q].second, marks[q + 1].second);
    int ph = marks[q].first;
    if (ph == wrfgpu::PH_END) continue;
    ms_out[ph] += ms;
    if (launches_out) launches_out[ph] += 1;
  }
  for (auto& m : marks) cudaEventDestroy(m.second);
  return (int)wrfgpu::NPHASE - 1;
}

const char* wrfgpu_phase_name(int phase) {
  if (phase < 0 || phase >= (int)wrfgpu::NPHASE) return "";
  return wrfgpu::PHASE_NAMES[phase];
}

const char* wrfgpu_version(void) { return "wrf-gb300 dyn 0.1 (sm_103a)"; }

}  // extern "C"
