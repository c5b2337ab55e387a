// Host-side launch wrappers of the device kernels (one translation unit per
// kernel family; no relocatable device code needed).
#pragma once
#include <cuda_runtime.h>
#include "common.cuh"

namespace wrfgpu {

struct HaloJob {
  int id;        // field id (3-D or 2-D), ignored for species
  int kind;      // 3 or 2
  int species;   // >= 0: species index (uses q / qo), -1 otherwise
  int old;       // species: 1 = old (_1) copy
  char var;      // reference stagger code: 'u','v','w','p','t'
  char pad[3];
};
constexpr int MAX_HALO_JOBS = 24;
struct HaloJobs {
  int n;
  HaloJob job[MAX_HALO_JOBS];
};

// Stage / iteration arguments shared by the step kernels.
struct StepArgs {
  int rk_step;     // 1..3
  int iteration;   // acoustic iteration (1-based) or 0
  int species;     // species index for scalar kernels
  int flags;       // kernel-specific variant bits
};

// Variant bits of the tendency kernels (rk_tendency pieces).
enum : int {
  TF_ZERO = 1,      // start from zero (zero_tend) instead of accumulating
  TF_ADV = 2,       // advect_u / advect_v / advect_w / advect_scalar / rhs_ph
  TF_PG = 4,        // horizontal_pressure_gradient / pg_buoy_w
  TF_COR = 8,       // coriolis
  TF_CURV = 16,     // curvature
  TF_ALL = 31
};

// Run-time tuned launch variants (the autotuner in driver.cu times them on
// the real step and keeps the fastest).  Every variant of a family computes
// the same bits: they differ only in launch bounds (registers per thread,
// so blocks per SM) or in how many level chunks a column kernel is split into.
enum Tune { TU_PD = 0, TU_ADV, TU_AW, TU_AUV, TU_SUMF, TU_PREP, TU_SSF, TU_SSP, TU_CFL, TU_TENDW, TU_TENDU, TU_TENDV,
            TU_CPRP, TU_AMUT, NTUNE };
constexpr int TUNE_MAXVAR = 4;
constexpr int TUNE_NVAR[NTUNE] = {2, 3, 3, 4, 4, 2, 2, 4, 4, 3, 4, 4, 4, 4};
constexpr int TUNE_DEFAULT[NTUNE] = {1, 1, 1, 0, 0, 1, 1, 2, 2, 1, 0, 0, 2, 0};
// the parameter each variant stands for: blocks per SM, level chunks, or
// (advance_uv, sumflux, rk_tend_u, rk_tend_v) 10 x blocks per SM + level chunks
constexpr int TUNE_PARAM[NTUNE][TUNE_MAXVAR] = {{1, 2, 0, 0}, {2, 3, 4, 0}, {2, 3, 4, 0}, {32, 42, 34, 44}, {32, 42, 34, 44},
                                                {3, 8, 0, 0}, {4, 8, 0, 0}, {1, 2, 4, 8}, {2, 4, 8, 16}, {2, 3, 4, 0},
                                                {32, 42, 34, 44}, {32, 42, 34, 44}, {1, 2, 4, 8}, {2, 3, 4, 5}};

void launch_rk_step_prep(const Launch& L, int nblocks, cudaStream_t s, int var = TUNE_DEFAULT[TU_PREP]);
void launch_fill_halo(const Mem* d_mems, int nmem, const HaloJobs& jobs, int blocks_per_job, cudaStream_t s);

// rk_tendency
void launch_tend_u(const Launch& L3, int nblocks, int flags, cudaStream_t s);
void launch_tend_v(const Launch& L3, int nblocks, int flags, cudaStream_t s);
void launch_tend_w(const Launch& L2, int nblocks, int flags, cudaStream_t s);
void launch_tend_w_col(const TileLaunch& L, int nblocks, int var, cudaStream_t s);  // TF_ALL, staggered tiles, tuned
void launch_tend_t(const Launch& L3, int nblocks, int flags, cudaStream_t s);
void launch_tend_ph(const Launch& L3, int nblocks, int flags, cudaStream_t s);
// column forms over tiles of the staggered extents
void launch_tend_u_col(const TileLaunch& L, int nblocks, int flags, cudaStream_t s, int var = 0);
void launch_tend_v_col(const TileLaunch& L, int nblocks, int flags, cudaStream_t s, int var = 0);
void launch_tend_t_col(const TileLaunch& L, int nblocks, int flags, cudaStream_t s);
void launch_tend_ph_col(const TileLaunch& L, int nblocks, int flags, cudaStream_t s);
// sixth-order diffusion of the dry state at stage 1, and rk_addtend_dry (k_diff.cu)
// mode 0: u, v, w, theta into ru_tendf .. t_tendf; 1: the species into sc_tend
void launch_forward_diff(const Launch& L, int nblocks, int mode, cudaStream_t s);
void launch_species_diff_routine(const Launch& L, int nblocks, int qv, cudaStream_t s);
void launch_addtend_dry_routine(const Launch& L, int nblocks, int rk_step, cudaStream_t s);
void launch_rayleigh_damp(const Launch& L2, int nblocks, cudaStream_t s, bool acc_all = false);
void launch_addtend_dry(const Launch& L, int nblocks, cudaStream_t s);

// acoustic steps
// 2-D part over column blocks, then the 3-D part over staggered tiles x level chunks
void launch_small_step_prep(const Launch& L2, int nb2, const TileLaunch& LST, int nb_st, StepArgs a, cudaStream_t s,
                            int var = TUNE_DEFAULT[TU_SSP]);
void launch_calc_p_rho(const Launch& L3, int nblocks, StepArgs a, cudaStream_t s);
void launch_calc_coef_w(const Launch& L2, int nblocks, StepArgs a, bool fp64, cudaStream_t s);
void launch_calc_coef_w_col(const TileLaunch& L, int nblocks, StepArgs a, bool fp64, cudaStream_t s);  // mass tiles
void launch_advance_uv(const Launch& L3, int nblocks, StepArgs a, cudaStream_t s);
void launch_advance_mu_t(const Launch& L2, int nblocks, StepArgs a, bool fp64, cudaStream_t s);
void launch_advance_w(const Launch& L2, int nblocks, StepArgs a, bool fp64, cudaStream_t s);
void launch_sumflux_p_rho(const Launch& L3, int nblocks, StepArgs a, bool do_p_rho, cudaStream_t s);
void launch_sumflux(const Launch& L3, int nblocks, StepArgs a, cudaStream_t s);
// calc_mus: calc_mu_uv_1 fused in (the step); false: the caller's muus, muvs
void launch_small_step_finish(const Launch& L2, int nblocks, StepArgs a, cudaStream_t s, int var = TUNE_DEFAULT[TU_SSF],
                              bool calc_mus = true);

// scalars and diagnosis
void launch_update_scalar_pd(const Launch& L3, int nblocks, StepArgs a, cudaStream_t s);
void launch_advect_scalar(const Launch& L3, int nblocks, StepArgs a, cudaStream_t s);
void launch_advect_scalar_pd2(const Launch& L3, int nblocks, StepArgs a, float* const* d_scratch, cudaStream_t s);
void launch_update_scalar(const Launch& L3, int nblocks, StepArgs a, cudaStream_t s);
void launch_update_scalar_routine(const Launch& L3, int nblocks, int rk_step, int pd, cudaStream_t s);
void launch_calc_p_rho_phi(const Launch& L3, int nblocks, cudaStream_t s);
// host <-> device field copies through a contiguous staging buffer
void launch_unpack_rows(const float* src, float* dst, float* dst2, int cols, int rows, int pitch, cudaStream_t s);
void launch_pack_rows(const float* src, float* dst, int cols, int rows, int pitch, cudaStream_t s);
void launch_unpack_species(const Mem* mems, int member, int s, const float* src, int cols, int rows, int pitch,
                           cudaStream_t st);
void launch_pack_species(const Mem* mems, int member, int s, float* dst, int cols, int rows, int pitch,
                         cudaStream_t st);
void launch_calc_p_rho_col(const TileLaunch& L, int nblocks, StepArgs a, cudaStream_t s);        // mass tiles
// sct: some member stores the species' sixth-order diffusion tendency sc_tend
void launch_update_scalar_pd_col(const TileLaunch& L, int nblocks, StepArgs a, cudaStream_t s, bool sct = false);  // mass tiles
void launch_calc_p_rho_phi_col(const TileLaunch& L, int nblocks, cudaStream_t s, int var = TUNE_DEFAULT[TU_CPRP]);  // mass tiles
void launch_set_w_surface(const Launch& L2, int nblocks, cudaStream_t s);
void launch_cfl_check_col(const TileLaunch& L, int nblocks, cudaStream_t s, int var = TUNE_DEFAULT[TU_CFL]);  // mass tiles

// fused scalar transport (k_scalar_fused.cu): one block per (tile, pair of
// species); `pairs` selects the pairs this launch transports (bit p: pair p)
void launch_scalar_adv_update(const TileLaunch& L, int nblocks, int rk_step, cudaStream_t s, int var = TUNE_DEFAULT[TU_ADV],
                              bool sct = false, unsigned pairs = ~0u);
// the face Courant numbers of the PD transport, once per step before it (column layout)
void launch_pd_courant(const Launch& L2, int nblocks, int rk_step, cudaStream_t s);
// nlev_max: the largest kme - kms + 1 of the members (sizes a per-level table in shared memory)
void launch_scalar_pd_update(const TileLaunch& L, int nblocks, int nlev_max, int rk_step, cudaStream_t s,
                             int var = TUNE_DEFAULT[TU_PD]);
void launch_swap_species(Mem* d_mems, int nmem, cudaStream_t s);

// column-marching acoustic kernels (k_acoustic_col.cu): one block per tile
// of the staggered extents
void launch_sumflux_p_rho_col(const TileLaunch& L, int nblocks, int rk_step, int iteration, cudaStream_t s,
                              int var = TUNE_DEFAULT[TU_SUMF]);
void launch_advance_uv_col(const TileLaunch& L, int nblocks, int rk_step, int iteration, cudaStream_t s,
                           int var = TUNE_DEFAULT[TU_AUV]);
// one block per tile of mass columns
void launch_advance_mu_t_col(const TileLaunch& L, int nblocks, int rk_step, int iteration, bool fp64, cudaStream_t s,
                             int var = TUNE_DEFAULT[TU_AMUT]);
// damp: some member uses damp_opt = 3 (compiles the damping into the kernel)
void launch_advance_w_col(const TileLaunch& L, int nblocks, int rk_step, int iteration, bool fp64, cudaStream_t s,
                          int var = TUNE_DEFAULT[TU_AW], bool damp = false);

// edge strips of members with open lateral boundaries (open_adv.cuh): the
// tendencies of u, v, theta and ph after their tile kernels (k_tend.cu), rw_tend
// before its tile kernel (per column), and the scalar transport after its
// tile kernels (k_scalar.cu)
void launch_strip_tend(const StripLaunch& L, int nblocks, cudaStream_t s);
void launch_strip_tend_w(const StripLaunch& L, int nblocks, cudaStream_t s);
void launch_strip_scalar(const StripLaunch& L, int nblocks, int rk_step, cudaStream_t s);
// the positive-definite species at the last stage, one species at a time
// through the member's PD scratch: limiter factors over `wide`, then the
// limited divergence and update over L
void launch_strip_pd(const StripLaunch& wide, int nb_wide, const StripLaunch& L, int nb, int rk_step, int nsp_max,
                     float* const* d_scratch, cudaStream_t s);

}  // namespace wrfgpu
