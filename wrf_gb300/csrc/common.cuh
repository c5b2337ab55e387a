// Shared device definitions of the GB300 WRF-ARW large-step kernels.
//
// Data layout in HBM: every field keeps the reference's Fortran memory layout
// (ims:ime, kms:kme, jms:jme), i fastest, halo 4 (the serial build's
// bdyzone), so a Fortran caller's arrays map onto device buffers by a plain
// copy and the halo-fill sites of solve_em map one to one.  A domain is a
// "member": a descriptor (Mem) holding its index bounds, strides and the
// device pointers of all of its fields.  Every kernel is written against a
// table of members; a launch covers all members' blocks through a prefix
// table (block_start), so one launch advances a single domain (the plain
// drop-in form) or a whole uneven ensemble (the batched form) with the same
// per-point arithmetic.
//
// Arithmetic: the plain form is compiled with --fmad=false and IEEE division
// so every expression rounds in the reference's left-to-right order.  The
// log and pow of calc_p_rho_phi are correctly rounded (ffmath.h), as a
// correctly rounded libm would give them to the reference's FP32 build.
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>
#include "../../include/wrfgpu.h"
#include "cdiv.h"

namespace wrfgpu {

constexpr int NSPMAX = 16;           // species per member (moist + passive)
constexpr int TMA_HALO = 4;          // halo of the staged planes
constexpr int BX = 32, BY = 4;       // thread block: 32 (i) x 4 (j)
constexpr float G = 9.81f;
constexpr float R_D = 287.f;
constexpr float CP = 7.f * R_D / 2.f;
constexpr float CV = CP - R_D;
constexpr float CPOVCV = CP / (CP - R_D);
constexpr float T0 = 300.f;
constexpr float P0 = 100000.f;
constexpr float RERADIUS = 1.f / 6370.0e03f;
constexpr float CB = 25.f;  // radiation-condition wave speed of open boundaries, module_model_constants.F:47
constexpr float PI_F = 3.14159274f;  // 4 atan(1) in FP32 (module_small_step_em.F:1283)
constexpr float W_ALPHA = 0.3f;  // w_damp strength (m/s/s), module_model_constants.F:88
constexpr float W_BETA = 1.0f;   // w_damp activation Courant number, :89

// Tensor maps (TMA descriptors) of every 3-D field buffer of a member: slot
// f < WRFGPU_N3D for the fields, WRFGPU_N3D + 3 s + {0, 1, 2} for species s's
// buffers (first current, old, first spare), PDC_SLOT + q for the PD
// transport's face array pdc[q].  Two boxes per slot: the tile plus a
// 4-point halo, (TX + 8) x 1 x (TY + 8) from (i0 - 4, j0 - 4), and the tile
// alone, TX x 1 x TY from (i0, j0).
constexpr int PDC_SLOT = WRFGPU_N3D + 3 * NSPMAX;
constexpr int NMAPSLOT = PDC_SLOT + 6;
constexpr int BOX_HALO = 0, BOX_TILE = 1, NBOX = 2;

// Error word bits (Mem::err): set by kernels, read by the host between steps.
constexpr unsigned ERR_NONFINITE = 1u;
constexpr unsigned ERR_CFL = 2u;
constexpr unsigned ERR_TIMEOUT = 4u;

struct alignas(16) Mem {
  int ids, ide, jds, jde, kds, kde;
  int ims, ime, jms, jme, kms, kme;
  int its, ite, jts, jte, kts, kte;
  long long sk, sj, s2;   // 3-D k and j strides, 2-D j stride (elements)
  float* f3[WRFGPU_N3D];
  float* f2[WRFGPU_N2D];
  float* f1[WRFGPU_N1D];
  float* q[NSPMAX];       // species current (_2)
  float* qo[NSPMAX];      // species old (_1)
  float* qa[NSPMAX];      // species spare buffer: the fused update writes the new
                          // value here and the pair (q, qa) is swapped after the stage
  int qmap[NSPMAX];       // tensor-map slots of q[s] and qa[s] (swapped with them)
  int qamap[NSPMAX];
  const CUtensorMap* tmap;  // this member's tensor maps [NMAPSLOT][2] (device memory)
  double* wd[3];          // FP64 a/alpha/gamma of the mixed-precision form (or null)
  float* pdc[6];          // PD transport's x, y, z faces: Courant numbers, then mu dx / dt (k_pd_courant)
  float* tendf[4];        // ru_tendf, rv_tendf, rw_tendf, t_tendf of the sixth-order diffusion (or null)
  float* sctend;          // species s's sc_tend at sctend + s * sct_n (sixth-order diffusion, or null)
  long long sct_n;
  int nsp, n_moist;
  int ns_total;           // acoustic steps per large step
  int pad0;
  float dt, rdx, rdy, cf1, cf2, cf3, cfn, cfn1, epssm, smdiv, emdiv, p_top;
  // stage constants given explicitly by a routine-level caller (> 0), else
  // derived from dt and the acoustic step count
  float dts_fix, dtrk_fix;
  int nsmall_fix, pad2;
  WrfDynConfig cf;
  unsigned* err;          // per-member error word
  float cfl_limit;        // vertical CFL above which ERR_CFL is raised (<=0: off)
  float pad1;
  float* cfl_out;         // [2]: max vertical, max horizontal CFL (atomic max)
};

// Species s's explicit (diff_opt = 1) and sixth-order diffusion switches
// (rk_scalar_tend's mix2_off / mix6_off, module_em.F:1378-1435).
__host__ __device__ inline bool mix2_on(const Mem& m, int s) {
  return m.cf.diff_opt == 1 && !(s < m.n_moist ? m.cf.moist_mix2_off : m.cf.scalar_mix2_off);
}
__host__ __device__ inline bool mix6_on(const Mem& m, int s) {
  return m.cf.diff_6th_opt != 0 && !(s < m.n_moist ? m.cf.moist_mix6_off : m.cf.scalar_mix6_off);
}
// Species s's stored diffusion tendency sc_tend, or null where the species is
// not diffused.
__host__ __device__ inline float* sc_tend_of(const Mem& m, int s) {
  if (m.sctend == nullptr) return nullptr;
  return mix2_on(m, s) || mix6_on(m, s) ? m.sctend + (long long)s * m.sct_n : nullptr;
}

// Tensor map of buffer slot `slot` (field id or species slot), box `box`.
__host__ __device__ inline const CUtensorMap* tmap_of(const Mem& m, int slot, int box) {
  return m.tmap + NBOX * slot + box;
}

// Stage constants of solve_em.F:601-615 for one member.
struct Stage {
  float dt_rk, dts_rk;
  int nsmall;
};
__host__ __device__ inline Stage stage_of(const Mem& m, int rk_step) {
  Stage s;
  float dts = m.dt / float(m.ns_total);
  if (rk_step == 1) { s.dt_rk = m.dt / 3.f; s.dts_rk = s.dt_rk; s.nsmall = 1; }
  else if (rk_step == 2) { s.dt_rk = 0.5f * m.dt; s.dts_rk = dts; s.nsmall = m.ns_total / 2; }
  else { s.dt_rk = m.dt; s.dts_rk = dts; s.nsmall = m.ns_total; }
  if (m.dts_fix > 0.f) s.dts_rk = m.dts_fix;
  if (m.dtrk_fix > 0.f) s.dt_rk = m.dtrk_fix;
  if (m.nsmall_fix > 0) s.nsmall = m.nsmall_fix;
  return s;
}

// ---------------------------------------------------------------------------
// Accessors (Fortran indices)
// ---------------------------------------------------------------------------
// ro(): read through the read-only (non-coherent) path, for arrays a kernel
// never writes: such loads do not alias the kernel's stores, so they can be
// issued ahead of them instead of waiting behind every store.
//
// Offsets are 32-bit: a field holds fewer than 2^31 elements (checked when a
// member is created), so one index costs an integer multiply-add per distinct
// (k, j) and a single wide add per field instead of 64-bit products.
struct F3 {
  float* __restrict__ p; int sk, sj, ims, kms, jms;
  __device__ __forceinline__ int off(int i, int k, int j) const { return (i - ims) + (k - kms) * sk + (j - jms) * sj; }
  __device__ __forceinline__ float& operator()(int i, int k, int j) const { return p[off(i, k, j)]; }
  __device__ __forceinline__ float ro(int i, int k, int j) const { return __ldg(p + off(i, k, j)); }
};
struct F2 {
  float* __restrict__ p; int sj, ims, jms;
  __device__ __forceinline__ float& operator()(int i, int j) const { return p[(i - ims) + (j - jms) * sj]; }
  __device__ __forceinline__ float ro(int i, int j) const { return __ldg(p + ((i - ims) + (j - jms) * sj)); }
};
struct F1 {
  const float* __restrict__ p; int kms;
  __device__ __forceinline__ float operator()(int k) const { return __ldg(p + (k - kms)); }
};
struct D3 {
  double* __restrict__ p; int sk, sj, ims, kms, jms;
  __device__ __forceinline__ double& operator()(int i, int k, int j) const {
    return p[(i - ims) + (k - kms) * sk + (j - jms) * sj];
  }
};
// 1 / d for the FP64 column arithmetic of the mixed form: an FP32 seed and
// two Newton-Raphson steps r <- r + r (1 - d r) in FP64 fma (each squares the
// relative error: 2^-24 -> 2^-48 -> below the FP64 rounding).  GB300 runs
// FP64 at 1/64 of the FP32 rate, so this replaces the longer IEEE double
// division in the per-level recursions; d is well inside the FP32 range.
__device__ __forceinline__ double drcp(double d) {
  double r = (double)(1.0f / (float)d);
  double e = fma(-d, r, 1.0);
  r = fma(r, e, r);
  e = fma(-d, r, 1.0);
  return fma(r, e, r);
}
// 1 / d in the column precision RC: IEEE division for the plain FP32 form
// (the reference's rounding), drcp for FP64.
template <typename RC> __device__ __forceinline__ RC rcp_rc(RC d) { return RC(1.) / d; }
template <> __device__ __forceinline__ double rcp_rc<double>(double d) { return drcp(d); }

__device__ __forceinline__ F3 f3(const Mem& m, int id) { return F3{m.f3[id], (int)m.sk, (int)m.sj, m.ims, m.kms, m.jms}; }
__device__ __forceinline__ F3 f3p(const Mem& m, float* p) { return F3{p, (int)m.sk, (int)m.sj, m.ims, m.kms, m.jms}; }
__device__ __forceinline__ F2 f2(const Mem& m, int id) {
  return F2{m.f2[id - WRFGPU_F2D_BASE], (int)m.s2, m.ims, m.jms};
}
__device__ __forceinline__ F1 f1(const Mem& m, int id) { return F1{m.f1[id - WRFGPU_F1D_BASE], m.kms}; }
__device__ __forceinline__ D3 d3(const Mem& m, double* p) { return D3{p, (int)m.sk, (int)m.sj, m.ims, m.kms, m.jms}; }

// ---------------------------------------------------------------------------
// Flux operators (module_advect_em.F:172-186; advect_scalar_pd's pre-divided
// coefficients :6165-6185).  sign(1,time_step) == 1 for forward runs.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float sgn1(float a) { return copysignf(1.f, a); }
// The divisions by 12 and 60 round exactly as IEEE division (cdiv.h).
__device__ __forceinline__ float flux4(float qm2, float qm1, float q, float qp1) {
  return wrfgpu_div12(7.f * (q + qm1) - (qp1 + qm2));
}
// flux4(...) + (1 sign(ua) (...)) / 12, the two quotients under one range test
__device__ __forceinline__ float flux3(float qm2, float qm1, float q, float qp1, float ua) {
  return wrfgpu_div12_add(7.f * (q + qm1) - (qp1 + qm2), 1.f * sgn1(ua) * ((qp1 - qm2) - 3.f * (q - qm1)));
}
__device__ __forceinline__ float flux6(float qm3, float qm2, float qm1, float q, float qp1, float qp2) {
  return wrfgpu_div60(37.f * (q + qm1) - 8.f * (qp1 + qm2) + (qp2 + qm3));
}
// flux6(...) - (1 sign(ua) (...)) / 60, the two quotients under one range test
__device__ __forceinline__ float flux5(float qm3, float qm2, float qm1, float q, float qp1, float qp2, float ua) {
  return wrfgpu_div60_sub(37.f * (q + qm1) - 8.f * (qp1 + qm2) + (qp2 + qm3),
                          1.f * sgn1(ua) * ((qp2 - qm3) - 5.f * (qp1 - qm2) + 10.f * (q - qm1)));
}
__device__ __forceinline__ float pflux4(float qm2, float qm1, float q, float qp1) {
  return (7.f / 12.f) * (q + qm1) - (1.f / 12.f) * (qp1 + qm2);
}
__device__ __forceinline__ float pflux3(float qm2, float qm1, float q, float qp1, float ua) {
  return pflux4(qm2, qm1, q, qp1) + 1.f * sgn1(ua) * (1.f / 12.f) * ((qp1 - qm2) - 3.f * (q - qm1));
}
__device__ __forceinline__ float pflux6(float qm3, float qm2, float qm1, float q, float qp1, float qp2) {
  return (37.f / 60.f) * (q + qm1) - (2.f / 15.f) * (qp1 + qm2) + (1.f / 60.f) * (qp2 + qm3);
}
__device__ __forceinline__ float pflux5(float qm3, float qm2, float qm1, float q, float qp1, float qp2, float ua) {
  return pflux6(qm3, qm2, qm1, q, qp1, qp2) -
         1.f * sgn1(ua) * (1.f / 60.f) * ((qp2 - qm3) - 5.f * (qp1 - qm2) + 10.f * (q - qm1));
}
__device__ __forceinline__ float fmaxf_f(float a, float b) { return a > b ? a : b; }   // Fortran MAX
__device__ __forceinline__ float fminf_f(float a, float b) { return a < b ? a : b; }   // Fortran MIN
__device__ __forceinline__ float flux_upwind(float qm1, float q, float cr) {
  return 0.5f * fminf_f(1.0f, (cr + fabsf(cr))) * qm1 + 0.5f * fmaxf_f(-1.0f, (cr - fabsf(cr))) * q;
}

// ---------------------------------------------------------------------------
// Launch geometry.  Every member's index space [ims+? ...] is cut into
// 32x4 (i x j) blocks covering i in [ims, ime], j in [jms, jme]; 3-D point
// kernels add a k index per block.  block_start[m] is the prefix of block
// counts; a block finds its member by binary search.
// ---------------------------------------------------------------------------
struct Launch {
  const Mem* mem;            // device array of members
  const int* block_start;    // [nmem+1] prefix over blocks of this launch kind
  int nmem;
  int kind;                  // 2: column blocks (i,j); 3: point blocks (i,j,k)
};

struct BlockPos {
  int m;      // member
  int i, j;   // Fortran indices of this thread
  int k;      // level (point kernels) or 0
  bool valid;
};

__device__ __forceinline__ int find_member(const int* __restrict__ bs, int nmem, int b) {
  int lo = 0, hi = nmem - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(bs + mid) <= b) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ BlockPos block_pos(const Launch& L) {
  BlockPos bp;
  int b = blockIdx.x;
  bp.m = find_member(L.block_start, L.nmem, b);
  const Mem& m = L.mem[bp.m];
  int lb = b - __ldg(L.block_start + bp.m);
  int nbx = (m.ime - m.ims + 1 + BX - 1) / BX;
  int nby = (m.jme - m.jms + 1 + BY - 1) / BY;
  int bxy = lb;
  bp.k = 0;
  if (L.kind == 3) { bp.k = lb / (nbx * nby) + m.kms; bxy = lb % (nbx * nby); }
  int bx = bxy % nbx, by = bxy / nbx;
  bp.i = m.ims + bx * BX + (int)threadIdx.x;
  bp.j = m.jms + by * BY + (int)threadIdx.y;
  bp.valid = bp.i <= m.ime && bp.j <= m.jme && (L.kind != 3 || bp.k <= m.kme);
  return bp;
}

inline int blocks_for(const int ims, const int ime, const int jms, const int jme, const int nk, int kind) {
  int nbx = (ime - ims + 1 + BX - 1) / BX;
  int nby = (jme - jms + 1 + BY - 1) / BY;
  return nbx * nby * (kind == 3 ? nk : 1);
}

// The block's member descriptor copied into shared memory.  Kernels then read
// bounds, strides and field pointers from there: a store to global memory
// cannot alias it, so they are not reloaded from the global member table
// after every store.  Every thread of the block must call it (it syncs).
__device__ __forceinline__ const Mem& block_member(const Mem* mems, int m) {
  __shared__ Mem s_mem;
  const int nthr = blockDim.x * blockDim.y, tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int4* src = reinterpret_cast<const int4*>(mems + m);
  int4* dst = reinterpret_cast<int4*>(&s_mem);
  for (int w = tid; w < (int)(sizeof(Mem) / 16); w += nthr) dst[w] = __ldg(src + w);
  __syncthreads();
  return s_mem;
}

// Column loop k = k0..k1 whose levels are independent of each other: the
// inputs of C levels are loaded (load(k, v)) before any of them is computed
// and stored (store(k, v)), so one memory round trip serves C levels instead
// of one.  Per-level arithmetic is untouched.
template <int C, typename T, typename LoadF, typename StoreF>
__device__ __forceinline__ void chunked_levels(int k0, int k1, LoadF load, StoreF store) {
  for (int kb = k0; kb <= k1; kb += C) {
    T v[C];
#pragma unroll
    for (int q = 0; q < C; ++q)
      if (kb + q <= k1) load(kb + q, v[q]);
#pragma unroll
    for (int q = 0; q < C; ++q)
      if (kb + q <= k1) store(kb + q, v[q]);
  }
}

__device__ __forceinline__ void raise_err(const Mem& m, unsigned bits) {
  if (m.err) atomicOr(m.err, bits);
}

// ---------------------------------------------------------------------------
// Tiled column-marching geometry.  A block owns a TX x TY tile of mass
// columns (i, j) and marches up k; horizontal stencil neighbours are staged
// per level in shared memory, vertical ones stay in registers.  Tiles cover
// the computed mass region [its, min(ite, ide-1)] x [jts, min(jte, jde-1)]
// of each member; `per_tile` blocks per tile (species for the scalar
// kernels, fastest-varying so the blocks of one tile run together and share
// the mass fluxes through L2).
// ---------------------------------------------------------------------------
constexpr int TX = 32, TY = 8;

// Asynchronous global -> shared copies (cp.async, 4 bytes per element) used
// to keep several k levels of a tile's planes in flight.
__device__ __forceinline__ void cp_async4(float* smem, const float* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ void prefetch_l2(const float* p) { asm volatile("prefetch.global.L2 [%0];\n" ::"l"(p)); }

// TMA tile loads completing on an mbarrier (transaction bytes).
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Bounded wait for phase `parity` of the barrier; false after `polls` polls
// (2^22 by default: seconds), in which case the caller flags ERR_TIMEOUT and
// carries on.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int polls = 1 << 22) {
  const unsigned a = smem_u32(bar);
  for (int it = 0; it < polls; ++it) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void tma_load_3d(float* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// A ring of level slots for column kernels: each slot holds NF planes of one
// level, all of one TMA box (PW x PH floats, row by row) and completes on its
// own mbarrier.  Thread 0 issues; every thread waits.  A slot is reused for
// level k + NSLOT only after a block barrier that follows the last read of
// level k (the caller's loop places it).
// Every plane starts on a 128-byte boundary (the TMA destination rule), and
// SMEM is a multiple of 128 bytes so that rings can be stacked.
template <int NF, int NSLOT, int PW = TX, int PH = TY>
struct LevelRing {
  float* buf;      // [NSLOT][NF][PSTRIDE]
  uint64_t* bar;   // [NSLOT]
  int k0;          // first level staged
  static constexpr unsigned PLANE = PW * PH;               // floats a box delivers
  static constexpr unsigned PSTRIDE = (PLANE + 31) / 32 * 32;  // floats between planes
  static constexpr size_t DATA = (size_t)NSLOT * NF * PSTRIDE * 4;
  static constexpr size_t SMEM = DATA + (NSLOT * 8 + 127) / 128 * 128;
  __device__ int slot_of(int k) const { return (k - k0) % NSLOT; }
  __device__ const float* plane(int k, int f) const { return buf + (slot_of(k) * NF + f) * PSTRIDE; }
  // carve the ring out of shared memory at `smem` (128-byte aligned)
  __device__ void init(unsigned char* smem, int first_level) {
    buf = (float*)smem;
    bar = (uint64_t*)(smem + DATA);
    k0 = first_level;
  }
  __device__ void init_barriers() const {
    for (int q = 0; q < NSLOT; ++q) mbar_init(&bar[q], 1);
  }
  // thread 0: level k of the NF fields into its slot (box origin x0, z0)
  __device__ void issue(int k, const CUtensorMap* const* maps, int x0, int z0, int kms) const {
    const int sl = slot_of(k);
    fence_proxy_async_smem();
    mbar_expect_tx(&bar[sl], NF * PLANE * 4);
    for (int f = 0; f < NF; ++f) tma_load_3d(buf + (sl * NF + f) * PSTRIDE, maps[f], x0, k - kms, z0, &bar[sl]);
  }
  __device__ bool wait(int k) const { return mbar_wait(&bar[slot_of(k)], ((k - k0) / NSLOT) & 1); }
};
template <int NF, int NSLOT> using TileRing = LevelRing<NF, NSLOT, TX, TY>;

// The interior mass point (i, j) and every halo point whose periodic image
// (or, with symmetric y boundaries, mirror image) it is: the points that
// the halo fill of a mass-point field ('p', 'w' or 't', share/module_bc.F:
// 651-1000) gives its value (the x halo of the interior rows, then whole
// halo rows ims..ide+3).  A producer that stores through store() leaves out
// the fill that would follow it.  Formed once per column; a point away from
// the edges has no image and store() is one store.
struct MassImages {
  static constexpr int NONE = -1000000;
  int i, j, xa, xb, ya, yb;  // the point, and its x and y images (NONE: absent)
  bool any;
  __device__ __forceinline__ void init(const Mem& m, int i_, int j_) {
    i = i_; j = j_;
    xa = xb = ya = yb = NONE;
    if (m.cf.periodic_x) {
      const int np = m.ide - 1;
      if (i - np >= m.ims) xa = i - np;
      if (i + np <= m.ide + WRFGPU_HALO - 1) xb = i + np;
    }
    const int npy = m.jde - 1;
    if (m.cf.periodic_y) {
      if (j - npy >= m.jms) ya = j - npy;
      if (j + npy <= m.jde + WRFGPU_HALO - 1) yb = j + npy;
    } else if (m.cf.symmetric_ys && m.cf.symmetric_ye) {
      if (1 - j >= m.jms) ya = 1 - j;
      if (2 * npy + 1 - j <= m.jde + WRFGPU_HALO - 1) yb = 2 * npy + 1 - j;
    }
    any = xa != NONE || xb != NONE || ya != NONE || yb != NONE;
  }
  template <class ST>
  __device__ __forceinline__ void row(int jj, ST& st) const {
    st(i, jj);
    if (xa != NONE) st(xa, jj);
    if (xb != NONE) st(xb, jj);
  }
  template <class ST>
  __device__ __forceinline__ void store(ST st) const {
    if (!any) { st(i, j); return; }
    row(j, st);
    if (ya != NONE) row(ya, st);
    if (yb != NONE) row(yb, st);
  }
};

// Edge-strip launches of members with open boundaries (open_adv.cuh):
// blocks of STRIP_THREADS over each member's strip points.
constexpr int STRIP_THREADS = 256;
struct StripLaunch {
  const Mem* mem;
  const int* block_start;  // [nmem+1] prefix over strip blocks
  int nmem;
  int w;  // strip width: the columns within w - 1 of an open edge
  int h;  // 1: the x strips also cover the halo row jds-1 and the y strips the halo column ids-1
};

struct TileLaunch {
  const Mem* mem;
  const int* block_start;  // [nmem+1] prefix over tiles x per_tile
  int nmem;
};

struct TilePos {
  int m;       // member
  int i0, j0;  // first column of the tile
  int sub;     // 0 .. per_tile-1 (species)
};

// stag: tiles cover the staggered extents [its, ite] x [jts, jte] (u, v and
// mass points of the same column handled together) instead of the mass ones.
__host__ __device__ inline int tiles_x(const Mem& m, bool stag = false) {
  const int itf = stag ? m.ite : (m.ite < m.ide - 1 ? m.ite : m.ide - 1);
  return (itf - m.its + TX) / TX;
}
__host__ __device__ inline int tiles_y(const Mem& m, bool stag = false) {
  const int jtf = stag ? m.jte : (m.jte < m.jde - 1 ? m.jte : m.jde - 1);
  return (jtf - m.jts + TY) / TY;
}

// Blocks per tile: one, one per species, or one per pair of species
// (species 2 sub and 2 sub + 1).
enum { TILE_ONE = 0, TILE_PER_SPECIES = 1, TILE_PER_PAIR = 2 };
__host__ __device__ inline int blocks_per_tile(int nsp, int per_mode) {
  return per_mode == TILE_PER_SPECIES ? nsp : per_mode == TILE_PER_PAIR ? (nsp + 1) / 2 : 1;
}
__device__ __forceinline__ TilePos tile_pos(const TileLaunch& L, int per_mode, bool stag = false) {
  TilePos t;
  const int b = blockIdx.x;
  t.m = find_member(L.block_start, L.nmem, b);
  const Mem& m = L.mem[t.m];
  const int lb = b - __ldg(L.block_start + t.m);
  const int per = blocks_per_tile(m.nsp, per_mode);
  const int tile = lb / per;
  t.sub = lb - tile * per;
  const int ntx = tiles_x(m, stag);
  t.i0 = m.its + (tile % ntx) * TX;
  t.j0 = m.jts + (tile / ntx) * TY;
  return t;
}

}  // namespace wrfgpu
