// On-device halo fill: the single-GPU replacement of the reference's
// set_physical_bc3d / set_physical_bc2d (share/module_bc.F:202-1107) at each
// sync site of solve_em, for periodic or open lateral boundaries in x and
// periodic, symmetric or open boundaries in y.
//
// The reference fills the x halo first and then copies whole rows into the
// y halo, so every halo point ends up holding the value of one other point:
// its periodic image, its mirror image (with a sign change for the normal
// velocity v), or, next to an open boundary, the edge value copied into
// three halo points (module_bc.F:864-1107, for the variables of
// open_bc_copy).  This kernel computes that source point directly, so all
// points of a field are written in one pass with no ordering between them.
// The points written and the values they receive are the reference's,
// except the never-read column ime of fields that are not x-staggered,
// which the reference fills with whatever its x pass left there and this
// kernel leaves untouched.
// Roofline: pure copy, 2 x 4 B per halo point; a few percent of a step.
#include "common.cuh"
#include "kernels.h"

namespace wrfgpu {

// Source index along one direction of halo index t (1-based domain extent
// n, nper = n - 1 interior mass points).  Periodic: the image one period
// away (|halo| <= 5 < nper, so one conditional add replaces the modulo).
__device__ __forceinline__ int bc_src(int t, int n, bool stag, bool periodic, bool normal_flip, bool* neg) {
  const int nper = n - 1;
  if (periodic) return t < 1 ? t + nper : (t > nper ? t - nper : t);
  if (!stag) {
    if (t < 1) return 1 - t;                  // dat(ids-i) = dat(ids+i-1)
    if (t > nper) return 2 * nper + 1 - t;    // dat(ide+i-1) = dat(ide-i)
    return t;
  }
  if (t < 1) { if (normal_flip) *neg = !*neg; return 2 - t; }      // dat(ids-i) = -dat(ids+i)
  if (t > n) { if (normal_flip) *neg = !*neg; return 2 * n - t; }  // dat(ide+i) = -dat(ide-i)
  return t;
}

// Open boundaries (module_bc.F:864-925 in x, :1059-1107 in y): the source of
// halo index t, or t itself where the open copy writes nothing (the fourth
// halo point, and t = ide+3 / ide+4 beyond the three copies).
__device__ __forceinline__ int open_src(int t, int n, bool stag) {
  if (t >= -2 && t <= 0) return 1;
  if (stag) return (t >= n + 1 && t <= n + 3) ? n : t;
  return (t >= n && t <= n + 2) ? n - 1 : t;
}
// open_bc_copy of set_physical_bc3d (module_bc.F:699-704) and
// set_physical_bc2d (:248-251)
__device__ __forceinline__ bool open_copy(char v, bool f3d) {
  if (v == 'u' || v == 'v' || v == 'w' || v == 't' || v == 'x' || v == 'y' || v == 'r' || v == 'p') return true;
  return f3d && (v == 'd' || v == 'e' || v == 'f');
}

// grid: (blocks per job, jobs, members).  Work units: for the x halo
// (periodic x) one (level, row) segment of nxw <= 9 points per thread, for
// the y halo one (level, halo row, 128 points of i) piece per warp, four
// points per lane.  A unit's loads are all issued before its stores (a store
// may alias a later load as far as the compiler knows, so copying point by
// point would wait out one memory latency per point).  The points written by
// the two kinds of unit are disjoint and every source point is an interior
// point (or, without periodic x, a point no unit writes), so the units need
// no ordering.
__global__ void k_fill_halo(const Mem* __restrict__ mems, HaloJobs jobs) {
  const Mem& m = block_member(mems, blockIdx.z);
  const HaloJob& J = jobs.job[blockIdx.y];
  float* base = J.species >= 0 ? (J.species < m.nsp ? (J.old ? m.qo[J.species] : m.q[J.species]) : nullptr)
                               : (J.kind == 3 ? m.f3[J.id] : m.f2[J.id - WRFGPU_F2D_BASE]);
  if (!base) return;
  const char var = J.var;
  const bool us = (var == 'u' || var == 'x'), vs = (var == 'v' || var == 'y');
  const int istag = us ? 0 : -1, jstag = vs ? 0 : -1;
  int k_end = 1;
  if (J.kind == 3) {
    k_end = max(1, min(m.kde - 1, m.kte));
    if (var == 'w') k_end = min(m.kde, m.kte);
  }
  const int nk = (J.kind == 3) ? (k_end - m.kts + 1) : 1;
  const bool f3d = J.kind == 3;
  const bool px = m.cf.periodic_x, py = m.cf.periodic_y;
  const bool sy = m.cf.symmetric_ys && m.cf.symmetric_ye;
  const bool copy = open_copy(var, f3d);
  const bool ox = m.cf.open_xs && copy, oy = m.cf.open_ys && copy;  // open on both sides
  constexpr int NXW_MAX = 2 * WRFGPU_HALO + 1;
  // x halo columns written: periodic, ids-4..ids-1 and ide..ide+4+istag;
  // open, ids-3..ids-1 and three past the edge point
  const int nxl = ox ? 3 : WRFGPU_HALO;
  const int xr0 = ox ? (us ? m.ide + 1 : m.ide) : m.ide;
  const int xr1 = ox ? xr0 + 2 : m.ide + 4 + istag;
  const int nxw = nxl + (xr1 - xr0 + 1);  // <= NXW_MAX
  // y halo rows written
  const int ynl = oy ? 3 : WRFGPU_HALO;
  const int yr0 = oy ? (vs ? m.jde + 1 : m.jde) : (py ? m.jde : (vs ? m.jde + 1 : m.jde));
  const int yr1 = oy ? yr0 + 2 : (py ? m.jde + 4 + jstag : (vs ? m.jde + 4 : m.jde + 3));
  const int nyrows = ynl + (yr1 - yr0 + 1);
  // rows of the x units: the domain rows, and with open x and open y the two
  // 3-D rows of the x pass (jts-bdyzone .. jde+jstag+bdyzone, module_bc.F:870)
  // that the y pass does not overwrite
  const bool xextra = ox && oy && f3d;
  const int xj0 = m.jds, xj1 = m.jde + jstag;
  const int nxj = xj1 - xj0 + 1 + (xextra ? 2 : 0);
  const int yi0 = m.ims, yi1 = us ? m.ime : m.ide + 3;
  const int nyi = yi1 - yi0 + 1;
  // source column of x index ti as the x pass leaves it
  auto xsrc = [&](int ti, bool* neg) -> int {
    if (px) return bc_src(ti, m.ide, us, true, false, neg);
    if (ox) return open_src(ti, m.ide, us);
    return ti;
  };
  // 32-bit offsets of (i, k, j) / (i, j) in the field
  const int sk = (int)m.sk, sj = f3d ? (int)m.sj : (int)m.s2;
  auto off = [&](int i, int k, int j) { return (i - m.ims) + (f3d ? (k - m.kms) * sk : 0) + (j - m.jms) * sj; };
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nthr = gridDim.x * blockDim.x;
  if (px || ox) {
    const int nunits = nk * nxj;
    for (int u = tid; u < nunits; u += nthr) {
      const int kk = u / nxj;
      const int r = u - kk * nxj, k = kk + m.kts;
      const int tj = r <= xj1 - xj0 ? xj0 + r : (r == xj1 - xj0 + 1 ? m.jds - WRFGPU_HALO : m.jde + jstag + WRFGPU_HALO);
      bool negj = false;
      const int sjj = (py || sy) ? bc_src(tj, m.jde, vs, py, var == 'v', &negj) : tj;
      float val[NXW_MAX];
#pragma unroll
      for (int c = 0; c < NXW_MAX; ++c) {
        if (c < nxw) {
          const int ti = c < nxl ? m.ids - nxl + c : xr0 + (c - nxl);
          bool neg = false;
          const int si = xsrc(ti, &neg);
          val[c] = base[off(si, k, sjj)];
        }
      }
#pragma unroll
      for (int c = 0; c < NXW_MAX; ++c) {
        if (c < nxw) {
          const int ti = c < nxl ? m.ids - nxl + c : xr0 + (c - nxl);
          base[off(ti, k, tj)] = negj ? -val[c] : val[c];
        }
      }
    }
  }
  if (py || sy || oy) {
    constexpr int PER = 4;  // points per lane
    const int lane = threadIdx.x & 31, warp = tid >> 5, nwarps = nthr >> 5;
    const int npiece = (nyi + 32 * PER - 1) / (32 * PER);
    const int nunits = nk * nyrows * npiece;
    for (int w = warp; w < nunits; w += nwarps) {
      const int row = w / npiece, pc = w - row * npiece;
      const int kk = row / nyrows, r = row - kk * nyrows;
      const int k = kk + m.kts;
      const int tj = r < ynl ? m.jds - ynl + r : yr0 + (r - ynl);
      bool negj = false;
      const int sjj = oy ? open_src(tj, m.jde, vs) : bc_src(tj, m.jde, vs, py, var == 'v', &negj);
      float val[PER];
      bool neg[PER];
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        const int ii = pc * 32 * PER + q * 32 + lane;
        neg[q] = negj;
        if (ii < nyi) {
          const int ti = yi0 + ii;
          const int si = xsrc(ti, &neg[q]);
          val[q] = base[off(si, k, sjj)];
        }
      }
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        const int ii = pc * 32 * PER + q * 32 + lane;
        if (ii < nyi) base[off(yi0 + ii, k, tj)] = neg[q] ? -val[q] : val[q];
      }
    }
  }
}

// Row copies between a contiguous buffer (rows of `cols` values, the
// caller's Fortran layout) and a field's padded device rows (`pitch` apart);
// `dst2`, when given, receives the same rows (a species' spare buffer).  One
// warp per row, the rows grid-strided over a grid of a few blocks per SM:
// coalesced loads and stores, and no launch of one tiny block per row
// fragment.
__device__ __forceinline__ void copy_rows(const float* __restrict__ src, size_t src_pitch, float* __restrict__ dst,
                                          float* __restrict__ dst2, size_t dst_pitch, int cols, int rows) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarp = (gridDim.x * blockDim.x) >> 5;
  for (int r = warp; r < rows; r += nwarp) {
    const float* sr = src + (size_t)r * src_pitch;
    float* dr = dst + (size_t)r * dst_pitch;
    float* dr2 = dst2 ? dst2 + (size_t)r * dst_pitch : nullptr;
    for (int c = lane; c < cols; c += 32) {
      const float v = sr[c];
      dr[c] = v;
      if (dr2) dr2[c] = v;
    }
  }
}
__global__ void k_unpack_rows(const float* __restrict__ src, float* __restrict__ dst, float* __restrict__ dst2,
                              int cols, int rows, int pitch) {
  copy_rows(src, cols, dst, dst2, pitch, cols, rows);
}
__global__ void k_pack_rows(const float* __restrict__ src, float* __restrict__ dst, int cols, int rows, int pitch) {
  copy_rows(src, pitch, dst, nullptr, cols, cols, rows);
}
// The same for species s of member `member`, whose current and spare buffers
// are read from the device member table when the copy runs (the buffers
// exchange roles at every scalar update, so a captured copy must not hold
// their addresses).  Unpacking writes both buffers.
__global__ void k_unpack_species(const Mem* __restrict__ mems, int member, int s, const float* __restrict__ src,
                                 int cols, int rows, int pitch) {
  copy_rows(src, cols, mems[member].q[s], mems[member].qa[s], pitch, cols, rows);
}
__global__ void k_pack_species(const Mem* __restrict__ mems, int member, int s, float* __restrict__ dst, int cols,
                               int rows, int pitch) {
  copy_rows(mems[member].q[s], pitch, dst, nullptr, cols, cols, rows);
}
static int rows_grid(int rows) {  // 256-thread blocks of 8 row-warps, at most 8 blocks per SM of 152
  return rows / 8 + 1 < 8 * 152 ? rows / 8 + 1 : 8 * 152;
}
void launch_unpack_rows(const float* src, float* dst, float* dst2, int cols, int rows, int pitch, cudaStream_t s) {
  if (cols > 0 && rows > 0) k_unpack_rows<<<rows_grid(rows), 256, 0, s>>>(src, dst, dst2, cols, rows, pitch);
}
void launch_pack_rows(const float* src, float* dst, int cols, int rows, int pitch, cudaStream_t s) {
  if (cols > 0 && rows > 0) k_pack_rows<<<rows_grid(rows), 256, 0, s>>>(src, dst, cols, rows, pitch);
}
void launch_unpack_species(const Mem* mems, int member, int s, const float* src, int cols, int rows, int pitch,
                           cudaStream_t st) {
  if (cols > 0 && rows > 0) k_unpack_species<<<rows_grid(rows), 256, 0, st>>>(mems, member, s, src, cols, rows, pitch);
}
void launch_pack_species(const Mem* mems, int member, int s, float* dst, int cols, int rows, int pitch,
                         cudaStream_t st) {
  if (cols > 0 && rows > 0) k_pack_species<<<rows_grid(rows), 256, 0, st>>>(mems, member, s, dst, cols, rows, pitch);
}

void launch_fill_halo(const Mem* d_mems, int nmem, const HaloJobs& jobs, int blocks_per_job, cudaStream_t s) {
  if (jobs.n <= 0 || nmem <= 0) return;
  k_fill_halo<<<dim3(blocks_per_job, jobs.n, nmem), 256, 0, s>>>(d_mems, jobs);
}

}  // namespace wrfgpu
