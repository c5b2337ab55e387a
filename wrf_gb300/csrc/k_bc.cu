// On-device halo fill: the single-GPU replacement of the reference's
// set_physical_bc3d / set_physical_bc2d (share/module_bc.F:202-1000) at each
// sync site of solve_em, for periodic lateral boundaries in x and periodic
// or symmetric boundaries in y.
//
// The reference fills the x halo of rows jds..jde(+stag) first and then
// copies whole rows into the y halo, so every halo point ends up holding the
// value of one interior point: its periodic image, or its mirror image (with
// a sign change for the normal velocity v).  This kernel computes that source
// point directly, so all points of a field are written in one pass with no
// ordering between them.  The points written and the values they receive
// are the reference's, except the never-read column ime of fields that are
// not x-staggered, which the reference fills with whatever its x pass left
// there and this kernel leaves untouched.
// Roofline: pure copy, 2 x 4 B per halo point; a few percent of a step.
#include "common.cuh"
#include "kernels.h"

namespace wrfgpu {

__device__ __forceinline__ int bc_src(int t, int n, bool stag, bool periodic, bool normal_flip, bool* neg) {
  const int nper = n - 1;
  if (periodic) return ((t - 1) % nper + nper) % nper + 1;
  if (!stag) {
    if (t < 1) return 1 - t;                  // dat(ids-i) = dat(ids+i-1)
    if (t > nper) return 2 * nper + 1 - t;    // dat(ide+i-1) = dat(ide-i)
    return t;
  }
  if (t < 1) { if (normal_flip) *neg = !*neg; return 2 - t; }      // dat(ids-i) = -dat(ids+i)
  if (t > n) { if (normal_flip) *neg = !*neg; return 2 * n - t; }  // dat(ide+i) = -dat(ide-i)
  return t;
}

// grid: (blocks per job, jobs, members)
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
  const bool px = m.cf.periodic_x, py = m.cf.periodic_y;
  const bool sy = m.cf.symmetric_ys && m.cf.symmetric_ye;
  const int nxl = WRFGPU_HALO;
  const int xr0 = m.ide, xr1 = m.ide + 4 + istag;  // periodic x only
  const int nxr = xr1 - xr0 + 1;
  const int yr0 = py ? m.jde : (vs ? m.jde + 1 : m.jde);
  const int yr1 = py ? m.jde + 4 + jstag : (vs ? m.jde + 4 : m.jde + 3);
  const int nyr = yr1 - yr0 + 1;
  const int xj0 = m.jds, xj1 = m.jde + jstag;
  const int yi0 = m.ims, yi1 = us ? m.ime : m.ide + 3;
  // 32-bit index space (a member's field holds < 2^31 points); points of a
  // level are consecutive, i (or the x-halo column) fastest
  const int nxw = nxl + nxr, nyi = yi1 - yi0 + 1;
  const int nxpts = px ? nxw * (xj1 - xj0 + 1) : 0;
  const int nypts = (py || sy) ? (WRFGPU_HALO + nyr) * nyi : 0;
  const int npts = nxpts + nypts;
  const int total = npts * nk;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int kk = t / npts;
    const int pt = t - kk * npts;
    const int k = kk + m.kts;
    int ti, tj;
    if (pt < nxpts) {
      const int r = pt / nxw, c = pt - r * nxw;
      tj = xj0 + r;
      ti = c < nxl ? m.ids - nxl + c : xr0 + (c - nxl);
    } else {
      const int q = pt - nxpts;
      const int r = q / nyi;
      ti = yi0 + (q - r * nyi);
      tj = r < WRFGPU_HALO ? m.jds - WRFGPU_HALO + r : yr0 + (r - WRFGPU_HALO);
    }
    bool neg = false;
    int si = px ? bc_src(ti, m.ide, us, true, false, &neg) : ti;
    int sj = (py || sy) ? bc_src(tj, m.jde, vs, py, var == 'v', &neg) : tj;
    if (J.kind == 3) {
      F3 a = f3p(m, base);
      float val = a(si, k, sj);
      a(ti, k, tj) = neg ? -val : val;
    } else {
      F2 a{base, (int)m.s2, m.ims, m.jms};
      float val = a(si, sj);
      a(ti, tj) = neg ? -val : val;
    }
  }
}

void launch_fill_halo(const Mem* d_mems, int nmem, const HaloJobs& jobs, int blocks_per_job, cudaStream_t s) {
  if (jobs.n <= 0 || nmem <= 0) return;
  k_fill_halo<<<dim3(blocks_per_job, jobs.n, nmem), 256, 0, s>>>(d_mems, jobs);
}

}  // namespace wrfgpu
