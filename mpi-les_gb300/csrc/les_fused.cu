// les_fused.cu -- fused stage kernels of the whole time step (velfg+feedbf, les, les+adam).
//
// Same arithmetic as the per-subroutine kernels (bit for bit), organised for speed:
//   * each face quantity pair (nou_n, diu_n) of vel2.f95:74-197 is formed once per
//     face a cell needs, and cov_n = nou_n*diu_n reuses it;
//   * when every x and y spacing of the grid is one power of two (checked at set-up:
//     dx1, dy1, dxs, dys all equal to the same 2^e), a division by dx1, dy1, dxs, dys
//     or by the sum of two of them is a multiplication by the exact reciprocal: both
//     round the same real number, so the results are identical;
//   * when every spacing, spacing sum and scalar divisor lies in [2^-20, 2^20] (checked
//     at set-up), the other divisions by set-up constants use dvz (les_common.cuh): a
//     reciprocal multiply with one exact remainder correction, giving the IEEE quotient
//     bit for bit, without branches; the rare cell with a dividend outside that range
//     is recomputed with IEEE divisions;
//   * the wall plane (speeds, log-law gradients, u/uspd ratios) is a separate small
//     kernel, so the 3-D kernels hold no division by a computed value;
//   * velfg stores the nine diu fields it forms (as the reference's vel2 does) and
//     les reads them back with plain stencil loads, so les does no gradient work;
//   * feedbf (feedbf.f95:35-61) is applied in the velfg epilogue and adam
//     (adam.f95:30-44) in the les epilogue when the step runs them back to back.
#include <cuda_runtime.h>

#include <algorithm>

#include "les_common.cuh"
#include "les_kernels.cuh"

namespace {

// Thread blocks cover FX x FY x FZ cells (i, j, k); several k planes per block keep the
// k-1/k+1 neighbours of the stencils inside one block's L1 working set.
constexpr int FX = 32, FY = 2, FZ = 4;

#define FUSED_IJK                                     \
  const int i = blockIdx.x * FX + threadIdx.x + 1;    \
  const int j = blockIdx.y * FY + threadIdx.y + 1;    \
  const int k = blockIdx.z * FZ + threadIdx.z + 1;    \
  if (i > d.im || j > d.jm || k > d.km) return;

// Inputs the fused kernels only read go through the read-only (non-coherent) path:
// u, v, w in velfg; sm, diu and the wall ratios in les.
#define DIU_(n, i, j, k) __ldg(&d.diu[n][lix(d, (i), (j), (k))])
#define UR_(i, j, k) __ldg(&d.u[lix(d, (i), (j), (k))])
#define VR_(i, j, k) __ldg(&d.v[lix(d, (i), (j), (k))])
#define WR_(i, j, k) __ldg(&d.w[lix(d, (i), (j), (k))])

struct NouDiu {
  float nou, diu;
};

// ---- the nine face pairs of vel2.f95:74-197, with the halo copies of :202-318 as
// index remaps.  P2 / ZF select the division forms (dvs, dvz); bd collects dividends
// outside the reciprocal-corrected range.
template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face1(const LesDom &d, int i, int j, int k, unsigned &bd) {
  const int ii = min(i, d.im);
  const float a = UR_(ii - 1, j, k), b = UR_(ii, j, k);
  return {(a + b) / 2.f, dvs<P2, ZF>(-a + b, d.gr.dx1[ii], d.gr.rdx1[ii], bd)};
}
template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face2(const LesDom &d, int i, int j, int k, unsigned &bd) {
  const int jj = (j > d.jm) ? 1 : j;
  const float *dx1 = d.gr.dx1, *dy1 = d.gr.dy1;
  const float nou = dvs<P2, ZF>(dx1[i + 1] * VR_(i, jj - 1, k) + dx1[i] * VR_(i + 1, jj - 1, k), dx1[i] + dx1[i + 1],
                                d.gr.rdx1s[i], bd);
  const float diu = dvs<P2, ZF>(2.f * (-UR_(i, jj - 1, k) + UR_(i, jj, k)), dy1[jj - 1] + dy1[jj], d.gr.rdy1s[jj - 1], bd);
  return {nou, diu};
}
// diu3 at k = 1 is the log-law wall gradient, stored by k_wall before this kernel runs
template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face3(const LesDom &d, int i, int j, int k, unsigned &bd) {
  const float *dx1 = d.gr.dx1;
  if (k == 1) {
    const float nou = dvs<P2, ZF>(0.5f * (dx1[i + 1] * WR_(i, j, 1) + dx1[i] * WR_(i + 1, j, 1)), dx1[i] + dx1[i + 1],
                                  d.gr.rdx1s[i], bd);
    return {nou, DIU_(3, i, j, 1)};
  }
  const float nou = dvs<P2, ZF>(dx1[i + 1] * WR_(i, j, k - 1) + dx1[i] * WR_(i + 1, j, k - 1), dx1[i] + dx1[i + 1],
                                d.gr.rdx1s[i], bd);
  return {nou, dvz<ZF>(-UR_(i, j, k - 1) + UR_(i, j, k), d.gr.dzs[k - 1], d.gr.rdzs[k - 1], bd)};
}
template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face4(const LesDom &d, int i, int j, int k, unsigned &bd) {
  const int ii = min(i, d.im);
  const float *dx1 = d.gr.dx1, *dy1 = d.gr.dy1;
  const float nou = dvs<P2, ZF>(dy1[j + 1] * UR_(ii - 1, j, k) + dy1[j] * UR_(ii - 1, j + 1, k), dy1[j] + dy1[j + 1],
                                d.gr.rdy1s[j], bd);
  const float diu = dvs<P2, ZF>(2.f * (-VR_(ii - 1, j, k) + VR_(ii, j, k)), dx1[ii - 1] + dx1[ii], d.gr.rdx1s[ii - 1], bd);
  return {nou - 0.f, diu};
}
template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face5(const LesDom &d, int i, int j, int k, unsigned &bd) {
  const int jj = (j > d.jm) ? 1 : j;
  const float a = VR_(i, jj - 1, k), b = VR_(i, jj, k);
  return {(a + b) / 2.f, dvs<P2, ZF>(-a + b, d.gr.dy1[jj], d.gr.rdy1[jj], bd)};
}
// diu6 at k = 1: stored by k_wall
template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face6(const LesDom &d, int i, int j, int k, unsigned &bd) {
  const float *dy1 = d.gr.dy1;
  if (k == 1) {
    const float nou = dvs<P2, ZF>(0.5f * (dy1[j + 1] * WR_(i, j, 1) + dy1[j] * WR_(i, j + 1, 1)), dy1[j] + dy1[j + 1],
                                  d.gr.rdy1s[j], bd);
    return {nou, DIU_(6, i, j, 1)};
  }
  const float nou = dvs<P2, ZF>(dy1[j + 1] * WR_(i, j, k - 1) + dy1[j] * WR_(i, j + 1, k - 1), dy1[j] + dy1[j + 1],
                                d.gr.rdy1s[j], bd);
  return {nou, dvz<ZF>(-VR_(i, j, k - 1) + VR_(i, j, k), d.gr.dzs[k - 1], d.gr.rdzs[k - 1], bd)};
}
template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face7(const LesDom &d, int i, int j, int k, unsigned &bd) {
  const int ii = min(i, d.im);
  const float *dx1 = d.gr.dx1, *dzn = d.gr.dzn;
  const float nou =
      dvz<ZF>(dzn[k + 1] * UR_(ii - 1, j, k) + dzn[k] * UR_(ii - 1, j, k + 1), dzn[k] + dzn[k + 1], d.gr.rdzsum[k], bd);
  const float diu = dvs<P2, ZF>(2.f * (-WR_(ii - 1, j, k) + WR_(ii, j, k)), dx1[ii - 1] + dx1[ii], d.gr.rdx1s[ii - 1], bd);
  return {nou - 0.f, diu};
}
template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face8(const LesDom &d, int i, int j, int k, unsigned &bd) {
  const int jj = (j > d.jm) ? 1 : j;
  const float *dy1 = d.gr.dy1, *dzn = d.gr.dzn;
  const float nou =
      dvz<ZF>(dzn[k + 1] * VR_(i, jj - 1, k) + dzn[k] * VR_(i, jj - 1, k + 1), dzn[k] + dzn[k + 1], d.gr.rdzsum[k], bd);
  const float diu = dvs<P2, ZF>(2.f * (-WR_(i, jj - 1, k) + WR_(i, jj, k)), dy1[jj - 1] + dy1[jj], d.gr.rdy1s[jj - 1], bd);
  return {nou, diu};
}
template <bool ZF>
__device__ __forceinline__ NouDiu face9(const LesDom &d, int i, int j, int k, unsigned &bd) {
  const float a = WR_(i, j, k - 1), b = WR_(i, j, k);
  return {(a + b) / 2.f, dvz<ZF>(-a + b, d.gr.dzn[k], d.gr.rdzn[k], bd)};
}

// ------------------------------------------------------------------ vel2.f95:54-65,138,173,351-356
// Wall plane k = 1: the speeds uspd, vspd, the log-law gradients diu3(i,j,1), diu6(i,j,1)
// and the ratios u/uspd, v/vspd that les reads.  Divisions by the speeds stay IEEE.
__global__ void k_wall(LesDom d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y + 1;
  if (i > d.im) return;
  const float us = uspd_raw(d, i, j), vs = vspd_raw(d, i, j);
  const float u = U_(i, j, 1), v = V_(i, j, 1);
  const int c2 = (j + LES_JOFF) * d.pi + i + LES_IOFF;
  d.ruspd[c2] = u / us;
  d.rvspd[c2] = v / vs;
  const int c = lix(d, i, j, 1);
  d.diu[3][c] = wall_grad(d, us, u);
  d.diu[6][c] = wall_grad(d, vs, v);
}

// ------------------------------------------------------------------ velFG.f95:64-110
// One cell's f, g (k = 1..km), h (k = 1..km-1) and the diu it forms.
struct VelfgOut {
  float f, g, h;
  float d1, d2, d3, d4, d5, d6, d7, d8, d9;
  float d3t, d6t;  // diu3, diu6 at km+1 (k = km only)
};
template <bool P2, bool ZF>
__device__ __forceinline__ void velfg_cell(const LesDom &d, int i, int j, int k, int c, VelfgOut &o, unsigned &bd) {
  const float *dx1 = d.gr.dx1, *dy1 = d.gr.dy1, *dzn = d.gr.dzn, *dzs = d.gr.dzs;
  const float *rdx1 = d.gr.rdx1, *rdx1s = d.gr.rdx1s, *rdy1 = d.gr.rdy1, *rdy1s = d.gr.rdy1s;
  const float *rdzn = d.gr.rdzn, *rdzs = d.gr.rdzs, *rdzsum = d.gr.rdzsum;
  {  // u
    const NouDiu a = face1<P2, ZF>(d, i, j, k, bd), b = face1<P2, ZF>(d, i + 1, j, k, bd);
    const NouDiu y0 = face2<P2, ZF>(d, i, j, k, bd), y1 = face2<P2, ZF>(d, i, j + 1, k, bd);
    const NouDiu z0 = face3<P2, ZF>(d, i, j, k, bd), z1 = face3<P2, ZF>(d, i, j, k + 1, bd);
    o.d1 = a.diu; o.d2 = y0.diu; o.d3 = z0.diu; o.d3t = z1.diu;
    const float covx1 = dvs<P2, ZF>(dx1[i + 1] * (a.nou * a.diu) + dx1[i] * (b.nou * b.diu), dx1[i] + dx1[i + 1], rdx1s[i], bd);
    const float covy1 = (y0.nou * y0.diu + y1.nou * y1.diu) / 2.f;
    const float covz1 = (z0.nou * z0.diu + z1.nou * z1.diu) / 2.f;
    const float covc = covx1 + covy1 + covz1;
    const float dfu1 = dvs<P2, ZF>(2.f * (-a.diu + b.diu), dx1[i] + dx1[i + 1], rdx1s[i], bd) +
                       dvs<P2, ZF>(-y0.diu + y1.diu, dy1[j], rdy1[j], bd) + dvz<ZF>(-z0.diu + z1.diu, dzn[k], rdzn[k], bd);
    o.f = (-covc + d.vn * dfu1);
  }
  {  // v
    const NouDiu a = face4<P2, ZF>(d, i, j, k, bd), b = face4<P2, ZF>(d, i + 1, j, k, bd);
    const NouDiu y0 = face5<P2, ZF>(d, i, j, k, bd), y1 = face5<P2, ZF>(d, i, j + 1, k, bd);
    const NouDiu z0 = face6<P2, ZF>(d, i, j, k, bd), z1 = face6<P2, ZF>(d, i, j, k + 1, bd);
    o.d4 = a.diu; o.d5 = y0.diu; o.d6 = z0.diu; o.d6t = z1.diu;
    const float covx1 = (a.nou * a.diu + b.nou * b.diu) / 2.f;
    const float covy1 = dvs<P2, ZF>(dy1[j + 1] * (y0.nou * y0.diu) + dy1[j] * (y1.nou * y1.diu), dy1[j] + dy1[j + 1], rdy1s[j], bd);
    const float covz1 = (z0.nou * z0.diu + z1.nou * z1.diu) / 2.f;
    const float covc = covx1 + covy1 + covz1;
    const float dfv1 = dvs<P2, ZF>(-a.diu + b.diu, dx1[i], rdx1[i], bd) +
                       dvs<P2, ZF>(2.f * (-y0.diu + y1.diu), dy1[j] + dy1[j + 1], rdy1s[j], bd) +
                       dvz<ZF>(-z0.diu + z1.diu, dzn[k], rdzn[k], bd);
    o.g = (-covc + d.vn * dfv1);
  }
  if (k <= d.km - 1) {  // w
    const NouDiu a = face7<P2, ZF>(d, i, j, k, bd), b = face7<P2, ZF>(d, i + 1, j, k, bd);
    const NouDiu y0 = face8<P2, ZF>(d, i, j, k, bd), y1 = face8<P2, ZF>(d, i, j + 1, k, bd);
    const NouDiu z0 = face9<ZF>(d, i, j, k, bd), z1 = face9<ZF>(d, i, j, k + 1, bd);
    o.d7 = a.diu; o.d8 = y0.diu; o.d9 = z0.diu;
    const float covx1 = (a.nou * a.diu + b.nou * b.diu) / 2.f;
    const float covy1 = (y0.nou * y0.diu + y1.nou * y1.diu) / 2.f;
    const float covz1 = dvz<ZF>(dzn[k + 1] * (z0.nou * z0.diu) + dzn[k] * (z1.nou * z1.diu), dzn[k] + dzn[k + 1], rdzsum[k], bd);
    const float covc = covx1 + covy1 + covz1;
    const float dfw1 = dvs<P2, ZF>(-a.diu + b.diu, dx1[i], rdx1[i], bd) + dvs<P2, ZF>(-y0.diu + y1.diu, dy1[j], rdy1[j], bd) +
                       dvz<ZF>(-z0.diu + z1.diu, dzs[k], rdzs[k], bd);
    o.h = (-covc + d.vn * dfw1);
  } else {  // k = km: h keeps its value; diu7, diu8 are never written there by the reference (zero)
    o.h = d.h[c];
    o.d7 = 0.f;
    o.d8 = 0.f;
    o.d9 = face9<ZF>(d, i, j, k, bd).diu;
  }
}

// velfg (+ feedbf.f95:35-61 when FB) of the block (bx, by, bz).  With FB the feedback
// force is added to f, g, h for k = 1..km (h(km) keeps velfg's untouched value).
// ZF: reciprocal-corrected divisions, blocks with a dividend outside their range
// deferred to the fixup kernel; !ZF: IEEE divisions.
template <bool P2, bool ZF, bool FB>
__device__ __forceinline__ void velfg_block(const LesDom &d, int bx, int by, int bz) {
  // threads past the domain edge compute the edge cell again (straight-line code) and store nothing
  const int i0 = bx * FX + threadIdx.x + 1, j0 = by * FY + threadIdx.y + 1, k0 = bz * FZ + threadIdx.z + 1;
  const bool in = (i0 <= d.im && j0 <= d.jm && k0 <= d.km);
  const int i = min(i0, d.im), j = min(j0, d.jm), k = min(k0, d.km);
  const int c = lix(d, i, j, k);
  VelfgOut o;
  unsigned bd = 0;
  velfg_cell<P2, ZF>(d, i, j, k, c, o, bd);
  if (ZF && defer_block(bd, d.fix[FIX_VELFG])) return;
  if (!in) return;
  d.diu[1][c] = o.d1;
  d.diu[2][c] = o.d2;
  if (k > 1) d.diu[3][c] = o.d3;  // k = 1: the wall gradient stored by k_wall
  d.diu[4][c] = o.d4;
  d.diu[5][c] = o.d5;
  if (k > 1) d.diu[6][c] = o.d6;
  d.diu[7][c] = o.d7;
  d.diu[8][c] = o.d8;
  d.diu[9][c] = o.d9;
  if (k == d.km) {
    d.diu[3][c + d.np] = o.d3t;
    d.diu[6][c + d.np] = o.d6t;
  }
  float fv = o.f, gv = o.g, hv = o.h;
  if (FB) {  // feedbf.f95:35-61
    const uint8_t m = d.mask[c];
    const float bm = (m & 1) ? 1.f : 0.f, cm = (m & 2) ? 1.f : 0.f, dm = (m & 4) ? 1.f : 0.f;
    const float u = d.u[c], v = d.v[c], w = d.w[c];
    const float us = (d.usum[c] + u) * bm;
    const float vs = (d.vsum[c] + v) * cm;
    const float ws = (d.wsum[c] + w) * dm;
    d.usum[c] = us; d.vsum[c] = vs; d.wsum[c] = ws;
    fv = fv + (d.alpha * us * d.dt + d.beta * u * bm);
    gv = gv + (d.alpha * vs * d.dt + d.beta * v * cm);
    hv = hv + (d.alpha * ws * d.dt + d.beta * w * dm);
  }
  d.f[c] = fv;
  d.g[c] = gv;
  if (FB || k <= d.km - 1) d.h[c] = hv;
}

template <bool P2, bool ZF, bool FB>
__global__ void __launch_bounds__(FX *FY *FZ) k_velfg2(LesDom d) {
  velfg_block<P2, ZF, FB>(d, blockIdx.x, blockIdx.y, blockIdx.z);
}
// the deferred blocks of k_velfg2<P2, true, FB>, with IEEE divisions
template <bool P2, bool FB>
__global__ void __launch_bounds__(FX *FY *FZ) k_velfg2_fix(LesDom d, uint3 g) {
  for_deferred(d.fix[FIX_VELFG], g, [&](int bx, int by, int bz) { velfg_block<P2, false, FB>(d, bx, by, bz); });
}

#define SM_(i, j, k) __ldg(&d.sm[lix(d, (i), (j), (k))])

// Smagorinsky face viscosity x/y interpolations: (dx1(i+1)*a + dx1(i)*b)/(dx1(i)+dx1(i+1))
template <bool P2, bool ZF>
__device__ __forceinline__ float ix_(const LesDom &d, int i, float a, float b, unsigned &bd) {
  return dvs<P2, ZF>(d.gr.dx1[i + 1] * a + d.gr.dx1[i] * b, d.gr.dx1[i] + d.gr.dx1[i + 1], d.gr.rdx1s[i], bd);
}
template <bool P2, bool ZF>  // (dx1(i)*a + dx1(i-1)*b)/(dx1(i-1)+dx1(i))
__device__ __forceinline__ float ixm_(const LesDom &d, int i, float a, float b, unsigned &bd) {
  return dvs<P2, ZF>(d.gr.dx1[i] * a + d.gr.dx1[i - 1] * b, d.gr.dx1[i - 1] + d.gr.dx1[i], d.gr.rdx1s[i - 1], bd);
}
template <bool P2, bool ZF>  // (dy1(j+1)*a + dy1(j)*b)/(dy1(j)+dy1(j+1))
__device__ __forceinline__ float jy_(const LesDom &d, int j, float a, float b, unsigned &bd) {
  return dvs<P2, ZF>(d.gr.dy1[j + 1] * a + d.gr.dy1[j] * b, d.gr.dy1[j] + d.gr.dy1[j + 1], d.gr.rdy1s[j], bd);
}
template <bool P2, bool ZF>  // (dy1(j)*a + dy1(j-1)*b)/(dy1(j-1)+dy1(j))
__device__ __forceinline__ float jym_(const LesDom &d, int j, float a, float b, unsigned &bd) {
  return dvs<P2, ZF>(d.gr.dy1[j] * a + d.gr.dy1[j - 1] * b, d.gr.dy1[j - 1] + d.gr.dy1[j], d.gr.rdy1s[j - 1], bd);
}

// ---- diu as les reads the reference arrays, loaded from what velfg stored: the
// halo copies become index remaps and never-written entries read as zero
__device__ __forceinline__ float e1(const LesDom &d, int i, int j, int k) { return DIU_(1, min(i, d.im), j, k); }
__device__ __forceinline__ float e2(const LesDom &d, int i, int j, int k) {
  return (i <= 0) ? 0.f : DIU_(2, i, (j > d.jm) ? 1 : j, k);
}
__device__ __forceinline__ float e3(const LesDom &d, int i, int j, int k) { return (i <= 0) ? 0.f : DIU_(3, i, j, k); }
__device__ __forceinline__ float e4(const LesDom &d, int i, int j, int k) {
  return DIU_(4, min(i, d.im), (j <= 0) ? d.jm : j, k);
}
__device__ __forceinline__ float e5(const LesDom &d, int i, int j, int k) { return DIU_(5, i, (j > d.jm) ? 1 : j, k); }
__device__ __forceinline__ float e6(const LesDom &d, int i, int j, int k) { return DIU_(6, i, (j <= 0) ? d.jm : j, k); }
__device__ __forceinline__ float e7(const LesDom &d, int i, int j, int k) {
  return (k <= 0 || k >= d.km) ? 0.f : DIU_(7, min(i, d.im), j, k);
}
__device__ __forceinline__ float e8(const LesDom &d, int i, int j, int k) {
  return (k <= 0 || k >= d.km) ? 0.f : DIU_(8, i, (j > d.jm) ? 1 : j, k);
}
__device__ __forceinline__ float e9(const LesDom &d, int i, int j, int k) { return (k > d.km) ? 0.f : DIU_(9, i, j, k); }

// ------------------------------------------------------------------ les.f95:45-65
__global__ void __launch_bounds__(FX *FY *FZ) k_les_sm3(LesDom d) {
  FUSED_IJK
  const float dudxx1 = e1(d, i, j, k);
  const float dudyx1 = (e2(d, i - 1, j, k) + e2(d, i - 1, j + 1, k) + e2(d, i, j, k) + e2(d, i, j + 1, k)) * .25f;
  const float dudzx1 = (e3(d, i - 1, j, k) + e3(d, i - 1, j, k + 1) + e3(d, i, j, k) + e3(d, i, j, k + 1)) * .25f;
  const float dvdxx1 = (e4(d, i, j, k) + e4(d, i, j - 1, k) + e4(d, i + 1, j, k) + e4(d, i + 1, j - 1, k)) * .25f;
  const float dvdyx1 = e5(d, i, j, k);
  const float dvdzx1 = (e6(d, i, j - 1, k) + e6(d, i, j - 1, k + 1) + e6(d, i, j, k) + e6(d, i, j, k + 1)) * .25f;
  const float dwdxx1 = (e7(d, i, j, k) + e7(d, i, j, k - 1) + e7(d, i + 1, j, k) + e7(d, i + 1, j, k - 1)) * .25f;
  const float dwdyx1 = (e8(d, i, j, k) + e8(d, i, j, k - 1) + e8(d, i, j + 1, k) + e8(d, i, j + 1, k - 1)) * .25f;
  const float dwdzx1 = e9(d, i, j, k);
  const float cd = 0.1f * d.gr.delx1[k];
  const float s1 = dudyx1 + dvdxx1, s2 = dwdyx1 + dvdzx1, s3 = dudzx1 + dwdxx1;
  d.sm[lix(d, i, j, k)] =
      cd * cd * __fsqrt_rn(2.f * (dudxx1 * dudxx1 + dvdyx1 * dvdyx1 + dwdzx1 * dwdzx1) + s1 * s1 + s2 * s2 + s3 * s3);
}

// ------------------------------------------------------------------ les.f95:83-242
// The viscous terms of one cell added to f, g, h; gradients from the stored diu, wall
// ratios from k_wall.
template <bool P2, bool ZF>
__device__ __forceinline__ void visc_cell(const LesDom &d, int i, int j, int k, int c, float &fv, float &gv, float &hv,
                                          unsigned &bd) {
  const float *dzn = d.gr.dzn, *rdzn = d.gr.rdzn, *rdzsum = d.gr.rdzsum;
  const float *dx1 = d.gr.dx1, *dy1 = d.gr.dy1, *dxs = d.gr.dxs, *dys = d.gr.dys;
  const float *rdx1 = d.gr.rdx1, *rdy1 = d.gr.rdy1, *rdxs = d.gr.rdxs, *rdys = d.gr.rdys;
  const float s_c = SM_(i, j, k), s_e = SM_(i + 1, j, k), s_w = SM_(i - 1, j, k);
  const float s_n = SM_(i, j + 1, k), s_s = SM_(i, j - 1, k);
  const float s_ne = SM_(i + 1, j + 1, k), s_se = SM_(i + 1, j - 1, k), s_nw = SM_(i - 1, j + 1, k);
  const float s_u = SM_(i, j, k + 1), s_eu = SM_(i + 1, j, k + 1), s_wu = SM_(i - 1, j, k + 1);
  const float s_nu = SM_(i, j + 1, k + 1), s_su = SM_(i, j - 1, k + 1);
  const float s_d = SM_(i, j, k - 1), s_ed = SM_(i + 1, j, k - 1);  // plane k-1 (unused at k = 1)
  // gradients around the cell
  const float g1c = e1(d, i, j, k), g1e = e1(d, i + 1, j, k);
  const float g2c = e2(d, i, j, k), g2n = e2(d, i, j + 1, k), g2wn = e2(d, i - 1, j + 1, k);
  const float g3c = e3(d, i, j, k), g3u = e3(d, i, j, k + 1), g3wu = e3(d, i - 1, j, k + 1);
  const float g4c = e4(d, i, j, k), g4e = e4(d, i + 1, j, k), g4es = e4(d, i + 1, j - 1, k);
  const float g5c = e5(d, i, j, k), g5n = e5(d, i, j + 1, k);
  const float g6c = e6(d, i, j, k), g6u = e6(d, i, j, k + 1), g6su = e6(d, i, j - 1, k + 1);
  const float g7c = e7(d, i, j, k), g7e = e7(d, i + 1, j, k), g7ed = e7(d, i + 1, j, k - 1);
  const float g8c = e8(d, i, j, k), g8n = e8(d, i, j + 1, k), g8nd = e8(d, i, j + 1, k - 1);
  const float g9c = e9(d, i, j, k), g9u = e9(d, i, j, k + 1);
  const float f0 = d.f[c], g0 = d.g[c], h0 = d.h[c];
  const float xc = ix_<P2, ZF>(d, i, s_c, s_e, bd);
  const float xu = ix_<P2, ZF>(d, i, s_u, s_eu, bd);
  // x component
  {
    const float evsx2 = s_e, evsx1 = s_c;
    const float evsy2 = jy_<P2, ZF>(d, j, xc, ix_<P2, ZF>(d, i, s_n, s_ne, bd), bd);
    const float evsy1 = jy_<P2, ZF>(d, j, ix_<P2, ZF>(d, i, s_s, s_se, bd), xc, bd);
    const float visux2 = (evsx2) * 2.f * g1e;
    const float visux1 = (evsx1) * 2.f * g1c;
    const float visuy2 = (evsy2) * (g2n + g4e);
    const float visuy1 = (evsy1) * (g2c + g4es);
    float vfu;
    if (k >= 2) {
      const float evsz2 = dvz<ZF>(dzn[k + 1] * xc + dzn[k] * xu, dzn[k] + dzn[k + 1], rdzsum[k], bd);
      const float evsz1 = dvz<ZF>(dzn[k] * ix_<P2, ZF>(d, i, s_d, s_ed, bd) + dzn[k - 1] * xc, dzn[k - 1] + dzn[k], rdzsum[k - 1], bd);
      const float visuz2 = (evsz2) * (g3u + g7e);
      const float visuz1 = (evsz1) * (g3c + g7ed);
      vfu = dvs<P2, ZF>(visux2 - visux1, dxs[i], rdxs[i], bd) + dvs<P2, ZF>(visuy2 - visuy1, dy1[j], rdy1[j], bd) +
            dvz<ZF>(visuz2 - visuz1, dzn[k], rdzn[k], bd);
    } else {  // les.f95:118-139: the y and z terms appear twice, as written
      const float evsz2 = dvz<ZF>(dzn[2] * xc + dzn[1] * xu, dzn[1] + dzn[2], rdzsum[1], bd);
      const float visuz2 = (evsz2) * (g3u + g7e);
      const float r = __ldg(&d.ruspd[(j + LES_JOFF) * d.pi + i + LES_IOFF]);
      const float t = dvz<ZF>(0.4f * r, d.logz, d.rlogz, bd);
      const float visuz1 = t * t * r;
      const float ty = dvs<P2, ZF>(visuy2 - visuy1, dy1[j], rdy1[j], bd);
      const float tz = dvz<ZF>(visuz2 - visuz1, dzn[1], rdzn[1], bd);
      vfu = dvs<P2, ZF>(visux2 - visux1, dxs[i], rdxs[i], bd) + ty + tz + ty + tz;
    }
    fv = f0 + vfu;
  }
  // y component
  {
    const float evsy2 = s_n, evsy1 = s_c;
    const float evsx2 = jy_<P2, ZF>(d, j, xc, ix_<P2, ZF>(d, i, s_n, s_ne, bd), bd);
    const float evsx1 = jy_<P2, ZF>(d, j, ixm_<P2, ZF>(d, i, s_w, s_c, bd), ixm_<P2, ZF>(d, i, s_nw, s_n, bd), bd);
    const float visvx2 = (evsx2) * (g2n + g4e);
    const float visvx1 = (evsx1) * (g2wn + g4c);
    const float visvy2 = (evsy2) * 2.f * g5n;
    const float visvy1 = (evsy1) * 2.f * g5c;
    float vfv;
    if (k >= 2) {
      const float evsz2 = dvz<ZF>(dzn[k + 1] * xc + dzn[k] * xu, dzn[k] + dzn[k + 1], rdzsum[k], bd);
      const float evsz1 = dvz<ZF>(dzn[k] * ix_<P2, ZF>(d, i, s_d, s_ed, bd) + dzn[k - 1] * xc, dzn[k - 1] + dzn[k], rdzsum[k - 1], bd);
      const float visvz2 = (evsz2) * (g6u + g8n);
      const float visvz1 = (evsz1) * (g6c + g8nd);
      vfv = dvs<P2, ZF>(visvx2 - visvx1, dx1[i], rdx1[i], bd) + dvs<P2, ZF>(visvy2 - visvy1, dys[j], rdys[j], bd) +
            dvz<ZF>(visvz2 - visvz1, dzn[k], rdzn[k], bd);
    } else {  // les.f95:178-201
      const float evsz2 = dvz<ZF>(dzn[2] * xc + dzn[1] * xu, dzn[1] + dzn[2], rdzsum[1], bd);
      const float visvz2 = (evsz2) * (g6u + g8n);
      const float r = __ldg(&d.rvspd[(j + LES_JOFF) * d.pi + i + LES_IOFF]);
      const float t = dvz<ZF>(0.4f * r, d.logz, d.rlogz, bd);
      const float visvz1 = t * t * r;
      vfv = dvs<P2, ZF>(visvx2 - visvx1, dx1[i], rdx1[i], bd) + dvs<P2, ZF>(visvy2 - visvy1, dys[j], rdys[j], bd) +
            dvz<ZF>(visvz2 - visvz1, dzn[1], rdzn[1], bd);
    }
    gv = g0 + vfv;
  }
  // z component, k = 1..km
  {
    const float dzc = dzn[k] + dzn[k + 1], rdzc = rdzsum[k];
    const float evsz2 = s_u, evsz1 = s_c;
    const float evsx2 = dvz<ZF>(dzn[k + 1] * xc + dzn[k] * xu, dzc, rdzc, bd);
    const float evsx1 = dvz<ZF>(dzn[k + 1] * ixm_<P2, ZF>(d, i, s_w, s_c, bd) + dzn[k] * ixm_<P2, ZF>(d, i, s_wu, s_u, bd), dzc, rdzc, bd);
    const float evsy2 = dvz<ZF>(dzn[k + 1] * jy_<P2, ZF>(d, j, s_c, s_n, bd) + dzn[k] * jy_<P2, ZF>(d, j, s_u, s_nu, bd), dzc, rdzc, bd);
    const float evsy1 = dvz<ZF>(dzn[k + 1] * jym_<P2, ZF>(d, j, s_s, s_c, bd) + dzn[k] * jym_<P2, ZF>(d, j, s_su, s_u, bd), dzc, rdzc, bd);
    const float viswx2 = (evsx2) * (g3u + g7e);
    const float viswx1 = (evsx1) * (g3wu + g7c);
    const float viswy2 = (evsy2) * (g6u + g8n);
    const float viswy1 = (evsy1) * (g6su + g8c);
    const float viswz2 = (evsz2) * 2.f * g9u;
    const float viswz1 = (evsz1) * 2.f * g9c;
    const float vfw = dvs<P2, ZF>(viswx2 - viswx1, dx1[i], rdx1[i], bd) + dvs<P2, ZF>(viswy2 - viswy1, dy1[j], rdy1[j], bd) +
                      dvz<ZF>(viswz2 - viswz1, dzn[k], rdzn[k], bd);
    hv = h0 + vfw;
  }
}

// les viscous terms (+ adam.f95:30-44 when AD) of the block (bx, by, bz); ZF as in
// velfg_block.
template <bool P2, bool ZF, bool AD>
__device__ __forceinline__ void visc_block(const LesDom &d, int bx, int by, int bz) {
  const int i0 = bx * FX + threadIdx.x + 1, j0 = by * FY + threadIdx.y + 1, k0 = bz * FZ + threadIdx.z + 1;
  const bool in = (i0 <= d.im && j0 <= d.jm && k0 <= d.km);
  const int i = min(i0, d.im), j = min(j0, d.jm), k = min(k0, d.km);
  const int c = lix(d, i, j, k);
  float fv, gv, hv;
  unsigned bd = 0;
  visc_cell<P2, ZF>(d, i, j, k, c, fv, gv, hv, bd);
  if (ZF && defer_block(bd, d.fix[FIX_VISC])) return;
  if (!in) return;
  if (AD) {  // adam.f95:30-44
    const float fo = d.fold[c], go = d.gold[c], ho = d.hold[c];
    d.fold[c] = fv; d.gold[c] = gv; d.hold[c] = hv;
    fv = 1.5f * fv - 0.5f * fo;
    gv = 1.5f * gv - 0.5f * go;
    hv = 1.5f * hv - 0.5f * ho;
  }
  d.f[c] = fv;
  d.g[c] = gv;
  d.h[c] = hv;
}
template <bool P2, bool ZF, bool AD>
__global__ void __launch_bounds__(FX *FY *FZ) k_les_visc3(LesDom d) {
  visc_block<P2, ZF, AD>(d, blockIdx.x, blockIdx.y, blockIdx.z);
}
template <bool P2, bool AD>
__global__ void __launch_bounds__(FX *FY *FZ) k_les_visc3_fix(LesDom d, uint3 g) {
  for_deferred(d.fix[FIX_VISC], g, [&](int bx, int by, int bz) { visc_block<P2, false, AD>(d, bx, by, bz); });
}

inline dim3 fgrid(const LesDom &d) { return dim3((d.im + FX - 1) / FX, (d.jm + FY - 1) / FY, (d.km + FZ - 1) / FZ); }

}  // namespace

#define LAUNCH(ctx, ...)                \
  do {                                  \
    __VA_ARGS__;                        \
    ++*(ctx).nlaunch;                   \
  } while (0)

namespace {
// Launch a fused kernel K<P2, ZF, X> for the domain's spacing modes; with ZF its fixup
// kernel F<P2, X> follows (it does nothing when no block was deferred).
template <template <bool, bool, bool> class K, template <bool, bool> class F>
void launch_variant(const LesDom &d, bool x, LesCtx ctx) {
  const dim3 g = fgrid(d), b(FX, FY, FZ);
  const uint3 gu = make_uint3(g.x, g.y, g.z);
  const unsigned nfix = std::min<unsigned>(g.x * g.y * g.z, (unsigned)std::max(1, 2 * d.sms));
  const int v = (d.xy_pow2 ? 4 : 0) | (d.zfast ? 2 : 0) | (x ? 1 : 0);
  switch (v) {
    case 0: LAUNCH(ctx, (K<false, false, false>::fn<<<g, b, 0, ctx.s>>>(d))); break;
    case 1: LAUNCH(ctx, (K<false, false, true>::fn<<<g, b, 0, ctx.s>>>(d))); break;
    case 2: LAUNCH(ctx, (K<false, true, false>::fn<<<g, b, 0, ctx.s>>>(d)));
            LAUNCH(ctx, (F<false, false>::fn<<<nfix, b, 0, ctx.s>>>(d, gu))); break;
    case 3: LAUNCH(ctx, (K<false, true, true>::fn<<<g, b, 0, ctx.s>>>(d)));
            LAUNCH(ctx, (F<false, true>::fn<<<nfix, b, 0, ctx.s>>>(d, gu))); break;
    case 4: LAUNCH(ctx, (K<true, false, false>::fn<<<g, b, 0, ctx.s>>>(d))); break;
    case 5: LAUNCH(ctx, (K<true, false, true>::fn<<<g, b, 0, ctx.s>>>(d))); break;
    case 6: LAUNCH(ctx, (K<true, true, false>::fn<<<g, b, 0, ctx.s>>>(d)));
            LAUNCH(ctx, (F<true, false>::fn<<<nfix, b, 0, ctx.s>>>(d, gu))); break;
    default: LAUNCH(ctx, (K<true, true, true>::fn<<<g, b, 0, ctx.s>>>(d)));
             LAUNCH(ctx, (F<true, true>::fn<<<nfix, b, 0, ctx.s>>>(d, gu))); break;
  }
}
template <bool A, bool B, bool C>
struct VelfgK {
  static constexpr auto fn = k_velfg2<A, B, C>;
};
template <bool A, bool C>
struct VelfgF {
  static constexpr auto fn = k_velfg2_fix<A, C>;
};
template <bool A, bool B, bool C>
struct ViscK {
  static constexpr auto fn = k_les_visc3<A, B, C>;
};
template <bool A, bool C>
struct ViscF {
  static constexpr auto fn = k_les_visc3_fix<A, C>;
};
}  // namespace

void les_launch_velfg_fused(const LesDom &d, bool with_feedbf, LesCtx ctx) {
  LAUNCH(ctx, (k_wall<<<dim3((d.im + 127) / 128, d.jm), 128, 0, ctx.s>>>(d)));
  launch_variant<VelfgK, VelfgF>(d, with_feedbf, ctx);
}

void les_launch_les_fused(const LesDom &d, bool with_adam, LesCtx ctx) {
  const dim3 g = fgrid(d), b(FX, FY, FZ);
  LAUNCH(ctx, k_les_sm3<<<g, b, 0, ctx.s>>>(d));
  les_launch_boundsm(d, ctx);
  launch_variant<ViscK, ViscF>(d, with_adam, ctx);
}
