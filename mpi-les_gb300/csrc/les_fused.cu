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
#include <cstdint>
#include <cstdlib>
#include <map>
#include <mutex>
#include <vector>

#include "les_common.cuh"
#include "les_kernels.cuh"
#include "les_sor.cuh"
#include "les_tma.cuh"

namespace {

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
// index remaps.  Each face is split into its loads (fload<N>: the velocities it reads)
// and its arithmetic (fcomp<N>), so a kernel can issue the loads of one plane while it
// computes another; faceN = fcomp<N>(fload<N>).  P2 / ZF select the division forms
// (dvs, dvz); bd collects dividends outside the reciprocal-corrected range.
struct FRaw {
  float a = 0.f, b = 0.f, c = 0.f, e = 0.f;
};

template <int N>
__device__ __forceinline__ FRaw fload(const LesDom &d, int i, int j, int k) {
  FRaw r;
  const int ii = min(i, d.im), jj = (j > d.jm) ? 1 : j;
  if (N == 1) { r.a = UR_(ii - 1, j, k); r.b = UR_(ii, j, k); }
  if (N == 2) { r.a = VR_(i, jj - 1, k); r.b = VR_(i + 1, jj - 1, k); r.c = UR_(i, jj - 1, k); r.e = UR_(i, jj, k); }
  if (N == 3) {
    if (k == 1) { r.a = WR_(i, j, 1); r.b = WR_(i + 1, j, 1); r.c = DIU_(3, i, j, 1); }
    else { r.a = WR_(i, j, k - 1); r.b = WR_(i + 1, j, k - 1); r.c = UR_(i, j, k - 1); r.e = UR_(i, j, k); }
  }
  if (N == 4) { r.a = UR_(ii - 1, j, k); r.b = UR_(ii - 1, j + 1, k); r.c = VR_(ii - 1, j, k); r.e = VR_(ii, j, k); }
  if (N == 5) { r.a = VR_(i, jj - 1, k); r.b = VR_(i, jj, k); }
  if (N == 6) {
    if (k == 1) { r.a = WR_(i, j, 1); r.b = WR_(i, j + 1, 1); r.c = DIU_(6, i, j, 1); }
    else { r.a = WR_(i, j, k - 1); r.b = WR_(i, j + 1, k - 1); r.c = VR_(i, j, k - 1); r.e = VR_(i, j, k); }
  }
  if (N == 7) { r.a = UR_(ii - 1, j, k); r.b = UR_(ii - 1, j, k + 1); r.c = WR_(ii - 1, j, k); r.e = WR_(ii, j, k); }
  if (N == 8) { r.a = VR_(i, jj - 1, k); r.b = VR_(i, jj - 1, k + 1); r.c = WR_(i, jj - 1, k); r.e = WR_(i, jj, k); }
  if (N == 9) { r.a = WR_(i, j, k - 1); r.b = WR_(i, j, k); }
  return r;
}

// diu3 and diu6 at k = 1 are the log-law wall gradients, stored by k_wall before velfg runs
template <int N, bool P2, bool ZF>
__device__ __forceinline__ NouDiu fcomp(const LesDom &d, const FRaw &r, int i, int j, int k, unsigned &bd) {
  const float *dzn = d.gr.dzn;
  const int ii = min(i, d.im), jj = (j > d.jm) ? 1 : j;
  if (N == 1) return {(r.a + r.b) / 2.f, dvs<P2, ZF>(-r.a + r.b, sx1<P2>(d, ii), rx1<P2>(d, ii), bd)};
  if (N == 2)
    return {dvs<P2, ZF>(sx1<P2>(d, i + 1) * r.a + sx1<P2>(d, i) * r.b, sx1<P2>(d, i) + sx1<P2>(d, i + 1),
                        rx1s<P2>(d, i), bd),
            dvs<P2, ZF>(2.f * (-r.c + r.e), sy1<P2>(d, jj - 1) + sy1<P2>(d, jj), ry1s<P2>(d, jj - 1), bd)};
  if (N == 3) {
    if (k == 1)
      return {dvs<P2, ZF>(0.5f * (sx1<P2>(d, i + 1) * r.a + sx1<P2>(d, i) * r.b), sx1<P2>(d, i) + sx1<P2>(d, i + 1),
                          rx1s<P2>(d, i), bd),
              r.c};
    return {dvs<P2, ZF>(sx1<P2>(d, i + 1) * r.a + sx1<P2>(d, i) * r.b, sx1<P2>(d, i) + sx1<P2>(d, i + 1),
                        rx1s<P2>(d, i), bd),
            dvz<ZF>(-r.c + r.e, d.gr.dzs[k - 1], d.gr.rdzs[k - 1], bd)};
  }
  if (N == 4)
    return {dvs<P2, ZF>(sy1<P2>(d, j + 1) * r.a + sy1<P2>(d, j) * r.b, sy1<P2>(d, j) + sy1<P2>(d, j + 1),
                        ry1s<P2>(d, j), bd) - 0.f,
            dvs<P2, ZF>(2.f * (-r.c + r.e), sx1<P2>(d, ii - 1) + sx1<P2>(d, ii), rx1s<P2>(d, ii - 1), bd)};
  if (N == 5) return {(r.a + r.b) / 2.f, dvs<P2, ZF>(-r.a + r.b, sy1<P2>(d, jj), ry1<P2>(d, jj), bd)};
  if (N == 6) {
    if (k == 1)
      return {dvs<P2, ZF>(0.5f * (sy1<P2>(d, j + 1) * r.a + sy1<P2>(d, j) * r.b), sy1<P2>(d, j) + sy1<P2>(d, j + 1),
                          ry1s<P2>(d, j), bd),
              r.c};
    return {dvs<P2, ZF>(sy1<P2>(d, j + 1) * r.a + sy1<P2>(d, j) * r.b, sy1<P2>(d, j) + sy1<P2>(d, j + 1),
                        ry1s<P2>(d, j), bd),
            dvz<ZF>(-r.c + r.e, d.gr.dzs[k - 1], d.gr.rdzs[k - 1], bd)};
  }
  if (N == 7)
    return {dvz<ZF>(dzn[k + 1] * r.a + dzn[k] * r.b, dzn[k] + dzn[k + 1], d.gr.rdzsum[k], bd) - 0.f,
            dvs<P2, ZF>(2.f * (-r.c + r.e), sx1<P2>(d, ii - 1) + sx1<P2>(d, ii), rx1s<P2>(d, ii - 1), bd)};
  if (N == 8)
    return {dvz<ZF>(dzn[k + 1] * r.a + dzn[k] * r.b, dzn[k] + dzn[k + 1], d.gr.rdzsum[k], bd),
            dvs<P2, ZF>(2.f * (-r.c + r.e), sy1<P2>(d, jj - 1) + sy1<P2>(d, jj), ry1s<P2>(d, jj - 1), bd)};
  return {(r.a + r.b) / 2.f, dvz<ZF>(-r.a + r.b, dzn[k], d.gr.rdzn[k], bd)};  // N == 9
}

template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face1(const LesDom &d, int i, int j, int k, unsigned &bd) {
  return fcomp<1, P2, ZF>(d, fload<1>(d, i, j, k), i, j, k, bd);
}
template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face2(const LesDom &d, int i, int j, int k, unsigned &bd) {
  return fcomp<2, P2, ZF>(d, fload<2>(d, i, j, k), i, j, k, bd);
}
template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face3(const LesDom &d, int i, int j, int k, unsigned &bd) {
  return fcomp<3, P2, ZF>(d, fload<3>(d, i, j, k), i, j, k, bd);
}
template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face4(const LesDom &d, int i, int j, int k, unsigned &bd) {
  return fcomp<4, P2, ZF>(d, fload<4>(d, i, j, k), i, j, k, bd);
}
template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face5(const LesDom &d, int i, int j, int k, unsigned &bd) {
  return fcomp<5, P2, ZF>(d, fload<5>(d, i, j, k), i, j, k, bd);
}
template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face6(const LesDom &d, int i, int j, int k, unsigned &bd) {
  return fcomp<6, P2, ZF>(d, fload<6>(d, i, j, k), i, j, k, bd);
}
template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face7(const LesDom &d, int i, int j, int k, unsigned &bd) {
  return fcomp<7, P2, ZF>(d, fload<7>(d, i, j, k), i, j, k, bd);
}
template <bool P2, bool ZF>
__device__ __forceinline__ NouDiu face8(const LesDom &d, int i, int j, int k, unsigned &bd) {
  return fcomp<8, P2, ZF>(d, fload<8>(d, i, j, k), i, j, k, bd);
}
template <bool ZF>
__device__ __forceinline__ NouDiu face9(const LesDom &d, int i, int j, int k, unsigned &bd) {
  return fcomp<9, false, ZF>(d, fload<9>(d, i, j, k), i, j, k, bd);
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
// The momentum terms of one cell from its six face pairs per component: a, b at i and
// i+1, y0, y1 at j and j+1, z0, z1 at k and k+1 (velFG.f95:64-110).
template <bool P2, bool ZF>
__device__ __forceinline__ float velfg_fu(const LesDom &d, int i, int j, int k, const NouDiu &a, const NouDiu &b,
                                          const NouDiu &y0, const NouDiu &y1, const NouDiu &z0, const NouDiu &z1,
                                          unsigned &bd) {
  const float covx1 =
      dvs<P2, ZF>(sx1<P2>(d, i + 1) * (a.nou * a.diu) + sx1<P2>(d, i) * (b.nou * b.diu),
                  sx1<P2>(d, i) + sx1<P2>(d, i + 1), rx1s<P2>(d, i), bd);
  const float covy1 = (y0.nou * y0.diu + y1.nou * y1.diu) / 2.f;
  const float covz1 = (z0.nou * z0.diu + z1.nou * z1.diu) / 2.f;
  const float covc = covx1 + covy1 + covz1;
  const float dfu1 = dvs<P2, ZF>(2.f * (-a.diu + b.diu), sx1<P2>(d, i) + sx1<P2>(d, i + 1), rx1s<P2>(d, i), bd) +
                     dvs<P2, ZF>(-y0.diu + y1.diu, sy1<P2>(d, j), ry1<P2>(d, j), bd) +
                     dvz<ZF>(-z0.diu + z1.diu, d.gr.dzn[k], d.gr.rdzn[k], bd);
  return (-covc + d.vn * dfu1);
}
template <bool P2, bool ZF>
__device__ __forceinline__ float velfg_fv(const LesDom &d, int i, int j, int k, const NouDiu &a, const NouDiu &b,
                                          const NouDiu &y0, const NouDiu &y1, const NouDiu &z0, const NouDiu &z1,
                                          unsigned &bd) {
  const float covx1 = (a.nou * a.diu + b.nou * b.diu) / 2.f;
  const float covy1 =
      dvs<P2, ZF>(sy1<P2>(d, j + 1) * (y0.nou * y0.diu) + sy1<P2>(d, j) * (y1.nou * y1.diu),
                  sy1<P2>(d, j) + sy1<P2>(d, j + 1), ry1s<P2>(d, j), bd);
  const float covz1 = (z0.nou * z0.diu + z1.nou * z1.diu) / 2.f;
  const float covc = covx1 + covy1 + covz1;
  const float dfv1 = dvs<P2, ZF>(-a.diu + b.diu, sx1<P2>(d, i), rx1<P2>(d, i), bd) +
                     dvs<P2, ZF>(2.f * (-y0.diu + y1.diu), sy1<P2>(d, j) + sy1<P2>(d, j + 1), ry1s<P2>(d, j), bd) +
                     dvz<ZF>(-z0.diu + z1.diu, d.gr.dzn[k], d.gr.rdzn[k], bd);
  return (-covc + d.vn * dfv1);
}
template <bool P2, bool ZF>
__device__ __forceinline__ float velfg_fw(const LesDom &d, int i, int j, int k, const NouDiu &a, const NouDiu &b,
                                          const NouDiu &y0, const NouDiu &y1, const NouDiu &z0, const NouDiu &z1,
                                          unsigned &bd) {
  const float *dzn = d.gr.dzn;
  const float covx1 = (a.nou * a.diu + b.nou * b.diu) / 2.f;
  const float covy1 = (y0.nou * y0.diu + y1.nou * y1.diu) / 2.f;
  const float covz1 =
      dvz<ZF>(dzn[k + 1] * (z0.nou * z0.diu) + dzn[k] * (z1.nou * z1.diu), dzn[k] + dzn[k + 1], d.gr.rdzsum[k], bd);
  const float covc = covx1 + covy1 + covz1;
  const float dfw1 = dvs<P2, ZF>(-a.diu + b.diu, sx1<P2>(d, i), rx1<P2>(d, i), bd) +
                     dvs<P2, ZF>(-y0.diu + y1.diu, sy1<P2>(d, j), ry1<P2>(d, j), bd) +
                     dvz<ZF>(-z0.diu + z1.diu, d.gr.dzs[k], d.gr.rdzs[k], bd);
  return (-covc + d.vn * dfw1);
}

template <bool P2, bool ZF>
__device__ __forceinline__ void velfg_cell(const LesDom &d, int i, int j, int k, int c, VelfgOut &o, unsigned &bd) {
  {  // u
    const NouDiu a = face1<P2, ZF>(d, i, j, k, bd), b = face1<P2, ZF>(d, i + 1, j, k, bd);
    const NouDiu y0 = face2<P2, ZF>(d, i, j, k, bd), y1 = face2<P2, ZF>(d, i, j + 1, k, bd);
    const NouDiu z0 = face3<P2, ZF>(d, i, j, k, bd), z1 = face3<P2, ZF>(d, i, j, k + 1, bd);
    o.d1 = a.diu; o.d2 = y0.diu; o.d3 = z0.diu; o.d3t = z1.diu;
    o.f = velfg_fu<P2, ZF>(d, i, j, k, a, b, y0, y1, z0, z1, bd);
  }
  {  // v
    const NouDiu a = face4<P2, ZF>(d, i, j, k, bd), b = face4<P2, ZF>(d, i + 1, j, k, bd);
    const NouDiu y0 = face5<P2, ZF>(d, i, j, k, bd), y1 = face5<P2, ZF>(d, i, j + 1, k, bd);
    const NouDiu z0 = face6<P2, ZF>(d, i, j, k, bd), z1 = face6<P2, ZF>(d, i, j, k + 1, bd);
    o.d4 = a.diu; o.d5 = y0.diu; o.d6 = z0.diu; o.d6t = z1.diu;
    o.g = velfg_fv<P2, ZF>(d, i, j, k, a, b, y0, y1, z0, z1, bd);
  }
  if (k <= d.km - 1) {  // w
    const NouDiu a = face7<P2, ZF>(d, i, j, k, bd), b = face7<P2, ZF>(d, i + 1, j, k, bd);
    const NouDiu y0 = face8<P2, ZF>(d, i, j, k, bd), y1 = face8<P2, ZF>(d, i, j + 1, k, bd);
    const NouDiu z0 = face9<ZF>(d, i, j, k, bd), z1 = face9<ZF>(d, i, j, k + 1, bd);
    o.d7 = a.diu; o.d8 = y0.diu; o.d9 = z0.diu;
    o.h = velfg_fw<P2, ZF>(d, i, j, k, a, b, y0, y1, z0, z1, bd);
  } else {  // k = km: h keeps its value; diu7, diu8 are never written there by the reference (zero)
    o.h = d.h[c];
    o.d7 = 0.f;
    o.d8 = 0.f;
    o.d9 = face9<ZF>(d, i, j, k, bd).diu;
  }
}

// Operands of feedbf (feedbf.f95:35-61) for one cell, loaded ahead of use.
struct FbIn {
  uint8_t m = 0;
  float u = 0.f, v = 0.f, w = 0.f, su = 0.f, sv = 0.f, sw = 0.f;
};
__device__ __forceinline__ FbIn fb_load(const LesDom &d, int c) {
  FbIn x;
  x.m = d.mask[c];
  x.u = d.u[c]; x.v = d.v[c]; x.w = d.w[c];
  x.su = d.usum[c]; x.sv = d.vsum[c]; x.sw = d.wsum[c];
  return x;
}

// Stores of one cell: the diu it formed, then f, g, h (+ feedbf when FB: the feedback
// force added to f, g, h for k = 1..km; h(km) keeps velfg's untouched value).
template <bool FB>
__device__ __forceinline__ void velfg_store(const LesDom &d, int c, int k, const VelfgOut &o, const FbIn &x) {
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
    const float bm = (x.m & 1) ? 1.f : 0.f, cm = (x.m & 2) ? 1.f : 0.f, dm = (x.m & 4) ? 1.f : 0.f;
    const float us = (x.su + x.u) * bm;
    const float vs = (x.sv + x.v) * cm;
    const float ws = (x.sw + x.w) * dm;
    d.usum[c] = us; d.vsum[c] = vs; d.wsum[c] = ws;
    fv = fv + (d.alpha * us * d.dt + d.beta * x.u * bm);
    gv = gv + (d.alpha * vs * d.dt + d.beta * x.v * cm);
    hv = hv + (d.alpha * ws * d.dt + d.beta * x.w * dm);
  }
  d.f[c] = fv;
  d.g[c] = gv;
  if (FB || k <= d.km - 1) d.h[c] = hv;
}

// ---- the velfg k-march -------------------------------------------------------------
// A block owns MTI x MTY columns (31 cells of i per 32 lanes, 8 rows of j) and marches
// k over a chunk of planes.  Each face pair is formed once per face, not once per cell
// that reads it: the i faces (face1, 4, 7) by the lane of the cell on their east side
// and passed west by warp shuffle (the 32nd lane of a row forms the face east of the
// tile), the j faces (face2, 5, 8) by the row south of them and passed north through
// shared memory (row 0 forms the face south of the tile), the k faces (face3, 6, 9)
// once per plane, kept in registers for the plane above.  Step k forms the faces of
// plane k+1 and combines those of plane k; one barrier per step orders the j faces and decides whether the plane is stored (a
// dividend outside dvz's range anywhere in the tile plane hands the plane to the fixup
// kernel, which recomputes it with IEEE divisions).  The rows of u, v, w a thread reads
// are requested into L1 (prefetch.global.L1) three planes before their faces are formed.
constexpr int MTX = 32, MTI = 31, MTY = 8;

struct MFaces {  // faces of one column position: u, v, w components
  NouDiu u, v, w;
};

// The loads of the faces a thread forms for one plane.
struct MRaw {
  FRaw x1, x4, x7;  // i faces at (ia, j)
  FRaw y2, y5, y8;  // j faces at (i, j+1)
  FRaw s2, s5, s8;  // row 0: j faces at (i, j0)
  FRaw z3, z6, z9;  // k faces at the plane above
};

template <bool P2, bool ZF, bool FB>
__global__ void __launch_bounds__(MTX *MTY, 3) k_velfg_march(LesDom d, int kchunk) {
  // j-face pairs of rows j0 .. j0+MTY for two planes (plane parity): [.][row][lane]
  __shared__ MFaces ys[2][MTY + 1][MTX];
  const int lane = threadIdx.x, ty = threadIdx.y;
  const int i0 = blockIdx.x * MTI + 1, j0 = blockIdx.y * MTY + 1;
  const int k0 = blockIdx.z * kchunk + 1, k1 = min(k0 + kchunk - 1, d.km);
  const int iraw = i0 + lane, jraw = j0 + ty;
  const bool in = lane < MTI && iraw <= d.im && jraw <= d.jm;
  // the cell's column (clamped into the domain: lanes and rows past it recompute the
  // edge and store nothing) and the column of the i face this lane forms (i = im+1 is
  // the face east of cell im)
  const int i = min(iraw, d.im), j = min(jraw, d.jm), ia = min(iraw, d.im + 1);
  const int km = d.km;

  // loads of plane kk's i and j faces and of the k faces at kz (kz = kk + 1)
  auto load = [&](int kk, int kz) {
    MRaw r;
    r.x1 = fload<1>(d, ia, j, kk);
    r.x4 = fload<4>(d, ia, j, kk);
    r.y2 = fload<2>(d, i, j + 1, kk);
    r.y5 = fload<5>(d, i, j + 1, kk);
    if (kk <= km - 1) {
      r.x7 = fload<7>(d, ia, j, kk);
      r.y8 = fload<8>(d, i, j + 1, kk);
    }
    if (ty == 0) {
      r.s2 = fload<2>(d, i, j, kk);
      r.s5 = fload<5>(d, i, j, kk);
      if (kk <= km - 1) r.s8 = fload<8>(d, i, j, kk);
    }
    r.z3 = fload<3>(d, i, j, kz);
    r.z6 = fload<6>(d, i, j, kz);
    if (kz <= km) r.z9 = fload<9>(d, i, j, kz);
    return r;
  };
  // faces of plane kk from its loads: i faces returned, j faces into shared memory, k faces at kz
  auto form = [&](const MRaw &r, int kk, int kz, MFaces &X, MFaces &Z, unsigned &fxy, unsigned &fz) {
    X.u = fcomp<1, P2, ZF>(d, r.x1, ia, j, kk, fxy);
    X.v = fcomp<4, P2, ZF>(d, r.x4, ia, j, kk, fxy);
    X.w = (kk <= km - 1) ? fcomp<7, P2, ZF>(d, r.x7, ia, j, kk, fxy) : NouDiu{0.f, 0.f};
    MFaces Y;
    Y.u = fcomp<2, P2, ZF>(d, r.y2, i, j + 1, kk, fxy);
    Y.v = fcomp<5, P2, ZF>(d, r.y5, i, j + 1, kk, fxy);
    Y.w = (kk <= km - 1) ? fcomp<8, P2, ZF>(d, r.y8, i, j + 1, kk, fxy) : NouDiu{0.f, 0.f};
    ys[kk & 1][ty + 1][lane] = Y;
    if (ty == 0) {
      MFaces S;
      S.u = fcomp<2, P2, ZF>(d, r.s2, i, j, kk, fxy);
      S.v = fcomp<5, P2, ZF>(d, r.s5, i, j, kk, fxy);
      S.w = (kk <= km - 1) ? fcomp<8, P2, ZF>(d, r.s8, i, j, kk, fxy) : NouDiu{0.f, 0.f};
      ys[kk & 1][0][lane] = S;
    }
    Z.u = fcomp<3, P2, ZF>(d, r.z3, i, j, kz, fz);
    Z.v = fcomp<6, P2, ZF>(d, r.z6, i, j, kz, fz);
    Z.w = (kz <= km) ? fcomp<9, false, ZF>(d, r.z9, i, j, kz, fz) : NouDiu{0.f, 0.f};
  };

  // prologue: the faces of plane k0 and the k faces at k0, k0+1
  unsigned fz0 = 0, fz1 = 0, fxy = 0;
  MFaces X, Z0, Z1;
  {
    const MRaw r = load(k0, k0 + 1);
    form(r, k0, k0 + 1, X, Z1, fxy, fz1);
    Z0.u = fcomp<3, P2, ZF>(d, fload<3>(d, i, j, k0), i, j, k0, fz0);
    Z0.v = fcomp<6, P2, ZF>(d, fload<6>(d, i, j, k0), i, j, k0, fz0);
    Z0.w = fcomp<9, false, ZF>(d, fload<9>(d, i, j, k0), i, j, k0, fz0);
  }
  int c = lix(d, i, j, k0);
  FbIn fb;
  if (FB) fb = fb_load(d, c);
  float hkm = (k0 == km) ? d.h[c] : 0.f;
  __syncthreads();

  // the rows of u, v, w in plane kk that this thread's faces read, requested into L1
  // ahead of time (row 0 also reads the row south of the tile, the top row the row north)
  auto prefetch_plane = [&](int kk) {
    const int cp = lix(d, i, j, kk);
    const float *q[3] = {d.u + cp, d.v + cp, d.w + cp};
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      asm volatile("prefetch.global.L1 [%0];" ::"l"(q[f]));
      if (ty == 0 && f == 1) asm volatile("prefetch.global.L1 [%0];" ::"l"(q[f] - d.pi));
      if (ty == MTY - 1) asm volatile("prefetch.global.L1 [%0];" ::"l"(q[f] + d.pi));
    }
  };

  for (int k = k0; k <= k1; ++k) {
    const bool more = k < k1;
    if (k + 3 <= km + 1) prefetch_plane(k + 3);
    // ---- the faces of plane k+1 (j faces into the other half of shared memory) and its
    // k faces at k+2; the feedbf operands of plane k+1, used after the next combine
    MFaces Xn = X, Z2 = Z1;
    unsigned fxyn = 0, fz2 = 0;
    FbIn fbn;
    float hkmn = 0.f;
    if (more) {
      form(load(k + 1, k + 2), k + 1, k + 2, Xn, Z2, fxyn, fz2);
      if (FB) fbn = fb_load(d, c + d.np);
      if (k + 1 == km) hkmn = d.h[c + d.np];
    }
    // ---- combine plane k: i faces from the lane to the east, j faces from shared memory
    unsigned bd = fxy | fz0 | fz1;
    MFaces B;
    B.u.nou = __shfl_down_sync(0xffffffffu, X.u.nou, 1);
    B.u.diu = __shfl_down_sync(0xffffffffu, X.u.diu, 1);
    B.v.nou = __shfl_down_sync(0xffffffffu, X.v.nou, 1);
    B.v.diu = __shfl_down_sync(0xffffffffu, X.v.diu, 1);
    B.w.nou = __shfl_down_sync(0xffffffffu, X.w.nou, 1);
    B.w.diu = __shfl_down_sync(0xffffffffu, X.w.diu, 1);
    const MFaces Y0 = ys[k & 1][ty][lane], Y1 = ys[k & 1][ty + 1][lane];
    VelfgOut o;
    o.d1 = X.u.diu; o.d2 = Y0.u.diu; o.d3 = Z0.u.diu; o.d3t = Z1.u.diu;
    o.f = velfg_fu<P2, ZF>(d, i, j, k, X.u, B.u, Y0.u, Y1.u, Z0.u, Z1.u, bd);
    o.d4 = X.v.diu; o.d5 = Y0.v.diu; o.d6 = Z0.v.diu; o.d6t = Z1.v.diu;
    o.g = velfg_fv<P2, ZF>(d, i, j, k, X.v, B.v, Y0.v, Y1.v, Z0.v, Z1.v, bd);
    if (k <= km - 1) {
      o.d7 = X.w.diu; o.d8 = Y0.w.diu; o.d9 = Z0.w.diu;
      o.h = velfg_fw<P2, ZF>(d, i, j, k, X.w, B.w, Y0.w, Y1.w, Z0.w, Z1.w, bd);
    } else {  // k = km: h keeps its value; diu7, diu8 are never written there (zero)
      o.h = hkm;
      o.d7 = 0.f;
      o.d8 = 0.f;
      o.d9 = Z0.w.diu;
    }
    // plane k's j faces are read and plane k+1's written; a plane with a deferred cell is
    // stored by the fixup kernel (lanes and rows past the domain count: their faces feed
    // the cells inside)
    const bool defer = ZF && __syncthreads_or(bd);
    if (!ZF) __syncthreads();
    if (defer) {
      if (lane == 0 && ty == 0) {
        int *list = d.fix[FIX_VELFG];
        const int s = atomicAdd(list, 1);
        list[2 + s] = (int)(((k - 1) * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x);
      }
    } else if (in) {
      velfg_store<FB>(d, c, k, o, fb);
    }
    X = Xn;
    Z0 = Z1;
    Z1 = Z2;
    fxy = fxyn;
    fz0 = fz1;
    fz1 = fz2;
    fb = fbn;
    hkm = hkmn;
    c += d.np;
  }
}

// deferred planes of k_velfg_march: entry ((k-1)*gy + by)*gx + bx, recomputed cell by
// cell with IEEE divisions
template <bool P2, bool FB>
__global__ void __launch_bounds__(MTX *MTY) k_velfg_march_fix(LesDom d, uint3 g) {
  for_deferred(d.fix[FIX_VELFG], g, [&](int bx, int by, int bz) {
    const int i = bx * MTI + (int)threadIdx.x + 1, j = by * MTY + (int)threadIdx.y + 1, k = bz + 1;
    if ((int)threadIdx.x >= MTI || i > d.im || j > d.jm) return;
    const int c = lix(d, i, j, k);
    FbIn fb;
    if (FB) fb = fb_load(d, c);
    VelfgOut o;
    unsigned bd = 0;
    velfg_cell<P2, false>(d, i, j, k, c, o, bd);
    velfg_store<FB>(d, c, k, o, fb);
  });
}

#define SM_(i, j, k) __ldg(&d.sm[lix(d, (i), (j), (k))])

// Smagorinsky face viscosity x/y interpolations: (dx1(i+1)*a + dx1(i)*b)/(dx1(i)+dx1(i+1))
template <bool P2, bool ZF>
__device__ __forceinline__ float ix_(const LesDom &d, int i, float a, float b, unsigned &bd) {
  return dvs<P2, ZF>(sx1<P2>(d, i + 1) * a + sx1<P2>(d, i) * b, sx1<P2>(d, i) + sx1<P2>(d, i + 1), rx1s<P2>(d, i),
                     bd);
}
template <bool P2, bool ZF>  // (dx1(i)*a + dx1(i-1)*b)/(dx1(i-1)+dx1(i))
__device__ __forceinline__ float ixm_(const LesDom &d, int i, float a, float b, unsigned &bd) {
  return dvs<P2, ZF>(sx1<P2>(d, i) * a + sx1<P2>(d, i - 1) * b, sx1<P2>(d, i - 1) + sx1<P2>(d, i),
                     rx1s<P2>(d, i - 1), bd);
}
template <bool P2, bool ZF>  // (dy1(j+1)*a + dy1(j)*b)/(dy1(j)+dy1(j+1))
__device__ __forceinline__ float jy_(const LesDom &d, int j, float a, float b, unsigned &bd) {
  return dvs<P2, ZF>(sy1<P2>(d, j + 1) * a + sy1<P2>(d, j) * b, sy1<P2>(d, j) + sy1<P2>(d, j + 1), ry1s<P2>(d, j),
                     bd);
}
template <bool P2, bool ZF>  // (dy1(j)*a + dy1(j-1)*b)/(dy1(j-1)+dy1(j))
__device__ __forceinline__ float jym_(const LesDom &d, int j, float a, float b, unsigned &bd) {
  return dvs<P2, ZF>(sy1<P2>(d, j) * a + sy1<P2>(d, j - 1) * b, sy1<P2>(d, j - 1) + sy1<P2>(d, j),
                     ry1s<P2>(d, j - 1), bd);
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
// sm, as a k-march: a thread owns column (i, j) and walks a chunk of planes.  Of the 27
// diu values a cell reads, the eight it shares with the plane above or below (e3, e6 at
// k and k+1; e7, e8 at k-1 and k) are carried in registers, so a plane loads 19; the
// next plane's 19 are requested before this plane's arithmetic.
constexpr int STX = 32, STY = 8;

struct SmPlane {  // the values of plane k+1 (k-faces) / k (in-plane) one step needs
  float a3, b3, a6, b6;       // e3(i-1,j), e3(i,j), e6(i,j-1), e6(i,j) at the plane above
  float a7, b7, a8, b8;       // e7(i,j), e7(i+1,j), e8(i,j), e8(i,j+1) at the plane itself
  float e1, e5, e9;           // at the cell
  float e2[4], e4[4];         // e2 at (i-1,j), (i-1,j+1), (i,j), (i,j+1); e4 at (i,j), (i,j-1), (i+1,j), (i+1,j-1)
};

__device__ __forceinline__ SmPlane sm_load(const LesDom &d, int i, int j, int k) {
  SmPlane p;
  p.a3 = e3(d, i - 1, j, k + 1); p.b3 = e3(d, i, j, k + 1);
  p.a6 = e6(d, i, j - 1, k + 1); p.b6 = e6(d, i, j, k + 1);
  p.a7 = e7(d, i, j, k); p.b7 = e7(d, i + 1, j, k);
  p.a8 = e8(d, i, j, k); p.b8 = e8(d, i, j + 1, k);
  p.e1 = e1(d, i, j, k); p.e5 = e5(d, i, j, k); p.e9 = e9(d, i, j, k);
  p.e2[0] = e2(d, i - 1, j, k); p.e2[1] = e2(d, i - 1, j + 1, k); p.e2[2] = e2(d, i, j, k); p.e2[3] = e2(d, i, j + 1, k);
  p.e4[0] = e4(d, i, j, k); p.e4[1] = e4(d, i, j - 1, k); p.e4[2] = e4(d, i + 1, j, k); p.e4[3] = e4(d, i + 1, j - 1, k);
  return p;
}

__global__ void __launch_bounds__(STX *STY) k_les_sm3(LesDom d, int kchunk) {
  const int i = blockIdx.x * STX + threadIdx.x + 1, j = blockIdx.y * STY + threadIdx.y + 1;
  if (i > d.im || j > d.jm) return;
  const int k0 = blockIdx.z * kchunk + 1, k1 = min(k0 + kchunk - 1, d.km);
  // carried: e3, e6 at plane k (a3c, b3c, a6c, b6c) and e7, e8 at plane k-1
  float a3c = e3(d, i - 1, j, k0), b3c = e3(d, i, j, k0), a6c = e6(d, i, j - 1, k0), b6c = e6(d, i, j, k0);
  float a7m = e7(d, i, j, k0 - 1), b7m = e7(d, i + 1, j, k0 - 1), a8m = e8(d, i, j, k0 - 1),
        b8m = e8(d, i, j + 1, k0 - 1);
  SmPlane cur = sm_load(d, i, j, k0);
  for (int k = k0; k <= k1; ++k) {
    SmPlane nxt = cur;
    if (k < k1) nxt = sm_load(d, i, j, k + 1);
    const float dudxx1 = cur.e1;
    const float dudyx1 = (cur.e2[0] + cur.e2[1] + cur.e2[2] + cur.e2[3]) * .25f;
    const float dudzx1 = (a3c + cur.a3 + b3c + cur.b3) * .25f;
    const float dvdxx1 = (cur.e4[0] + cur.e4[1] + cur.e4[2] + cur.e4[3]) * .25f;
    const float dvdyx1 = cur.e5;
    const float dvdzx1 = (a6c + cur.a6 + b6c + cur.b6) * .25f;
    const float dwdxx1 = (cur.a7 + a7m + cur.b7 + b7m) * .25f;
    const float dwdyx1 = (cur.a8 + a8m + cur.b8 + b8m) * .25f;
    const float dwdzx1 = cur.e9;
    const float cd = 0.1f * d.gr.delx1[k];
    const float s1 = dudyx1 + dvdxx1, s2 = dwdyx1 + dvdzx1, s3 = dudzx1 + dwdxx1;
    d.sm[lix(d, i, j, k)] =
        cd * cd * __fsqrt_rn(2.f * (dudxx1 * dudxx1 + dvdyx1 * dvdyx1 + dwdzx1 * dwdzx1) + s1 * s1 + s2 * s2 + s3 * s3);
    a3c = cur.a3; b3c = cur.b3; a6c = cur.a6; b6c = cur.b6;
    a7m = cur.a7; b7m = cur.b7; a8m = cur.a8; b8m = cur.b8;
    cur = nxt;
  }
}

// ------------------------------------------------------------------ les.f95:83-242
// The viscous terms of one cell added to f, g, h.  visc_compute is the arithmetic on
// gathered inputs; visc_cell gathers them from global memory (the fixup path), the
// k-march kernel below gathers them from its shared-memory planes.  Both run the same
// FP32 operations, so their results are identical.

// the stencil values one cell reads: sm (s_*), diu as les reads it (g<n>*), f, g, h
struct ViscIn {
  float s_c, s_e, s_w, s_n, s_s, s_ne, s_se, s_nw, s_u, s_eu, s_wu, s_nu, s_su, s_d, s_ed;
  float g1c, g1e, g2c, g2n, g2wn, g3c, g3u, g3wu, g4c, g4e, g4es, g5c, g5n;
  float g6c, g6u, g6su, g7c, g7e, g7ed, g8c, g8n, g8nd, g9c, g9u;
  float f0, g0, h0;
  float ru, rv;  // u/uspd, v/vspd at k = 1 (k_wall)
};
// column constants: spacings around (i, j), their neighbour sums, reciprocals
struct ViscCol {
  float dx1m, dx1c, dx1p, sxm, sxc, rsxm, rsxc, dxs, rdxs, rdx1;
  float dy1m, dy1c, dy1p, sym, syc, rsym, rsyc, dys, rdys, rdy1;
};
// plane constants at k
struct ViscZ {
  float dznm, dznc, dznp, rdznc, rsumc, rsumm;
};
template <bool P2>
__device__ __forceinline__ ViscCol visc_col(const LesDom &d, int i, int j) {
  ViscCol c;
  c.dx1m = sx1<P2>(d, i - 1); c.dx1c = sx1<P2>(d, i); c.dx1p = sx1<P2>(d, i + 1);
  c.sxm = c.dx1m + c.dx1c; c.sxc = c.dx1c + c.dx1p; c.rsxm = rx1s<P2>(d, i - 1); c.rsxc = rx1s<P2>(d, i);
  c.dxs = sxs<P2>(d, i); c.rdxs = rxs<P2>(d, i); c.rdx1 = rx1<P2>(d, i);
  c.dy1m = sy1<P2>(d, j - 1); c.dy1c = sy1<P2>(d, j); c.dy1p = sy1<P2>(d, j + 1);
  c.sym = c.dy1m + c.dy1c; c.syc = c.dy1c + c.dy1p; c.rsym = ry1s<P2>(d, j - 1); c.rsyc = ry1s<P2>(d, j);
  c.dys = sys<P2>(d, j); c.rdys = rys<P2>(d, j); c.rdy1 = ry1<P2>(d, j);
  return c;
}
__device__ __forceinline__ ViscZ visc_z(const LesDom &d, int k) {
  const LesGrid1 &g = d.gr;
  ViscZ z;
  z.dznm = g.dzn[k - 1]; z.dznc = g.dzn[k]; z.dznp = g.dzn[k + 1];
  z.rdznc = g.rdzn[k]; z.rsumc = g.rdzsum[k]; z.rsumm = g.rdzsum[k - 1];
  return z;
}

template <bool P2, bool ZF>
__device__ __forceinline__ void visc_compute(const LesDom &d, const ViscIn &v, const ViscCol &cc, const ViscZ &z,
                                             int k, float &fv, float &gv, float &hv, unsigned &bd) {
  // (dx1(i+1)*a + dx1(i)*b)/(dx1(i)+dx1(i+1)) and the shifted / y forms of les.f95
  auto ix = [&](float a, float b) { return dvs<P2, ZF>(cc.dx1p * a + cc.dx1c * b, cc.sxc, cc.rsxc, bd); };
  auto ixm = [&](float a, float b) { return dvs<P2, ZF>(cc.dx1c * a + cc.dx1m * b, cc.sxm, cc.rsxm, bd); };
  auto jy = [&](float a, float b) { return dvs<P2, ZF>(cc.dy1p * a + cc.dy1c * b, cc.syc, cc.rsyc, bd); };
  auto jym = [&](float a, float b) { return dvs<P2, ZF>(cc.dy1c * a + cc.dy1m * b, cc.sym, cc.rsym, bd); };
  const float xc = ix(v.s_c, v.s_e);
  const float xu = ix(v.s_u, v.s_eu);
  // x component
  {
    const float evsx2 = v.s_e, evsx1 = v.s_c;
    const float evsy2 = jy(xc, ix(v.s_n, v.s_ne));
    const float evsy1 = jy(ix(v.s_s, v.s_se), xc);
    const float visux2 = (evsx2) * 2.f * v.g1e;
    const float visux1 = (evsx1) * 2.f * v.g1c;
    const float visuy2 = (evsy2) * (v.g2n + v.g4e);
    const float visuy1 = (evsy1) * (v.g2c + v.g4es);
    float vfu;
    if (k >= 2) {
      const float evsz2 = dvz<ZF>(z.dznp * xc + z.dznc * xu, z.dznc + z.dznp, z.rsumc, bd);
      const float evsz1 = dvz<ZF>(z.dznc * ix(v.s_d, v.s_ed) + z.dznm * xc, z.dznm + z.dznc, z.rsumm, bd);
      const float visuz2 = (evsz2) * (v.g3u + v.g7e);
      const float visuz1 = (evsz1) * (v.g3c + v.g7ed);
      vfu = dvs<P2, ZF>(visux2 - visux1, cc.dxs, cc.rdxs, bd) + dvs<P2, ZF>(visuy2 - visuy1, cc.dy1c, cc.rdy1, bd) +
            dvz<ZF>(visuz2 - visuz1, z.dznc, z.rdznc, bd);
    } else {  // les.f95:118-139: the y and z terms appear twice, as written (k = 1: dznc = dzn(1))
      const float evsz2 = dvz<ZF>(z.dznp * xc + z.dznc * xu, z.dznc + z.dznp, z.rsumc, bd);
      const float visuz2 = (evsz2) * (v.g3u + v.g7e);
      const float t = dvz<ZF>(0.4f * v.ru, d.logz, d.rlogz, bd);
      const float visuz1 = t * t * v.ru;
      const float ty = dvs<P2, ZF>(visuy2 - visuy1, cc.dy1c, cc.rdy1, bd);
      const float tz = dvz<ZF>(visuz2 - visuz1, z.dznc, z.rdznc, bd);
      vfu = dvs<P2, ZF>(visux2 - visux1, cc.dxs, cc.rdxs, bd) + ty + tz + ty + tz;
    }
    fv = v.f0 + vfu;
  }
  // y component
  {
    const float evsy2 = v.s_n, evsy1 = v.s_c;
    const float evsx2 = jy(xc, ix(v.s_n, v.s_ne));
    const float evsx1 = jy(ixm(v.s_w, v.s_c), ixm(v.s_nw, v.s_n));
    const float visvx2 = (evsx2) * (v.g2n + v.g4e);
    const float visvx1 = (evsx1) * (v.g2wn + v.g4c);
    const float visvy2 = (evsy2) * 2.f * v.g5n;
    const float visvy1 = (evsy1) * 2.f * v.g5c;
    float vfv;
    if (k >= 2) {
      const float evsz2 = dvz<ZF>(z.dznp * xc + z.dznc * xu, z.dznc + z.dznp, z.rsumc, bd);
      const float evsz1 = dvz<ZF>(z.dznc * ix(v.s_d, v.s_ed) + z.dznm * xc, z.dznm + z.dznc, z.rsumm, bd);
      const float visvz2 = (evsz2) * (v.g6u + v.g8n);
      const float visvz1 = (evsz1) * (v.g6c + v.g8nd);
      vfv = dvs<P2, ZF>(visvx2 - visvx1, cc.dx1c, cc.rdx1, bd) + dvs<P2, ZF>(visvy2 - visvy1, cc.dys, cc.rdys, bd) +
            dvz<ZF>(visvz2 - visvz1, z.dznc, z.rdznc, bd);
    } else {  // les.f95:178-201
      const float evsz2 = dvz<ZF>(z.dznp * xc + z.dznc * xu, z.dznc + z.dznp, z.rsumc, bd);
      const float visvz2 = (evsz2) * (v.g6u + v.g8n);
      const float t = dvz<ZF>(0.4f * v.rv, d.logz, d.rlogz, bd);
      const float visvz1 = t * t * v.rv;
      vfv = dvs<P2, ZF>(visvx2 - visvx1, cc.dx1c, cc.rdx1, bd) + dvs<P2, ZF>(visvy2 - visvy1, cc.dys, cc.rdys, bd) +
            dvz<ZF>(visvz2 - visvz1, z.dznc, z.rdznc, bd);
    }
    gv = v.g0 + vfv;
  }
  // z component, k = 1..km
  {
    const float dzc = z.dznc + z.dznp, rdzc = z.rsumc;
    const float evsz2 = v.s_u, evsz1 = v.s_c;
    const float evsx2 = dvz<ZF>(z.dznp * xc + z.dznc * xu, dzc, rdzc, bd);
    const float evsx1 = dvz<ZF>(z.dznp * ixm(v.s_w, v.s_c) + z.dznc * ixm(v.s_wu, v.s_u), dzc, rdzc, bd);
    const float evsy2 = dvz<ZF>(z.dznp * jy(v.s_c, v.s_n) + z.dznc * jy(v.s_u, v.s_nu), dzc, rdzc, bd);
    const float evsy1 = dvz<ZF>(z.dznp * jym(v.s_s, v.s_c) + z.dznc * jym(v.s_su, v.s_u), dzc, rdzc, bd);
    const float viswx2 = (evsx2) * (v.g3u + v.g7e);
    const float viswx1 = (evsx1) * (v.g3wu + v.g7c);
    const float viswy2 = (evsy2) * (v.g6u + v.g8n);
    const float viswy1 = (evsy1) * (v.g6su + v.g8c);
    const float viswz2 = (evsz2) * 2.f * v.g9u;
    const float viswz1 = (evsz1) * 2.f * v.g9c;
    const float vfw = dvs<P2, ZF>(viswx2 - viswx1, cc.dx1c, cc.rdx1, bd) + dvs<P2, ZF>(viswy2 - viswy1, cc.dy1c, cc.rdy1, bd) +
                      dvz<ZF>(viswz2 - viswz1, z.dznc, z.rdznc, bd);
    hv = v.h0 + vfw;
  }
}

// gradients and sm around (i, j, k) from global memory
template <bool P2, bool ZF>
__device__ __forceinline__ void visc_cell(const LesDom &d, int i, int j, int k, int c, float &fv, float &gv, float &hv,
                                          unsigned &bd) {
  ViscIn v;
  v.s_c = SM_(i, j, k); v.s_e = SM_(i + 1, j, k); v.s_w = SM_(i - 1, j, k);
  v.s_n = SM_(i, j + 1, k); v.s_s = SM_(i, j - 1, k);
  v.s_ne = SM_(i + 1, j + 1, k); v.s_se = SM_(i + 1, j - 1, k); v.s_nw = SM_(i - 1, j + 1, k);
  v.s_u = SM_(i, j, k + 1); v.s_eu = SM_(i + 1, j, k + 1); v.s_wu = SM_(i - 1, j, k + 1);
  v.s_nu = SM_(i, j + 1, k + 1); v.s_su = SM_(i, j - 1, k + 1);
  v.s_d = SM_(i, j, k - 1); v.s_ed = SM_(i + 1, j, k - 1);
  v.g1c = e1(d, i, j, k); v.g1e = e1(d, i + 1, j, k);
  v.g2c = e2(d, i, j, k); v.g2n = e2(d, i, j + 1, k); v.g2wn = e2(d, i - 1, j + 1, k);
  v.g3c = e3(d, i, j, k); v.g3u = e3(d, i, j, k + 1); v.g3wu = e3(d, i - 1, j, k + 1);
  v.g4c = e4(d, i, j, k); v.g4e = e4(d, i + 1, j, k); v.g4es = e4(d, i + 1, j - 1, k);
  v.g5c = e5(d, i, j, k); v.g5n = e5(d, i, j + 1, k);
  v.g6c = e6(d, i, j, k); v.g6u = e6(d, i, j, k + 1); v.g6su = e6(d, i, j - 1, k + 1);
  v.g7c = e7(d, i, j, k); v.g7e = e7(d, i + 1, j, k); v.g7ed = e7(d, i + 1, j, k - 1);
  v.g8c = e8(d, i, j, k); v.g8n = e8(d, i, j + 1, k); v.g8nd = e8(d, i, j + 1, k - 1);
  v.g9c = e9(d, i, j, k); v.g9u = e9(d, i, j, k + 1);
  v.f0 = d.f[c]; v.g0 = d.g[c]; v.h0 = d.h[c];
  v.ru = (k == 1) ? __ldg(&d.ruspd[(j + LES_JOFF) * d.pi + i + LES_IOFF]) : 0.f;
  v.rv = (k == 1) ? __ldg(&d.rvspd[(j + LES_JOFF) * d.pi + i + LES_IOFF]) : 0.f;
  visc_compute<P2, ZF>(d, v, visc_col<P2>(d, i, j), visc_z(d, k), k, fv, gv, hv, bd);
}

// adam.f95:30-44 (when AD; fo, go, ho: fold, gold, hold loaded by the caller ahead of
// time, so their latency hides behind the viscous arithmetic) and the stores of one cell
template <bool AD>
__device__ __forceinline__ void visc_store(const LesDom &d, int c, float fv, float gv, float hv, float fo, float go,
                                           float ho) {
  if (AD) {
    d.fold[c] = fv; d.gold[c] = gv; d.hold[c] = hv;
    fv = 1.5f * fv - 0.5f * fo;
    gv = 1.5f * gv - 0.5f * go;
    hv = 1.5f * hv - 0.5f * ho;
  }
  d.f[c] = fv;
  d.g[c] = gv;
  d.h[c] = hv;
}

// ---- the k-march kernel ------------------------------------------------------------
// A block owns a VTX x VTY tile of columns and marches k over a chunk of VKC planes.
// The planes of sm and diu1..9 that a cell reads (as les reads them: index remaps and
// zero entries applied at load time) sit in a shared-memory ring with a one-cell halo;
// each step's new planes are loaded into registers while the current plane computes.
constexpr int VTX = 32, VTY = 8, VTW = VTX + 2, VTH = VTY + 2, VTN = VTW * VTH, VKC = 30;
constexpr int VEL = (VTN + VTX * VTY - 1) / (VTX * VTY);  // tile elements per thread (2)
// ring slots: sm 3 planes; diu1, 2, 4, 5 one; diu3, 6, 9 (k, k+1) and diu7, 8 (k-1, k) two
enum { S_SM = 0, S_E1 = 3, S_E2, S_E4, S_E5, S_E3 = 7, S_E6 = 9, S_E9 = 11, S_E7 = 13, S_E8 = 15, S_N = 17 };

// value of array q (0 = sm, n = diu_n as les reads it) at tile point (ii, jj, kk);
// points past the domain edge are clamped into the allocation (never used)
__device__ __forceinline__ float visc_src(const LesDom &d, int q, int ii, int jj, int kk) {
  ii = min(ii, d.im + 2);
  jj = min(jj, d.jm + 2);
  const int iA = min(ii, d.im), jP = (jj > d.jm) ? 1 : jj, jM = (jj <= 0) ? d.jm : jj;
  const bool kz7 = (kk <= 0 || kk >= d.km);
  switch (q) {
    case 0: return SM_(ii, jj, kk);
    case 1: return DIU_(1, iA, jj, kk);
    case 2: return (ii <= 0) ? 0.f : DIU_(2, ii, jP, kk);
    case 3: return (ii <= 0) ? 0.f : DIU_(3, ii, jj, kk);
    case 4: return DIU_(4, iA, jM, kk);
    case 5: return DIU_(5, ii, jP, kk);
    case 6: return DIU_(6, ii, jM, kk);
    case 7: return kz7 ? 0.f : DIU_(7, iA, jj, kk);
    case 8: return kz7 ? 0.f : DIU_(8, ii, jP, kk);
    default: return (kk > d.km) ? 0.f : DIU_(9, ii, jj, kk);
  }
}

template <bool P2, bool ZF, bool AD>
__global__ void __launch_bounds__(VTX *VTY, 2) k_les_visc_march(LesDom d) {
  __shared__ float ring[S_N * VTN];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * VTX + tx;
  const int i0 = blockIdx.x * VTX, j0 = blockIdx.y * VTY;  // tile origin (halo) at (i0, j0)
  const int k0 = blockIdx.z * VKC + 1, k1 = min(k0 + VKC - 1, d.km);
  const int i = i0 + tx + 1, j = j0 + ty + 1;
  const bool in = (i <= d.im && j <= d.jm);
  const int ic = min(i, d.im), jc = min(j, d.jm);
  // this thread's tile elements
  int ea[VEL], eb[VEL];
  bool ev[VEL];
#pragma unroll
  for (int q = 0; q < VEL; ++q) {
    const int e = tid + q * VTX * VTY;
    ev[q] = e < VTN;
    ea[q] = e % VTW;
    eb[q] = e / VTW;
  }
  auto put = [&](int slot, int q, int kk) {  // load one plane of array q into `slot` (synchronous)
#pragma unroll
    for (int t = 0; t < VEL; ++t)
      if (ev[t]) ring[slot * VTN + eb[t] * VTW + ea[t]] = visc_src(d, q, i0 + ea[t], j0 + eb[t], kk);
  };
  // prologue: the planes step k0 reads
  put(S_SM + (k0 - 1) % 3, 0, k0 - 1);
  put(S_SM + k0 % 3, 0, k0);
  put(S_SM + (k0 + 1) % 3, 0, k0 + 1);
  put(S_E1, 1, k0); put(S_E2, 2, k0); put(S_E4, 4, k0); put(S_E5, 5, k0);
  put(S_E3 + (k0 & 1), 3, k0); put(S_E3 + ((k0 + 1) & 1), 3, k0 + 1);
  put(S_E6 + (k0 & 1), 6, k0); put(S_E6 + ((k0 + 1) & 1), 6, k0 + 1);
  put(S_E9 + (k0 & 1), 9, k0); put(S_E9 + ((k0 + 1) & 1), 9, k0 + 1);
  put(S_E7 + ((k0 - 1) & 1), 7, k0 - 1); put(S_E7 + (k0 & 1), 7, k0);
  put(S_E8 + ((k0 - 1) & 1), 8, k0 - 1); put(S_E8 + (k0 & 1), 8, k0);
  const ViscCol cc = visc_col<P2>(d, ic, jc);
  float ru = 0.f, rv = 0.f;
  if (k0 == 1) {
    ru = __ldg(&d.ruspd[(jc + LES_JOFF) * d.pi + ic + LES_IOFF]);
    rv = __ldg(&d.rvspd[(jc + LES_JOFF) * d.pi + ic + LES_IOFF]);
  }
  int c = lix(d, ic, jc, k0);
  float f0 = d.f[c], g0 = d.g[c], h0 = d.h[c];
  float fo = 0.f, go = 0.f, ho = 0.f;
  if (AD) { fo = d.fold[c]; go = d.gold[c]; ho = d.hold[c]; }
  __syncthreads();
  const int a = tx + 1, b = ty + 1;
#define RS(slot, da, db) ring[(slot) * VTN + (b + (db)) * VTW + (a + (da))]
  for (int k = k0; k <= k1; ++k) {
    const bool more = k < k1;
    // next step's planes and cell values, in flight while this plane computes
    float nx[10][VEL];
    float nf = 0.f, ng = 0.f, nh = 0.f, nfo = 0.f, ngo = 0.f, nho = 0.f;
    if (more) {
#pragma unroll
      for (int t = 0; t < VEL; ++t) {
        if (!ev[t]) continue;
        const int ii = i0 + ea[t], jj = j0 + eb[t];
        nx[0][t] = visc_src(d, 0, ii, jj, k + 2);
        nx[1][t] = visc_src(d, 1, ii, jj, k + 1);
        nx[2][t] = visc_src(d, 2, ii, jj, k + 1);
        nx[4][t] = visc_src(d, 4, ii, jj, k + 1);
        nx[5][t] = visc_src(d, 5, ii, jj, k + 1);
        nx[3][t] = visc_src(d, 3, ii, jj, k + 2);
        nx[6][t] = visc_src(d, 6, ii, jj, k + 2);
        nx[9][t] = visc_src(d, 9, ii, jj, k + 2);
        nx[7][t] = visc_src(d, 7, ii, jj, k + 1);
        nx[8][t] = visc_src(d, 8, ii, jj, k + 1);
      }
      const int cn = c + d.np;
      nf = d.f[cn]; ng = d.g[cn]; nh = d.h[cn];
      if (AD) { nfo = d.fold[cn]; ngo = d.gold[cn]; nho = d.hold[cn]; }
    }
    // gather this cell's stencil from the ring
    const int sm0 = S_SM + (k - 1) % 3, sm1 = S_SM + k % 3, sm2 = S_SM + (k + 1) % 3;
    const int e3c = S_E3 + (k & 1), e3u = S_E3 + ((k + 1) & 1);
    const int e6c = S_E6 + (k & 1), e6u = S_E6 + ((k + 1) & 1);
    const int e9c = S_E9 + (k & 1), e9u = S_E9 + ((k + 1) & 1);
    const int e7c = S_E7 + (k & 1), e7d = S_E7 + ((k - 1) & 1);
    const int e8c = S_E8 + (k & 1), e8d = S_E8 + ((k - 1) & 1);
    ViscIn v;
    v.s_c = RS(sm1, 0, 0); v.s_e = RS(sm1, 1, 0); v.s_w = RS(sm1, -1, 0);
    v.s_n = RS(sm1, 0, 1); v.s_s = RS(sm1, 0, -1);
    v.s_ne = RS(sm1, 1, 1); v.s_se = RS(sm1, 1, -1); v.s_nw = RS(sm1, -1, 1);
    v.s_u = RS(sm2, 0, 0); v.s_eu = RS(sm2, 1, 0); v.s_wu = RS(sm2, -1, 0);
    v.s_nu = RS(sm2, 0, 1); v.s_su = RS(sm2, 0, -1);
    v.s_d = RS(sm0, 0, 0); v.s_ed = RS(sm0, 1, 0);
    v.g1c = RS(S_E1, 0, 0); v.g1e = RS(S_E1, 1, 0);
    v.g2c = RS(S_E2, 0, 0); v.g2n = RS(S_E2, 0, 1); v.g2wn = RS(S_E2, -1, 1);
    v.g3c = RS(e3c, 0, 0); v.g3u = RS(e3u, 0, 0); v.g3wu = RS(e3u, -1, 0);
    v.g4c = RS(S_E4, 0, 0); v.g4e = RS(S_E4, 1, 0); v.g4es = RS(S_E4, 1, -1);
    v.g5c = RS(S_E5, 0, 0); v.g5n = RS(S_E5, 0, 1);
    v.g6c = RS(e6c, 0, 0); v.g6u = RS(e6u, 0, 0); v.g6su = RS(e6u, 0, -1);
    v.g7c = RS(e7c, 0, 0); v.g7e = RS(e7c, 1, 0); v.g7ed = RS(e7d, 1, 0);
    v.g8c = RS(e8c, 0, 0); v.g8n = RS(e8c, 0, 1); v.g8nd = RS(e8d, 0, 1);
    v.g9c = RS(e9c, 0, 0); v.g9u = RS(e9u, 0, 0);
    v.f0 = f0; v.g0 = g0; v.h0 = h0;
    v.ru = ru; v.rv = rv;
    float fv, gv, hv;
    unsigned bd = 0;
    visc_compute<P2, ZF>(d, v, cc, visc_z(d, k), k, fv, gv, hv, bd);
    // every thread is done with the ring; a plane with a deferred cell is stored by the fixup
    const bool defer = ZF && __syncthreads_or(in ? bd : 0u);
    if (!ZF) __syncthreads();
    if (defer) {
      if (tid == 0) {
        int *list = d.fix[FIX_VISC];
        const int s = atomicAdd(list, 1);
        list[2 + s] = (int)(((k - 1) * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x);
      }
    } else if (in) {
      visc_store<AD>(d, c, fv, gv, hv, fo, go, ho);
    }
    if (more) {
#pragma unroll
      for (int t = 0; t < VEL; ++t) {
        if (!ev[t]) continue;
        const int o = eb[t] * VTW + ea[t];
        ring[(S_SM + (k + 2) % 3) * VTN + o] = nx[0][t];
        ring[S_E1 * VTN + o] = nx[1][t];
        ring[S_E2 * VTN + o] = nx[2][t];
        ring[S_E4 * VTN + o] = nx[4][t];
        ring[S_E5 * VTN + o] = nx[5][t];
        ring[(S_E3 + (k & 1)) * VTN + o] = nx[3][t];
        ring[(S_E6 + (k & 1)) * VTN + o] = nx[6][t];
        ring[(S_E9 + (k & 1)) * VTN + o] = nx[9][t];
        ring[(S_E7 + ((k + 1) & 1)) * VTN + o] = nx[7][t];
        ring[(S_E8 + ((k + 1) & 1)) * VTN + o] = nx[8][t];
      }
      c += d.np;
      f0 = nf; g0 = ng; h0 = nh;
      fo = nfo; go = ngo; ho = nho;
      ru = 0.f; rv = 0.f;
      __syncthreads();
    }
  }
#undef RS
}

// deferred planes of k_les_visc_march: entry ((k-1)*gy + by)*gx + bx, recomputed
// cell by cell with IEEE divisions from global memory
template <bool P2, bool AD>
__global__ void __launch_bounds__(VTX *VTY) k_les_visc_fix(LesDom d, uint3 g) {
  for_deferred(d.fix[FIX_VISC], g, [&](int bx, int by, int bz) {
    const int i = bx * VTX + (int)threadIdx.x + 1, j = by * VTY + (int)threadIdx.y + 1, k = bz + 1;
    if (i > d.im || j > d.jm) return;
    const int c = lix(d, i, j, k);
    float fv, gv, hv;
    unsigned bd = 0;
    float fo = 0.f, go = 0.f, ho = 0.f;
    if (AD) { fo = d.fold[c]; go = d.gold[c]; ho = d.hold[c]; }
    visc_cell<P2, false>(d, i, j, k, c, fv, gv, hv, bd);
    visc_store<AD>(d, c, fv, gv, hv, fo, go, ho);
  });
}


// ---- the halo entries of diu that les reads through index remaps ----------------------
// The copies vel2.f95:202-318 makes, written into the stored arrays after velfg (and its
// fixup) so that the TMA-fed sm pass and viscous march read plain boxes: diu1, diu4,
// diu7 at i = im+1 (the values at i = im), diu2, diu5, diu8 at j = jm+1 (at j = 1), diu4
// at j = 0 (at j = jm) for k = 1..km, diu6 at j = 0 for k = 1..km+1, and diu4 at
// (im+1, 0) (at (im, jm)).  The
// other remapped entries read as zero (diu2, diu3 at i = 0; diu7, diu8 at k = 0; diu9 at
// k = km+1): nothing writes them, and the arrays start zeroed.  One thread per face
// point (jm of the i face, im of the j faces, the corner), one block row per plane.
__global__ void k_diu_halo(LesDom d) {
  const int k = blockIdx.y + 1;  // 1 .. km+1
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int jmp = d.jm * d.pi;
  if (t < d.jm) {
    if (k > d.km) return;
    const int c = lix(d, d.im, t + 1, k);
    d.diu[1][c + 1] = d.diu[1][c];
    d.diu[4][c + 1] = d.diu[4][c];
    d.diu[7][c + 1] = d.diu[7][c];
  } else if (t < d.jm + d.im) {
    const int i = t - d.jm + 1;
    if (k <= d.km) {
      const int c1 = lix(d, i, 1, k);
      d.diu[2][c1 + jmp] = d.diu[2][c1];
      d.diu[5][c1 + jmp] = d.diu[5][c1];
      d.diu[8][c1 + jmp] = d.diu[8][c1];
      const int cm = lix(d, i, d.jm, k);
      d.diu[4][cm - jmp] = d.diu[4][cm];
    }
    const int cm = lix(d, i, d.jm, k);
    d.diu[6][cm - jmp] = d.diu[6][cm];
  } else if (t == d.jm + d.im && k <= d.km) {
    const int c = lix(d, d.im, d.jm, k);
    d.diu[4][c + 1 - jmp] = d.diu[4][c];
  }
}

// halo boxes of the TMA-fed les kernels: 40 x 10 floats (VHB), slots VHS floats apart
// (a 128-byte multiple); cell boxes 32 x 8 (VCB)
constexpr int VBW = 40, VHB = VBW * VTH, VHS = 416, VCB = VTX * VTY;

// ---- sm from TMA-staged diu planes ---------------------------------------------------
// k_les_sm3's arithmetic (les.f95:45-65) on 32 x 8 column tiles marching k, with the diu
// planes it reads brought by tensor copies (40 x 10 boxes, as the viscous march below
// reads them; k_diu_halo has stored the remapped halo entries).  Copy group kk brings
// diu1,2,4,5,9,7,8 at kk and diu3,6 at kk+1; step k reads groups k and k-1 (diu3,6 at
// k and k+1, diu7,8 at k-1 and k).  Rings: diu3,6,7,8 2+VLA planes, the rest 1+VLA;
// once every thread has finished step k the group of plane k+1+VLA is issued.
template <int VLA>
struct SmSmem {
  float z[4][2 + VLA][VHS];  // diu3, diu6 (at kk+1), diu7, diu8 (at kk)
  float x[5][1 + VLA][VHS];  // diu1, diu2, diu4, diu5, diu9 (at kk)
  uint64_t bar[2 + VLA];
};
struct LesSmMaps {
  CUtensorMap m[9];  // diu1..9
};

template <int VLA>
__global__ void __launch_bounds__(VTX *VTY) k_les_sm_tma(LesDom d, const __grid_constant__ LesSmMaps M, int kchunk) {
  extern __shared__ __align__(1024) unsigned char ssm_raw[];
  constexpr int NB = 2 + VLA, NZ = 2 + VLA, NX1 = 1 + VLA;
  SmSmem<VLA> &S = *reinterpret_cast<SmSmem<VLA> *>(ssm_raw);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * VTX + tx;
  const int i0 = blockIdx.x * VTX, j0 = blockIdx.y * VTY;
  const int k0 = blockIdx.z * kchunk + 1, k1 = min(k0 + kchunk - 1, d.km);
  const int i = i0 + tx + 1, j = j0 + ty + 1;
  const bool in = (i <= d.im && j <= d.jm);
  const int last_t = k1 - k0 + 1;  // group t holds plane kk = k0 - 1 + t
  // diu_n of the box lanes issue: lane q < 9 copies diu(q+1); group 0 needs diu3, 6, 7, 8 only
  auto issue = [&](int t) {  // by the 32 lanes of warp 0
    const int q = t % NB, kk = k0 - 1 + t;
    const uint32_t bytes = (t == 0 ? 4u : 9u) * VHB * 4u;
    if (tx == 0) mbar_expect_tx(&S.bar[q], bytes);
    __syncwarp();
    const int n = tx + 1;
    if (tx < 9 && (t > 0 || n == 3 || n == 6 || n == 7 || n == 8)) {
      float *dst;
      int z = kk;
      if (n == 3 || n == 6) { dst = S.z[n / 3 - 1][t % NZ]; z = kk + 1; }
      else if (n == 7 || n == 8) dst = S.z[n - 5][t % NZ];
      else dst = S.x[n == 1 ? 0 : n == 2 ? 1 : n == 4 ? 2 : n == 5 ? 3 : 4][t % NX1];
      tma_load_3d(dst, &M.m[tx], i0, j0 + LES_JOFF, z + LES_KOFF, &S.bar[q]);
    }
  };
  if (tid == 0) {
    for (int q = 0; q < NB; ++q) mbar_init(&S.bar[q], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  int issued = -1;
  if (ty == 0)
    for (int t = 0; t < NB && t <= last_t; ++t) {
      issue(t);
      issued = t;
    }
  bool bad = false;
  int waited = -1;
  auto wait_group = [&](int t) {
    if (bad) return;
    if (mbar_wait(&S.bar[t % NB], (uint32_t)((t / NB) & 1))) {
      waited = t;
    } else {
      bad = true;
      d.ctl[CT_ERROR] = 1;
    }
  };
  wait_group(0);
  const int o = (ty + 1) * VBW + tx + 4;  // this cell in a halo box
  int c = lix(d, min(i, d.im), min(j, d.jm), k0);
  for (int k = k0; k <= k1; ++k) {
    const int t = k - k0 + 1;
    wait_group(t);
    const int za = t % NZ, zb = (t - 1) % NZ, xa = t % NX1;
#define ZA(n, da, db) S.z[n][za][o + (db) * VBW + (da)]
#define ZB(n, da, db) S.z[n][zb][o + (db) * VBW + (da)]
#define XA(n, da, db) S.x[n][xa][o + (db) * VBW + (da)]
    const float dudxx1 = XA(0, 0, 0);
    const float dudyx1 = (XA(1, -1, 0) + XA(1, -1, 1) + XA(1, 0, 0) + XA(1, 0, 1)) * .25f;
    const float dudzx1 = (ZB(0, -1, 0) + ZA(0, -1, 0) + ZB(0, 0, 0) + ZA(0, 0, 0)) * .25f;
    const float dvdxx1 = (XA(2, 0, 0) + XA(2, 0, -1) + XA(2, 1, 0) + XA(2, 1, -1)) * .25f;
    const float dvdyx1 = XA(3, 0, 0);
    const float dvdzx1 = (ZB(1, 0, -1) + ZA(1, 0, -1) + ZB(1, 0, 0) + ZA(1, 0, 0)) * .25f;
    const float dwdxx1 = (ZA(2, 0, 0) + ZB(2, 0, 0) + ZA(2, 1, 0) + ZB(2, 1, 0)) * .25f;
    const float dwdyx1 = (ZA(3, 0, 0) + ZB(3, 0, 0) + ZA(3, 0, 1) + ZB(3, 0, 1)) * .25f;
    const float dwdzx1 = XA(4, 0, 0);
#undef ZA
#undef ZB
#undef XA
    const float cd = 0.1f * d.gr.delx1[k];
    const float s1 = dudyx1 + dvdxx1, s2 = dwdyx1 + dvdzx1, s3 = dudzx1 + dwdxx1;
    const float smv =
        cd * cd * __fsqrt_rn(2.f * (dudxx1 * dudxx1 + dvdyx1 * dvdyx1 + dwdzx1 * dwdzx1) + s1 * s1 + s2 * s2 + s3 * s3);
    __syncthreads();  // every thread has read step k: group k+1+VLA may take the slots of k-1 and k
    if (ty == 0) {    // warp 0 (uniform: issue holds a __syncwarp); none of it issues after a failed wait
      const bool wbad = __any_sync(0xffffffffu, bad);
      if (!wbad && t + 1 + VLA <= last_t) {
        issue(t + 1 + VLA);
        issued = t + 1 + VLA;
      }
    }
    if (in) d.sm[c] = smv;
    c += d.np;
  }
  if (ty == 0 && bad)
    for (int t = waited + 1; t <= issued; ++t) (void)mbar_wait(&S.bar[t % NB], (uint32_t)((t / NB) & 1));
}

// ---- the TMA-fed viscous march -------------------------------------------------------
// k_les_visc_march with its planes brought into shared memory by tensor copies instead
// of loads staged through registers.  k_diu_halo has stored the halo entries of the diu
// arrays that les reads through index remaps, so every plane the march reads is a plain
// box of a padded array: sm and diu1..9 as 40 x 10 boxes (i0-3 .. i0+36, the
// tile's columns with their one-cell ring widened to 16-byte boundaries; rows j0 ..
// j0+9), f, g, h (and fold, gold, hold with adam) as 32 x 8 boxes of the tile's cells.
// Copy group kk brings sm(kk+1), diu1,2,4,5,7,8(kk), diu3,6,9(kk+1) and the cells'
// arrays at kk; step k reads the groups of planes k, k-1 and k-2, and once every thread
// has finished step k the group of plane k+1+VLA is issued, so the copies of VLA steps
// are in flight while a step computes.  Each array has a ring of its own, as deep as its
// reach: sm 3+VLA planes (read at k-1, k, k+1), diu3,6,9,7,8 2+VLA (two planes each),
// diu1,2,4,5 and the cell arrays 1+VLA, so that three CTAs fit an SM's shared memory.
// Warp 0 issues a group (one copy per lane) after lane 0 has armed the group's mbarrier
// with the bytes to expect; every thread waits (bounded) for the groups it reads.  The arithmetic is visc_compute's,
// so the fields are bitwise those of k_les_visc_march.
struct LesViscMaps {
  CUtensorMap m[16];  // sm, diu1..9, f, g, h, fold, gold, hold
};
template <int VLA>
struct ViscSmem {
  float sm[3 + VLA][VHS];    // sm(kk+1) of group kk in slot kk % (3+VLA)
  float z[5][2 + VLA][VHS];  // diu3, diu6, diu9 (at kk+1), diu7, diu8 (at kk)
  float x[4][1 + VLA][VHS];  // diu1, diu2, diu4, diu5 (at kk)
  float c[6][1 + VLA][VCB];  // f, g, h, fold, gold, hold (at kk)
  uint64_t bar[3 + VLA];     // one per group in flight
};

template <bool P2, bool ZF, bool AD, int VLA>
__global__ void __launch_bounds__(VTX *VTY, P2 ? 3 : 2) k_les_visc_tma(LesDom d, const __grid_constant__ LesViscMaps M) {
  extern __shared__ __align__(1024) unsigned char vsm_raw[];
  constexpr int NS = 3 + VLA, NZ = 2 + VLA, NX1 = 1 + VLA;
  constexpr int NMAP = AD ? 16 : 13;
  ViscSmem<VLA> &S = *reinterpret_cast<ViscSmem<VLA> *>(vsm_raw);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * VTX + tx;
  const int i0 = blockIdx.x * VTX, j0 = blockIdx.y * VTY;  // tile origin (halo) at (i0, j0)
  const int k0 = blockIdx.z * VKC + 1, k1 = min(k0 + VKC - 1, d.km);
  const int i = i0 + tx + 1, j = j0 + ty + 1;
  const bool in = (i <= d.im && j <= d.jm);
  const int ic = min(i, d.im), jc = min(j, d.jm);
  const int last_t = k1 - k0 + 2;  // group t holds plane kk = k0 - 2 + t

  // group t: t = 0 needs only sm(k0-1), t = 1 sm(k0), diu3,6,9(k0), diu7,8(k0-1)
  auto issue = [&](int t) {  // by the 32 lanes of warp 0
    const int q = t % NS, kk = k0 - 2 + t;
    const uint32_t mask = (t == 0) ? 0x1u : (t == 1) ? 0x3c9u : 0xffffu;  // maps issued
    const uint32_t bytes = (t == 0) ? VHB * 4u : (t == 1) ? 6u * VHB * 4u : (10u * VHB + (NMAP - 10u) * VCB) * 4u;
    if (tx == 0) mbar_expect_tx(&S.bar[q], bytes);
    __syncwarp();
    if (tx < NMAP && ((mask >> tx) & 1u)) {
      if (tx < 10) {
        float *dst;
        int z = kk;
        if (tx == 0) { dst = S.sm[t % NS]; z = kk + 1; }
        else if (tx == 3 || tx == 6 || tx == 9) { dst = S.z[tx / 3 - 1][t % NZ]; z = kk + 1; }
        else if (tx == 7 || tx == 8) dst = S.z[tx - 4][t % NZ];
        else dst = S.x[tx == 1 ? 0 : tx == 2 ? 1 : tx == 4 ? 2 : 3][t % NX1];
        tma_load_3d(dst, &M.m[tx], i0, j0 + LES_JOFF, z + LES_KOFF, &S.bar[q]);
      } else {
        tma_load_3d(S.c[tx - 10][t % NX1], &M.m[tx], i0 + 1 + LES_IOFF, j0 + 1 + LES_JOFF, kk + LES_KOFF, &S.bar[q]);
      }
    }
  };
  if (tid == 0) {
    for (int q = 0; q < NS; ++q) mbar_init(&S.bar[q], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  int issued = -1;
  if (ty == 0)
    for (int t = 0; t < NS && t <= last_t; ++t) {
      issue(t);
      issued = t;
    }
  // a wait that gives up sets CT_ERROR; this thread then skips its later waits (the
  // step's results are void and reported) so the march still ends in bounded time
  bool bad = false;
  int waited = -1;
  auto wait_group = [&](int t) {
    if (bad) return;
    if (mbar_wait(&S.bar[t % NS], (uint32_t)((t / NS) & 1))) {
      waited = t;
    } else {
      bad = true;
      d.ctl[CT_ERROR] = 1;
    }
  };
  const ViscCol cc = visc_col<P2>(d, ic, jc);
  float ru = 0.f, rv = 0.f;
  if (k0 == 1) {
    ru = __ldg(&d.ruspd[(jc + LES_JOFF) * d.pi + ic + LES_IOFF]);
    rv = __ldg(&d.rvspd[(jc + LES_JOFF) * d.pi + ic + LES_IOFF]);
  }
  int c = lix(d, ic, jc, k0);
  wait_group(0);
  wait_group(1);
  const int o = (ty + 1) * VBW + tx + 4;  // this cell in a halo box
  const int oc = ty * VTX + tx;           // and in a cell box
  for (int k = k0; k <= k1; ++k) {
    const int t = k - k0 + 2;
    wait_group(t);
    const float *smA = S.sm[t % NS], *smB = S.sm[(t - 1) % NS], *smC = S.sm[(t - 2) % NS];
    const int za = t % NZ, zb = (t - 1) % NZ, xa = t % NX1;
#define SA(da, db) smA[o + (db) * VBW + (da)]
#define SB(da, db) smB[o + (db) * VBW + (da)]
#define SC(da, db) smC[o + (db) * VBW + (da)]
#define ZA(n, da, db) S.z[n][za][o + (db) * VBW + (da)]
#define ZB(n, da, db) S.z[n][zb][o + (db) * VBW + (da)]
#define XA(n, da, db) S.x[n][xa][o + (db) * VBW + (da)]
    ViscIn v;
    v.s_c = SB(0, 0); v.s_e = SB(1, 0); v.s_w = SB(-1, 0);
    v.s_n = SB(0, 1); v.s_s = SB(0, -1);
    v.s_ne = SB(1, 1); v.s_se = SB(1, -1); v.s_nw = SB(-1, 1);
    v.s_u = SA(0, 0); v.s_eu = SA(1, 0); v.s_wu = SA(-1, 0);
    v.s_nu = SA(0, 1); v.s_su = SA(0, -1);
    v.s_d = SC(0, 0); v.s_ed = SC(1, 0);
    v.g1c = XA(0, 0, 0); v.g1e = XA(0, 1, 0);
    v.g2c = XA(1, 0, 0); v.g2n = XA(1, 0, 1); v.g2wn = XA(1, -1, 1);
    v.g3c = ZB(0, 0, 0); v.g3u = ZA(0, 0, 0); v.g3wu = ZA(0, -1, 0);
    v.g4c = XA(2, 0, 0); v.g4e = XA(2, 1, 0); v.g4es = XA(2, 1, -1);
    v.g5c = XA(3, 0, 0); v.g5n = XA(3, 0, 1);
    v.g6c = ZB(1, 0, 0); v.g6u = ZA(1, 0, 0); v.g6su = ZA(1, 0, -1);
    v.g7c = ZA(3, 0, 0); v.g7e = ZA(3, 1, 0); v.g7ed = ZB(3, 1, 0);
    v.g8c = ZA(4, 0, 0); v.g8n = ZA(4, 0, 1); v.g8nd = ZB(4, 0, 1);
    v.g9c = ZB(2, 0, 0); v.g9u = ZA(2, 0, 0);
#undef SA
#undef SB
#undef SC
#undef ZA
#undef ZB
#undef XA
    v.f0 = S.c[0][xa][oc]; v.g0 = S.c[1][xa][oc]; v.h0 = S.c[2][xa][oc];
    float fo = 0.f, go = 0.f, ho = 0.f;
    if (AD) { fo = S.c[3][xa][oc]; go = S.c[4][xa][oc]; ho = S.c[5][xa][oc]; }
    v.ru = ru; v.rv = rv;
    float fv, gv, hv;
    unsigned bd = 0;
    visc_compute<P2, ZF>(d, v, cc, visc_z(d, k), k, fv, gv, hv, bd);
    // every thread is done with this step's reads: group t+1+VLA may take the slots they
    // used; a plane with a deferred cell is stored by the fixup
    const bool defer = ZF && __syncthreads_or(in ? bd : 0u);
    if (!ZF) __syncthreads();
    if (ty == 0) {  // warp 0 (uniform: issue holds a __syncwarp); none of it issues after a failed wait
      const bool wbad = __any_sync(0xffffffffu, bad);
      if (!wbad && t + 1 + VLA <= last_t) {
        issue(t + 1 + VLA);
        issued = t + 1 + VLA;
      }
    }
    if (defer) {
      if (tid == 0) {
        int *list = d.fix[FIX_VISC];
        const int s = atomicAdd(list, 1);
        list[2 + s] = (int)(((k - 1) * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x);
      }
    } else if (in) {
      visc_store<AD>(d, c, fv, gv, hv, fo, go, ho);
    }
    c += d.np;
    ru = 0.f;
    rv = 0.f;
  }
  // after a wait gave up, wait (bounded) for the copies this warp issued before leaving
  if (ty == 0 && bad)
    for (int t = waited + 1; t <= issued; ++t) (void)mbar_wait(&S.bar[t % NS], (uint32_t)((t / NS) & 1));
}


}  // namespace

#define LAUNCH(ctx, ...)                \
  do {                                  \
    __VA_ARGS__;                        \
    ++*(ctx).nlaunch;                   \
  } while (0)

namespace {
// Launch a fused kernel K<P2, ZF, X> for the domain's spacing modes; with ZF its fixup
// kernel F<P2, X> follows (it does nothing when no block was deferred).
template <template <bool, bool, bool> class K, template <bool, bool> class F, typename... Args>
void launch_variant(const LesDom &d, bool x, LesCtx ctx, dim3 g, dim3 b, Args... args) {
  const uint3 gu = make_uint3(g.x, g.y, g.z);
  const unsigned nfix = std::min<unsigned>(g.x * g.y * g.z, (unsigned)std::max(1, 2 * d.sms));
  const int v = (d.xy_pow2 ? 4 : 0) | (d.zfast ? 2 : 0) | (x ? 1 : 0);
  switch (v) {
    case 0: LAUNCH(ctx, (K<false, false, false>::fn<<<g, b, 0, ctx.s>>>(d, args...))); break;
    case 1: LAUNCH(ctx, (K<false, false, true>::fn<<<g, b, 0, ctx.s>>>(d, args...))); break;
    case 2: LAUNCH(ctx, (K<false, true, false>::fn<<<g, b, 0, ctx.s>>>(d, args...)));
            LAUNCH(ctx, (F<false, false>::fn<<<nfix, b, 0, ctx.s>>>(d, gu))); break;
    case 3: LAUNCH(ctx, (K<false, true, true>::fn<<<g, b, 0, ctx.s>>>(d, args...)));
            LAUNCH(ctx, (F<false, true>::fn<<<nfix, b, 0, ctx.s>>>(d, gu))); break;
    case 4: LAUNCH(ctx, (K<true, false, false>::fn<<<g, b, 0, ctx.s>>>(d, args...))); break;
    case 5: LAUNCH(ctx, (K<true, false, true>::fn<<<g, b, 0, ctx.s>>>(d, args...))); break;
    case 6: LAUNCH(ctx, (K<true, true, false>::fn<<<g, b, 0, ctx.s>>>(d, args...)));
            LAUNCH(ctx, (F<true, false>::fn<<<nfix, b, 0, ctx.s>>>(d, gu))); break;
    default: LAUNCH(ctx, (K<true, true, true>::fn<<<g, b, 0, ctx.s>>>(d, args...)));
             LAUNCH(ctx, (F<true, true>::fn<<<nfix, b, 0, ctx.s>>>(d, gu))); break;
  }
}
template <template <bool, bool, bool> class K, template <bool, bool> class F, typename... Args>
void launch_variant_smem(const LesDom &d, bool x, LesCtx ctx, dim3 g, dim3 b, size_t smem, Args... args) {
  const uint3 gu = make_uint3(g.x, g.y, g.z);
  const unsigned nfix = std::min<unsigned>(g.x * g.y * g.z, (unsigned)std::max(1, 2 * d.sms));
  const int v = (d.xy_pow2 ? 4 : 0) | (d.zfast ? 2 : 0) | (x ? 1 : 0);
  switch (v) {
    case 0: LAUNCH(ctx, (K<false, false, false>::fn<<<g, b, smem, ctx.s>>>(d, args...))); break;
    case 1: LAUNCH(ctx, (K<false, false, true>::fn<<<g, b, smem, ctx.s>>>(d, args...))); break;
    case 2: LAUNCH(ctx, (K<false, true, false>::fn<<<g, b, smem, ctx.s>>>(d, args...)));
            LAUNCH(ctx, (F<false, false>::fn<<<nfix, b, 0, ctx.s>>>(d, gu))); break;
    case 3: LAUNCH(ctx, (K<false, true, true>::fn<<<g, b, smem, ctx.s>>>(d, args...)));
            LAUNCH(ctx, (F<false, true>::fn<<<nfix, b, 0, ctx.s>>>(d, gu))); break;
    case 4: LAUNCH(ctx, (K<true, false, false>::fn<<<g, b, smem, ctx.s>>>(d, args...))); break;
    case 5: LAUNCH(ctx, (K<true, false, true>::fn<<<g, b, smem, ctx.s>>>(d, args...))); break;
    case 6: LAUNCH(ctx, (K<true, true, false>::fn<<<g, b, smem, ctx.s>>>(d, args...)));
            LAUNCH(ctx, (F<true, false>::fn<<<nfix, b, 0, ctx.s>>>(d, gu))); break;
    default: LAUNCH(ctx, (K<true, true, true>::fn<<<g, b, smem, ctx.s>>>(d, args...)));
             LAUNCH(ctx, (F<true, true>::fn<<<nfix, b, 0, ctx.s>>>(d, gu))); break;
  }
}
template <bool A, bool B, bool C>
struct VelfgK {
  static constexpr auto fn = k_velfg_march<A, B, C>;
};
template <bool A, bool C>
struct VelfgF {
  static constexpr auto fn = k_velfg_march_fix<A, C>;
};
template <bool A, bool B, bool C>
struct ViscK {
  static constexpr auto fn = k_les_visc_march<A, B, C>;
};
template <bool A, bool C>
struct ViscF {
  static constexpr auto fn = k_les_visc_fix<A, C>;
};
constexpr int kViscLookahead = 1;  // stages in flight beyond the three a step reads
constexpr int kSmLookahead = 1;    // copy groups in flight beyond the two a step of the sm pass reads
template <bool A, bool B, bool C>
struct ViscTmaK {
  static constexpr auto fn = k_les_visc_tma<A, B, C, kViscLookahead>;
};

// Tensor maps of the arrays the TMA-fed sm pass and viscous march read (sm, diu1..9 as
// halo boxes, f..hold as cell boxes), cached per domain layout (the maps hold only base
// addresses, extents and strides).
bool visc_maps(const LesDom &d, LesViscMaps *out) {
  static std::mutex mu;
  static std::map<std::vector<uintptr_t>, LesViscMaps> cache;
  const float *bases[16] = {d.sm, d.diu[1], d.diu[2], d.diu[3], d.diu[4], d.diu[5], d.diu[6], d.diu[7],
                            d.diu[8], d.diu[9], d.f, d.g, d.h, d.fold, d.gold, d.hold};
  std::vector<uintptr_t> key = {(uintptr_t)d.pi, (uintptr_t)d.nj, (uintptr_t)d.km};
  for (const float *b : bases) key.push_back((uintptr_t)b);
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(key);
  if (it != cache.end()) {
    *out = it->second;
    return true;
  }
  LesViscMaps m;
  for (int q = 0; q < 16; ++q) {
    if (!bases[q] || ((uintptr_t)bases[q] & 15u)) return false;
    if (les_tensor_map_3d(&m.m[q], d, bases[q], q < 10 ? VBW : VTX, q < 10 ? VTH : VTY) != 0) return false;
  }
  if (cache.size() >= 4096) cache.clear();
  cache.emplace(key, m);
  *out = m;
  return true;
}
}  // namespace

// Planes per block of the velfg march: chunks enough for about twelve blocks per SM,
// of 6 to 20 planes (a chunk re-forms the faces of its first plane).
static int velfg_kchunk(const LesDom &d) {
  if (const char *e = getenv("LES_VELFG_KCHUNK")) {  // A/B measurements
    const int v = atoi(e);
    if (v > 0) return std::min(v, d.km);
  }
  const long long tiles = (long long)((d.im + MTI - 1) / MTI) * ((d.jm + MTY - 1) / MTY);
  const int sms = d.sms > 0 ? d.sms : 152;
  const int nch = (int)std::max<long long>(1, (12LL * sms + tiles - 1) / tiles);
  const int kc = (d.km + nch - 1) / nch;
  return std::min(d.km, std::max(6, std::min(20, kc)));
}

void les_launch_velfg_fused(const LesDom &d, bool with_feedbf, LesCtx ctx) {
  LAUNCH(ctx, (k_wall<<<dim3((d.im + 127) / 128, d.jm), 128, 0, ctx.s>>>(d)));
  const int kc = velfg_kchunk(d);
  const dim3 g((d.im + MTI - 1) / MTI, (d.jm + MTY - 1) / MTY, (d.km + kc - 1) / kc);
  launch_variant<VelfgK, VelfgF>(d, with_feedbf, ctx, g, dim3(MTX, MTY), kc);
}

void les_launch_les_fused(const LesDom &d, bool with_adam, LesCtx ctx) {
  static const int kind = [] {  // LES_VISC_KIND=0: the register-staged sm pass and march (A/B measurements)
    const char *e = getenv("LES_VISC_KIND");
    return e ? atoi(e) : 1;
  }();
  LesViscMaps maps;
  const bool tma = kind != 0 && (d.pi * 4) % 16 == 0 && visc_maps(d, &maps);
  if (tma) {
    // the diu halo entries the TMA boxes read, then sm from the staged diu planes
    LAUNCH(ctx, (k_diu_halo<<<dim3((d.im + d.jm + 1 + 255) / 256, d.km + 1), 256, 0, ctx.s>>>(d)));
    LesSmMaps sm_maps;
    for (int q = 0; q < 9; ++q) sm_maps.m[q] = maps.m[q + 1];
    static const int kc_env = [] {  // LES_SM_KCHUNK: planes per CTA of the sm pass (A/B measurements)
      const char *e = getenv("LES_SM_KCHUNK");
      return e ? atoi(e) : 0;
    }();
    const int kc = std::max(1, std::min(d.km, kc_env > 0 ? kc_env : 15));  // 15 to 30 planes measured alike
    const size_t bytes = sizeof(SmSmem<kSmLookahead>);
    cudaFuncSetAttribute(k_les_sm_tma<kSmLookahead>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    const dim3 g((d.im + VTX - 1) / VTX, (d.jm + VTY - 1) / VTY, (d.km + kc - 1) / kc);
    LAUNCH(ctx, (k_les_sm_tma<kSmLookahead><<<g, dim3(VTX, VTY), bytes, ctx.s>>>(d, sm_maps, kc)));
  } else {  // sm: chunks of planes enough for about sixteen blocks per SM, 8 to 32 planes each
    const long long tiles = (long long)((d.im + STX - 1) / STX) * ((d.jm + STY - 1) / STY);
    const int sms = d.sms > 0 ? d.sms : 152;
    const int nch = (int)std::max<long long>(1, (16LL * sms + tiles - 1) / tiles);
    const int kc = std::min(d.km, std::max(8, std::min(32, (d.km + nch - 1) / nch)));
    const dim3 g((d.im + STX - 1) / STX, (d.jm + STY - 1) / STY, (d.km + kc - 1) / kc);
    LAUNCH(ctx, k_les_sm3<<<g, dim3(STX, STY), 0, ctx.s>>>(d, kc));
  }
  les_launch_boundsm(d, ctx);
  // the k-march: 32 x 8 column tiles, chunks of VKC planes; TMA-fed when the arrays'
  // tensor maps could be made (row pitch a multiple of 16 bytes), else register-staged
  const dim3 gv((d.im + VTX - 1) / VTX, (d.jm + VTY - 1) / VTY, (d.km + VKC - 1) / VKC);
  if (tma) {
    const size_t bytes = sizeof(ViscSmem<kViscLookahead>);
    const int v = (d.xy_pow2 ? 4 : 0) | (d.zfast ? 2 : 0) | (with_adam ? 1 : 0);
    auto set_attr = [&](const void *fn) {
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    };
    switch (v) {
      case 0: set_attr((const void *)ViscTmaK<false, false, false>::fn); break;
      case 1: set_attr((const void *)ViscTmaK<false, false, true>::fn); break;
      case 2: set_attr((const void *)ViscTmaK<false, true, false>::fn); break;
      case 3: set_attr((const void *)ViscTmaK<false, true, true>::fn); break;
      case 4: set_attr((const void *)ViscTmaK<true, false, false>::fn); break;
      case 5: set_attr((const void *)ViscTmaK<true, false, true>::fn); break;
      case 6: set_attr((const void *)ViscTmaK<true, true, false>::fn); break;
      default: set_attr((const void *)ViscTmaK<true, true, true>::fn); break;
    }
    launch_variant_smem<ViscTmaK, ViscF>(d, with_adam, ctx, gv, dim3(VTX, VTY), bytes, maps);
    return;
  }
  launch_variant<ViscK, ViscF>(d, with_adam, ctx, gv, dim3(VTX, VTY));
}
