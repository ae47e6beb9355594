// les_kernels.cu -- per-subroutine kernels of the MPI-LES solver (sm_103a).
//
// One kernel (or a short fixed sequence of small kernels) per reference subroutine,
// each a drop-in for that subroutine on device-resident state.  These are the
// building blocks behind the per-subroutine C-ABI entry points; the whole-step path
// uses the fused kernels of les_fused.cu and les_sor.cu instead.
//
// Exactness: every interior update is an independent function of values no other
// thread of the same launch writes, so a one-thread-per-cell launch reproduces the
// reference's sequential loops bit for bit.  Halo fills that the reference runs as
// ordered loops run as ordered launches.  Sums (uout max/min, rhsav, pav, the SOR
// residual) are per-domain deterministic reductions: FP64 where the reference sums
// many FP32 terms.
#include <cuda_runtime.h>

#include "les_common.cuh"
#include "les_kernels.cuh"

namespace {

constexpr int BX = 64, BY = 4;

inline dim3 interior_grid(const LesDom &d, int kn) {
  return dim3((d.im + BX - 1) / BX, (d.jm + BY - 1) / BY, kn);
}

#define INTERIOR_IJK                                  \
  const int i = blockIdx.x * BX + threadIdx.x + 1;    \
  const int j = blockIdx.y * BY + threadIdx.y + 1;    \
  const int k = blockIdx.z + 1;                       \
  if (i > d.im || j > d.jm) return;

// ------------------------------------------------------------------ velnw.f95:27-59
__global__ void __launch_bounds__(BX *BY) k_velnw(LesDom d) {
  INTERIOR_IJK
  const int c = lix(d, i, j, k);
  const float pc = d.p[c];
  float pz = (-pc + d.p[c + 1]) / d.ro / d.gr.dxs[i];
  d.u[c] = d.u[c] + d.dt * (d.f[c] - pz);
  pz = (-pc + d.p[c + d.pi]) / d.ro / d.gr.dys[j];
  d.v[c] = d.v[c] + d.dt * (d.g[c] - pz);
  if (k <= d.km - 1) {
    pz = (-pc + d.p[c + d.np]) / d.ro / d.gr.dzs[k];
    d.w[c] = d.w[c] + d.dt * (d.h[c] - pz);
  }
}

// ------------------------------------------------------------------ bondv1.f95
// inflow planes i = 0,1 (bondv1.f95:33-54, the profile given by the scenario)
__global__ void k_bondv1_inflow(LesDom d) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int k = blockIdx.y + 1;
  if (j > d.jm) return;
  const int q = (j - 1) + (k - 1) * d.jm;
  const float a = d.uin[q], b = d.vin[q], c = d.win[q];
  for (int i = 0; i <= 1; ++i) {
    const int x = lix(d, i, j, k);
    d.u[x] = a; d.v[x] = b; d.w[x] = c;
  }
}
// n == 1 initial fill, i = 2..im (bondv1.f95:152-160)
__global__ void __launch_bounds__(BX *BY) k_bondv1_fill(LesDom d) {
  const int i = blockIdx.x * BX + threadIdx.x + 2;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > d.im || j > d.jm) return;
  const int x = lix(d, i, j, k), x1 = lix(d, 1, j, k);
  d.u[x] = d.u[x1]; d.v[x] = d.v[x1]; d.w[x] = d.w[x1];
}
// uout = (max(0, max u(im)) + min(0, min u(im)))/2 (bondv1.f95:171-187); one block.
__global__ void __launch_bounds__(1024) k_bondv1_uout(LesDom d) {
  __shared__ float smax[32], smin[32];
  float aaa = 0.f, bbb = 0.f;
  const int n = d.jm * d.km;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int j = q % d.jm + 1, k = q / d.jm + 1;
    const float x = U_(d.im, j, k);
    aaa = fmaxf(aaa, x);
    bbb = fminf(bbb, x);
  }
  for (int o = 16; o > 0; o >>= 1) {
    aaa = fmaxf(aaa, __shfl_down_sync(0xffffffffu, aaa, o));
    bbb = fminf(bbb, __shfl_down_sync(0xffffffffu, bbb, o));
  }
  if ((threadIdx.x & 31) == 0) { smax[threadIdx.x >> 5] = aaa; smin[threadIdx.x >> 5] = bbb; }
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.f, b = 0.f;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { a = fmaxf(a, smax[q]); b = fminf(b, smin[q]); }
    const float uout = (a + b) / 2.f;
    d.fscal[SC_UOUT] = uout;
    d.scal[SC_UOUT] = (double)uout;
  }
}
// advective outflow (bondv1.f95:191-207)
__global__ void k_bondv1_outflow(LesDom d) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int k = blockIdx.y + 1;
  if (j > d.jm) return;
  const float uout = d.fscal[SC_UOUT];
  const float rdx = d.gr.dxs[d.im];
  const int c = lix(d, d.im, j, k), c2 = c + 1;
  d.u[c] = d.u[c] - d.dt * uout * (d.u[c] - d.u[c - 1]) / rdx;
  d.v[c2] = d.v[c2] - d.dt * uout * (d.v[c2] - d.v[c]) / rdx;
  d.w[c2] = d.w[c2] - d.dt * uout * (d.w[c2] - d.w[c]) / rdx;
}
// periodic side flow, k = 0..km+1 (w: 0..km), i = 0..im+1 (bondv1.f95:210-229)
__global__ void k_bondv1_periodic(LesDom d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (i > d.im + 1) return;
  const int r0 = lix(d, i, 0, k), rj = lix(d, i, d.jm, k), r1 = lix(d, i, 1, k), rj1 = lix(d, i, d.jm + 1, k);
  d.u[r0] = d.u[rj]; d.u[rj1] = d.u[r1];
  d.v[r0] = d.v[rj]; d.v[rj1] = d.v[r1];
  if (k <= d.km) { d.w[r0] = d.w[rj]; d.w[rj1] = d.w[r1]; }
}
// top and underground (bondv1.f95:249-268)
__global__ void k_bondv1_topbottom(LesDom d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y - 1;
  if (i > d.im + 1) return;
  if (j >= 0) {
    const int b0 = lix(d, i, j, 0), b1 = lix(d, i, j, 1), tk = lix(d, i, j, d.km), tk1 = lix(d, i, j, d.km + 1);
    d.u[b0] = -d.u[b1]; d.u[tk1] = d.u[tk];
    d.v[b0] = -d.v[b1]; d.v[tk1] = d.v[tk];
  }
  d.w[lix(d, i, j, 0)] = 0.f;
  d.w[lix(d, i, j, d.km)] = 0.f;
}

// ------------------------------------------------------------------ velFG.f95:64-110
__global__ void __launch_bounds__(BX *BY) k_velfg(LesDom d) {
  INTERIOR_IJK
  const float *dx1 = d.gr.dx1, *dy1 = d.gr.dy1, *dzn = d.gr.dzn, *dzs = d.gr.dzs;
  const int c = lix(d, i, j, k);
  {  // u
    const float covx1 = (dx1[i + 1] * cov1(d, i, j, k) + dx1[i] * cov1(d, i + 1, j, k)) / (dx1[i] + dx1[i + 1]);
    const float covy1 = (cov2(d, i, j, k) + cov2(d, i, j + 1, k)) / 2.f;
    const float covz1 = (cov3(d, i, j, k) + cov3(d, i, j, k + 1)) / 2.f;
    const float covc = covx1 + covy1 + covz1;
    const float dfu1 = 2.f * (-diu1(d, i, j, k) + diu1(d, i + 1, j, k)) / (dx1[i] + dx1[i + 1]) +
                       (-diu2(d, i, j, k) + diu2(d, i, j + 1, k)) / dy1[j] +
                       (-diu3(d, i, j, k) + diu3(d, i, j, k + 1)) / dzn[k];
    const float df = d.vn * dfu1;
    d.f[c] = (-covc + df);
  }
  {  // v
    const float covx1 = (cov4(d, i, j, k) + cov4(d, i + 1, j, k)) / 2.f;
    const float covy1 = (dy1[j + 1] * cov5(d, i, j, k) + dy1[j] * cov5(d, i, j + 1, k)) / (dy1[j] + dy1[j + 1]);
    const float covz1 = (cov6(d, i, j, k) + cov6(d, i, j, k + 1)) / 2.f;
    const float covc = covx1 + covy1 + covz1;
    const float dfv1 = (-diu4(d, i, j, k) + diu4(d, i + 1, j, k)) / dx1[i] +
                       2.f * (-diu5(d, i, j, k) + diu5(d, i, j + 1, k)) / (dy1[j] + dy1[j + 1]) +
                       (-diu6(d, i, j, k) + diu6(d, i, j, k + 1)) / dzn[k];
    const float df = d.vn * dfv1;
    d.g[c] = (-covc + df);
  }
  if (k <= d.km - 1) {  // w
    const float covx1 = (cov7(d, i, j, k) + cov7(d, i + 1, j, k)) / 2.f;
    const float covy1 = (cov8(d, i, j, k) + cov8(d, i, j + 1, k)) / 2.f;
    const float covz1 = (dzn[k + 1] * cov9(d, i, j, k) + dzn[k] * cov9(d, i, j, k + 1)) / (dzn[k] + dzn[k + 1]);
    const float covc = covx1 + covy1 + covz1;
    const float dfw1 = (-diu7(d, i, j, k) + diu7(d, i + 1, j, k)) / dx1[i] +
                       (-diu8(d, i, j, k) + diu8(d, i, j + 1, k)) / dy1[j] +
                       (-diu9(d, i, j, k) + diu9(d, i, j, k + 1)) / dzs[k];
    const float df = d.vn * dfw1;
    d.h[c] = (-covc + df);
  }
}

// ------------------------------------------------------------------ feedbf.f95:35-61
__global__ void __launch_bounds__(BX *BY) k_feedbf(LesDom d) {
  INTERIOR_IJK
  const int c = lix(d, i, j, k);
  const uint8_t m = d.mask[c];
  const float bm = (m & 1) ? 1.f : 0.f, cm = (m & 2) ? 1.f : 0.f, dm = (m & 4) ? 1.f : 0.f;
  const float u = d.u[c], v = d.v[c], w = d.w[c];
  const float us = (d.usum[c] + u) * bm;
  const float vs = (d.vsum[c] + v) * cm;
  const float ws = (d.wsum[c] + w) * dm;
  d.usum[c] = us; d.vsum[c] = vs; d.wsum[c] = ws;
  const float fx = d.alpha * us * d.dt + d.beta * u * bm;
  const float fy = d.alpha * vs * d.dt + d.beta * v * cm;
  const float fz = d.alpha * ws * d.dt + d.beta * w * dm;
  d.f[c] = d.f[c] + fx;
  d.g[c] = d.g[c] + fy;
  d.h[c] = d.h[c] + fz;
}

// ------------------------------------------------------------------ les.f95:45-65
__global__ void __launch_bounds__(BX *BY) k_les_sm(LesDom d) {
  INTERIOR_IJK
  const float dudxx1 = diu1(d, i, j, k);
  const float dudyx1 = (diu2(d, i - 1, j, k) + diu2(d, i - 1, j + 1, k) + diu2(d, i, j, k) + diu2(d, i, j + 1, k)) * .25f;
  const float dudzx1 = (diu3(d, i - 1, j, k) + diu3(d, i - 1, j, k + 1) + diu3(d, i, j, k) + diu3(d, i, j, k + 1)) * .25f;
  const float dvdxx1 = (diu4(d, i, j, k) + diu4(d, i, j - 1, k) + diu4(d, i + 1, j, k) + diu4(d, i + 1, j - 1, k)) * .25f;
  const float dvdyx1 = diu5(d, i, j, k);
  const float dvdzx1 = (diu6(d, i, j - 1, k) + diu6(d, i, j - 1, k + 1) + diu6(d, i, j, k) + diu6(d, i, j, k + 1)) * .25f;
  const float dwdxx1 = (diu7(d, i, j, k) + diu7(d, i, j, k - 1) + diu7(d, i + 1, j, k) + diu7(d, i + 1, j, k - 1)) * .25f;
  const float dwdyx1 = (diu8(d, i, j, k) + diu8(d, i, j, k - 1) + diu8(d, i, j + 1, k) + diu8(d, i, j + 1, k - 1)) * .25f;
  const float dwdzx1 = diu9(d, i, j, k);
  const float cd = 0.1f * d.gr.delx1[k];
  const float s1 = dudyx1 + dvdxx1, s2 = dwdyx1 + dvdzx1, s3 = dudzx1 + dwdxx1;
  d.sm[lix(d, i, j, k)] =
      cd * cd * __fsqrt_rn(2.f * (dudxx1 * dudxx1 + dvdyx1 * dvdyx1 + dwdzx1 * dwdzx1) + s1 * s1 + s2 * s2 + s3 * s3);
}
// boundsm.f95:18-64, three ordered phases
__global__ void k_boundsm_i(LesDom d) {  // j = -1..jm+1, k = 0..km+1
  const int j = blockIdx.x * blockDim.x + threadIdx.x - 1;
  const int k = blockIdx.y;
  if (j > d.jm + 1) return;
  d.sm[lix(d, 0, j, k)] = d.sm[lix(d, 1, j, k)];
  d.sm[lix(d, d.im + 1, j, k)] = d.sm[lix(d, d.im, j, k)];
}
__global__ void k_boundsm_j(LesDom d) {  // i = 0..im+1, k = 0..km+1
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (i > d.im + 1) return;
  d.sm[lix(d, i, d.jm + 1, k)] = d.sm[lix(d, i, d.jm, k)];
  d.sm[lix(d, i, 0, k)] = d.sm[lix(d, i, 1, k)];
}
__global__ void k_boundsm_k(LesDom d) {  // i = 0..im+1, j = -1..jm+1
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y - 1;
  if (i > d.im + 1) return;
  d.sm[lix(d, i, j, 0)] = -d.sm[lix(d, i, j, 1)];
  d.sm[lix(d, i, j, d.km + 1)] = d.sm[lix(d, i, j, d.km)];
}

#define SM_(i, j, k) d.sm[lix(d, (i), (j), (k))]

// viscous terms of f, g, h (les.f95:83-242), with the k = 1 wall functions
__global__ void __launch_bounds__(BX *BY) k_les_visc(LesDom d) {
  INTERIOR_IJK
  const float *dx1 = d.gr.dx1, *dy1 = d.gr.dy1, *dzn = d.gr.dzn, *dxs = d.gr.dxs, *dys = d.gr.dys;
  const int c = lix(d, i, j, k);
  const float dxa = dx1[i] + dx1[i + 1];
  const float dxb = dx1[i - 1] + dx1[i];
  const float dya = dy1[j] + dy1[j + 1];
  // x component
  {
    const float evsx2 = SM_(i + 1, j, k);
    const float evsx1 = SM_(i, j, k);
    const float evsy2 = (dy1[j + 1] * ((dx1[i + 1] * SM_(i, j, k) + dx1[i] * SM_(i + 1, j, k)) / dxa) +
                         dy1[j] * ((dx1[i + 1] * SM_(i, j + 1, k) + dx1[i] * SM_(i + 1, j + 1, k)) / dxa)) / dya;
    const float evsy1 = (dy1[j + 1] * ((dx1[i + 1] * SM_(i, j - 1, k) + dx1[i] * SM_(i + 1, j - 1, k)) / dxa) +
                         dy1[j] * ((dx1[i + 1] * SM_(i, j, k) + dx1[i] * SM_(i + 1, j, k)) / dxa)) / dya;
    float vfu;
    if (k >= 2) {
      const float evsz2 = (dzn[k + 1] * ((dx1[i + 1] * SM_(i, j, k) + dx1[i] * SM_(i + 1, j, k)) / dxa) +
                           dzn[k] * ((dx1[i + 1] * SM_(i, j, k + 1) + dx1[i] * SM_(i + 1, j, k + 1)) / dxa)) /
                          (dzn[k] + dzn[k + 1]);
      const float evsz1 = (dzn[k] * ((dx1[i + 1] * SM_(i, j, k - 1) + dx1[i] * SM_(i + 1, j, k - 1)) / dxa) +
                           dzn[k - 1] * ((dx1[i + 1] * SM_(i, j, k) + dx1[i] * SM_(i + 1, j, k)) / dxa)) /
                          (dzn[k - 1] + dzn[k]);
      const float visux2 = (evsx2) * 2.f * diu1(d, i + 1, j, k);
      const float visux1 = (evsx1) * 2.f * diu1(d, i, j, k);
      const float visuy2 = (evsy2) * (diu2(d, i, j + 1, k) + diu4(d, i + 1, j, k));
      const float visuy1 = (evsy1) * (diu2(d, i, j, k) + diu4(d, i + 1, j - 1, k));
      const float visuz2 = (evsz2) * (diu3(d, i, j, k + 1) + diu7(d, i + 1, j, k));
      const float visuz1 = (evsz1) * (diu3(d, i, j, k) + diu7(d, i + 1, j, k - 1));
      vfu = (visux2 - visux1) / dxs[i] + (visuy2 - visuy1) / dy1[j] + (visuz2 - visuz1) / dzn[k];
    } else {  // wall function (les.f95:118-139): y and z terms appear twice, as written
      const float evsz2 = (dzn[2] * ((dx1[i + 1] * SM_(i, j, 1) + dx1[i] * SM_(i + 1, j, 1)) / dxa) +
                           dzn[1] * ((dx1[i + 1] * SM_(i, j, 2) + dx1[i] * SM_(i + 1, j, 2)) / dxa)) /
                          (dzn[1] + dzn[2]);
      const float visux2 = (evsx2) * 2.f * diu1(d, i + 1, j, 1);
      const float visux1 = (evsx1) * 2.f * diu1(d, i, j, 1);
      const float visuy2 = (evsy2) * (diu2(d, i, j + 1, 1) + diu4(d, i + 1, j, 1));
      const float visuy1 = (evsy1) * (diu2(d, i, j, 1) + diu4(d, i + 1, j - 1, 1));
      const float visuz2 = (evsz2) * (diu3(d, i, j, 2) + diu7(d, i + 1, j, 1));
      const float r = U_(i, j, 1) / uspd_raw(d, i, j);  // uspd after vel2.f95:353
      const float t = 0.4f * r / d.logz;
      const float visuz1 = t * t * r;
      vfu = (visux2 - visux1) / dxs[i] + (visuy2 - visuy1) / dy1[j] + (visuz2 - visuz1) / dzn[1] +
            (visuy2 - visuy1) / dy1[j] + (visuz2 - visuz1) / dzn[1];
    }
    d.f[c] = (d.f[c] + vfu);
  }
  // y component
  {
    const float evsy2 = SM_(i, j + 1, k);
    const float evsy1 = SM_(i, j, k);
    const float evsx2 = (dy1[j + 1] * ((dx1[i + 1] * SM_(i, j, k) + dx1[i] * SM_(i + 1, j, k)) / dxa) +
                         dy1[j] * ((dx1[i + 1] * SM_(i, j + 1, k) + dx1[i] * SM_(i + 1, j + 1, k)) / dxa)) / dya;
    const float evsx1 = (dy1[j + 1] * ((dx1[i] * SM_(i - 1, j, k) + dx1[i - 1] * SM_(i, j, k)) / dxb) +
                         dy1[j] * ((dx1[i] * SM_(i - 1, j + 1, k) + dx1[i - 1] * SM_(i, j + 1, k)) / dxb)) / dya;
    float vfv;
    if (k >= 2) {
      const float evsz2 = (dzn[k + 1] * ((dx1[i + 1] * SM_(i, j, k) + dx1[i] * SM_(i + 1, j, k)) / dxa) +
                           dzn[k] * ((dx1[i + 1] * SM_(i, j, k + 1) + dx1[i] * SM_(i + 1, j, k + 1)) / dxa)) /
                          (dzn[k] + dzn[k + 1]);
      const float evsz1 = (dzn[k] * ((dx1[i + 1] * SM_(i, j, k - 1) + dx1[i] * SM_(i + 1, j, k - 1)) / dxa) +
                           dzn[k - 1] * ((dx1[i + 1] * SM_(i, j, k) + dx1[i] * SM_(i + 1, j, k)) / dxa)) /
                          (dzn[k - 1] + dzn[k]);
      const float visvx2 = (evsx2) * (diu2(d, i, j + 1, k) + diu4(d, i + 1, j, k));
      const float visvx1 = (evsx1) * (diu2(d, i - 1, j + 1, k) + diu4(d, i, j, k));
      const float visvy2 = (evsy2) * 2.f * diu5(d, i, j + 1, k);
      const float visvy1 = (evsy1) * 2.f * diu5(d, i, j, k);
      const float visvz2 = (evsz2) * (diu6(d, i, j, k + 1) + diu8(d, i, j + 1, k));
      const float visvz1 = (evsz1) * (diu6(d, i, j, k) + diu8(d, i, j + 1, k - 1));
      vfv = (visvx2 - visvx1) / dx1[i] + (visvy2 - visvy1) / dys[j] + (visvz2 - visvz1) / dzn[k];
    } else {  // wall function (les.f95:178-201)
      const float evsz2 = (dzn[2] * ((dx1[i + 1] * SM_(i, j, 1) + dx1[i] * SM_(i + 1, j, 1)) / dxa) +
                           dzn[1] * ((dx1[i + 1] * SM_(i, j, 2) + dx1[i] * SM_(i + 1, j, 2)) / dxa)) /
                          (dzn[1] + dzn[2]);
      const float visvx2 = (evsx2) * (diu2(d, i, j + 1, 1) + diu4(d, i + 1, j, 1));
      const float visvx1 = (evsx1) * (diu2(d, i - 1, j + 1, 1) + diu4(d, i, j, 1));
      const float visvy2 = (evsy2) * 2.f * diu5(d, i, j + 1, 1);
      const float visvy1 = (evsy1) * 2.f * diu5(d, i, j, 1);
      const float visvz2 = (evsz2) * (diu6(d, i, j, 2) + diu8(d, i, j + 1, 1));
      const float r = V_(i, j, 1) / vspd_raw(d, i, j);  // vspd after vel2.f95:354
      const float t = 0.4f * r / d.logz;
      const float visvz1 = t * t * r;
      vfv = (visvx2 - visvx1) / dx1[i] + (visvy2 - visvy1) / dys[j] + (visvz2 - visvz1) / dzn[1];
    }
    d.g[c] = (d.g[c] + vfv);
  }
  // z component, k = 1..km
  {
    const float dzc = dzn[k] + dzn[k + 1];
    const float evsz2 = SM_(i, j, k + 1);
    const float evsz1 = SM_(i, j, k);
    const float evsx2 = (dzn[k + 1] * ((dx1[i + 1] * SM_(i, j, k) + dx1[i] * SM_(i + 1, j, k)) / dxa) +
                         dzn[k] * ((dx1[i + 1] * SM_(i, j, k + 1) + dx1[i] * SM_(i + 1, j, k + 1)) / dxa)) / dzc;
    const float evsx1 = (dzn[k + 1] * ((dx1[i] * SM_(i - 1, j, k) + dx1[i - 1] * SM_(i, j, k)) / dxb) +
                         dzn[k] * ((dx1[i] * SM_(i - 1, j, k + 1) + dx1[i - 1] * SM_(i, j, k + 1)) / dxb)) / dzc;
    const float evsy2 = (dzn[k + 1] * ((dy1[j + 1] * SM_(i, j, k) + dy1[j] * SM_(i, j + 1, k)) / dya) +
                         dzn[k] * ((dy1[j + 1] * SM_(i, j, k + 1) + dy1[j] * SM_(i, j + 1, k + 1)) / dya)) / dzc;
    const float dyb = dy1[j - 1] + dy1[j];
    const float evsy1 = (dzn[k + 1] * ((dy1[j] * SM_(i, j - 1, k) + dy1[j - 1] * SM_(i, j, k)) / dyb) +
                         dzn[k] * ((dy1[j] * SM_(i, j - 1, k + 1) + dy1[j - 1] * SM_(i, j, k + 1)) / dyb)) / dzc;
    const float viswx2 = (evsx2) * (diu3(d, i, j, k + 1) + diu7(d, i + 1, j, k));
    const float viswx1 = (evsx1) * (diu3(d, i - 1, j, k + 1) + diu7(d, i, j, k));
    const float viswy2 = (evsy2) * (diu6(d, i, j, k + 1) + diu8(d, i, j + 1, k));
    const float viswy1 = (evsy1) * (diu6(d, i, j - 1, k + 1) + diu8(d, i, j, k));
    const float viswz2 = (evsz2) * 2.f * diu9(d, i, j, k + 1);
    const float viswz1 = (evsz1) * 2.f * diu9(d, i, j, k);
    const float vfw = (viswx2 - viswx1) / dx1[i] + (viswy2 - viswy1) / dy1[j] + (viswz2 - viswz1) / dzn[k];
    d.h[c] = (d.h[c] + vfw);
  }
}

// ------------------------------------------------------------------ adam.f95:30-44
__global__ void __launch_bounds__(BX *BY) k_adam(LesDom d) {
  INTERIOR_IJK
  const int c = lix(d, i, j, k);
  const float fd = d.f[c], gd = d.g[c], hd = d.h[c];
  d.f[c] = 1.5f * fd - 0.5f * d.fold[c];
  d.g[c] = 1.5f * gd - 0.5f * d.gold[c];
  d.h[c] = 1.5f * hd - 0.5f * d.hold[c];
  d.fold[c] = fd; d.gold[c] = gd; d.hold[c] = hd;
}

// ------------------------------------------------------------------ bondFG.f95:18-42
__global__ void k_bondfg(LesDom d) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int n1 = d.jm * d.km, n2 = d.im * d.km, n3 = d.im * d.jm;
  if (t < n1) {
    const int j = t % d.jm + 1, k = t / d.jm + 1;
    d.f[lix(d, 0, j, k)] = d.f[lix(d, 1, j, k)];
  } else if (t < n1 + n2) {
    const int q = t - n1, i = q % d.im + 1, k = q / d.im + 1;
    d.g[lix(d, i, 0, k)] = d.g[lix(d, i, d.jm, k)];
  } else if (t < n1 + n2 + n3) {
    const int q = t - n1 - n2, i = q % d.im + 1, j = q / d.im + 1;
    d.h[lix(d, i, j, 0)] = 0.f;
    d.h[lix(d, i, j, d.km)] = 0.f;
  }
}

// ------------------------------------------------------------------ press.f95:49-60
// rhs, plus the FP64 block partials of sum(dx1*dy1*dzn*rhs) (press.f95:63-72)
// dst: the rhs array (rhs = d.rhs) or the SOR's internal rhs buffer, which also takes
// periodic ghost copies of rows 1, 2, jm-1, jm in rows jm+1, jm+2, -1, 0.
__global__ void __launch_bounds__(BX *BY) k_rhs(LesDom d, float *dst, int ghost) {
  __shared__ double sh[32];
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  double term = 0.0;
  if (i <= d.im && j <= d.jm) {
    const float *dx1 = d.gr.dx1, *dy1 = d.gr.dy1, *dzn = d.gr.dzn;
    const int c = lix(d, i, j, k);
    const float r = (-d.u[c - 1] + d.u[c]) / dx1[i] + (-d.v[c - d.pi] + d.v[c]) / dy1[j] +
                    (-d.w[c - d.np] + d.w[c]) / dzn[k];
    const float rr = (d.f[c] - d.f[c - 1]) / dx1[i] + (d.g[c] - d.g[c - d.pi]) / dy1[j] +
                     (d.h[c] - d.h[c - d.np]) / dzn[k] + r / d.dt;
    dst[c] = rr;
    if (ghost) {
      if (j == 1) dst[lix(d, i, d.jm + 1, k)] = rr;
      if (j == 2) dst[lix(d, i, d.jm + 2, k)] = rr;
      if (j == d.jm - 1) dst[lix(d, i, -1, k)] = rr;
      if (j == d.jm) dst[lix(d, i, 0, k)] = rr;
    }
    term = (double)(dx1[i] * dy1[j] * dzn[k] * rr);
  }
  const int tid = threadIdx.y * BX + threadIdx.x;
  double x = term;
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  if ((tid & 31) == 0) sh[tid >> 5] = x;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int q = 0; q < BX * BY / 32; ++q) s += sh[q];
    d.part[(blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = s;
  }
}
// pav partials: sum(p*dx1*dy1*dzn) (press.f95:124-133)
__global__ void __launch_bounds__(BX *BY) k_pav_part(LesDom d) {
  __shared__ double sh[32];
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  double term = 0.0;
  if (i <= d.im && j <= d.jm) {
    term = (double)(d.p[lix(d, i, j, k)] * d.gr.dx1[i] * d.gr.dy1[j] * d.gr.dzn[k]);
  }
  const int tid = threadIdx.y * BX + threadIdx.x;
  double x = term;
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  if ((tid & 31) == 0) sh[tid >> 5] = x;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int q = 0; q < BX * BY / 32; ++q) s += sh[q];
    d.part[(blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = s;
  }
}
// mean = (float)(sum of partials / area); one block, fixed order
__global__ void __launch_bounds__(1024) k_finish_mean(LesDom d, int nparts, int slot) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int q = threadIdx.x; q < nparts; q += blockDim.x) s += d.part[q];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sh[q];
    const float mean = (float)(t / d.scal[SC_AREA]);
    d.fscal[slot] = mean;
    d.scal[slot] = (double)mean;
  }
}
__global__ void __launch_bounds__(BX *BY) k_sub_mean(LesDom d, float *a, int slot) {
  INTERIOR_IJK
  const int c = lix(d, i, j, k);
  a[c] = a[c] - d.fscal[slot];
}

// ------------------------------------------------------------------ press.f95:89-122
__global__ void k_sor_begin(LesDom d) {
  d.ctl[CT_CONVERGED] = 0;
  d.ctl[CT_ITERS] = 0;
}
// one colour of one SOR iteration: nrd = 0 updates i+j+k odd, nrd = 1 even
__global__ void __launch_bounds__(BX *BY) k_sor_colour(LesDom d, int nrd, int nblk) {
  __shared__ double sh[32];
  if (d.ctl[CT_CONVERGED]) return;
  const int t = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  const int i = 1 + ((k + j + nrd) & 1) + 2 * t;
  float r2 = 0.f;
  if (i <= d.im && j <= d.jm) {
    const int c = lix(d, i, j, k);
    const float *p = d.p;
    float cn1;
    if (d.cn1) cn1 = d.cn1[(i - 1) + (j - 1) * d.im + (k - 1) * d.im * d.jm];
    else if (d.gr.cn1k) cn1 = d.gr.cn1k[k];
    else cn1 = 1.f / (d.gr.cn1a[i] + d.gr.cn1b[j] + d.gr.cn1c[k]);
    const float reltmp =
        d.omega * (cn1 * (d.gr.cn2l[i] * p[c + 1] + d.gr.cn2s[i] * p[c - 1] + d.gr.cn3l[j] * p[c + d.pi] +
                          d.gr.cn3s[j] * p[c - d.pi] + d.gr.cn4l[k] * p[c + d.np] + d.gr.cn4s[k] * p[c - d.np] -
                          d.rhs[c]) -
                   p[c]);
    d.p[c] = p[c] + reltmp;
    r2 = reltmp * reltmp;
  }
  const int tid = threadIdx.y * BX + threadIdx.x;
  for (int o = 16; o > 0; o >>= 1) r2 += __shfl_down_sync(0xffffffffu, r2, o);
  if ((tid & 31) == 0) sh[tid >> 5] = (double)r2;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int q = 0; q < BX * BY / 32; ++q) s += sh[q];
    d.part[nrd * nblk + (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = s;
  }
}
// boundp1 phase 1: i halos for j = 0..jm+1, k = 0..km+1 (boundp.f95:44-58)
__global__ void k_boundp1_i(LesDom d, int obey) {
  if (obey && d.ctl[CT_CONVERGED]) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (j > d.jm + 1) return;
  d.p[lix(d, 0, j, k)] = d.p[lix(d, 1, j, k)];
  d.p[lix(d, d.im + 1, j, k)] = d.p[lix(d, d.im, j, k)];
}
// boundp1 phase 2: periodic j halos for i = 0..im+1, k = 0..km+1 (boundp.f95:64-69)
__global__ void k_boundp1_j(LesDom d, int obey) {
  if (obey && d.ctl[CT_CONVERGED]) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (i > d.im + 1) return;
  d.p[lix(d, i, 0, k)] = d.p[lix(d, i, d.jm, k)];
  d.p[lix(d, i, d.jm + 1, k)] = d.p[lix(d, i, 1, k)];
}
// boundp2: k halos for i = 0..im+1, j = 0..jm+1 (boundp.f95:16-21)
__global__ void k_boundp2(LesDom d, int obey) {
  if (obey && d.ctl[CT_CONVERGED]) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i > d.im + 1) return;
  d.p[lix(d, i, j, 0)] = d.p[lix(d, i, j, 1)];
  d.p[lix(d, i, j, d.km + 1)] = d.p[lix(d, i, j, d.km)];
}
// end of one SOR iteration: residual sum, iteration count, convergence test
__global__ void __launch_bounds__(1024) k_sor_check(LesDom d, int nparts) {
  __shared__ double sh[32];
  if (d.ctl[CT_CONVERGED]) return;
  double s = 0.0;
  for (int q = threadIdx.x; q < nparts; q += blockDim.x) s += d.part[q];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sh[q];
    d.scal[SC_SOR] = t;
    d.ctl[CT_ITERS] += 1;
    if (!d.sor_fixed && t < (double)d.pjuge) d.ctl[CT_CONVERGED] = 1;
  }
}

// non-finite detector over the interior of u, v, w, p
__global__ void __launch_bounds__(BX *BY) k_count_nonfinite(LesDom d, unsigned long long *bad) {
  INTERIOR_IJK
  const int c = lix(d, i, j, k);
  int nb = 0;
  nb += !isfinite(d.u[c]);
  nb += !isfinite(d.v[c]);
  nb += !isfinite(d.w[c]);
  nb += !isfinite(d.p[c]);
  if (nb) atomicAdd(bad, (unsigned long long)nb);
}

}  // namespace

// =========================================================================== launchers
#define LAUNCH(ctx, ...)                \
  do {                                  \
    __VA_ARGS__;                        \
    ++*(ctx).nlaunch;                   \
  } while (0)

void les_launch_velnw(const LesDom &d, LesCtx ctx) {
  LAUNCH(ctx, k_velnw<<<interior_grid(d, d.km), dim3(BX, BY), 0, ctx.s>>>(d));
}

void les_launch_bondv1(const LesDom &d, int n, LesCtx ctx) {
  LAUNCH(ctx, k_bondv1_inflow<<<dim3((d.jm + 127) / 128, d.km), 128, 0, ctx.s>>>(d));
  if (n == 1) {
    LAUNCH(ctx, k_bondv1_fill<<<dim3((d.im - 1 + BX - 1) / BX, (d.jm + BY - 1) / BY, d.km), dim3(BX, BY), 0, ctx.s>>>(d));
  }
  LAUNCH(ctx, k_bondv1_uout<<<1, 1024, 0, ctx.s>>>(d));
  LAUNCH(ctx, k_bondv1_outflow<<<dim3((d.jm + 127) / 128, d.km), 128, 0, ctx.s>>>(d));
  LAUNCH(ctx, k_bondv1_periodic<<<dim3((d.im + 2 + 127) / 128, d.km + 2), 128, 0, ctx.s>>>(d));
  LAUNCH(ctx, k_bondv1_topbottom<<<dim3((d.im + 2 + 127) / 128, d.jm + 3), 128, 0, ctx.s>>>(d));
}

void les_launch_velfg(const LesDom &d, LesCtx ctx) {
  LAUNCH(ctx, k_velfg<<<interior_grid(d, d.km), dim3(BX, BY), 0, ctx.s>>>(d));
}

void les_launch_feedbf(const LesDom &d, LesCtx ctx) {
  LAUNCH(ctx, k_feedbf<<<interior_grid(d, d.km), dim3(BX, BY), 0, ctx.s>>>(d));
}

void les_launch_les(const LesDom &d, LesCtx ctx) {
  LAUNCH(ctx, k_les_sm<<<interior_grid(d, d.km), dim3(BX, BY), 0, ctx.s>>>(d));
  LAUNCH(ctx, k_boundsm_i<<<dim3((d.jm + 3 + 127) / 128, d.km + 2), 128, 0, ctx.s>>>(d));
  LAUNCH(ctx, k_boundsm_j<<<dim3((d.im + 2 + 127) / 128, d.km + 2), 128, 0, ctx.s>>>(d));
  LAUNCH(ctx, k_boundsm_k<<<dim3((d.im + 2 + 127) / 128, d.jm + 3), 128, 0, ctx.s>>>(d));
  LAUNCH(ctx, k_les_visc<<<interior_grid(d, d.km), dim3(BX, BY), 0, ctx.s>>>(d));
}

void les_launch_adam(const LesDom &d, LesCtx ctx) {
  LAUNCH(ctx, k_adam<<<interior_grid(d, d.km), dim3(BX, BY), 0, ctx.s>>>(d));
}

void les_launch_bondfg(const LesDom &d, LesCtx ctx) {
  const int n = d.jm * d.km + d.im * d.km + d.im * d.jm;
  LAUNCH(ctx, k_bondfg<<<(n + 255) / 256, 256, 0, ctx.s>>>(d));
}

void les_launch_boundp1(const LesDom &d, LesCtx ctx, int obey) {
  LAUNCH(ctx, k_boundp1_i<<<dim3((d.jm + 2 + 127) / 128, d.km + 2), 128, 0, ctx.s>>>(d, obey));
  LAUNCH(ctx, k_boundp1_j<<<dim3((d.im + 2 + 127) / 128, d.km + 2), 128, 0, ctx.s>>>(d, obey));
}

void les_launch_boundp2(const LesDom &d, LesCtx ctx, int obey) {
  LAUNCH(ctx, k_boundp2<<<dim3((d.im + 2 + 127) / 128, d.jm + 2), 128, 0, ctx.s>>>(d, obey));
}

int les_interior_blocks(const LesDom &d) {
  const dim3 g = interior_grid(d, d.km);
  return (int)(g.x * g.y * g.z);
}

void les_launch_rhs_mean(const LesDom &d, LesCtx ctx) {
  const int nb = les_interior_blocks(d);
  LAUNCH(ctx, k_rhs<<<interior_grid(d, d.km), dim3(BX, BY), 0, ctx.s>>>(d, d.rhs, 0));
  LAUNCH(ctx, k_finish_mean<<<1, 1024, 0, ctx.s>>>(d, nb, SC_RHSAV));
  LAUNCH(ctx, k_sub_mean<<<interior_grid(d, d.km), dim3(BX, BY), 0, ctx.s>>>(d, d.rhs, SC_RHSAV));
}

void les_launch_rhs_sor(const LesDom &d, LesCtx ctx) {
  const int nb = les_interior_blocks(d);
  LAUNCH(ctx, k_rhs<<<interior_grid(d, d.km), dim3(BX, BY), 0, ctx.s>>>(d, d.sorR, 1));
  LAUNCH(ctx, k_finish_mean<<<1, 1024, 0, ctx.s>>>(d, nb, SC_RHSAV));
}

void les_launch_sor_begin(const LesDom &d, LesCtx ctx) {
  LAUNCH(ctx, k_sor_begin<<<1, 1, 0, ctx.s>>>(d));
}

void les_launch_sor_simple(const LesDom &d, int nmaxp, LesCtx ctx) {
  const dim3 gs((d.im / 2 + 1 + BX - 1) / BX, (d.jm + BY - 1) / BY, d.km);
  const int nb = (int)(gs.x * gs.y * gs.z);
  LAUNCH(ctx, k_sor_begin<<<1, 1, 0, ctx.s>>>(d));
  for (int l = 1; l <= nmaxp; ++l) {
    for (int nrd = 0; nrd <= 1; ++nrd) {
      LAUNCH(ctx, k_sor_colour<<<gs, dim3(BX, BY), 0, ctx.s>>>(d, nrd, nb));
      les_launch_boundp1(d, ctx, 1);
    }
    les_launch_boundp2(d, ctx, 1);
    LAUNCH(ctx, k_sor_check<<<1, 1024, 0, ctx.s>>>(d, 2 * nb));
  }
}

int les_sor_simple_parts(const LesDom &d) {
  const dim3 gs((d.im / 2 + 1 + BX - 1) / BX, (d.jm + BY - 1) / BY, d.km);
  return 2 * (int)(gs.x * gs.y * gs.z);
}

void les_launch_pav_adjust(const LesDom &d, LesCtx ctx) {
  const int nb = les_interior_blocks(d);
  LAUNCH(ctx, k_pav_part<<<interior_grid(d, d.km), dim3(BX, BY), 0, ctx.s>>>(d));
  LAUNCH(ctx, k_finish_mean<<<1, 1024, 0, ctx.s>>>(d, nb, SC_PAV));
  LAUNCH(ctx, k_sub_mean<<<interior_grid(d, d.km), dim3(BX, BY), 0, ctx.s>>>(d, d.p, SC_PAV));
  les_launch_boundp1(d, ctx, 0);
  les_launch_boundp2(d, ctx, 0);
}

void les_launch_count_nonfinite(const LesDom &d, unsigned long long *bad, LesCtx ctx) {
  LAUNCH(ctx, k_count_nonfinite<<<interior_grid(d, d.km), dim3(BX, BY), 0, ctx.s>>>(d, bad));
}
