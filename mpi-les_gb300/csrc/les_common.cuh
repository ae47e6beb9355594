// les_common.cuh -- device data layout and the face quantities of the MPI-LES stencils.
//
// Layout in HBM.  Every 3-D field of a domain uses one padded layout: i fastest,
// then j rows, then k planes.  Logical indices cover i in [-3, pi-4], j in [-1, jm+2],
// k in [-1, km+2], which holds every declared extent of src/main.f95:63-159.  The
// interior cell i = 1 sits at column 4, so interior rows start 16-byte aligned and the
// row pitch pi (floats) is a multiple of 16 (64 bytes).
//
// Face quantities.  The reference's vel2 (src/vel2.f95:74-356) stores 27 temporary
// arrays (nou1-9, diu1-9, cov1-9) that velFG and les then read.  Here they are never
// stored: each kernel recomputes the value the reference array holds at the index it
// reads, from u, v, w, with the same FP32 expression.  The halo copies of
// vel2.f95:202-318 become index remaps (i = im+1 -> im, j = jm+1 -> 1, j = 0 -> jm)
// and entries the reference never writes read as 0 (diu2/diu3 at i = 0, diu7/diu8 at
// k = 0 and k >= km, diu9 at k = km+1).  Recomputation is exact: FP32 arithmetic is
// deterministic, and the kernels are built with --fmad=false and IEEE div/sqrt.
#pragma once
#include <cstdint>

#define LES_IOFF 3
#define LES_JOFF 1
#define LES_KOFF 1

// 1-D arrays, each pointer shifted so that the Fortran index addresses it directly.
struct LesGrid1 {
  const float *dx1, *dy1, *dzn, *dzs, *dxs, *dys, *z2;
  const float *cn2l, *cn2s, *cn3l, *cn3s, *cn4l, *cn4s, *delx1;
  const float *cn1a, *cn1b, *cn1c;  // 2/(dxs(i-1)dxs(i)), 2/(dys(j-1)dys(j)), 2/(dzs(k-1)dzs(k))
  const float *cn1k;                // 1/((a+b)+c) when a and b are the same for all i, j
};

// Device scalar slots (double) of a domain.
enum {
  SC_UOUT = 0,    // bondv1 uout (float value)
  SC_RHSAV,       // press rhsav (float value)
  SC_PAV,         // press pav (float value)
  SC_SOR,         // residual sum of the last SOR iteration
  SC_AREA,        // sum of cell volumes (FP64, fixed per domain)
  SC_COUNT = 8
};
// Device control words (int) of a domain.
enum {
  CT_CONVERGED = 0,  // SOR converged flag of the current press call
  CT_ITERS,          // SOR iterations run in the current press call
  CT_ERROR,          // set by a kernel whose bounded wait gave up (never expected)
  CT_COUNT = 4
};

struct LesDom {
  int im, jm, km;
  int pi, nj, np;  // row pitch (floats), rows per plane, floats per plane
  float *u, *v, *w, *p, *f, *g, *h, *fold, *gold, *hold, *usum, *vsum, *wsum, *rhs, *sm;
  const float *cn1;            // full cn1 (1:im,1:jm,1:km) if not separable, else nullptr
  const uint8_t *mask;         // bit0 bmask1, bit1 cmask1, bit2 dmask1 (padded layout)
  const float *uin, *vin, *win;  // inflow planes (1:jm,1:km), index (j-1)+(k-1)*jm
  LesGrid1 gr;
  float dt, ro, vn, alpha, beta, omega, pjuge;
  float logz;      // alog(0.5*dzn(1)/0.1), vel2.f95:138 and les.f95:133
  int sor_fixed;
  double *scal;    // SC_* slots
  int *ctl;        // CT_* slots
  double *part;    // per-block partial sums
  float *fscal;    // float copies of uout/rhsav/pav for kernels
  float *sorA, *sorB;  // ping-pong p buffers of the fused SOR sweep (with periodic ghost rows)
  float *sorR;         // rhs of the fused SOR sweep (with periodic ghost rows)
  unsigned int *cnt;  // CTA completion ticket of the fused SOR sweep
  int sms;         // SMs of the device (grid sizing)
};

__host__ __device__ __forceinline__ int lix(const LesDom &d, int i, int j, int k) {
  return (k + LES_KOFF) * d.np + (j + LES_JOFF) * d.pi + (i + LES_IOFF);
}

// x**0.5 of the reference (vel2.f95:56-63): IEEE sqrt.  gfortran calls powf(x,0.5),
// which glibc rounds differently from sqrt for about 0.06% of inputs (1 ulp).
__device__ __forceinline__ float pow_half(float x) { return __fsqrt_rn(x); }

#define U_(i, j, k) d.u[lix(d, (i), (j), (k))]
#define V_(i, j, k) d.v[lix(d, (i), (j), (k))]
#define W_(i, j, k) d.w[lix(d, (i), (j), (k))]

// ---- wall-function speeds (vel2.f95:54-65), before the u/uspd rewrite ----------
__device__ __forceinline__ float uspd_raw(const LesDom &d, int i, int j) {
  const float *dx1 = d.gr.dx1;
  const float a = U_(i, j, 1);
  const float b = (0.5f * (V_(i, j - 1, 1) + V_(i, j, 1)) * dx1[i + 1] +
                   0.5f * (V_(i + 1, j - 1, 1) + V_(i + 1, j, 1)) * dx1[i]) /
                  (dx1[i] + dx1[i + 1]);
  return pow_half(a * a + b * b);
}
__device__ __forceinline__ float vspd_raw(const LesDom &d, int i, int j) {
  const float *dy1 = d.gr.dy1;
  const float a = V_(i, j, 1);
  const float b = (0.5f * (U_(i - 1, j, 1) + U_(i, j, 1)) * dy1[j + 1] +
                   0.5f * (U_(i - 1, j + 1, 1) + U_(i, j + 1, 1)) * dy1[j]) /
                  (dy1[j] + dy1[j + 1]);
  return pow_half(a * a + b * b);
}
// log-law wall gradients diu3(i,j,1), diu6(i,j,1) (vel2.f95:138,173)
__device__ __forceinline__ float wall_grad(const LesDom &d, float spd, float vel) {
  const float hz = 0.5f * d.gr.dzn[1];
  return spd * 0.4f / d.logz / hz / 0.4f * vel / spd;
}

// ---- diu1..9 as the reference arrays hold them after vel2 (read ranges of les) --
__device__ __forceinline__ float diu1(const LesDom &d, int i, int j, int k) {
  const int ii = min(i, d.im);
  return (-U_(ii - 1, j, k) + U_(ii, j, k)) / d.gr.dx1[ii];
}
__device__ __forceinline__ float diu2(const LesDom &d, int i, int j, int k) {
  if (i <= 0) return 0.f;
  const int jj = (j > d.jm) ? 1 : j;
  return 2.f * (-U_(i, jj - 1, k) + U_(i, jj, k)) / (d.gr.dy1[jj - 1] + d.gr.dy1[jj]);
}
__device__ __forceinline__ float diu3(const LesDom &d, int i, int j, int k) {
  if (i <= 0) return 0.f;
  if (k == 1) return wall_grad(d, uspd_raw(d, i, j), U_(i, j, 1));
  return (-U_(i, j, k - 1) + U_(i, j, k)) / d.gr.dzs[k - 1];
}
__device__ __forceinline__ float diu4(const LesDom &d, int i, int j, int k) {
  const int ii = min(i, d.im);
  const int jj = (j <= 0) ? d.jm : j;
  return 2.f * (-V_(ii - 1, jj, k) + V_(ii, jj, k)) / (d.gr.dx1[ii - 1] + d.gr.dx1[ii]);
}
__device__ __forceinline__ float diu5(const LesDom &d, int i, int j, int k) {
  const int jj = (j > d.jm) ? 1 : j;
  return (-V_(i, jj - 1, k) + V_(i, jj, k)) / d.gr.dy1[jj];
}
__device__ __forceinline__ float diu6(const LesDom &d, int i, int j, int k) {
  const int jj = (j <= 0) ? d.jm : j;
  if (k == 1) return wall_grad(d, vspd_raw(d, i, jj), V_(i, jj, 1));
  return (-V_(i, jj, k - 1) + V_(i, jj, k)) / d.gr.dzs[k - 1];
}
__device__ __forceinline__ float diu7(const LesDom &d, int i, int j, int k) {
  if (k <= 0 || k >= d.km) return 0.f;
  const int ii = min(i, d.im);
  return 2.f * (-W_(ii - 1, j, k) + W_(ii, j, k)) / (d.gr.dx1[ii - 1] + d.gr.dx1[ii]);
}
__device__ __forceinline__ float diu8(const LesDom &d, int i, int j, int k) {
  if (k <= 0 || k >= d.km) return 0.f;
  const int jj = (j > d.jm) ? 1 : j;
  return 2.f * (-W_(i, jj - 1, k) + W_(i, jj, k)) / (d.gr.dy1[jj - 1] + d.gr.dy1[jj]);
}
__device__ __forceinline__ float diu9(const LesDom &d, int i, int j, int k) {
  if (k > d.km) return 0.f;
  return (-W_(i, j, k - 1) + W_(i, j, k)) / d.gr.dzn[k];
}

// ---- cov1..9 = nou*diu as read by velFG (velFG.f95:64-110) --------------------
__device__ __forceinline__ float cov1(const LesDom &d, int i, int j, int k) {
  const int ii = min(i, d.im);
  const float a = U_(ii - 1, j, k), b = U_(ii, j, k);
  return ((a + b) / 2.f) * ((-a + b) / d.gr.dx1[ii]);
}
__device__ __forceinline__ float cov2(const LesDom &d, int i, int j, int k) {
  const int jj = (j > d.jm) ? 1 : j;
  const float *dx1 = d.gr.dx1, *dy1 = d.gr.dy1;
  const float nou = (dx1[i + 1] * V_(i, jj - 1, k) + dx1[i] * V_(i + 1, jj - 1, k)) / (dx1[i] + dx1[i + 1]);
  const float diu = 2.f * (-U_(i, jj - 1, k) + U_(i, jj, k)) / (dy1[jj - 1] + dy1[jj]);
  return nou * diu;
}
__device__ __forceinline__ float cov3(const LesDom &d, int i, int j, int k) {
  const float *dx1 = d.gr.dx1;
  if (k == 1) {
    const float nou = 0.5f * (dx1[i + 1] * W_(i, j, 1) + dx1[i] * W_(i + 1, j, 1)) / (dx1[i] + dx1[i + 1]);
    return nou * wall_grad(d, uspd_raw(d, i, j), U_(i, j, 1));
  }
  const float nou = (dx1[i + 1] * W_(i, j, k - 1) + dx1[i] * W_(i + 1, j, k - 1)) / (dx1[i] + dx1[i + 1]);
  const float diu = (-U_(i, j, k - 1) + U_(i, j, k)) / d.gr.dzs[k - 1];
  return nou * diu;
}
__device__ __forceinline__ float cov4(const LesDom &d, int i, int j, int k) {
  const int ii = min(i, d.im);
  const float *dx1 = d.gr.dx1, *dy1 = d.gr.dy1;
  const float nou = (dy1[j + 1] * U_(ii - 1, j, k) + dy1[j] * U_(ii - 1, j + 1, k)) / (dy1[j] + dy1[j + 1]);
  const float diu = 2.f * (-V_(ii - 1, j, k) + V_(ii, j, k)) / (dx1[ii - 1] + dx1[ii]);
  return (nou - 0.f) * diu;
}
__device__ __forceinline__ float cov5(const LesDom &d, int i, int j, int k) {
  const int jj = (j > d.jm) ? 1 : j;
  const float a = V_(i, jj - 1, k), b = V_(i, jj, k);
  return ((a + b) / 2.f) * ((-a + b) / d.gr.dy1[jj]);
}
__device__ __forceinline__ float cov6(const LesDom &d, int i, int j, int k) {
  const float *dy1 = d.gr.dy1;
  if (k == 1) {
    const float nou = 0.5f * (dy1[j + 1] * W_(i, j, 1) + dy1[j] * W_(i, j + 1, 1)) / (dy1[j] + dy1[j + 1]);
    return nou * wall_grad(d, vspd_raw(d, i, j), V_(i, j, 1));
  }
  const float nou = (dy1[j + 1] * W_(i, j, k - 1) + dy1[j] * W_(i, j + 1, k - 1)) / (dy1[j] + dy1[j + 1]);
  const float diu = (-V_(i, j, k - 1) + V_(i, j, k)) / d.gr.dzs[k - 1];
  return nou * diu;
}
__device__ __forceinline__ float cov7(const LesDom &d, int i, int j, int k) {
  const int ii = min(i, d.im);
  const float *dx1 = d.gr.dx1, *dzn = d.gr.dzn;
  const float nou = (dzn[k + 1] * U_(ii - 1, j, k) + dzn[k] * U_(ii - 1, j, k + 1)) / (dzn[k] + dzn[k + 1]);
  const float diu = 2.f * (-W_(ii - 1, j, k) + W_(ii, j, k)) / (dx1[ii - 1] + dx1[ii]);
  return (nou - 0.f) * diu;
}
__device__ __forceinline__ float cov8(const LesDom &d, int i, int j, int k) {
  const int jj = (j > d.jm) ? 1 : j;
  const float *dy1 = d.gr.dy1, *dzn = d.gr.dzn;
  const float nou = (dzn[k + 1] * V_(i, jj - 1, k) + dzn[k] * V_(i, jj - 1, k + 1)) / (dzn[k] + dzn[k + 1]);
  const float diu = 2.f * (-W_(i, jj - 1, k) + W_(i, jj, k)) / (dy1[jj - 1] + dy1[jj]);
  return nou * diu;
}
__device__ __forceinline__ float cov9(const LesDom &d, int i, int j, int k) {
  const float a = W_(i, j, k - 1), b = W_(i, j, k);
  return ((a + b) / 2.f) * ((-a + b) / d.gr.dzn[k]);
}

// Warp-level FP32 sum followed by an FP64 block sum: one double per block.  FP32
// inside a warp keeps the (slow on this part) FP64 pipe out of the per-cell path.
template <int NT>
__device__ __forceinline__ double block_sum_f32_to_f64(float x, double *sh) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = (double)x;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int q = 0; q < NT / 32; ++q) s += sh[q];
  }
  __syncthreads();
  return s;
}
// FP64 block sum of per-thread FP64 values (used where each term must enter in FP64).
template <int NT>
__device__ __forceinline__ double block_sum_f64(double x, double *sh) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = x;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int q = 0; q < NT / 32; ++q) s += sh[q];
  }
  __syncthreads();
  return s;
}
