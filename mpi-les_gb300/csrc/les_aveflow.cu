// les_aveflow.cu -- time averages of the flow (aveflow.f95:5-200), on the device.
//
// The reference calls aveflow after every step (main.f95:320): from step n1 on it adds
// v, p, sm, the squares of u, v, w, sm and the u-w flux 0.5*(u(k-1)+u(k))*0.5*(w(k-1)+
// w(i+1,k-1)) into its arrays, u and w over k = 0..km (w over i = 1..im+1); at nmax it
// divides by the number of steps, removes the mean flux from uwfx and turns the mean
// squares of u, v, w into rms fluctuations sqrt(|<x^2> - <x>^2|).  Every cell is
// independent of the others within one pass, so each pass is one elementwise kernel in
// the padded field layout; the only cross-cell reads (uwfx's final correction reads
// aveu(k-1), avew(i+1,k-1)) come after the division pass has completed.  The FP32
// operations are the reference's, left to right (x**2 as x*x, IEEE division and sqrt).
#include <cuda_runtime.h>

#include "les_aveflow.cuh"

namespace {

struct AveIdx {
  int i, j, k, c;
  bool full, row_u, row_w;  // k >= 1 and i <= im; i <= im; i <= im+1
};

// i = 1 .. im+1 over blocks in x, j over y, k = 0 .. km over z
__device__ __forceinline__ AveIdx ave_idx(const LesDom &d) {
  AveIdx x;
  x.i = (int)(blockIdx.x * blockDim.x + threadIdx.x) + 1;
  x.j = (int)blockIdx.y + 1;
  x.k = (int)blockIdx.z;
  x.c = lix(d, x.i, x.j, x.k);
  x.row_u = x.i <= d.im;
  x.row_w = x.i <= d.im + 1;
  x.full = x.row_u && x.k >= 1;
  return x;
}

// aveflow.f95:82-114 (n == n1)
__global__ void k_ave_zero(LesDom d, LesAve A) {
  const AveIdx x = ave_idx(d);
  if (!x.row_w) return;
  const int c = x.c;
  if (x.full) {
    A.avev[c] = 0.f; A.avep[c] = 0.f; A.avel[c] = 0.f;
    A.aveuu[c] = 0.f; A.avevv[c] = 0.f; A.aveww[c] = 0.f;
    A.avesm[c] = 0.f; A.avesmsm[c] = 0.f; A.uwfx[c] = 0.f;
  }
  if (x.row_u) A.aveu[c] = 0.f;
  A.avew[c] = 0.f;
}

// aveflow.f95:117-149 (n >= n1), four cells of a row per thread as float4: cell i0 =
// 1 + 4t sits at a 16-byte boundary of the padded row (i + 3 = 4t + 4).  Groups that
// reach past im (the row's last cells, where u and w have different extents) take the
// per-cell path.
__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void add4(float *p, float4 x) {
  float4 a = *reinterpret_cast<float4 *>(p);
  a.x = a.x + x.x; a.y = a.y + x.y; a.z = a.z + x.z; a.w = a.w + x.w;
  *reinterpret_cast<float4 *>(p) = a;
}
__device__ __forceinline__ float4 sq4(float4 x) { return make_float4(x.x * x.x, x.y * x.y, x.z * x.z, x.w * x.w); }

__device__ __forceinline__ void ave_acc_cell(const LesDom &d, const LesAve &A, int i, int c, bool k1) {
  const bool row_u = i <= d.im, full = row_u && k1;
  if (full) {
    const float u = d.u[c], v = d.v[c], w = d.w[c], s = d.sm[c];
    A.avev[c] = A.avev[c] + v;
    A.avep[c] = A.avep[c] + d.p[c];
    A.aveuu[c] = A.aveuu[c] + u * u;
    A.avevv[c] = A.avevv[c] + v * v;
    A.aveww[c] = A.aveww[c] + w * w;
    A.avesm[c] = A.avesm[c] + s;
    A.avesmsm[c] = A.avesmsm[c] + s * s;
    const int cd = c - d.np;
    A.uwfx[c] = A.uwfx[c] + 0.5f * (d.u[cd] + u) * 0.5f * (d.w[cd] + d.w[cd + 1]);
  }
  if (row_u) A.aveu[c] = A.aveu[c] + d.u[c];
  A.avew[c] = A.avew[c] + d.w[c];
}

__global__ void k_ave_acc4(LesDom d, LesAve A) {
  const int i0 = 1 + 4 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i0 > d.im + 1) return;
  const int j = (int)blockIdx.y + 1, k = (int)blockIdx.z;
  const int c = lix(d, i0, j, k);
  if (i0 + 3 > d.im) {
    for (int e = 0; e < 4 && i0 + e <= d.im + 1; ++e) ave_acc_cell(d, A, i0 + e, c + e, k >= 1);
    return;
  }
  const float4 u = ld4(d.u + c), w = ld4(d.w + c);
  add4(A.aveu + c, u);
  add4(A.avew + c, w);
  if (k < 1) return;
  const float4 v = ld4(d.v + c), s = ld4(d.sm + c);
  add4(A.avev + c, v);
  add4(A.avep + c, ld4(d.p + c));
  add4(A.aveuu + c, sq4(u));
  add4(A.avevv + c, sq4(v));
  add4(A.aveww + c, sq4(w));
  add4(A.avesm + c, s);
  add4(A.avesmsm + c, sq4(s));
  const int cd = c - d.np;
  const float4 ud = ld4(d.u + cd), wd = ld4(d.w + cd);
  const float w4 = d.w[cd + 4];
  float4 f;
  f.x = 0.5f * (ud.x + u.x) * 0.5f * (wd.x + wd.y);
  f.y = 0.5f * (ud.y + u.y) * 0.5f * (wd.y + wd.z);
  f.z = 0.5f * (ud.z + u.z) * 0.5f * (wd.z + wd.w);
  f.w = 0.5f * (ud.w + u.w) * 0.5f * (wd.w + w4);
  add4(A.uwfx + c, f);
}

// aveflow.f95:151-185 (n == nmax): the divisions
__global__ void k_ave_div(LesDom d, LesAve A, float cnt) {
  const AveIdx x = ave_idx(d);
  if (!x.row_w) return;
  const int c = x.c;
  if (x.full) {
    A.avev[c] = A.avev[c] / cnt; A.avep[c] = A.avep[c] / cnt; A.avel[c] = A.avel[c] / cnt;
    A.aveuu[c] = A.aveuu[c] / cnt; A.avevv[c] = A.avevv[c] / cnt; A.aveww[c] = A.aveww[c] / cnt;
    A.avesm[c] = A.avesm[c] / cnt; A.avesmsm[c] = A.avesmsm[c] / cnt;
  }
  if (x.row_u) A.aveu[c] = A.aveu[c] / cnt;
  A.avew[c] = A.avew[c] / cnt;
}

// aveflow.f95:188-209 (n == nmax, after every division): the mean flux and the rms
__global__ void k_ave_final(LesDom d, LesAve A, float cnt) {
  const AveIdx x = ave_idx(d);
  if (!x.full) return;
  const int c = x.c, cd = c - d.np;
  A.uwfx[c] = A.uwfx[c] / cnt - 0.5f * (A.aveu[cd] + A.aveu[c]) * 0.5f * (A.avew[cd] + A.avew[cd + 1]);
  const float mu = A.aveu[c], mv = A.avev[c], mw = A.avew[c];
  A.aveuu[c] = __fsqrt_rn(fabsf(A.aveuu[c] - mu * mu));
  A.avevv[c] = __fsqrt_rn(fabsf(A.avevv[c] - mv * mv));
  A.aveww[c] = __fsqrt_rn(fabsf(A.aveww[c] - mw * mw));
}

}  // namespace

void les_launch_aveflow(const LesDom &d, const LesAve &A, int n, int n1, int nmax, LesCtx ctx) {
  const dim3 b(128), g((d.im + 1 + 127) / 128, d.jm, d.km + 1);
  if (n == n1) {
    k_ave_zero<<<g, b, 0, ctx.s>>>(d, A);
    ++*ctx.nlaunch;
  }
  if (n >= n1) {
    const int groups = (d.im + 1 + 3) / 4;  // cells 1 .. im+1, four per thread
    k_ave_acc4<<<dim3((groups + 127) / 128, d.jm, d.km + 1), b, 0, ctx.s>>>(d, A);
    ++*ctx.nlaunch;
  }
  if (n == nmax) {
    const float cnt = (float)(nmax - n1 + 1);  // float(nmax-n1+1)
    k_ave_div<<<g, b, 0, ctx.s>>>(d, A, cnt);
    k_ave_final<<<g, b, 0, ctx.s>>>(d, A, cnt);
    *ctx.nlaunch += 2;
  }
}
