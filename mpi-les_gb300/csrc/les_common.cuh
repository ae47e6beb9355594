// les_common.cuh -- device data layout and the face quantities of the MPI-LES stencils.
//
// Layout in HBM.  Every 3-D field of a domain uses one padded layout: i fastest,
// then j rows, then k planes.  Logical indices cover i in [-3, pi-4], j in [-3, jm+4],
// k in [-1, km+2], which holds every declared extent of src/main.f95:63-159 and the
// four periodic ghost rows per side that the SOR sweep fusing two iterations reads.
// The interior cell i = 1 sits at column 4, so interior rows start 16-byte aligned and
// the row pitch pi (floats) is a multiple of 16 (64 bytes).
//
// Face quantities.  The reference's vel2 (src/vel2.f95:74-356) stores 27 temporary
// arrays (nou1-9, diu1-9, cov1-9) that velFG and les then read.  Here nou and cov are
// never stored (velfg forms them where it needs them) and only diu1-9 are: les reads
// them back.  The halo copies of vel2.f95:202-318 become index remaps (i = im+1 -> im,
// j = jm+1 -> 1, j = 0 -> jm) and entries the reference never writes read as 0
// (diu2/diu3 at i = 0, diu7/diu8 at k = 0 and k >= km, diu9 at k = km+1).  The FP32
// arithmetic is the reference's, operation for operation: the kernels are built with
// --fmad=false, and every division gives the IEEE quotient (dvz, dvs below).
#pragma once
#include <cstdint>

#define LES_IOFF 3
#define LES_JOFF 3
#define LES_KOFF 1

// 1-D arrays, each pointer shifted so that the Fortran index addresses it directly.
struct LesGrid1 {
  const float *dx1, *dy1, *dzn, *dzs, *dxs, *dys, *z2;
  const float *cn2l, *cn2s, *cn3l, *cn3s, *cn4l, *cn4s, *delx1;
  const float *cn1a, *cn1b, *cn1c;  // 2/(dxs(i-1)dxs(i)), 2/(dys(j-1)dys(j)), 2/(dzs(k-1)dzs(k))
  const float *cn1k;                // 1/((a+b)+c) when a and b are the same for all i, j
  // correctly rounded FP32 reciprocals of the spacings and of the neighbour sums:
  // 1/dx1(i), 1/(dx1(i)+dx1(i+1)), 1/dxs(i), the same in y, 1/dzn(k), 1/dzs(k),
  // 1/(dzn(k)+dzn(k+1)), indexed like the spacing arrays
  const float *rdx1, *rdx1s, *rdxs, *rdy1, *rdy1s, *rdys, *rdzn, *rdzs, *rdzsum;
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
  CT_REDO,           // a two-iteration SOR launch must be cut back to its first iteration
  CT_LASTBUF,        // where the last SOR launch wrote p: 0 sorA, 1 sorB, 2 p
  CT_COUNT = 8
};

// deferred-block lists, one per kernel that divides with dvz
enum { FIX_VELNW = 0, FIX_VELFG, FIX_VISC, FIX_RHS, FIX_COUNT };

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
  int sor_ksplit;  // 1: never split the SOR k-march (les_params.sor_ksplit)
  double *scal;    // SC_* slots
  int *ctl;        // CT_* slots
  double *part;    // per-block partial sums
  float *fscal;    // float copies of uout/rhsav/pav for kernels
  float *sorA, *sorB;  // ping-pong p buffers of the fused SOR sweep (with periodic ghost rows)
  float *sorR;         // rhs of the fused SOR sweep (with periodic ghost rows)
  float *prow;         // p's row jm+2 (i = 1..im, k = 1..km, i fastest), saved while the
                       // fused sweep's first iteration reads that row as a ghost copy
  unsigned int *cnt;  // CTA completion tickets: [0] fused SOR sweep, [8] finish_mean, [12] bondv1 uout
  double *part2;      // second-level partial sums of finish_mean (FIN_BLOCKS)
  int sms;         // SMs of the device (grid sizing)
  // xy_pow2: every x and y spacing is the same power of two (dvs multiplies);
  // zfast: every spacing, spacing sum and scalar divisor lies in [2^-20, 2^20] (dvz),
  // with the reciprocals of ro, dt and logz
  int xy_pow2;
  int zfast;
  float rro, rdt, rlogz;
  // sor_uni: cn2l, cn2s, cn3l and cn3s each hold one value over i (j), so the two-
  // iteration SOR sweep reads them as scalars
  int sor_uni;
  // with xy_pow2: the one x spacing hx and y spacing hy, 1/hx, 1/(2 hx), 1/hy, 1/(2 hy)
  float hx, hy, rhx, rhx2, rhy, rhy2;
  // deferred-block lists of the kernels that use dvz (FIX_*): [0] count, [1] ticket of
  // the fixup kernel, then the linear ids of the blocks left to the fixup kernel
  int *fix[4];
  // diu1..9 as velfg computed them (vel2.f95:74-197), interior cells (plus plane km+1
  // of diu3/diu6), read by les the way les.f95 reads the reference's arrays; and the
  // wall-function ratios u(i,j,1)/uspd, v(i,j,1)/vspd of vel2.f95:351-356 (one plane)
  float *diu[10];
  float *ruspd, *rvspd;
};

__host__ __device__ __forceinline__ int lix(const LesDom &d, int i, int j, int k) {
  return (k + LES_KOFF) * d.np + (j + LES_JOFF) * d.pi + (i + LES_IOFF);
}

// Periodic ghost rows of the SOR buffers: rows j in [-3, 0] and [jm+1, jm+4] hold row
// 1 + (j-1) mod jm.  ghost_mask(j, jm) has bit b set when row j + m jm is such a ghost
// row, for m = -2, -1, 1, 2 (b = 0..3): at most four (jm = 2), none for rows 5..jm-4.
// for_ghost_rows(j, jm, mask, f) calls f(m jm) for each set bit.
__host__ __device__ __forceinline__ unsigned ghost_mask(int j, int jm) {
  unsigned g = 0;
  const int ms[4] = {-2, -1, 1, 2};
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const int t = j + ms[b] * jm;
    if (t >= -3 && t <= jm + 4) g |= 1u << b;
  }
  return g;
}
template <class F>
__host__ __device__ __forceinline__ void for_ghost_rows(int jm, unsigned mask, F f) {
  if (!mask) return;
  if (mask & 1u) f(-2 * jm);
  if (mask & 2u) f(-jm);
  if (mask & 4u) f(jm);
  if (mask & 8u) f(2 * jm);
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
// a / b for a divisor b fixed at set-up, with y = RN(1/b) computed on the host.
// ZF: Markstein's corrected quotient q0 = a*y, r = a - b*q0 (exact by FMA), q = q0 + r*y
// (P. Markstein, IBM J. Res. Dev. 34(1), 1990: with y the correctly rounded reciprocal,
// q is the correctly rounded a/b while r and q stay normal).  That holds for
// |b| in [2^-20, 2^20] (checked at set-up) and |a| in [2^-100, 2^100]; a zero dividend
// is exact as a*y (sign included).  Any other dividend (tiny, huge, inf, NaN) sets
// `bad` and the caller recomputes its cell with IEEE divisions.  The path is free of
// branches and calls, so a kernel can issue its whole stencil's loads up front.
// !ZF: the IEEE division.
template <bool ZF>
__device__ __forceinline__ float dvz(float a, float b, float y, unsigned &bad) {
  if (!ZF) return a / b;
  const float aa = fabsf(a);
  const float q0 = __fmul_rn(a, y);
  const float r = __fmaf_rn(-q0, b, a);
  const float q1 = __fmaf_rn(r, y, q0);
  bad |= (unsigned)(!(aa >= 0x1p-100f && aa <= 0x1p100f) && aa != 0.f);
  return aa == 0.f ? q0 : q1;
}
// x / (an x or y spacing, or the sum of two): P2 (all x and y spacings the same power
// of two) makes it a multiplication by the exact reciprocal -- both round the same
// real number -- else as dvz
template <bool P2, bool ZF>
__device__ __forceinline__ float dvs(float x, float den, float rden, unsigned &bad) {
  return P2 ? x * rden : dvz<ZF>(x, den, rden, bad);
}

// The x and y spacings and their reciprocals as the kernels read them: dx1(i), dxs(i),
// 1/dx1(i), 1/(dx1(i)+dx1(i+1)), 1/dxs(i) and the same in y.  With P2 every x and y
// spacing is one power of two (checked at set-up), so these are the domain's uniform
// values -- the numbers the arrays hold -- and cost no loads.
template <bool P2> __device__ __forceinline__ float sx1(const LesDom &d, int i) { return P2 ? d.hx : d.gr.dx1[i]; }
template <bool P2> __device__ __forceinline__ float sy1(const LesDom &d, int j) { return P2 ? d.hy : d.gr.dy1[j]; }
template <bool P2> __device__ __forceinline__ float sxs(const LesDom &d, int i) { return P2 ? d.hx : d.gr.dxs[i]; }
template <bool P2> __device__ __forceinline__ float sys(const LesDom &d, int j) { return P2 ? d.hy : d.gr.dys[j]; }
template <bool P2> __device__ __forceinline__ float rx1(const LesDom &d, int i) { return P2 ? d.rhx : d.gr.rdx1[i]; }
template <bool P2> __device__ __forceinline__ float rx1s(const LesDom &d, int i) { return P2 ? d.rhx2 : d.gr.rdx1s[i]; }
template <bool P2> __device__ __forceinline__ float rxs(const LesDom &d, int i) { return P2 ? d.rhx : d.gr.rdxs[i]; }
template <bool P2> __device__ __forceinline__ float ry1(const LesDom &d, int j) { return P2 ? d.rhy : d.gr.rdy1[j]; }
template <bool P2> __device__ __forceinline__ float ry1s(const LesDom &d, int j) { return P2 ? d.rhy2 : d.gr.rdy1s[j]; }
template <bool P2> __device__ __forceinline__ float rys(const LesDom &d, int j) { return P2 ? d.rhy : d.gr.rdys[j]; }

// Block-level deferral.  A block in which some thread met a dividend outside dvz's range
// stores nothing; thread 0 appends the block's linear id to `list`, and a fixup kernel
// launched next recomputes the listed blocks with IEEE divisions.  The hot kernels thus
// hold no IEEE division code at all, whose presence alone (even never executed) slows
// their memory pipeline several-fold.  Every thread of the block must call this.
__device__ __forceinline__ bool defer_block(unsigned bad, int *list) {
  if (!__syncthreads_or(bad)) return false;
  if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
    const int s = atomicAdd(list, 1);
    list[2 + s] = (int)((blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x);
  }
  return true;
}
// The fixup side: body(bx, by, bz) for every listed block of a main grid g, then the
// last CTA to finish resets the list for the next launch.
template <class F>
__device__ __forceinline__ void for_deferred(int *list, uint3 g, F body) {
  const int n = *(volatile int *)list;
  for (int q = blockIdx.x; q < n; q += gridDim.x) {
    const int id = list[2 + q];
    body((int)(id % g.x), (int)((id / g.x) % g.y), (int)(id / (g.x * g.y)));
  }
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
    __threadfence();
    if (atomicAdd(list + 1, 1) == (int)gridDim.x - 1) {
      list[0] = 0;
      list[1] = 0;
    }
  }
}

// log-law wall gradients diu3(i,j,1), diu6(i,j,1) (vel2.f95:138,173), IEEE divisions
__device__ __forceinline__ float wall_grad(const LesDom &d, float spd, float vel) {
  const float hz = 0.5f * d.gr.dzn[1];
  return spd * 0.4f / d.logz / hz / 0.4f * vel / spd;
}

// Knuth's TwoSum: s = fl(a + b) and e with s + e == a + b exactly (the kernels are
// built with --fmad=false, so nothing here is contracted).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
