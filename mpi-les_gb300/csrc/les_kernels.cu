// les_kernels.cu -- per-subroutine kernels of the MPI-LES solver (sm_103a).
//
// One kernel (or a short fixed sequence of small kernels) per reference subroutine,
// each a drop-in for that subroutine on device-resident state.  These are the
// building blocks behind the per-subroutine C-ABI entry points.  velfg and les live in
// les_fused.cu (shared with the whole step); the whole step's SOR is les_sor.cu.
//
// Exactness: every interior update is an independent function of values no other
// thread of the same launch writes, so a one-thread-per-cell launch reproduces the
// reference's sequential loops bit for bit.  Halo fills that the reference runs as
// ordered loops run as ordered launches.  Sums (uout max/min, rhsav, pav, the SOR
// residual) are per-domain deterministic reductions: FP64 where the reference sums
// many FP32 terms.
#include <cuda_runtime.h>

#include <algorithm>

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
// new u, v, w of one cell; P2 / ZF: division forms of dvs / dvz (les_common.cuh)
// (p, f, g, h are only read here: read-only loads)
template <bool P2, bool ZF>
__device__ __forceinline__ void velnw_cell(const LesDom &d, int i, int j, int k, int c, float &un, float &vn, float &wn,
                                           unsigned &bd) {
  const float pc = __ldg(d.p + c);
  float pz = dvs<P2, ZF>(dvz<ZF>(-pc + __ldg(d.p + c + 1), d.ro, d.rro, bd), sxs<P2>(d, i), rxs<P2>(d, i), bd);
  un = d.u[c] + d.dt * (__ldg(d.f + c) - pz);
  pz = dvs<P2, ZF>(dvz<ZF>(-pc + __ldg(d.p + c + d.pi), d.ro, d.rro, bd), sys<P2>(d, j), rys<P2>(d, j), bd);
  vn = d.v[c] + d.dt * (__ldg(d.g + c) - pz);
  if (k <= d.km - 1) {
    pz = dvz<ZF>(dvz<ZF>(-pc + __ldg(d.p + c + d.np), d.ro, d.rro, bd), d.gr.dzs[k], d.gr.rdzs[k], bd);
    wn = d.w[c] + d.dt * (__ldg(d.h + c) - pz);
  }
}
// velnw of the block (bx, by, bz): planes bz*VNK+1 .. bz*VNK+VNK of its columns, all
// computed before any is stored (each cell reads only its own u, v, w, so the update in
// place is safe); ZF: reciprocal-corrected divisions with blocks that meet a dividend
// outside their range deferred to k_velnw_fix (les_common.cuh)
constexpr int VNK = 4;
template <bool P2, bool ZF>
__device__ __forceinline__ void velnw_block(const LesDom &d, int bx, int by, int bz) {
  const int i0 = bx * BX + threadIdx.x + 1, j0 = by * BY + threadIdx.y + 1, ka = bz * VNK + 1;
  const bool in = (i0 <= d.im && j0 <= d.jm);
  const int i = min(i0, d.im), j = min(j0, d.jm);  // past the edge: the edge cell again, not stored
  float un[VNK], vn[VNK], wn[VNK];
  unsigned bd = 0;
#pragma unroll
  for (int q = 0; q < VNK; ++q) {
    un[q] = vn[q] = wn[q] = 0.f;
    if (ka + q <= d.km) velnw_cell<P2, ZF>(d, i, j, ka + q, lix(d, i, j, ka + q), un[q], vn[q], wn[q], bd);
  }
  if (ZF && defer_block(bd, d.fix[FIX_VELNW])) return;
  if (!in) return;
#pragma unroll
  for (int q = 0; q < VNK; ++q) {
    const int k = ka + q;
    if (k > d.km) break;
    const int c = lix(d, i, j, k);
    d.u[c] = un[q];
    d.v[c] = vn[q];
    if (k <= d.km - 1) d.w[c] = wn[q];
  }
}
template <bool P2, bool ZF>
__global__ void __launch_bounds__(BX *BY) k_velnw(LesDom d) {
  velnw_block<P2, ZF>(d, blockIdx.x, blockIdx.y, blockIdx.z);
}
template <bool P2>
__global__ void __launch_bounds__(BX *BY) k_velnw_fix(LesDom d, uint3 g) {
  for_deferred(d.fix[FIX_VELNW], g, [&](int bx, int by, int bz) { velnw_block<P2, false>(d, bx, by, bz); });
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
// uout = (max(0, max u(im)) + min(0, min u(im)))/2 (bondv1.f95:171-187).  The values
// u(im, j, k) are one per row, so many blocks gather them; each block's max and min go
// to part[], and the last block to finish combines them, all its threads at once (max
// and min are exact in any order).
// With INFLOW the same grid-stride loop also writes the inflow planes i = 0, 1 of
// k_bondv1_inflow (it reads only i = im >= 3, so the two are independent); a step with
// the n = 1 fill (which reads i = 1 and writes up to im) keeps them apart.
constexpr int UOUT_BLOCKS = 64, UOUT_THREADS = 256;
template <bool INFLOW>
__global__ void __launch_bounds__(UOUT_THREADS) k_bondv1_uout(LesDom d) {
  __shared__ float smax[UOUT_THREADS / 32], smin[UOUT_THREADS / 32];
  __shared__ int last;
  float aaa = 0.f, bbb = 0.f;
  const int n = d.jm * d.km;
  for (int q = blockIdx.x * UOUT_THREADS + threadIdx.x; q < n; q += gridDim.x * UOUT_THREADS) {
    const int j = q % d.jm + 1, k = q / d.jm + 1;
    if (INFLOW) {
      const float a = d.uin[q], b = d.vin[q], c = d.win[q];
      for (int i = 0; i <= 1; ++i) {
        const int x = lix(d, i, j, k);
        d.u[x] = a; d.v[x] = b; d.w[x] = c;
      }
    }
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
    for (int q = 0; q < UOUT_THREADS / 32; ++q) { a = fmaxf(a, smax[q]); b = fminf(b, smin[q]); }
    d.part[2 * blockIdx.x] = (double)a;
    d.part[2 * blockIdx.x + 1] = (double)b;
    __threadfence();
    last = (atomicAdd(d.cnt + 12, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  aaa = 0.f;
  bbb = 0.f;
  for (int q = threadIdx.x; q < (int)gridDim.x; q += UOUT_THREADS) {
    aaa = fmaxf(aaa, (float)((volatile double *)d.part)[2 * q]);
    bbb = fminf(bbb, (float)((volatile double *)d.part)[2 * q + 1]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    aaa = fmaxf(aaa, __shfl_down_sync(0xffffffffu, aaa, o));
    bbb = fminf(bbb, __shfl_down_sync(0xffffffffu, bbb, o));
  }
  if ((threadIdx.x & 31) == 0) { smax[threadIdx.x >> 5] = aaa; smin[threadIdx.x >> 5] = bbb; }
  __syncthreads();
  if (threadIdx.x != 0) return;
  float a = 0.f, b = 0.f;
  for (int q = 0; q < UOUT_THREADS / 32; ++q) { a = fmaxf(a, smax[q]); b = fminf(b, smin[q]); }
  const float uout = (a + b) / 2.f;
  d.fscal[SC_UOUT] = uout;
  d.scal[SC_UOUT] = (double)uout;
  d.cnt[12] = 0u;
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
// the periodic side flow then the top and underground of bondv1 (bondv1.f95:210-268) as
// one pass.  The two passes (j halos 0 and jm+1 of u, v for k = 0..km+1 and of w for
// k = 0..km, for i = 0..im+1; then u, v k halos for j = 0..jm+1 (negated at k = 0) and
// w = 0 on k = 0 and k = km for j = -1..jm+1) compose to: u, v at a j-halo row point or
// a k-halo plane point take the value at the source point (j = 0 -> jm, jm+1 -> 1; k
// clamped into 1..km), negated on k = 0; w is 0 on k = 0 and km, and its j-halo rows
// for k = 1..km-1 take the wrapped row's value.  No source point is written here.
__global__ void k_bondv1_sides(LesDom d) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long ni = d.im + 2;
  const long long na = 2LL * d.km * ni, nb = 2LL * (d.jm + 2) * ni, nc = 2LL * (d.jm + 3) * ni;
  if (t < na) {  // u, v (and w for k <= km-1) on the j-halo rows, k = 1..km
    const long long r = t % (d.km * ni);
    const int j = (t < d.km * ni) ? 0 : d.jm + 1, i = (int)(r % ni), k = (int)(r / ni) + 1;
    const int js = (j == 0) ? d.jm : 1;
    const int c = lix(d, i, j, k), cs = lix(d, i, js, k);
    d.u[c] = d.u[cs];
    d.v[c] = d.v[cs];
    if (k <= d.km - 1) d.w[c] = d.w[cs];
  } else if (t < na + nb) {  // u, v on the k-halo planes, j = 0..jm+1
    const long long u = t - na, r = u % ((d.jm + 2) * ni);
    const int k = (u < (d.jm + 2) * ni) ? 0 : d.km + 1, i = (int)(r % ni), j = (int)(r / ni);
    const int js = (j == 0) ? d.jm : (j == d.jm + 1) ? 1 : j, ks = (k == 0) ? 1 : d.km;
    const int c = lix(d, i, j, k), cs = lix(d, i, js, ks);
    d.u[c] = (k == 0) ? -d.u[cs] : d.u[cs];
    d.v[c] = (k == 0) ? -d.v[cs] : d.v[cs];
  } else if (t < na + nb + nc) {  // w = 0 on k = 0 and k = km, j = -1..jm+1
    const long long u = t - na - nb, r = u % ((d.jm + 3) * ni);
    const int k = (u < (d.jm + 3) * ni) ? 0 : d.km, i = (int)(r % ni), j = (int)(r / ni) - 1;
    d.w[lix(d, i, j, k)] = 0.f;
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

// boundsm.f95:18-64, three ordered phases
// boundsm.f95:5-69 as one pass.  The reference's three passes (i halos for j = -1..jm+1,
// then j halos 0 and jm+1 for i = 0..im+1, then k halos 0 (negated) and km+1 for i =
// 0..im+1, j = -1..jm+1, each reading what the one before wrote) compose to: a halo
// point takes the value at its source point, clamped into i = 1..im, j = 1..jm (row
// j = -1 stays -1: no pass writes it for i = 1..im) and k = 1..km, negated on k = 0.
// No source point is a halo point this kernel writes, so the points are independent.
// One thread per point of the k faces (k = 0, km+1: (im+2) x (jm+3) each), the i faces
// (i = 0, im+1; j = -1..jm+1; k = 1..km) and the j faces (j = 0, jm+1; i = 1..im;
// k = 1..km).
__global__ void k_boundsm_all(LesDom d) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nk = (long long)(d.im + 2) * (d.jm + 3), ni = (long long)(d.jm + 3) * d.km,
                  nj = (long long)d.im * d.km;
  int i, j, k;
  if (t < 2 * nk) {
    const long long r = t % nk;
    k = (t < nk) ? 0 : d.km + 1;
    i = (int)(r % (d.im + 2));
    j = (int)(r / (d.im + 2)) - 1;
  } else if (t < 2 * nk + 2 * ni) {
    const long long u = t - 2 * nk, r = u % ni;
    i = (u < ni) ? 0 : d.im + 1;
    j = (int)(r % (d.jm + 3)) - 1;
    k = (int)(r / (d.jm + 3)) + 1;
  } else if (t < 2 * nk + 2 * ni + 2 * nj) {
    const long long u = t - 2 * nk - 2 * ni, r = u % nj;
    j = (u < nj) ? 0 : d.jm + 1;
    i = (int)(r % d.im) + 1;
    k = (int)(r / d.im) + 1;
  } else {
    return;
  }
  const int is = min(max(i, 1), d.im), js = (j == -1) ? -1 : min(max(j, 1), d.jm), ks = min(max(k, 1), d.km);
  const float v = d.sm[lix(d, is, js, ks)];
  d.sm[lix(d, i, j, k)] = (k == 0) ? -v : v;
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
// (u, v, w, f, g, h are only read here: read-only loads)
// The values one cell reads: u(i-1), u, v(j-1), v, w(k-1), w, f(i-1), f, g(j-1), g,
// h(k-1), h at (i, j, k).
struct RhsIn {
  float um, uc, vm, vc, wm, wc, fm, fc, gm, gc, hm, hc;
};
__device__ __forceinline__ RhsIn rhs_load(const LesDom &d, int c) {
  RhsIn x;
  x.um = __ldg(d.u + c - 1); x.uc = __ldg(d.u + c);
  x.vm = __ldg(d.v + c - d.pi); x.vc = __ldg(d.v + c);
  x.wm = __ldg(d.w + c - d.np); x.wc = __ldg(d.w + c);
  x.fm = __ldg(d.f + c - 1); x.fc = __ldg(d.f + c);
  x.gm = __ldg(d.g + c - d.pi); x.gc = __ldg(d.g + c);
  x.hm = __ldg(d.h + c - d.np); x.hc = __ldg(d.h + c);
  return x;
}
template <bool P2, bool ZF>
__device__ __forceinline__ float rhs_comp(const LesDom &d, int i, int j, int k, const RhsIn &x, unsigned &bd) {
  const float *dzn = d.gr.dzn;
  const float hx = sx1<P2>(d, i), hy = sy1<P2>(d, j);
  const float rx = rx1<P2>(d, i), ry = ry1<P2>(d, j), rz = d.gr.rdzn[k];
  const float r = dvs<P2, ZF>(-x.um + x.uc, hx, rx, bd) + dvs<P2, ZF>(-x.vm + x.vc, hy, ry, bd) +
                  dvz<ZF>(-x.wm + x.wc, dzn[k], rz, bd);
  return dvs<P2, ZF>(x.fc - x.fm, hx, rx, bd) + dvs<P2, ZF>(x.gc - x.gm, hy, ry, bd) +
         dvz<ZF>(x.hc - x.hm, dzn[k], rz, bd) + dvz<ZF>(r, d.dt, d.rdt, bd);
}
template <bool P2, bool ZF>
__device__ __forceinline__ float rhs_cell(const LesDom &d, int i, int j, int k, int c, unsigned &bd) {
  return rhs_comp<P2, ZF>(d, i, j, k, rhs_load(d, c), bd);
}
// Compensated running sum of FP32 terms: hi by TwoSum, lo gathers the rounding errors.
struct PairSum {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float t) {
    float s, e;
    two_sum(hi, t, s, e);
    hi = s;
    lo += e;
  }
};
// Block sum of each thread's pair (BX x BY threads) into part[slot]: warp trees of
// pairs, then the warps in FP64 in order.
__device__ __forceinline__ void block_part(const LesDom &d, PairSum p, int slot) {
  __shared__ double sh[BX * BY / 32];
  const int tid = threadIdx.y * BX + threadIdx.x;
  float hi = p.hi, lo = p.lo;
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_down_sync(0xffffffffu, hi, o), l2 = __shfl_down_sync(0xffffffffu, lo, o);
    float s, e;
    two_sum(hi, h2, s, e);
    hi = s;
    lo = (lo + l2) + e;
  }
  if ((tid & 31) == 0) sh[tid >> 5] = (double)hi + (double)lo;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int q = 0; q < BX * BY / 32; ++q) s += sh[q];
    d.part[slot] = s;
  }
  __syncthreads();  // sh is reused when a fixup CTA loops over several blocks
}

// k planes per block of the reduction kernels (one partial per BX x BY x RKC cells)
constexpr int RKC = 16;
inline dim3 reduce_grid(const LesDom &d) { return dim3((d.im + BX - 1) / BX, (d.jm + BY - 1) / BY, (d.km + RKC - 1) / RKC); }

// rhs of the cells of block (bx, by, bz) -- columns (i, j), planes bz*RKC+1 .. -- plus
// its partial of sum(dx1*dy1*dzn*rhs) (press.f95:63-72).  dst: the rhs array (rhs =
// d.rhs) or the SOR's internal rhs buffer, which also takes periodic ghost copies of
// rows 1..4 in rows jm+1..jm+4 and of rows jm-3..jm in rows -3..0 (ghost_rows).  On that
// path p takes the same copies, so that the fused sweep's first iteration reads p by
// tensor copies: rows 0 and jm+1 already hold them (boundp, periodic in j), rows -3..-1
// and jm+3, jm+4 lie outside p's declared extent, and row jm+2, which lies inside it and
// which the reference's press never writes, is saved into d.prow first and put back by
// the sweep's copy-out (rhs reads no p).  ZF: reciprocal-corrected divisions;
// a block that met a dividend outside their range is recomputed whole by the fixup
// (rhs only reads u, v, w, f, g, h, so recomputing overwrites with the same cells).
// PG: also write p's ghost copies (the main kernel; its fixup recomputes deferred blocks'
// rhs only, the p copies having been written already)
template <bool P2, bool ZF, bool PG>
__device__ __forceinline__ void rhs_block(const LesDom &d, float *dst, int ghost, int bx, int by, int bz, uint3 g) {
  const int i0 = bx * BX + threadIdx.x + 1, j0 = by * BY + threadIdx.y + 1;
  const bool in = (i0 <= d.im && j0 <= d.jm);
  const int i = min(i0, d.im), j = min(j0, d.jm);  // past the edge: the edge cell again, not stored
  const int ka = bz * RKC + 1, kb = min(ka + RKC - 1, d.km);
  const float axy = d.gr.dx1[i] * d.gr.dy1[j];
  const unsigned gmask = ghost ? ghost_mask(j, d.jm) : 0u;  // periodic ghost copies of this row
  unsigned bd = 0;
  PairSum acc;
  // the loads of plane k+1 are issued before plane k's arithmetic
  int c = lix(d, i, j, ka);
  RhsIn cur = rhs_load(d, c);
  for (int k = ka; k <= kb; ++k) {
    RhsIn nxt = cur;
    if (k < kb) nxt = rhs_load(d, c + d.np);
    const float rr = rhs_comp<P2, ZF>(d, i, j, k, cur, bd);
    if (in) {
      dst[c] = rr;
      if (gmask) {
        const float pv = PG ? d.p[c] : 0.f;
        for_ghost_rows(d.jm, gmask, [&](int off) {
          dst[c + off * d.pi] = rr;
          if (PG) {
            if (j + off == d.jm + 2) d.prow[(k - 1) * d.im + (i - 1)] = d.p[c + off * d.pi];
            d.p[c + off * d.pi] = pv;
          }
        });
      }
      acc.add(axy * d.gr.dzn[k] * rr);
    }
    cur = nxt;
    c += d.np;
  }
  if (ZF && defer_block(bd, d.fix[FIX_RHS])) return;
  block_part(d, acc, (int)((bz * g.y + by) * g.x + bx));
}
template <bool P2, bool ZF>
__global__ void __launch_bounds__(BX *BY) k_rhs(LesDom d, float *dst, int ghost) {
  rhs_block<P2, ZF, true>(d, dst, ghost, blockIdx.x, blockIdx.y, blockIdx.z, make_uint3(gridDim.x, gridDim.y, gridDim.z));
}
template <bool P2>
__global__ void __launch_bounds__(BX *BY) k_rhs_fix(LesDom d, float *dst, int ghost, uint3 g) {
  for_deferred(d.fix[FIX_RHS], g, [&](int bx, int by, int bz) {
    rhs_block<P2, false, false>(d, dst, ghost, bx, by, bz, g);
  });
}
// pav partials: sum(p*dx1*dy1*dzn) (press.f95:124-133), one per block of RKC planes
__global__ void __launch_bounds__(BX *BY) k_pav_part(LesDom d) {
  const int i = blockIdx.x * BX + threadIdx.x + 1;
  const int j = blockIdx.y * BY + threadIdx.y + 1;
  const int ka = blockIdx.z * RKC + 1, kb = min(ka + RKC - 1, d.km);
  PairSum acc;
  if (i <= d.im && j <= d.jm) {
    const float dx = d.gr.dx1[i], dy = d.gr.dy1[j];
    for (int k = ka; k <= kb; ++k) acc.add(__ldg(d.p + lix(d, i, j, k)) * dx * dy * d.gr.dzn[k]);
  }
  block_part(d, acc, (int)((blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x));
}
// mean = (float)(sum of partials / area), summed in a fixed order: FIN_BLOCKS chunks,
// each a strided FP64 sum and a fixed tree, then the chunks in order by the last block
constexpr int FIN_BLOCKS = LES_FIN_BLOCKS, FIN_THREADS = 256;
__global__ void __launch_bounds__(FIN_THREADS) k_finish_mean(LesDom d, int nparts, int slot) {
  __shared__ double sh[FIN_THREADS / 32];
  __shared__ int last;
  const int chunk = (nparts + FIN_BLOCKS - 1) / FIN_BLOCKS;
  const int lo = blockIdx.x * chunk, hi = min(nparts, lo + chunk);
  double s = 0.0;
  for (int q = lo + (int)threadIdx.x; q < hi; q += FIN_THREADS) s += d.part[q];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < FIN_THREADS / 32; ++q) t += sh[q];
    d.part2[blockIdx.x] = t;
    __threadfence();
    last = (atomicAdd(d.cnt + 8, 1u) == FIN_BLOCKS - 1);
  }
  __syncthreads();
  if (!last || threadIdx.x >= 32) return;
  __threadfence();
  double t = 0.0;
  for (int q = (int)threadIdx.x; q < FIN_BLOCKS; q += 32) t += __ldcg(d.part2 + q);
  for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  if (threadIdx.x == 0) {
    const float mean = (float)(t / d.scal[SC_AREA]);
    d.fscal[slot] = mean;
    d.scal[slot] = (double)mean;
    d.cnt[8] = 0u;
  }
}
// a -= mean over the interior: one warp per row (j, k), float4 columns (interior rows
// start 16-byte aligned), the ragged end of a row one float at a time
constexpr int SUB_ROWS = 8;
__global__ void __launch_bounds__(32 * SUB_ROWS) k_sub_mean(LesDom d, float *a, int slot) {
  const int row = blockIdx.x * SUB_ROWS + (int)(threadIdx.x >> 5);  // (j-1) + jm*(k-1)
  if (row >= d.jm * d.km) return;
  const int lane = threadIdx.x & 31;
  const int j = row % d.jm + 1, k = row / d.jm + 1;
  float *r = a + lix(d, 1, j, k);
  const float m = d.fscal[slot];
  const int nq = d.im >> 2;
  float4 *r4 = reinterpret_cast<float4 *>(r);
  for (int q = lane; q < nq; q += 32) {
    float4 v = r4[q];
    v.x = v.x - m; v.y = v.y - m; v.z = v.z - m; v.w = v.w - m;
    r4[q] = v;
  }
  for (int i = 4 * nq + lane; i < d.im; i += 32) r[i] = r[i] - m;
}
inline unsigned sub_mean_blocks(const LesDom &d) { return (unsigned)((d.jm * d.km + SUB_ROWS - 1) / SUB_ROWS); }

// ------------------------------------------------------------------ press.f95:89-122
__global__ void k_sor_begin(LesDom d) {
  d.ctl[CT_CONVERGED] = 0;
  d.ctl[CT_ITERS] = 0;
  d.ctl[CT_REDO] = 0;
  d.ctl[CT_LASTBUF] = 2;
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
// boundp1 then boundp2 as one pass (the end of press): the i halos (Neumann) for j =
// 0..jm+1, then the periodic j halos for i = 0..im+1, then the k halos (Neumann) for
// i = 0..im+1, j = 0..jm+1, each reading what the one before wrote, compose to: a halo
// point takes the value at its source point, i clamped into 1..im, j = 0 -> jm and
// jm+1 -> 1, k clamped into 1..km.  No source point is a halo point, so the points are
// independent.  One thread per point of the k faces ((im+2) x (jm+2) each), the i faces
// (j = 0..jm+1, k = 1..km) and the j faces (i = 1..im, k = 1..km).
__global__ void k_boundp_all(LesDom d) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nk = (long long)(d.im + 2) * (d.jm + 2), ni = (long long)(d.jm + 2) * d.km,
                  nj = (long long)d.im * d.km;
  int i, j, k;
  if (t < 2 * nk) {
    const long long r = t % nk;
    k = (t < nk) ? 0 : d.km + 1;
    i = (int)(r % (d.im + 2));
    j = (int)(r / (d.im + 2));
  } else if (t < 2 * nk + 2 * ni) {
    const long long u = t - 2 * nk, r = u % ni;
    i = (u < ni) ? 0 : d.im + 1;
    j = (int)(r % (d.jm + 2));
    k = (int)(r / (d.jm + 2)) + 1;
  } else if (t < 2 * nk + 2 * ni + 2 * nj) {
    const long long u = t - 2 * nk - 2 * ni, r = u % nj;
    j = (u < nj) ? 0 : d.jm + 1;
    i = (int)(r % d.im) + 1;
    k = (int)(r / d.im) + 1;
  } else {
    return;
  }
  const int is = min(max(i, 1), d.im), js = (j == 0) ? d.jm : (j == d.jm + 1) ? 1 : j, ks = min(max(k, 1), d.km);
  d.p[lix(d, i, j, k)] = d.p[lix(d, is, js, ks)];
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

// the kernel variant for the domain's spacing modes (power-of-two x/y, div_k range)
#define LES_PZ_SWITCH(d, K, ...)                            \
  do {                                                      \
    if ((d).xy_pow2 && (d).zfast) K<true, true>__VA_ARGS__; \
    else if ((d).xy_pow2) K<true, false>__VA_ARGS__;        \
    else if ((d).zfast) K<false, true>__VA_ARGS__;          \
    else K<false, false>__VA_ARGS__;                        \
  } while (0)

// the fixup grid of a deferred-block list: a few CTAs per SM at most
inline unsigned fix_grid(const LesDom &d, dim3 g) {
  return std::min<unsigned>(g.x * g.y * g.z, (unsigned)std::max(1, 2 * d.sms));
}
inline uint3 u3(dim3 g) { return make_uint3(g.x, g.y, g.z); }

// feedbfm.f95:87-95 sets amask1 = 0 where the building top zbm(i,j) is above the cell
// centre z2(k) + 0.5*dzn(k); :106-116 set b, c, dmask1 = 1 there.  Every padded cell is
// written, halos and ground-free cells 0, so the result does not depend on what the
// mask buffer held.
__global__ void k_feedbfm(uint8_t *mask, const float *zbm, const float *thr, int im, int jm, int km, int pi, int nj) {
  const int ip = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (ip >= pi) return;
  const int i = ip - LES_IOFF, j = (int)blockIdx.y - LES_JOFF, k = (int)blockIdx.z - LES_KOFF;
  uint8_t m = 0;
  if (i >= 1 && i <= im && j >= 1 && j <= jm && k >= 1 && k <= km)
    m = zbm[(size_t)(i - 1) + (size_t)(j - 1) * im] > thr[k - 1] ? 7 : 0;
  mask[((size_t)blockIdx.z * nj + blockIdx.y) * pi + ip] = m;
}

void les_launch_feedbfm(uint8_t *mask, const float *zbm, const float *thr, int im, int jm, int km, int pi,
                        int nj, int nk, LesCtx ctx) {
  k_feedbfm<<<dim3((pi + 127) / 128, nj, nk), 128, 0, ctx.s>>>(mask, zbm, thr, im, jm, km, pi, nj);
  ++*ctx.nlaunch;
}

void les_launch_velnw(const LesDom &d, LesCtx ctx) {
  const dim3 g = interior_grid(d, (d.km + VNK - 1) / VNK), b(BX, BY);
  LAUNCH(ctx, LES_PZ_SWITCH(d, k_velnw, <<<g, b, 0, ctx.s>>>(d)));
  if (d.zfast) {
    if (d.xy_pow2) LAUNCH(ctx, (k_velnw_fix<true><<<fix_grid(d, g), b, 0, ctx.s>>>(d, u3(g))));
    else LAUNCH(ctx, (k_velnw_fix<false><<<fix_grid(d, g), b, 0, ctx.s>>>(d, u3(g))));
  }
}

// rhs into dst, its fixup, and the mean
static void launch_rhs(const LesDom &d, float *dst, int ghost, LesCtx ctx) {
  const dim3 g = reduce_grid(d), b(BX, BY);
  LAUNCH(ctx, LES_PZ_SWITCH(d, k_rhs, <<<g, b, 0, ctx.s>>>(d, dst, ghost)));
  if (d.zfast) {
    if (d.xy_pow2) LAUNCH(ctx, (k_rhs_fix<true><<<fix_grid(d, g), b, 0, ctx.s>>>(d, dst, ghost, u3(g))));
    else LAUNCH(ctx, (k_rhs_fix<false><<<fix_grid(d, g), b, 0, ctx.s>>>(d, dst, ghost, u3(g))));
  }
  LAUNCH(ctx, k_finish_mean<<<FIN_BLOCKS, FIN_THREADS, 0, ctx.s>>>(d, (int)(g.x * g.y * g.z), SC_RHSAV));
}

void les_launch_bondv1(const LesDom &d, int n, LesCtx ctx) {
  if (n == 1) {
    LAUNCH(ctx, k_bondv1_inflow<<<dim3((d.jm + 127) / 128, d.km), 128, 0, ctx.s>>>(d));
    LAUNCH(ctx, k_bondv1_fill<<<dim3((d.im - 1 + BX - 1) / BX, (d.jm + BY - 1) / BY, d.km), dim3(BX, BY), 0, ctx.s>>>(d));
    LAUNCH(ctx, k_bondv1_uout<false><<<UOUT_BLOCKS, UOUT_THREADS, 0, ctx.s>>>(d));
  } else {
    LAUNCH(ctx, k_bondv1_uout<true><<<UOUT_BLOCKS, UOUT_THREADS, 0, ctx.s>>>(d));
  }
  LAUNCH(ctx, k_bondv1_outflow<<<dim3((d.jm + 127) / 128, d.km), 128, 0, ctx.s>>>(d));
  const long long ns = 2LL * (d.im + 2) * (d.km + (d.jm + 2) + (d.jm + 3));
  LAUNCH(ctx, k_bondv1_sides<<<(unsigned)((ns + 255) / 256), 256, 0, ctx.s>>>(d));
}


void les_launch_feedbf(const LesDom &d, LesCtx ctx) {
  LAUNCH(ctx, k_feedbf<<<interior_grid(d, d.km), dim3(BX, BY), 0, ctx.s>>>(d));
}

void les_launch_boundsm(const LesDom &d, LesCtx ctx) {
  const long long n = 2LL * (d.im + 2) * (d.jm + 3) + 2LL * (d.jm + 3) * d.km + 2LL * d.im * d.km;
  LAUNCH(ctx, k_boundsm_all<<<(unsigned)((n + 255) / 256), 256, 0, ctx.s>>>(d));
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

int les_reduce_blocks(const LesDom &d) {
  const dim3 g = reduce_grid(d);
  return (int)(g.x * g.y * g.z);
}

void les_launch_rhs_mean(const LesDom &d, LesCtx ctx) {
  launch_rhs(d, d.rhs, 0, ctx);
  LAUNCH(ctx, k_sub_mean<<<sub_mean_blocks(d), 32 * SUB_ROWS, 0, ctx.s>>>(d, d.rhs, SC_RHSAV));
}

void les_launch_rhs_sor(const LesDom &d, LesCtx ctx) { launch_rhs(d, d.sorR, 1, ctx); }

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

void les_launch_interior_mean(const LesDom &d, LesCtx ctx) {
  const dim3 g = reduce_grid(d);
  LAUNCH(ctx, k_pav_part<<<g, dim3(BX, BY), 0, ctx.s>>>(d));
  LAUNCH(ctx, k_finish_mean<<<FIN_BLOCKS, FIN_THREADS, 0, ctx.s>>>(d, (int)(g.x * g.y * g.z), SC_PAV));
}

void les_launch_pav_adjust(const LesDom &d, LesCtx ctx) {
  const dim3 gr = reduce_grid(d);
  const int nb = (int)(gr.x * gr.y * gr.z);
  LAUNCH(ctx, k_pav_part<<<gr, dim3(BX, BY), 0, ctx.s>>>(d));
  LAUNCH(ctx, k_finish_mean<<<FIN_BLOCKS, FIN_THREADS, 0, ctx.s>>>(d, nb, SC_PAV));
  LAUNCH(ctx, k_sub_mean<<<sub_mean_blocks(d), 32 * SUB_ROWS, 0, ctx.s>>>(d, d.p, SC_PAV));
  const long long n = 2LL * (d.im + 2) * (d.jm + 2) + 2LL * (d.jm + 2) * d.km + 2LL * d.im * d.km;
  LAUNCH(ctx, k_boundp_all<<<(unsigned)((n + 255) / 256), 256, 0, ctx.s>>>(d));  // boundp1, boundp2
}

void les_launch_count_nonfinite(const LesDom &d, unsigned long long *bad, LesCtx ctx) {
  LAUNCH(ctx, k_count_nonfinite<<<interior_grid(d, d.km), dim3(BX, BY), 0, ctx.s>>>(d, bad));
}
