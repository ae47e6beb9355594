// les_sor2.cu -- two red-black SOR iterations in one k-march (press.f95:89-122).
//
// The one-iteration sweep (les_sor.cu) streams p and rhs from HBM once per iteration.
// Here iteration l+1 trails iteration l by two planes inside the same march, so p and
// rhs cross HBM once per two iterations.  At march step s a CTA performs, in order:
//   A  the red cells of plane s for iteration l     (old black neighbours),
//   B  the black cells of plane s-1 for iteration l  (red of l at s-2, s-1, s),
//   C  the red cells of plane s-2 for iteration l+1  (black of l at s-3, s-2, s-1),
//   D  the black cells of plane s-3 for iteration l+1 (red of l+1 at s-4, s-3, s-2),
// and stores plane s-3.  Every update reads exactly the values the reference's order
// (all red, boundp1, all black, boundp1, boundp2 per iteration) gives it, so the fields
// are bitwise those of two one-iteration sweeps; only the residual's summation order
// differs.
//
// Tile: 32 float4 columns (120 interior i cells and a 4-cell ring each side) by NY rows
// (NY-8 interior j rows and a 4-row ring each side, read from the buffers' four
// periodic ghost rows).  Each stage is valid on a ring one cell narrower than the one
// before: A on rows 1..NY-2, B on 2..NY-3, C on 3..NY-4, D (stored) on 4..NY-5; in i the
// outer ring cells go stale one per stage and never reach the interior.  In-plane j
// neighbours come from shared memory: the TMA-staged old plane for A, and for B, C, D
// the previous step's outputs of A, B, C (one plane each, written after a second
// barrier per step).  i neighbours at float4 edges come by warp shuffle; k neighbours
// from a five-plane register window per thread (compile-time slots, the march unrolled
// five times).  The k halos p(0) = p(1), p(km+1) = p(km) (boundp2) are copies in the
// window's plane-0 and plane-(km+1) slots, refreshed after iteration l's black pass.
//
// Residuals: iteration l (A + B) and l+1 (C + D) are summed separately over the owned
// cells, FP32 per thread (Kahan across groups of five planes), FP64 per CTA, and the
// last CTA finishes both.  Early exit (press.f95:119-121): if iteration l already met
// sor < pjuge, the launch flags CT_REDO and the next launch in the step (a one-iteration
// sweep in redo mode) recomputes iteration l alone from the same source into the same
// destination; the iteration count and residual are those of iteration l.
#include <cuda.h>
#include <cuda_runtime.h>

#include "les_common.cuh"
#include "les_sor.cuh"
#include "les_sor_kern.cuh"

namespace {

constexpr int T2X = 32;             // float4 columns per tile row (one warp)
constexpr int T2I = 4 * T2X - 8;    // interior i cells per tile (120)
constexpr int DPS = 4, DRS = 6;     // TMA ring stages of p and of rhs

template <int NY>
struct Sor2Smem {
  float4 p[DPS][NY][T2X];    // old p planes (TMA)
  float4 rhs[DRS][NY][T2X];  // rhs planes (TMA)
  float4 st[3][NY][T2X];     // previous step's outputs of stages A, B, C
  float c4l[LES_SOR_KMAX], c4s[LES_SOR_KMAX], ck[LES_SOR_KMAX];
  uint64_t barp[DPS], barr[DRS];
  double warp[2][NY];
  int last, abort_;
};

template <int U>
struct IC5 {
  static constexpr int value = U;
};

// Residuals of both iterations: warp sums, FP64 per CTA (partials [cta] and
// [ntiles + cta]), the last CTA sums them in order and applies the exit test.
template <int NY>
__device__ __forceinline__ void finish_residual2(const LesDom &d, const SorArgs &a, float acc0, float acc1,
                                                 double (*warp)[NY], int *last) {
  const int lane = threadIdx.x, wid = threadIdx.y, tid = wid * T2X + lane;
  float x0 = acc0, x1 = acc1;
  for (int o = 16; o > 0; o >>= 1) {
    x0 += __shfl_down_sync(0xffffffffu, x0, o);
    x1 += __shfl_down_sync(0xffffffffu, x1, o);
  }
  if (lane == 0) {
    warp[0][wid] = (double)x0;
    warp[1][wid] = (double)x1;
  }
  __syncthreads();
  const int cta = blockIdx.y * gridDim.x + blockIdx.x;
  if (tid == 0) {
    double t0 = 0.0, t1 = 0.0;
    for (int q = 0; q < NY; ++q) {
      t0 += warp[0][q];
      t1 += warp[1][q];
    }
    a.part[cta] = t0;
    a.part[a.ntiles + cta] = t1;
    __threadfence();
    *last = (atomicAdd(a.counter, 1u) == (unsigned)(a.ntiles - 1));
  }
  __syncthreads();
  if (!*last) return;
  __threadfence();
  double t0 = 0.0, t1 = 0.0;
  for (int q = tid; q < a.ntiles; q += T2X * NY) {
    t0 += ((volatile double *)a.part)[q];
    t1 += ((volatile double *)a.part)[a.ntiles + q];
  }
  for (int o = 16; o > 0; o >>= 1) {
    t0 += __shfl_down_sync(0xffffffffu, t0, o);
    t1 += __shfl_down_sync(0xffffffffu, t1, o);
  }
  if (lane == 0) {
    warp[0][wid] = t0;
    warp[1][wid] = t1;
  }
  __syncthreads();
  if (tid == 0) {
    double tot0 = 0.0, tot1 = 0.0;
    for (int q = 0; q < NY; ++q) {
      tot0 += warp[0][q];
      tot1 += warp[1][q];
    }
    d.ctl[CT_LASTBUF] = a.dstcode;
    if (!d.sor_fixed && tot0 < (double)d.pjuge) {  // iteration l met the exit test: undo l+1
      d.scal[SC_SOR] = tot0;
      d.ctl[CT_ITERS] += 1;
      d.ctl[CT_CONVERGED] = 1;
      d.ctl[CT_REDO] = 1;
    } else {
      d.scal[SC_SOR] = tot1;
      d.ctl[CT_ITERS] += 2;
      if (!d.sor_fixed && tot1 < (double)d.pjuge) d.ctl[CT_CONVERGED] = 1;
    }
    *a.counter = 0u;
  }
}

template <int NY>
__global__ void __launch_bounds__(T2X *NY, 1)
    k_sor_tma2(LesDom d, SorArgs a, const __grid_constant__ CUtensorMap tmP, const __grid_constant__ CUtensorMap tmR) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  Sor2Smem<NY> &S = *reinterpret_cast<Sor2Smem<NY> *>(smem_raw);
  if (d.ctl[CT_CONVERGED]) return;  // early exit of press.f95:119-121

  constexpr int TJ = NY - 8;
  const int c4 = threadIdx.x, r = threadIdx.y;
  const int km = d.km;
  const int i0 = 1 + (int)blockIdx.x * T2I, j0 = 1 + (int)blockIdx.y * TJ;
  const int ib = i0 - 4 + 4 * c4, jr = j0 - 4 + r;
  const bool rowA = (r >= 1) && (r <= NY - 2), rowB = (r >= 2) && (r <= NY - 3);
  const bool rowC = (r >= 3) && (r <= NY - 4), rowD = (r >= 4) && (r <= NY - 5);
  const bool owned = rowD && (jr <= d.jm) && (c4 >= 1) && (c4 <= T2X - 2);
  bool ival[4];
  float m[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    ival[e] = (ib + e >= 1) && (ib + e <= d.im);
    m[e] = (owned && ival[e]) ? 1.f : 0.f;
  }
  const bool west0 = (ib == 1);
  const int east_e = d.im - ib;
  const unsigned gmask = ghost_mask(jr, d.jm);
  const float c2l_ = d.gr.cn2l[1], c2s_ = d.gr.cn2s[1];
  const float c2l[4] = {c2l_, c2l_, c2l_, c2l_}, c2s[4] = {c2s_, c2s_, c2s_, c2s_};
  const float c3l = d.gr.cn3l[1], c3s = d.gr.cn3s[1];
  const float rhsav = d.fscal[SC_RHSAV];
  constexpr float omega = 1.f;  // press.f95:45, the only value this kernel is launched for
  const bool producer = (r == 0) && (c4 == 0);
  const int tx = (int)blockIdx.x * T2I;                 // padded column of i0 - 4
  const int ty = (int)blockIdx.y * TJ + (LES_JOFF - 3);  // padded row of j0 - 4
  constexpr uint32_t plane_bytes = (uint32_t)(NY * T2X * 16);

  auto issue_p = [&](int mm) {
    const int q = (mm - 1) % DPS;
    mbar_expect_tx(&S.barp[q], plane_bytes);
    tma_load_3d(&S.p[q][0][0], &tmP, tx, ty, mm + LES_KOFF, &S.barp[q]);
  };
  auto issue_r = [&](int mm) {
    const int q = (mm - 1) % DRS;
    mbar_expect_tx(&S.barr[q], plane_bytes);
    tma_load_3d(&S.rhs[q][0][0], &tmR, tx, ty, mm + LES_KOFF, &S.barr[q]);
  };
  if (producer) {
    for (int q = 0; q < DPS; ++q) mbar_init(&S.barp[q], 1);
    for (int q = 0; q < DRS; ++q) mbar_init(&S.barr[q], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    S.abort_ = 0;
  }
  for (int q = r * T2X + c4; q <= km; q += T2X * NY) {
    if (q >= 1) {
      S.c4l[q] = d.gr.cn4l[q];
      S.c4s[q] = d.gr.cn4s[q];
      S.ck[q] = d.gr.cn1k[q];
    }
  }
  __syncthreads();
  if (producer) {
    for (int mm = 1; mm <= DPS && mm <= km; ++mm) issue_p(mm);
    for (int mm = 1; mm <= DRS && mm <= km; ++mm) issue_r(mm);
  }
  int failed = 0;  // a bounded wait gave up: stop computing, keep meeting the barriers
  auto wait_p = [&](int mm) {
    if (!mbar_wait(&S.barp[(mm - 1) % DPS], (uint32_t)(((mm - 1) / DPS) & 1))) {
      S.abort_ = 1;
      d.ctl[CT_ERROR] = 1;
      failed = 1;
    }
  };
  auto wait_r = [&](int mm) {
    if (!mbar_wait(&S.barr[(mm - 1) % DRS], (uint32_t)(((mm - 1) / DRS) & 1))) {
      S.abort_ = 1;
      d.ctl[CT_ERROR] = 1;
      failed = 1;
    }
  };
  if (km >= 1) wait_p(1);

  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 W[5];  // plane t of this column in slot t % 5
#pragma unroll
  for (int t = 0; t < 5; ++t) W[t] = zero4;
  float acc0 = 0.f, comp0 = 0.f, grp0 = 0.f, acc1 = 0.f, comp1 = 0.f, grp1 = 0.f;
  auto fold = [&]() {
    {
      const float y = grp0 - comp0, t = acc0 + y;
      comp0 = (t - acc0) - y;
      acc0 = t;
    }
    {
      const float y = grp1 - comp1, t = acc1 + y;
      comp1 = (t - acc1) - y;
      acc1 = t;
    }
    grp0 = grp1 = 0.f;
  };

  auto store = [&](int k, const float4 &v) {
    auto put = [&](int jrow) {
      float *dst = a.pdst + (k + LES_KOFF) * d.np + (jrow + LES_JOFF) * d.pi + ib + LES_IOFF;
      if (ival[0] && ival[3]) {
        *reinterpret_cast<float4 *>(dst) = v;
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (ival[e]) dst[e] = f4get(v, e);
      }
    };
    put(jr);
    if (a.ghost) for_ghost_rows(d.jm, gmask, [&](int off) { put(jr + off); });
  };

  auto step = [&](auto UC, int s) {
    constexpr int U = decltype(UC)::value;  // s = U modulo 5
    constexpr int S0 = U, SM1 = (U + 4) % 5, SM2 = (U + 3) % 5, SM3 = (U + 2) % 5, SM4 = (U + 1) % 5;
    __syncthreads();
    const bool ab = S.abort_ != 0;
    if (!ab) {
      // stages freed by step s-1: p of plane s-1, rhs of plane s-4
      if (producer) {
        if (s - 1 >= 1 && s - 1 + DPS <= km) issue_p(s - 1 + DPS);
        if (s - 4 >= 1 && s - 4 + DRS <= km) issue_r(s - 4 + DRS);
      }
      const int q = (jr + s) & 1;  // red elements of plane s (= black of s-1, red of s-2, black of s-3)
      float part0 = 0.f, part1 = 0.f;
      // ---- A: red cells of plane s, iteration l
      if (s <= km) {
        if (s + 1 <= km) wait_p(s + 1);
        wait_r(s);
        const int sp = (s - 1) % DPS;
        W[S0] = S.p[sp][r][c4];
        if (s == 1) W[SM1] = W[S0];  // plane 0 reads as plane 1 (boundp2), before its red update
        const float4 pup = (s < km) ? S.p[s % DPS][r][c4] : W[S0];
        const float pl = __shfl_up_sync(0xffffffffu, W[S0].w, 1);
        const float pr = __shfl_down_sync(0xffffffffu, W[S0].x, 1);
        if (rowA) {
          const float4 pn = S.p[sp][r + 1][c4], ps = S.p[sp][r - 1][c4];
          const float4 rr = S.rhs[(s - 1) % DRS][r][c4];
          part0 += relax_pair_m(q, W[S0], pl, pr, pn, ps, pup, W[SM1], rr, rhsav, omega, S.ck[s], c2l, c2s, c3l,
                                c3s, S.c4l[s], S.c4s[s], west0, east_e, m);
        }
      }
      // ---- B: black cells of plane s-1, iteration l
      if (s - 1 >= 1 && s - 1 <= km) {
        const int k = s - 1;
        if (k == km) W[S0] = W[SM1];  // plane km+1 reads as plane km (its black cells still old)
        const float pl = __shfl_up_sync(0xffffffffu, W[SM1].w, 1);
        const float pr = __shfl_down_sync(0xffffffffu, W[SM1].x, 1);
        if (rowB) {
          const float4 pn = S.st[0][r + 1][c4], ps = S.st[0][r - 1][c4];
          const float4 rr = S.rhs[(k - 1) % DRS][r][c4];
          part0 += relax_pair_m(q, W[SM1], pl, pr, pn, ps, W[S0], W[SM2], rr, rhsav, omega, S.ck[k], c2l, c2s, c3l,
                                c3s, S.c4l[k], S.c4s[k], west0, east_e, m);
        }
        if (k == 1) W[SM2] = W[SM1];  // plane 0 := plane 1 after iteration l (boundp2)
        if (k == km) W[S0] = W[SM1];  // plane km+1 := plane km after iteration l
      }
      // ---- C: red cells of plane s-2, iteration l+1
      if (s - 2 >= 1 && s - 2 <= km) {
        const int k = s - 2;
        const float pl = __shfl_up_sync(0xffffffffu, W[SM2].w, 1);
        const float pr = __shfl_down_sync(0xffffffffu, W[SM2].x, 1);
        if (rowC) {
          const float4 pn = S.st[1][r + 1][c4], ps = S.st[1][r - 1][c4];
          const float4 rr = S.rhs[(k - 1) % DRS][r][c4];
          part1 += relax_pair_m(q, W[SM2], pl, pr, pn, ps, W[SM1], W[SM3], rr, rhsav, omega, S.ck[k], c2l, c2s, c3l,
                                c3s, S.c4l[k], S.c4s[k], west0, east_e, m);
        }
      }
      // ---- D: black cells of plane s-3, iteration l+1; plane s-3 is final
      if (s - 3 >= 1 && s - 3 <= km) {
        const int k = s - 3;
        const float pl = __shfl_up_sync(0xffffffffu, W[SM3].w, 1);
        const float pr = __shfl_down_sync(0xffffffffu, W[SM3].x, 1);
        if (rowD) {
          const float4 pn = S.st[2][r + 1][c4], ps = S.st[2][r - 1][c4];
          const float4 rr = S.rhs[(k - 1) % DRS][r][c4];
          part1 += relax_pair_m(q, W[SM3], pl, pr, pn, ps, W[SM2], W[SM4], rr, rhsav, omega, S.ck[k], c2l, c2s, c3l,
                                c3s, S.c4l[k], S.c4s[k], west0, east_e, m);
          if (owned) store(k, W[SM3]);
        }
      }
      grp0 += part0;
      grp1 += part1;
    }
    __syncthreads();
    if (!ab) {  // this step's outputs of A, B, C: the in-plane neighbours of the next step
      S.st[0][r][c4] = W[S0];
      S.st[1][r][c4] = W[SM1];
      S.st[2][r][c4] = W[SM2];
    }
  };
  const int s_end = km + 3;
  for (int s0 = 0; s0 <= s_end; s0 += 5) {
    if (s0 >= 1) step(IC5<0>{}, s0);
    if (s0 + 1 > s_end) break;
    step(IC5<1>{}, s0 + 1);
    if (s0 + 2 > s_end) break;
    step(IC5<2>{}, s0 + 2);
    if (s0 + 3 > s_end) break;
    step(IC5<3>{}, s0 + 3);
    if (s0 + 4 > s_end) break;
    step(IC5<4>{}, s0 + 4);
    fold();
  }
  fold();
  // after a failed wait, wait (bounded) for every copy this CTA issued before leaving
  if (failed) {
    for (int q = 0; q < DPS; ++q) (void)mbar_wait(&S.barp[q], 0u), (void)mbar_wait(&S.barp[q], 1u);
    for (int q = 0; q < DRS; ++q) (void)mbar_wait(&S.barr[q], 0u), (void)mbar_wait(&S.barr[q], 1u);
  }
  finish_residual2<NY>(d, a, acc0, acc1, S.warp, &S.last);
}

template <int NY>
void launch2(const LesDom &d, const SorArgs &a, const CUtensorMap &tp, const CUtensorMap &tr, cudaStream_t s) {
  const dim3 grid((d.im + T2I - 1) / T2I, (d.jm + (NY - 8) - 1) / (NY - 8), 1);
  const size_t bytes = sizeof(Sor2Smem<NY>);
  cudaFuncSetAttribute(k_sor_tma2<NY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k_sor_tma2<NY><<<grid, dim3(T2X, NY), bytes, s>>>(d, a, tp, tr);
}

}  // namespace

bool les_sor_two_ok(const LesDom &d, SorShape sh) {
  return sh.depth == 2 && sh.nx == 32 && (sh.ny == 24 || sh.ny == 28 || sh.ny == 32) &&
         (sh.kchunk <= 0 || sh.kchunk >= d.km) && d.gr.cn1k && !d.cn1 && d.omega == 1.f && d.sor_uni &&
         d.km + 1 < LES_SOR_KMAX && d.jm % 2 == 0 && d.jm >= 4;
}

void les_launch_sor_iter2(const LesDom &d, const SorArgs &a, int ny, const CUtensorMap &tp, const CUtensorMap &tr,
                          cudaStream_t s) {
  switch (ny) {
    case 24: launch2<24>(d, a, tp, tr, s); break;
    case 32: launch2<32>(d, a, tp, tr, s); break;
    default: launch2<28>(d, a, tp, tr, s); break;
  }
}
