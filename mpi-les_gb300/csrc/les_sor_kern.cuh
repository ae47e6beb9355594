// les_sor_kern.cuh -- device code of the fused red-black SOR sweep (press.f95:89-122),
// templated on the tile shape.  Included by les_sor.cu (32-column tiles) and
// les_sor16.cu (16-column tiles) so the two families compile in parallel; the
// algorithm is described at the top of les_sor.cu.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "les_common.cuh"
#include "les_sor.cuh"
#include "les_tma.cuh"

namespace {

// A tile row is NX float4 columns: NX = 32 (one warp, 120 interior i cells) or NX = 16
// (half a warp, 56 cells).  The first and last column are the two-cell i ring.
__host__ __device__ constexpr int tile_i(int nx) { return 4 * nx - 8; }

__device__ __forceinline__ float f4get(const float4 &v, int e) {
  return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w;
}
__device__ __forceinline__ void f4set(float4 &v, int e, float x) {
  if (e == 0) v.x = x; else if (e == 1) v.y = x; else if (e == 2) v.z = x; else v.w = x;
}

// One relaxation: reltmp = omega*(cn1*(sum of neighbour terms - rhs) - p), left to right.
__device__ __forceinline__ float relax(float omega, float cn1, float c2l, float pe, float c2s, float pw,
                                       float c3l, float pn, float c3s, float ps, float c4l, float pu,
                                       float c4s, float pd, float rhs, float pc) {
  return omega * (cn1 * (c2l * pe + c2s * pw + c3l * pn + c3s * ps + c4l * pu + c4s * pd - rhs) - pc);
}

// Relaxation of element E of a float4 (one code path for every lane): the west and
// east neighbours come from the float4 itself or, at its edges, from the neighbouring
// columns (pl, pr); at i = 1 and i = im the virtual Neumann halos p(0) = p(1) and
// p(im+1) = p(im) are selected instead.
template <int E>
__device__ __forceinline__ float relax_e(const float4 &cur, float pl, float pr, const float4 &pn,
                                         const float4 &pso, const float4 &pu, const float4 &pdn,
                                         const float4 &rr, float rhsav, float omega, float cn1,
                                         const float (&c2l)[4], const float (&c2s)[4], float c3l, float c3s,
                                         float c4l, float c4s, bool west_wall, bool east_wall) {
  const float pc = f4get(cur, E);
  float pw = (E == 0) ? pl : f4get(cur, E - 1);
  float pe = (E == 3) ? pr : f4get(cur, E + 1);
  pw = west_wall ? pc : pw;
  pe = east_wall ? pc : pe;
  return relax(omega, cn1, c2l[E], pe, c2s[E], pw, c3l, f4get(pn, E), c3s, f4get(pso, E), c4l,
               f4get(pu, E), c4s, f4get(pdn, E), f4get(rr, E) - rhsav, pc);
}

// Red (or black) cells of one float4: e = q and q+2, with q = (j+s) mod 2 (the i of
// element 0 is odd).  Returns the summed squares of the owned corrections.
__device__ __forceinline__ float relax_pair(int q, float4 &cur, float pl, float pr, const float4 &pn,
                                            const float4 &pso, const float4 &pu, const float4 &pdn,
                                            const float4 &rr, float rhsav, float omega, float cn1,
                                            const float (&c2l)[4], const float (&c2s)[4], float c3l, float c3s,
                                            float c4l, float c4s, bool west0, int east_e, bool own,
                                            const bool (&ival)[4]) {
  const float4 c = cur;
  float part;
  if (q == 0) {
    const float ra = relax_e<0>(c, pl, pr, pn, pso, pu, pdn, rr, rhsav, omega, cn1, c2l, c2s, c3l, c3s, c4l, c4s, west0, east_e == 0);
    const float rb = relax_e<2>(c, pl, pr, pn, pso, pu, pdn, rr, rhsav, omega, cn1, c2l, c2s, c3l, c3s, c4l, c4s, false, east_e == 2);
    cur.x = c.x + ra;
    cur.z = c.z + rb;
    part = (own && ival[0] ? ra * ra : 0.f) + (own && ival[2] ? rb * rb : 0.f);
  } else {
    const float ra = relax_e<1>(c, pl, pr, pn, pso, pu, pdn, rr, rhsav, omega, cn1, c2l, c2s, c3l, c3s, c4l, c4s, false, east_e == 1);
    const float rb = relax_e<3>(c, pl, pr, pn, pso, pu, pdn, rr, rhsav, omega, cn1, c2l, c2s, c3l, c3s, c4l, c4s, false, east_e == 3);
    cur.y = c.y + ra;
    cur.w = c.w + rb;
    part = (own && ival[1] ? ra * ra : 0.f) + (own && ival[3] ? rb * rb : 0.f);
  }
  return part;
}

// relax_pair for the TMA march: the squared corrections of the relaxed elements are
// weighted by m[e] (1 for the cells this thread owns, 0 for ring and outside cells:
// multiplies, which the FP pipe has room for, instead of selects).
__device__ __forceinline__ float relax_pair_m(int q, float4 &cur, float pl, float pr, const float4 &pn,
                                              const float4 &pso, const float4 &pu, const float4 &pdn,
                                              const float4 &rr, float rhsav, float omega, float cn1,
                                              const float (&c2l)[4], const float (&c2s)[4], float c3l, float c3s,
                                              float c4l, float c4s, bool west0, int east_e, const float (&m)[4]) {
  const float4 c = cur;
  if (q == 0) {
    const float ra = relax_e<0>(c, pl, pr, pn, pso, pu, pdn, rr, rhsav, omega, cn1, c2l, c2s, c3l, c3s, c4l, c4s,
                                west0, east_e == 0);
    const float rb = relax_e<2>(c, pl, pr, pn, pso, pu, pdn, rr, rhsav, omega, cn1, c2l, c2s, c3l, c3s, c4l, c4s,
                                false, east_e == 2);
    cur.x = c.x + ra;
    cur.z = c.z + rb;
    return ra * ra * m[0] + rb * rb * m[2];
  }
  const float ra = relax_e<1>(c, pl, pr, pn, pso, pu, pdn, rr, rhsav, omega, cn1, c2l, c2s, c3l, c3s, c4l, c4s,
                              false, east_e == 1);
  const float rb = relax_e<3>(c, pl, pr, pn, pso, pu, pdn, rr, rhsav, omega, cn1, c2l, c2s, c3l, c3s, c4l, c4s,
                              false, east_e == 3);
  cur.y = c.y + ra;
  cur.w = c.w + rb;
  return ra * ra * m[1] + rb * rb * m[3];
}

// Per-thread geometry shared by both kernels.
struct Lane {
  int c4, r, ib, jr, jw;
  bool row_owned, row_red, col_owned, owned, west0;
  int east_e;
  bool ival[4];
  // periodic ghost rows that copy row jr (NO_GHOST: none): rows jm+1.., -1.. for the
  // two-row ghost band (SorArgs.ghost 1), jm+1..jm+4, -3..0 for the four-row band
  // (ghost 2, jm >= 4: at most two per row).  Held as two precomputed rows: a general
  // loop over the candidates costs the sweep 3% (97.5 against 100.6 us per iteration).
  int ghost1, ghost2;
};

// bx, by: the tile's column and row in the domain's tile grid; ghost: SorArgs.ghost
constexpr int NO_GHOST = -1000;
template <int NX>
__device__ __forceinline__ Lane make_lane(const LesDom &d, int tj, int ny, int bx, int by, int ghost) {
  Lane L;
  L.c4 = threadIdx.x;
  // 16-column tiles: a warp holds two rows two apart (rows 0,2 | 1,3 | 4,6 | 5,7 ...), so
  // both rows have the same red/black parity and the colour branch stays warp-uniform
  L.r = (NX == 16) ? 4 * ((int)threadIdx.y >> 2) + (((int)threadIdx.y >> 1) & 1) + 2 * ((int)threadIdx.y & 1)
                   : (int)threadIdx.y;
  const int i0 = 1 + bx * tile_i(NX);
  const int j0 = 1 + by * tj;
  L.ib = i0 - 4 + 4 * L.c4;
  L.jr = j0 - 2 + L.r;
  int jw = (L.jr - 1) % d.jm;
  if (jw < 0) jw += d.jm;
  L.jw = jw + 1;
  L.row_owned = (L.r >= 2) && (L.r <= ny - 3) && (L.jr <= d.jm);
  L.row_red = (L.r >= 1) && (L.r <= ny - 2);
  L.col_owned = (L.c4 >= 1) && (L.c4 <= NX - 2);
  L.owned = L.row_owned && L.col_owned;
  L.west0 = (L.ib == 1);
  L.east_e = d.im - L.ib;
#pragma unroll
  for (int e = 0; e < 4; ++e) L.ival[e] = (L.ib + e >= 1) && (L.ib + e <= d.im);
  const int band = (ghost == 2) ? 4 : 2;
  L.ghost1 = (L.jr <= band && L.jr >= 1) ? L.jr + d.jm : NO_GHOST;
  L.ghost2 = (L.jr > d.jm - band && L.jr <= d.jm) ? L.jr - d.jm : NO_GHOST;
  return L;
}

// Store the final float4 of plane k (owned cells), plus its periodic ghost rows when
// the destination is an internal buffer.
__device__ __forceinline__ void store_final(const LesDom &d, const SorArgs &a, const Lane &L, int k,
                                            const float4 &v) {
  auto put = [&](int jrow) {
    float *dst = a.pdst + (k + LES_KOFF) * d.np + (jrow + LES_JOFF) * d.pi + L.ib + LES_IOFF;
    if (L.ival[0] && L.ival[3]) {
      *reinterpret_cast<float4 *>(dst) = v;
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (L.ival[e]) dst[e] = f4get(v, e);
    }
  };
  put(L.jr);
  if (a.ghost) {
    if (L.ghost1 != NO_GHOST) put(L.ghost1);
    if (L.ghost2 != NO_GHOST) put(L.ghost2);
  }
}

// FP32 (Kahan) per thread -> FP64 per CTA -> last CTA sums the CTA partials in order.
// warp[] holds one double per warp of the CTA (NX * NY / 32).
// cta: the CTA's index among the a.ntiles partials of this iteration
template <int NX, int NY>
__device__ __forceinline__ void finish_residual(const LesDom &d, const SorArgs &a, float acc, double *warp,
                                                int *last, int cta) {
  constexpr int NW = NX * NY / 32;
  const int tid = threadIdx.y * NX + threadIdx.x, lane = tid & 31, wid = tid >> 5;
  float x = acc;
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  if (lane == 0) warp[wid] = (double)x;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int q = 0; q < NW; ++q) t += warp[q];
    a.part[cta] = t;
    __threadfence();
    const unsigned ticket = atomicAdd(a.counter, 1u);
    *last = (ticket == (unsigned)(a.ntiles - 1));
  }
  __syncthreads();
  if (*last && a.redo) {  // a recomputed first iteration: its residual is already recorded
    if (tid == 0) {
      d.ctl[CT_REDO] = 0;
      *a.counter = 0u;
    }
    return;
  }
  if (*last) {
    __threadfence();
    double t = 0.0;
    for (int q = tid; q < a.ntiles; q += NX * NY) t += ((volatile double *)a.part)[q];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) warp[wid] = t;
    __syncthreads();
    if (tid == 0) {
      double tot = 0.0;
      for (int q = 0; q < NW; ++q) tot += warp[q];
      d.scal[SC_SOR] = tot;
      d.ctl[CT_ITERS] += 1;
      d.ctl[CT_LASTBUF] = a.dstcode;
      if (!d.sor_fixed && tot < (double)d.pjuge) d.ctl[CT_CONVERGED] = 1;
      *a.counter = 0u;
    }
  }
}

template <int N>
struct IC {
  static constexpr int value = N;
};

// ---------------------------------------------------------------------------------
// Register kernel: each thread loads its own float4 columns straight into registers,
// prefetched three march steps ahead.  Reads j ring rows by wrapping, so it runs on p
// itself (the first iteration) and on any cn1 (uniform, stored or separable).
// CTAs per SM the launch bounds ask for: a 16-column tile is half the threads, so two
// of them share an SM.
__host__ __device__ constexpr int min_ctas(int nx) { return nx == 16 ? 2 : 1; }

template <int NX, int NY, int CN1MODE, bool KC>
__global__ void __launch_bounds__(NX *NY, min_ctas(NX)) k_sor_reg(LesDom d, SorArgs a) {
  __shared__ float4 sOld[2][NY][NX];
  __shared__ float4 sRed[2][NY][NX];
  __shared__ float sC4l[LES_SOR_KMAX], sC4s[LES_SOR_KMAX], sCk[LES_SOR_KMAX];
  __shared__ double sWarp[NX * NY / 32];
  __shared__ int sLast;
  // early exit of press.f95:119-121; in redo mode: run only when a two-iteration launch
  // must be cut back to its first iteration
  if (a.redo ? d.ctl[CT_REDO] == 0 : d.ctl[CT_CONVERGED] != 0) return;

  const Lane L = make_lane<NX>(d, a.tj, NY, blockIdx.x, blockIdx.y, a.ghost);
  const int c4 = L.c4, r = L.r, ib = L.ib, jw = L.jw;
  const int im = d.im, jm = d.jm, km = d.km;
  const bool col_load = (ib <= im + 1);
  // this CTA's k chunk [ka, kb], marched from ka-1 (a red ring plane) to kb+1
  const int ka = KC ? 1 + (int)blockIdx.z * a.kchunk : 1;
  const int kb = KC ? min(km, ka + a.kchunk - 1) : km;
  const int s_begin = KC ? max(1, ka - 1) : 1;
  const int s_end = KC ? min(km + 1, kb + 1) : km + 1;

  for (int q = r * NX + c4; q <= km; q += NX * NY) {
    if (q >= 1) {
      sC4l[q] = d.gr.cn4l[q];
      sC4s[q] = d.gr.cn4s[q];
      sCk[q] = (CN1MODE == 0) ? d.gr.cn1k[q] : d.gr.cn1c[q];
    }
  }
  float c2l[4], c2s[4], cn1a[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = ib + e;
    c2l[e] = L.ival[e] ? d.gr.cn2l[i] : 0.f;
    c2s[e] = L.ival[e] ? d.gr.cn2s[i] : 0.f;
    cn1a[e] = L.ival[e] ? d.gr.cn1a[i] : 0.f;
  }
  const float c3l = d.gr.cn3l[jw], c3s = d.gr.cn3s[jw];
  const float cn1b = d.gr.cn1b[jw];
  const float rhsav = d.fscal[SC_RHSAV];
  const float omega = d.omega;
  const float *__restrict__ ps = a.psrc;
  const float *__restrict__ rh = a.rhs;
  const int colbase = (jw + LES_JOFF) * d.pi + ib + LES_IOFF;  // + (k+1)*np
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);

  // plane 0 and plane km+1 are read as planes 1 and km (boundp2's Neumann copies)
  auto ldp = [&](int k) -> float4 {
    if (!col_load || k > km + 1) return zero4;
    const int kk = (k == 0) ? 1 : (k == km + 1) ? km : k;
    return __ldg(reinterpret_cast<const float4 *>(ps + (kk + LES_KOFF) * d.np + colbase));
  };
  auto ldr = [&](int k) -> float4 {
    if (!col_load || k < 1 || k > km || !L.row_red) return zero4;
    return __ldg(reinterpret_cast<const float4 *>(rh + (k + LES_KOFF) * d.np + colbase));
  };
  auto cn1_at = [&](int e, int k) -> float {
    if (CN1MODE == 1) return d.cn1[(ib + e - 1) + (jw - 1) * im + (k - 1) * im * jm];
    return 1.f / (cn1a[e] + cn1b + sCk[k]);
  };

  // Register rings: plane q of p lives in P[q % 6], plane q of rhs in R[q % 6].  The
  // march is unrolled 6 times so every slot index is a compile-time constant: the
  // loads issued for planes s+4 (p) and s+3 (rhs) land in the slots just freed and are
  // first used three steps later, so their latency overlaps three steps of work.
  float4 P[6], R[6];
  if (!KC) {
    P[0] = ldp(0); P[1] = ldp(1); P[2] = ldp(2); P[3] = ldp(3); P[4] = ldp(4); P[5] = zero4;
    R[0] = zero4; R[1] = ldr(1); R[2] = ldr(2); R[3] = ldr(3); R[4] = zero4; R[5] = zero4;
  } else {
    // planes s_begin-1 .. s_begin+3 of p and s_begin .. s_begin+2 of rhs, in slot plane % 6
#pragma unroll
    for (int t = 0; t < 6; ++t) P[t] = R[t] = zero4;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      const int m = s_begin - 1 + q, slot = m % 6;
#pragma unroll
      for (int t = 0; t < 6; ++t)
        if (t == slot) {
          P[t] = ldp(m);
          if (q >= 1 && q <= 3) R[t] = ldr(m);
        }
    }
  }
  float acc = 0.f, comp = 0.f;

  auto step = [&](auto UC, int s) {
    constexpr int U = decltype(UC)::value;
    if (KC && s < s_begin) return;  // before this chunk's start (the unrolled march is aligned to 6)
    const bool inr = !KC || (s >= ka && s <= kb);  // red of an owned plane (not a ring plane)
    constexpr int S0 = (1 + U) % 6, SM1 = (S0 + 5) % 6, SM2 = (S0 + 4) % 6, SP1 = (S0 + 1) % 6;
    constexpr int RP3 = (S0 + 3) % 6;
    constexpr int B = (1 + U) & 1, BB = U & 1;  // shared-memory parities of planes s, s-1
    sOld[B][r][c4] = P[S0];
    __syncthreads();
    float part = 0.f;
    const int q = (jw + s) & 1;
    // ---- red cells of plane s on tile + 1-cell ring
    // i-neighbours of the float4 edges from the adjacent lanes (NX lanes are a tile row)
    // i-neighbours of the float4 edges from the adjacent lanes (NX lanes are a tile row)
    const float rpl = __shfl_up_sync(0xffffffffu, P[S0].w, 1, NX);
    const float rpr = __shfl_down_sync(0xffffffffu, P[S0].x, 1, NX);
    const float bpl = __shfl_up_sync(0xffffffffu, P[SM1].w, 1, NX);
    const float bpr = __shfl_down_sync(0xffffffffu, P[SM1].x, 1, NX);
    if (s <= km && L.row_red) {
      const float4 pn = sOld[B][r + 1][c4], pso = sOld[B][r - 1][c4];
      const float pl = rpl, pr = rpr;
      const float c4l = sC4l[s], c4s = sC4s[s];
      if (CN1MODE == 0) {
        part += relax_pair(q, P[S0], pl, pr, pn, pso, P[SP1], P[SM1], R[S0], rhsav, omega, sCk[s], c2l, c2s,
                           c3l, c3s, c4l, c4s, L.west0, L.east_e, L.owned && inr, L.ival);
      } else {
        const float4 cur = P[S0];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = ib + e;
          if (!L.ival[e] || ((i + jw + s) & 1) == 0) continue;
          const float pc = f4get(cur, e);
          const float pw = (i == 1) ? pc : (e == 0) ? pl : f4get(cur, e - 1);
          const float pe = (i == im) ? pc : (e == 3) ? pr : f4get(cur, e + 1);
          const float rt = relax(omega, cn1_at(e, s), c2l[e], pe, c2s[e], pw, c3l, f4get(pn, e), c3s,
                                 f4get(pso, e), c4l, f4get(P[SP1], e), c4s, f4get(P[SM1], e),
                                 f4get(R[S0], e) - rhsav, pc);
          f4set(P[S0], e, pc + rt);
          if (L.owned && inr) part += rt * rt;
        }
      }
    }
    sRed[B][r][c4] = P[S0];
    // ---- black cells of plane s-1 on the tile
    if ((KC ? (s - 1 >= ka && s - 1 <= kb) : (s >= 2)) && L.owned) {
      const int k = s - 1;
      const float4 pn = sRed[BB][r + 1][c4], pso = sRed[BB][r - 1][c4];
      const float pl = bpl, pr = bpr;
      const float c4l = sC4l[k], c4s = sC4s[k];
      if (CN1MODE == 0) {
        part += relax_pair(q, P[SM1], pl, pr, pn, pso, P[S0], P[SM2], R[SM1], rhsav, omega, sCk[k], c2l, c2s,
                           c3l, c3s, c4l, c4s, L.west0, L.east_e, true, L.ival);
      } else {
        const float4 cur = P[SM1];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = ib + e;
          if (!L.ival[e] || ((i + jw + k) & 1) != 0) continue;
          const float pc = f4get(cur, e);
          const float pw = (i == 1) ? pc : (e == 0) ? pl : f4get(cur, e - 1);
          const float pe = (i == im) ? pc : (e == 3) ? pr : f4get(cur, e + 1);
          const float rt = relax(omega, cn1_at(e, k), c2l[e], pe, c2s[e], pw, c3l, f4get(pn, e), c3s,
                                 f4get(pso, e), c4l, f4get(P[S0], e), c4s, f4get(P[SM2], e),
                                 f4get(R[SM1], e) - rhsav, pc);
          f4set(P[SM1], e, pc + rt);
          part += rt * rt;
        }
      }
      store_final(d, a, L, k, P[SM1]);
    }
    {  // Kahan accumulation of this plane's squared corrections
      const float y = part - comp;
      const float t = acc + y;
      comp = (t - acc) - y;
      acc = t;
    }
    P[SM2] = ldp(s + 4);
    R[RP3] = ldr(s + 3);
  };

  for (int s0 = KC ? s_begin - (s_begin - 1) % 6 : 1; s0 <= s_end; s0 += 6) {
    step(IC<0>{}, s0);
    if (s0 + 1 > s_end) break;
    step(IC<1>{}, s0 + 1);
    if (s0 + 2 > s_end) break;
    step(IC<2>{}, s0 + 2);
    if (s0 + 3 > s_end) break;
    step(IC<3>{}, s0 + 3);
    if (s0 + 4 > s_end) break;
    step(IC<4>{}, s0 + 4);
    if (s0 + 5 > s_end) break;
    step(IC<5>{}, s0 + 5);
  }
  finish_residual<NX, NY>(d, a, acc, sWarp, &sLast, (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x);
}

// ---------------------------------------------------------------------------------
// TMA kernel: one thread brings each tile plane of p and of rhs into a D-stage shared
// ring with a single tensor copy apiece (cp.async.bulk.tensor, 4 NX x NY floats),
// signalled by an mbarrier, D-2 march steps ahead of first use.  Needs a source with
// periodic ghost rows (an internal buffer) and a uniform cn1.  Waits are bounded: if
// a stage never arrives the CTA stops computing, sets CT_ERROR and still meets every
// barrier, then waits (bounded) for the copies it issued.

template <int NX, int NY, int D>
struct TmaSmem {
  float4 p[D][NY][NX];    // old planes of p (tile + 2-cell ring)
  float4 rhs[D][NY][NX];  // planes of rhs
  float4 red[2][NY][NX];  // red-updated planes
  float c4l[LES_SOR_KMAX], c4s[LES_SOR_KMAX], ck[LES_SOR_KMAX];
  uint64_t bar[D];
  double warp[NX * NY / 32];
  int last, abort_;
};

// One tile of one iteration, for the batched launch (les_sor_batch.cu): tile (bx, by) of
// the domain's tile grid, k chunk bz.  maps(0) / maps(1) give the tensor maps of the
// source p buffer and of rhs, and cta() the tile's partial slot; both are evaluated
// where they are used rather than held across the march (a value held live across the
// march measurably slows it: 6% for the partial slot alone).  Every thread of the CTA
// calls it; it leaves the mbarriers quiescent (every copy it issued has been waited
// for).  k_sor_tma below is the same sweep written out for one domain per launch.
template <int NX, int NY, int D, bool KC, class MapFn, class CtaFn>
__device__ __forceinline__ void sor_tma_tile(const LesDom &d, const SorArgs &a, MapFn maps, int bx, int by, int bz,
                                             CtaFn cta, TmaSmem<NX, NY, D> &S) {
  const Lane L = make_lane<NX>(d, a.tj, NY, bx, by, a.ghost);
  const int c4 = L.c4, r = L.r, ib = L.ib, jw = L.jw;
  const int km = d.km;
  float c2l[4], c2s[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    c2l[e] = L.ival[e] ? d.gr.cn2l[ib + e] : 0.f;
    c2s[e] = L.ival[e] ? d.gr.cn2s[ib + e] : 0.f;
  }
  const float c3l = d.gr.cn3l[jw], c3s = d.gr.cn3s[jw];
  const float rhsav = d.fscal[SC_RHSAV];
  // omega = 1 (press.f95:45, the only value this kernel is launched for): omega * x is x
  constexpr float omega = 1.f;
  const bool producer = (r == 0) && (c4 == 0);
  const int tx = bx * tile_i(NX);               // padded column of i0 - 4
  const int ty = by * a.tj + (LES_JOFF - 1);     // padded row of j0 - 2
  const uint32_t stage_bytes = 2u * NY * NX * 16u;
  // this CTA's k chunk [ka, kb], marched from ka-1 (a red ring plane) to kb+1; it
  // loads planes mfirst .. mlast, plane m into stage (m - mfirst) % D
  const int ka = KC ? 1 + bz * a.kchunk : 1;
  const int kb = KC ? min(km, ka + a.kchunk - 1) : km;
  const int s_begin = KC ? max(1, ka - 1) : 1;
  const int s_end = KC ? min(km + 1, kb + 1) : km + 1;
  const int mfirst = KC ? max(1, s_begin - 1) : 1;
  const int mlast = KC ? min(km, kb + 2) : km;
  auto issue = [&](int m) {  // plane m (mfirst..mlast) into stage (m - mfirst) % D
    const int q = (m - mfirst) % D;
    mbar_expect_tx(&S.bar[q], stage_bytes);
    tma_load_3d(&S.p[q][0][0], maps(0), tx, ty, m + LES_KOFF, &S.bar[q]);
    tma_load_3d(&S.rhs[q][0][0], maps(1), tx, ty, m + LES_KOFF, &S.bar[q]);
  };

  if (producer) {
    for (int q = 0; q < D; ++q) mbar_init(&S.bar[q], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    S.abort_ = 0;
  }
  for (int q = r * NX + c4; q <= km; q += NX * NY) {
    if (q >= 1) {
      S.c4l[q] = d.gr.cn4l[q];
      S.c4s[q] = d.gr.cn4s[q];
      S.ck[q] = d.gr.cn1k[q];
    }
  }
  __syncthreads();
  if (producer)
    for (int m = mfirst; m < mfirst + D && m <= mlast; ++m) issue(m);

  int failed_at = 0;
  // plane m sits in stage (m - mfirst) % D with mbarrier phase parity ((m - mfirst) / D) & 1
  auto wait_stage = [&](int m, int st, uint32_t ph) {
    if (!mbar_wait(&S.bar[st], ph)) {
      S.abort_ = 1;
      d.ctl[CT_ERROR] = 1;
      if (!failed_at) failed_at = m;
    }
  };
  auto wait_plane = [&](int m) { wait_stage(m, (m - mfirst) % D, (uint32_t)(((m - mfirst) / D) & 1)); };

  // Plane m of p lives in register slot P[m % 4] and its rhs and coefficients in slot
  // m % 2; the march is unrolled 4 times so every slot is a compile-time register and
  // the planes never move between registers.  Plane 0 reads as plane 1 (boundp2's
  // Neumann copy): with slot s_begin-1 a copy of plane 1 taken before its red update,
  // every k-halo read below finds the cell's own current value (red at s = 1 reads that
  // copy, black at k = 1 reads it one step later, and at the top the slot of plane
  // km+1 is a copy of plane km), so the march needs no halo selects.
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 P[4], R[2];
  float CK[2] = {0.f, 0.f}, C4L[2] = {0.f, 0.f}, C4S[2] = {0.f, 0.f};
#pragma unroll
  for (int t = 0; t < 4; ++t) P[t] = zero4;
  R[0] = R[1] = zero4;
  {
    wait_plane(s_begin);
    const float4 p0 = S.p[(s_begin - mfirst) % D][r][c4];
    float4 pm1 = p0;
    if (KC && s_begin > 1) {
      wait_plane(s_begin - 1);
      pm1 = S.p[(s_begin - 1 - mfirst) % D][r][c4];
    }
    const int t0 = s_begin % 4, t1 = (s_begin + 3) % 4;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      if (t == t0) P[t] = p0;
      if (t == t1) P[t] = pm1;
    }
  }
  // residual: plain FP32 sums over a group of four steps, Kahan-compensated across groups
  float acc = 0.f, comp = 0.f, grp = 0.f;
  auto fold_group = [&]() {
    const float y = grp - comp;
    const float t = acc + y;
    comp = (t - acc) - y;
    acc = t;
    grp = 0.f;
  };
  // stage and phase of plane s (st0) and of plane s+1 (st1, ph1), advanced per step
  int st0 = (s_begin - mfirst) % D, st1 = (s_begin + 1 - mfirst) % D;
  uint32_t ph1 = (uint32_t)(((s_begin + 1 - mfirst) / D) & 1);

  // residual weights: red counts the owned cells of the tile, black runs on owned
  // threads only
  float mred[4], mblack[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    mblack[e] = L.ival[e] ? 1.f : 0.f;
    mred[e] = (L.owned && L.ival[e]) ? 1.f : 0.f;
  }

  auto step = [&](auto UC, int s) {
    constexpr int U = decltype(UC)::value;  // s = U modulo 4
    constexpr int S0 = U, SP1 = (U + 1) % 4, SM1 = (U + 3) % 4, SM2 = (U + 2) % 4;
    constexpr int C0 = U % 2, CM = (U + 1) % 2;
    if (s < s_begin) return;  // before this chunk's start (the unrolled march is aligned to 4)
    __syncthreads();
    if (S.abort_) return;
    // the stage of plane s-1 is free: every thread has left step s-1 (or the prologue)
    if (producer && s - 1 >= mfirst && s - 1 + D <= mlast) issue(s - 1 + D);
    P[SP1] = P[S0];  // plane km+1 reads as plane km, before its red update
    R[C0] = zero4;
    if (s + 1 <= mlast) {
      wait_stage(s + 1, st1, ph1);
      P[SP1] = S.p[st1][r][c4];
    }
    float part = 0.f;
    const int q = (jw + s) & 1;
    const float rpl = __shfl_up_sync(0xffffffffu, P[S0].w, 1, NX);
    const float rpr = __shfl_down_sync(0xffffffffu, P[S0].x, 1, NX);
    const float bpl = __shfl_up_sync(0xffffffffu, P[SM1].w, 1, NX);
    const float bpr = __shfl_down_sync(0xffffffffu, P[SM1].x, 1, NX);
    // ---- red cells of plane s on the tile + 1-cell ring
    if (s <= km) {
      CK[C0] = S.ck[s];
      C4L[C0] = S.c4l[s];
      C4S[C0] = S.c4s[s];
      if (L.row_red) {
        R[C0] = S.rhs[st0][r][c4];
        const float4 pn = S.p[st0][r + 1][c4], pso = S.p[st0][r - 1][c4];
        const float pr_ = relax_pair_m(q, P[S0], rpl, rpr, pn, pso, P[SP1], P[SM1], R[C0], rhsav, omega, CK[C0], c2l,
                                       c2s, c3l, c3s, C4L[C0], C4S[C0], L.west0, L.east_e, mred);
        if (!KC || (s >= ka && s <= kb)) part += pr_;
      }
    }
    S.red[U & 1][r][c4] = P[S0];
    // ---- black cells of plane s-1 on the tile
    if ((KC ? (s - 1 >= ka && s - 1 <= kb) : (s >= 2)) && L.owned) {
      const int k = s - 1;
      const float4 pn = S.red[(U + 1) & 1][r + 1][c4], pso = S.red[(U + 1) & 1][r - 1][c4];
      part += relax_pair_m(q, P[SM1], bpl, bpr, pn, pso, P[S0], P[SM2], R[CM], rhsav, omega, CK[CM], c2l, c2s, c3l,
                           c3s, C4L[CM], C4S[CM], L.west0, L.east_e, mblack);
      store_final(d, a, L, k, P[SM1]);
    }
    grp += part;
    st0 = st1;
    if (++st1 == D) {
      st1 = 0;
      ph1 ^= 1u;
    }
  };
  for (int s0 = s_begin - s_begin % 4; s0 <= s_end; s0 += 4) {
    step(IC<0>{}, s0);
    if (s0 + 1 > s_end) break;
    step(IC<1>{}, s0 + 1);
    if (s0 + 2 > s_end) break;
    step(IC<2>{}, s0 + 2);
    if (s0 + 3 > s_end) break;
    step(IC<3>{}, s0 + 3);
    fold_group();
  }
  fold_group();  // the last, partial group
  // after a failed wait, wait (bounded) for the copies already issued before leaving
  if (failed_at) {
    for (int m = failed_at; m <= mlast && m < failed_at + D; ++m)
      (void)mbar_wait(&S.bar[(m - mfirst) % D], (uint32_t)(((m - mfirst) / D) & 1));
  }
  finish_residual<NX, NY>(d, a, acc, S.warp, &S.last, cta());
}

template <int NX, int NY, int D, bool KC>
__global__ void __launch_bounds__(NX *NY, min_ctas(NX))
    k_sor_tma(LesDom d, SorArgs a, const __grid_constant__ CUtensorMap tmP, const __grid_constant__ CUtensorMap tmR) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TmaSmem<NX, NY, D> &S = *reinterpret_cast<TmaSmem<NX, NY, D> *>(smem_raw);
  // early exit of press.f95:119-121; in redo mode: run only when a two-iteration launch
  // must be cut back to its first iteration
  if (a.redo ? d.ctl[CT_REDO] == 0 : d.ctl[CT_CONVERGED] != 0) return;

  const Lane L = make_lane<NX>(d, a.tj, NY, blockIdx.x, blockIdx.y, a.ghost);
  const int c4 = L.c4, r = L.r, ib = L.ib, jw = L.jw;
  const int km = d.km;
  float c2l[4], c2s[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    c2l[e] = L.ival[e] ? d.gr.cn2l[ib + e] : 0.f;
    c2s[e] = L.ival[e] ? d.gr.cn2s[ib + e] : 0.f;
  }
  const float c3l = d.gr.cn3l[jw], c3s = d.gr.cn3s[jw];
  const float rhsav = d.fscal[SC_RHSAV];
  // omega = 1 (press.f95:45, the only value this kernel is launched for): omega * x is x
  constexpr float omega = 1.f;
  const bool producer = (r == 0) && (c4 == 0);
  const int tx = blockIdx.x * tile_i(NX);  // padded column of i0 - 4
  const int ty = blockIdx.y * a.tj + (LES_JOFF - 1);  // padded row of j0 - 2
  const uint32_t stage_bytes = 2u * NY * NX * 16u;
  // this CTA's k chunk [ka, kb], marched from ka-1 (a red ring plane) to kb+1; it
  // loads planes mfirst .. mlast, plane m into stage (m - mfirst) % D
  const int ka = KC ? 1 + (int)blockIdx.z * a.kchunk : 1;
  const int kb = KC ? min(km, ka + a.kchunk - 1) : km;
  const int s_begin = KC ? max(1, ka - 1) : 1;
  const int s_end = KC ? min(km + 1, kb + 1) : km + 1;
  const int mfirst = KC ? max(1, s_begin - 1) : 1;
  const int mlast = KC ? min(km, kb + 2) : km;
  auto issue = [&](int m) {  // plane m (mfirst..mlast) into stage (m - mfirst) % D
    const int q = (m - mfirst) % D;
    mbar_expect_tx(&S.bar[q], stage_bytes);
    tma_load_3d(&S.p[q][0][0], &tmP, tx, ty, m + LES_KOFF, &S.bar[q]);
    tma_load_3d(&S.rhs[q][0][0], &tmR, tx, ty, m + LES_KOFF, &S.bar[q]);
  };

  if (producer) {
    for (int q = 0; q < D; ++q) mbar_init(&S.bar[q], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    S.abort_ = 0;
  }
  for (int q = r * NX + c4; q <= km; q += NX * NY) {
    if (q >= 1) {
      S.c4l[q] = d.gr.cn4l[q];
      S.c4s[q] = d.gr.cn4s[q];
      S.ck[q] = d.gr.cn1k[q];
    }
  }
  __syncthreads();
  if (producer)
    for (int m = mfirst; m < mfirst + D && m <= mlast; ++m) issue(m);

  int failed_at = 0;
  // plane m sits in stage (m - mfirst) % D with mbarrier phase parity ((m - mfirst) / D) & 1
  auto wait_stage = [&](int m, int st, uint32_t ph) {
    if (!mbar_wait(&S.bar[st], ph)) {
      S.abort_ = 1;
      d.ctl[CT_ERROR] = 1;
      if (!failed_at) failed_at = m;
    }
  };
  auto wait_plane = [&](int m) { wait_stage(m, (m - mfirst) % D, (uint32_t)(((m - mfirst) / D) & 1)); };

  // Plane m of p lives in register slot P[m % 4] and its rhs and coefficients in slot
  // m % 2; the march is unrolled 4 times so every slot is a compile-time register and
  // the planes never move between registers.  Plane 0 reads as plane 1 (boundp2's
  // Neumann copy): with slot s_begin-1 a copy of plane 1 taken before its red update,
  // every k-halo read below finds the cell's own current value (red at s = 1 reads that
  // copy, black at k = 1 reads it one step later, and at the top the slot of plane
  // km+1 is a copy of plane km), so the march needs no halo selects.
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 P[4], R[2];
  float CK[2] = {0.f, 0.f}, C4L[2] = {0.f, 0.f}, C4S[2] = {0.f, 0.f};
#pragma unroll
  for (int t = 0; t < 4; ++t) P[t] = zero4;
  R[0] = R[1] = zero4;
  {
    wait_plane(s_begin);
    const float4 p0 = S.p[(s_begin - mfirst) % D][r][c4];
    float4 pm1 = p0;
    if (KC && s_begin > 1) {
      wait_plane(s_begin - 1);
      pm1 = S.p[(s_begin - 1 - mfirst) % D][r][c4];
    }
    const int t0 = s_begin % 4, t1 = (s_begin + 3) % 4;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      if (t == t0) P[t] = p0;
      if (t == t1) P[t] = pm1;
    }
  }
  // residual: plain FP32 sums over a group of four steps, Kahan-compensated across groups
  float acc = 0.f, comp = 0.f, grp = 0.f;
  auto fold_group = [&]() {
    const float y = grp - comp;
    const float t = acc + y;
    comp = (t - acc) - y;
    acc = t;
    grp = 0.f;
  };
  // stage and phase of plane s (st0) and of plane s+1 (st1, ph1), advanced per step
  int st0 = (s_begin - mfirst) % D, st1 = (s_begin + 1 - mfirst) % D;
  uint32_t ph1 = (uint32_t)(((s_begin + 1 - mfirst) / D) & 1);

  // residual weights: red counts the owned cells of the tile, black runs on owned
  // threads only
  float mred[4], mblack[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    mblack[e] = L.ival[e] ? 1.f : 0.f;
    mred[e] = (L.owned && L.ival[e]) ? 1.f : 0.f;
  }

  auto step = [&](auto UC, int s) {
    constexpr int U = decltype(UC)::value;  // s = U modulo 4
    constexpr int S0 = U, SP1 = (U + 1) % 4, SM1 = (U + 3) % 4, SM2 = (U + 2) % 4;
    constexpr int C0 = U % 2, CM = (U + 1) % 2;
    if (s < s_begin) return;  // before this chunk's start (the unrolled march is aligned to 4)
    __syncthreads();
    if (S.abort_) return;
    // the stage of plane s-1 is free: every thread has left step s-1 (or the prologue)
    if (producer && s - 1 >= mfirst && s - 1 + D <= mlast) issue(s - 1 + D);
    P[SP1] = P[S0];  // plane km+1 reads as plane km, before its red update
    R[C0] = zero4;
    if (s + 1 <= mlast) {
      wait_stage(s + 1, st1, ph1);
      P[SP1] = S.p[st1][r][c4];
    }
    float part = 0.f;
    const int q = (jw + s) & 1;
    const float rpl = __shfl_up_sync(0xffffffffu, P[S0].w, 1, NX);
    const float rpr = __shfl_down_sync(0xffffffffu, P[S0].x, 1, NX);
    const float bpl = __shfl_up_sync(0xffffffffu, P[SM1].w, 1, NX);
    const float bpr = __shfl_down_sync(0xffffffffu, P[SM1].x, 1, NX);
    // ---- red cells of plane s on the tile + 1-cell ring
    if (s <= km) {
      CK[C0] = S.ck[s];
      C4L[C0] = S.c4l[s];
      C4S[C0] = S.c4s[s];
      if (L.row_red) {
        R[C0] = S.rhs[st0][r][c4];
        const float4 pn = S.p[st0][r + 1][c4], pso = S.p[st0][r - 1][c4];
        const float pr_ = relax_pair_m(q, P[S0], rpl, rpr, pn, pso, P[SP1], P[SM1], R[C0], rhsav, omega, CK[C0], c2l,
                                       c2s, c3l, c3s, C4L[C0], C4S[C0], L.west0, L.east_e, mred);
        if (!KC || (s >= ka && s <= kb)) part += pr_;
      }
    }
    S.red[U & 1][r][c4] = P[S0];
    // ---- black cells of plane s-1 on the tile
    if ((KC ? (s - 1 >= ka && s - 1 <= kb) : (s >= 2)) && L.owned) {
      const int k = s - 1;
      const float4 pn = S.red[(U + 1) & 1][r + 1][c4], pso = S.red[(U + 1) & 1][r - 1][c4];
      part += relax_pair_m(q, P[SM1], bpl, bpr, pn, pso, P[S0], P[SM2], R[CM], rhsav, omega, CK[CM], c2l, c2s, c3l,
                           c3s, C4L[CM], C4S[CM], L.west0, L.east_e, mblack);
      store_final(d, a, L, k, P[SM1]);
    }
    grp += part;
    st0 = st1;
    if (++st1 == D) {
      st1 = 0;
      ph1 ^= 1u;
    }
  };
  for (int s0 = s_begin - s_begin % 4; s0 <= s_end; s0 += 4) {
    step(IC<0>{}, s0);
    if (s0 + 1 > s_end) break;
    step(IC<1>{}, s0 + 1);
    if (s0 + 2 > s_end) break;
    step(IC<2>{}, s0 + 2);
    if (s0 + 3 > s_end) break;
    step(IC<3>{}, s0 + 3);
    fold_group();
  }
  fold_group();  // the last, partial group
  // after a failed wait, wait (bounded) for the copies already issued before leaving
  if (failed_at) {
    for (int m = failed_at; m <= mlast && m < failed_at + D; ++m)
      (void)mbar_wait(&S.bar[(m - mfirst) % D], (uint32_t)(((m - mfirst) / D) & 1));
  }
  finish_residual<NX, NY>(d, a, acc, S.warp, &S.last, (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x);
}

template <int NX, int NY, bool KC>
void launch_reg_kc(const LesDom &d, const SorArgs &a, int cn1mode, cudaStream_t s) {
  const dim3 grid((d.im + tile_i(NX) - 1) / tile_i(NX), (d.jm + a.tj - 1) / a.tj, KC ? a.nchunk : 1);
  const dim3 block(NX, NY);
  if (cn1mode == 1) k_sor_reg<NX, NY, 1, KC><<<grid, block, 0, s>>>(d, a);
  else if (cn1mode == 2) k_sor_reg<NX, NY, 2, KC><<<grid, block, 0, s>>>(d, a);
  else k_sor_reg<NX, NY, 0, KC><<<grid, block, 0, s>>>(d, a);
}

template <int NX, int NY, int D, bool KC>
void launch_tma_kc(const LesDom &d, const SorArgs &a, const CUtensorMap &tp, const CUtensorMap &tr, cudaStream_t s) {
  const dim3 grid((d.im + tile_i(NX) - 1) / tile_i(NX), (d.jm + a.tj - 1) / a.tj, KC ? a.nchunk : 1);
  const size_t bytes = sizeof(TmaSmem<NX, NY, D>);
  cudaFuncSetAttribute(k_sor_tma<NX, NY, D, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k_sor_tma<NX, NY, D, KC><<<grid, dim3(NX, NY), bytes, s>>>(d, a, tp, tr);
}

}  // namespace
