// les_sor.cu -- fused red-black SOR sweep of press.f95:89-122 (one launch per iteration).
//
// Reference semantics (press.f95:89-122, boundp.f95): per iteration, all red cells
// (i+j+k odd) are relaxed, then boundp1 refreshes the i and j halos; then all black
// cells, boundp1 again; then boundp2 refreshes the k halos.  Within a colour every
// update reads only cells of the other colour, so a colour is order-free.
//
// GB300 mapping.  A CTA owns a tile of TI (i) x TJ (j) interior cells and marches up
// k; TI = 4 NX - 8 with NX = 32 (120 cells) or 16 (56 cells, for narrow domains that
// share the GPU).  Each thread owns one float4 column (4 consecutive i at one j).  At march step s
// the CTA relaxes the red cells of plane s and then the black cells of plane s-1
// (which need the red values of planes s-2, s-1 and s), so one launch performs a whole
// iteration with one pass over p and rhs.  In-plane j neighbours come from shared
// memory (the old plane for red, the red-updated plane for black); the i neighbours
// at the float4 edges come from the adjacent lanes by warp shuffle.  Red is also computed on a one-cell ring around the tile (from a two-cell
// ring of loaded values) so the tile's black cells have all their red neighbours;
// the ring work is redundant but exact.
//
// Halos are virtual.  With p's halos consistent with its interior at entry (true
// between time steps), every halo value the reference reads during the sweep equals
// a value of the cell it was copied from: p(0) = p(1), p(im+1) = p(im), p(k=0) =
// p(k=1), p(km+1) = p(km) at the moment of reading (each cell is the only reader of
// its own Neumann image), and the periodic j images p(0) = p(jm), p(jm+1) = p(1) are
// cells of the other colour (jm even), unchanged by the sweep that reads them.  So
// the sweep never reads or writes p's halo storage; press's final boundp1/boundp2
// (after removing pav) writes the whole halo state the reference leaves.
//
// Buffers.  Tiles march at different speeds, so an iteration reads one buffer and
// writes another.  Iteration 1 reads p itself (the register kernel below, which wraps
// j); later iterations ping-pong between two internal buffers that carry periodic
// ghost rows (j = -1, 0, jm+1, jm+2), so a tile plane is a plain rectangle that one
// tensor TMA copy can bring in; the last iteration writes p.
//
// k chunks: when the tiles alone would leave SMs idle (small domains), grid z splits
// the march into chunks of planes [ka, kb] (the KC kernel variants).  A chunk starts
// one plane early, at ka-1, relaxing its red cells as a ring plane (from the old black
// values around it, exactly as the chunk below does) so that its black cells of plane
// ka have their red neighbours; ring planes are neither stored nor counted in the
// residual.
//
// Residual: each thread accumulates reltmp^2 of its owned cells in FP32 with Kahan
// compensation, CTAs reduce to FP64 partials, and the last CTA to finish sums them in
// a fixed order (no spin waits) and applies the convergence test of press.f95:119.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "les_common.cuh"
#include "les_sor.cuh"
#include "les_sor_kern.cuh"

namespace {

// Copy the interior of the buffer the last executed launch wrote back into p, when the
// sweep stopped before its final (p-writing) launch or ran a single iteration.
__global__ void k_sor_copyout(LesDom d, int restore_prow) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y + 1;
  if (i > d.im) return;
  // p's row jm+2 as it was before the press (no sweep writes it): plane k by the threads
  // of row j = 1 + (k-1) mod jm, so the rows share the planes
  if (restore_prow)
    for (int k = j; k <= d.km; k += d.jm) d.p[lix(d, i, d.jm + 2, k)] = d.prow[(k - 1) * d.im + (i - 1)];
  if (d.ctl[CT_ITERS] < 1 || d.ctl[CT_LASTBUF] == 2) return;  // nothing ran, or p was written
  const float *src = (d.ctl[CT_LASTBUF] == 1) ? d.sorB : d.sorA;
  for (int k = 1; k <= d.km; ++k) {
    const int c = lix(d, i, j, k);
    d.p[c] = src[c];
  }
}

template <int NY>
void launch_reg(const LesDom &d, const SorArgs &a, int cn1mode, cudaStream_t s) {
  if (a.nchunk > 1) launch_reg_kc<32, NY, true>(d, a, cn1mode, s);
  else launch_reg_kc<32, NY, false>(d, a, cn1mode, s);
}
template <int NY, int D>
void launch_tma(const LesDom &d, const SorArgs &a, const CUtensorMap &tp, const CUtensorMap &tr, cudaStream_t s) {
  if (a.nchunk > 1) launch_tma_kc<32, NY, D, true>(d, a, tp, tr, s);
  else launch_tma_kc<32, NY, D, false>(d, a, tp, tr, s);
}

}  // namespace

int les_sor_fused_tiles(int im, int jm, SorShape sh) {
  const int ti = 4 * sh.nx - 8, tj = sh.ny - 4 * (sh.depth == 2 ? 2 : 1);
  return ((im + ti - 1) / ti) * ((jm + tj - 1) / tj);
}

SorShape les_sor_pick_shape(int im, int jm, int sms, bool shared_gpu) {
  static const int nys[] = {16, 20, 24, 28};
  SorShape best{32, 24};
  double best_cost = 1e30;
  if (!shared_gpu) {
    // A domain alone: each 32-column CTA holds one SM.  Pick the tile height whose
    // CTA count fills the SMs in the fewest waves, preferring less ring overhead on
    // ties (the k-split then fills the SMs that are still idle).
    for (int ny : nys) {
      const int tiles = les_sor_fused_tiles(im, jm, SorShape{32, ny});
      const double cost = ((tiles + sms - 1) / sms) * (double)ny;
      if (cost < best_cost - 1e-9) { best_cost = cost; best = SorShape{32, ny}; }
    }
    return best;
  }
  // A domain sharing the GPU with others: the SMs stay busy, so the cost is the
  // thread-planes the launch issues, ring columns and rows included (tiles x NX x NY).
  // 16-column tiles waste fewer ring and padding columns on narrow domains.
  for (int nx : {32, 16})
    for (int ny : nys) {
      const SorShape sh{nx, ny};
      const double cost = (double)les_sor_fused_tiles(im, jm, sh) * nx * ny;
      if (cost < best_cost - 1e-9) { best_cost = cost; best = sh; }
    }
  return best;
}

int les_sor_pick_kchunk(int tiles, int km, int sms) {
  if (const char *e = getenv("LES_SOR_KCHUNK")) {  // A/B measurements
    const int v = atoi(e);
    if (v > 0) return v;
  }
  if (tiles <= 0 || 2 * tiles >= sms) return km;
  int nch = (sms + tiles - 1) / tiles;
  nch = std::max(1, std::min(nch, km / 8));
  return (km + nch - 1) / nch;
}

int les_tensor_map_3d(CUtensorMap *m, const LesDom &d, const float *base, int boxx, int boxy) {
  using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static EncodeFn encode = nullptr;
  if (!encode) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return -1;
    encode = reinterpret_cast<EncodeFn>(fn);
  }
  const cuuint64_t dims[3] = {(cuuint64_t)d.pi, (cuuint64_t)d.nj, (cuuint64_t)(d.km + 4)};
  const cuuint64_t strides[2] = {(cuuint64_t)d.pi * 4u, (cuuint64_t)d.np * 4u};
  const cuuint32_t box[3] = {(cuuint32_t)boxx, (cuuint32_t)boxy, 1u};
  const cuuint32_t estr[3] = {1u, 1u, 1u};
  const CUresult rc = encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box,
                             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return rc == CUDA_SUCCESS ? 0 : -2;
}

int les_sor_make_maps(const LesDom &d, SorShape sh, LesSorMaps *maps) {
  const float *bases[4] = {d.sorA, d.sorB, d.sorR, d.p};
  for (int q = 0; q < 4; ++q) {
    const int rc = les_tensor_map_3d(&maps->m[q], d, bases[q], sh.nx * 4, sh.ny);
    if (rc != 0) return rc;
  }
  maps->shape = sh;
  maps->valid = 1;
  return 0;
}

void les_launch_sor_iter(const LesDom &d, const SorArgs &a, SorShape sh, const LesSorMaps *maps, cudaStream_t s) {
  const int cn1mode = d.gr.cn1k ? 0 : (d.cn1 ? 1 : 2);
  // LES_SOR_KIND=0 forces the register kernel everywhere (A/B measurements)
  static const int kind = [] {
    const char *e = getenv("LES_SOR_KIND");
    return e ? atoi(e) : 1;
  }();
  // the TMA sweep is built for omega = 1 (press.f95:45); another omega takes the register kernel
  const bool tma = kind != 0 && maps && maps->valid && maps->shape.nx == sh.nx && maps->shape.ny == sh.ny &&
                   cn1mode == 0 && d.omega == 1.f &&
                   (a.psrc == d.sorA || a.psrc == d.sorB || (a.psrc == d.p && a.src_ghosts && a.depth == 1));
  const CUtensorMap *tp =
      tma ? ((a.psrc == d.sorA) ? &maps->m[0] : (a.psrc == d.sorB) ? &maps->m[1] : &maps->m[3]) : nullptr;
  const CUtensorMap *tr = tma ? &maps->m[2] : nullptr;
  if (a.depth == 2) {  // the caller checked les_sor_two_ok
    les_launch_sor_iter2(d, a, sh.ny, *tp, *tr, s);
    return;
  }
  if (sh.nx == 16) {
    les_launch_sor_iter_nx16(d, a, sh.ny, tp, tr, s);
    return;
  }
  if (tma) {
    switch (sh.ny) {
      case 16: launch_tma<16, 6>(d, a, *tp, *tr, s); return;
      case 20: launch_tma<20, 6>(d, a, *tp, *tr, s); return;
      case 28: launch_tma<28, 4>(d, a, *tp, *tr, s); return;
      default: launch_tma<24, 6>(d, a, *tp, *tr, s); return;
    }
  }
  switch (sh.ny) {
    case 16: launch_reg<16>(d, a, cn1mode, s); break;
    case 20: launch_reg<20>(d, a, cn1mode, s); break;
    case 28: launch_reg<28>(d, a, cn1mode, s); break;
    default: launch_reg<24>(d, a, cn1mode, s); break;
  }
}

void les_launch_sor_redo(const LesDom &d, const SorArgs &two, cudaStream_t s) {
  SorArgs a = two;
  a.redo = 1;
  a.depth = 1;
  a.tj = 24 - 4;
  a.kchunk = d.km;
  a.nchunk = 1;
  a.ntiles = les_sor_fused_tiles(d.im, d.jm, SorShape{32, 24, 0, 1});
  launch_reg_kc<32, 24, false>(d, a, 0, s);
}

void les_launch_sor_copyout(const LesDom &d, int restore_prow, cudaStream_t s) {
  k_sor_copyout<<<dim3((d.im + 127) / 128, d.jm), 128, 0, s>>>(d, restore_prow);
}
