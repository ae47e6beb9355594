// les_sor.cuh -- launchers of the fused red-black SOR sweep (les_sor.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "les_common.cuh"

// planes whose per-k coefficients the fused sweep stages in shared memory (km < KMAX)
#define LES_SOR_KMAX 512

struct SorArgs {
  const float *psrc;     // p at the start of the iteration (read only)
  float *pdst;           // p at the end of the iteration (interior written)
  const float *rhs;      // rhs before the rhsav shift (the sweep subtracts rhsav)
  int tj;                // interior rows per tile (tile height ny - 4)
  int ntiles;            // CTAs in the launch
  double *part;          // per-CTA residual partials (>= ntiles)
  unsigned int *counter; // CTA completion ticket, zero between launches
  int ghost;             // also write pdst's periodic ghost rows (internal buffers): 1 two
                         // rows per side, 2 four (read by two-iteration marches, jm >= 4)
  int kchunk;            // k planes per CTA (grid z = nchunk chunks); >= km: one chunk
  int nchunk;            // chunks (grid z)
  int depth = 1;         // iterations this launch performs (1, or 2: les_sor2.cu)
  int redo = 0;          // 1: recompute one iteration only if CT_REDO is set (after a
                         // two-iteration launch whose first iteration met the exit test)
  int dstcode = 0;       // where pdst is, for the copy-out: 0 sorA, 1 sorB, 2 p itself
  int src_ghosts = 0;    // psrc == p and the SOR-path rhs kernel has just written p's
                         // periodic ghost rows: the TMA sweep may read p
};

// Tile shape of the fused sweep: nx float4 columns (32 or 16; the interior i cells per
// tile are 4 nx - 8) by ny rows, kchunk k planes per CTA (>= km: the whole march), and
// the iterations fused into one k-march (depth 1; or 2: 32-column tiles, ny 24/28/32,
// the whole march).  The interior j rows of a tile are ny - 4 depth.  ny == 0 selects
// the per-subroutine path instead.
struct SorShape {
  int nx = 0, ny = 0, kchunk = 0, depth = 1;
};

// Tensor maps of the internal buffers (sorA, sorB, sorR) and of p for one tile shape.
struct LesSorMaps {
  CUtensorMap m[4];
  SorShape shape;
  int valid = 0;
};

int les_sor_fused_tiles(int im, int jm, SorShape sh);
// The tile shape for a domain alone on the GPU (fewest waves of one-SM CTAs) or
// sharing it with other domains (fewest thread-planes, ring cells included).
SorShape les_sor_pick_shape(int im, int jm, int sms, bool shared_gpu);
// Planes per k chunk: one chunk when the tiles fill the SMs, else enough chunks to
// fill them (each at least 8 planes: a chunk recomputes one red plane below it).
int les_sor_pick_kchunk(int tiles, int km, int sms);
int les_sor_make_maps(const LesDom &d, SorShape sh, LesSorMaps *maps);
// A tiled tensor map of one padded 3-D field of the domain (float32; dims pi x nj x
// km+4, its rows and planes as strides) with boxes of boxx x boxy x 1 (boxx * 4 bytes a
// multiple of 16).  0 on success.
int les_tensor_map_3d(CUtensorMap *m, const LesDom &d, const float *base, int boxx, int boxy);
// One SOR iteration: the TMA kernel when the source is an internal buffer with valid
// maps and cn1 is uniform, the register kernel otherwise.  With a.depth == 2 (only when
// les_sor_two_ok holds): two iterations in one launch (les_sor2.cu).
void les_launch_sor_iter(const LesDom &d, const SorArgs &a, SorShape sh, const LesSorMaps *maps, cudaStream_t s);
// Whether shape sh can run two iterations per launch on this domain from internal
// buffers: 32-column tiles, ny 24/28/32, the whole march, omega = 1, a cn1 uniform in i
// and j, and x and y coefficients cn2l, cn2s, cn3l, cn3s each one value (sor_uni).
bool les_sor_two_ok(const LesDom &d, SorShape sh);
void les_launch_sor_iter2(const LesDom &d, const SorArgs &a, int ny, const CUtensorMap &tp, const CUtensorMap &tr,
                          cudaStream_t s);
// 16-column tiles (les_sor16.cu): the TMA kernel when tp and tr are given, the register
// kernel (uniform cn1, one k chunk) otherwise.
void les_launch_sor_iter_nx16(const LesDom &d, const SorArgs &a, int ny, const CUtensorMap *tp,
                              const CUtensorMap *tr, cudaStream_t s);
// restore_prow: the press's rhs kernel saved p's row jm+2 (les_kernels.cu): put it back
void les_launch_sor_copyout(const LesDom &d, int restore_prow, cudaStream_t s);
// After a two-iteration launch `two` (sor_fixed == 0): recompute its first iteration
// alone, from the same source into the same destination, if that iteration met the
// exit test (CT_REDO); otherwise the launch returns at once.
void les_launch_sor_redo(const LesDom &d, const SorArgs &two, cudaStream_t s);
