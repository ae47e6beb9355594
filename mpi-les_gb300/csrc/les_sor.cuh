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
  int tj;                // interior rows per tile (tile height NY - 4)
  int ntiles;            // CTAs in the launch
  double *part;          // per-CTA residual partials (>= ntiles)
  unsigned int *counter; // CTA completion ticket, zero between launches
  int ghost;             // 1: also write pdst's periodic ghost rows (internal buffers)
  int kchunk;            // k planes per CTA (grid z = nchunk chunks); >= km: one chunk
  int nchunk;            // chunks (grid z)
};

// Tensor maps of the internal buffers (sorA, sorB, sorR) for one tile height.
struct LesSorMaps {
  CUtensorMap m[3];
  int ny = 0;
  int valid = 0;
};

int les_sor_fused_tiles(int im, int jm, int ny);
int les_sor_pick_ny(int im, int jm, int sms);
// Planes per k chunk: one chunk when the tiles fill the SMs, else enough chunks to
// fill them (each at least 8 planes: a chunk recomputes one red plane below it).
int les_sor_pick_kchunk(int tiles, int km, int sms);
int les_sor_make_maps(const LesDom &d, int ny, LesSorMaps *maps);
// One SOR iteration: the TMA kernel when the source is an internal buffer with valid
// maps and cn1 is uniform, the register kernel otherwise.
void les_launch_sor_iter(const LesDom &d, const SorArgs &a, int ny, const LesSorMaps *maps, cudaStream_t s);
void les_launch_sor_copyout(const LesDom &d, int nmaxp, cudaStream_t s);
