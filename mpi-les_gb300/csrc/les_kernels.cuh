// les_kernels.cuh -- host-side launchers of the solver kernels.
#pragma once
#include <cuda_runtime.h>

#include "les_common.cuh"

// Launch context: the stream work goes to and the counter of kernel launches.
struct LesCtx {
  cudaStream_t s;
  long long *nlaunch;
};

// per-subroutine kernels (les_kernels.cu)
void les_launch_velnw(const LesDom &d, LesCtx ctx);
void les_launch_bondv1(const LesDom &d, int n, LesCtx ctx);
void les_launch_feedbf(const LesDom &d, LesCtx ctx);
void les_launch_boundsm(const LesDom &d, LesCtx ctx);
// feedbfm.f95:87-116 on the device: the b, c, d mask bits (1, 2, 4) of every padded cell
// of a domain with row pitch pi, nj rows per plane and nk planes, from zbm(1:im,1:jm)
// and thr(k) = z2(k) + 0.5*dzn(k), k = 1..km (thr[k-1])
void les_launch_feedbfm(uint8_t *mask, const float *zbm, const float *thr, int im, int jm, int km, int pi,
                        int nj, int nk, LesCtx ctx);
// les_fused.cu: velfg (optionally with feedbf) and les (optionally with adam)
void les_launch_velfg_fused(const LesDom &d, bool with_feedbf, LesCtx ctx);
void les_launch_les_fused(const LesDom &d, bool with_adam, LesCtx ctx);
void les_launch_adam(const LesDom &d, LesCtx ctx);
void les_launch_bondfg(const LesDom &d, LesCtx ctx);
void les_launch_boundp1(const LesDom &d, LesCtx ctx, int obey_converged);
void les_launch_boundp2(const LesDom &d, LesCtx ctx, int obey_converged);
void les_launch_rhs_mean(const LesDom &d, LesCtx ctx);
void les_launch_rhs_sor(const LesDom &d, LesCtx ctx);    // rhs into the SOR buffer (+ ghost rows) and rhsav
void les_launch_sor_begin(const LesDom &d, LesCtx ctx);
// Blocks of the second reduction level of k_finish_mean (buffer d.part2).
constexpr int LES_FIN_BLOCKS = 128;
// The volume-weighted interior mean of d.p (press.f95:124-133, the pav reduction) into
// d.fscal[SC_PAV] and d.scal[SC_PAV]; partials in d.part (les_reduce_blocks(d)
// doubles), d.part2 (LES_FIN_BLOCKS doubles), ticket d.cnt[8] (zero on entry, zero on
// exit); reads d.scal[SC_AREA].
void les_launch_interior_mean(const LesDom &d, LesCtx ctx);
void les_launch_sor_simple(const LesDom &d, int nmaxp, LesCtx ctx);
void les_launch_pav_adjust(const LesDom &d, LesCtx ctx);
void les_launch_count_nonfinite(const LesDom &d, unsigned long long *bad, LesCtx ctx);
int les_interior_blocks(const LesDom &d);
// Blocks (= partial sums) of the rhs and pav reductions: (im+63)/64 * (jm+3)/4 * ((km+15)/16)
int les_reduce_blocks(const LesDom &d);
int les_sor_simple_parts(const LesDom &d);
