// les_aveflow.cuh -- time averages of the flow (aveflow.f95:5-200), les_aveflow.cu.
#pragma once
#include <cuda_runtime.h>

#include "les_common.cuh"
#include "les_kernels.cuh"

// The averaging arrays of aveflow.f95:7-22, in the padded field layout: aveu, avev
// (1:im,1:jm,0:km), avew (1:im+1,1:jm,0:km+2), the others (1:im,1:jm,1:km).
struct LesAve {
  float *aveu, *avev, *avew, *avep, *avel, *aveuu, *avevv, *aveww, *avesm, *avesmsm, *uwfx;
};

// aveflow at step n, averaging from step n1 to nmax: zero at n == n1, accumulate for
// n >= n1, finalise at n == nmax.
void les_launch_aveflow(const LesDom &d, const LesAve &A, int n, int n1, int nmax, LesCtx ctx);
