// les_step.cuh -- the whole time step (main.f95:260-296) as one launch sequence.
#pragma once
#include <cuda_runtime.h>

#include "../../include/les_gpu.h"
#include "les_common.cuh"
#include "les_kernels.cuh"
#include "les_sor.cuh"

// Captured CUDA graphs of one step: [0] for n == 1 (bondv1's initial fill), [1] for n > 1.
struct LesStepPlan {
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  long long launches[2] = {0, 0};  // kernels inside each graph
  int sor_ny = 0;                  // fused SOR tile height (warps per CTA), 0 = simple path
  LesSorMaps maps;                 // tensor maps of the SOR buffers for sor_ny
};

int les_step_parts_needed(int im, int jm, int km, int sms);
void les_step_plan_free(LesStepPlan *plan);
// Queue one step on ctx.s.  Returns 0 or a CUDA error code.
int les_step_run(const LesDom &d, const les_params &prm, LesStepPlan *plan, int n, int nmax, LesCtx ctx);
// Single passes of the step's heavy kernels, for profiling (les_gpu_profile).
int les_step_sor_pass(const LesDom &d, const les_params &prm, LesStepPlan *plan, LesCtx ctx);  // iterations run
int les_step_pick_ny(const LesDom &d);
void les_step_velfg_pass(const LesDom &d, LesCtx ctx);
void les_step_les_pass(const LesDom &d, LesCtx ctx);
// The launch sequence itself (no graph), used for capture and by tests.
void les_step_enqueue(const LesDom &d, const les_params &prm, int ny, const LesSorMaps *maps, int n, LesCtx ctx);
