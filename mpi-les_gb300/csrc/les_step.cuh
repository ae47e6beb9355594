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
  // the step cut around SOR iterations 2..nmaxp, for batches whose SOR runs in one
  // persistent launch over all members: [0] before (n == 1), [1] before (n > 1), [2] after
  cudaGraphExec_t part_exec[3] = {nullptr, nullptr, nullptr};
  long long part_launches[3] = {0, 0, 0};
  SorShape sor;                    // fused SOR tile shape (sor.ny == 0: per-subroutine path)
  int sor_picked = 0;              // sor chosen (and maps made) for this plan
  LesSorMaps maps;                 // tensor maps of the SOR buffers for sor
  SorShape fixed{0, 0, 0, 0};      // caller's choice (les_gpu_set_sor_shape), 0 = automatic;
                                   // kept across les_step_plan_free
  long long part_cap = 0;          // residual partials the domain's buffer holds
};

int les_step_parts_needed(int im, int jm, int km, int sms);
void les_step_plan_free(LesStepPlan *plan);
// Queue one step on ctx.s.  Returns 0 or a CUDA error code.
int les_step_run(const LesDom &d, const les_params &prm, LesStepPlan *plan, int n, int nmax, LesCtx ctx);
// Single passes of the step's heavy kernels, for profiling (les_gpu_profile).
int les_step_sor_pass(const LesDom &d, const les_params &prm, LesStepPlan *plan, LesCtx ctx);  // iterations run
// One SOR pass as the step runs it, with a recorded after the first sweep and b after the
// last: returns the sweeps between them (0: no fused sweep for this domain)
int les_step_sor_sweeps(const LesDom &d, const les_params &prm, LesStepPlan *plan, LesCtx ctx, cudaEvent_t a,
                        cudaEvent_t b);
SorShape les_step_pick_shape(const LesDom &d);
// The plan's SOR shape (picked on first use): the automatic choice with the fixed
// parts applied.
SorShape les_step_plan_shape(const LesDom &d, LesStepPlan *plan);
void les_step_velfg_pass(const LesDom &d, LesCtx ctx);
void les_step_les_pass(const LesDom &d, LesCtx ctx);
// The launch sequence itself (no graph), used for capture and by tests.
void les_step_enqueue(const LesDom &d, const les_params &prm, SorShape sh, const LesSorMaps *maps, int n, LesCtx ctx);
// The step in two parts around SOR iterations 2..nmaxp (which a batched launch runs,
// les_sor_batch.cu): part 1 is velnw .. rhs and SOR iteration 1 (p into sorB), part 2
// the copy-out of the last SOR result, pav and the final boundary conditions.  Needs a
// plan with a fused sweep.  Returns 0 or a CUDA error code.
int les_step_run_part(const LesDom &d, const les_params &prm, LesStepPlan *plan, int n, int part, LesCtx ctx);
