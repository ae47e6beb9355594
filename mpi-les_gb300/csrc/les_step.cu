// les_step.cu -- one whole time step, captured once per domain as a CUDA graph.
//
// The step is the reference's subroutine sequence (main.f95:260-296).  Its launch
// sequence is recorded into a graph the first time a step runs (one graph for n == 1,
// which includes bondv1's initial fill, one for n > 1) and replayed afterwards, so a
// step costs one graph launch on the host.  The SOR early exit of press.f95:119 is a
// device-side flag: once set, the remaining SOR launches of the graph return at once.
#include <cuda_runtime.h>

#include "les_step.cuh"

int les_step_parts_needed(int im, int jm, int km) {
  (void)im; (void)jm; (void)km;
  return 0;
}

void les_step_plan_free(LesStepPlan *plan) {
  for (int q = 0; q < 2; ++q) {
    if (plan->exec[q]) cudaGraphExecDestroy(plan->exec[q]);
    plan->exec[q] = nullptr;
    plan->launches[q] = 0;
  }
}

void les_step_enqueue(const LesDom &d, const les_params &prm, int sor_depth, int n, LesCtx ctx) {
  (void)sor_depth;
  les_launch_velnw(d, ctx);
  les_launch_bondv1(d, n, ctx);
  les_launch_velfg(d, ctx);
  les_launch_feedbf(d, ctx);
  les_launch_les(d, ctx);
  les_launch_adam(d, ctx);
  les_launch_bondfg(d, ctx);
  les_launch_rhs_mean(d, ctx);
  les_launch_sor_simple(d, prm.nmaxp, ctx);
  les_launch_pav_adjust(d, ctx);
}

int les_step_run(const LesDom &d, const les_params &prm, LesStepPlan *plan, int n, int nmax, LesCtx ctx) {
  (void)nmax;
  const int q = (n == 1) ? 0 : 1;
  if (!plan->exec[q]) {
    cudaGraph_t g = nullptr;
    long long cnt = 0;
    LesCtx cap{ctx.s, &cnt};
    cudaError_t e = cudaStreamBeginCapture(ctx.s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return (int)e;
    les_step_enqueue(d, prm, plan->sor_depth, n, cap);
    e = cudaStreamEndCapture(ctx.s, &g);
    if (e != cudaSuccess) return (int)e;
    e = cudaGraphInstantiate(&plan->exec[q], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      plan->exec[q] = nullptr;
      return (int)e;
    }
    plan->launches[q] = cnt;
  }
  cudaError_t e = cudaGraphLaunch(plan->exec[q], ctx.s);
  if (e != cudaSuccess) return (int)e;
  *ctx.nlaunch += plan->launches[q];
  return 0;
}

void les_step_sor_pass(const LesDom &d, const les_params &prm, LesStepPlan *plan, LesCtx ctx) {
  (void)prm; (void)plan;
  les_launch_sor_simple(d, 1, ctx);
}
void les_step_velfg_pass(const LesDom &d, LesCtx ctx) {
  les_launch_velfg(d, ctx);
  les_launch_feedbf(d, ctx);
}
void les_step_les_pass(const LesDom &d, LesCtx ctx) {
  les_launch_les(d, ctx);
  les_launch_adam(d, ctx);
}
