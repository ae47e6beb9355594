// les_step.cu -- one whole time step, captured once per domain as a CUDA graph.
//
// The step is the reference's subroutine sequence (main.f95:260-296).  Its launch
// sequence is recorded into a graph the first time a step runs (one graph for n == 1,
// which includes bondv1's initial fill, one for n > 1) and replayed afterwards, so a
// step costs one graph launch on the host.  press runs its SOR as the fused red-black
// sweep of les_sor.cu (one launch per iteration, ping-ponging p between two buffers);
// the early exit of press.f95:119 is a device-side flag that turns the remaining
// sweeps of the graph into no-ops.
#include <cuda_runtime.h>

#include <cstdlib>

#include "les_sor.cuh"
#include "les_step.cuh"
#include "les_tune.cuh"

int les_step_parts_needed(int im, int jm, int km, int sms) {
  int worst = 0;
  for (int nx : {32, 16})
    for (int ny = 16; ny <= 28; ny += 4) {
      const int t = les_sor_fused_tiles(im, jm, SorShape{nx, ny});
      const int kc = les_sor_pick_kchunk(t, km, sms > 0 ? sms : 152);
      const int parts = t * ((km + kc - 1) / kc);
      worst = parts > worst ? parts : worst;
    }
  for (int ny = 24; ny <= 32; ny += 4) {  // two-iteration marches: two partials per tile
    const int parts = 2 * les_sor_fused_tiles(im, jm, SorShape{32, ny, km, 2});
    worst = parts > worst ? parts : worst;
  }
  return worst + 64;
}

void les_step_plan_free(LesStepPlan *plan) {
  for (int q = 0; q < 2; ++q) {
    if (plan->exec[q]) cudaGraphExecDestroy(plan->exec[q]);
    plan->exec[q] = nullptr;
    plan->launches[q] = 0;
  }
  for (int q = 0; q < 3; ++q) {
    if (plan->part_exec[q]) cudaGraphExecDestroy(plan->part_exec[q]);
    plan->part_exec[q] = nullptr;
    plan->part_launches[q] = 0;
  }
  plan->sor = SorShape{};
  plan->sor_picked = 0;
  plan->maps.valid = 0;
}

SorShape les_step_pick_shape(const LesDom &d) {
  if (d.jm % 2 != 0) return SorShape{};            // the wrapped j ring needs an even jm
  if (d.km + 1 >= LES_SOR_KMAX) return SorShape{};  // per-k coefficients staged in shared memory
  const int sms = d.sms > 0 ? d.sms : 152;
  SorShape sh;
  // a measured shape for the size class (les_tune_sor), else the model's choice
  if (!les_tune_lookup(d.im, d.jm, d.km, d.sor_ksplit != 0, sms, &sh)) sh = les_sor_pick_shape(d.im, d.jm, sms, d.sor_ksplit != 0);
  // A/B measurements: LES_SOR_NX (32, 16), LES_SOR_NY (16, 20, 24, 28, 32), LES_SOR_DEPTH (1, 2)
  if (const char *e = getenv("LES_SOR_NX")) {
    const int v = atoi(e);
    if (v == 16 || v == 32) sh.nx = v;
  }
  if (const char *e = getenv("LES_SOR_NY")) {
    const int v = atoi(e);
    if (v == 16 || v == 20 || v == 24 || v == 28 || v == 32) sh.ny = v;
  }
  if (const char *e = getenv("LES_SOR_DEPTH")) {
    const int v = atoi(e);
    if (v == 1 || v == 2) sh.depth = v;
  }
  if (!d.gr.cn1k) sh.nx = 32;  // 16-column tiles are built for a uniform cn1 only
  return sh;
}

static void plan_pick(const LesDom &d, LesStepPlan *plan) {
  if (plan->sor_picked) return;
  SorShape sh = les_step_pick_shape(d);
  if (sh.ny > 0) {
    if (plan->fixed.nx && (plan->fixed.nx == 32 || d.gr.cn1k)) sh.nx = plan->fixed.nx;
    if (plan->fixed.ny) sh.ny = plan->fixed.ny;
    if (plan->fixed.depth) sh.depth = plan->fixed.depth;
    // two iterations per march: the whole march, where the domain allows it and its
    // partials fit; else one iteration per launch (32-row tiles exist for depth 2 only)
    if (sh.depth == 2) {
      SorShape two = sh;
      two.kchunk = d.km;
      if (!les_sor_two_ok(d, two) ||
          (plan->part_cap > 0 && 2LL * les_sor_fused_tiles(d.im, d.jm, two) > plan->part_cap))
        sh.depth = 1;
    }
    if (sh.depth != 2) sh.depth = 1;
    if (sh.depth == 1 && sh.ny == 32) sh.ny = 28;
    const int tiles = les_sor_fused_tiles(d.im, d.jm, sh);
    // k chunks: fixed by the caller, else tuned for the class, else (alone on the GPU,
    // 32-column tiles) enough to fill the SMs
    int kc = d.km;
    if (plan->fixed.kchunk > 0) kc = plan->fixed.kchunk;
    else if (sh.kchunk > 0 && !plan->fixed.nx && !plan->fixed.ny) kc = sh.kchunk;  // tuned
    else if (sh.nx == 32 && !d.sor_ksplit) kc = les_sor_pick_kchunk(tiles, d.km, d.sms > 0 ? d.sms : 152);
    kc = kc < 1 ? 1 : (kc > d.km ? d.km : kc);
    if (plan->part_cap > 0 && (long long)tiles * ((d.km + kc - 1) / kc) > plan->part_cap) kc = d.km;
    if (sh.depth == 2) kc = d.km;
    sh.kchunk = kc;
  }
  plan->sor = sh;
  plan->maps.valid = 0;
  if (sh.ny > 0 && les_sor_make_maps(d, sh, &plan->maps) != 0) plan->maps.valid = 0;
  plan->sor_picked = 1;
}

SorShape les_step_plan_shape(const LesDom &d, LesStepPlan *plan) {
  plan_pick(d, plan);
  return plan->sor;
}

// Iteration 1 reads p and writes sorB; each later launch (one iteration, or two with
// sh.depth == 2) reads the buffer the previous launch wrote and writes the other one,
// or, for the launch that ends with iteration nmaxp, p itself.  A copy-out moves the
// result into p when the sweep stopped early (press.f95:119) or ran a single
// iteration.  With the exit test on, each two-iteration launch is followed by a redo
// launch that cuts it back to its first iteration if that one met the test.
// ev_first / ev_last (optional) are recorded after the first and after the last launch.
// p_ghosts: the SOR-path rhs kernel has just written p's periodic ghost rows (saving
// row jm+2), so the first iteration may read p by tensor copies and the copy-out puts
// row jm+2 back.
static void enqueue_sor_fused(const LesDom &d, const les_params &prm, SorShape sh, const LesSorMaps *maps,
                              LesCtx ctx, cudaEvent_t ev_first = nullptr, cudaEvent_t ev_last = nullptr,
                              bool p_ghosts = false) {
  les_launch_sor_begin(d, ctx);
  const int nit = prm.nmaxp;
  SorShape one = sh;
  one.depth = 1;
  if (one.ny == 32) one.ny = 28;
  const bool two_ok = sh.depth == 2 && maps && maps->valid && les_sor_two_ok(d, sh);
  const float *cur = d.p;
  for (int l = 1; l <= nit;) {
    const bool two = two_ok && l >= 2 && l + 1 <= nit;
    const SorShape &use = two ? sh : one;
    const int lend = two ? l + 1 : l;
    const int tiles = les_sor_fused_tiles(d.im, d.jm, use);
    const int kchunk = (!two && use.kchunk > 0) ? use.kchunk : d.km;
    const int nchunk = (d.km + kchunk - 1) / kchunk;
    SorArgs a;
    a.psrc = cur;
    const bool last = (lend == nit) && (nit > 1);
    a.pdst = last ? d.p : ((cur == d.sorB) ? d.sorA : d.sorB);
    a.dstcode = last ? 2 : (a.pdst == d.sorA ? 0 : 1);
    a.ghost = last ? 0 : (two_ok ? 2 : 1);  // a two-iteration plan reads four ghost rows
    a.rhs = d.sorR;
    a.depth = two ? 2 : 1;
    a.tj = use.ny - 4 * a.depth;
    a.kchunk = kchunk;
    a.nchunk = nchunk;
    a.ntiles = tiles * nchunk;
    a.part = d.part;
    a.counter = d.cnt;
    a.src_ghosts = (cur == d.p && p_ghosts) ? 1 : 0;
    // a one-iteration launch on a depth-2 plan takes the maps' tile height only if it
    // has a one-iteration kernel (not ny = 32: then the register kernel runs)
    les_launch_sor_iter(d, a, (two || maps == nullptr || maps->shape.ny == one.ny) ? use : one,
                        (two || (maps && maps->shape.ny == one.ny)) ? maps : nullptr, ctx.s);
    ++*ctx.nlaunch;
    if (two && !prm.sor_fixed) {
      les_launch_sor_redo(d, a, ctx.s);
      ++*ctx.nlaunch;
    }
    if (l == 1 && ev_first) cudaEventRecord(ev_first, ctx.s);
    if (lend == nit && ev_last) cudaEventRecord(ev_last, ctx.s);
    cur = a.pdst;
    l = lend + 1;
  }
  les_launch_sor_copyout(d, p_ghosts ? 1 : 0, ctx.s);
  ++*ctx.nlaunch;
}

void les_step_enqueue(const LesDom &d, const les_params &prm, SorShape sh, const LesSorMaps *maps, int n, LesCtx ctx) {
  les_launch_velnw(d, ctx);
  les_launch_bondv1(d, n, ctx);
  les_launch_velfg_fused(d, true, ctx);  // velfg + feedbf
  les_launch_les_fused(d, true, ctx);    // les + adam
  les_launch_bondfg(d, ctx);
  if (sh.ny > 0) {
    les_launch_rhs_sor(d, ctx);
    enqueue_sor_fused(d, prm, sh, maps, ctx, nullptr, nullptr, true);
  } else {
    les_launch_rhs_mean(d, ctx);
    les_launch_sor_simple(d, prm.nmaxp, ctx);
  }
  les_launch_pav_adjust(d, ctx);
}

// Part 1: the step up to SOR iteration 1; part 2: after the last SOR iteration.
static void enqueue_part(const LesDom &d, const les_params &prm, SorShape sh, const LesSorMaps *maps, int n, int part,
                         LesCtx ctx) {
  if (part == 1) {
    les_launch_velnw(d, ctx);
    les_launch_bondv1(d, n, ctx);
    les_launch_velfg_fused(d, true, ctx);  // velfg + feedbf
    les_launch_les_fused(d, true, ctx);    // les + adam
    les_launch_bondfg(d, ctx);
    les_launch_rhs_sor(d, ctx);
    les_launch_sor_begin(d, ctx);
    SorShape one = sh;
    one.depth = 1;
    const int kchunk = one.kchunk > 0 ? one.kchunk : d.km;
    const int nchunk = (d.km + kchunk - 1) / kchunk;
    SorArgs a;
    a.psrc = d.p;
    a.pdst = d.sorB;  // iteration 1 always leaves p for the batched iterations (or the copy-out)
    a.dstcode = 1;
    a.ghost = 1;
    a.rhs = d.sorR;
    a.depth = 1;
    a.tj = one.ny - 4;
    a.kchunk = kchunk;
    a.nchunk = nchunk;
    a.ntiles = les_sor_fused_tiles(d.im, d.jm, one) * nchunk;
    a.part = d.part;
    a.counter = d.cnt;
    a.src_ghosts = 1;  // les_launch_rhs_sor above wrote p's ghost rows
    const bool fit = maps && maps->valid && maps->shape.nx == one.nx && maps->shape.ny == one.ny;
    les_launch_sor_iter(d, a, one, fit ? maps : nullptr, ctx.s);
    ++*ctx.nlaunch;
    (void)prm;
  } else {
    les_launch_sor_copyout(d, 1, ctx.s);  // part 1 ran the SOR-path rhs kernel
    ++*ctx.nlaunch;
    les_launch_pav_adjust(d, ctx);
  }
}

int les_step_run_part(const LesDom &d, const les_params &prm, LesStepPlan *plan, int n, int part, LesCtx ctx) {
  plan_pick(d, plan);
  if (plan->sor.ny <= 0) return (int)cudaErrorInvalidValue;
  const int q = (part == 2) ? 2 : ((n == 1) ? 0 : 1);
  if (!plan->part_exec[q]) {
    cudaGraph_t g = nullptr;
    long long cnt = 0;
    LesCtx cap{ctx.s, &cnt};
    cudaError_t e = cudaStreamBeginCapture(ctx.s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return (int)e;
    enqueue_part(d, prm, plan->sor, &plan->maps, n, part, cap);
    e = cudaStreamEndCapture(ctx.s, &g);
    if (e != cudaSuccess) return (int)e;
    e = cudaGraphInstantiate(&plan->part_exec[q], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      plan->part_exec[q] = nullptr;
      return (int)e;
    }
    plan->part_launches[q] = cnt;
  }
  cudaError_t e = cudaGraphLaunch(plan->part_exec[q], ctx.s);
  if (e != cudaSuccess) return (int)e;
  *ctx.nlaunch += plan->part_launches[q];
  return 0;
}

int les_step_run(const LesDom &d, const les_params &prm, LesStepPlan *plan, int n, int nmax, LesCtx ctx) {
  (void)nmax;
  const int q = (n == 1) ? 0 : 1;
  if (!plan->exec[q]) {
    plan_pick(d, plan);
    cudaGraph_t g = nullptr;
    long long cnt = 0;
    LesCtx cap{ctx.s, &cnt};
    cudaError_t e = cudaStreamBeginCapture(ctx.s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return (int)e;
    les_step_enqueue(d, prm, plan->sor, &plan->maps, n, cap);
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

int les_step_sor_pass(const LesDom &d, const les_params &prm, LesStepPlan *plan, LesCtx ctx) {
  plan_pick(d, plan);
  if (plan->sor.ny == 0) {
    les_launch_sor_simple(d, 1, ctx);
    return 1;
  }
  // ten iterations as the step runs them: the first reads p, the last writes p
  les_params ten = prm;
  ten.nmaxp = 10;
  enqueue_sor_fused(d, ten, plan->sor, &plan->maps, ctx);
  return 10;
}
int les_step_sor_sweeps(const LesDom &d, const les_params &prm, LesStepPlan *plan, LesCtx ctx, cudaEvent_t a,
                        cudaEvent_t b) {
  plan_pick(d, plan);
  if (plan->sor.ny == 0 || prm.nmaxp < 2) return 0;
  enqueue_sor_fused(d, prm, plan->sor, &plan->maps, ctx, a, b);  // the step's iteration count
  return prm.nmaxp - 1;
}
void les_step_velfg_pass(const LesDom &d, LesCtx ctx) { les_launch_velfg_fused(d, true, ctx); }
void les_step_les_pass(const LesDom &d, LesCtx ctx) { les_launch_les_fused(d, true, ctx); }
