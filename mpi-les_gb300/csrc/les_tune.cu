// les_tune.cu -- measured choice of the fused SOR sweep's tile shape per size class.
//
// The shape that runs press's SOR fastest depends on how the domain shares the GPU:
// alone, its tiles (and k chunks) must fill the SMs and the CTA size sets how much
// latency one SM hides; as one of many batch members, the SMs are full anyway and
// what counts is the work the tiles issue, ring cells included, and how well two
// CTAs share an SM.  Neither is captured well by a formula, so the tuner times the
// candidates: it copies the domain's LesDom, points the SOR buffers (p ping-pong,
// rhs, residual partials, tickets, control words) at scratch memory and runs SOR
// iterations of R such replicas at once in one CUDA graph -- R = 1 for a domain alone,
// enough replicas for four waves of CTAs for a batch member -- and keeps the shape
// with the least time per replica and iteration.  The grid coefficients are the
// domain's own (read only); the iteration count is fixed (sor_fixed), so every
// candidate does the same work.  Results go into a process-wide table keyed by
// (im, jm, km, shared, SMs) that the step planner consults.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "les_sor.cuh"
#include "les_tune.cuh"

namespace {

struct Key {
  int im, jm, km, shared, sms;
  bool operator<(const Key &o) const {
    return std::tie(im, jm, km, shared, sms) < std::tie(o.im, o.jm, o.km, o.shared, o.sms);
  }
};
std::mutex g_mu;
std::map<Key, SorShape> g_table;

int sms_of(const LesDom &d) { return d.sms > 0 ? d.sms : 152; }

std::vector<SorShape> candidates(const LesDom &d, bool shared) {
  std::vector<SorShape> c;
  const int sms = sms_of(d);
  for (int ny : {16, 20, 24, 28})
    for (int nx : {32, 16}) {
      if (shared) {
        c.push_back(SorShape{nx, ny, d.km});
        continue;
      }
      // alone: the whole march and k splits up to two waves of CTAs (a 32-column CTA
      // holds an SM, two 16-column ones share one), chunks of >= 4 planes
      const int tiles = les_sor_fused_tiles(d.im, d.jm, SorShape{nx, ny, 0});
      const long long slots = (nx == 16 ? 2LL : 1LL) * sms;
      int last = -1;
      for (int nch : {1, 2, 3, 4, 6, 8, 12, 16, 24}) {
        const int kc = (d.km + nch - 1) / nch;
        const int n = (d.km + kc - 1) / kc;
        if (kc == last || (nch > 1 && (kc < 4 || (long long)tiles * n > 2LL * slots))) continue;
        c.push_back(SorShape{nx, ny, kc});
        last = kc;
      }
    }
  // two iterations per k-march (les_sor2.cu): 32-column tiles, the whole march
  for (int ny : {24, 28, 32}) {
    const SorShape two{32, ny, d.km, 2};
    if (les_sor_two_ok(d, two)) c.push_back(two);
  }
  return c;
}

// Scratch SOR state of R replicas in one allocation.
struct Scratch {
  char *base = nullptr;
  std::vector<LesDom> dom;
  std::vector<LesSorMaps> maps;
  std::vector<cudaStream_t> st;
  size_t nfloat = 0, npart = 0;
  ~Scratch() {
    for (cudaStream_t s : st) cudaStreamDestroy(s);
    if (base) cudaFree(base);
  }
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t replica_bytes(size_t nfloat, size_t npart) {
  return 3 * align256(nfloat * sizeof(float)) + align256(npart * sizeof(double)) + 256 /*cnt*/ +
         256 /*ctl*/ + 256 /*scal*/ + 256 /*fscal*/;
}

int make_scratch(const LesDom &d0, int R, size_t npart, Scratch *S) {
  S->nfloat = (size_t)d0.np * (size_t)(d0.km + 4);
  S->npart = npart;
  const size_t per = replica_bytes(S->nfloat, npart);
  if (cudaMalloc(&S->base, per * R) != cudaSuccess) {
    (void)cudaGetLastError();
    S->base = nullptr;
    return -1;
  }
  if (cudaMemset(S->base, 0, per * R) != cudaSuccess) return -2;
  S->dom.resize(R);
  S->maps.resize(R);
  S->st.resize(R, nullptr);
  for (int r = 0; r < R; ++r) {
    char *q = S->base + per * r;
    LesDom d = d0;
    auto take = [&](size_t bytes) {
      char *p = q;
      q += bytes;
      return p;
    };
    d.sorA = reinterpret_cast<float *>(take(align256(S->nfloat * sizeof(float))));
    d.sorB = reinterpret_cast<float *>(take(align256(S->nfloat * sizeof(float))));
    d.sorR = reinterpret_cast<float *>(take(align256(S->nfloat * sizeof(float))));
    d.part = reinterpret_cast<double *>(take(align256(npart * sizeof(double))));
    d.cnt = reinterpret_cast<unsigned int *>(take(256));
    d.ctl = reinterpret_cast<int *>(take(256));
    d.scal = reinterpret_cast<double *>(take(256));
    d.fscal = reinterpret_cast<float *>(take(256));
    d.p = d.sorA;      // never read: only iterations on the internal buffers are timed
    d.sor_fixed = 1;   // no convergence exit: every candidate runs every iteration
    S->dom[r] = d;
    if (cudaStreamCreateWithFlags(&S->st[r], cudaStreamNonBlocking) != cudaSuccess) return -3;
  }
  return 0;
}

// Seconds per replica and iteration of shape sh (the least of `reps` graph launches).
int time_shape(Scratch &S, SorShape sh, int iters, int reps, cudaStream_t s0, double *sec) {
  const int R = (int)S.dom.size();
  for (int r = 0; r < R; ++r)
    if (les_sor_make_maps(S.dom[r], sh, &S.maps[r]) != 0) return -1;
  const int tiles = les_sor_fused_tiles(S.dom[0].im, S.dom[0].jm, sh);
  const int kc = sh.kchunk > 0 ? sh.kchunk : S.dom[0].km;
  const int nch = (S.dom[0].km + kc - 1) / kc;
  const int per = (sh.depth == 2) ? 2 : 1;  // iterations per launch
  if ((size_t)tiles * nch * per > S.npart) return -2;
  cudaEvent_t fork, t0, t1;
  std::vector<cudaEvent_t> join(R);
  cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
  for (auto &e : join) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  int rc = 0;
  if (cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = -3;
  if (!rc) {
    cudaEventRecord(fork, s0);
    for (int r = 0; r < R; ++r) {
      cudaStreamWaitEvent(S.st[r], fork, 0);
      const LesDom &d = S.dom[r];
      for (int l = 0; l < iters; l += per) {
        SorArgs a;
        a.psrc = ((l / per) & 1) ? d.sorB : d.sorA;
        a.pdst = ((l / per) & 1) ? d.sorA : d.sorB;
        a.ghost = 1;
        a.rhs = d.sorR;
        a.depth = per;
        a.tj = sh.ny - 4 * per;
        a.kchunk = kc;
        a.nchunk = nch;
        a.ntiles = tiles * nch;
        a.part = d.part;
        a.counter = d.cnt;
        les_launch_sor_iter(d, a, sh, &S.maps[r], S.st[r]);
      }
      cudaEventRecord(join[r], S.st[r]);
      cudaStreamWaitEvent(s0, join[r], 0);
    }
    if (cudaStreamEndCapture(s0, &g) != cudaSuccess) rc = -4;
  }
  if (!rc && cudaGraphInstantiate(&ge, g, 0) != cudaSuccess) rc = -5;
  double best = 1e30;
  if (!rc) {
    cudaGraphLaunch(ge, s0);  // warm-up
    for (int q = 0; q < reps && !rc; ++q) {
      cudaEventRecord(t0, s0);
      cudaGraphLaunch(ge, s0);
      cudaEventRecord(t1, s0);
      if (cudaEventSynchronize(t1) != cudaSuccess) rc = -6;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, t0, t1);
      best = std::min(best, (double)ms * 1e-3);
    }
  }
  if (ge) cudaGraphExecDestroy(ge);
  if (g) cudaGraphDestroy(g);
  cudaEventDestroy(fork);
  for (auto &e : join) cudaEventDestroy(e);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (!rc && cudaGetLastError() != cudaSuccess) rc = -7;
  *sec = best / ((double)R * iters);
  return rc;
}

}  // namespace

bool les_tune_lookup(int im, int jm, int km, int shared, int sms, SorShape *out) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_table.find(Key{im, jm, km, shared ? 1 : 0, sms});
  if (it == g_table.end()) return false;
  *out = it->second;
  return true;
}

void les_tune_store(int im, int jm, int km, int shared, int sms, SorShape sh) {
  std::lock_guard<std::mutex> lk(g_mu);
  const Key k{im, jm, km, shared ? 1 : 0, sms};
  if (sh.nx == 0) g_table.erase(k);
  else g_table[k] = sh;
}

int les_tune_sor(const LesDom &d, bool shared, size_t mem_budget, SorShape *best, double *best_sec,
                 std::string *report) {
  if (d.jm % 2 != 0 || d.km + 1 >= LES_SOR_KMAX || !d.gr.cn1k) return 1;  // no fused sweep to tune
  const std::vector<SorShape> cands = candidates(d, shared);
  const int sms = sms_of(d);
  size_t npart = 64;
  int min_tiles = 1 << 30;
  for (const SorShape &c : cands) {
    const int t = les_sor_fused_tiles(d.im, d.jm, c);
    npart = std::max(npart, (size_t)t * (size_t)((d.km + c.kchunk - 1) / c.kchunk) * (size_t)c.depth + 64);
    min_tiles = std::min(min_tiles, t);
  }
  // batch members: about four waves of two CTAs per SM, within the memory budget
  int R = 1;
  if (shared) {
    R = std::max(1, (8 * sms + min_tiles - 1) / min_tiles);
    const size_t per = replica_bytes((size_t)d.np * (d.km + 4), npart);
    R = (int)std::min<size_t>((size_t)R, std::max<size_t>(1, mem_budget / per));
    R = std::min(R, 256);
  }
  Scratch S;
  if (make_scratch(d, R, npart, &S) != 0) return -1;
  cudaStream_t s0;
  if (cudaStreamCreateWithFlags(&s0, cudaStreamNonBlocking) != cudaSuccess) return -2;
  const int iters = shared ? 4 : 8;
  *best_sec = 1e30;
  char line[96];
  if (report) {
    snprintf(line, sizeof line, "im=%d jm=%d km=%d shared=%d replicas=%d iters=%d\n", d.im, d.jm, d.km,
             shared ? 1 : 0, R, iters);
    *report += line;
  }
  int rc = 0;
  for (const SorShape &c : cands) {
    double sec = 0.0;
    rc = time_shape(S, c, iters, 3, s0, &sec);
    if (rc) break;
    if (report) {
      snprintf(line, sizeof line, "  nx=%d ny=%d kchunk=%d depth=%d: %.2f us\n", c.nx, c.ny, c.kchunk, c.depth,
               sec * 1e6);
      *report += line;
    }
    if (sec < *best_sec) {
      *best_sec = sec;
      *best = c;
    }
  }
  // a wait that gave up inside a timed kernel (never expected) voids the result
  int ctl_err = 0;
  for (const LesDom &r : S.dom) {
    int ctl[CT_COUNT] = {0};
    if (cudaMemcpy(ctl, r.ctl, sizeof ctl, cudaMemcpyDeviceToHost) != cudaSuccess) rc = rc ? rc : -8;
    ctl_err |= ctl[CT_ERROR];
  }
  cudaStreamDestroy(s0);
  if (rc) return rc;
  if (ctl_err) return -9;
  les_tune_store(d.im, d.jm, d.km, shared, sms, *best);
  return 0;
}
