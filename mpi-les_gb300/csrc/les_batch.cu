// les_batch.cu -- many resident domains advanced together: batched ensembles and the
// continuous batching of the serving loop.
//
// A batch holds domain handles (each with its own device state, CUDA stream and
// captured step graphs) and a per-slot step counter.  les_batch_step enqueues one time
// step of every live member without host synchronisation, in one of two ways:
//   - (default) each member's whole-step graph on its own stream: the members' kernels
//     overlap on the GPU (a 150x150x90 domain fills a fraction of the 152 SMs per
//     kernel, many of them fill it);
//   - (les_batch_set_sor_launch(b, 1)) SOR iterations 2..nmaxp of all members as one
//     persistent launch per tile shape over a work-list of every member's tiles
//     (les_sor_batch.cu): each member's step runs up to its first SOR iteration on its
//     own stream (a captured graph), the batched launch waits for them on the batch's
//     stream, and each member's copy-out, pav and boundary conditions follow it.
//     Members without a fused SOR sweep (odd jm, km too large, a state just uploaded)
//     step through their whole-step graph.  Measured on a GB300 it is 7% (64 domains of
//     150x150x90) and 9% (96 uneven domains) slower than the default: each member's
//     first part must finish before the launch starts, and every item of the work-list
//     pays its own pipeline start.
// Members join and leave between steps (continuous batching); nothing in a member's
// arithmetic depends on the others, so a domain's result is the same alone and in any
// mix, bit for bit, either way.  Calls on one batch are serialised by its mutex.
//
// Concurrency across streams is limited by CUDA_DEVICE_MAX_CONNECTIONS (8 unless the
// process sets it, before CUDA initialises, up to 32).  Members share the GPU, so
// joining a batch turns off the k-split of a member's SOR march (les_params.sor_ksplit):
// the split's ring planes are extra work that pays only on an otherwise idle GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/les_gpu.h"
#include "les_sor_batch.cuh"

// les_api.cu: stop splitting the member's SOR march (the GPU is shared); the member's
// view for a batched SOR launch; its step parts around the batched iterations
void les_handle_share_gpu(les_handle *h);
int les_handle_batch_view(les_handle *h, const LesDom **d, SorShape *sh, const LesSorMaps **maps, int *nmaxp,
                          cudaStream_t *s, int *ok);
int les_handle_step_part(les_handle *h, int n, int part);
int les_handle_sync_stream(les_handle *h);
void les_handle_clear_wait_error(les_handle *h);

struct les_batch {
  struct Slot {
    les_handle *h = nullptr;
    int n = 0, nmax = 0;  // next step index; the member is finished once n > nmax
    bool used = false;
    cudaEvent_t ev = nullptr;  // end of the member's part 1 in this step
  };
  // one batched SOR launch: the members of one tile shape and iteration count
  struct Group {
    SorShape sh;
    int nmaxp = 0;
    std::vector<int> slots;
    SorBatchBuffers buf;
    cudaStream_t s = nullptr;
    cudaEvent_t done = nullptr;
  };
  std::vector<Slot> slots;
  std::vector<Group> groups;
  std::vector<std::tuple<int, les_handle *, int, int, int>> key;  // (slot, handle, nx, ny, nmaxp) of the groups
  long long spin_limit = 1LL << 23;  // polls (about 128 ns each) before a dependency wait gives up
  cudaStream_t bs = nullptr;         // the stream of the batched SOR launches
  int group_size = 1 << 30;          // members per batched SOR launch (LES_BATCH_GROUP overrides);
                                     // concurrent persistent launches starve each other, so one
                                     // launch per shape is the default
  bool batched_sor = false;          // true: SOR iterations 2..nmaxp of all members in one
                                     // persistent launch (les_batch_set_sor_launch; LES_BATCH_SOR)
  int hold_slot = -1;                // test hook: this member's wait can never end
  int sms = 0;
  std::mutex mu;
  std::string err;
};

namespace {
int bfail(les_batch *b, int code, const std::string &m) {
  b->err = m;
  return code;
}
}  // namespace

extern "C" int les_batch_create(les_batch **out) {
  if (!out) return LES_ERR_ARG;
  *out = new les_batch();
  if (const char *e = getenv("LES_BATCH_GROUP")) {  // A/B measurements
    const int v = atoi(e);
    if (v > 0) (*out)->group_size = v;
  }
  if (const char *e = getenv("LES_BATCH_SOR")) (*out)->batched_sor = atoi(e) != 0;
  return LES_OK;
}

extern "C" int les_batch_destroy(les_batch *b) {
  if (!b) return LES_OK;
  {
    std::lock_guard<std::mutex> lock(b->mu);
    for (auto &s : b->slots)
      if (s.used && s.h) les_gpu_sync(s.h);
    for (auto &g : b->groups) {
      if (g.s) cudaStreamSynchronize(g.s);
      les_sor_batch_free(&g.buf);
      if (g.done) cudaEventDestroy(g.done);
    }
    for (auto &s : b->slots)
      if (s.ev) cudaEventDestroy(s.ev);
    if (b->bs) cudaStreamDestroy(b->bs);
  }
  delete b;
  return LES_OK;
}

extern "C" int les_batch_admit(const les_dims *dims, size_t reserve_bytes, int *ok) {
  if (!dims || !ok) return LES_ERR_ARG;
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    (void)cudaGetLastError();
    return LES_ERR_CUDA;
  }
  *ok = (fr >= les_domain_bytes(dims->im, dims->jm, dims->km) + reserve_bytes) ? 1 : 0;
  return LES_OK;
}

extern "C" int les_batch_add(les_batch *b, les_handle *h, int n0, int nmax, int *slot) {
  if (!b || !h || !slot || n0 < 1 || nmax < n0 - 1) return LES_ERR_ARG;
  std::lock_guard<std::mutex> lock(b->mu);
  for (auto &s : b->slots)
    if (s.used && s.h == h) return bfail(b, LES_ERR_ARG, "batch_add: handle already in the batch");
  int q = -1;
  for (int i = 0; i < (int)b->slots.size(); ++i)
    if (!b->slots[i].used) { q = i; break; }
  if (q < 0) {
    q = (int)b->slots.size();
    b->slots.emplace_back();
  }
  les_handle_share_gpu(h);
  b->slots[q].h = h;
  b->slots[q].n = n0;
  b->slots[q].nmax = nmax;
  b->slots[q].used = true;
  *slot = q;
  return LES_OK;
}

extern "C" int les_batch_remove(les_batch *b, int slot) {
  if (!b) return LES_ERR_ARG;
  std::lock_guard<std::mutex> lock(b->mu);
  if (slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].used)
    return bfail(b, LES_ERR_ARG, "batch_remove: no such slot");
  les_gpu_sync(b->slots[slot].h);
  cudaEvent_t ev = b->slots[slot].ev;
  b->slots[slot] = les_batch::Slot();
  b->slots[slot].ev = ev;
  return LES_OK;
}

namespace {

// Group the batched members by (tile shape, iteration count) and bring each group's
// member table and work list up to date.  Tables are compared by content (a handle freed
// and another created at the same address is a different member); when any differs,
// the launches in flight finish before the new tables are uploaded.
int regroup(les_batch *b, const std::vector<std::tuple<int, les_handle *, int, int, int>> &key,
            const std::vector<const LesDom *> &doms, const std::vector<const LesSorMaps *> &maps) {
  // (nx, ny, nmaxp, chunk) -> indices into key.  Members of one shape are split into
  // chunks of at most group_size: each chunk's launch waits only for its own members'
  // first part, so one chunk's SOR overlaps the other chunks' remaining kernels.
  std::map<std::tuple<int, int, int>, std::vector<int>> shape;
  for (int q = 0; q < (int)key.size(); ++q)
    shape[{std::get<2>(key[q]), std::get<3>(key[q]), std::get<4>(key[q])}].push_back(q);
  std::map<std::tuple<int, int, int, int>, std::vector<int>> by;
  for (auto &kv : shape) {
    const int n = (int)kv.second.size();
    const int nch = std::max(1, (n + b->group_size - 1) / b->group_size);
    for (int q = 0; q < n; ++q)
      by[{std::get<0>(kv.first), std::get<1>(kv.first), std::get<2>(kv.first), q * nch / n}].push_back(kv.second[q]);
  }
  while (b->groups.size() < by.size()) b->groups.emplace_back();
  struct Pending {
    size_t g;
    std::vector<SorBatchDom> host;
    std::vector<int> owner;
  };
  std::vector<Pending> changed;
  size_t gi = 0;
  for (auto &kv : by) {
    les_batch::Group &g = b->groups[gi];
    if (!b->bs && cudaStreamCreateWithFlags(&b->bs, cudaStreamNonBlocking) != cudaSuccess) return LES_ERR_CUDA;
    g.s = b->bs;  // one stream: the batched launches never run side by side (they would starve each other)
    if (!g.done && cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming) != cudaSuccess) return LES_ERR_CUDA;
    const SorShape sh{std::get<0>(kv.first), std::get<1>(kv.first), 0, 1};
    const int nmaxp = std::get<2>(kv.first);
    std::vector<const LesDom *> gd;
    std::vector<const LesSorMaps *> gm;
    std::vector<int> slots;
    for (int q : kv.second) {
      slots.push_back(std::get<0>(key[q]));
      gd.push_back(doms[q]);
      gm.push_back(maps[q]);
    }
    Pending p{gi, {}, {}};
    if (les_sor_batch_build(gd, gm, sh, nmaxp, g.buf, &p.host, &p.owner)) changed.push_back(std::move(p));
    g.sh = sh;
    g.nmaxp = nmaxp;
    g.slots = slots;
    ++gi;
  }
  for (size_t q = gi; q < b->groups.size(); ++q) b->groups[q].slots.clear();  // unused now
  if (!changed.empty()) {
    for (auto &g : b->groups)
      if (g.s && cudaStreamSynchronize(g.s) != cudaSuccess) return LES_ERR_CUDA;
    for (auto &p : changed) {
      les_batch::Group &g = b->groups[p.g];
      if (les_sor_batch_upload(std::move(p.host), std::move(p.owner), g.sh, g.nmaxp, &g.buf) != 0) return LES_ERR_NOMEM;
    }
  }
  b->key = key;
  return LES_OK;
}

}  // namespace

extern "C" int les_batch_step(les_batch *b, int *nlive) {
  if (!b) return LES_ERR_ARG;
  std::lock_guard<std::mutex> lock(b->mu);
  if (!b->sms) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      (void)cudaGetLastError();
      b->sms = 152;
    }
  }
  auto member_fail = [&](int q, int rc, const char *what) {
    char m[256];
    les_gpu_last_error(b->slots[q].h, m, sizeof m);
    return bfail(b, rc, std::string("batch_step: slot ") + std::to_string(q) + " " + what + ": " + m);
  };
  // the live members, and which of them take part in the batched SOR launches
  std::vector<std::tuple<int, les_handle *, int, int, int>> key;
  std::vector<const LesDom *> doms;
  std::vector<const LesSorMaps *> maps;
  std::vector<int> alone;
  std::vector<cudaStream_t> streams(b->slots.size(), nullptr);
  for (int q = 0; q < (int)b->slots.size(); ++q) {
    auto &s = b->slots[q];
    if (!s.used || s.n > s.nmax) continue;
    const LesDom *d = nullptr;
    SorShape sh;
    const LesSorMaps *mp = nullptr;
    int nmaxp = 0, ok = 0;
    les_handle_batch_view(s.h, &d, &sh, &mp, &nmaxp, &streams[q], &ok);
    if (!ok || nmaxp < 2 || !b->batched_sor) {
      alone.push_back(q);
      continue;
    }
    key.emplace_back(q, s.h, sh.nx, sh.ny, nmaxp);
    doms.push_back(d);
    maps.push_back(mp);
  }
  int rc = regroup(b, key, doms, maps);
  if (rc) return bfail(b, rc, "batch_step: building the batched SOR work list failed");
  // 1. each batched member up to its first SOR iteration, on its own stream
  for (const auto &g : b->groups)
    for (int q : g.slots) {
      auto &s = b->slots[q];
      if ((rc = les_handle_step_part(s.h, s.n, 1))) return member_fail(q, rc, "part 1");
      if (!s.ev && cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming) != cudaSuccess)
        return bfail(b, LES_ERR_CUDA, "batch_step: event");
      if (cudaEventRecord(s.ev, streams[q]) != cudaSuccess) return bfail(b, LES_ERR_CUDA, "batch_step: event record");
    }
  // 2. SOR iterations 2..nmaxp of each group's members in one persistent launch
  for (auto &g : b->groups) {
    if (g.slots.empty()) continue;
    for (int q : g.slots)
      if (cudaStreamWaitEvent(g.s, b->slots[q].ev, 0) != cudaSuccess) return bfail(b, LES_ERR_CUDA, "batch_step: wait");
    int hold = -1;
    for (int m = 0; m < (int)g.slots.size(); ++m)
      if (g.slots[m] == b->hold_slot) hold = m;
    if (les_sor_batch_launch(g.buf, b->sms, b->spin_limit, hold, g.s) != 0)
      return bfail(b, LES_ERR_CUDA, std::string("batch_step: batched SOR launch: ") + cudaGetErrorString(cudaGetLastError()));
    if (cudaEventRecord(g.done, g.s) != cudaSuccess) return bfail(b, LES_ERR_CUDA, "batch_step: event record");
  }
  // 3. each batched member's copy-out, pav and boundary conditions, after its group
  for (const auto &g : b->groups)
    for (int q : g.slots) {
      if (cudaStreamWaitEvent(streams[q], g.done, 0) != cudaSuccess) return bfail(b, LES_ERR_CUDA, "batch_step: wait");
      if ((rc = les_handle_step_part(b->slots[q].h, b->slots[q].n, 2))) return member_fail(q, rc, "part 2");
    }
  // members outside the batched launches: their whole step
  for (int q : alone) {
    auto &s = b->slots[q];
    if ((rc = les_gpu_step(s.h, s.n, s.nmax))) return member_fail(q, rc, "step");
  }
  int live = 0;
  for (auto &s : b->slots) {
    if (!s.used || s.n > s.nmax) continue;
    ++s.n;
    if (s.n <= s.nmax) ++live;
  }
  if (nlive) *nlive = live;
  return LES_OK;
}

extern "C" int les_batch_set_sor_launch(les_batch *b, int persistent) {
  if (!b || persistent < 0 || persistent > 1) return LES_ERR_ARG;
  std::lock_guard<std::mutex> lock(b->mu);
  b->batched_sor = persistent != 0;
  return LES_OK;
}

extern "C" int les_batch_set_wait_limit(les_batch *b, long long polls, int hold_slot) {
  if (!b || polls < 1) return LES_ERR_ARG;
  std::lock_guard<std::mutex> lock(b->mu);
  b->spin_limit = polls;
  b->hold_slot = hold_slot;
  return LES_OK;
}

extern "C" int les_batch_sync(les_batch *b) {
  if (!b) return LES_ERR_ARG;
  std::lock_guard<std::mutex> lock(b->mu);
  for (int q = 0; q < (int)b->slots.size(); ++q) {
    auto &s = b->slots[q];
    if (!s.used) continue;
    const int rc = les_handle_sync_stream(s.h);
    if (rc) return bfail(b, rc, "batch_sync: slot " + std::to_string(q));
  }
  for (auto &g : b->groups) {
    if (!g.s) continue;
    int st = 0;
    if (les_sor_batch_status(g.buf, g.s, &st) != 0) return bfail(b, LES_ERR_CUDA, "batch_sync: batched SOR");
    if (st) {
      // clear the record, so that later steps report only their own failures
      if (g.buf.counters) cudaMemsetAsync(g.buf.counters + 1, 0, sizeof(unsigned), g.s);
      cudaStreamSynchronize(g.s);
      for (auto &s : b->slots)
        if (s.used) les_handle_clear_wait_error(s.h);
      return bfail(b, LES_ERR_STATE,
                   "batch_sync: a dependency wait of the batched SOR launch gave up; the members' SOR of that step "
                   "did not finish");
    }
  }
  for (int q = 0; q < (int)b->slots.size(); ++q) {  // a member kernel's own give-up
    auto &s = b->slots[q];
    if (!s.used) continue;
    const int rc = les_gpu_sync(s.h);
    if (rc) {
      char msg[256] = {0};
      les_gpu_last_error(s.h, msg, sizeof msg);
      return bfail(b, rc, "batch_sync: slot " + std::to_string(q) + ": " + msg);
    }
  }
  return LES_OK;
}

extern "C" int les_batch_slot(les_batch *b, int slot, int *n, int *nmax) {
  if (!b) return LES_ERR_ARG;
  std::lock_guard<std::mutex> lock(b->mu);
  if (slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].used) return LES_ERR_ARG;
  if (n) *n = b->slots[slot].n;
  if (nmax) *nmax = b->slots[slot].nmax;
  return LES_OK;
}

extern "C" int les_batch_last_error(les_batch *b, char *buf, size_t len) {
  if (!b || !buf || len == 0) return LES_ERR_ARG;
  std::lock_guard<std::mutex> lock(b->mu);
  const size_t n = std::min(len - 1, b->err.size());
  b->err.copy(buf, n);
  buf[n] = 0;
  return LES_OK;
}
