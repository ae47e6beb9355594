// les_batch.cu -- many resident domains advanced together: batched ensembles and the
// continuous batching of the serving loop.
//
// A batch holds domain handles (each with its own device state, CUDA stream and
// captured step graph) and a per-slot step counter.  les_batch_step enqueues one time
// step of every live member -- each member's graph on its own stream, no host
// synchronisation -- so the members' kernels overlap on the GPU: a 150x150x90 domain
// fills only a fraction of the 152 SMs per kernel, many of them fill it.  Members join
// and leave between steps (continuous batching); nothing in a member's arithmetic
// depends on the others, so a domain's result is the same alone and in any mix.
// Calls on one batch are serialised by its mutex.
//
// Concurrency across streams is limited by CUDA_DEVICE_MAX_CONNECTIONS (8 unless the
// process sets it, before CUDA initialises, up to 32).  Members share the GPU, so
// joining a batch turns off the k-split of a member's SOR march (les_params.sor_ksplit):
// the split's ring planes are extra work that pays only on an otherwise idle GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/les_gpu.h"

// les_api.cu: stop splitting the member's SOR march (the GPU is shared)
void les_handle_share_gpu(les_handle *h);

struct les_batch {
  struct Slot {
    les_handle *h = nullptr;
    int n = 0, nmax = 0;  // next step index; the member is finished once n > nmax
    bool used = false;
  };
  std::vector<Slot> slots;
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
  return LES_OK;
}

extern "C" int les_batch_destroy(les_batch *b) {
  if (!b) return LES_OK;
  {
    std::lock_guard<std::mutex> lock(b->mu);
    for (auto &s : b->slots)
      if (s.used && s.h) les_gpu_sync(s.h);
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
  b->slots[slot] = les_batch::Slot();
  return LES_OK;
}

extern "C" int les_batch_step(les_batch *b, int *nlive) {
  if (!b) return LES_ERR_ARG;
  std::lock_guard<std::mutex> lock(b->mu);
  int live = 0;
  for (int q = 0; q < (int)b->slots.size(); ++q) {
    auto &s = b->slots[q];
    if (!s.used || s.n > s.nmax) continue;
    const int rc = les_gpu_step(s.h, s.n, s.nmax);
    if (rc) {
      char m[256];
      les_gpu_last_error(s.h, m, sizeof m);
      return bfail(b, rc, "batch_step: slot " + std::to_string(q) + ": " + m);
    }
    ++s.n;
    if (s.n <= s.nmax) ++live;
  }
  if (nlive) *nlive = live;
  return LES_OK;
}

extern "C" int les_batch_sync(les_batch *b) {
  if (!b) return LES_ERR_ARG;
  std::lock_guard<std::mutex> lock(b->mu);
  for (int q = 0; q < (int)b->slots.size(); ++q) {
    auto &s = b->slots[q];
    if (!s.used) continue;
    const int rc = les_gpu_sync(s.h);
    if (rc) return bfail(b, rc, "batch_sync: slot " + std::to_string(q));
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
