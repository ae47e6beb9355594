// les_sor_batch.cu -- press's SOR iterations 2..nmaxp of many domains in one persistent
// kernel over a tile work-list (batched ensembles and the serving loop).
//
// Run one domain at a time, an SOR iteration is one launch of the fused sweep: 49
// launches per step and domain, each ending in a tail where the CTAs of the last wave
// finish while SMs idle.  For a batch, the work of every member's iterations 2..nmaxp is
// one list of items (level, member, tile): level l = iteration l + 2, items ordered
// level by level, each level listing every member's tiles.  A persistent grid of CTAs
// takes items in list order from one atomic counter.  Before it starts item (l, m, t) a
// CTA waits until member m has completed all its tiles of level l-1 (a per-member count
// of finished tiles): iteration l reads the buffer iteration l-1 wrote.  Every item a
// CTA waits for comes earlier in the list and was taken by a running CTA, so the waits
// always end; while member m's level l-1 finishes, the CTAs work on the other members'
// tiles, so nothing idles between iterations.  Each wait is bounded: after spin_limit
// polls the CTA records the failure in *status and CT_ERROR, and every CTA stops
// taking items.  Each item is one tile of the one-iteration TMA sweep (sor_tma_tile,
// les_sor_kern.cuh) with the member's own buffers, tensor maps, residual partials and
// ticket, so a member's fields, residuals and iteration count are bitwise those of its
// own launches; a member whose SOR already met the exit test (press.f95:119-121) has
// the rest of its items counted without work.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "les_common.cuh"
#include "les_sor.cuh"
#include "les_sor_batch.cuh"
#include "les_sor_kern.cuh"

namespace {

__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <int NX, int NY, int D>
__global__ void __launch_bounds__(NX *NY, min_ctas(NX)) k_sor_batch(SorBatchArgs B) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TmaSmem<NX, NY, D> &S = *reinterpret_cast<TmaSmem<NX, NY, D> *>(smem_raw);
  // the item: its index, whether to compute it, its member's domain view and the
  // iteration's arguments, all in shared memory at fixed addresses, so the march holds
  // no extra live registers for them
  __shared__ unsigned s_item;
  __shared__ int s_work, s_m;
  __shared__ LesDom s_d;
  __shared__ __align__(16) unsigned char s_a_raw[sizeof(SorArgs)];  // SorArgs has member initialisers
  SorArgs &s_a = *reinterpret_cast<SorArgs *>(s_a_raw);
  const int tid = threadIdx.y * NX + threadIdx.x;
  const unsigned total = (unsigned)B.per_level * (unsigned)B.levels;
  for (;;) {
    if (tid == 0) {
      unsigned t = atomicAdd(B.queue, 1u);
      if (t < total && *(volatile int *)B.status) t = total;  // a wait gave up: stop
      int work = 0, m = 0;
      if (t < total) {
        const int lvl = (int)(t / (unsigned)B.per_level);
        m = B.owner[t % (unsigned)B.per_level];
        const SorBatchDom &M = B.doms[m];
        // level lvl needs every tile of level lvl-1; the test hook holds one member's
        // level 1 on a count that is never reached
        const unsigned need = (unsigned)(lvl * M.ntiles) + ((m == B.hold_member && lvl == 1) ? 1u : 0u);
        long long it = 0;
        while (ld_acquire(B.done + m) < need) {
          if (*(volatile int *)B.status) { t = total; break; }
          if (++it > B.spin_limit) {
            atomicExch(B.status, 1);
            M.d.ctl[CT_ERROR] = 2;
            t = total;
            break;
          }
          __nanosleep(128);
        }
        if (t < total) {
          work = M.d.ctl[CT_CONVERGED] ? 0 : 1;
          // the TMA reads of this item (async proxy) follow the other CTAs' stores, and
          // its tensor maps (global memory, rewritten between launches) are current
          asm volatile("fence.proxy.async.global;" ::: "memory");
          const int l = lvl + 2;
          const CUtensorMap *mp = (l & 1) ? &M.mA : &M.mB;
          asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(mp) : "memory");
          asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(&M.mR) : "memory");
          if (work) {
            const LesDom &d = M.d;
            const bool last = (l == B.nmaxp);
            SorArgs a;
            a.psrc = (l & 1) ? d.sorA : d.sorB;  // iteration l-1 wrote sorB if l-1 is odd
            a.pdst = last ? d.p : ((l & 1) ? d.sorB : d.sorA);
            a.dstcode = last ? 2 : ((l & 1) ? 1 : 0);
            a.ghost = last ? 0 : 1;
            a.rhs = d.sorR;
            a.tj = NY - 4;
            a.kchunk = d.km;
            a.nchunk = 1;
            a.ntiles = M.ntiles;
            a.part = d.part;
            a.counter = d.cnt;
            s_a = a;
          }
        }
      }
      s_item = t;
      s_work = work;
      s_m = m;
    }
    __syncthreads();
    const unsigned t = s_item;
    if (t >= total) break;
    if (s_work) {
      {  // the member's domain view into shared memory, word by word
        const unsigned *src = reinterpret_cast<const unsigned *>(&B.doms[s_m].d);
        unsigned *dst = reinterpret_cast<unsigned *>(&s_d);
        for (int w = tid; w < (int)(sizeof(LesDom) / 4); w += NX * NY) dst[w] = src[w];
      }
      __syncthreads();
      auto item_tile = [&]() {
        const int r = (int)(s_item % (unsigned)B.per_level);
        return r - B.doms[s_m].first;
      };
      auto maps = [&](int which) -> const CUtensorMap * {
        const SorBatchDom &M = B.doms[s_m];
        if (which) return &M.mR;
        const int l = (int)(s_item / (unsigned)B.per_level) + 2;
        return (l & 1) ? &M.mA : &M.mB;
      };
      const int tile = item_tile(), tx = B.doms[s_m].tiles_x;
      sor_tma_tile<NX, NY, D, false>(s_d, s_a, maps, tile % tx, tile / tx, 0, item_tile, S);
    }
    __syncthreads();
    if (tid == 0) {
      if (s_work)
        for (int q = 0; q < D; ++q) mbar_inval(&S.bar[q]);  // quiescent: re-initialised by the next item
      __threadfence();
      atomicAdd(B.done + s_m, 1u);
    }
  }
}

template <int NX, int NY, int D>
int launch(const SorBatchArgs &B, int sms, cudaStream_t s) {
  const size_t bytes = sizeof(TmaSmem<NX, NY, D>);
  if (cudaFuncSetAttribute(k_sor_batch<NX, NY, D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
      cudaSuccess)
    return -1;
  const long long total = (long long)B.per_level * B.levels;
  const long long ctas = std::min<long long>(total, (long long)min_ctas(NX) * sms);
  if (ctas <= 0) return 0;
  k_sor_batch<NX, NY, D><<<(unsigned)ctas, dim3(NX, NY), bytes, s>>>(B);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

}  // namespace

bool les_sor_batch_ok(const LesDom &d, SorShape sh, const LesSorMaps *maps) {
  return sh.ny >= 16 && sh.ny <= 28 && (sh.nx == 16 || sh.nx == 32) && maps && maps->valid &&
         maps->shape.nx == sh.nx && maps->shape.ny == sh.ny && d.gr.cn1k && !d.cn1 && d.omega == 1.f &&
         d.jm % 2 == 0 && d.km + 1 < LES_SOR_KMAX;
}

bool les_sor_batch_build(const std::vector<const LesDom *> &doms, const std::vector<const LesSorMaps *> &maps,
                         SorShape sh, int nmaxp, const SorBatchBuffers &buf, std::vector<SorBatchDom> *host,
                         std::vector<int> *owner) {
  const int n = (int)doms.size();
  host->assign(n, SorBatchDom{});  // value-initialised: padding zero, so tables compare bytewise
  owner->clear();
  int first = 0;
  for (int m = 0; m < n; ++m) {
    SorBatchDom &M = (*host)[m];
    M.mA = maps[m]->m[0];
    M.mB = maps[m]->m[1];
    M.mR = maps[m]->m[2];
    M.d = *doms[m];
    const SorShape one{sh.nx, sh.ny, doms[m]->km, 1};
    M.tiles_x = (doms[m]->im + (4 * sh.nx - 8) - 1) / (4 * sh.nx - 8);
    M.ntiles = les_sor_fused_tiles(doms[m]->im, doms[m]->jm, one);
    M.first = first;
    for (int t = 0; t < M.ntiles; ++t) owner->push_back(m);
    first += M.ntiles;
  }
  return !(buf.nmaxp == nmaxp && buf.shape.nx == sh.nx && buf.shape.ny == sh.ny && buf.owner_host == *owner &&
           buf.host.size() == host->size() &&
           (host->empty() || memcmp(buf.host.data(), host->data(), sizeof(SorBatchDom) * host->size()) == 0));
}

int les_sor_batch_upload(std::vector<SorBatchDom> host, std::vector<int> owner, SorShape sh, int nmaxp,
                         SorBatchBuffers *buf) {
  const int n = (int)host.size();
  // (re)allocate on growth
  if (buf->cap_dom < n || buf->cap_owner < (int)owner.size()) {
    cudaFree(buf->doms);
    cudaFree(buf->owner);
    cudaFree(buf->counters);
    buf->doms = nullptr;
    buf->owner = nullptr;
    buf->counters = nullptr;
    buf->cap_dom = std::max(n, 2 * buf->cap_dom);
    buf->cap_owner = std::max((int)owner.size(), 2 * buf->cap_owner);
    if (cudaMalloc(&buf->doms, sizeof(SorBatchDom) * buf->cap_dom) != cudaSuccess ||
        cudaMalloc(&buf->owner, sizeof(int) * buf->cap_owner) != cudaSuccess ||
        cudaMalloc(&buf->counters, sizeof(unsigned) * (2 + buf->cap_dom)) != cudaSuccess) {
      (void)cudaGetLastError();
      buf->cap_dom = buf->cap_owner = 0;
      return -1;
    }
  }
  if ((n && cudaMemcpy(buf->doms, host.data(), sizeof(SorBatchDom) * n, cudaMemcpyHostToDevice) != cudaSuccess) ||
      (!owner.empty() &&
       cudaMemcpy(buf->owner, owner.data(), sizeof(int) * owner.size(), cudaMemcpyHostToDevice) != cudaSuccess)) {
    (void)cudaGetLastError();
    return -2;
  }
  buf->ndom = n;
  buf->per_level = (int)owner.size();
  buf->nmaxp = nmaxp;
  buf->shape = sh;
  buf->host = std::move(host);
  buf->owner_host = std::move(owner);
  return 0;
}

int les_sor_batch_launch(const SorBatchBuffers &buf, int sms, long long spin_limit, int hold_member, cudaStream_t s) {
  if (buf.ndom <= 0 || buf.nmaxp < 2) return 0;
  // counters: [0] queue, [1] status, [2..] tiles done per member
  if (cudaMemsetAsync(buf.counters, 0, sizeof(unsigned) * (2 + buf.ndom), s) != cudaSuccess) return -3;
  SorBatchArgs B;
  B.doms = buf.doms;
  B.owner = buf.owner;
  B.ndom = buf.ndom;
  B.per_level = buf.per_level;
  B.levels = buf.nmaxp - 1;
  B.nmaxp = buf.nmaxp;
  B.queue = buf.counters;
  B.status = reinterpret_cast<int *>(buf.counters + 1);
  B.done = buf.counters + 2;
  B.spin_limit = spin_limit;
  B.hold_member = hold_member;
  const SorShape sh = buf.shape;
  if (sh.nx == 16) {
    switch (sh.ny) {
      case 16: return launch<16, 16, 6>(B, sms, s);
      case 20: return launch<16, 20, 6>(B, sms, s);
      case 28: return launch<16, 28, 4>(B, sms, s);
      default: return launch<16, 24, 6>(B, sms, s);
    }
  }
  switch (sh.ny) {
    case 16: return launch<32, 16, 6>(B, sms, s);
    case 20: return launch<32, 20, 6>(B, sms, s);
    case 28: return launch<32, 28, 4>(B, sms, s);
    default: return launch<32, 24, 6>(B, sms, s);
  }
}

void les_sor_batch_free(SorBatchBuffers *buf) {
  cudaFree(buf->doms);
  cudaFree(buf->owner);
  cudaFree(buf->counters);
  *buf = SorBatchBuffers();
}

int les_sor_batch_status(const SorBatchBuffers &buf, cudaStream_t s, int *status) {
  *status = 0;
  if (!buf.counters) return 0;
  if (cudaMemcpyAsync(status, buf.counters + 1, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return -1;
  return cudaStreamSynchronize(s) == cudaSuccess ? 0 : -2;
}
