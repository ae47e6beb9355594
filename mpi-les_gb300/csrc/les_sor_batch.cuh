// les_sor_batch.cuh -- press's SOR iterations 2..nmaxp of many domains in one persistent
// kernel over a tile work-list (les_sor_batch.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <vector>

#include "les_common.cuh"
#include "les_sor.cuh"

// One member of a batched SOR launch, in device memory: its tensor maps (sorA, sorB,
// rhs; CUtensorMap is 64-byte aligned), its domain view, and its tiles in the work list.
struct SorBatchDom {
  CUtensorMap mA, mB, mR;
  LesDom d;
  int tiles_x, ntiles;  // the member's tile grid for the launch's shape
  int first;            // index of its first tile among the items of one level
};

struct SorBatchArgs {
  const SorBatchDom *doms;
  const int *owner;     // item of a level -> member
  int ndom, per_level, levels, nmaxp;
  unsigned *queue;      // next item to take (zero on entry)
  int *status;          // 1 once a dependency wait gave up (zero on entry)
  unsigned *done;       // tiles completed per member (zero on entry)
  long long spin_limit; // polls before a dependency wait gives up
  int hold_member;      // test hook: this member's first level waits on a count never reached (-1: none)
};

// Device buffers of one batched launch group (one tile shape), with the host copies of
// what was uploaded last.
struct SorBatchBuffers {
  SorBatchDom *doms = nullptr;
  int *owner = nullptr;
  unsigned *counters = nullptr;  // [0] queue, [1] status, [2 + m] tiles done of member m
  int cap_dom = 0, cap_owner = 0;
  int ndom = 0, per_level = 0, nmaxp = 0;
  SorShape shape;
  std::vector<SorBatchDom> host;
  std::vector<int> owner_host;
};

// A member can take part in a batched SOR launch of shape sh: the one-iteration TMA
// sweep applies (uniform cn1, omega = 1, even jm) and its maps are for sh.
bool les_sor_batch_ok(const LesDom &d, SorShape sh, const LesSorMaps *maps);
// The member table and work list of a group, built on the host.  Returns true if they
// differ from what buf holds (members, their domains' device views or tensor maps, the
// shape or the iteration count): a handle freed and another created at the same address
// is a different member.
bool les_sor_batch_build(const std::vector<const LesDom *> &doms, const std::vector<const LesSorMaps *> &maps,
                         SorShape sh, int nmaxp, const SorBatchBuffers &buf, std::vector<SorBatchDom> *host,
                         std::vector<int> *owner);
// Upload a built table and work list (synchronous: call it with no launch of this group
// in flight).  0 on success.
int les_sor_batch_upload(std::vector<SorBatchDom> host, std::vector<int> owner, SorShape sh, int nmaxp,
                         SorBatchBuffers *buf);
// Queue iterations 2..nmaxp of every member on stream s (the members' rhs, iteration 1
// and sor_begin must precede it on s).  spin_limit bounds each dependency wait.
int les_sor_batch_launch(const SorBatchBuffers &buf, int sms, long long spin_limit, int hold_member, cudaStream_t s);
void les_sor_batch_free(SorBatchBuffers *buf);
// *status = 1 if a dependency wait of the last launch gave up (synchronises s).
int les_sor_batch_status(const SorBatchBuffers &buf, cudaStream_t s, int *status);
