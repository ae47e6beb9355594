// les_noalloc.cu -- the volume-weighted field mean with no allocation at all.
//
// Who needs it: a caller that may not allocate device memory when it asks -- code
// running under a memory cap that was sized up front, a host framework whose own
// allocator owns the device, or a monitor called between steps that must not add
// a cudaMalloc/cudaFree to the step's timeline.  The handle's own reductions use
// its workspace; this one keeps every scratch word in a fixed static device array,
// so a call issues only memsets, copies and kernel launches on the handle's stream.
//
// The reduction is press's pav reduction (press.f95:124-133): per-block partial
// sums of x*dx1*dy1*dzn, a fixed-order two-level FP64 finish, divided by the FP64
// domain volume, rounded to FP32 as press rounds pav.
//
// Limits and sharing.  The scratch holds LES_NOALLOC_MAX_PARTS block partials, one
// per 64 x 4 x 16 cells: a domain with more reduction blocks ((im+63)/64 * (jm+3)/4 *
// ((km+15)/16), les_reduce_blocks) is refused with LES_ERR_ARG.  All calls in the process share the one array per device and it keeps
// what the last call left there; each call clears the words that must start at zero
// (the completion ticket).  Two calls whose kernels overlap in time (different
// streams or threads without ordering) race on the array and give wrong results.
// The array's device address is looked up the first time a handle on a device calls
// in (cudaGetSymbolAddress, with that device made current for the lookup); make that
// first call outside any stream capture.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>

#include "../../include/les_gpu.h"
#include "les_common.cuh"
#include "les_kernels.cuh"

namespace {

// Scratch layout, in doubles: block partials, second-level partials, scalar slots,
// float slots (8 floats), completion tickets (16 unsigned ints).
constexpr int kParts = LES_NOALLOC_MAX_PARTS;
constexpr int kPart2 = kParts;
constexpr int kScal = kPart2 + LES_FIN_BLOCKS;
constexpr int kFscal = kScal + SC_COUNT;
constexpr int kTicket = kFscal + 4;
constexpr int kTotal = kTicket + 8;

static __device__ __align__(256) double g_scratch[kTotal];

std::mutex g_mu;
std::map<int, double *> g_addr;  // device -> address of g_scratch on it

// Address of the scratch array on `dev`, looked up once per device.
int scratch_on(int dev, double **out, std::string *err) {
  std::lock_guard<std::mutex> lock(g_mu);
  auto it = g_addr.find(dev);
  if (it != g_addr.end()) {
    *out = it->second;
    return LES_OK;
  }
  int cur = -1;
  cudaError_t e = cudaGetDevice(&cur);
  if (e == cudaSuccess && cur != dev) e = cudaSetDevice(dev);
  double *p = nullptr;
  if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&p, g_scratch);
  if (cur >= 0 && cur != dev) (void)cudaSetDevice(cur);
  if (e != cudaSuccess || !p) {
    *err = std::string("field_mean_noalloc: scratch address lookup failed: ") + cudaGetErrorString(e);
    (void)cudaGetLastError();
    return LES_ERR_CUDA;
  }
  g_addr[dev] = p;
  *out = p;
  return LES_OK;
}

}  // namespace

int les_noalloc_interior_mean(const LesDom &dom, const float *x, const double *area_dev, cudaStream_t s,
                              long long *nlaunch, int dev, double *mean, std::string *err) {
  if (les_reduce_blocks(dom) > kParts) {
    *err = "field_mean_noalloc: the domain has " + std::to_string(les_reduce_blocks(dom)) +
           " reduction blocks; the static scratch holds " + std::to_string(kParts);
    return LES_ERR_ARG;
  }
  double *sc = nullptr;
  int rc = scratch_on(dev, &sc, err);
  if (rc) return rc;
  LesDom d = dom;
  d.p = const_cast<float *>(x);  // read only: the partial kernel loads d.p
  d.part = sc;
  d.part2 = sc + kPart2;
  d.scal = sc + kScal;
  d.fscal = reinterpret_cast<float *>(sc + kFscal);
  d.cnt = reinterpret_cast<unsigned int *>(sc + kTicket);
  cudaError_t e = cudaMemsetAsync(sc + kTicket, 0, 8 * sizeof(double), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(sc + kScal + SC_AREA, area_dev, sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) {
    les_launch_interior_mean(d, LesCtx{s, nlaunch});
    e = cudaGetLastError();
  }
  double out = 0.0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&out, sc + kScal + SC_PAV, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    *err = std::string("field_mean_noalloc: ") + cudaGetErrorString(e);
    (void)cudaGetLastError();
    return LES_ERR_CUDA;
  }
  *mean = out;
  return LES_OK;
}
