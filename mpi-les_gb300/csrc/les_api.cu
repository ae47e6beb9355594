// les_api.cu -- the C-ABI of include/les_gpu.h: one resident domain per handle.
//
// Replaces the reference's buffer set-up and per-step driver of the OpenCL path
// (initialise_LES_kernel / run_LES_kernel, src/module_LES_combined_ocl.f95:14,350)
// and, entry point by entry point, the eight Fortran solver subroutines.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/les_gpu.h"
#include "les_aveflow.cuh"
#include "les_common.cuh"
#include "les_kernels.cuh"
#include "les_sor_batch.cuh"
#include "les_step.cuh"
#include "les_tune.cuh"

namespace {

constexpr int kNumFields = 15;  // LES_FIELD_U .. LES_FIELD_SM

struct Ext {
  int lb[3], ub[3];
};

// Declared extents of each field in the reference (src/main.f95:63-159).
bool declared_extents(int id, int im, int jm, int km, Ext *e) {
  auto set = [&](int a0, int b0, int a1, int b1, int a2, int b2) {
    e->lb[0] = a0; e->ub[0] = b0; e->lb[1] = a1; e->ub[1] = b1; e->lb[2] = a2; e->ub[2] = b2;
  };
  switch (id) {
    case LES_FIELD_U: case LES_FIELD_V: set(0, im + 1, -1, jm + 1, 0, km + 1); return true;
    case LES_FIELD_W: set(0, im + 1, -1, jm + 1, -1, km + 1); return true;
    case LES_FIELD_P: set(0, im + 2, 0, jm + 2, 0, km + 1); return true;
    case LES_FIELD_F: case LES_FIELD_G: case LES_FIELD_H:
    case LES_FIELD_USUM: case LES_FIELD_VSUM: case LES_FIELD_WSUM: set(0, im, 0, jm, 0, km); return true;
    case LES_FIELD_FOLD: case LES_FIELD_GOLD: case LES_FIELD_HOLD: set(1, im, 1, jm, 1, km); return true;
    case LES_FIELD_RHS: set(0, im + 1, 0, jm + 1, 0, km + 1); return true;
    case LES_FIELD_SM: set(-1, im + 1, -1, jm + 1, 0, km + 1); return true;
    case LES_FIELD_BMASK1: set(-1, im + 1, 0, jm + 1, 0, km + 1); return true;
    case LES_FIELD_CMASK1: set(0, im + 1, -1, jm + 1, 0, km + 1); return true;
    case LES_FIELD_DMASK1: set(0, im + 1, 0, jm + 1, 0, km + 1); return true;
    case LES_FIELD_CN1: set(1, im, 1, jm, 1, km); return true;
    case LES_FIELD_DX1: set(-1, im + 1, 0, 0, 0, 0); return true;
    case LES_FIELD_DY1: set(0, jm + 1, 0, 0, 0, 0); return true;
    case LES_FIELD_DZN: case LES_FIELD_DZS: set(-1, km + 2, 0, 0, 0, 0); return true;
    case LES_FIELD_DXS: set(0, im, 0, 0, 0, 0); return true;
    case LES_FIELD_DYS: set(0, jm, 0, 0, 0, 0); return true;
    case LES_FIELD_Z2: set(0, km + 2, 0, 0, 0, 0); return true;
    case LES_FIELD_CN2L: case LES_FIELD_CN2S: set(1, im, 0, 0, 0, 0); return true;
    case LES_FIELD_CN3L: case LES_FIELD_CN3S: set(1, jm, 0, 0, 0, 0); return true;
    case LES_FIELD_CN4L: case LES_FIELD_CN4S: case LES_FIELD_DELX1: set(1, km, 0, 0, 0, 0); return true;
    case LES_FIELD_UIN: case LES_FIELD_VIN: case LES_FIELD_WIN: set(1, jm, 1, km, 0, 0); return true;
    case LES_FIELD_AVEU: case LES_FIELD_AVEV: set(1, im, 1, jm, 0, km); return true;
    case LES_FIELD_AVEW: set(1, im + 1, 1, jm, 0, km + 2); return true;
    case LES_FIELD_AVEP: case LES_FIELD_AVEL: case LES_FIELD_AVEUU: case LES_FIELD_AVEVV: case LES_FIELD_AVEWW:
    case LES_FIELD_AVESM: case LES_FIELD_AVESMSM: case LES_FIELD_UWFX: set(1, im, 1, jm, 1, km); return true;
    default: return false;
  }
}

bool is_1d(int id) { return id >= LES_FIELD_DX1 && id <= LES_FIELD_DELX1; }
bool is_inflow(int id) { return id >= LES_FIELD_UIN && id <= LES_FIELD_WIN; }
bool is_ave(int id) { return id >= LES_FIELD_AVEU && id <= LES_FIELD_UWFX; }
constexpr int kNumAve = LES_FIELD_UWFX - LES_FIELD_AVEU + 1;

}  // namespace

struct les_handle {
  les_dims dims{};
  les_params prm{};
  int pi = 0, nj = 0, np = 0;
  size_t nfloat = 0;  // floats per padded 3-D field
  int dev = 0;
  cudaStream_t s = nullptr;
  float *fields[kNumFields] = {};
  uint8_t *mask_d = nullptr;
  std::vector<uint8_t> mask_h;
  bool mask_dirty = true;
  bool mask_on_device = false;  // les_gpu_feedbfm wrote mask_d; mask_h is stale
  std::map<int, std::vector<float>> h1d;  // 1-D arrays and inflow planes (host copies)
  float *g1_d = nullptr;                  // 1-D arrays on the device
  float *inflow_d = nullptr;
  std::vector<float> cn1_h;
  bool cn1_given = false;
  float *cn1_d = nullptr;
  double *scal_d = nullptr;
  int *ctl_d = nullptr;
  double *part_d = nullptr;
  float *fscal_d = nullptr;
  unsigned long long *bad_d = nullptr;
  float *sor_d[3] = {};           // internal buffers of the fused SOR sweep (A, B, rhs)
  float *prow_d = nullptr;        // p's row jm+2 while the fused sweep reads it (LesDom.prow)
  float *diu_d[10] = {};          // diu1..9 stored by velfg for les ([0] unused)
  float *rsp_d = nullptr;         // two planes: u/uspd and v/vspd at k = 1
  unsigned int *cnt_d = nullptr;  // CTA tickets (fused SOR sweep, finish_mean, uout)
  int *fix_d = nullptr;           // deferred-block lists (FIX_COUNT lists of fix_len ints)
  size_t fix_len = 0;
  int sms = 0;
  // p's i/j halos may disagree with its interior (set by an upload of p, cleared by
  // press): the next step then runs the per-subroutine kernels, exact for any state
  bool p_dirty = false;
  size_t npart = 0;
  bool committed = false;
  LesDom dom{};
  long long nlaunch = 0;
  std::string err;
  LesStepPlan plan{};
  // downloads: a box is packed on h->s into a staging slot, then copied to the host on
  // the copy stream cs (les_gpu_download_async); slots are reused in ticket order
  struct DlSlot {
    float *buf = nullptr;
    size_t cap = 0;  // floats
    cudaEvent_t packed = nullptr, done = nullptr;
    long long ticket = -1;
  };
  static constexpr int kDlSlots = 8;
  float *ave_d[kNumAve] = {};  // aveflow's averaging arrays (les_gpu_aveflow allocates them)
  DlSlot dl[kDlSlots];
  cudaStream_t cs = nullptr;
  long long next_ticket = 0;
};

namespace {

int fail(les_handle *h, int code, const std::string &msg) {
  if (h) h->err = msg;
  return code;
}

int cuda_fail(les_handle *h, cudaError_t e, const char *what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  (void)cudaGetLastError();
  return fail(h, e == cudaErrorMemoryAllocation ? LES_ERR_NOMEM : LES_ERR_CUDA, m);
}

#define CK(h, call)                                   \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
  } while (0)

int check_launch(les_handle *h, const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, what);
  return LES_OK;
}

LesCtx ctx_of(les_handle *h) { return LesCtx{h->s, &h->nlaunch}; }

int pitch_for(int im) { return ((im + 6) + 15) / 16 * 16; }

}  // namespace

extern "C" size_t les_domain_bytes(int im, int jm, int km) {
  const size_t pi = (size_t)pitch_for(im), nj = (size_t)jm + 8, nk = (size_t)km + 4;
  const size_t field = pi * nj * nk * sizeof(float);
  const size_t part = ((size_t)(im + 63) / 64 + 1) * ((size_t)(jm + 3) / 4 + 1) * (size_t)km * 2 * sizeof(double);
  // deferred-block lists (les_gpu_create): FIX_COUNT lists over the largest grid of those kernels
  const size_t fused = (size_t)((im + 30) / 31) * ((jm + 7) / 8) * km;  // velfg k-march: tile planes
  const size_t inter = (size_t)((im + 63) / 64) * ((jm + 3) / 4) * km;
  const size_t march = (size_t)((im + 31) / 32) * ((jm + 7) / 8) * km;
  const size_t fix = FIX_COUNT * (2 + std::max({fused, inter, march})) * sizeof(int);
  return (kNumFields + 3 + 9) * field + pi * nj * nk /*mask bytes*/ + 2 * pi * nj * sizeof(float) + part + fix +
         (size_t)im * km * sizeof(float) /*p's row jm+2*/ + 64 * 1024;
}

extern "C" int les_gpu_create(const les_dims *dims, const les_params *params, les_handle **out) {
  if (!dims || !params || !out) return LES_ERR_ARG;
  *out = nullptr;
  const int im = dims->im, jm = dims->jm, km = dims->km;
  if (im < 3 || jm < 2 || km < 3) return LES_ERR_ARG;
  if (params->nmaxp < 0 || params->nmaxp > 100000) return LES_ERR_ARG;
  les_handle *h = new les_handle();
  h->dims = *dims;
  h->prm = *params;
  h->pi = pitch_for(im);
  h->nj = jm + 8;
  h->np = h->pi * h->nj;
  h->nfloat = (size_t)h->np * (size_t)(km + 4);
  if (h->nfloat >= (size_t)1 << 31) {
    delete h;
    return LES_ERR_ARG;  // 32-bit indexing inside the kernels
  }
  auto cleanup = [&](int code) {
    les_gpu_destroy(h);
    return code;
  };
  cudaError_t e = cudaGetDevice(&h->dev);
  if (e != cudaSuccess) { (void)cudaGetLastError(); return cleanup(LES_ERR_CUDA); }
  if ((e = cudaStreamCreateWithFlags(&h->s, cudaStreamNonBlocking)) != cudaSuccess) { (void)cudaGetLastError(); return cleanup(LES_ERR_CUDA); }
  for (int f = 0; f < kNumFields; ++f) {
    if ((e = cudaMalloc(&h->fields[f], h->nfloat * sizeof(float))) != cudaSuccess) {
      (void)cudaGetLastError();
      return cleanup(LES_ERR_NOMEM);
    }
    if ((e = cudaMemsetAsync(h->fields[f], 0, h->nfloat * sizeof(float), h->s)) != cudaSuccess) {
      (void)cudaGetLastError();
      return cleanup(LES_ERR_CUDA);
    }
  }
  if (cudaMalloc(&h->mask_d, h->nfloat) != cudaSuccess) { (void)cudaGetLastError(); return cleanup(LES_ERR_NOMEM); }
  for (int q = 0; q < 3; ++q) {
    if (cudaMalloc(&h->sor_d[q], h->nfloat * sizeof(float)) != cudaSuccess) {
      (void)cudaGetLastError();
      return cleanup(LES_ERR_NOMEM);
    }
    cudaMemsetAsync(h->sor_d[q], 0, h->nfloat * sizeof(float), h->s);
  }
  if (cudaMalloc(&h->prow_d, (size_t)im * km * sizeof(float)) != cudaSuccess) {
    (void)cudaGetLastError();
    return cleanup(LES_ERR_NOMEM);
  }
  for (int q = 1; q <= 9; ++q) {
    if (cudaMalloc(&h->diu_d[q], h->nfloat * sizeof(float)) != cudaSuccess) {
      (void)cudaGetLastError();
      return cleanup(LES_ERR_NOMEM);
    }
    cudaMemsetAsync(h->diu_d[q], 0, h->nfloat * sizeof(float), h->s);
  }
  if (cudaMalloc(&h->rsp_d, 2 * (size_t)h->np * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&h->cnt_d, 64) != cudaSuccess) {
    (void)cudaGetLastError();
    return cleanup(LES_ERR_NOMEM);
  }
  cudaMemsetAsync(h->rsp_d, 0, 2 * (size_t)h->np * sizeof(float), h->s);
  cudaMemsetAsync(h->cnt_d, 0, 64, h->s);
  cudaMemsetAsync(h->mask_d, 0, h->nfloat, h->s);
  if (cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->dev) != cudaSuccess) {
    (void)cudaGetLastError();
    h->sms = 0;
  }
  h->mask_h.assign(h->nfloat, 0);
  // partial-sum buffer: the largest per-block count of any reduction kernel
  h->npart = (size_t)std::max<long long>(
      {(long long)((im + 63) / 64) * ((jm + 3) / 4) * km * 2 + 64, (long long)les_step_parts_needed(im, jm, km, h->sms)});
  h->plan.part_cap = (long long)h->npart;
  // deferred-block lists: [count, ticket, ids...] for the largest grid of those kernels
  {
    const long long fused = (long long)((im + 30) / 31) * ((jm + 7) / 8) * km;  // velfg k-march: tile planes
    const long long inter = (long long)((im + 63) / 64) * ((jm + 3) / 4) * km;
    const long long march = (long long)((im + 31) / 32) * ((jm + 7) / 8) * km;  // les k-march: tile planes
    h->fix_len = 2 + (size_t)std::max({fused, inter, march});
  }
  if (cudaMalloc(&h->fix_d, FIX_COUNT * h->fix_len * sizeof(int)) != cudaSuccess) {
    (void)cudaGetLastError();
    return cleanup(LES_ERR_NOMEM);
  }
  cudaMemsetAsync(h->fix_d, 0, FIX_COUNT * h->fix_len * sizeof(int), h->s);
  if (cudaMalloc(&h->part_d, (h->npart + 256) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&h->scal_d, SC_COUNT * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&h->ctl_d, CT_COUNT * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&h->fscal_d, SC_COUNT * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&h->bad_d, sizeof(unsigned long long)) != cudaSuccess) {
    (void)cudaGetLastError();
    return cleanup(LES_ERR_NOMEM);
  }
  cudaMemsetAsync(h->scal_d, 0, SC_COUNT * sizeof(double), h->s);
  cudaMemsetAsync(h->ctl_d, 0, CT_COUNT * sizeof(int), h->s);
  cudaMemsetAsync(h->fscal_d, 0, SC_COUNT * sizeof(float), h->s);
  if ((e = cudaStreamSynchronize(h->s)) != cudaSuccess) { (void)cudaGetLastError(); return cleanup(LES_ERR_CUDA); }
  *out = h;
  return LES_OK;
}

extern "C" int les_gpu_destroy(les_handle *h) {
  if (!h) return LES_OK;
  if (h->s) cudaStreamSynchronize(h->s);
  if (h->cs) cudaStreamSynchronize(h->cs);
  for (auto &sl : h->dl) {
    cudaFree(sl.buf);
    if (sl.packed) cudaEventDestroy(sl.packed);
    if (sl.done) cudaEventDestroy(sl.done);
  }
  if (h->cs) cudaStreamDestroy(h->cs);
  for (float *a : h->ave_d) cudaFree(a);
  les_step_plan_free(&h->plan);
  for (int f = 0; f < kNumFields; ++f) cudaFree(h->fields[f]);
  cudaFree(h->mask_d);
  cudaFree(h->g1_d);
  cudaFree(h->inflow_d);
  cudaFree(h->cn1_d);
  cudaFree(h->scal_d);
  cudaFree(h->ctl_d);
  cudaFree(h->part_d);
  cudaFree(h->fscal_d);
  cudaFree(h->bad_d);
  for (int q = 0; q < 3; ++q) cudaFree(h->sor_d[q]);
  cudaFree(h->prow_d);
  for (int q = 1; q <= 9; ++q) cudaFree(h->diu_d[q]);
  cudaFree(h->rsp_d);
  cudaFree(h->cnt_d);
  cudaFree(h->fix_d);
  if (h->s) cudaStreamDestroy(h->s);
  (void)cudaGetLastError();
  delete h;
  return LES_OK;
}

namespace {

int check_ext(les_handle *h, int field, const int lb[3], const int ub[3], Ext *decl) {
  if (!declared_extents(field, h->dims.im, h->dims.jm, h->dims.km, decl))
    return fail(h, LES_ERR_ARG, "unknown field id " + std::to_string(field));
  for (int a = 0; a < 3; ++a) {
    if (lb[a] < decl->lb[a] || ub[a] > decl->ub[a] || ub[a] < lb[a]) {
      char b[200];
      snprintf(b, sizeof b, "extents (%d:%d,%d:%d,%d:%d) exceed the declared (%d:%d,%d:%d,%d:%d) of field %d",
               lb[0], ub[0], lb[1], ub[1], lb[2], ub[2], decl->lb[0], decl->ub[0], decl->lb[1], decl->ub[1],
               decl->lb[2], decl->ub[2], field);
      return fail(h, LES_ERR_ARG, b);
    }
  }
  return LES_OK;
}

cudaMemcpy3DParms copy_parms(les_handle *h, float *dev, float *host, const int lb[3], const int ub[3], bool h2d) {
  const size_t nx = (size_t)(ub[0] - lb[0] + 1), ny = (size_t)(ub[1] - lb[1] + 1), nz = (size_t)(ub[2] - lb[2] + 1);
  cudaMemcpy3DParms p;
  memset(&p, 0, sizeof p);
  cudaPitchedPtr hp = make_cudaPitchedPtr(host, nx * sizeof(float), nx * sizeof(float), ny);
  cudaPitchedPtr dp = make_cudaPitchedPtr(dev, (size_t)h->pi * sizeof(float), (size_t)h->pi * sizeof(float), (size_t)h->nj);
  cudaPos dpos = make_cudaPos((size_t)(lb[0] + LES_IOFF) * sizeof(float), (size_t)(lb[1] + LES_JOFF), (size_t)(lb[2] + LES_KOFF));
  if (h2d) { p.srcPtr = hp; p.dstPtr = dp; p.dstPos = dpos; p.kind = cudaMemcpyHostToDevice; }
  else { p.srcPtr = dp; p.srcPos = dpos; p.dstPtr = hp; p.kind = cudaMemcpyDeviceToHost; }
  p.extent = make_cudaExtent(nx * sizeof(float), ny, nz);
  return p;
}

}  // namespace

extern "C" int les_gpu_upload(les_handle *h, int field, const float *host, const int lb[3], const int ub[3]) {
  if (!h || !host || !lb || !ub) return LES_ERR_ARG;
  Ext decl;
  int rc = check_ext(h, field, lb, ub, &decl);
  if (rc) return rc;
  const int im = h->dims.im, jm = h->dims.jm, km = h->dims.km;
  const size_t nx = ub[0] - lb[0] + 1, ny = ub[1] - lb[1] + 1;
  if (field >= LES_FIELD_U && field <= LES_FIELD_SM) {
    cudaMemcpy3DParms p = copy_parms(h, h->fields[field - 1], const_cast<float *>(host), lb, ub, true);
    CK(h, cudaMemcpy3DAsync(&p, h->s));
    if (field == LES_FIELD_P) h->p_dirty = true;
    return LES_OK;
  }
  if (field >= LES_FIELD_BMASK1 && field <= LES_FIELD_DMASK1) {
    const uint8_t bit = (uint8_t)(1u << (field - LES_FIELD_BMASK1));
    if (h->mask_on_device) {  // the device holds the masks les_gpu_feedbfm made: start from them
      CK(h, cudaMemcpyAsync(h->mask_h.data(), h->mask_d, h->nfloat, cudaMemcpyDeviceToHost, h->s));
      CK(h, cudaStreamSynchronize(h->s));
      h->mask_on_device = false;
    }
    for (int k = lb[2]; k <= ub[2]; ++k)
      for (int j = lb[1]; j <= ub[1]; ++j)
        for (int i = lb[0]; i <= ub[0]; ++i) {
          if (i < 1 || i > im || j < 1 || j > jm || k < 1 || k > km) continue;  // halos unused
          const float x = host[(i - lb[0]) + nx * ((j - lb[1]) + ny * (size_t)(k - lb[2]))];
          if (x != 0.f && x != 1.f) return fail(h, LES_ERR_ARG, "mask values must be 0 or 1");
          uint8_t &m = h->mask_h[(size_t)(k + LES_KOFF) * h->np + (size_t)(j + LES_JOFF) * h->pi + (i + LES_IOFF)];
          m = (uint8_t)(x != 0.f ? (m | bit) : (m & ~bit));
        }
    h->mask_dirty = true;
    return LES_OK;
  }
  if (field == LES_FIELD_CN1) {
    h->cn1_h.assign((size_t)im * jm * km, 0.f);
    if (lb[0] != 1 || ub[0] != im || lb[1] != 1 || ub[1] != jm || lb[2] != 1 || ub[2] != km)
      return fail(h, LES_ERR_ARG, "cn1 must be uploaded whole (1:im,1:jm,1:km)");
    std::copy(host, host + (size_t)im * jm * km, h->cn1_h.begin());
    h->cn1_given = true;
    h->committed = false;
    return LES_OK;
  }
  if (field == LES_FIELD_DELX1) return fail(h, LES_ERR_ARG, "delx1 is an output of les (les.f95:38-42)");
  // 1-D arrays and inflow planes: keep a host copy at the declared extents
  std::vector<float> &v = h->h1d[field];
  const size_t dn0 = decl.ub[0] - decl.lb[0] + 1, dn1 = decl.ub[1] - decl.lb[1] + 1;
  if (v.size() != dn0 * dn1) v.assign(dn0 * dn1, 0.f);
  for (int j = lb[1]; j <= ub[1]; ++j)
    for (int i = lb[0]; i <= ub[0]; ++i)
      v[(i - decl.lb[0]) + dn0 * (size_t)(j - decl.lb[1])] = host[(i - lb[0]) + nx * (size_t)(j - lb[1])];
  if (is_inflow(field) && h->committed && h->inflow_d) {
    // inflow planes may change between steps (a time-varying inflow): refresh now
    const size_t n = (size_t)jm * km;
    CK(h, cudaMemcpyAsync(h->inflow_d + (size_t)(field - LES_FIELD_UIN) * n, v.data(), n * sizeof(float),
                          cudaMemcpyHostToDevice, h->s));
    return LES_OK;
  }
  h->committed = false;
  return LES_OK;
}

namespace {

// Box (i0.., j0.., k0.., nx x ny) x nz of a padded field into a contiguous array in
// Fortran order: one row of the box (fixed j, k) per block.
__global__ void k_pack_box(const float *__restrict__ src, float *__restrict__ dst, int pi, int nj, int i0, int j0,
                           int k0, int nx, int ny) {
  const int row = blockIdx.x;  // (j - j0) + ny * (k - k0)
  const int jj = row % ny, kk = row / ny;
  const float *s = src + ((size_t)(k0 + kk + LES_KOFF) * nj + (j0 + jj + LES_JOFF)) * pi + (i0 + LES_IOFF);
  float *o = dst + (size_t)row * nx;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) o[i] = s[i];
}

// k_pack_box for boxes whose rows start on 16-byte words at both ends (i0 + 3 a multiple
// of 4, nx a multiple of 4): float4 copies, PACK_ROWS rows per block, one float4 of a
// row per thread.
constexpr int PACK_ROWS = 8;
__global__ void k_pack_box4(const float4 *__restrict__ src, float4 *__restrict__ dst, int pi4, int nj, int i04,
                            int j0, int k0, int nx4, int ny, int rows) {
  const int c = threadIdx.x;
  if (c >= nx4) return;
#pragma unroll
  for (int q = 0; q < PACK_ROWS; ++q) {
    const int row = blockIdx.x * PACK_ROWS + q;  // (j - j0) + ny * (k - k0)
    if (row >= rows) return;
    const int jj = row % ny, kk = row / ny;
    dst[(size_t)row * nx4 + c] = src[((size_t)(k0 + kk + LES_KOFF) * nj + (j0 + jj + LES_JOFF)) * pi4 + i04 + c];
  }
}

// Snapshot the box on h->s and queue its copy to `host` on the copy stream.
int download_async(les_handle *h, int field, float *host, const int lb[3], const int ub[3], long long *ticket) {
  const int nx = ub[0] - lb[0] + 1, ny = ub[1] - lb[1] + 1, nz = ub[2] - lb[2] + 1;
  const size_t n = (size_t)nx * ny * nz;
  if (!h->cs) CK(h, cudaStreamCreateWithFlags(&h->cs, cudaStreamNonBlocking));
  const long long t = h->next_ticket++;
  les_handle::DlSlot &sl = h->dl[t % les_handle::kDlSlots];
  if (!sl.done) {
    CK(h, cudaEventCreateWithFlags(&sl.packed, cudaEventDisableTiming));
    CK(h, cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
  }
  // the slot's previous copy must be in host memory before its staging is rewritten
  if (sl.ticket >= 0) CK(h, cudaEventSynchronize(sl.done));
  if (sl.cap < n) {
    cudaFree(sl.buf);
    sl.buf = nullptr;
    sl.cap = 0;
    CK(h, cudaMalloc(&sl.buf, n * sizeof(float)));
    sl.cap = n;
  }
  const unsigned rows = (unsigned)ny * (unsigned)nz;
  if (rows > 0) {
    const float *src = is_ave(field) ? h->ave_d[field - LES_FIELD_AVEU] : h->fields[field - 1];
    if ((lb[0] + LES_IOFF) % 4 == 0 && nx % 4 == 0 && nx / 4 <= 1024) {
      const int nx4 = nx / 4, threads = (nx4 + 31) / 32 * 32;
      k_pack_box4<<<(rows + PACK_ROWS - 1) / PACK_ROWS, threads, 0, h->s>>>(
          reinterpret_cast<const float4 *>(src), reinterpret_cast<float4 *>(sl.buf), h->pi / 4, h->nj,
          (lb[0] + LES_IOFF) / 4, lb[1], lb[2], nx4, ny, (int)rows);
    } else {
      k_pack_box<<<rows, 128, 0, h->s>>>(src, sl.buf, h->pi, h->nj, lb[0], lb[1], lb[2], nx, ny);
    }
    CK(h, cudaGetLastError());
  }
  CK(h, cudaEventRecord(sl.packed, h->s));
  CK(h, cudaStreamWaitEvent(h->cs, sl.packed, 0));
  CK(h, cudaMemcpyAsync(host, sl.buf, n * sizeof(float), cudaMemcpyDeviceToHost, h->cs));
  CK(h, cudaEventRecord(sl.done, h->cs));
  sl.ticket = t;
  *ticket = t;
  return LES_OK;
}

int download_wait(les_handle *h, long long ticket) {
  if (ticket < 0 || ticket >= h->next_ticket) return fail(h, LES_ERR_ARG, "unknown download ticket");
  const les_handle::DlSlot &sl = h->dl[ticket % les_handle::kDlSlots];
  // a slot reused since then waited for this ticket's copy before it was reused
  if (sl.ticket == ticket) CK(h, cudaEventSynchronize(sl.done));
  return LES_OK;
}

}  // namespace

extern "C" int les_gpu_download_async(les_handle *h, int field, float *host, const int lb[3], const int ub[3],
                                      long long *ticket) {
  if (!h || !host || !lb || !ub || !ticket) return LES_ERR_ARG;
  Ext decl;
  int rc = check_ext(h, field, lb, ub, &decl);
  if (rc) return rc;
  if (is_ave(field)) {
    if (!h->ave_d[0]) return fail(h, LES_ERR_STATE, "download_async: les_gpu_aveflow not called yet");
  } else if (field < LES_FIELD_U || field > LES_FIELD_SM) {
    return fail(h, LES_ERR_ARG, "download_async: 3-D fields only");
  }
  return download_async(h, field, host, lb, ub, ticket);
}

extern "C" int les_gpu_download_wait(les_handle *h, long long ticket) {
  if (!h) return LES_ERR_ARG;
  return download_wait(h, ticket);
}

extern "C" int les_gpu_download(les_handle *h, int field, float *host, const int lb[3], const int ub[3]) {
  if (!h || !host || !lb || !ub) return LES_ERR_ARG;
  Ext decl;
  int rc = check_ext(h, field, lb, ub, &decl);
  if (rc) return rc;
  if ((field >= LES_FIELD_U && field <= LES_FIELD_SM) || is_ave(field)) {
    if (is_ave(field) && !h->ave_d[0]) return fail(h, LES_ERR_STATE, "download: les_gpu_aveflow not called yet");
    long long t = -1;
    rc = download_async(h, field, host, lb, ub, &t);
    if (rc) return rc;
    return download_wait(h, t);
  }
  if (field >= LES_FIELD_BMASK1 && field <= LES_FIELD_DMASK1) {
    // the masks as the kernels see them: the device's bits if les_gpu_feedbfm made them
    // or a commit uploaded them, else the host copy not yet committed
    const uint8_t bit = (uint8_t)(1u << (field - LES_FIELD_BMASK1));
    std::vector<uint8_t> dev;
    const uint8_t *m = h->mask_h.data();
    if (!h->mask_dirty) {
      dev.resize(h->nfloat);
      CK(h, cudaMemcpyAsync(dev.data(), h->mask_d, h->nfloat, cudaMemcpyDeviceToHost, h->s));
      CK(h, cudaStreamSynchronize(h->s));
      m = dev.data();
    }
    const size_t nx = ub[0] - lb[0] + 1, ny = ub[1] - lb[1] + 1;
    for (int k = lb[2]; k <= ub[2]; ++k)
      for (int j = lb[1]; j <= ub[1]; ++j)
        for (int i = lb[0]; i <= ub[0]; ++i) {
          const bool in = i >= -LES_IOFF && i < h->pi - LES_IOFF && j >= -LES_JOFF && j < h->nj - LES_JOFF &&
                          k >= -LES_KOFF && k < h->dims.km + 4 - LES_KOFF;
          const uint8_t v = in ? m[(size_t)(k + LES_KOFF) * h->np + (size_t)(j + LES_JOFF) * h->pi + (i + LES_IOFF)] : 0;
          host[(i - lb[0]) + nx * ((j - lb[1]) + ny * (size_t)(k - lb[2]))] = (v & bit) ? 1.f : 0.f;
        }
    return LES_OK;
  }
  if (field == LES_FIELD_DELX1) {
    if (!h->committed) return fail(h, LES_ERR_STATE, "delx1 is derived at commit");
    auto it = h->h1d.find(LES_FIELD_DELX1);
    for (int i = lb[0]; i <= ub[0]; ++i) host[i - lb[0]] = it->second[i - 1];
    return LES_OK;
  }
  if (is_1d(field) || is_inflow(field)) {
    auto it = h->h1d.find(field);
    if (it == h->h1d.end()) return fail(h, LES_ERR_STATE, "field not uploaded");
    const size_t nx = ub[0] - lb[0] + 1, dn0 = decl.ub[0] - decl.lb[0] + 1;
    for (int j = lb[1]; j <= ub[1]; ++j)
      for (int i = lb[0]; i <= ub[0]; ++i)
        host[(i - lb[0]) + nx * (size_t)(j - lb[1])] = it->second[(i - decl.lb[0]) + dn0 * (size_t)(j - decl.lb[1])];
    return LES_OK;
  }
  return fail(h, LES_ERR_ARG, "field is upload-only");
}

extern "C" int les_gpu_commit_setup(les_handle *h) {
  if (!h) return LES_ERR_ARG;
  const int im = h->dims.im, jm = h->dims.jm, km = h->dims.km;
  static const int need[] = {LES_FIELD_DX1, LES_FIELD_DY1, LES_FIELD_DZN, LES_FIELD_DZS, LES_FIELD_DXS,
                             LES_FIELD_DYS, LES_FIELD_CN2L, LES_FIELD_CN2S, LES_FIELD_CN3L, LES_FIELD_CN3S,
                             LES_FIELD_CN4L, LES_FIELD_CN4S, LES_FIELD_UIN, LES_FIELD_VIN, LES_FIELD_WIN};
  for (int id : need)
    if (!h->h1d.count(id)) return fail(h, LES_ERR_STATE, "commit: field " + std::to_string(id) + " not uploaded");
  auto A = [&](int id, int lo) { return [&h, id, lo](int i) { return h->h1d[id][i - lo]; }; };
  auto dx1 = A(LES_FIELD_DX1, -1);
  auto dy1 = A(LES_FIELD_DY1, 0);
  auto dzn = A(LES_FIELD_DZN, -1);
  auto dzs = A(LES_FIELD_DZS, -1);
  auto dxs = A(LES_FIELD_DXS, 0);
  auto dys = A(LES_FIELD_DYS, 0);
  // derived constants, evaluated on the host with the same FP32 expressions as the
  // reference: the log-law factor (vel2.f95:138) and the les length scale (les.f95:41)
  const float logz = logf(0.5f * dzn(1) / 0.1f);
  if (!std::isfinite(logz) || logz == 0.f) return fail(h, LES_ERR_ARG, "commit: log(0.5*dzn(1)/0.1) not usable");
  std::vector<float> delx1(km);
  for (int k = 1; k <= km; ++k) delx1[k - 1] = powf(dx1(0) * dy1(0) * dzn(k), 1.f / 3.f);
  h->h1d[LES_FIELD_DELX1] = delx1;
  // cn1 = 1/(2/(dxs(i-1)dxs(i)) + 2/(dys(j-1)dys(j)) + 2/(dzs(k-1)dzs(k))) (init.f95:98-104)
  std::vector<float> ca(im + 1), cb(jm + 1), cc(km + 1), ck(km + 1, 0.f);
  for (int i = 1; i <= im; ++i) ca[i] = 2.f / (dxs(i - 1) * dxs(i));
  for (int j = 1; j <= jm; ++j) cb[j] = 2.f / (dys(j - 1) * dys(j));
  for (int k = 1; k <= km; ++k) cc[k] = 2.f / (dzs(k - 1) * dzs(k));
  bool uniform = true;
  for (int i = 2; i <= im; ++i) uniform = uniform && (ca[i] == ca[1]);
  for (int j = 2; j <= jm; ++j) uniform = uniform && (cb[j] == cb[1]);
  if (uniform)
    for (int k = 1; k <= km; ++k) ck[k] = 1.f / (ca[1] + cb[1] + cc[k]);
  bool need_cn1 = false;
  if (h->cn1_given) {
    for (int k = 1; k <= km && !need_cn1; ++k)
      for (int j = 1; j <= jm && !need_cn1; ++j)
        for (int i = 1; i <= im; ++i) {
          const float f = 1.f / (ca[i] + cb[j] + cc[k]);
          const float g = h->cn1_h[(size_t)(i - 1) + (size_t)(j - 1) * im + (size_t)(k - 1) * im * jm];
          if (memcmp(&f, &g, 4) != 0) { need_cn1 = true; break; }
        }
  }
  // correctly rounded reciprocals of the spacings and of neighbour sums (dvs, dvz)
  std::vector<float> rx1(im + 3), rx1s(im + 2), rxs(im + 1), ry1(jm + 2), ry1s(jm + 1), rys(jm + 1);
  std::vector<float> rzn(km + 4), rzs(km + 4), rzsum(km + 3);
  for (int i = -1; i <= im + 1; ++i) rx1[i + 1] = 1.f / dx1(i);
  for (int i = -1; i <= im; ++i) rx1s[i + 1] = 1.f / (dx1(i) + dx1(i + 1));
  for (int i = 0; i <= im; ++i) rxs[i] = 1.f / dxs(i);
  for (int j = 0; j <= jm + 1; ++j) ry1[j] = 1.f / dy1(j);
  for (int j = 0; j <= jm; ++j) { ry1s[j] = 1.f / (dy1(j) + dy1(j + 1)); rys[j] = 1.f / dys(j); }
  for (int k = -1; k <= km + 2; ++k) { rzn[k + 1] = 1.f / dzn(k); rzs[k + 1] = 1.f / dzs(k); }
  for (int k = -1; k <= km + 1; ++k) rzsum[k + 1] = 1.f / (dzn(k) + dzn(k + 1));
  // 1-D device buffer: [dx1 dy1 dzn dzs dxs dys z2 cn2l cn2s cn3l cn3s cn4l cn4s delx1 ca cb cc ck
  //                     and the reciprocals]
  struct Seg { int id; int lo; int n; const float *src; };
  std::vector<float> z2v(km + 3, 0.f);
  if (h->h1d.count(LES_FIELD_Z2)) z2v = h->h1d[LES_FIELD_Z2];
  std::vector<Seg> segs = {
      {LES_FIELD_DX1, -1, im + 3, h->h1d[LES_FIELD_DX1].data()}, {LES_FIELD_DY1, 0, jm + 2, h->h1d[LES_FIELD_DY1].data()},
      {LES_FIELD_DZN, -1, km + 4, h->h1d[LES_FIELD_DZN].data()}, {LES_FIELD_DZS, -1, km + 4, h->h1d[LES_FIELD_DZS].data()},
      {LES_FIELD_DXS, 0, im + 1, h->h1d[LES_FIELD_DXS].data()},  {LES_FIELD_DYS, 0, jm + 1, h->h1d[LES_FIELD_DYS].data()},
      {LES_FIELD_Z2, 0, km + 3, z2v.data()},
      {LES_FIELD_CN2L, 1, im, h->h1d[LES_FIELD_CN2L].data()},    {LES_FIELD_CN2S, 1, im, h->h1d[LES_FIELD_CN2S].data()},
      {LES_FIELD_CN3L, 1, jm, h->h1d[LES_FIELD_CN3L].data()},    {LES_FIELD_CN3S, 1, jm, h->h1d[LES_FIELD_CN3S].data()},
      {LES_FIELD_CN4L, 1, km, h->h1d[LES_FIELD_CN4L].data()},    {LES_FIELD_CN4S, 1, km, h->h1d[LES_FIELD_CN4S].data()},
      {LES_FIELD_DELX1, 1, km, h->h1d[LES_FIELD_DELX1].data()},
      {-1, 0, im + 1, ca.data()}, {-2, 0, jm + 1, cb.data()}, {-3, 0, km + 1, cc.data()}, {-4, 0, km + 1, ck.data()},
      {-5, -1, km + 4, rzn.data()}, {-6, -1, km + 4, rzs.data()}, {-7, -1, km + 3, rzsum.data()},
      {-8, -1, im + 3, rx1.data()}, {-9, -1, im + 2, rx1s.data()}, {-10, 0, im + 1, rxs.data()},
      {-11, 0, jm + 2, ry1.data()}, {-12, 0, jm + 1, ry1s.data()}, {-13, 0, jm + 1, rys.data()}};
  size_t total = 0;
  std::vector<size_t> off(segs.size());
  for (size_t q = 0; q < segs.size(); ++q) { off[q] = total; total += (segs[q].n + 7) / 8 * 8; }
  std::vector<float> buf(total, 0.f);
  for (size_t q = 0; q < segs.size(); ++q) std::copy(segs[q].src, segs[q].src + segs[q].n, buf.begin() + off[q]);
  CK(h, cudaStreamSynchronize(h->s));
  cudaFree(h->g1_d); h->g1_d = nullptr;
  CK(h, cudaMalloc(&h->g1_d, total * sizeof(float)));
  CK(h, cudaMemcpyAsync(h->g1_d, buf.data(), total * sizeof(float), cudaMemcpyHostToDevice, h->s));
  auto P = [&](size_t q) { return (const float *)(h->g1_d + off[q] - segs[q].lo); };
  LesGrid1 g;
  g.dx1 = P(0); g.dy1 = P(1); g.dzn = P(2); g.dzs = P(3); g.dxs = P(4); g.dys = P(5); g.z2 = P(6);
  g.cn2l = P(7); g.cn2s = P(8); g.cn3l = P(9); g.cn3s = P(10); g.cn4l = P(11); g.cn4s = P(12); g.delx1 = P(13);
  g.cn1a = P(14); g.cn1b = P(15); g.cn1c = P(16); g.cn1k = uniform ? P(17) : nullptr;
  g.rdzn = P(18); g.rdzs = P(19); g.rdzsum = P(20);
  g.rdx1 = P(21); g.rdx1s = P(22); g.rdxs = P(23); g.rdy1 = P(24); g.rdy1s = P(25); g.rdys = P(26);
  // full cn1 only if the uploaded one is not the separable formula bit for bit
  cudaFree(h->cn1_d); h->cn1_d = nullptr;
  if (need_cn1) {
    CK(h, cudaMalloc(&h->cn1_d, h->cn1_h.size() * sizeof(float)));
    CK(h, cudaMemcpyAsync(h->cn1_d, h->cn1_h.data(), h->cn1_h.size() * sizeof(float), cudaMemcpyHostToDevice, h->s));
  }
  // inflow planes
  const size_t nin = (size_t)jm * km;
  cudaFree(h->inflow_d); h->inflow_d = nullptr;
  CK(h, cudaMalloc(&h->inflow_d, 3 * nin * sizeof(float)));
  for (int q = 0; q < 3; ++q)
    CK(h, cudaMemcpyAsync(h->inflow_d + q * nin, h->h1d[LES_FIELD_UIN + q].data(), nin * sizeof(float),
                          cudaMemcpyHostToDevice, h->s));
  // masks
  if (h->mask_dirty) {
    CK(h, cudaMemcpyAsync(h->mask_d, h->mask_h.data(), h->nfloat, cudaMemcpyHostToDevice, h->s));
    h->mask_dirty = false;
  }
  // sum of cell volumes in FP64, as summed sequentially in the reference's loop order
  // (press.f95:65-72)
  double area = 0.0;
  if (int rc = les_setup_area(im, jm, km, h->h1d[LES_FIELD_DX1].data(), h->h1d[LES_FIELD_DY1].data(),
                           h->h1d[LES_FIELD_DZN].data(), &area))
    return fail(h, rc, "commit: les_setup_area failed");
  CK(h, cudaMemcpyAsync(h->scal_d + SC_AREA, &area, sizeof(double), cudaMemcpyHostToDevice, h->s));
  CK(h, cudaStreamSynchronize(h->s));
  // domain view
  LesDom &d = h->dom;
  d.im = im; d.jm = jm; d.km = km; d.pi = h->pi; d.nj = h->nj; d.np = h->np;
  float **F = h->fields;
  d.u = F[0]; d.v = F[1]; d.w = F[2]; d.p = F[3]; d.f = F[4]; d.g = F[5]; d.h = F[6];
  d.fold = F[7]; d.gold = F[8]; d.hold = F[9]; d.usum = F[10]; d.vsum = F[11]; d.wsum = F[12];
  d.rhs = F[13]; d.sm = F[14];
  d.cn1 = h->cn1_d;
  d.mask = h->mask_d;
  d.uin = h->inflow_d; d.vin = h->inflow_d + nin; d.win = h->inflow_d + 2 * nin;
  d.gr = g;
  d.dt = h->prm.dt; d.ro = h->prm.ro; d.vn = h->prm.vn; d.alpha = h->prm.alpha; d.beta = h->prm.beta;
  d.omega = h->prm.omega; d.pjuge = h->prm.pjuge;
  d.logz = logz;
  d.sor_fixed = h->prm.sor_fixed;
  d.sor_ksplit = h->prm.sor_ksplit;
  d.scal = h->scal_d; d.ctl = h->ctl_d; d.part = h->part_d; d.fscal = h->fscal_d;
  d.sorA = h->sor_d[0]; d.sorB = h->sor_d[1]; d.sorR = h->sor_d[2]; d.prow = h->prow_d;
  {  // power-of-two x/y spacings: exact reciprocal multiplications (dvs)
    auto pow2 = [](float x) { int e; return x > 0.f && std::isfinite(x) && std::frexp(x, &e) == 0.5f; };
    const float P = dx1(1), Q = dy1(1);
    bool ok = pow2(P) && pow2(Q);
    for (int i = -1; i <= im + 1 && ok; ++i) ok = (dx1(i) == P);
    for (int i = 0; i <= im && ok; ++i) ok = (dxs(i) == P);
    for (int j = 0; j <= jm + 1 && ok; ++j) ok = (dy1(j) == Q);
    for (int j = 0; j <= jm && ok; ++j) ok = (dys(j) == Q);
    d.xy_pow2 = ok ? 1 : 0;
    // the uniform spacings the P2 kernels use in place of the arrays' (equal) entries
    d.hx = ok ? P : 0.f; d.hy = ok ? Q : 0.f;
    d.rhx = ok ? 1.f / P : 0.f; d.rhx2 = ok ? 1.f / (P + P) : 0.f;
    d.rhy = ok ? 1.f / Q : 0.f; d.rhy2 = ok ? 1.f / (Q + Q) : 0.f;
  }
  {  // one value each for cn2l, cn2s, cn3l, cn3s: the two-iteration SOR sweep reads scalars
    auto one = [&](int id) {
      const std::vector<float> &v = h->h1d[id];
      if (v.empty()) return false;
      for (float x : v)
        if (memcmp(&x, &v[0], sizeof(float)) != 0) return false;
      return true;
    };
    d.sor_uni = (one(LES_FIELD_CN2L) && one(LES_FIELD_CN2S) && one(LES_FIELD_CN3L) && one(LES_FIELD_CN3S)) ? 1 : 0;
  }
  {  // every divisor in [2^-20, 2^20]: reciprocal-corrected divisions (dvz)
    auto inr = [](float x) { const float a = std::fabs(x); return std::isfinite(x) && a >= 0x1p-20f && a <= 0x1p20f; };
    bool ok = inr(logz) && inr(h->prm.ro) && inr(h->prm.dt);
    for (int i = -1; i <= im + 1 && ok; ++i) ok = inr(dx1(i)) && (i > im || inr(dx1(i) + dx1(i + 1)));
    for (int i = 0; i <= im && ok; ++i) ok = inr(dxs(i));
    for (int j = 0; j <= jm + 1 && ok; ++j) ok = inr(dy1(j)) && (j > jm || (inr(dy1(j) + dy1(j + 1)) && inr(dys(j))));
    for (int k = -1; k <= km + 2 && ok; ++k) ok = inr(dzn(k)) && inr(dzs(k));
    for (int k = -1; k <= km + 1 && ok; ++k) ok = inr(dzn(k) + dzn(k + 1));
    d.zfast = ok ? 1 : 0;
    if (getenv("LES_IEEE_DIV")) d.xy_pow2 = d.zfast = 0;  // every division an IEEE division (tests)
    d.rro = 1.f / h->prm.ro; d.rdt = 1.f / h->prm.dt; d.rlogz = 1.f / logz;
  }
  d.cnt = h->cnt_d; d.sms = h->sms;
  d.part2 = h->part_d + h->npart;
  for (int q = 0; q < FIX_COUNT; ++q) d.fix[q] = h->fix_d + q * h->fix_len;
  for (int q = 0; q <= 9; ++q) d.diu[q] = h->diu_d[q];
  d.ruspd = h->rsp_d; d.rvspd = h->rsp_d + h->np;
  les_step_plan_free(&h->plan);
  h->committed = true;
  return LES_OK;
}

extern "C" int les_gpu_feedbfm(les_handle *h, const float *zbm) {
  if (!h || !zbm) return LES_ERR_ARG;
  const int im = h->dims.im, jm = h->dims.jm, km = h->dims.km;
  auto z2 = h->h1d.find(LES_FIELD_Z2), dzn = h->h1d.find(LES_FIELD_DZN);
  if (z2 == h->h1d.end() || dzn == h->h1d.end())
    return fail(h, LES_ERR_STATE, "feedbfm: upload z2 and dzn first");
  // the threshold z2(k) + 0.5*dzn(k) in FP32 on the host, as feedbfm.f95:91 rounds it
  const size_t nz = (size_t)im * jm;
  std::vector<float> buf(nz + km);
  std::copy(zbm, zbm + nz, buf.begin());
  for (int k = 1; k <= km; ++k) buf[nz + k - 1] = z2->second[k] + 0.5f * dzn->second[k + 1];
  float *tmp = nullptr;
  CK(h, cudaMallocAsync((void **)&tmp, buf.size() * sizeof(float), h->s));
  CK(h, cudaMemcpyAsync(tmp, buf.data(), buf.size() * sizeof(float), cudaMemcpyHostToDevice, h->s));
  LesCtx c{h->s, &h->nlaunch};
  les_launch_feedbfm(h->mask_d, tmp, tmp + nz, im, jm, km, h->pi, h->nj, km + 4, c);
  CK(h, cudaFreeAsync(tmp, h->s));
  CK(h, cudaStreamSynchronize(h->s));  // buf is freed on return
  h->mask_dirty = false;
  h->mask_on_device = true;
  return check_launch(h, "feedbfm");
}

extern "C" int les_gpu_setup_scenario(les_handle *h, const les_scenario *sc) {
  if (!h || !sc) return LES_ERR_ARG;
  const int im = h->dims.im, jm = h->dims.jm, km = h->dims.km;
  if (sc->im != im || sc->jm != jm || sc->km != km) return fail(h, LES_ERR_ARG, "scenario dims differ from handle dims");
  std::vector<float> dx1(im + 3), dxl(im + 1), dxs(im + 1), dy1(jm + 2), dyl(jm + 1), dys(jm + 1), dzn(km + 4),
      dzs(km + 4), z2(km + 3);
  int rc = les_setup_grid(im, jm, km, sc->dx, sc->dy, sc->dz_law, sc->dz0, sc->dz_ratio, dx1.data(), dxl.data(),
                          dxs.data(), dy1.data(), dyl.data(), dys.data(), dzn.data(), dzs.data(), z2.data());
  if (rc) return fail(h, rc, "les_setup_grid failed");
  std::vector<float> cn2s(im), cn2l(im), cn3s(jm), cn3l(jm), cn4s(km), cn4l(km);
  rc = les_setup_poisson(im, jm, km, dxs.data(), dys.data(), dzs.data(), cn2s.data(), cn2l.data(), cn3s.data(),
                         cn3l.data(), cn4s.data(), cn4l.data(), nullptr);
  if (rc) return fail(h, rc, "les_setup_poisson failed");
  std::vector<float> zbm((size_t)im * jm), uin((size_t)jm * km), vin((size_t)jm * km), win((size_t)jm * km);
  rc = les_scenario_generate(sc, zbm.data(), uin.data(), vin.data(), win.data());
  if (rc) return fail(h, rc, "les_scenario_generate failed");
  struct U1 { int id; const float *p; int lo, hi; };
  const U1 ones[] = {{LES_FIELD_DX1, dx1.data(), -1, im + 1}, {LES_FIELD_DY1, dy1.data(), 0, jm + 1},
                     {LES_FIELD_DZN, dzn.data(), -1, km + 2}, {LES_FIELD_DZS, dzs.data(), -1, km + 2},
                     {LES_FIELD_DXS, dxs.data(), 0, im},      {LES_FIELD_DYS, dys.data(), 0, jm},
                     {LES_FIELD_Z2, z2.data(), 0, km + 2},    {LES_FIELD_CN2L, cn2l.data(), 1, im},
                     {LES_FIELD_CN2S, cn2s.data(), 1, im},    {LES_FIELD_CN3L, cn3l.data(), 1, jm},
                     {LES_FIELD_CN3S, cn3s.data(), 1, jm},    {LES_FIELD_CN4L, cn4l.data(), 1, km},
                     {LES_FIELD_CN4S, cn4s.data(), 1, km}};
  for (const U1 &u : ones) {
    const int lb[3] = {u.lo, 0, 0}, ub[3] = {u.hi, 0, 0};
    if ((rc = les_gpu_upload(h, u.id, u.p, lb, ub))) return rc;
  }
  const int lbi[3] = {1, 1, 0}, ubi[3] = {jm, km, 0};
  if ((rc = les_gpu_upload(h, LES_FIELD_UIN, uin.data(), lbi, ubi))) return rc;
  if ((rc = les_gpu_upload(h, LES_FIELD_VIN, vin.data(), lbi, ubi))) return rc;
  if ((rc = les_gpu_upload(h, LES_FIELD_WIN, win.data(), lbi, ubi))) return rc;
  // the masks are made on the device from the heightmap (feedbfm.f95:87-116)
  if ((rc = les_gpu_feedbfm(h, zbm.data()))) return rc;
  return les_gpu_commit_setup(h);
}

#define NEED_COMMIT(h)                                                                     \
  do {                                                                                     \
    if (!(h)) return LES_ERR_ARG;                                                          \
    if (!(h)->committed) return fail((h), LES_ERR_STATE, "les_gpu_commit_setup not called"); \
  } while (0)

// Mark a handle as sharing the GPU with other domains (les_batch_add): its SOR march
// is no longer split in k; a step graph captured with splits is dropped.
void les_handle_share_gpu(les_handle *h) {
  if (h->prm.sor_ksplit) return;
  h->prm.sor_ksplit = 1;
  h->dom.sor_ksplit = 1;
  if (h->s) cudaStreamSynchronize(h->s);
  les_step_plan_free(&h->plan);
}

// les_noalloc.cu
int les_noalloc_interior_mean(const LesDom &dom, const float *x, const double *area_dev, cudaStream_t s,
                              long long *nlaunch, int dev, double *mean, std::string *err);

extern "C" int les_gpu_field_mean_noalloc(les_handle *h, int field, double *mean) {
  if (!h || !mean) return LES_ERR_ARG;
  if (field < LES_FIELD_U || field > LES_FIELD_SM)
    return fail(h, LES_ERR_ARG, "field_mean_noalloc: field must be a 3-D field (LES_FIELD_U .. LES_FIELD_SM)");
  LesDom shape{};
  shape.im = h->dims.im; shape.jm = h->dims.jm; shape.km = h->dims.km;
  const long long nparts = les_reduce_blocks(shape);
  if (nparts > LES_NOALLOC_MAX_PARTS)
    return fail(h, LES_ERR_ARG, "field_mean_noalloc: the domain has " + std::to_string(nparts) +
                                    " reduction blocks ((im+63)/64*(jm+3)/4*((km+15)/16)); the static scratch holds " +
                                    std::to_string(LES_NOALLOC_MAX_PARTS));
  NEED_COMMIT(h);
  std::string err;
  const int rc = les_noalloc_interior_mean(h->dom, h->fields[field - 1], h->scal_d + SC_AREA, h->s, &h->nlaunch,
                                           h->dev, mean, &err);
  return rc ? fail(h, rc, err) : LES_OK;
}

extern "C" int les_gpu_velnw(les_handle *h) {
  NEED_COMMIT(h);
  les_launch_velnw(h->dom, ctx_of(h));
  return check_launch(h, "velnw");
}
extern "C" int les_gpu_bondv1(les_handle *h, int n) {
  NEED_COMMIT(h);
  les_launch_bondv1(h->dom, n, ctx_of(h));
  return check_launch(h, "bondv1");
}
extern "C" int les_gpu_velfg(les_handle *h) {
  NEED_COMMIT(h);
  les_launch_velfg_fused(h->dom, false, ctx_of(h));
  return check_launch(h, "velfg");
}
extern "C" int les_gpu_feedbf(les_handle *h) {
  NEED_COMMIT(h);
  les_launch_feedbf(h->dom, ctx_of(h));
  return check_launch(h, "feedbf");
}
extern "C" int les_gpu_les(les_handle *h) {
  NEED_COMMIT(h);
  les_launch_les_fused(h->dom, false, ctx_of(h));
  return check_launch(h, "les");
}
extern "C" int les_gpu_adam(les_handle *h) {
  NEED_COMMIT(h);
  les_launch_adam(h->dom, ctx_of(h));
  return check_launch(h, "adam");
}
extern "C" int les_gpu_bondfg(les_handle *h) {
  NEED_COMMIT(h);
  les_launch_bondfg(h->dom, ctx_of(h));
  return check_launch(h, "bondfg");
}
extern "C" int les_gpu_boundp1(les_handle *h) {
  NEED_COMMIT(h);
  les_launch_boundp1(h->dom, ctx_of(h), 0);
  return check_launch(h, "boundp1");
}
extern "C" int les_gpu_boundp2(les_handle *h) {
  NEED_COMMIT(h);
  les_launch_boundp2(h->dom, ctx_of(h), 0);
  return check_launch(h, "boundp2");
}
extern "C" int les_gpu_press(les_handle *h, int n, int nmax) {
  NEED_COMMIT(h);
  (void)n; (void)nmax;
  LesCtx c = ctx_of(h);
  les_launch_bondfg(h->dom, c);
  les_launch_rhs_mean(h->dom, c);
  les_launch_sor_simple(h->dom, h->prm.nmaxp, c);
  les_launch_pav_adjust(h->dom, c);
  h->p_dirty = false;
  return check_launch(h, "press");
}

extern "C" int les_gpu_step(les_handle *h, int n, int nmax) {
  NEED_COMMIT(h);
  if (h->p_dirty) {
    // p was uploaded: run this step through the per-subroutine kernels, which read p's
    // halos exactly as stored; press leaves them consistent for the fused graph
    les_step_enqueue(h->dom, h->prm, SorShape{}, nullptr, n, ctx_of(h));
    h->p_dirty = false;
    return check_launch(h, "step");
  }
  int rc = les_step_run(h->dom, h->prm, &h->plan, n, nmax, ctx_of(h));
  if (rc) return fail(h, LES_ERR_CUDA, std::string("step: ") + cudaGetErrorString(cudaGetLastError()));
  return check_launch(h, "step");
}

// ---- for les_batch.cu: a member's view for a batched SOR launch, and its step parts
// *ok = 1 when the member's SOR iterations 2..nmaxp can run in a batched launch: a
// committed domain, p consistent with its halos, a fused-sweep plan whose tensor maps
// fit the one-iteration TMA sweep.
int les_handle_batch_view(les_handle *h, const LesDom **d, SorShape *sh, const LesSorMaps **maps, int *nmaxp,
                          cudaStream_t *s, int *ok) {
  *ok = 0;
  if (!h || !h->committed) return LES_OK;
  *s = h->s;
  if (h->p_dirty) return LES_OK;
  const SorShape plan = les_step_plan_shape(h->dom, &h->plan);
  if (plan.ny <= 0 || !les_sor_batch_ok(h->dom, plan, &h->plan.maps)) return LES_OK;
  *d = &h->dom;
  *sh = SorShape{plan.nx, plan.ny, h->dom.km, 1};
  *maps = &h->plan.maps;
  *nmaxp = h->prm.nmaxp;
  *ok = 1;
  return LES_OK;
}
int les_handle_step_part(les_handle *h, int n, int part) {
  NEED_COMMIT(h);
  const int rc = les_step_run_part(h->dom, h->prm, &h->plan, n, part, ctx_of(h));
  if (rc) return fail(h, LES_ERR_CUDA, std::string("step part: ") + cudaGetErrorString(cudaGetLastError()));
  return check_launch(h, "step part");
}
void les_handle_count_launches(les_handle *h, long long k) { h->nlaunch += k; }

extern "C" int les_gpu_run(les_handle *h, int n0, int nsteps, int nmax) {
  NEED_COMMIT(h);
  for (int n = n0; n < n0 + nsteps; ++n) {
    int rc = les_gpu_step(h, n, nmax);
    if (rc) return rc;
  }
  return LES_OK;
}

// For les_batch.cu: the member's stream alone, and clearing its give-up word after the
// batch has reported the failure itself.
int les_handle_sync_stream(les_handle *h) {
  CK(h, cudaStreamSynchronize(h->s));
  return LES_OK;
}
void les_handle_clear_wait_error(les_handle *h) {
  if (h->ctl_d) {
    cudaMemsetAsync(h->ctl_d + CT_ERROR, 0, sizeof(int), h->s);
    cudaStreamSynchronize(h->s);
  }
}

extern "C" int les_gpu_sync(les_handle *h) {
  if (!h) return LES_ERR_ARG;
  CK(h, cudaStreamSynchronize(h->s));
  if (h->ctl_d) {  // a kernel whose bounded wait gave up: the work since the last sync is void
    int err = 0;
    CK(h, cudaMemcpyAsync(&err, h->ctl_d + CT_ERROR, sizeof err, cudaMemcpyDeviceToHost, h->s));
    CK(h, cudaStreamSynchronize(h->s));
    if (err) {
      les_handle_clear_wait_error(h);
      return fail(h, LES_ERR_STATE, "a kernel's bounded wait for its copies gave up; the steps since the last sync are void");
    }
  }
  return LES_OK;
}

extern "C" int les_gpu_diag(les_handle *h, double out[5]) {
  if (!h || !out) return LES_ERR_ARG;
  double sc[SC_COUNT];
  int ct[CT_COUNT];
  CK(h, cudaMemcpyAsync(sc, h->scal_d, sizeof sc, cudaMemcpyDeviceToHost, h->s));
  CK(h, cudaMemcpyAsync(ct, h->ctl_d, sizeof ct, cudaMemcpyDeviceToHost, h->s));
  CK(h, cudaStreamSynchronize(h->s));
  out[0] = ct[CT_ITERS];
  out[1] = sc[SC_SOR];
  out[2] = sc[SC_UOUT];
  out[3] = sc[SC_RHSAV];
  out[4] = sc[SC_PAV];
  return LES_OK;
}

extern "C" int les_gpu_aveflow(les_handle *h, int n, int n1, int nmax) {
  NEED_COMMIT(h);
  if (n1 < 1 || nmax < n1) return fail(h, LES_ERR_ARG, "aveflow: need 1 <= n1 <= nmax");
  if (!h->ave_d[0]) {
    for (int q = 0; q < kNumAve; ++q) {
      if (cudaMalloc(&h->ave_d[q], h->nfloat * sizeof(float)) != cudaSuccess) {
        (void)cudaGetLastError();
        for (float *&a : h->ave_d) { cudaFree(a); a = nullptr; }
        return fail(h, LES_ERR_NOMEM, "aveflow: no device memory for the averaging arrays");
      }
      CK(h, cudaMemsetAsync(h->ave_d[q], 0, h->nfloat * sizeof(float), h->s));
    }
  }
  float **a = h->ave_d;
  const LesAve A{a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10]};
  les_launch_aveflow(h->dom, A, n, n1, nmax, ctx_of(h));
  return check_launch(h, "aveflow");
}

extern "C" int les_gpu_set_sor_shape(les_handle *h, int nx, int ny, int kchunk, int depth) {
  if (!h) return LES_ERR_ARG;
  if ((nx != 0 && nx != 16 && nx != 32) || (ny != 0 && ny != 16 && ny != 20 && ny != 24 && ny != 28 && ny != 32) ||
      kchunk < 0 || depth < 0 || depth > 2)
    return fail(h, LES_ERR_ARG, "set_sor_shape: nx in {0,16,32}, ny in {0,16,20,24,28,32}, kchunk >= 0, depth 0..2");
  if (ny == 32 && depth != 2)
    return fail(h, LES_ERR_ARG, "set_sor_shape: 32-row tiles run two iterations per march only (depth 2)");
  if (depth == 2 && (nx == 16 || ny == 16 || ny == 20 || (kchunk > 0 && kchunk < h->dims.km)))
    return fail(h, LES_ERR_ARG, "set_sor_shape: depth 2 takes 32-column tiles, ny 24/28/32 and the whole march");
  if (h->s) CK(h, cudaStreamSynchronize(h->s));
  h->plan.fixed = SorShape{nx, ny, kchunk, depth};
  les_step_plan_free(&h->plan);  // the next step re-plans and captures its graphs again
  return LES_OK;
}

extern "C" int les_gpu_sor_shape(les_handle *h, int out[4]) {
  NEED_COMMIT(h);
  if (!out) return LES_ERR_ARG;
  const SorShape sh = les_step_plan_shape(h->dom, &h->plan);
  out[0] = sh.ny > 0 ? sh.nx : 0;
  out[1] = sh.ny;
  out[2] = sh.ny > 0 ? sh.kchunk : 0;
  out[3] = sh.ny > 0 ? sh.depth : 0;
  return LES_OK;
}

extern "C" int les_gpu_tune_sor(les_handle *h, int shared, int out[4], double *us, char *report, size_t len) {
  NEED_COMMIT(h);
  CK(h, cudaSetDevice(h->dev));
  CK(h, cudaStreamSynchronize(h->s));
  size_t free_b = 0, total_b = 0;
  CK(h, cudaMemGetInfo(&free_b, &total_b));
  const size_t budget = std::min<size_t>((size_t)4 << 30, free_b / 4);
  LesDom d = h->dom;
  d.sor_ksplit = shared ? 1 : 0;
  SorShape best;
  double sec = 0.0;
  std::string rep;
  const int rc = les_tune_sor(d, shared != 0, budget, &best, &sec, &rep);
  if (report && len > 0) {
    const size_t n = std::min(len - 1, rep.size());
    memcpy(report, rep.data(), n);
    report[n] = 0;
  }
  if (rc == 1) {  // odd jm or km too large: the per-subroutine SOR has no shape
    if (out) out[0] = out[1] = out[2] = out[3] = 0;
    if (us) *us = 0.0;
    return LES_OK;
  }
  if (rc != 0) return fail(h, LES_ERR_CUDA, "tune_sor: timing failed (" + std::to_string(rc) + ")");
  if (out) {
    out[0] = best.nx;
    out[1] = best.ny;
    out[2] = best.kchunk;
    out[3] = best.depth;
  }
  if (us) *us = sec * 1e6;
  les_step_plan_free(&h->plan);  // re-plan with the tuned shape at the next step
  return LES_OK;
}

extern "C" int les_sor_tuned(int im, int jm, int km, int shared, int device, int out[4]) {
  if (!out) return LES_ERR_ARG;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
    (void)cudaGetLastError();
    return LES_ERR_CUDA;
  }
  SorShape sh;
  if (!les_tune_lookup(im, jm, km, shared, sms, &sh)) return 0;
  out[0] = sh.nx;
  out[1] = sh.ny;
  out[2] = sh.kchunk;
  out[3] = sh.depth;
  return 1;
}

extern "C" int les_sor_set_tuned(int im, int jm, int km, int shared, int device, int nx, int ny, int kchunk,
                                 int depth) {
  if (im < 1 || jm < 1 || km < 1 || (nx != 0 && nx != 16 && nx != 32) || kchunk < 0) return LES_ERR_ARG;
  if (nx != 0) {
    if (ny != 16 && ny != 20 && ny != 24 && ny != 28 && ny != 32) return LES_ERR_ARG;
    if (depth != 1 && depth != 2) return LES_ERR_ARG;
    if (ny == 32 && depth != 2) return LES_ERR_ARG;  // 32-row tiles are built for depth 2 only
    if (depth == 2 && (nx != 32 || ny < 24 || (kchunk > 0 && kchunk < km))) return LES_ERR_ARG;
  }
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
    (void)cudaGetLastError();
    return LES_ERR_CUDA;
  }
  les_tune_store(im, jm, km, shared, sms, SorShape{nx, ny, kchunk > 0 ? std::min(kchunk, km) : km, depth});
  return LES_OK;
}

extern "C" int les_gpu_check_finite(les_handle *h, long long *bad) {
  NEED_COMMIT(h);
  if (!bad) return LES_ERR_ARG;
  CK(h, cudaMemsetAsync(h->bad_d, 0, sizeof(unsigned long long), h->s));
  les_launch_count_nonfinite(h->dom, h->bad_d, ctx_of(h));
  int rc = check_launch(h, "check_finite");
  if (rc) return rc;
  unsigned long long b = 0;
  CK(h, cudaMemcpyAsync(&b, h->bad_d, sizeof b, cudaMemcpyDeviceToHost, h->s));
  CK(h, cudaStreamSynchronize(h->s));
  *bad = (long long)b;
  return b ? LES_ERR_NUMERIC : LES_OK;
}

extern "C" int les_gpu_stream(les_handle *h, void **stream) {
  if (!h || !stream) return LES_ERR_ARG;
  *stream = (void *)h->s;
  return LES_OK;
}

extern "C" long long les_gpu_launch_count(les_handle *h) { return h ? h->nlaunch : -1; }

extern "C" int les_gpu_last_error(les_handle *h, char *buf, size_t len) {
  if (!h || !buf || len == 0) return LES_ERR_ARG;
  snprintf(buf, len, "%s", h->err.c_str());
  return LES_OK;
}

extern "C" int les_gpu_profile(les_handle *h, int what, int reps, double *ms_avg) {
  NEED_COMMIT(h);
  if (!ms_avg || reps < 1) return LES_ERR_ARG;
  if (what == LES_PROF_SOR_SWEEP) {  // events around sweeps 2..nmaxp of each pass
    std::vector<cudaEvent_t> ev(2 * (size_t)reps, nullptr);
    for (auto &e : ev) CK(h, cudaEventCreate(&e));
    LesCtx c = ctx_of(h);
    int per = 0;
    for (int r = 0; r < reps; ++r) per = les_step_sor_sweeps(h->dom, h->prm, &h->plan, c, ev[2 * r], ev[2 * r + 1]);
    double total = 0.0;
    int rc = LES_OK;
    if (per > 0) {
      CK(h, cudaEventSynchronize(ev.back()));
      for (int r = 0; r < reps; ++r) {
        float ms = 0.f;
        CK(h, cudaEventElapsedTime(&ms, ev[2 * r], ev[2 * r + 1]));
        total += ms;
      }
      *ms_avg = total / reps / per;
    } else {
      rc = fail(h, LES_ERR_STATE, "profile: this domain's SOR has no fused sweeps after the first");
    }
    CK(h, cudaStreamSynchronize(h->s));
    for (auto &e : ev) cudaEventDestroy(e);
    return rc ? rc : check_launch(h, "profile");
  }
  cudaEvent_t a, b;
  CK(h, cudaEventCreate(&a));
  CK(h, cudaEventCreate(&b));
  LesCtx c = ctx_of(h);
  CK(h, cudaEventRecord(a, h->s));
  int per_rep = 1;  // SOR: iterations per repetition, so the result is per iteration
  for (int r = 0; r < reps; ++r) {
    switch (what) {
      case LES_PROF_SOR: per_rep = les_step_sor_pass(h->dom, h->prm, &h->plan, c); break;
      case LES_PROF_VELFG: les_step_velfg_pass(h->dom, c); break;
      case LES_PROF_LES: les_step_les_pass(h->dom, c); break;
      case LES_PROF_VELNW: les_launch_velnw(h->dom, c); break;
      case LES_PROF_STEP: {
        int rc = les_step_run(h->dom, h->prm, &h->plan, 2, 2, c);
        if (rc) return fail(h, LES_ERR_CUDA, "profile: step failed");
        break;
      }
      default: cudaEventDestroy(a); cudaEventDestroy(b); return fail(h, LES_ERR_ARG, "profile: unknown stage");
    }
  }
  CK(h, cudaEventRecord(b, h->s));
  CK(h, cudaEventSynchronize(b));
  float ms = 0.f;
  CK(h, cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms_avg = (double)ms / reps / per_rep;
  return check_launch(h, "profile");
}

// Handle access for the file readers and writers of les_io.cpp (host code that sits on
// the entry points above).
int les_handle_dims(const les_handle *h, int *im, int *jm, int *km) {
  if (!h) return LES_ERR_ARG;
  *im = h->dims.im;
  *jm = h->dims.jm;
  *km = h->dims.km;
  return LES_OK;
}

int les_handle_fail(les_handle *h, int code, const char *msg) { return fail(h, code, msg); }
