// setup.cpp -- host-side producers of the solver's inputs (run once per domain).
//
// These are the reference's set-up subroutines for runtime sizes: grid.f95 (grid
// spacings), init.f95:82-107 (Poisson coefficients) and feedbfm.f95:87-116 (building
// masks from a heightmap), plus the seeded synthetic scenario that replaces the
// missing GIS files and the fixed inflow of bondv1.f95:33-54.  Built with
// -ffp-contract=off so each FP32 operation rounds as gfortran's does.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/les_gpu.h"

namespace {

// Fortran-extent 1-D view: a[i] for i in [lo, hi] stored at p[i-lo].
struct V1 {
  float *p;
  int lo;
  float &operator[](int i) const { return p[i - lo]; }
};
struct C1 {
  const float *p;
  int lo;
  float operator[](int i) const { return p[i - lo]; }
};

// splitmix64 -> portable, platform-independent stream of 64-bit words
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
  int irange(int a, int b) {  // inclusive
    return a + (int)(uniform() * (double)(b - a + 1));
  }
};

}  // namespace

extern "C" int les_setup_grid(int im, int jm, int km, float dx, float dy, int dz_law, float dz0,
                              float dz_ratio, float *dx1_, float *dxl_, float *dxs_, float *dy1_,
                              float *dyl_, float *dys_, float *dzn_, float *dzs_, float *z2_) {
  if (im < 3 || jm < 2 || km < 3 || !dx1_ || !dxl_ || !dxs_ || !dy1_ || !dyl_ || !dys_ || !dzn_ ||
      !dzs_ || !z2_)
    return LES_ERR_ARG;
  if (dz_law == 0 && km < 58) return LES_ERR_ARG;  // the piecewise law runs to k=58
  const int ip = im, jp = jm, kp = km;
  V1 dx1{dx1_, -1}, dxl{dxl_, 0}, dxs{dxs_, 0}, dy1{dy1_, 0}, dyl{dyl_, 0}, dys{dys_, 0};
  V1 dzn{dzn_, -1}, dzs{dzs_, -1}, z2{z2_, 0};
  for (int k = -1; k <= kp + 2; ++k) { dzn[k] = 0.f; dzs[k] = 0.f; }
  for (int k = 0; k <= kp + 2; ++k) z2[k] = 0.f;
  for (int i = -1; i <= ip + 1; ++i) dx1[i] = dx;                    // grid.f95:36-38
  dxl[0] = 0.f;
  for (int i = 1; i <= ip; ++i) dxl[i] = dxl[i - 1] + dx1[i];        // grid.f95:50-53
  for (int j = 0; j <= jp + 1; ++j) dy1[j] = dy;                     // grid.f95:67-69
  dyl[0] = 0.f;
  for (int j = 1; j <= jp; ++j) dyl[j] = dyl[j - 1] + dy1[j];        // grid.f95:81-84
  if (dz_law == 0) {                                                  // grid.f95:114-132
    z2[0] = 1.f; dzn[0] = 1.f; z2[1] = 1.f; dzn[1] = 1.f;
    for (int k = 2; k <= 15; ++k) dzn[k] = dzn[k - 1] * 1.1f;
    for (int k = 16; k <= 44; ++k) dzn[k] = 4.f;
    for (int k = 45; k <= 58; ++k) dzn[k] = dzn[k - 1] * 1.1f;
    for (int k = 59; k <= kp + 1; ++k) dzn[k] = 16.f;
  } else {
    z2[0] = dz0; dzn[0] = dz0; z2[1] = dz0; dzn[1] = dz0;
    for (int k = 2; k <= kp + 1; ++k) dzn[k] = dzn[k - 1] * dz_ratio;
  }
  for (int k = 2; k <= kp + 2; ++k) z2[k] = z2[k - 1] + dzn[k];      // grid.f95:133-135
  dzn[kp + 1] = dzn[kp];                                              // grid.f95:147-152
  dzn[kp + 2] = dzn[kp + 1];
  dzn[0] = dzn[1];
  dzn[-1] = dzn[0];
  for (int k = 0; k <= kp; ++k) dzs[k] = dzn[k + 1] / 2.f + dzn[k] / 2.f;   // grid.f95:154-156
  for (int i = 0; i <= ip; ++i) dxs[i] = dx1[i] / 2.f + dx1[i + 1] / 2.f;   // grid.f95:160-162
  for (int j = 0; j <= jp; ++j) dys[j] = dy1[j] / 2.f + dy1[j + 1] / 2.f;   // grid.f95:166-168
  dzs[kp + 1] = dzs[kp];                                              // grid.f95:170-172
  dzs[kp + 2] = dzs[kp + 1];
  dzs[-1] = dzs[0];
  return LES_OK;
}

extern "C" int les_setup_poisson(int im, int jm, int km, const float *dxs_, const float *dys_,
                                 const float *dzs_, float *cn2s_, float *cn2l_, float *cn3s_,
                                 float *cn3l_, float *cn4s_, float *cn4l_, float *cn1) {
  if (im < 1 || jm < 1 || km < 1 || !dxs_ || !dys_ || !dzs_ || !cn2s_ || !cn2l_ || !cn3s_ ||
      !cn3l_ || !cn4s_ || !cn4l_)
    return LES_ERR_ARG;
  C1 dxs{dxs_, 0}, dys{dys_, 0}, dzs{dzs_, -1};
  V1 cn2s{cn2s_, 1}, cn2l{cn2l_, 1}, cn3s{cn3s_, 1}, cn3l{cn3l_, 1}, cn4s{cn4s_, 1}, cn4l{cn4l_, 1};
  for (int i = 1; i <= im; ++i) {                                     // init.f95:82-85
    cn2s[i] = 2.f / (dxs[i - 1] * (dxs[i - 1] + dxs[i]));
    cn2l[i] = 2.f / (dxs[i] * (dxs[i - 1] + dxs[i]));
  }
  for (int j = 1; j <= jm; ++j) {                                     // init.f95:86-89
    cn3s[j] = 2.f / (dys[j - 1] * (dys[j - 1] + dys[j]));
    cn3l[j] = 2.f / (dys[j] * (dys[j - 1] + dys[j]));
  }
  for (int k = 1; k <= km; ++k) {                                     // init.f95:91-107
    const float dz1 = dzs[k - 1], dz2 = dzs[k];
    cn4s[k] = 2.f / (dz1 * (dz1 + dz2));
    cn4l[k] = 2.f / (dz2 * (dz1 + dz2));
    if (cn1) {
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          const float c = 2.f / (dxs[i - 1] * dxs[i]) + 2.f / (dys[j - 1] * dys[j]) + 2.f / (dz1 * dz2);
          cn1[(size_t)(i - 1) + (size_t)(j - 1) * im + (size_t)(k - 1) * im * jm] = 1.f / c;
        }
    }
  }
  return LES_OK;
}

extern "C" int les_setup_masks(int im, int jm, int km, const float *zbm, const float *z2_,
                               const float *dzn_, float *amask1, float *bmask1, float *cmask1,
                               float *dmask1) {
  if (im < 1 || jm < 1 || km < 1 || !zbm || !z2_ || !dzn_) return LES_ERR_ARG;
  C1 z2{z2_, 0}, dzn{dzn_, -1};
  // extents: amask1,dmask1 (0:im+1,0:jm+1,0:km+1); bmask1 (-1:im+1,0:jm+1,0:km+1);
  // cmask1 (0:im+1,-1:jm+1,0:km+1).  Halos stay 0 (feedbfm.f95 writes the interior).
  const long na = (long)(im + 2) * (jm + 2) * (km + 2);
  const long nb = (long)(im + 3) * (jm + 2) * (km + 2);
  const long nc = (long)(im + 2) * (jm + 3) * (km + 2);
  if (amask1) std::fill(amask1, amask1 + na, 0.f);
  if (dmask1) std::fill(dmask1, dmask1 + na, 0.f);
  if (bmask1) std::fill(bmask1, bmask1 + nb, 0.f);
  if (cmask1) std::fill(cmask1, cmask1 + nc, 0.f);
  for (int k = 1; k <= km; ++k)
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) {
        // feedbfm.f95:25-34 then :87-95 then :106-116
        float a = 1.f;
        if (zbm[(size_t)(i - 1) + (size_t)(j - 1) * im] > z2[k] + 0.5f * dzn[k]) a = 0.f;
        const float b = (a == 0.f) ? 1.f : 0.f;
        if (amask1) amask1[i + (long)j * (im + 2) + (long)k * (im + 2) * (jm + 2)] = a;
        if (dmask1) dmask1[i + (long)j * (im + 2) + (long)k * (im + 2) * (jm + 2)] = b;
        if (bmask1) bmask1[(i + 1) + (long)j * (im + 3) + (long)k * (im + 3) * (jm + 2)] = b;
        if (cmask1) cmask1[i + (long)(j + 1) * (im + 2) + (long)k * (im + 2) * (jm + 3)] = b;
      }
  return LES_OK;
}

namespace {

// Value of the last bit of a positive normal float.
double ulp_of(float t) {
  int e;
  std::frexp(t, &e);  // t = m * 2^e, m in [0.5, 1)
  return std::ldexp(1.0, e - 24);
}

}  // namespace

extern "C" int les_setup_area(int im, int jm, int km, const float *dx1_, const float *dy1_,
                              const float *dzn_, double *area) {
  if (im < 1 || jm < 1 || km < 1 || !dx1_ || !dy1_ || !dzn_ || !area) return LES_ERR_ARG;
  C1 dx1{dx1_, -1}, dy1{dy1_, 0}, dzn{dzn_, -1};
  // Distinct spacings with their multiplicities: the product dx1(i)*dy1(j)*dzn(k)
  // depends on i and j only through dx1(i) and dy1(j).
  auto groups = [](auto get, int n) {
    std::vector<std::pair<float, double>> g;
    for (int q = 1; q <= n; ++q) {
      const float x = get(q);
      auto it = std::find_if(g.begin(), g.end(), [&](const std::pair<float, double> &e) {
        return std::memcmp(&e.first, &x, 4) == 0;
      });
      if (it == g.end()) {
        if (g.size() >= 64) return std::vector<std::pair<float, double>>();  // too many: give up
        g.push_back({x, 1.0});
      } else {
        it->second += 1.0;
      }
    }
    return g;
  };
  const auto ga = groups([&](int i) { return dx1[i]; }, im);
  const auto gb = groups([&](int j) { return dy1[j]; }, jm);
  bool exact = !ga.empty() && !gb.empty();
  double sum = 0.0, umin = INFINITY;
  for (int k = 1; k <= km && exact; ++k)
    for (const auto &a : ga)
      for (const auto &b : gb) {
        const float t = a.first * b.first * dzn[k];
        if (!(t > 0.f) || !std::isfinite(t) || !std::isnormal(t)) { exact = false; break; }
        umin = std::min(umin, ulp_of(t));
        // count * t is a sum of equal terms below the bound checked next, so exact
        sum += (a.second * b.second) * (double)t;
      }
  // Every term is a multiple of umin; while the whole sum stays below 2^53 umin every
  // partial sum, in any order, is a multiple of umin that FP64 holds exactly, so the
  // grouped sum equals the sequential one.  2^52 leaves room for rounding of `sum`.
  if (exact && sum <= std::ldexp(umin, 52)) {
    *area = sum;
    return LES_OK;
  }
  double s = 0.0;
  for (int k = 1; k <= km; ++k)
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) s += (double)(dx1[i] * dy1[j] * dzn[k]);
  *area = s;
  return LES_OK;
}

extern "C" int les_scenario_generate(const les_scenario *sc, float *zbm, float *uin, float *vin,
                                     float *win) {
  if (!sc || !zbm || !uin || !vin || !win) return LES_ERR_ARG;
  const int im = sc->im, jm = sc->jm, km = sc->km;
  if (im < 3 || jm < 2 || km < 3) return LES_ERR_ARG;
  std::vector<float> dx1(im + 3), dxl(im + 1), dxs(im + 1), dy1(jm + 2), dyl(jm + 1), dys(jm + 1),
      dzn(km + 4), dzs(km + 4), z2(km + 3);
  int rc = les_setup_grid(im, jm, km, sc->dx, sc->dy, sc->dz_law, sc->dz0, sc->dz_ratio, dx1.data(),
                          dxl.data(), dxs.data(), dy1.data(), dyl.data(), dys.data(), dzn.data(),
                          dzs.data(), z2.data());
  if (rc) return rc;
  Rng rng(sc->seed ^ 0x4c45535f47423330ull);
  // Heightmap: rectangular blocks, footprint sides uniform in [fp_min, fp_max] cells,
  // heights uniform in [h_min, h_max] m, placed until the plan coverage target is met.
  // Blocks keep clear of the inflow planes and of the advective outflow: i stays in
  // [im/8, im - im/8].  j wraps periodically, like the flow.
  std::fill(zbm, zbm + (size_t)im * jm, 0.f);
  if (sc->coverage > 0.f) {
    const int ilo = std::max(3, im / 8), ihi = im - std::max(3, im / 8);
    const int fpmin = std::max(1, sc->fp_min), fpmax = std::max(fpmin, sc->fp_max);
    const long target = (long)std::ceil((double)sc->coverage * im * jm);
    long covered = 0;
    for (int tries = 0; tries < 200000 && covered < target; ++tries) {
      const int wx = std::min(rng.irange(fpmin, fpmax), std::max(1, ihi - ilo));
      const int wy = std::min(rng.irange(fpmin, fpmax), jm);
      const int i0 = rng.irange(ilo, std::max(ilo, ihi - wx));
      const int j0 = rng.irange(1, jm);
      const float ht = (float)(sc->h_min + (sc->h_max - sc->h_min) * rng.uniform());
      for (int jj = 0; jj < wy; ++jj)
        for (int ii = 0; ii < wx; ++ii) {
          const int i = i0 + ii, j = 1 + (j0 - 1 + jj) % jm;
          if (i > ihi) continue;
          float &z = zbm[(size_t)(i - 1) + (size_t)(j - 1) * im];
          if (z <= 0.f) ++covered;
          z = std::max(z, ht);
        }
    }
  }
  // Inflow planes.  The quarter-turn part of the direction is absorbed by the building
  // layout (a block field turned by 90 degrees is another draw of the same generator);
  // the residual angle r in [-45, 45) degrees sets (u, v) = U(z) (cos r, sin r).
  double deg = std::fmod((double)sc->direction_deg, 360.0);
  if (deg < 0) deg += 360.0;
  double r = deg - 90.0 * std::floor((deg + 45.0) / 90.0);
  const double rr = r * 3.14159265358979323846 / 180.0;
  const double cr = std::cos(rr), sr = std::sin(rr);
  for (int k = 1; k <= km; ++k) {
    double U;
    if (sc->inflow_law == 0) {
      U = 5.0;  // bondv1.f95:112 (u(k>=79) = u(77) = 5 as well)
    } else {
      const double z = (double)z2[k] + 0.5 * (double)dzn[k + 1];  // z2(k)+0.5*dzn(k), bondv1.f95:109
      U = (double)sc->u_ref * std::pow(z / (double)sc->z_ref, (double)sc->pl_exp);
    }
    for (int j = 1; j <= jm; ++j) {
      const size_t q = (size_t)(j - 1) + (size_t)(k - 1) * jm;
      const double nu = sc->noise * (2.0 * rng.uniform() - 1.0);
      const double nv = sc->noise * (2.0 * rng.uniform() - 1.0);
      const double nw = sc->noise * (2.0 * rng.uniform() - 1.0);
      uin[q] = (float)(U * cr + nu);
      vin[q] = (float)(U * sr + nv);
      win[q] = (float)nw;
    }
  }
  return LES_OK;
}
