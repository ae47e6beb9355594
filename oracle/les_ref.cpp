// les_ref.cpp -- CPU oracle: loop-by-loop C++ restatement of the MPI-LES per-step solver.
//
// TEST INFRASTRUCTURE ONLY (the parity checker; never part of the GPU product).
//
// Every routine below follows one reference subroutine loop by loop, with the same
// index ranges, the same halo writes and the same left-to-right FP expression order.
// Rules of the restatement (the reference is Fortran 95 compiled by gfortran -O with
// `implicit real*4`):
//   * T = float reproduces real(kind=4); T = double is the -freal-4-real-8 build.
//   * x**2 -> x*x;  x**0.5 -> powf(x,0.5) (or sqrt with REF_OPT_SQRT_HALF);
//     x**(1./3.) -> pow(x, 1/3);  alog -> log;  sqrt -> sqrt.
//   * built with -ffp-contract=off so no multiply-add is fused.
//   * arrays carry their Fortran lower/upper bounds (FA<T>); entries the reference
//     never writes stay zero, as gfortran's static main-program arrays do.
//   * non-MPI preprocessing: both branches of every `isTopRow ... else` run
//     (src/boundp.f95:41-61, src/boundsm.f95:15-57).
// Runtime sizes replace the compile-time ip,jp,kp (src/params_common_sn.f95:48); the
// reference requires im=ip etc. (src/ifdata.f95:238-241), so ip==im here.
#include "les_ref.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// The fast build (-fopenmp -DLES_REF_PAR, the timed CPU baseline) runs the stencil
// loops over k planes on all host threads: each cell of such a loop depends only on
// other arrays or on cells of the other SOR colour, so the fields are unchanged.  Only
// the SOR residual is summed differently there (per-plane partials, in plane order).
#if defined(_OPENMP) && defined(LES_REF_PAR)
#define LES_REF_OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define LES_REF_OMP_FOR
#endif

thread_local std::string g_err;

struct RefError {
  std::string msg;
};

#ifdef LES_REF_CHECK
#define FA_CHECK(cond, ...)                                                      \
  do {                                                                           \
    if (!(cond)) {                                                               \
      char b_[256];                                                              \
      snprintf(b_, sizeof b_, __VA_ARGS__);                                      \
      throw RefError{b_};                                                        \
    }                                                                            \
  } while (0)
#else
#define FA_CHECK(cond, ...) \
  do {                      \
  } while (0)
#endif

// Fortran-ordered array with arbitrary lower bounds (rank <= 3, i fastest).
template <class T>
struct FA {
  std::vector<T> d;
  int l0 = 0, u0 = -1, l1 = 0, u1 = 0, l2 = 0, u2 = 0;
  long s1 = 0, s2 = 0;
  const char *name = "";
  void alloc(const char *nm, int a0, int b0, int a1 = 0, int b1 = 0, int a2 = 0, int b2 = 0) {
    name = nm;
    l0 = a0; u0 = b0; l1 = a1; u1 = b1; l2 = a2; u2 = b2;
    s1 = b0 - a0 + 1;
    s2 = s1 * (b1 - a1 + 1);
    d.assign((size_t)s2 * (size_t)(b2 - a2 + 1), T(0));
  }
  inline T &operator()(int i, int j = 0, int k = 0) {
    FA_CHECK(i >= l0 && i <= u0 && j >= l1 && j <= u1 && k >= l2 && k <= u2,
             "index (%d,%d,%d) out of bounds of %s(%d:%d,%d:%d,%d:%d)", i, j, k, name, l0,
             u0, l1, u1, l2, u2);
    return d[(size_t)((i - l0) + (j - l1) * s1 + (k - l2) * s2)];
  }
};

// Fortran literal of default kind: the float literal for T=float, the double
// literal for T=double (-freal-4-real-8 promotes literals as well).
#define L(x) (sizeof(T) == 4 ? T(x##f) : T(x))

template <class T>
T pow_half(T x, int sqrt_half) {
  if (sqrt_half) return std::sqrt(x);
  return std::pow(x, L(0.5));
}

template <class T>
struct Ref {
  int im, jm, km;
  int nmaxp, sor_fixed, red64, sqrt_half, dz_law;
  T dt, ro, vn, alpha, beta, omega, pjuge;
  T cdx, cdy, dz0, dzratio;

  FA<T> dx1, dxl, dxs, dy1, dyl, dys, dzn, dzs, z2;
  FA<T> cn2l, cn2s, cn3l, cn3s, cn4l, cn4s, delx1;
  FA<T> amask1, bmask1, cmask1, dmask1, cn1;
  FA<T> u, v, w, p, f, g, h, fold, gold, hold, usum, vsum, wsum, rhs, sm, fx, fy, fz;
  FA<T> uspd, vspd, zbm, uin, vin, win;
  FA<T> nou[10], diu[10], cov[10];
  FA<T> dfu1, dfv1, dfw1;
  // aveflow.f95:7-22 (time averages; allocated on the first aveflow call)
  FA<T> aveu, avev, avew, avep, avel, aveuu, avevv, aveww, avesm, avesmsm, uwfx;
  bool ave_alloc = false;

  // trap_wall: stop with an error where the wall function would form 0/0 (a wall speed
  // of zero, vel2.f95:138,173) instead of producing the NaN the reference produces
  bool trap_wall = false;
  void wall_check(T speed, int i, int j, const char *which) const {
    if (!trap_wall || speed != L(0.)) return;
    char b[160];
    snprintf(b, sizeof b, "vel2.f95: %s(%d,%d) = 0: the wall function divides 0 by 0", which, i, j);
    throw RefError{b};
  }

  // diagnostics of the last step
  int last_iters = 0;
  double last_sor = 0, last_uout = 0, last_rhsav = 0, last_pav = 0, last_area = 0, last_pco = 0;

  void allocate() {
    const int ip = im, jp = jm, kp = km;
    // main.f95:63-159 (declared extents)
    amask1.alloc("amask1", 0, ip + 1, 0, jp + 1, 0, kp + 1);
    bmask1.alloc("bmask1", -1, ip + 1, 0, jp + 1, 0, kp + 1);
    cmask1.alloc("cmask1", 0, ip + 1, -1, jp + 1, 0, kp + 1);
    dmask1.alloc("dmask1", 0, ip + 1, 0, jp + 1, 0, kp + 1);
    cn1.alloc("cn1", 1, ip, 1, jp, 1, kp);
    cn2l.alloc("cn2l", 1, ip); cn2s.alloc("cn2s", 1, ip);
    cn3l.alloc("cn3l", 1, jp); cn3s.alloc("cn3s", 1, jp);
    cn4l.alloc("cn4l", 1, kp); cn4s.alloc("cn4s", 1, kp);
    static const char *nn[10] = {"", "nou1", "nou2", "nou3", "nou4", "nou5", "nou6", "nou7", "nou8", "nou9"};
    static const char *dn[10] = {"", "diu1", "diu2", "diu3", "diu4", "diu5", "diu6", "diu7", "diu8", "diu9"};
    static const char *cnm[10] = {"", "cov1", "cov2", "cov3", "cov4", "cov5", "cov6", "cov7", "cov8", "cov9"};
    for (int q = 1; q <= 9; ++q) {
      const int lo = (q == 1 || q == 5) ? -1 : 0;
      nou[q].alloc(nn[q], lo, ip + 2, 0, jp + 2, 0, kp + 2);
      diu[q].alloc(dn[q], lo, ip + 2, 0, jp + 2, 0, kp + 2);
      cov[q].alloc(cnm[q], lo, ip + 2, 0, jp + 2, 0, kp + 2);
    }
    delx1.alloc("delx1", 1, kp);
    dfu1.alloc("dfu1", 0, ip, 1, jp, 1, kp);
    dfv1.alloc("dfv1", 1, ip, 0, jp, 1, kp);
    dfw1.alloc("dfw1", 1, ip, 1, jp, 1, kp);
    dx1.alloc("dx1", -1, ip + 1); dxl.alloc("dxl", 0, ip); dxs.alloc("dxs", 0, ip);
    dy1.alloc("dy1", 0, jp + 1); dyl.alloc("dyl", 0, jp); dys.alloc("dys", 0, jp);
    dzn.alloc("dzn", -1, kp + 2); dzs.alloc("dzs", -1, kp + 2);
    f.alloc("f", 0, ip, 0, jp, 0, kp); g.alloc("g", 0, ip, 0, jp, 0, kp); h.alloc("h", 0, ip, 0, jp, 0, kp);
    fold.alloc("fold", 1, ip, 1, jp, 1, kp); gold.alloc("gold", 1, ip, 1, jp, 1, kp);
    hold.alloc("hold", 1, ip, 1, jp, 1, kp);
    fx.alloc("fx", 0, ip, 0, jp, 0, kp); fy.alloc("fy", 0, ip, 0, jp, 0, kp); fz.alloc("fz", 0, ip, 0, jp, 0, kp);
    p.alloc("p", 0, ip + 2, 0, jp + 2, 0, kp + 1);
    rhs.alloc("rhs", 0, ip + 1, 0, jp + 1, 0, kp + 1);
    sm.alloc("sm", -1, ip + 1, -1, jp + 1, 0, kp + 1);
    u.alloc("u", 0, ip + 1, -1, jp + 1, 0, kp + 1);
    v.alloc("v", 0, ip + 1, -1, jp + 1, 0, kp + 1);
    w.alloc("w", 0, ip + 1, -1, jp + 1, -1, kp + 1);
    usum.alloc("usum", 0, ip, 0, jp, 0, kp); vsum.alloc("vsum", 0, ip, 0, jp, 0, kp);
    wsum.alloc("wsum", 0, ip, 0, jp, 0, kp);
    z2.alloc("z2", 0, kp + 2);
    zbm.alloc("zbm", -1, ip + 1, -1, jp + 1);
    uspd.alloc("uspd", 0, ip + 1, 0, jp + 1); vspd.alloc("vspd", 0, ip + 1, 0, jp + 1);
    uin.alloc("uin", 1, jp, 1, kp); vin.alloc("vin", 1, jp, 1, kp); win.alloc("win", 1, jp, 1, kp);
  }

  // ---------------------------------------------------------------- grid.f95:5-182
  void grid() {
    const int ip = im, jp = jm, kp = km;
    for (int i = -1; i <= ip + 1; ++i) dx1(i) = cdx;                    // grid.f95:36-38
    dxl(0) = L(0.);
    for (int i = 1; i <= ip; ++i) dxl(i) = dxl(i - 1) + dx1(i);         // :50-53
    for (int j = 0; j <= jp + 1; ++j) dy1(j) = cdy;                     // :67-69
    dyl(0) = L(0.);
    for (int j = 1; j <= jp; ++j) dyl(j) = dyl(j - 1) + dy1(j);         // :81-84
    if (dz_law == 0) {
      // grid.f95:114-135: 1 m x1.1 up to k=15, 4 m to 44, x1.1 to 58, 16 m above
      if (kp < 58) throw RefError{"reference dz law needs km >= 58 (grid.f95:127-132)"};
      z2(0) = L(1.); dzn(0) = L(1.); z2(1) = L(1.); dzn(1) = L(1.);
      for (int k = 2; k <= 15; ++k) dzn(k) = dzn(k - 1) * L(1.1);
      for (int k = 16; k <= 44; ++k) dzn(k) = L(4.);
      for (int k = 45; k <= 58; ++k) dzn(k) = dzn(k - 1) * L(1.1);
      for (int k = 59; k <= kp + 1; ++k) dzn(k) = L(16.);
    } else {
      // geometric law (the configs' "dz0 at ground, stretched by ratio"), written
      // in the same shape: dzn(0)=dzn(1)=z2(0)=z2(1)=dz0, dzn(k)=dzn(k-1)*ratio
      z2(0) = dz0; dzn(0) = dz0; z2(1) = dz0; dzn(1) = dz0;
      for (int k = 2; k <= kp + 1; ++k) dzn(k) = dzn(k - 1) * dzratio;
    }
    for (int k = 2; k <= kp + 2; ++k) z2(k) = z2(k - 1) + dzn(k);      // :133-135
    dzn(kp + 1) = dzn(kp);                                              // :147-152
    dzn(kp + 2) = dzn(kp + 1);
    dzn(0) = dzn(1);
    dzn(-1) = dzn(0);
    for (int k = 0; k <= kp; ++k) dzs(k) = dzn(k + 1) / L(2.) + dzn(k) / L(2.);   // :154-156
    for (int i = 0; i <= ip; ++i) dxs(i) = dx1(i) / L(2.) + dx1(i + 1) / L(2.);   // :160-162
    for (int j = 0; j <= jp; ++j) dys(j) = dy1(j) / L(2.) + dy1(j + 1) / L(2.);   // :166-168
    dzs(kp + 1) = dzs(kp);                                              // :170-172
    dzs(kp + 2) = dzs(kp + 1);
    dzs(-1) = dzs(0);
  }

  // ---------------------------------------------------------------- feedbfm.f95:25-116
  void feedbfm() {
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          amask1(i, j, k) = L(1.);
          bmask1(i, j, k) = L(0.);
          cmask1(i, j, k) = L(0.);
          dmask1(i, j, k) = L(0.);
        }
    // zbm comes from the scenario heightmap instead of the GIS files (feedbfm.f95:52-77)
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i)
        for (int k = 1; k <= km; ++k)
          if (zbm(i, j) > z2(k) + L(0.5) * dzn(k)) amask1(i, j, k) = L(0.0);
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i)
          if (amask1(i, j, k) == L(0.0)) {
            bmask1(i, j, k) = L(1.0);
            cmask1(i, j, k) = L(1.0);
            dmask1(i, j, k) = L(1.0);
          }
  }

  // ---------------------------------------------------------------- init.f95:46-107
  void init() {
    // u, v, w, p are zero from allocation (init.f95:46-69)
    feedbfm();
    for (int i = 1; i <= im; ++i) {
      cn2s(i) = L(2.) / (dxs(i - 1) * (dxs(i - 1) + dxs(i)));
      cn2l(i) = L(2.) / (dxs(i) * (dxs(i - 1) + dxs(i)));
    }
    for (int j = 1; j <= jm; ++j) {
      cn3s(j) = L(2.) / (dys(j - 1) * (dys(j - 1) + dys(j)));
      cn3l(j) = L(2.) / (dys(j) * (dys(j - 1) + dys(j)));
    }
    for (int k = 1; k <= km; ++k) {
      const T dz1 = dzs(k - 1);
      const T dz2 = dzs(k);
      cn4s(k) = L(2.) / (dz1 * (dz1 + dz2));
      cn4l(k) = L(2.) / (dz2 * (dz1 + dz2));
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          cn1(i, j, k) = L(2.) / (dxs(i - 1) * dxs(i)) + L(2.) / (dys(j - 1) * dys(j)) +
                         L(2.) / (dz1 * dz2);
          cn1(i, j, k) = L(1.) / cn1(i, j, k);
        }
    }
  }

  // ---------------------------------------------------------------- velnw.f95:27-59
  void velnw() {
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          const T pz = (-p(i, j, k) + p(i + 1, j, k)) / ro / dxs(i);
          u(i, j, k) = u(i, j, k) + dt * (f(i, j, k) - pz);
        }
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          const T pz = (-p(i, j, k) + p(i, j + 1, k)) / ro / dys(j);
          v(i, j, k) = v(i, j, k) + dt * (g(i, j, k) - pz);
        }
    LES_REF_OMP_FOR
    for (int k = 1; k <= km - 1; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          const T pz = (-p(i, j, k) + p(i, j, k + 1)) / ro / dzs(k);
          w(i, j, k) = w(i, j, k) + dt * (h(i, j, k) - pz);
        }
  }

  // ---------------------------------------------------------------- bondv1.f95:5-200
  void bondv1(int n) {
    // inflow planes i=0,1 (bondv1.f95:33-54).  The reference hard-codes u=5 m/s for
    // k<=78 and u(k>=79)=u(77); here the planes come from the scenario and the k loop
    // is bounded by km.
    for (int i = 0; i <= 1; ++i)
      for (int k = 1; k <= km; ++k)
        for (int j = 1; j <= jm; ++j) {
          u(i, j, k) = uin(j, k);
          v(i, j, k) = vin(j, k);
          w(i, j, k) = win(j, k);
        }
    if (n == 1) {  // ICAL == 0 initial fill (bondv1.f95:59-89)
      for (int k = 1; k <= km; ++k)
        for (int j = 1; j <= jm; ++j)
          for (int i = 2; i <= im; ++i) {
            u(i, j, k) = u(1, j, k);
            v(i, j, k) = v(1, j, k);
            w(i, j, k) = w(1, j, k);
          }
    }
    // advective outflow (bondv1.f95:98-134)
    T aaa = L(0.0), bbb = L(0.0);
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j) {
        aaa = std::max(aaa, u(im, j, k));   // amax1
        bbb = std::min(bbb, u(im, j, k));   // amin1
      }
    const T uout = (aaa + bbb) / L(2.);
    last_uout = (double)uout;
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        u(im, j, k) = u(im, j, k) - dt * uout * (u(im, j, k) - u(im - 1, j, k)) / dxs(im);
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        v(im + 1, j, k) = v(im + 1, j, k) - dt * uout * (v(im + 1, j, k) - v(im, j, k)) / dxs(im);
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        w(im + 1, j, k) = w(im + 1, j, k) - dt * uout * (w(im + 1, j, k) - w(im, j, k)) / dxs(im);
    // periodic side flow (bondv1.f95:136-156)
    for (int k = 0; k <= km + 1; ++k)
      for (int i = 0; i <= im + 1; ++i) {
        u(i, 0, k) = u(i, jm, k);
        u(i, jm + 1, k) = u(i, 1, k);
      }
    for (int k = 0; k <= km + 1; ++k)
      for (int i = 0; i <= im + 1; ++i) {
        v(i, 0, k) = v(i, jm, k);
        v(i, jm + 1, k) = v(i, 1, k);
      }
    for (int k = 0; k <= km; ++k)
      for (int i = 0; i <= im + 1; ++i) {
        w(i, 0, k) = w(i, jm, k);
        w(i, jm + 1, k) = w(i, 1, k);
      }
    // top and underground (bondv1.f95:176-195)
    for (int j = 0; j <= jm + 1; ++j)
      for (int i = 0; i <= im + 1; ++i) {
        u(i, j, 0) = -u(i, j, 1);
        u(i, j, km + 1) = u(i, j, km);
      }
    for (int j = 0; j <= jm + 1; ++j)
      for (int i = 0; i <= im + 1; ++i) {
        v(i, j, 0) = -v(i, j, 1);
        v(i, j, km + 1) = v(i, j, km);
      }
    for (int j = -1; j <= jm + 1; ++j)
      for (int i = 0; i <= im + 1; ++i) {
        w(i, j, 0) = L(0.0);
        w(i, j, km) = L(0.0);
      }
  }

  // ---------------------------------------------------------------- vel2.f95:4-364
  void vel2() {
    FA<T> &nou1 = nou[1], &nou2 = nou[2], &nou3 = nou[3], &nou4 = nou[4], &nou5 = nou[5],
          &nou6 = nou[6], &nou7 = nou[7], &nou8 = nou[8], &nou9 = nou[9];
    FA<T> &diu1 = diu[1], &diu2 = diu[2], &diu3 = diu[3], &diu4 = diu[4], &diu5 = diu[5],
          &diu6 = diu[6], &diu7 = diu[7], &diu8 = diu[8], &diu9 = diu[9];
    FA<T> &cov1 = cov[1], &cov2 = cov[2], &cov3 = cov[3], &cov4 = cov[4], &cov5 = cov[5],
          &cov6 = cov[6], &cov7 = cov[7], &cov8 = cov[8], &cov9 = cov[9];
    const T u0 = L(0.);  // integer parameter u0 = 0 (vel2.f95:49)
    // wall-function speeds (vel2.f95:54-65)
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) {
        const T a = u(i, j, 1);
        const T b = (L(0.5) * (v(i, j - 1, 1) + v(i, j, 1)) * dx1(i + 1) +
                     L(0.5) * (v(i + 1, j - 1, 1) + v(i + 1, j, 1)) * dx1(i)) /
                    (dx1(i) + dx1(i + 1));
        uspd(i, j) = pow_half(a * a + b * b, sqrt_half);
      }
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) {
        const T a = v(i, j, 1);
        const T b = (L(0.5) * (u(i - 1, j, 1) + u(i, j, 1)) * dy1(j + 1) +
                     L(0.5) * (u(i - 1, j + 1, 1) + u(i, j + 1, 1)) * dy1(j)) /
                    (dy1(j) + dy1(j + 1));
        vspd(i, j) = pow_half(a * a + b * b, sqrt_half);
      }
    // vel2.f95:74-89
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          nou1(i, j, k) = (u(i - 1, j, k) + u(i, j, k)) / L(2.);
          diu1(i, j, k) = (-u(i - 1, j, k) + u(i, j, k)) / dx1(i);
          nou5(i, j, k) = (v(i, j - 1, k) + v(i, j, k)) / L(2.);
          diu5(i, j, k) = (-v(i, j - 1, k) + v(i, j, k)) / dy1(j);
          nou9(i, j, k) = (w(i, j, k - 1) + w(i, j, k)) / L(2.);
          diu9(i, j, k) = (-w(i, j, k - 1) + w(i, j, k)) / dzn(k);
          cov1(i, j, k) = nou1(i, j, k) * diu1(i, j, k);
          cov5(i, j, k) = nou5(i, j, k) * diu5(i, j, k);
          cov9(i, j, k) = nou9(i, j, k) * diu9(i, j, k);
        }
    // vel2.f95:103-111
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          nou2(i, j, k) = (dx1(i + 1) * v(i, j - 1, k) + dx1(i) * v(i + 1, j - 1, k)) / (dx1(i) + dx1(i + 1));
          diu2(i, j, k) = L(2.) * (-u(i, j - 1, k) + u(i, j, k)) / (dy1(j - 1) + dy1(j));
          cov2(i, j, k) = nou2(i, j, k) * diu2(i, j, k);
        }
    // vel2.f95:119-127
    LES_REF_OMP_FOR
    for (int k = 2; k <= km + 1; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          nou3(i, j, k) = (dx1(i + 1) * w(i, j, k - 1) + dx1(i) * w(i + 1, j, k - 1)) / (dx1(i) + dx1(i + 1));
          diu3(i, j, k) = (-u(i, j, k - 1) + u(i, j, k)) / dzs(k - 1);
          cov3(i, j, k) = nou3(i, j, k) * diu3(i, j, k);
        }
    // log-law wall gradient at k=1 (vel2.f95:135-141)
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) {
        nou3(i, j, 1) = L(0.5) * (dx1(i + 1) * w(i, j, 1) + dx1(i) * w(i + 1, j, 1)) / (dx1(i) + dx1(i + 1));
        wall_check(uspd(i, j), i, j, "uspd");
        diu3(i, j, 1) = uspd(i, j) * L(0.4) / std::log(L(0.5) * dzn(1) / L(0.1)) / (L(0.5) * dzn(1)) /
                        L(0.4) * u(i, j, 1) / uspd(i, j);
        cov3(i, j, 1) = nou3(i, j, 1) * diu3(i, j, 1);
      }
    // vel2.f95:144-152
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          nou4(i, j, k) = (dy1(j + 1) * u(i - 1, j, k) + dy1(j) * u(i - 1, j + 1, k)) / (dy1(j) + dy1(j + 1));
          diu4(i, j, k) = L(2.) * (-v(i - 1, j, k) + v(i, j, k)) / (dx1(i - 1) + dx1(i));
          cov4(i, j, k) = (nou4(i, j, k) - u0) * diu4(i, j, k);
        }
    // vel2.f95:154-162
    LES_REF_OMP_FOR
    for (int k = 2; k <= km + 1; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          nou6(i, j, k) = (dy1(j + 1) * w(i, j, k - 1) + dy1(j) * w(i, j + 1, k - 1)) / (dy1(j) + dy1(j + 1));
          diu6(i, j, k) = (-v(i, j, k - 1) + v(i, j, k)) / dzs(k - 1);
          cov6(i, j, k) = nou6(i, j, k) * diu6(i, j, k);
        }
    // vel2.f95:170-176
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) {
        nou6(i, j, 1) = L(0.5) * (dy1(j + 1) * w(i, j, 1) + dy1(j) * w(i, j + 1, 1)) / (dy1(j) + dy1(j + 1));
        wall_check(vspd(i, j), i, j, "vspd");
        diu6(i, j, 1) = vspd(i, j) * L(0.4) / std::log(L(0.5) * dzn(1) / L(0.1)) / (L(0.5) * dzn(1)) /
                        L(0.4) * v(i, j, 1) / vspd(i, j);
        cov6(i, j, 1) = nou6(i, j, 1) * diu6(i, j, 1);
      }
    // vel2.f95:179-187
    LES_REF_OMP_FOR
    for (int k = 1; k <= km - 1; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          nou7(i, j, k) = (dzn(k + 1) * u(i - 1, j, k) + dzn(k) * u(i - 1, j, k + 1)) / (dzn(k) + dzn(k + 1));
          diu7(i, j, k) = L(2.) * (-w(i - 1, j, k) + w(i, j, k)) / (dx1(i - 1) + dx1(i));
          cov7(i, j, k) = (nou7(i, j, k) - u0) * diu7(i, j, k);
        }
    // vel2.f95:189-197
    LES_REF_OMP_FOR
    for (int k = 1; k <= km - 1; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          nou8(i, j, k) = (dzn(k + 1) * v(i, j - 1, k) + dzn(k) * v(i, j - 1, k + 1)) / (dzn(k) + dzn(k + 1));
          diu8(i, j, k) = L(2.) * (-w(i, j - 1, k) + w(i, j, k)) / (dy1(j - 1) + dy1(j));
          cov8(i, j, k) = nou8(i, j, k) * diu8(i, j, k);
        }
    // halo copies (vel2.f95:202-318), non-MPI branches
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j) {
        nou1(im + 1, j, k) = nou1(im, j, k);
        diu1(im + 1, j, k) = diu1(im, j, k);
        cov1(im + 1, j, k) = cov1(im, j, k);
      }
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int i = 1; i <= im; ++i) {
        nou2(i, 0, k) = nou2(i, jm, k);
        diu2(i, 0, k) = diu2(i, jm, k);
        cov2(i, 0, k) = cov2(i, jm, k);
        nou2(i, jm + 1, k) = nou2(i, 1, k);
        diu2(i, jm + 1, k) = diu2(i, 1, k);
        cov2(i, jm + 1, k) = cov2(i, 1, k);
      }
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j) {
        nou4(im + 1, j, k) = nou4(im, j, k);
        diu4(im + 1, j, k) = diu4(im, j, k);
        cov4(im + 1, j, k) = cov4(im, j, k);
      }
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int i = 1; i <= im; ++i) {
        nou5(i, 0, k) = nou5(i, jm, k);
        diu5(i, 0, k) = diu5(i, jm, k);
        cov5(i, 0, k) = cov5(i, jm, k);
        nou5(i, jm + 1, k) = nou5(i, 1, k);
        diu5(i, jm + 1, k) = diu5(i, 1, k);
        cov5(i, jm + 1, k) = cov5(i, 1, k);
      }
    LES_REF_OMP_FOR
    for (int k = 1; k <= km - 1; ++k)
      for (int j = 1; j <= jm; ++j) {
        nou7(im + 1, j, k) = nou7(im, j, k);
        diu7(im + 1, j, k) = diu7(im, j, k);
        cov7(im + 1, j, k) = cov7(im, j, k);
      }
    LES_REF_OMP_FOR
    for (int k = 1; k <= km - 1; ++k)
      for (int i = 1; i <= im; ++i) {
        nou8(i, 0, k) = nou8(i, jm, k);
        diu8(i, 0, k) = diu8(i, jm, k);
        cov8(i, 0, k) = cov8(i, jm, k);
        nou8(i, jm + 1, k) = nou8(i, 1, k);
        diu8(i, jm + 1, k) = diu8(i, 1, k);
        cov8(i, jm + 1, k) = cov8(i, 1, k);
      }
    LES_REF_OMP_FOR
    for (int k = 1; k <= km + 1; ++k)
      for (int j = 1; j <= jm + 1; ++j) {
        diu2(im + 1, j, k) = diu2(im, j, k);
        diu3(im + 1, j, k) = diu3(im, j, k);
      }
    LES_REF_OMP_FOR
    for (int k = 1; k <= km + 1; ++k)
      for (int i = 1; i <= im + 1; ++i) {
        diu4(i, 0, k) = diu4(i, jm, k);
        diu6(i, 0, k) = diu6(i, jm, k);
      }
    // uspd := u/uspd, vspd := v/vspd (vel2.f95:351-356)
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) {
        uspd(i, j) = u(i, j, 1) / uspd(i, j);
        vspd(i, j) = v(i, j, 1) / vspd(i, j);
      }
  }

  // ---------------------------------------------------------------- velFG.f95:61-110
  void velfg() {
    vel2();
    FA<T> &cov1 = cov[1], &cov2 = cov[2], &cov3 = cov[3], &cov4 = cov[4], &cov5 = cov[5],
          &cov6 = cov[6], &cov7 = cov[7], &cov8 = cov[8], &cov9 = cov[9];
    FA<T> &diu1 = diu[1], &diu2 = diu[2], &diu3 = diu[3], &diu4 = diu[4], &diu5 = diu[5],
          &diu6 = diu[6], &diu7 = diu[7], &diu8 = diu[8], &diu9 = diu[9];
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          const T covx1 = (dx1(i + 1) * cov1(i, j, k) + dx1(i) * cov1(i + 1, j, k)) / (dx1(i) + dx1(i + 1));
          const T covy1 = (cov2(i, j, k) + cov2(i, j + 1, k)) / L(2.);
          const T covz1 = (cov3(i, j, k) + cov3(i, j, k + 1)) / L(2.);
          const T covc = covx1 + covy1 + covz1;
          dfu1(i, j, k) = L(2.) * (-diu1(i, j, k) + diu1(i + 1, j, k)) / (dx1(i) + dx1(i + 1)) +
                          (-diu2(i, j, k) + diu2(i, j + 1, k)) / dy1(j) +
                          (-diu3(i, j, k) + diu3(i, j, k + 1)) / dzn(k);
          const T df = vn * dfu1(i, j, k);
          f(i, j, k) = (-covc + df);
        }
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          const T covx1 = (cov4(i, j, k) + cov4(i + 1, j, k)) / L(2.);
          const T covy1 = (dy1(j + 1) * cov5(i, j, k) + dy1(j) * cov5(i, j + 1, k)) / (dy1(j) + dy1(j + 1));
          const T covz1 = (cov6(i, j, k) + cov6(i, j, k + 1)) / L(2.);
          const T covc = covx1 + covy1 + covz1;
          dfv1(i, j, k) = (-diu4(i, j, k) + diu4(i + 1, j, k)) / dx1(i) +
                          L(2.) * (-diu5(i, j, k) + diu5(i, j + 1, k)) / (dy1(j) + dy1(j + 1)) +
                          (-diu6(i, j, k) + diu6(i, j, k + 1)) / dzn(k);
          const T df = vn * dfv1(i, j, k);
          g(i, j, k) = (-covc + df);
        }
    LES_REF_OMP_FOR
    for (int k = 1; k <= km - 1; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          const T covx1 = (cov7(i, j, k) + cov7(i + 1, j, k)) / L(2.);
          const T covy1 = (cov8(i, j, k) + cov8(i, j + 1, k)) / L(2.);
          const T covz1 = (dzn(k + 1) * cov9(i, j, k) + dzn(k) * cov9(i, j, k + 1)) / (dzn(k) + dzn(k + 1));
          const T covc = covx1 + covy1 + covz1;
          dfw1(i, j, k) = (-diu7(i, j, k) + diu7(i + 1, j, k)) / dx1(i) +
                          (-diu8(i, j, k) + diu8(i, j + 1, k)) / dy1(j) +
                          (-diu9(i, j, k) + diu9(i, j, k + 1)) / dzs(k);
          const T df = vn * dfw1(i, j, k);
          h(i, j, k) = (-covc + df);
        }
  }

  // ---------------------------------------------------------------- feedbf.f95:35-61
  void feedbf() {
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          usum(i, j, k) = (usum(i, j, k) + u(i, j, k)) * bmask1(i, j, k);
          vsum(i, j, k) = (vsum(i, j, k) + v(i, j, k)) * cmask1(i, j, k);
          wsum(i, j, k) = (wsum(i, j, k) + w(i, j, k)) * dmask1(i, j, k);
          const T f1x = alpha * usum(i, j, k) * dt;
          const T f1y = alpha * vsum(i, j, k) * dt;
          const T f1z = alpha * wsum(i, j, k) * dt;
          const T f2x = beta * u(i, j, k) * bmask1(i, j, k);
          const T f2y = beta * v(i, j, k) * cmask1(i, j, k);
          const T f2z = beta * w(i, j, k) * dmask1(i, j, k);
          fx(i, j, k) = f1x + f2x;
          fy(i, j, k) = f1y + f2y;
          fz(i, j, k) = f1z + f2z;
        }
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          f(i, j, k) = f(i, j, k) + fx(i, j, k);
          g(i, j, k) = g(i, j, k) + fy(i, j, k);
          h(i, j, k) = h(i, j, k) + fz(i, j, k);
        }
  }

  // ---------------------------------------------------------------- boundsm.f95:18-64
  void boundsm() {
    for (int k = 0; k <= km + 1; ++k)
      for (int j = -1; j <= jm + 1; ++j) {
        sm(0, j, k) = sm(1, j, k);
        sm(im + 1, j, k) = sm(im, j, k);
      }
    for (int k = 0; k <= km + 1; ++k)
      for (int i = 0; i <= im + 1; ++i) {
        sm(i, jm + 1, k) = sm(i, jm, k);
        sm(i, 0, k) = sm(i, 1, k);
      }
    for (int j = -1; j <= jm + 1; ++j)
      for (int i = 0; i <= im + 1; ++i) {
        sm(i, j, 0) = -sm(i, j, 1);
        sm(i, j, km + 1) = sm(i, j, km);
      }
  }

  // ---------------------------------------------------------------- les.f95:36-242
  void les() {
    FA<T> &diu1 = diu[1], &diu2 = diu[2], &diu3 = diu[3], &diu4 = diu[4], &diu5 = diu[5],
          &diu6 = diu[6], &diu7 = diu[7], &diu8 = diu[8], &diu9 = diu[9];
    const T cs0 = L(.1);
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      delx1(k) = std::pow(dx1(0) * dy1(0) * dzn(k), L(1.) / L(3.));   // les.f95:38-42
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          const T dudxx1 = diu1(i, j, k);
          const T dudyx1 = (diu2(i - 1, j, k) + diu2(i - 1, j + 1, k) + diu2(i, j, k) + diu2(i, j + 1, k)) * L(.25);
          const T dudzx1 = (diu3(i - 1, j, k) + diu3(i - 1, j, k + 1) + diu3(i, j, k) + diu3(i, j, k + 1)) * L(.25);
          const T dvdxx1 = (diu4(i, j, k) + diu4(i, j - 1, k) + diu4(i + 1, j, k) + diu4(i + 1, j - 1, k)) * L(.25);
          const T dvdyx1 = diu5(i, j, k);
          const T dvdzx1 = (diu6(i, j - 1, k) + diu6(i, j - 1, k + 1) + diu6(i, j, k) + diu6(i, j, k + 1)) * L(.25);
          const T dwdxx1 = (diu7(i, j, k) + diu7(i, j, k - 1) + diu7(i + 1, j, k) + diu7(i + 1, j, k - 1)) * L(.25);
          const T dwdyx1 = (diu8(i, j, k) + diu8(i, j, k - 1) + diu8(i, j + 1, k) + diu8(i, j + 1, k - 1)) * L(.25);
          const T dwdzx1 = diu9(i, j, k);
          const T csx1 = cs0;
          const T cd = csx1 * delx1(k);
          const T s1 = dudyx1 + dvdxx1, s2 = dwdyx1 + dvdzx1, s3 = dudzx1 + dwdxx1;
          sm(i, j, k) = cd * cd *
                        std::sqrt(L(2.) * (dudxx1 * dudxx1 + dvdyx1 * dvdyx1 + dwdzx1 * dwdzx1) + s1 * s1 +
                                  s2 * s2 + s3 * s3);
        }
    boundsm();
    // x-component (les.f95:83-114)
    LES_REF_OMP_FOR
    for (int k = 2; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          const T evsx2 = sm(i + 1, j, k);
          const T evsx1 = sm(i, j, k);
          const T evsy2 = (dy1(j + 1) * ((dx1(i + 1) * sm(i, j, k) + dx1(i) * sm(i + 1, j, k)) / (dx1(i) + dx1(i + 1))) +
                           dy1(j) * ((dx1(i + 1) * sm(i, j + 1, k) + dx1(i) * sm(i + 1, j + 1, k)) / (dx1(i) + dx1(i + 1)))) /
                          (dy1(j) + dy1(j + 1));
          const T evsy1 = (dy1(j + 1) * ((dx1(i + 1) * sm(i, j - 1, k) + dx1(i) * sm(i + 1, j - 1, k)) / (dx1(i) + dx1(i + 1))) +
                           dy1(j) * ((dx1(i + 1) * sm(i, j, k) + dx1(i) * sm(i + 1, j, k)) / (dx1(i) + dx1(i + 1)))) /
                          (dy1(j) + dy1(j + 1));
          const T evsz2 = (dzn(k + 1) * ((dx1(i + 1) * sm(i, j, k) + dx1(i) * sm(i + 1, j, k)) / (dx1(i) + dx1(i + 1))) +
                           dzn(k) * ((dx1(i + 1) * sm(i, j, k + 1) + dx1(i) * sm(i + 1, j, k + 1)) / (dx1(i) + dx1(i + 1)))) /
                          (dzn(k) + dzn(k + 1));
          const T evsz1 = (dzn(k) * ((dx1(i + 1) * sm(i, j, k - 1) + dx1(i) * sm(i + 1, j, k - 1)) / (dx1(i) + dx1(i + 1))) +
                           dzn(k - 1) * ((dx1(i + 1) * sm(i, j, k) + dx1(i) * sm(i + 1, j, k)) / (dx1(i) + dx1(i + 1)))) /
                          (dzn(k - 1) + dzn(k));
          const T visux2 = (evsx2) * L(2.) * diu1(i + 1, j, k);
          const T visux1 = (evsx1) * L(2.) * diu1(i, j, k);
          const T visuy2 = (evsy2) * (diu2(i, j + 1, k) + diu4(i + 1, j, k));
          const T visuy1 = (evsy1) * (diu2(i, j, k) + diu4(i + 1, j - 1, k));
          const T visuz2 = (evsz2) * (diu3(i, j, k + 1) + diu7(i + 1, j, k));
          const T visuz1 = (evsz1) * (diu3(i, j, k) + diu7(i + 1, j, k - 1));
          const T vfu = (visux2 - visux1) / dxs(i) + (visuy2 - visuy1) / dy1(j) + (visuz2 - visuz1) / dzn(k);
          f(i, j, k) = (f(i, j, k) + vfu);
        }
    // x wall function (les.f95:118-139); the y and z terms are added twice, as written
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) {
        const T evsx2 = sm(i + 1, j, 1);
        const T evsx1 = sm(i, j, 1);
        const T evsy2 = (dy1(j + 1) * ((dx1(i + 1) * sm(i, j, 1) + dx1(i) * sm(i + 1, j, 1)) / (dx1(i) + dx1(i + 1))) +
                         dy1(j) * ((dx1(i + 1) * sm(i, j + 1, 1) + dx1(i) * sm(i + 1, j + 1, 1)) / (dx1(i) + dx1(i + 1)))) /
                        (dy1(j) + dy1(j + 1));
        const T evsy1 = (dy1(j + 1) * ((dx1(i + 1) * sm(i, j - 1, 1) + dx1(i) * sm(i + 1, j - 1, 1)) / (dx1(i) + dx1(i + 1))) +
                         dy1(j) * ((dx1(i + 1) * sm(i, j, 1) + dx1(i) * sm(i + 1, j, 1)) / (dx1(i) + dx1(i + 1)))) /
                        (dy1(j) + dy1(j + 1));
        const T evsz2 = (dzn(2) * ((dx1(i + 1) * sm(i, j, 1) + dx1(i) * sm(i + 1, j, 1)) / (dx1(i) + dx1(i + 1))) +
                         dzn(1) * ((dx1(i + 1) * sm(i, j, 2) + dx1(i) * sm(i + 1, j, 2)) / (dx1(i) + dx1(i + 1)))) /
                        (dzn(1) + dzn(2));
        const T visux2 = (evsx2) * L(2.) * diu1(i + 1, j, 1);
        const T visux1 = (evsx1) * L(2.) * diu1(i, j, 1);
        const T visuy2 = (evsy2) * (diu2(i, j + 1, 1) + diu4(i + 1, j, 1));
        const T visuy1 = (evsy1) * (diu2(i, j, 1) + diu4(i + 1, j - 1, 1));
        const T visuz2 = (evsz2) * (diu3(i, j, 2) + diu7(i + 1, j, 1));
        const T t = L(0.4) * uspd(i, j) / std::log(L(0.5) * dzn(1) / L(0.1));
        const T visuz1 = t * t * uspd(i, j);
        const T vfu = (visux2 - visux1) / dxs(i) + (visuy2 - visuy1) / dy1(j) + (visuz2 - visuz1) / dzn(1) +
                      (visuy2 - visuy1) / dy1(j) + (visuz2 - visuz1) / dzn(1);
        f(i, j, 1) = (f(i, j, 1) + vfu);
      }
    // y-component (les.f95:143-174)
    LES_REF_OMP_FOR
    for (int k = 2; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          const T evsy2 = sm(i, j + 1, k);
          const T evsy1 = sm(i, j, k);
          const T evsx2 = (dy1(j + 1) * ((dx1(i + 1) * sm(i, j, k) + dx1(i) * sm(i + 1, j, k)) / (dx1(i) + dx1(i + 1))) +
                           dy1(j) * ((dx1(i + 1) * sm(i, j + 1, k) + dx1(i) * sm(i + 1, j + 1, k)) / (dx1(i) + dx1(i + 1)))) /
                          (dy1(j) + dy1(j + 1));
          const T evsx1 = (dy1(j + 1) * ((dx1(i) * sm(i - 1, j, k) + dx1(i - 1) * sm(i, j, k)) / (dx1(i - 1) + dx1(i))) +
                           dy1(j) * ((dx1(i) * sm(i - 1, j + 1, k) + dx1(i - 1) * sm(i, j + 1, k)) / (dx1(i - 1) + dx1(i)))) /
                          (dy1(j) + dy1(j + 1));
          const T evsz2 = (dzn(k + 1) * ((dx1(i + 1) * sm(i, j, k) + dx1(i) * sm(i + 1, j, k)) / (dx1(i) + dx1(i + 1))) +
                           dzn(k) * ((dx1(i + 1) * sm(i, j, k + 1) + dx1(i) * sm(i + 1, j, k + 1)) / (dx1(i) + dx1(i + 1)))) /
                          (dzn(k) + dzn(k + 1));
          const T evsz1 = (dzn(k) * ((dx1(i + 1) * sm(i, j, k - 1) + dx1(i) * sm(i + 1, j, k - 1)) / (dx1(i) + dx1(i + 1))) +
                           dzn(k - 1) * ((dx1(i + 1) * sm(i, j, k) + dx1(i) * sm(i + 1, j, k)) / (dx1(i) + dx1(i + 1)))) /
                          (dzn(k - 1) + dzn(k));
          const T visvx2 = (evsx2) * (diu2(i, j + 1, k) + diu4(i + 1, j, k));
          const T visvx1 = (evsx1) * (diu2(i - 1, j + 1, k) + diu4(i, j, k));
          const T visvy2 = (evsy2) * L(2.) * diu5(i, j + 1, k);
          const T visvy1 = (evsy1) * L(2.) * diu5(i, j, k);
          const T visvz2 = (evsz2) * (diu6(i, j, k + 1) + diu8(i, j + 1, k));
          const T visvz1 = (evsz1) * (diu6(i, j, k) + diu8(i, j + 1, k - 1));
          const T vfv = (visvx2 - visvx1) / dx1(i) + (visvy2 - visvy1) / dys(j) + (visvz2 - visvz1) / dzn(k);
          g(i, j, k) = (g(i, j, k) + vfv);
        }
    // y wall function (les.f95:178-201)
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) {
        const T evsy2 = sm(i, j + 1, 1);
        const T evsy1 = sm(i, j, 1);
        const T evsx2 = (dy1(j + 1) * ((dx1(i + 1) * sm(i, j, 1) + dx1(i) * sm(i + 1, j, 1)) / (dx1(i) + dx1(i + 1))) +
                         dy1(j) * ((dx1(i + 1) * sm(i, j + 1, 1) + dx1(i) * sm(i + 1, j + 1, 1)) / (dx1(i) + dx1(i + 1)))) /
                        (dy1(j) + dy1(j + 1));
        const T evsx1 = (dy1(j + 1) * ((dx1(i) * sm(i - 1, j, 1) + dx1(i - 1) * sm(i, j, 1)) / (dx1(i - 1) + dx1(i))) +
                         dy1(j) * ((dx1(i) * sm(i - 1, j + 1, 1) + dx1(i - 1) * sm(i, j + 1, 1)) / (dx1(i - 1) + dx1(i)))) /
                        (dy1(j) + dy1(j + 1));
        const T evsz2 = (dzn(2) * ((dx1(i + 1) * sm(i, j, 1) + dx1(i) * sm(i + 1, j, 1)) / (dx1(i) + dx1(i + 1))) +
                         dzn(1) * ((dx1(i + 1) * sm(i, j, 2) + dx1(i) * sm(i + 1, j, 2)) / (dx1(i) + dx1(i + 1)))) /
                        (dzn(1) + dzn(2));
        const T visvx2 = (evsx2) * (diu2(i, j + 1, 1) + diu4(i + 1, j, 1));
        const T visvx1 = (evsx1) * (diu2(i - 1, j + 1, 1) + diu4(i, j, 1));
        const T visvy2 = (evsy2) * L(2.) * diu5(i, j + 1, 1);
        const T visvy1 = (evsy1) * L(2.) * diu5(i, j, 1);
        const T visvz2 = (evsz2) * (diu6(i, j, 2) + diu8(i, j + 1, 1));
        const T t = L(0.4) * vspd(i, j) / std::log(L(0.5) * dzn(1) / L(0.1));
        const T visvz1 = t * t * vspd(i, j);
        const T vfv = (visvx2 - visvx1) / dx1(i) + (visvy2 - visvy1) / dys(j) + (visvz2 - visvz1) / dzn(1);
        g(i, j, 1) = (g(i, j, 1) + vfv);
      }
    // z-component (les.f95:206-242)
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          const T evsz2 = sm(i, j, k + 1);
          const T evsz1 = sm(i, j, k);
          const T evsx2 = (dzn(k + 1) * ((dx1(i + 1) * sm(i, j, k) + dx1(i) * sm(i + 1, j, k)) / (dx1(i) + dx1(i + 1))) +
                           dzn(k) * ((dx1(i + 1) * sm(i, j, k + 1) + dx1(i) * sm(i + 1, j, k + 1)) / (dx1(i) + dx1(i + 1)))) /
                          (dzn(k) + dzn(k + 1));
          const T evsx1 = (dzn(k + 1) * ((dx1(i) * sm(i - 1, j, k) + dx1(i - 1) * sm(i, j, k)) / (dx1(i - 1) + dx1(i))) +
                           dzn(k) * ((dx1(i) * sm(i - 1, j, k + 1) + dx1(i - 1) * sm(i, j, k + 1)) / (dx1(i - 1) + dx1(i)))) /
                          (dzn(k) + dzn(k + 1));
          const T evsy2 = (dzn(k + 1) * ((dy1(j + 1) * sm(i, j, k) + dy1(j) * sm(i, j + 1, k)) / (dy1(j) + dy1(j + 1))) +
                           dzn(k) * ((dy1(j + 1) * sm(i, j, k + 1) + dy1(j) * sm(i, j + 1, k + 1)) / (dy1(j) + dy1(j + 1)))) /
                          (dzn(k) + dzn(k + 1));
          const T evsy1 = (dzn(k + 1) * ((dy1(j) * sm(i, j - 1, k) + dy1(j - 1) * sm(i, j, k)) / (dy1(j - 1) + dy1(j))) +
                           dzn(k) * ((dy1(j) * sm(i, j - 1, k + 1) + dy1(j - 1) * sm(i, j, k + 1)) / (dy1(j - 1) + dy1(j)))) /
                          (dzn(k) + dzn(k + 1));
          const T viswx2 = (evsx2) * (diu3(i, j, k + 1) + diu7(i + 1, j, k));
          const T viswx1 = (evsx1) * (diu3(i - 1, j, k + 1) + diu7(i, j, k));
          const T viswy2 = (evsy2) * (diu6(i, j, k + 1) + diu8(i, j + 1, k));
          const T viswy1 = (evsy1) * (diu6(i, j - 1, k + 1) + diu8(i, j, k));
          const T viswz2 = (evsz2) * L(2.) * diu9(i, j, k + 1);
          const T viswz1 = (evsz1) * L(2.) * diu9(i, j, k);
          const T vfw = (viswx2 - viswx1) / dx1(i) + (viswy2 - viswy1) / dy1(j) + (viswz2 - viswz1) / dzn(k);
          h(i, j, k) = (h(i, j, k) + vfw);
        }
  }

  // ---------------------------------------------------------------- adam.f95:30-44
  void adam() {
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          const T fd = f(i, j, k), gd = g(i, j, k), hd = h(i, j, k);
          f(i, j, k) = L(1.5) * f(i, j, k) - L(0.5) * fold(i, j, k);
          g(i, j, k) = L(1.5) * g(i, j, k) - L(0.5) * gold(i, j, k);
          h(i, j, k) = L(1.5) * h(i, j, k) - L(0.5) * hold(i, j, k);
          fold(i, j, k) = fd;
          gold(i, j, k) = gd;
          hold(i, j, k) = hd;
        }
  }

  // ---------------------------------------------------------------- bondFG.f95:18-42
  void bondfg() {
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j) f(0, j, k) = f(1, j, k);
    for (int k = 1; k <= km; ++k)
      for (int i = 1; i <= im; ++i) g(i, 0, k) = g(i, jm, k);
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) {
        h(i, j, 0) = L(0.0);
        h(i, j, km) = L(0.0);
      }
  }

  // ---------------------------------------------------------------- boundp.f95:7-78
  void boundp2() {
    for (int j = 0; j <= jm + 1; ++j)
      for (int i = 0; i <= im + 1; ++i) {
        p(i, j, 0) = p(i, j, 1);
        p(i, j, km + 1) = p(i, j, km);
      }
  }
  void boundp1() {
    for (int k = 0; k <= km + 1; ++k)
      for (int j = 0; j <= jm + 1; ++j) {
        p(0, j, k) = p(1, j, k);
        p(im + 1, j, k) = p(im, j, k);
      }
    for (int k = 0; k <= km + 1; ++k)
      for (int i = 0; i <= im + 1; ++i) {
        p(i, 0, k) = p(i, jm, k);
        p(i, jm + 1, k) = p(i, 1, k);
      }
  }

  // ---------------------------------------------------------------- press.f95:47-159
  // Sums run as sequential FP32 (the reference) or, with red64, sequential FP64 of
  // the same FP32 terms; the mean is then rounded back to FP32.
  void press() {
    bondfg();
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) {
          const T r = (-u(i - 1, j, k) + u(i, j, k)) / dx1(i) + (-v(i, j - 1, k) + v(i, j, k)) / dy1(j) +
                      (-w(i, j, k - 1) + w(i, j, k)) / dzn(k);
          rhs(i, j, k) = (f(i, j, k) - f(i - 1, j, k)) / dx1(i) + (g(i, j, k) - g(i, j - 1, k)) / dy1(j) +
                         (h(i, j, k) - h(i, j, k - 1)) / dzn(k) + r / dt;
        }
    T rhsav;
    {
      T s = L(0.0), a = L(0.0);
      double sd = 0.0, ad = 0.0;
      for (int k = 1; k <= km; ++k)
        for (int j = 1; j <= jm; ++j)
          for (int i = 1; i <= im; ++i) {
            const T term = dx1(i) * dy1(j) * dzn(k) * rhs(i, j, k);
            const T vol = dx1(i) * dy1(j) * dzn(k);
            if (red64) { sd += (double)term; ad += (double)vol; }
            else { s = s + term; a = a + vol; }
          }
      if (red64) { rhsav = (T)(sd / ad); last_area = ad; }
      else { rhsav = s / a; last_area = (double)a; }
    }
    last_rhsav = (double)rhsav;
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) rhs(i, j, k) = rhs(i, j, k) - rhsav;
    // red-black SOR (press.f95:89-122)
    int l;
    double sor_out = 0.0;
    for (l = 1; l <= nmaxp; ++l) {
      T sor = L(0.0);
      double sord = 0.0;
      for (int nrd = 0; nrd <= 1; ++nrd) {
#if defined(_OPENMP) && defined(LES_REF_PAR)
        std::vector<T> sk(km + 1, L(0.0));
        std::vector<double> sdk(km + 1, 0.0);
        LES_REF_OMP_FOR
        for (int k = 1; k <= km; ++k) {
          T s1 = L(0.0);
          double sd1 = 0.0;
          for (int j = 1; j <= jm; ++j)
            for (int i = 1 + (k + j + nrd) % 2; i <= im; i += 2) {
              const T reltmp = omega * (cn1(i, j, k) * (cn2l(i) * p(i + 1, j, k) + cn2s(i) * p(i - 1, j, k) +
                                                        cn3l(j) * p(i, j + 1, k) + cn3s(j) * p(i, j - 1, k) +
                                                        cn4l(k) * p(i, j, k + 1) + cn4s(k) * p(i, j, k - 1) -
                                                        rhs(i, j, k)) -
                                        p(i, j, k));
              p(i, j, k) = p(i, j, k) + reltmp;
              if (red64) sd1 += (double)(reltmp * reltmp);
              else s1 = s1 + reltmp * reltmp;
            }
          sk[k] = s1;
          sdk[k] = sd1;
        }
        for (int k = 1; k <= km; ++k) {
          sor = sor + sk[k];
          sord += sdk[k];
        }
#else
        for (int k = 1; k <= km; ++k)
          for (int j = 1; j <= jm; ++j)
            for (int i = 1 + (k + j + nrd) % 2; i <= im; i += 2) {
              const T reltmp = omega * (cn1(i, j, k) * (cn2l(i) * p(i + 1, j, k) + cn2s(i) * p(i - 1, j, k) +
                                                        cn3l(j) * p(i, j + 1, k) + cn3s(j) * p(i, j - 1, k) +
                                                        cn4l(k) * p(i, j, k + 1) + cn4s(k) * p(i, j, k - 1) -
                                                        rhs(i, j, k)) -
                                        p(i, j, k));
              p(i, j, k) = p(i, j, k) + reltmp;
              if (red64) sord += (double)(reltmp * reltmp);
              else sor = sor + reltmp * reltmp;
            }
#endif
        boundp1();
      }
      boundp2();
      sor_out = red64 ? sord : (double)sor;
      const bool conv = red64 ? (sord < (double)pjuge) : (sor < pjuge);
      if (!sor_fixed && conv) break;
    }
    last_iters = (l > nmaxp) ? nmaxp : l;
    last_sor = sor_out;
    T pav;
    {
      T s = L(0.0), c = L(0.0);
      double sd = 0.0, cd = 0.0;
      for (int k = 1; k <= km; ++k)
        for (int j = 1; j <= jm; ++j)
          for (int i = 1; i <= im; ++i) {
            const T term = p(i, j, k) * dx1(i) * dy1(j) * dzn(k);
            const T vol = dx1(i) * dy1(j) * dzn(k);
            if (red64) { sd += (double)term; cd += (double)vol; }
            else { s = s + term; c = c + vol; }
          }
      if (red64) { pav = (T)(sd / cd); last_pco = cd; }
      else { pav = s / c; last_pco = (double)c; }
    }
    last_pav = (double)pav;
    LES_REF_OMP_FOR
    for (int k = 1; k <= km; ++k)
      for (int j = 1; j <= jm; ++j)
        for (int i = 1; i <= im; ++i) p(i, j, k) = p(i, j, k) - pav;
    boundp1();
    boundp2();
  }

  void step(int n, int nmax) {
    (void)nmax;
    velnw();
    bondv1(n);
    velfg();
    feedbf();
    les();
    adam();
    press();
  }

  // ---------------------------------------------------------------- aveflow.f95:5-200
  // Time averages of v, p, u, w, of the squares of u, v, w, sm, of sm and of the u-w
  // flux from step n1 on, finalised at n == nmax (the unformatted writes of
  // :200-350 are the host's: the arrays are read back instead).  x**2 is x*x.
  void aveflow(int n, int n1, int nmax) {
    if (!ave_alloc) {
      const int ip = im, jp = jm, kp = km;
      aveu.alloc("aveu", 1, ip, 1, jp, 0, kp); avev.alloc("avev", 1, ip, 1, jp, 0, kp);
      avew.alloc("avew", 1, ip + 1, 1, jp, 0, kp + 2);
      avep.alloc("avep", 1, ip, 1, jp, 1, kp); avel.alloc("avel", 1, ip, 1, jp, 1, kp);
      aveuu.alloc("aveuu", 1, ip, 1, jp, 1, kp); avevv.alloc("avevv", 1, ip, 1, jp, 1, kp);
      aveww.alloc("aveww", 1, ip, 1, jp, 1, kp); avesm.alloc("avesm", 1, ip, 1, jp, 1, kp);
      avesmsm.alloc("avesmsm", 1, ip, 1, jp, 1, kp); uwfx.alloc("uwfx", 1, ip, 1, jp, 1, kp);
      ave_alloc = true;
    }
    if (n == n1) {  // :82-114
      for (int k = 1; k <= km; ++k)
        for (int j = 1; j <= jm; ++j)
          for (int i = 1; i <= im; ++i) {
            avev(i, j, k) = L(0.0); avep(i, j, k) = L(0.0); avel(i, j, k) = L(0.0);
            aveuu(i, j, k) = L(0.0); avevv(i, j, k) = L(0.0); aveww(i, j, k) = L(0.0);
            avesm(i, j, k) = L(0.0); avesmsm(i, j, k) = L(0.0); uwfx(i, j, k) = L(0.0);
          }
      for (int k = 0; k <= km; ++k)
        for (int j = 1; j <= jm; ++j)
          for (int i = 1; i <= im; ++i) aveu(i, j, k) = L(0.0);
      for (int k = 0; k <= km; ++k)
        for (int j = 1; j <= jm; ++j)
          for (int i = 1; i <= im + 1; ++i) avew(i, j, k) = L(0.0);
    }
    if (n >= n1) {  // :117-149
      for (int k = 1; k <= km; ++k)
        for (int j = 1; j <= jm; ++j)
          for (int i = 1; i <= im; ++i) {
            avev(i, j, k) = avev(i, j, k) + v(i, j, k);
            avep(i, j, k) = avep(i, j, k) + p(i, j, k);
            aveuu(i, j, k) = aveuu(i, j, k) + u(i, j, k) * u(i, j, k);
            avevv(i, j, k) = avevv(i, j, k) + v(i, j, k) * v(i, j, k);
            aveww(i, j, k) = aveww(i, j, k) + w(i, j, k) * w(i, j, k);
            avesm(i, j, k) = avesm(i, j, k) + sm(i, j, k);
            avesmsm(i, j, k) = avesmsm(i, j, k) + sm(i, j, k) * sm(i, j, k);
            uwfx(i, j, k) = uwfx(i, j, k) + L(0.5) * (u(i, j, k - 1) + u(i, j, k)) * L(0.5) *
                                                (w(i, j, k - 1) + w(i + 1, j, k - 1));
          }
      for (int k = 0; k <= km; ++k)
        for (int j = 1; j <= jm; ++j)
          for (int i = 1; i <= im; ++i) aveu(i, j, k) = aveu(i, j, k) + u(i, j, k);
      for (int k = 0; k <= km; ++k)
        for (int j = 1; j <= jm; ++j)
          for (int i = 1; i <= im + 1; ++i) avew(i, j, k) = avew(i, j, k) + w(i, j, k);
    }
    if (n == nmax) {  // :151-200
      const T cnt = (T)(nmax - n1 + 1);  // float(nmax-n1+1)
      for (int k = 1; k <= km; ++k)
        for (int j = 1; j <= jm; ++j)
          for (int i = 1; i <= im; ++i) {
            avev(i, j, k) = avev(i, j, k) / cnt; avep(i, j, k) = avep(i, j, k) / cnt;
            avel(i, j, k) = avel(i, j, k) / cnt; aveuu(i, j, k) = aveuu(i, j, k) / cnt;
            avevv(i, j, k) = avevv(i, j, k) / cnt; aveww(i, j, k) = aveww(i, j, k) / cnt;
            avesm(i, j, k) = avesm(i, j, k) / cnt; avesmsm(i, j, k) = avesmsm(i, j, k) / cnt;
          }
      for (int k = 0; k <= km; ++k)
        for (int j = 1; j <= jm; ++j)
          for (int i = 1; i <= im; ++i) aveu(i, j, k) = aveu(i, j, k) / cnt;
      for (int k = 0; k <= km; ++k)
        for (int j = 1; j <= jm; ++j)
          for (int i = 1; i <= im + 1; ++i) avew(i, j, k) = avew(i, j, k) / cnt;
      for (int k = 1; k <= km; ++k)
        for (int j = 1; j <= jm; ++j)
          for (int i = 1; i <= im; ++i)
            uwfx(i, j, k) = uwfx(i, j, k) / cnt - L(0.5) * (aveu(i, j, k - 1) + aveu(i, j, k)) * L(0.5) *
                                                      (avew(i, j, k - 1) + avew(i + 1, j, k - 1));
      for (int k = 1; k <= km; ++k)
        for (int j = 1; j <= jm; ++j)
          for (int i = 1; i <= im; ++i) {
            aveuu(i, j, k) = std::sqrt(std::abs(aveuu(i, j, k) - aveu(i, j, k) * aveu(i, j, k)));
            avevv(i, j, k) = std::sqrt(std::abs(avevv(i, j, k) - avev(i, j, k) * avev(i, j, k)));
            aveww(i, j, k) = std::sqrt(std::abs(aveww(i, j, k) - avew(i, j, k) * avew(i, j, k)));
          }
    }
  }

  FA<T> *field(int id) {
    switch (id) {
      case 1: return &u; case 2: return &v; case 3: return &w; case 4: return &p;
      case 5: return &f; case 6: return &g; case 7: return &h;
      case 8: return &fold; case 9: return &gold; case 10: return &hold;
      case 11: return &usum; case 12: return &vsum; case 13: return &wsum;
      case 14: return &rhs; case 15: return &sm;
      case 16: return &bmask1; case 17: return &cmask1; case 18: return &dmask1;
      case 19: return &amask1; case 20: return &cn1;
      case 32: return &dx1; case 33: return &dy1; case 34: return &dzn; case 35: return &dzs;
      case 36: return &dxs; case 37: return &dys; case 38: return &z2;
      case 39: return &cn2l; case 40: return &cn2s; case 41: return &cn3l; case 42: return &cn3s;
      case 43: return &cn4l; case 44: return &cn4s; case 45: return &delx1;
      case 46: return &dxl; case 47: return &dyl;
      case 50: return &uspd; case 51: return &vspd; case 52: return &zbm;
      case 90: return &fx; case 91: return &fy; case 92: return &fz;
      case 93: return &dfu1; case 94: return &dfv1; case 95: return &dfw1;
      default: break;
    }
    if (ave_alloc) {  // aveflow arrays (product ids LES_FIELD_AVEU..LES_FIELD_UWFX)
      switch (id) {
        case 100: return &aveu; case 101: return &avev; case 102: return &avew; case 103: return &avep;
        case 104: return &avel; case 105: return &aveuu; case 106: return &avevv; case 107: return &aveww;
        case 108: return &avesm; case 109: return &avesmsm; case 110: return &uwfx;
        default: break;
      }
    }
    if (id >= 60 && id <= 68) return &diu[id - 59];
    if (id >= 70 && id <= 78) return &cov[id - 69];
    if (id >= 80 && id <= 88) return &nou[id - 79];
    return nullptr;
  }
};

struct Handle {
  int prec;
  Ref<float> *f32 = nullptr;
  Ref<double> *f64 = nullptr;
};

template <class T>
Ref<T> *make(int im, int jm, int km, const double *c, const int *o, const float *zbm,
             const float *uin, const float *vin, const float *win) {
  Ref<T> *r = new Ref<T>();
  r->im = im; r->jm = jm; r->km = km;
  r->nmaxp = o[REF_OPT_NMAXP]; r->sor_fixed = o[REF_OPT_SOR_FIXED]; r->red64 = o[REF_OPT_RED64];
  r->sqrt_half = o[REF_OPT_SQRT_HALF]; r->dz_law = o[REF_OPT_DZ_LAW];
  // set.f95:89-95 values arrive through consts[] (dt, ro, vn, alpha, beta); press.f95:43-45
  // omega and pjuge likewise.  Values are rounded to T as gfortran rounds literals.
  r->dt = (T)c[REF_C_DT]; r->ro = (T)c[REF_C_RO]; r->vn = (T)c[REF_C_VN];
  r->alpha = (T)c[REF_C_ALPHA]; r->beta = (T)c[REF_C_BETA]; r->omega = (T)c[REF_C_OMEGA];
  r->pjuge = (T)c[REF_C_PJUGE];
  r->cdx = (T)c[REF_C_DX]; r->cdy = (T)c[REF_C_DY]; r->dz0 = (T)c[REF_C_DZ0];
  r->dzratio = (T)c[REF_C_DZRATIO];
  r->allocate();
  for (int j = 1; j <= jm; ++j)
    for (int i = 1; i <= im; ++i) r->zbm(i, j) = (T)zbm[(i - 1) + (size_t)(j - 1) * im];
  for (int k = 1; k <= km; ++k)
    for (int j = 1; j <= jm; ++j) {
      const size_t q = (j - 1) + (size_t)(k - 1) * jm;
      r->uin(j, k) = (T)uin[q]; r->vin(j, k) = (T)vin[q]; r->win(j, k) = (T)win[q];
    }
  r->grid();
  r->init();
  return r;
}

template <class T>
int stage(Ref<T> *r, int s, int n, int nmax) {
  switch (s) {
    case REF_STEP: r->step(n, nmax); break;
    case REF_VELNW: r->velnw(); break;
    case REF_BONDV1: r->bondv1(n); break;
    case REF_VELFG: r->velfg(); break;
    case REF_FEEDBF: r->feedbf(); break;
    case REF_LES: r->les(); break;
    case REF_ADAM: r->adam(); break;
    case REF_PRESS: r->press(); break;
    case REF_BOUNDP1: r->boundp1(); break;
    case REF_BOUNDP2: r->boundp2(); break;
    case REF_BONDFG: r->bondfg(); break;
    default: g_err = "unknown stage"; return -1;
  }
  return 0;
}

template <class T>
int copy_field(Ref<T> *r, int id, double *buf, const int *lb, const int *ub, bool out) {
  FA<T> *a = r->field(id);
  if (!a) { g_err = "unknown field id"; return -1; }
  const int rank3 = 1;
  (void)rank3;
  if (lb[0] < a->l0 || ub[0] > a->u0 || lb[1] < a->l1 || ub[1] > a->u1 || lb[2] < a->l2 || ub[2] > a->u2) {
    g_err = std::string("requested extents exceed the declared extents of ") + a->name;
    return -2;
  }
  size_t q = 0;
  for (int k = lb[2]; k <= ub[2]; ++k)
    for (int j = lb[1]; j <= ub[1]; ++j)
      for (int i = lb[0]; i <= ub[0]; ++i, ++q) {
        if (out) buf[q] = (double)(*a)(i, j, k);
        else (*a)(i, j, k) = (T)buf[q];
      }
  return 0;
}

}  // namespace

extern "C" {

void *ref_create(int prec, int im, int jm, int km, const double *consts, const int *opts,
                 const float *zbm, const float *uin, const float *vin, const float *win) {
  try {
    if (im < 3 || jm < 2 || km < 3) { g_err = "ref_create: need im>=3, jm>=2, km>=3"; return nullptr; }
    Handle *h = new Handle();
    h->prec = prec;
    if (prec == 8) h->f64 = make<double>(im, jm, km, consts, opts, zbm, uin, vin, win);
    else h->f32 = make<float>(im, jm, km, consts, opts, zbm, uin, vin, win);
    return h;
  } catch (const RefError &e) {
    g_err = e.msg;
  } catch (const std::exception &e) {
    g_err = e.what();
  }
  return nullptr;
}

void ref_destroy(void *hv) {
  Handle *h = (Handle *)hv;
  if (!h) return;
  delete h->f32;
  delete h->f64;
  delete h;
}

int ref_stage(void *hv, int s, int n, int nmax) {
  Handle *h = (Handle *)hv;
  try {
    return h->f64 ? stage(h->f64, s, n, nmax) : stage(h->f32, s, n, nmax);
  } catch (const RefError &e) {
    g_err = e.msg;
  } catch (const std::exception &e) {
    g_err = e.what();
  }
  return -3;
}

int ref_aveflow(void *hv, int n, int n1, int nmax) {
  Handle *h = (Handle *)hv;
  try {
    if (h->f64) h->f64->aveflow(n, n1, nmax);
    else h->f32->aveflow(n, n1, nmax);
    return 0;
  } catch (const RefError &e) {
    g_err = e.msg;
  } catch (const std::exception &e) {
    g_err = e.what();
  }
  return -3;
}

int ref_get(void *hv, int field, double *out, const int *lb, const int *ub) {
  Handle *h = (Handle *)hv;
  return h->f64 ? copy_field(h->f64, field, out, lb, ub, true) : copy_field(h->f32, field, out, lb, ub, true);
}

int ref_set(void *hv, int field, const double *in, const int *lb, const int *ub) {
  Handle *h = (Handle *)hv;
  double *b = const_cast<double *>(in);
  return h->f64 ? copy_field(h->f64, field, b, lb, ub, false) : copy_field(h->f32, field, b, lb, ub, false);
}

int ref_extents(void *hv, int field, int *lb, int *ub) {
  Handle *h = (Handle *)hv;
  auto fill = [&](auto *r) -> int {
    auto *a = r->field(field);
    if (!a) return -1;
    lb[0] = a->l0; ub[0] = a->u0; lb[1] = a->l1; ub[1] = a->u1; lb[2] = a->l2; ub[2] = a->u2;
    return 0;
  };
  return h->f64 ? fill(h->f64) : fill(h->f32);
}

void ref_diag(void *hv, double *out) {
  Handle *h = (Handle *)hv;
  auto fill = [&](auto *r) {
    out[0] = r->last_iters; out[1] = r->last_sor; out[2] = r->last_uout; out[3] = r->last_rhsav;
    out[4] = r->last_pav; out[5] = r->last_area; out[6] = r->last_pco;
  };
  if (h->f64) fill(h->f64);
  else fill(h->f32);
}

int ref_bounds_checked(void) {
#ifdef LES_REF_CHECK
  return 1;
#else
  return 0;
#endif
}

const char *ref_last_error(void) { return g_err.c_str(); }

int ref_trap_wall(void *hv, int on) {
  Handle *h = (Handle *)hv;
  if (!h) return -1;
  if (h->f64) h->f64->trap_wall = on != 0;
  else h->f32->trap_wall = on != 0;
  return 0;
}

/* The configs' seeded synthetic scenario, restated here so that the checker and the
 * timed CPU baseline need nothing from the product.  Inputs: fl[] = {dz0, dz_ratio,
 * coverage, h_min, h_max, u_ref, z_ref, pl_exp, direction_deg, noise} (FP32 values, as
 * the product's les_scenario holds them), in[] = {dz_law, fp_min, fp_max, inflow_law}.
 * Heightmap: rectangular blocks, footprint sides uniform in [fp_min, fp_max] cells,
 * heights uniform in [h_min, h_max] m, drawn with SplitMix64 (Steele, Lea, Flood,
 * OOPSLA 2014) until the plan coverage is met, i within [max(3,im/8), im-max(3,im/8)],
 * j periodic.  Inflow planes (1:jm,1:km): U(z) = u_ref (z/z_ref)^pl_exp at z =
 * z2(k) + 0.5 dzn(k) (bondv1.f95:36's height; inflow_law 0: the reference's 5 m/s),
 * turned by the residual of the direction after whole quarter turns, r in [-45, 45)
 * degrees: (u, v) = U (cos r, sin r), plus a fixed uniform +-noise per cell and
 * component.  z2 and dzn are the FP32 grid of grid.f95:114-135 (dz_law 0) or the
 * geometric law (dz_law 1), as ref_create builds them. */
int ref_scenario(int im, int jm, int km, const float *fl, const int *in, unsigned long long seed, float *zbm,
                 float *uin, float *vin, float *win) {
  if (im < 3 || jm < 2 || km < 3 || !fl || !in || !zbm || !uin || !vin || !win) {
    g_err = "ref_scenario: bad arguments";
    return -1;
  }
  const float dz0 = fl[0], dzr = fl[1], coverage = fl[2], h_min = fl[3], h_max = fl[4], u_ref = fl[5];
  const float z_ref = fl[6], pl_exp = fl[7], direction = fl[8], noise = fl[9];
  const int dz_law = in[0], fp_min = in[1], fp_max = in[2], inflow_law = in[3];
  // vertical grid in FP32 (the same loops as Ref<float>::grid)
  std::vector<float> dzn(km + 4, 0.f), z2(km + 3, 0.f);  // dzn(k) at [k+1], z2(k) at [k]
  if (dz_law == 0) {
    if (km < 58) { g_err = "ref_scenario: the reference dz law needs km >= 58"; return -1; }
    z2[0] = 1.f; dzn[1] = 1.f; z2[1] = 1.f; dzn[2] = 1.f;
    for (int k = 2; k <= 15; ++k) dzn[k + 1] = dzn[k] * 1.1f;
    for (int k = 16; k <= 44; ++k) dzn[k + 1] = 4.f;
    for (int k = 45; k <= 58; ++k) dzn[k + 1] = dzn[k] * 1.1f;
    for (int k = 59; k <= km + 1; ++k) dzn[k + 1] = 16.f;
  } else {
    z2[0] = dz0; dzn[1] = dz0; z2[1] = dz0; dzn[2] = dz0;
    for (int k = 2; k <= km + 1; ++k) dzn[k + 1] = dzn[k] * dzr;
  }
  for (int k = 2; k <= km + 2; ++k) z2[k] = z2[k - 1] + dzn[k + 1];
  dzn[km + 2] = dzn[km + 1];
  // SplitMix64 stream
  uint64_t st = (uint64_t)seed ^ 0x4c45535f47423330ull;
  auto next = [&]() {
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  auto uni = [&]() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); };
  auto irange = [&](int a, int b) { return a + (int)(uni() * (double)(b - a + 1)); };
  for (size_t q = 0; q < (size_t)im * jm; ++q) zbm[q] = 0.f;
  if (coverage > 0.f) {
    const int edge = im / 8 > 3 ? im / 8 : 3;
    const int ilo = edge, ihi = im - edge;
    const int fpmin = fp_min > 1 ? fp_min : 1, fpmax = fp_max > fpmin ? fp_max : fpmin;
    const long target = (long)std::ceil((double)coverage * im * jm);
    long covered = 0;
    for (int tries = 0; tries < 200000 && covered < target; ++tries) {
      int wx = irange(fpmin, fpmax);
      const int span = ihi - ilo > 1 ? ihi - ilo : 1;
      if (wx > span) wx = span;
      int wy = irange(fpmin, fpmax);
      if (wy > jm) wy = jm;
      const int i0 = irange(ilo, ihi - wx > ilo ? ihi - wx : ilo);
      const int j0 = irange(1, jm);
      const float ht = (float)(h_min + (h_max - h_min) * uni());
      for (int jj = 0; jj < wy; ++jj)
        for (int ii = 0; ii < wx; ++ii) {
          const int i = i0 + ii, j = 1 + (j0 - 1 + jj) % jm;
          if (i > ihi) continue;
          float &z = zbm[(size_t)(i - 1) + (size_t)(j - 1) * im];
          if (z <= 0.f) ++covered;
          if (ht > z) z = ht;
        }
    }
  }
  double deg = std::fmod((double)direction, 360.0);
  if (deg < 0) deg += 360.0;
  const double r = deg - 90.0 * std::floor((deg + 45.0) / 90.0);
  const double rr = r * 3.14159265358979323846 / 180.0;
  const double cr = std::cos(rr), sr = std::sin(rr);
  for (int k = 1; k <= km; ++k) {
    double U = 5.0;  // bondv1.f95:33-54: 5 m/s (u(k>=79) = u(77) is 5 as well)
    if (inflow_law != 0) {
      const double z = (double)z2[k] + 0.5 * (double)dzn[k + 1];
      U = (double)u_ref * std::pow(z / (double)z_ref, (double)pl_exp);
    }
    for (int j = 1; j <= jm; ++j) {
      const size_t q = (size_t)(j - 1) + (size_t)(k - 1) * jm;
      const double nu = noise * (2.0 * uni() - 1.0);
      const double nv = noise * (2.0 * uni() - 1.0);
      const double nw = noise * (2.0 * uni() - 1.0);
      uin[q] = (float)(U * cr + nu);
      vin[q] = (float)(U * sr + nv);
      win[q] = (float)nw;
    }
  }
  return 0;
}

int ref_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

}  // extern "C"
