/*
 * vlct_oracle.cpp -- TEST INFRASTRUCTURE ONLY (see vlct_oracle.h).
 *
 * A CPU restatement of Enzo-E's VL+CT MHD step.  It follows the reference's
 * dataflow array pass by array pass, with the same index windows and the same
 * floating-point operation order, so that compiled with -O2
 * -ffp-contract=off it reproduces the reference bit for bit.  Every function
 * names the reference file:line it restates (paths relative to the Enzo-E
 * source tree).  No code here is shared with the CUDA product.
 */
#include "vlct_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

namespace {

/* ------------------------------------------------------------------------ */
/* Arrays                                                                   */
/* ------------------------------------------------------------------------ */

struct V3 {  // non-owning (z, y, x) view, x fastest
  double* p = nullptr;
  int n[3] = {0, 0, 0};  // extent along x, y, z
  double& at(int x, int y, int z) const {
    return p[((size_t)z * n[1] + y) * n[0] + x];
  }
  double& c(const int i[3]) const { return at(i[0], i[1], i[2]); }
};

struct A3 {  // owning array
  std::vector<double> v;
  V3 w;
  void alloc(int nx, int ny, int nz) {
    v.assign((size_t)nx * ny * nz, 0.0);
    w.p = v.data();
    w.n[0] = nx; w.n[1] = ny; w.n[2] = nz;
  }
};

inline V3 view(double* p, int nx, int ny, int nz) {
  V3 a; a.p = p; a.n[0] = nx; a.n[1] = ny; a.n[2] = nz; return a;
}

// loop over the box [lo, hi) (per axis), z outer, x inner
template <class F>
inline void box(const int lo[3], const int hi[3], F f) {
  int i[3];
  for (i[2] = lo[2]; i[2] < hi[2]; i[2]++)
    for (i[1] = lo[1]; i[1] < hi[1]; i[1]++)
      for (i[0] = lo[0]; i[0] < hi[0]; i[0]++) f(i);
}

/* ------------------------------------------------------------------------ */
/* Small helpers restating src/Enzo/utils/utils.hpp                         */
/* ------------------------------------------------------------------------ */

// enzo_utils::min (utils.hpp:82-89)
inline double min3(double a, double b, double c) {
  if (a < b) return (c < a) ? c : a;
  return (c < b) ? c : b;
}
// std::max / std::min semantics (first argument returned on ties)
inline double smax(double a, double b) { return (a < b) ? b : a; }
inline double smin(double a, double b) { return (b < a) ? b : a; }
// enzo_utils::apply_floor (utils.hpp:102-114) == std::max(value, floor)
inline double apply_floor(double v, double f) { return smax(v, f); }
// enzo_utils::squared_mag_vec3D (utils.hpp:71-74)
inline double sqmag(double i, double j, double k) {
  return ((i * i) + ((j * j) + (k * k)));
}
// sign() used by the PLM limiter (EnzoReconstructorPLM.hpp:253)
inline double sgn(double v) { return (double)((0.0 < v) - (v < 0.0)); }

/* ------------------------------------------------------------------------ */
/* Primitive / LUT ordering.  The reference's MHD primitive keys are          */
/* {density, bfield_x,y,z, velocity_x,y,z, pressure} (EnzoRiemannImpl.hpp:    */
/* 45-53 via get_quantity_keys, EnzoRiemannUtils.hpp:191-215).  Hydro drops   */
/* the bfield entries; we keep one 8-slot layout for both.                    */
/* ------------------------------------------------------------------------ */
enum { Q_RHO = 0, Q_BX = 1, Q_BY = 2, Q_BZ = 3, Q_VX = 4, Q_VY = 5, Q_VZ = 6,
       Q_P = 7, NQ = 8 };

struct Ctx {
  const OracleParams* prm;
  int m[3];  // ghosted cell extent along x, y, z
  bool mhd, de;
  double gamma;
  bool gravity = false;  // acceleration fields present
  V3 accel[3];
};

/* ------------------------------------------------------------------------ */
/* EOS (src/Enzo/fluid-props/EnzoEOSIdeal.hpp:58-140)                        */
/* ------------------------------------------------------------------------ */
inline double eos_cs2(double g, double d, double p) { return g * p / d; }
inline double eos_sound_speed(double g, double d, double p) {
  return std::sqrt(eos_cs2(g, d, p));
}
inline double eos_specific_eint(double g, double d, double p) {
  return p / ((g - 1.0) * d);
}
inline double eos_eint_dens(double g, double /*d*/, double p) {
  return p / (g - 1.0);
}
// fast_magnetosonic_speed<-1> (EnzoEOSIdeal.hpp:111-140, generic branch)
inline double eos_cfast(double g, double d, double p, double bi, double bj,
                        double bk) {
  const double B2 = sqmag(bi, bj, bk);
  const double cs2 = eos_cs2(g, d, p);
  const double inv_density = 1.0 / d;
  const double va2 = B2 * inv_density;
  const double va2_cos2 = (bi * bi) * inv_density;
  const double s = cs2 + va2;
  return std::sqrt(0.5 * (va2 + cs2 + std::sqrt(s * s - 4. * cs2 * va2_cos2)));
}
// fast_magnetosonic_speed<0> (EnzoEOSIdeal.hpp:124-126)
inline double eos_cfast0(double g, double d, double p, double bi, double bj,
                         double bk) {
  const double B2 = sqmag(bi, bj, bk);
  const double cs2 = eos_cs2(g, d, p);
  const double va2 = B2 / d;
  return std::sqrt(va2 + cs2);
}

/* ------------------------------------------------------------------------ */
/* Riemann solvers.  Inputs wl/wr hold the 8 primitives in LUT order         */
/* {rho, b_i, b_j, b_k, v_i, v_j, v_k, p} (already permuted to the face's     */
/* i,j,k frame); outputs are the 8 fluxes in the same frame plus the         */
/* internal-energy flux and the interface velocity v_i-bar.                  */
/* ------------------------------------------------------------------------ */
enum { L_RHO = 0, L_BI = 1, L_BJ = 2, L_BK = 3, L_VI = 4, L_VJ = 5, L_VK = 6,
       L_E = 7 };

// enzo_riemann_utils::passive_eint_flux (EnzoRiemannUtils.hpp:224-249)
inline double passive_eint_flux(double g, double dl, double pl, double dr,
                                double pr, double density_flux) {
  const double el = eos_specific_eint(g, dl, pl);
  const double er = eos_specific_eint(g, dr, pr);
  const double upwind = (double)(density_flux > 0) * el +
                        (double)(density_flux <= 0) * er;
  return upwind * density_flux;
}

// HLLD (riemann/EnzoRiemannHLLD.hpp:40-448)
void hlld(double g, const double* wli, const double* wri, double* flx,
          double* eflux, double* vbar) {
  const double SMALL = 1.0e-8;
  const double igm1 = 1.0 / (g - 1.0);
  struct C { double d, mx, my, mz, e, by, bz; };
  C ul, ur, ulst, uldst, urdst, urst, fl, fr;
  double spd[5];
  const double pressure_l = wli[L_E], pressure_r = wri[L_E];
  const double bxi = wli[L_BI];
  double bxsq = bxi * bxi;
  double pbl = 0.5 * (bxsq + (wli[L_BJ] * wli[L_BJ] + wli[L_BK] * wli[L_BK]));
  double pbr = 0.5 * (bxsq + (wri[L_BJ] * wri[L_BJ] + wri[L_BK] * wri[L_BK]));
  double kel = 0.5 * wli[L_RHO] *
               (wli[L_VI] * wli[L_VI] +
                (wli[L_VJ] * wli[L_VJ] + wli[L_VK] * wli[L_VK]));
  double ker = 0.5 * wri[L_RHO] *
               (wri[L_VI] * wri[L_VI] +
                (wri[L_VJ] * wri[L_VJ] + wri[L_VK] * wri[L_VK]));
  ul.d = wli[L_RHO];
  ul.mx = wli[L_VI] * ul.d;
  ul.my = wli[L_VJ] * ul.d;
  ul.mz = wli[L_VK] * ul.d;
  ul.e = pressure_l * igm1 + kel + pbl;
  ul.by = wli[L_BJ];
  ul.bz = wli[L_BK];
  ur.d = wri[L_RHO];
  ur.mx = wri[L_VI] * ur.d;
  ur.my = wri[L_VJ] * ur.d;
  ur.mz = wri[L_VK] * ur.d;
  ur.e = pressure_r * igm1 + ker + pbr;
  ur.by = wri[L_BJ];
  ur.bz = wri[L_BK];

  double cfl = eos_cfast(g, wli[L_RHO], pressure_l, wli[L_BI], wli[L_BJ],
                         wli[L_BK]);
  double cfr = eos_cfast(g, wri[L_RHO], pressure_r, wri[L_BI], wri[L_BJ],
                         wri[L_BK]);
  spd[0] = smin(wli[L_VI] - cfl, wri[L_VI] - cfr);
  spd[4] = smax(wli[L_VI] + cfl, wri[L_VI] + cfr);

  double ptl = pressure_l + pbl;
  double ptr = pressure_r + pbr;
  fl.d = ul.mx;
  fl.mx = ul.mx * wli[L_VI] + ptl - bxsq;
  fl.my = ul.my * wli[L_VI] - bxi * ul.by;
  fl.mz = ul.mz * wli[L_VI] - bxi * ul.bz;
  fl.e = wli[L_VI] * (ul.e + ptl - bxsq) -
         bxi * (wli[L_VJ] * ul.by + wli[L_VK] * ul.bz);
  fl.by = ul.by * wli[L_VI] - bxi * wli[L_VJ];
  fl.bz = ul.bz * wli[L_VI] - bxi * wli[L_VK];
  fr.d = ur.mx;
  fr.mx = ur.mx * wri[L_VI] + ptr - bxsq;
  fr.my = ur.my * wri[L_VI] - bxi * ur.by;
  fr.mz = ur.mz * wri[L_VI] - bxi * ur.bz;
  fr.e = wri[L_VI] * (ur.e + ptr - bxsq) -
         bxi * (wri[L_VJ] * ur.by + wri[L_VK] * ur.bz);
  fr.by = ur.by * wri[L_VI] - bxi * wri[L_VJ];
  fr.bz = ur.bz * wri[L_VI] - bxi * wri[L_VK];

  double sdl = spd[0] - wli[L_VI];
  double sdr = spd[4] - wri[L_VI];
  spd[2] = (sdr * ur.mx - sdl * ul.mx + (ptl - ptr)) / (sdr * ur.d - sdl * ul.d);
  double sdml = spd[0] - spd[2];
  double sdmr = spd[4] - spd[2];
  double sdml_inv = 1.0 / sdml;
  double sdmr_inv = 1.0 / sdmr;
  ulst.d = ul.d * sdl * sdml_inv;
  urst.d = ur.d * sdr * sdmr_inv;
  double ulst_d_inv = 1.0 / ulst.d;
  double urst_d_inv = 1.0 / urst.d;
  double sqrtdl = std::sqrt(ulst.d);
  double sqrtdr = std::sqrt(urst.d);
  spd[1] = spd[2] - std::fabs(bxi) / sqrtdl;
  spd[3] = spd[2] + std::fabs(bxi) / sqrtdr;

  double ptstl = ptl + ul.d * sdl * (spd[2] - wli[L_VI]);
  double ptstr = ptr + ur.d * sdr * (spd[2] - wri[L_VI]);
  double ptst = 0.5 * (ptstr + ptstl);

  ulst.mx = ulst.d * spd[2];
  if (std::fabs(ul.d * sdl * sdml - bxsq) < SMALL * ptst) {
    ulst.my = ulst.d * wli[L_VJ];
    ulst.mz = ulst.d * wli[L_VK];
    ulst.by = ul.by;
    ulst.bz = ul.bz;
  } else {
    double tmp = bxi * (sdl - sdml) / (ul.d * sdl * sdml - bxsq);
    ulst.my = ulst.d * (wli[L_VJ] - ul.by * tmp);
    ulst.mz = ulst.d * (wli[L_VK] - ul.bz * tmp);
    tmp = (ul.d * (sdl * sdl) - bxsq) / (ul.d * sdl * sdml - bxsq);
    ulst.by = ul.by * tmp;
    ulst.bz = ul.bz * tmp;
  }
  double vbstl = (ulst.mx * bxi + (ulst.my * ulst.by + ulst.mz * ulst.bz)) *
                 ulst_d_inv;
  ulst.e = (sdl * ul.e - ptl * wli[L_VI] + ptst * spd[2] +
            bxi * (wli[L_VI] * bxi + (wli[L_VJ] * ul.by + wli[L_VK] * ul.bz) -
                   vbstl)) *
           sdml_inv;

  urst.mx = urst.d * spd[2];
  if (std::fabs(ur.d * sdr * sdmr - bxsq) < SMALL * ptst) {
    urst.my = urst.d * wri[L_VJ];
    urst.mz = urst.d * wri[L_VK];
    urst.by = ur.by;
    urst.bz = ur.bz;
  } else {
    double tmp = bxi * (sdr - sdmr) / (ur.d * sdr * sdmr - bxsq);
    urst.my = urst.d * (wri[L_VJ] - ur.by * tmp);
    urst.mz = urst.d * (wri[L_VK] - ur.bz * tmp);
    tmp = (ur.d * (sdr * sdr) - bxsq) / (ur.d * sdr * sdmr - bxsq);
    urst.by = ur.by * tmp;
    urst.bz = ur.bz * tmp;
  }
  double vbstr = (urst.mx * bxi + (urst.my * urst.by + urst.mz * urst.bz)) *
                 urst_d_inv;
  urst.e = (sdr * ur.e - ptr * wri[L_VI] + ptst * spd[2] +
            bxi * (wri[L_VI] * bxi + (wri[L_VJ] * ur.by + wri[L_VK] * ur.bz) -
                   vbstr)) *
           sdmr_inv;

  if (0.5 * bxsq < SMALL * ptst) {
    uldst = ulst;
    urdst = urst;
  } else {
    double invsumd = 1.0 / (sqrtdl + sqrtdr);
    double bxsig = (bxi > 0.0 ? 1.0 : -1.0);
    uldst.d = ulst.d;
    urdst.d = urst.d;
    uldst.mx = ulst.mx;
    urdst.mx = urst.mx;
    double tmp = invsumd * (sqrtdl * (ulst.my * ulst_d_inv) +
                            sqrtdr * (urst.my * urst_d_inv) +
                            bxsig * (urst.by - ulst.by));
    uldst.my = uldst.d * tmp;
    urdst.my = urdst.d * tmp;
    tmp = invsumd * (sqrtdl * (ulst.mz * ulst_d_inv) +
                     sqrtdr * (urst.mz * urst_d_inv) +
                     bxsig * (urst.bz - ulst.bz));
    uldst.mz = uldst.d * tmp;
    urdst.mz = urdst.d * tmp;
    tmp = invsumd * (sqrtdl * urst.by + sqrtdr * ulst.by +
                     bxsig * sqrtdl * sqrtdr *
                         ((urst.my * urst_d_inv) - (ulst.my * ulst_d_inv)));
    uldst.by = urdst.by = tmp;
    tmp = invsumd * (sqrtdl * urst.bz + sqrtdr * ulst.bz +
                     bxsig * sqrtdl * sqrtdr *
                         ((urst.mz * urst_d_inv) - (ulst.mz * ulst_d_inv)));
    uldst.bz = urdst.bz = tmp;
    tmp = spd[2] * bxi + (uldst.my * uldst.by + uldst.mz * uldst.bz) / uldst.d;
    uldst.e = ulst.e - sqrtdl * bxsig * (vbstl - tmp);
    urdst.e = urst.e + sqrtdr * bxsig * (vbstr - tmp);
  }

  auto diff = [](C& a, const C& b, double s) {
    a.d = s * (a.d - b.d);
    a.mx = s * (a.mx - b.mx);
    a.my = s * (a.my - b.my);
    a.mz = s * (a.mz - b.mz);
    a.e = s * (a.e - b.e);
    a.by = s * (a.by - b.by);
    a.bz = s * (a.bz - b.bz);
  };
  diff(uldst, ulst, spd[1]);
  diff(ulst, ul, spd[0]);
  diff(urdst, urst, spd[3]);
  diff(urst, ur, spd[4]);

  C f;
  if (spd[0] >= 0.0) {
    f = fl;
  } else if (spd[4] <= 0.0) {
    f = fr;
  } else if (spd[1] >= 0.0) {
    f.d = fl.d + ulst.d; f.mx = fl.mx + ulst.mx; f.my = fl.my + ulst.my;
    f.mz = fl.mz + ulst.mz; f.e = fl.e + ulst.e; f.by = fl.by + ulst.by;
    f.bz = fl.bz + ulst.bz;
  } else if (spd[2] >= 0.0) {
    f.d = fl.d + ulst.d + uldst.d; f.mx = fl.mx + ulst.mx + uldst.mx;
    f.my = fl.my + ulst.my + uldst.my; f.mz = fl.mz + ulst.mz + uldst.mz;
    f.e = fl.e + ulst.e + uldst.e; f.by = fl.by + ulst.by + uldst.by;
    f.bz = fl.bz + ulst.bz + uldst.bz;
  } else if (spd[3] > 0.0) {
    f.d = fr.d + urst.d + urdst.d; f.mx = fr.mx + urst.mx + urdst.mx;
    f.my = fr.my + urst.my + urdst.my; f.mz = fr.mz + urst.mz + urdst.mz;
    f.e = fr.e + urst.e + urdst.e; f.by = fr.by + urst.by + urdst.by;
    f.bz = fr.bz + urst.bz + urdst.bz;
  } else {
    f.d = fr.d + urst.d; f.mx = fr.mx + urst.mx; f.my = fr.my + urst.my;
    f.mz = fr.mz + urst.mz; f.e = fr.e + urst.e; f.by = fr.by + urst.by;
    f.bz = fr.bz + urst.bz;
  }
  flx[L_RHO] = f.d;
  flx[L_VI] = f.mx;
  flx[L_VJ] = f.my;
  flx[L_VK] = f.mz;
  flx[L_BI] = 0.0;
  flx[L_BJ] = f.by;
  flx[L_BK] = f.bz;
  flx[L_E] = f.e;

  *eflux = passive_eint_flux(g, wli[L_RHO], pressure_l, wri[L_RHO], pressure_r,
                             flx[L_RHO]);
  const double S_M = spd[2], S_l = spd[0], S_r = spd[4];
  const double l_coef = (S_l - wli[L_VI]) / (S_l - S_M);
  const double r_coef = (S_r - wri[L_VI]) / (S_r - S_M);
  if (S_l > 0) {
    *vbar = wli[L_VI];
  } else if (S_r < 0) {
    *vbar = wri[L_VI];
  } else if (S_M >= 0) {
    *vbar = S_M * l_coef;
  } else {
    *vbar = S_M * r_coef;
  }
}

// compute_conserved (EnzoRiemannUtils.hpp:48-82)
void conserved(double g, bool mhd, const double* w, double* u) {
  u[L_RHO] = w[L_RHO];
  u[L_BI] = w[L_BI]; u[L_BJ] = w[L_BJ]; u[L_BK] = w[L_BK];
  u[L_VI] = w[L_VI] * w[L_RHO];
  u[L_VJ] = w[L_VJ] * w[L_RHO];
  u[L_VK] = w[L_VK] * w[L_RHO];
  const double density = w[L_RHO], pressure = w[L_E];
  const double internal_edens = eos_eint_dens(g, density, pressure);
  const double kinetic_edens =
      0.5 * density * sqmag(w[L_VI], w[L_VJ], w[L_VK]);
  const double magnetic_edens =
      mhd ? 0.5 * sqmag(w[L_BI], w[L_BJ], w[L_BK]) : 0.5 * sqmag(0., 0., 0.);
  u[L_E] = internal_edens + kinetic_edens + magnetic_edens;
}

// active_fluxes (EnzoRiemannUtils.hpp:111-149)
void active_fluxes(bool mhd, const double* w, const double* u, double pressure,
                   double* f) {
  const double vi = w[L_VI], vj = w[L_VJ], vk = w[L_VK];
  const double Bi = mhd ? w[L_BI] : 0, Bj = mhd ? w[L_BJ] : 0,
               Bk = mhd ? w[L_BK] : 0;
  const double etot = u[L_E];
  const double ptot = pressure + 0.5 * sqmag(Bi, Bj, Bk);
  const double mom_i = u[L_VI];
  f[L_RHO] = mom_i;
  f[L_VI] = mom_i * vi - Bi * Bi + ptot;
  f[L_VJ] = mom_i * vj - Bj * Bi;
  f[L_VK] = mom_i * vk - Bk * Bi;
  f[L_E] = ((etot + ptot) * vi - (Bi * vi + (Bj * vj + Bk * vk)) * Bi);
  f[L_BI] = 0;
  f[L_BJ] = Bj * vi - Bi * vj;
  f[L_BK] = Bk * vi - Bi * vk;
}

// EinfeldtWavespeed<MHDLUT|HydroLUT> (EnzoRiemannHLL.hpp:44-172)
void einfeldt(double g, bool mhd, const double* wl, const double* wr,
              const double* Ul, const double* Ur, double pl, double pr,
              double* bp, double* bm) {
  double c_l, c_r;
  if (mhd) {
    c_l = eos_cfast(g, wl[L_RHO], pl, wl[L_BI], wl[L_BJ], wl[L_BK]);
    c_r = eos_cfast(g, wr[L_RHO], pr, wr[L_BI], wr[L_BJ], wr[L_BK]);
  } else {
    c_l = eos_sound_speed(g, wl[L_RHO], pl);
    c_r = eos_sound_speed(g, wr[L_RHO], pr);
  }
  double left_speed = (wl[L_VI] - c_l);
  double right_speed = (wr[L_VI] + c_r);
  double sqrtrho_l = std::sqrt(wl[L_RHO]);
  double sqrtrho_r = std::sqrt(wr[L_RHO]);
  double inv_sqrtrho_tot = 1.0 / (sqrtrho_l + sqrtrho_r);
  double vi_roe =
      (sqrtrho_l * wl[L_VI] + sqrtrho_r * wr[L_VI]) * inv_sqrtrho_tot;
  double vj_roe =
      (sqrtrho_l * wl[L_VJ] + sqrtrho_r * wr[L_VJ]) * inv_sqrtrho_tot;
  double vk_roe =
      (sqrtrho_l * wl[L_VK] + sqrtrho_r * wr[L_VK]) * inv_sqrtrho_tot;
  double v_roe2 = vi_roe * vi_roe + vj_roe * vj_roe + vk_roe * vk_roe;
  double ptot_l = pl, ptot_r = pr;
  if (mhd) {
    ptot_l += 0.5 * sqmag(wl[L_BI], wl[L_BJ], wl[L_BK]);
    ptot_r += 0.5 * sqmag(wr[L_BI], wr[L_BJ], wr[L_BK]);
  }
  double h_l = (Ul[L_E] + ptot_l) / wl[L_RHO];
  double h_r = (Ur[L_E] + ptot_r) / wr[L_RHO];
  double h_roe = (sqrtrho_l * h_l + sqrtrho_r * h_r) * inv_sqrtrho_tot;
  double c_roe;
  if (mhd) {  // roe_cfast_ (EnzoRiemannHLL.hpp:134-172)
    double rho_roe = sqrtrho_l * sqrtrho_r;
    double bi_roe = wl[L_BI];
    double bj_roe = (sqrtrho_l * wr[L_BJ] + sqrtrho_r * wl[L_BJ]) *
                    inv_sqrtrho_tot;
    double bk_roe = (sqrtrho_l * wr[L_BK] + sqrtrho_r * wl[L_BK]) *
                    inv_sqrtrho_tot;
    double b_roe2 = bi_roe * bi_roe + bj_roe * bj_roe + bk_roe * bk_roe;
    double gamma_prime = g - 1.;
    double dbj = wl[L_BJ] - wr[L_BJ];
    double dbk = wl[L_BK] - wr[L_BK];
    double x_prime = ((dbj * dbj + dbk * dbk) * 0.5 * (gamma_prime - 1) *
                      inv_sqrtrho_tot);
    double y_prime = ((gamma_prime - 1) * (wl[L_RHO] + wr[L_RHO]) * 0.5 /
                      rho_roe);
    double tilde_a2 = (gamma_prime * (h_roe - 0.5 * v_roe2 - b_roe2 / rho_roe) -
                       x_prime);
    double tilde_vai2 = bi_roe * bi_roe / rho_roe;
    double tilde_va2 = (tilde_vai2 + (gamma_prime - y_prime) *
                                         (bj_roe * bj_roe + bk_roe * bk_roe) /
                                         rho_roe);
    double s = tilde_a2 + tilde_va2;
    c_roe = std::sqrt(0.5 * (tilde_a2 + tilde_va2 +
                             std::sqrt(s * s - 4 * tilde_a2 * tilde_vai2)));
  } else {  // roe_cs_ (EnzoRiemannHLL.hpp:123-130)
    double tiny2 = 0.;
    double temp = h_roe - 0.5 * v_roe2;
    c_roe = std::sqrt((g - 1) * smax(temp, tiny2));
  }
  *bp = std::fmax(vi_roe + c_roe, right_speed);
  *bm = std::fmin(vi_roe - c_roe, left_speed);
}

// HLLKernel<EinfeldtWavespeed<MHDLUT>> (EnzoRiemannHLL.hpp:238-345)
void hlle(double g, const double* wl, const double* wr, double* flux,
          double* eflux, double* vbar) {
  const double pl = wl[L_E], pr = wr[L_E];
  double Ul[8], Ur[8], Fl[8], Fr[8];
  conserved(g, true, wl, Ul);
  conserved(g, true, wr, Ur);
  active_fluxes(true, wl, Ul, pl, Fl);
  active_fluxes(true, wr, Ur, pr, Fr);
  double bp, bm;
  einfeldt(g, true, wl, wr, Ul, Ur, pl, pr, &bp, &bm);
  bp = std::fmax(bp, 0.0);
  bm = std::fmin(bm, 0.0);
  double inv_speed_diff = 1. / (bp - bm);
  for (int f = 0; f < 8; f++) {
    flux[f] = ((bp * Fl[f] - bm * Fr[f] + (Ur[f] - Ul[f]) * bp * bm) *
               inv_speed_diff);
  }
  *eflux = passive_eint_flux(g, wl[L_RHO], pl, wr[L_RHO], pr, flux[L_RHO]);
  *vbar = (bp * wl[L_VI] - bm * wr[L_VI]) * inv_speed_diff;
}

// HLLCKernel (EnzoRiemannHLLC.hpp:34-172); hydro only
void hllc(double g, const double* wl, const double* wr, double* flux,
          double* eflux, double* vbar) {
  const double pl = wl[L_E], pr = wr[L_E];
  double Ul[8], Ur[8];
  conserved(g, false, wl, Ul);
  conserved(g, false, wr, Ur);
  double cs_l, cs_r;
  einfeldt(g, false, wl, wr, Ul, Ur, pl, pr, &cs_r, &cs_l);
  double bm = std::fmin(cs_l, 0.0);
  double bp = std::fmax(cs_r, 0.0);
  double tl = (pl - (cs_l - wl[L_VI]) * wl[L_RHO] * wl[L_VI]);
  double tr = (pr - (cs_r - wr[L_VI]) * wr[L_RHO] * wr[L_VI]);
  double dl = wl[L_RHO] * (cs_l - wl[L_VI]);
  double dr = -wr[L_RHO] * (cs_r - wr[L_VI]);
  double q1 = 1.0 / (dl + dr);
  double cw = (tr - tl) * q1;
  double cp = (dl * tr + dr * tl) * q1;
  double sl, sr, sm;
  if (cw >= 0.) {
    sl = cw / (cw - bm);
    sr = 0.;
    sm = -bm / (cw - bm);
  } else {
    sl = 0.;
    sr = -cw / (bp - cw);
    sm = bp / (bp - cw);
  }
  cp = smax(cp, 0.0);
  double momentumi_l = Ul[L_VI], momentumi_r = Ur[L_VI];
  double dfl = momentumi_l - bm * wl[L_RHO];
  double dfr = momentumi_r - bp * wr[L_RHO];
  double ufl = momentumi_l * (wl[L_VI] - bm) + pl;
  double ufr = momentumi_r * (wr[L_VI] - bp) + pr;
  double vfl = (wl[L_RHO] * wl[L_VJ] * (wl[L_VI] - bm));
  double vfr = (wr[L_RHO] * wr[L_VJ] * (wr[L_VI] - bp));
  double wfl = (wl[L_RHO] * wl[L_VK] * (wl[L_VI] - bm));
  double wfr = (wr[L_RHO] * wr[L_VK] * (wr[L_VI] - bp));
  double efl = (Ul[L_E] * (wl[L_VI] - bm) + pl * wl[L_VI]);
  double efr = (Ur[L_E] * (wr[L_VI] - bp) + pr * wr[L_VI]);
  flux[L_RHO] = sl * dfl + sr * dfr;
  flux[L_VI] = sl * ufl + sr * ufr;
  flux[L_VJ] = sl * vfl + sr * vfr;
  flux[L_VK] = sl * wfl + sr * wfr;
  flux[L_E] = sl * efl + sr * efr;
  flux[L_VI] += (sm * cp);
  flux[L_E] += (sm * cp * cw);
  flux[L_BI] = flux[L_BJ] = flux[L_BK] = 0.0;
  *eflux = passive_eint_flux(g, wl[L_RHO], pl, wr[L_RHO], pr, flux[L_RHO]);
  *vbar = (sl * (wl[L_VI] - bm) + sr * (wr[L_VI] - bp));
}

/* ------------------------------------------------------------------------ */
/* Block views                                                              */
/* ------------------------------------------------------------------------ */
constexpr int NPASS = 4;  // passive scalars supported

struct Integ {  // views of the integration quantities (+ cell-centred B)
  V3 rho, vx, vy, vz, etot, eint;
  V3 b[3];
  V3 pass[NPASS];  // passive scalars, conserved form
  int np = 0;
  V3 v(int d) const { return d == 0 ? vx : (d == 1 ? vy : vz); }
};

struct Scratch {
  A3 prim[NQ];
  A3 wl[NQ], wr[NQ];
  A3 flux[3][NQ];
  A3 eflux[3], vbar[3];
  A3 dU[6];  // rho, mom x/y/z (specific velocity keys), etot, eint
  A3 weight[3];
  A3 center_e;
  A3 edge_e[3];
  A3 temp_face[3];
  A3 t_rho, t_vx, t_vy, t_vz, t_etot, t_eint, t_b[3];
  // passive scalars: specific form, reconstructions, fluxes, dU, half step
  A3 pprim[NPASS], pwl[NPASS], pwr[NPASS], pflux[3][NPASS], pdU[NPASS], t_pass[NPASS];
};

// Primitive quantities of one stage
// (fluid-props/EnzoPhysicsFluidProps.cpp:64-138, EnzoComputePressure.cpp:82-198)
void pressure_from_integration(const Ctx& c, const Integ& u, V3 p, int s) {
  const double gm1 = c.gamma - 1.0;
  int lo[3] = {s, s, s}, hi[3] = {c.m[0] - s, c.m[1] - s, c.m[2] - s};
  if (c.de) {
    box(lo, hi, [&](const int* i) { p.c(i) = gm1 * u.rho.c(i) * u.eint.c(i); });
  } else {
    box(lo, hi, [&](const int* i) {
      double vx = u.vx.c(i), vy = u.vy.c(i), vz = u.vz.c(i);
      double ke = 0.5 * (vx * vx + vy * vy + vz * vz);
      double me_den = 0.;
      if (c.mhd) {
        double bx = u.b[0].c(i), by = u.b[1].c(i), bz = u.b[2].c(i);
        me_den = 0.5 * (bx * bx + by * by + bz * bz);
      }
      p.c(i) = gm1 * (u.rho.c(i) * (u.etot.c(i) - ke) - me_den);
    });
  }
}

void primitive_from_integration(const Ctx& c, const Integ& u, Scratch& sc,
                                int s) {
  int lo[3] = {s, s, s}, hi[3] = {c.m[0] - s, c.m[1] - s, c.m[2] - s};
  box(lo, hi, [&](const int* i) {
    sc.prim[Q_RHO].w.c(i) = u.rho.c(i);
    sc.prim[Q_VX].w.c(i) = u.vx.c(i);
    sc.prim[Q_VY].w.c(i) = u.vy.c(i);
    sc.prim[Q_VZ].w.c(i) = u.vz.c(i);
    if (c.mhd) {
      sc.prim[Q_BX].w.c(i) = u.b[0].c(i);
      sc.prim[Q_BY].w.c(i) = u.b[1].c(i);
      sc.prim[Q_BZ].w.c(i) = u.b[2].c(i);
    }
  });
  pressure_from_integration(c, u, sc.prim[Q_P].w, s);
  // passive scalars from conserved to specific form
  // (EnzoPhysicsFluidProps.cpp:120-133)
  for (int k = 0; k < u.np; k++)
    box(lo, hi, [&](const int* i) { sc.pprim[k].w.c(i) = u.pass[k].c(i) / u.rho.c(i); });
}

inline bool key_active(const Ctx& c, int q) {
  return c.mhd || (q != Q_BX && q != Q_BY && q != Q_BZ);
}

// Reconstruction along dim (toolkit/EnzoReconstructorNN.cpp:14-49,
// toolkit/EnzoReconstructorPLM.hpp:167-345).  wl/wr index f <-> face f+1/2.
void reconstruct(const Ctx& c, Scratch& sc, int dim, int s, int recon, int np) {
  for (int qq = 0; qq < NQ + np; qq++) {
    const int q = qq < NQ ? qq : -1;  // -1: passive scalar qq - NQ (no floor)
    if (q >= 0 && !key_active(c, q)) continue;
    V3 w = q >= 0 ? sc.prim[q].w : sc.pprim[qq - NQ].w;
    V3 wl = q >= 0 ? sc.wl[q].w : sc.pwl[qq - NQ].w;
    V3 wr = q >= 0 ? sc.wr[q].w : sc.pwr[qq - NQ].w;
    int lo[3] = {s, s, s}, hi[3] = {c.m[0] - s, c.m[1] - s, c.m[2] - s};
    if (recon == ORC_NN) {
      hi[dim] -= 1;
      box(lo, hi, [&](const int* i) {
        int j[3] = {i[0], i[1], i[2]};
        j[dim] += 1;
        wl.c(i) = w.c(i);
        wr.c(i) = w.c(j);
      });
    } else {
      const bool use_floor = (q == Q_RHO) || (q == Q_P);
      const double fl = (q == Q_RHO) ? c.prm->density_floor
                                     : c.prm->pressure_floor;
      const double theta = c.prm->theta_limiter;
      lo[dim] += 1;
      hi[dim] -= 1;
      box(lo, hi, [&](const int* i) {
        int im[3] = {i[0], i[1], i[2]}, ip[3] = {i[0], i[1], i[2]};
        im[dim] -= 1;
        ip[dim] += 1;
        double vm1 = w.c(im), val = w.c(i), vp1 = w.c(ip);
        double dv;
        if (recon == ORC_PLM) {  // PLM_EnzoRKLimiter (:287-302)
          double dv_c = 0.5 * (vp1 - vm1);
          double dv_l = (val - vm1) * theta;
          double dv_r = (vp1 - val) * theta;
          dv = (0.5 * (sgn(dv_l) + sgn(dv_r))) *
               min3(std::fabs(dv_l), std::fabs(dv_r), std::fabs(dv_c));
        } else {  // PLM_AthenaLimiter (:337-345)
          double dv_l = (val - vm1);
          double dv_r = (vp1 - val);
          double temp = dv_l * dv_r;
          dv = (temp <= 0.) ? 0. : 2. * temp / (dv_l + dv_r);
        }
        double half_dv = dv * 0.5;
        double right_val, left_val;
        if (use_floor) {
          right_val = apply_floor(val - half_dv, fl);
          left_val = apply_floor(val + half_dv, fl);
        } else {
          right_val = val - half_dv;
          left_val = val + half_dv;
        }
        wr.c(im) = right_val;  // face c-1/2
        wl.c(i) = left_val;    // face c+1/2
      });
    }
  }
}

// Riemann solve over the non-stale faces (EnzoRiemannImpl.hpp:317-338)
void riemann(const Ctx& c, Scratch& sc, int dim, int S) {
  const int ext_vi = Q_VX + dim, ext_vj = Q_VX + (dim + 1) % 3,
            ext_vk = Q_VX + (dim + 2) % 3;
  const int ext_bi = Q_BX + dim, ext_bj = Q_BX + (dim + 1) % 3,
            ext_bk = Q_BX + (dim + 2) % 3;
  int lo[3] = {S, S, S}, hi[3] = {c.m[0] - S, c.m[1] - S, c.m[2] - S};
  hi[dim] -= 1;
  const int solver = c.prm->riemann;
  box(lo, hi, [&](const int* i) {
    double wl[8], wr[8], f[8], ef, vb;
    const int map[8] = {Q_RHO, ext_bi, ext_bj, ext_bk,
                        ext_vi, ext_vj, ext_vk, Q_P};
    for (int k = 0; k < 8; k++) {
      if (!c.mhd && (k == L_BI || k == L_BJ || k == L_BK)) {
        wl[k] = wr[k] = 0.0;
        continue;
      }
      wl[k] = sc.wl[map[k]].w.c(i);
      wr[k] = sc.wr[map[k]].w.c(i);
    }
    if (solver == ORC_HLLD) hlld(c.gamma, wl, wr, f, &ef, &vb);
    else if (solver == ORC_HLLE) hlle(c.gamma, wl, wr, f, &ef, &vb);
    else hllc(c.gamma, wl, wr, f, &ef, &vb);
    for (int k = 0; k < 8; k++) sc.flux[dim][map[k]].w.c(i) = f[k];
    sc.eflux[dim].w.c(i) = ef;
    sc.vbar[dim].w.c(i) = vb;
  });
}
// solve_passive_advection (EnzoRiemannUtils.hpp:224-314): upwind specific
// scalar times the density flux
void passive_fluxes(const Ctx& c, Scratch& sc, int dim, int S, int np) {
  int lo[3] = {S, S, S}, hi[3] = {c.m[0] - S, c.m[1] - S, c.m[2] - S};
  hi[dim] -= 1;
  const V3 dens_flux = sc.flux[dim][Q_RHO].w;
  for (int k = 0; k < np; k++) {
    const V3 wl = sc.pwl[k].w, wr = sc.pwr[k].w, F = sc.pflux[dim][k].w;
    box(lo, hi, [&](const int* i) {
      const double df = dens_flux.c(i);
      const double upwind = (df > 0) * wl.c(i) + (df <= 0) * wr.c(i);
      F.c(i) = upwind * df;
    });
  }
}

// EnzoIntegrationQuanUpdate::accumulate_flux_component (:105-147) and
// EnzoSourceInternalEnergy::calculate_source (:16-92)
void accumulate(const Ctx& c, Scratch& sc, int dim, double dt,
                double cell_width, int S, int np) {
  const double dtdx_i = dt / cell_width;
  int lo[3] = {S, S, S}, hi[3] = {c.m[0] - S, c.m[1] - S, c.m[2] - S};
  lo[dim] += 1;
  hi[dim] -= 1;
  // integration keys: density, velocity_x/y/z, total_energy[, internal_energy]
  const int fkey[5] = {Q_RHO, Q_VX, Q_VY, Q_VZ, Q_P};
  for (int k = 0; k < 5; k++) {
    V3 dU = sc.dU[k].w, F = sc.flux[dim][fkey[k]].w;
    box(lo, hi, [&](const int* i) {
      int im[3] = {i[0], i[1], i[2]};
      im[dim] -= 1;
      dU.c(i) -= dtdx_i * (F.c(i) - F.c(im));
    });
  }
  for (int k = 0; k < np; k++) {
    V3 dU = sc.pdU[k].w, F = sc.pflux[dim][k].w;
    box(lo, hi, [&](const int* i) {
      int im[3] = {i[0], i[1], i[2]};
      im[dim] -= 1;
      dU.c(i) -= dtdx_i * (F.c(i) - F.c(im));
    });
  }
  if (c.de) {
    V3 dU = sc.dU[5].w, F = sc.eflux[dim].w;
    box(lo, hi, [&](const int* i) {
      int im[3] = {i[0], i[1], i[2]};
      im[dim] -= 1;
      dU.c(i) -= dtdx_i * (F.c(i) - F.c(im));
    });
    const double dtdx = dt / cell_width;
    const double p_floor = c.prm->pressure_floor;
    V3 vb = sc.vbar[dim].w, P = sc.prim[Q_P].w;
    box(lo, hi, [&](const int* i) {
      int im[3] = {i[0], i[1], i[2]};
      im[dim] -= 1;
      double p = apply_floor(P.c(i), p_floor);
      dU.c(i) -= dtdx * p * (vb.c(i) - vb.c(im));
    });
  }
}

// EnzoBfieldMethodCT::identify_upwind (:170-216)
void identify_upwind(const Ctx& c, Scratch& sc, int dim, int S) {
  int lo[3] = {S, S, S}, hi[3] = {c.m[0] - S, c.m[1] - S, c.m[2] - S};
  hi[dim] -= 1;
  V3 F = sc.flux[dim][Q_RHO].w, W = sc.weight[dim].w;
  box(lo, hi, [&](const int* i) {
    double fr = F.c(i);
    W.c(i) = (fr > 0) ? 1.0 : ((fr < 0) ? 0.0 : 0.5);
  });
}

// EnzoBfieldMethodCT::correct_reconstructed_bfield (:122-166)
void correct_bfield(const Ctx& c, Scratch& sc, const V3* face_cur, int dim,
                    int S) {
  int lo[3] = {S, S, S}, hi[3] = {c.m[0] - S, c.m[1] - S, c.m[2] - S};
  hi[dim] -= 1;
  V3 L = sc.wl[Q_BX + dim].w, R = sc.wr[Q_BX + dim].w, B = face_cur[dim];
  box(lo, hi, [&](const int* i) {
    int k[3] = {i[0], i[1], i[2]};
    k[dim] += 1;
    double v = B.c(k);
    L.c(i) = v;
    R.c(i) = v;
  });
}

// EnzoBfieldMethodCT::compute_center_efield (:267-292) and
// compute_edge_efield / compute_edge_<true> (:384-557)
void edge_efields(const Ctx& c, Scratch& sc, const Integ& cur, int S) {
  for (int dim = 0; dim < 3; dim++) {
    const int j = (dim + 1) % 3, k = (dim + 2) % 3;
    {
      V3 E = sc.center_e.w, vj = cur.v(j), vk = cur.v(k), bj = cur.b[j],
         bk = cur.b[k];
      int lo[3] = {S, S, S}, hi[3] = {c.m[0] - S, c.m[1] - S, c.m[2] - S};
      box(lo, hi, [&](const int* i) {
        E.c(i) = (-vj.c(i) * bk.c(i) + vk.c(i) * bj.c(i));
      });
    }
    // jflux/kflux: for dim x -> (y, z); y -> (z, x); z -> (x, y)
    V3 Ejf = sc.flux[j][Q_BX + k].w;  // j-flux of B_k
    V3 Ekf = sc.flux[k][Q_BX + j].w;  // k-flux of B_j
    V3 Wj = sc.weight[j].w, Wk = sc.weight[k].w, Ec = sc.center_e.w;
    V3 Eedge = sc.edge_e[dim].w;
    int lo[3] = {S, S, S}, hi[3] = {c.m[0] - S - 1, c.m[1] - S - 1,
                                    c.m[2] - S - 1};
    lo[dim] = S + 1;
    box(lo, hi, [&](const int* i) {
      int ij[3] = {i[0], i[1], i[2]}, ik[3] = {i[0], i[1], i[2]},
          ijk[3] = {i[0], i[1], i[2]};
      ij[j] += 1; ik[k] += 1; ijk[j] += 1; ijk[k] += 1;
      const double Ej = Ejf.c(i), Ej_kp1 = Ejf.c(ik);
      const double Ek = Ekf.c(i), Ek_jp1 = Ekf.c(ij);
      const double wj = Wj.c(i), Wj_kp1 = Wj.c(ik);
      const double wk = Wk.c(i), Wk_jp1 = Wk.c(ij);
      const double ec = Ec.c(i), Ec_jp1 = Ec.c(ij), Ec_kp1 = Ec.c(ik),
                   Ec_jkp1 = Ec.c(ijk);
      double dEdj_r = Wk_jp1 * (Ec_jp1 + Ej) + (1 - Wk_jp1) * (Ec_jkp1 + Ej_kp1);
      double dEdj_l = wk * (-Ej - ec) + (1 - wk) * (-Ej_kp1 - Ec_kp1);
      double dEdk_r = Wj_kp1 * (Ec_kp1 - Ek) + (1 - Wj_kp1) * (Ec_jkp1 - Ek_jp1);
      double dEdk_l = wj * (Ek - ec) + (1 - wj) * (Ek_jp1 - Ec_jp1);
      double Ej_sum = Ej + Ej_kp1;
      Ej_sum *= -1;
      double Ek_sum = Ek + Ek_jp1;
      Eedge.c(i) = 0.25 * (Ej_sum + Ek_sum + (dEdj_l - dEdj_r) +
                           (dEdk_l - dEdk_r));
    });
  }
}

// EnzoBfieldMethodCT::update_bfield (:617-687): out = base - dt/dj dE_k +
// dt/dk dE_j on the interior faces.  Edge arrays: E_x(x, ey, ez) etc.
void update_bfield(const Ctx& c, Scratch& sc, const double* cw, int dim,
                   const V3& base, const V3& out, double dt, int S) {
  const int j = (dim + 1) % 3, k = (dim + 2) % 3;
  const double dtdj = dt / cw[j];
  const double dtdk = dt / cw[k];
  V3 Ej = sc.edge_e[j].w, Ek = sc.edge_e[k].w;
  int lo[3], hi[3];
  lo[dim] = S + 1; hi[dim] = c.m[dim] - S;  // face index f
  lo[j] = S + 1; hi[j] = c.m[j] - S - 1;
  lo[k] = S + 1; hi[k] = c.m[k] - S - 1;
  box(lo, hi, [&](const int* i) {
    // E_k at (face f-1/2 along dim, j-edges i_j -+ 1/2); E_j similar in k.
    int e[3] = {i[0], i[1], i[2]};
    e[dim] -= 1;  // edge index along dim (edge f-1 sits at face f)
    int ekL[3] = {e[0], e[1], e[2]}, ekR[3] = {e[0], e[1], e[2]};
    ekL[j] -= 1;
    int ejL[3] = {e[0], e[1], e[2]}, ejR[3] = {e[0], e[1], e[2]};
    ejL[k] -= 1;
    double E_k_term = dtdj * (Ek.c(ekR) - Ek.c(ekL));
    double E_j_term = dtdk * (Ej.c(ejR) - Ej.c(ejL));
    out.c(i) = base.c(i) - E_k_term + E_j_term;
  });
}

// EnzoBfieldMethodCT::compute_center_bfield (:702-728)
void center_bfield(const Ctx& c, int dim, const V3& bc, const V3& bf, int S) {
  int lo[3] = {S, S, S}, hi[3] = {c.m[0] - S, c.m[1] - S, c.m[2] - S};
  box(lo, hi, [&](const int* i) {
    int ip[3] = {i[0], i[1], i[2]};
    ip[dim] += 1;
    bc.c(i) = 0.5 * (bf.c(i) + bf.c(ip));
  });
}

// EnzoPhysicsFluidProps::apply_floor_to_energy_and_sync (:162-290)
void energy_floor_sync(const Ctx& c, const Integ& u, int s) {
  const double eta = c.de ? c.prm->eta : 0.0;
  const float ggm1 = c.gamma * (c.gamma - 1.);
  const double pressure_floor = c.prm->pressure_floor;
  const double inv_gm1 = 1. / (c.gamma - 1.);
  const double half_factor = (eta != 0.) ? 0.5 : 0.;
  int lo[3] = {s, s, s}, hi[3] = {c.m[0] - s, c.m[1] - s, c.m[2] - s};
  box(lo, hi, [&](const int* i) {
    double inv_rho = 1. / u.rho.c(i);
    double eint_floor = pressure_floor * inv_gm1 * inv_rho;
    double vx = u.vx.c(i), vy = u.vy.c(i), vz = u.vz.c(i);
    double v2 = (vx * vx + vy * vy + vz * vz);
    double non_thermal_e = 0.5 * v2;
    double b2 = 0;
    if (c.mhd) {
      double bx = u.b[0].c(i), by = u.b[1].c(i), bz = u.b[2].c(i);
      b2 = (bx * bx + by * by + bz * bz);
      non_thermal_e += (0.5 * b2 * inv_rho);
    }
    if (c.de) {
      double eint_1 = u.etot.c(i) - non_thermal_e;
      double cur_eint = u.eint.c(i);
      double cs2_1 = std::fmax(0., ggm1 * eint_1);
      if ((cs2_1 > std::fmax(eta * v2, eta * b2 * inv_rho)) &&
          (eint_1 > half_factor * cur_eint)) {
        cur_eint = eint_1;
      }
      cur_eint = apply_floor(cur_eint, eint_floor);
      u.eint.c(i) = cur_eint;
      u.etot.c(i) = cur_eint + non_thermal_e;
    } else {
      double etot_floor = eint_floor + non_thermal_e;
      u.etot.c(i) = apply_floor(u.etot.c(i), etot_floor);
    }
  });
}

// EnzoIntegrationQuanUpdate::update_quantities (:183-238)
void update_quantities(const Ctx& c, const Integ& begin, Scratch& sc,
                       const Integ& out, int S) {
  const double density_floor = c.prm->density_floor;
  int lo[3] = {S + 1, S + 1, S + 1},
      hi[3] = {c.m[0] - S - 1, c.m[1] - S - 1, c.m[2] - S - 1};
  box(lo, hi, [&](const int* i) {
    double old_rho = begin.rho.c(i);
    out.rho.c(i) = begin.rho.c(i) + sc.dU[0].w.c(i);
    double new_rho = out.rho.c(i);
    new_rho = apply_floor(new_rho, density_floor);
    out.rho.c(i) = new_rho;
    double inv_new_rho = 1. / new_rho;
    const V3 cur_spec[5] = {begin.vx, begin.vy, begin.vz, begin.etot,
                            begin.eint};
    const V3 out_spec[5] = {out.vx, out.vy, out.vz, out.etot, out.eint};
    const int nspec = c.de ? 5 : 4;
    for (int k = 0; k < nspec; k++) {
      out_spec[k].c(i) =
          (cur_spec[k].c(i) * old_rho + sc.dU[k + 1].w.c(i)) * inv_new_rho;
    }
  });
  energy_floor_sync(c, out, S + 1);
  // update_passive_scalars_ (EnzoIntegrationQuanUpdate.cpp:242-270)
  for (int k = 0; k < begin.np; k++)
    box(lo, hi, [&](const int* i) { out.pass[k].c(i) = begin.pass[k].c(i) + sc.pdU[k].w.c(i); });
}

int staling_total(int recon) { return recon == ORC_NN ? 1 : 2; }
int staling_immediate(int recon) { return recon == ORC_NN ? 0 : 1; }

// EnzoMHDIntegratorStageCommands::compute_update_stage (:102-203)
// EnzoSourceGravity::calculate_source (toolkit/EnzoSourceGravity.cpp:17-69):
// momentum and energy sources from the acceleration fields, with the density
// and velocity of the start of the timestep
void gravity_source(const Ctx& c, const Integ& begin, Scratch& sc, double dt,
                    int stale) {
  const V3 dmx = sc.dU[1].w, dmy = sc.dU[2].w, dmz = sc.dU[3].w, dE = sc.dU[4].w;
  for (int iz = stale; iz < c.m[2] - stale; iz++)
    for (int iy = stale; iy < c.m[1] - stale; iy++)
      for (int ix = stale; ix < c.m[0] - stale; ix++) {
        const double rho = begin.rho.at(ix, iy, iz);
        const double ax = c.accel[0].at(ix, iy, iz);
        const double ay = c.accel[1].at(ix, iy, iz);
        const double az = c.accel[2].at(ix, iy, iz);
        dmx.at(ix, iy, iz) += dt * rho * ax;
        dmy.at(ix, iy, iz) += dt * rho * ay;
        dmz.at(ix, iy, iz) += dt * rho * az;
        dE.at(ix, iy, iz) += dt * rho * ((begin.vx.at(ix, iy, iz) * ax) +
                                         (begin.vy.at(ix, iy, iz) * ay) +
                                         (begin.vz.at(ix, iy, iz) * az));
      }
}

void compute_update_stage(const Ctx& c, const Integ& begin, const Integ& cur,
                          const Integ& out, Scratch& sc, const V3* face_cur,
                          const V3* face_base, const V3* face_out,
                          const double* cw, int recon, double cur_dt,
                          int stale, bool full_timestep) {
  for (int k = 0; k < 6; k++) std::fill(sc.dU[k].v.begin(), sc.dU[k].v.end(), 0.0);
  const int np = cur.np;
  for (int k = 0; k < np; k++) std::fill(sc.pdU[k].v.begin(), sc.pdU[k].v.end(), 0.0);
  primitive_from_integration(c, cur, sc, stale);
  for (int dim = 0; dim < 3; dim++) {
    reconstruct(c, sc, dim, stale, recon, np);
    int cs = stale + staling_immediate(recon);
    if (c.mhd) correct_bfield(c, sc, face_cur, dim, cs);
    riemann(c, sc, dim, cs);
    passive_fluxes(c, sc, dim, cs, np);
    accumulate(c, sc, dim, cur_dt, cw[dim], cs, np);
    if (c.mhd) identify_upwind(c, sc, dim, cs);
  }
  stale += staling_immediate(recon);
  // compute_source_terms_ (EnzoMHDIntegratorStageCommands.cpp:267-297):
  // gravity on the full-timestep stage (stage index 1) only
  if (full_timestep && c.gravity) gravity_source(c, begin, sc, cur_dt, stale);
  if (c.mhd) {
    // update_all_bfield_components (EnzoBfieldMethodCT.cpp:220-263)
    edge_efields(c, sc, cur, stale);
    for (int dim = 0; dim < 3; dim++) {
      update_bfield(c, sc, cw, dim, face_base[dim], face_out[dim], cur_dt,
                    stale);
    }
    for (int dim = 0; dim < 3; dim++) {
      center_bfield(c, dim, out.b[dim], face_out[dim], stale);
    }
  }
  update_quantities(c, begin, sc, out, stale);
}

Integ integ_of(const OracleBlock* b, const int* m) {
  Integ u;
  u.rho = view(b->rho, m[0], m[1], m[2]);
  u.vx = view(b->vx, m[0], m[1], m[2]);
  u.vy = view(b->vy, m[0], m[1], m[2]);
  u.vz = view(b->vz, m[0], m[1], m[2]);
  u.etot = view(b->etot, m[0], m[1], m[2]);
  u.eint = view(b->eint, m[0], m[1], m[2]);
  u.b[0] = view(b->bx, m[0], m[1], m[2]);
  u.b[1] = view(b->by, m[0], m[1], m[2]);
  u.b[2] = view(b->bz, m[0], m[1], m[2]);
  u.np = std::max(0, std::min(b->npassive, NPASS));
  for (int k = 0; k < u.np; k++) u.pass[k] = view(b->passive[k], m[0], m[1], m[2]);
  return u;
}

void setup_ctx(Ctx& c, const OracleParams* p, const OracleBlock* b) {
  c.prm = p;
  c.m[0] = b->nx + 2 * b->g;
  c.m[1] = b->ny + 2 * b->g;
  c.m[2] = b->nz + 2 * b->g;
  c.mhd = p->mhd != 0;
  c.de = p->dual_energy != 0;
  c.gamma = p->gamma;
  c.gravity = b->ax && b->ay && b->az;
  if (c.gravity) {
    c.accel[0] = view(b->ax, c.m[0], c.m[1], c.m[2]);
    c.accel[1] = view(b->ay, c.m[0], c.m[1], c.m[2]);
    c.accel[2] = view(b->az, c.m[0], c.m[1], c.m[2]);
  }
}

long long g_flops = -1;

}  // namespace

/* ------------------------------------------------------------------------ */
/* C API                                                                    */
/* ------------------------------------------------------------------------ */

extern "C" long long oracle_flop_count(void) { return g_flops; }

// EnzoMethodMHDVlct::save_fluxes_for_corrections_ (EnzoMethodMHDVlct.cpp:
// 250-330): after the final stage, dt/dx_dim times the flux through the low
// (face g-1) and high (face m-g-1) active boundary of every axis, for the
// requested integration quantities.  out[(dim * 2 + side) * nq + iq] holds an
// array of the block's active face, last index fastest: axis 0 (nz, ny),
// axis 1 (nz, nx), axis 2 (ny, nx).  quantities: 0 density, 1-3 velocity
// x/y/z (the momentum flux), 4 total energy, 5 internal energy, 6-9 passive
// scalars 0-3 (the conserved-form flux: FluxData holds every field of the
// "conserved" group, EnzoMethodMHDVlct.cpp:265-272).
static void save_boundary_fluxes(const Ctx& c, const Scratch& sc, double dt,
                                 const double* cw, int g, double* const* out,
                                 int nq, const int* quantities) {
  const int* m = c.m;
  const int n[3] = {m[0] - 2 * g, m[1] - 2 * g, m[2] - 2 * g};
  for (int dim = 0; dim < 3; dim++) {
    const double dt_dxi = dt / cw[dim];
    for (int iq = 0; iq < nq; iq++) {
      const int q = quantities[iq];
      const V3 F = (q >= 6) ? sc.pflux[dim][q - 6].w
                 : (q == 5) ? sc.eflux[dim].w
                 : (q == 0) ? sc.flux[dim][Q_RHO].w
                 : (q == 4) ? sc.flux[dim][Q_P].w
                            : sc.flux[dim][Q_VX + (q - 1)].w;
      for (int side = 0; side < 2; side++) {
        double* dst = out[(dim * 2 + side) * nq + iq];
        if (!dst) continue;
        const int f = side == 0 ? g - 1 : m[dim] - g - 1;
        if (dim == 0) {
          for (int iz = 0; iz < n[2]; iz++)
            for (int iy = 0; iy < n[1]; iy++)
              dst[(size_t)iz * n[1] + iy] = dt_dxi * F.at(f, g + iy, g + iz);
        } else if (dim == 1) {
          for (int iz = 0; iz < n[2]; iz++)
            for (int ix = 0; ix < n[0]; ix++)
              dst[(size_t)iz * n[0] + ix] = dt_dxi * F.at(g + ix, f, g + iz);
        } else {
          for (int iy = 0; iy < n[1]; iy++)
            for (int ix = 0; ix < n[0]; ix++)
              dst[(size_t)iy * n[0] + ix] = dt_dxi * F.at(g + ix, g + iy, f);
        }
      }
    }
  }
}

static int step_impl(const OracleParams* p, OracleBlock* b, double dt,
                     double* const* fc_out, int fc_nq, const int* fc_q);

// EnzoMethodMHDVlct::compute (EnzoMethodMHDVlct.cpp:356-500)
extern "C" int oracle_step(const OracleParams* p, OracleBlock* b, double dt) {
  return step_impl(p, b, dt, nullptr, 0, nullptr);
}

// compute with store_fluxes_for_corrections (EnzoMethodMHDVlct.cpp:136-141,
// :483-490): hydro only, as the reference asserts
extern "C" int oracle_step_fc(const OracleParams* p, OracleBlock* b, double dt,
                              double* const* out, int nq, const int* quantities) {
  if (p->mhd) return 4;
  const int np = std::max(0, std::min(b->npassive, NPASS));
  for (int i = 0; i < nq; i++)
    if (quantities[i] < 0 || quantities[i] >= 6 + np ||
        (quantities[i] == 5 && !p->dual_energy))
      return 5;
  return step_impl(p, b, dt, out, nq, quantities);
}

static int step_impl(const OracleParams* p, OracleBlock* b, double dt,
                     double* const* fc_out, int fc_nq, const int* fc_q) {
  Ctx c;
  setup_ctx(c, p, b);
  const int* m = c.m;
  Scratch sc;
  for (int q = 0; q < NQ; q++) {
    sc.prim[q].alloc(m[0], m[1], m[2]);
    sc.wl[q].alloc(m[0], m[1], m[2]);
    sc.wr[q].alloc(m[0], m[1], m[2]);
    for (int d = 0; d < 3; d++)
      sc.flux[d][q].alloc(m[0] - (d == 0), m[1] - (d == 1), m[2] - (d == 2));
  }
  for (int d = 0; d < 3; d++) {
    sc.eflux[d].alloc(m[0] - (d == 0), m[1] - (d == 1), m[2] - (d == 2));
    sc.vbar[d].alloc(m[0] - (d == 0), m[1] - (d == 1), m[2] - (d == 2));
    sc.weight[d].alloc(m[0] - (d == 0), m[1] - (d == 1), m[2] - (d == 2));
    sc.temp_face[d].alloc(m[0] + (d == 0), m[1] + (d == 1), m[2] + (d == 2));
  }
  // edge E: E_x (mx, my-1, mz-1), E_y (mx-1, my, mz-1), E_z (mx-1, my-1, mz)
  sc.edge_e[0].alloc(m[0], m[1] - 1, m[2] - 1);
  sc.edge_e[1].alloc(m[0] - 1, m[1], m[2] - 1);
  sc.edge_e[2].alloc(m[0] - 1, m[1] - 1, m[2]);
  sc.center_e.alloc(m[0], m[1], m[2]);
  for (int k = 0; k < 6; k++) sc.dU[k].alloc(m[0], m[1], m[2]);
  sc.t_rho.alloc(m[0], m[1], m[2]);
  sc.t_vx.alloc(m[0], m[1], m[2]);
  sc.t_vy.alloc(m[0], m[1], m[2]);
  sc.t_vz.alloc(m[0], m[1], m[2]);
  sc.t_etot.alloc(m[0], m[1], m[2]);
  sc.t_eint.alloc(m[0], m[1], m[2]);
  for (int d = 0; d < 3; d++) sc.t_b[d].alloc(m[0], m[1], m[2]);

  Integ ext = integ_of(b, m);
  Integ tmp;
  tmp.rho = sc.t_rho.w; tmp.vx = sc.t_vx.w; tmp.vy = sc.t_vy.w;
  tmp.vz = sc.t_vz.w; tmp.etot = sc.t_etot.w; tmp.eint = sc.t_eint.w;
  for (int d = 0; d < 3; d++) tmp.b[d] = sc.t_b[d].w;
  tmp.np = ext.np;
  for (int k = 0; k < ext.np; k++) {
    sc.pprim[k].alloc(m[0], m[1], m[2]);
    sc.pwl[k].alloc(m[0], m[1], m[2]);
    sc.pwr[k].alloc(m[0], m[1], m[2]);
    sc.pdU[k].alloc(m[0], m[1], m[2]);
    sc.t_pass[k].alloc(m[0], m[1], m[2]);
    tmp.pass[k] = sc.t_pass[k].w;
    for (int d = 0; d < 3; d++)
      sc.pflux[d][k].alloc(m[0] - (d == 0), m[1] - (d == 1), m[2] - (d == 2));
  }

  V3 face[3];
  if (c.mhd) {
    face[0] = view(b->bfx, m[0] + 1, m[1], m[2]);
    face[1] = view(b->bfy, m[0], m[1] + 1, m[2]);
    face[2] = view(b->bfz, m[0], m[1], m[2] + 1);
  }
  V3 tface[3] = {sc.temp_face[0].w, sc.temp_face[1].w, sc.temp_face[2].w};
  const double cw[3] = {b->dx, b->dy, b->dz};

  // EnzoBfieldMethod.cpp:23-27: constrained transport requires the two
  // partial timesteps of the vl scheme (the reference ERRORs otherwise)
  if (p->euler && c.mhd) return 3;
  const int nstages = p->euler ? 1 : 2;
  int stale = 0;
  for (int st = 0; st < nstages; st++) {
    const bool final_stage = (st + 1) == nstages;
    const double cur_dt = (!final_stage) ? dt / 2. : dt;
    const int recon = (nstages == 2 && st == 0) ? ORC_NN : p->recon;
    const Integ& cur = (st == 0) ? ext : tmp;
    const Integ& out = final_stage ? ext : tmp;
    // CT state machine (EnzoBfieldMethodCT.cpp:122-137, :228-240)
    const V3* fcur = (st == 0) ? face : tface;
    const V3* fout = final_stage ? face : tface;
    compute_update_stage(c, ext, cur, out, sc, fcur, face, fout, cw, recon,
                         cur_dt, stale, st == 1);
    stale += staling_total(recon);
    if (final_stage && fc_out)
      save_boundary_fluxes(c, sc, dt, cw, b->g, fc_out, fc_nq, fc_q);
  }
  return 0;
}

// EnzoMethodMHDVlct::timestep (EnzoMethodMHDVlct.cpp:551-588) and
// EnzoMHDIntegratorStageCommands::timestep (:299-366)
extern "C" double oracle_timestep(const OracleParams* p, OracleBlock* b) {
  Ctx c;
  setup_ctx(c, p, b);
  Integ u = integ_of(b, c.m);
  if (c.de) energy_floor_sync(c, u, 0);
  V3 P = view(b->pressure, c.m[0], c.m[1], c.m[2]);
  pressure_from_integration(c, u, P, 0);
  const double dx = b->dx, dy = b->dy, dz = b->dz;
  double dtBaryons = 1.7976931348623157e308;
  int lo[3] = {0, 0, 0}, hi[3] = {c.m[0], c.m[1], c.m[2]};
  box(lo, hi, [&](const int* i) {
    double cf;
    if (c.mhd) {
      cf = eos_cfast0(c.gamma, u.rho.c(i), P.c(i), u.b[0].c(i), u.b[1].c(i),
                      u.b[2].c(i));
    } else {
      cf = eos_sound_speed(c.gamma, u.rho.c(i), P.c(i));
    }
    double local_dt = min3(dx / (std::fabs(u.vx.c(i)) + cf),
                           dy / (std::fabs(u.vy.c(i)) + cf),
                           dz / (std::fabs(u.vz.c(i)) + cf));
    dtBaryons = smin(dtBaryons, local_dt);
  });
  return dtBaryons * p->courant;
}

/* Same-level ghost refresh (src/Cello/control_refresh.cpp:243-360,
 * data_FieldFace.cpp:439-520, mesh_Box.cpp:150-206).  Along every axis a
 * cell-centred ghost index c takes the source index c+n (low ghosts) or c-n
 * (high ghosts); for a face-centred axis the block's own boundary faces
 * (g and g+n) are never overwritten, faces k<g take k+n and faces k>g+n take
 * k-n.  The source block along each axis is the low/high neighbour. */
namespace {
struct FieldRef { double* p; int n[3]; int face; };
inline int src_index(int i, int g, int n, int face_axis, int* side) {
  if (face_axis) {
    if (i < g) { *side = -1; return i + n; }
    if (i > g + n) { *side = +1; return i - n; }
    *side = 0; return i;
  }
  if (i < g) { *side = -1; return i + n; }
  if (i >= g + n) { *side = +1; return i - n; }
  *side = 0; return i;
}
void fill_fields(OracleBlock* blocks, int nbx, int nby, int nbz) {
  const int nb = nbx * nby * nbz;
  const int g = blocks[0].g;
  const int n[3] = {blocks[0].nx, blocks[0].ny, blocks[0].nz};
  const int m[3] = {n[0] + 2 * g, n[1] + 2 * g, n[2] + 2 * g};
  const int nfield = 20;  // every field (EnzoMethodMHDVlct.cpp:146-151)
  // copy sources first so that the refresh reads pre-refresh values only
  for (int f = 0; f < nfield; f++) {
    int face = -1;
    std::vector<std::vector<double>> snap(nb);
    auto ptr = [&](OracleBlock& b) -> double* {
      switch (f) {
        case 0: return b.rho; case 1: return b.vx; case 2: return b.vy;
        case 3: return b.vz; case 4: return b.etot; case 5: return b.eint;
        case 6: return b.bx; case 7: return b.by; case 8: return b.bz;
        case 9: return b.bfx; case 10: return b.bfy; case 11: return b.bfz;
        case 12: return b.pressure;
        case 13: return b.ax; case 14: return b.ay; case 15: return b.az;
        default: return f - 16 < b.npassive ? b.passive[f - 16] : nullptr;
      }
    };
    if (f == 9) face = 0;
    if (f == 10) face = 1;
    if (f == 11) face = 2;
    if (!ptr(blocks[0])) continue;
    int e[3] = {m[0] + (face == 0), m[1] + (face == 1), m[2] + (face == 2)};
    size_t sz = (size_t)e[0] * e[1] * e[2];
    for (int ib = 0; ib < nb; ib++)
      snap[ib].assign(ptr(blocks[ib]), ptr(blocks[ib]) + sz);
    for (int kz = 0; kz < nbz; kz++)
      for (int ky = 0; ky < nby; ky++)
        for (int kx = 0; kx < nbx; kx++) {
          int ib = (kz * nby + ky) * nbx + kx;
          double* dst = ptr(blocks[ib]);
          for (int z = 0; z < e[2]; z++)
            for (int y = 0; y < e[1]; y++)
              for (int x = 0; x < e[0]; x++) {
                int sd[3];
                int sx = src_index(x, g, n[0], face == 0, &sd[0]);
                int sy = src_index(y, g, n[1], face == 1, &sd[1]);
                int sz2 = src_index(z, g, n[2], face == 2, &sd[2]);
                if (sd[0] == 0 && sd[1] == 0 && sd[2] == 0) continue;
                int bx = (kx + sd[0] + nbx) % nbx;
                int by = (ky + sd[1] + nby) % nby;
                int bz = (kz + sd[2] + nbz) % nbz;
                int sb = (bz * nby + by) * nbx + bx;
                dst[((size_t)z * e[1] + y) * e[0] + x] =
                    snap[sb][((size_t)sz2 * e[1] + sy) * e[0] + sx];
              }
        }
  }
}

/* The same refresh with the source blocks taken from a 27-neighbour table
 * instead of a periodic brick: the ghost region at offset (sx, sy, sz) of
 * block i comes from block nbr[27 i + (sz+1) 9 + (sy+1) 3 + (sx+1)], which
 * has the same extents as block i (Cello refreshes same-level neighbours of
 * equal size; the blocks of the table may differ in size from one another).
 * This is the batch's mhdvlct_batch_set_neighbors refresh. */
void fill_fields_table(OracleBlock* blocks, int nb, const int* nbr) {
  const int nfield = 20;
  for (int f = 0; f < nfield; f++) {
    int face = -1;
    if (f == 9) face = 0;
    if (f == 10) face = 1;
    if (f == 11) face = 2;
    auto ptr = [&](OracleBlock& b) -> double* {
      switch (f) {
        case 0: return b.rho; case 1: return b.vx; case 2: return b.vy;
        case 3: return b.vz; case 4: return b.etot; case 5: return b.eint;
        case 6: return b.bx; case 7: return b.by; case 8: return b.bz;
        case 9: return b.bfx; case 10: return b.bfy; case 11: return b.bfz;
        case 12: return b.pressure;
        case 13: return b.ax; case 14: return b.ay; case 15: return b.az;
        default: return f - 16 < b.npassive ? b.passive[f - 16] : nullptr;
      }
    };
    if (!ptr(blocks[0])) continue;
    // sources first, so that the refresh reads pre-refresh values only
    std::vector<std::vector<double>> snap(nb);
    auto extent = [&](const OracleBlock& b, int e[3]) {
      const int g = b.g;
      e[0] = b.nx + 2 * g + (face == 0);
      e[1] = b.ny + 2 * g + (face == 1);
      e[2] = b.nz + 2 * g + (face == 2);
      return (size_t)e[0] * e[1] * e[2];
    };
    for (int ib = 0; ib < nb; ib++) {
      int e[3];
      const size_t sz = extent(blocks[ib], e);
      snap[ib].assign(ptr(blocks[ib]), ptr(blocks[ib]) + sz);
    }
    for (int ib = 0; ib < nb; ib++) {
      OracleBlock& b = blocks[ib];
      const int g = b.g;
      const int n[3] = {b.nx, b.ny, b.nz};
      int e[3];
      extent(b, e);
      double* dst = ptr(b);
      for (int z = 0; z < e[2]; z++)
        for (int y = 0; y < e[1]; y++)
          for (int x = 0; x < e[0]; x++) {
            int sd[3];
            const int sx = src_index(x, g, n[0], face == 0, &sd[0]);
            const int sy = src_index(y, g, n[1], face == 1, &sd[1]);
            const int sz2 = src_index(z, g, n[2], face == 2, &sd[2]);
            if (sd[0] == 0 && sd[1] == 0 && sd[2] == 0) continue;
            const int sb = nbr[27 * (size_t)ib + (sd[2] + 1) * 9 + (sd[1] + 1) * 3 + (sd[0] + 1)];
            dst[((size_t)z * e[1] + y) * e[0] + x] =
                snap[sb][((size_t)sz2 * e[1] + sy) * e[0] + sx];
          }
    }
  }
}
}  // namespace

extern "C" void oracle_fill_ghosts_periodic(OracleBlock* b) {
  fill_fields(b, 1, 1, 1);
}

extern "C" void oracle_fill_ghosts_table(OracleBlock* blocks, int nb, const int* nbr) {
  fill_fields_table(blocks, nb, nbr);
}

extern "C" void oracle_fill_ghosts_brick(OracleBlock* blocks, int nbx, int nby,
                                         int nbz) {
  fill_fields(blocks, nbx, nby, nbz);
}

/* ------------------------------------------------------------------------ */
/* Inclined linear wave IC (src/Enzo/initial/EnzoInitialInclinedWave.cpp)   */
/* ------------------------------------------------------------------------ */
namespace {
struct Rot {  // Rotation (EnzoInitialInclinedWave.cpp:54-103)
  double m[3][3];
  Rot(double a, double b) {
    m[0][0] = std::cos(a) * std::cos(b);
    m[0][1] = std::cos(a) * std::sin(b);
    m[0][2] = std::sin(a);
    m[1][0] = -1. * std::sin(b);
    m[1][1] = std::cos(b);
    m[1][2] = 0.;
    m[2][0] = -1. * std::sin(a) * std::cos(b);
    m[2][1] = -1. * std::sin(a) * std::sin(b);
    m[2][2] = std::cos(a);
  }
  void rot(double v0, double v1, double v2, double& r0, double& r1,
           double& r2) const {
    r0 = m[0][0] * v0 + m[0][1] * v1 + m[0][2] * v2;
    r1 = m[1][0] * v0 + m[1][1] * v1 + m[1][2] * v2;
    r2 = m[2][0] * v0 + m[2][1] * v1 + m[2][2] * v2;
  }
  void inv_rot(double r0, double r1, double r2, double& v0, double& v1,
               double& v2) const {
    v0 = m[0][0] * r0 + m[1][0] * r1 + m[2][0] * r2;
    v1 = m[0][1] * r0 + m[1][1] * r1 + m[2][1] * r2;
    v2 = m[0][2] * r0 + m[1][2] * r1 + m[2][2] * r2;
  }
};
const double PI = 3.14159265358979323846;
// LinearScalarInit (:120-160) with use_cosine=true
inline double lin_scalar(double back, double ev, double amp, double lambda,
                         double x0) {
  double tmp = x0 * 2. * PI / lambda;
  return (back + amp * ev * (1 * std::cos(tmp) + (1 - 1) * std::sin(tmp)));
}
}  // namespace

extern "C" int oracle_ic_inclined_wave(OracleBlock* b, const char* wave_c,
                                       double alpha, double beta, double gamma,
                                       double amplitude, double lambda,
                                       int positive_vel, double xl, double yl,
                                       double zl) {
  const std::string wave(wave_c);
  const int g = b->g;
  const int mx = b->nx + 2 * g, my = b->ny + 2 * g, mz = b->nz + 2 * g;
  const double dx = b->dx, dy = b->dy, dz = b->dz;
  auto px = [&](int i) { return xl + dx * (0.5 + (double)(i - g)); };
  auto py = [&](int j) { return yl + dy * (0.5 + (double)(j - g)); };
  auto pz = [&](int k) { return zl + dz * (0.5 + (double)(k - g)); };
  auto fx = [&](int i) { return xl + dx * (double)(i - g); };
  auto fy = [&](int j) { return yl + dy * (double)(j - g); };
  auto fz = [&](int k) { return zl + dz * (double)(k - g); };
  const Rot R(alpha, beta);
  double wsign = positive_vel ? 1. : -1;
  double density_back = 1, mom0_back = 0, mom1_back = 0, mom2_back = 0;
  double density_ev, mom0_ev, mom1_ev, mom2_ev, etot_ev, etot_back;
  double b1_ev = 0, b2_ev = 0;
  const bool mhd_wave = (wave == "fast" || wave == "alfven" || wave == "slow" ||
                         wave == "mhd_entropy");
  if (mhd_wave) {  // prepare_MHD_initializers_ (:590-700)
    etot_back = (1. / gamma) / (gamma - 1.) + 1.625;
    if (wave == "mhd_entropy") {
      mom0_back = wsign;
      etot_back += 0.5;
    }
    if (wave == "fast") {
      double coef = 0.5 / std::sqrt(5.);
      density_ev = 2. * coef; mom0_ev = wsign * 4. * coef;
      mom1_ev = -1. * wsign * 2. * coef; mom2_ev = 0; etot_ev = 9. * coef;
      b1_ev = 4. * coef; b2_ev = 0;
    } else if (wave == "alfven") {
      density_ev = 0; mom0_ev = 0; mom1_ev = 0; mom2_ev = -1. * wsign * 1;
      etot_ev = 0; b1_ev = 0; b2_ev = 1.;
    } else if (wave == "slow") {
      double coef = 0.5 / std::sqrt(5.);
      density_ev = 4. * coef; mom0_ev = wsign * 2. * coef;
      mom1_ev = wsign * 4. * coef; mom2_ev = 0; etot_ev = 3. * coef;
      b1_ev = -2. * coef; b2_ev = 0;
    } else {
      double coef = 0.5;
      density_ev = 2. * coef; mom0_ev = 2. * coef * wsign; mom1_ev = 0;
      mom2_ev = 0; etot_ev = 1. * coef; b1_ev = 0; b2_ev = 0;
    }
  } else if (wave == "sound" || wave == "hd_entropy") {
    // prepare_HD_initializers_ (:702-760)
    double v0_back = 0, v1_back = 0, v2_back = 0;
    if (wave != "sound") v0_back = wsign;
    double squared_v_back =
        v0_back * v0_back + v1_back * v1_back + v2_back * v2_back;
    mom0_back = v0_back; mom1_back = v1_back; mom2_back = v2_back;
    etot_back = ((1. / gamma) / (gamma - 1.) + 0.5 * squared_v_back);
    if (wave == "sound") {
      double h_back = 1 / (gamma - 1.) + 0.5 * squared_v_back;
      double signed_cs = wsign * 1;
      density_ev = 1; mom0_ev = v0_back + signed_cs; mom1_ev = v1_back;
      mom2_ev = v2_back; etot_ev = h_back + v0_back * signed_cs;
    } else {
      density_ev = 1; mom0_ev = v0_back; mom1_ev = v1_back; mom2_ev = v2_back;
      etot_ev = 0.5 * squared_v_back;
    }
  } else {
    return 1;
  }

  if (mhd_wave) {  // setup_bfield (:266-323) + EnzoInitialBCenter (:43-127)
    const double b0_back = 1., b1_back = 1.5, b2_back = 0.0;
    auto apot = [&](double x, double y, double z, double& v0, double& v1,
                    double& v2) {
      // RotatedVectorInit(LinearVectorPotentialInit) (:170-245)
      double x0, x1, x2, r0, r1, r2;
      R.rot(x, y, z, x0, x1, x2);
      r0 = (x2 * amplitude * b1_ev * std::cos(2. * PI * x0 / lambda) -
            x1 * amplitude * b2_ev * std::cos(2. * PI * x0 / lambda));
      r1 = b2_back * x0;
      r2 = b0_back * x1 - b1_back * x0;
      R.inv_rot(r0, r1, r2, v0, v1, v2);
    };
    std::vector<double> Ax((size_t)(mz + 1) * (my + 1) * mx),
        Ay((size_t)(mz + 1) * my * (mx + 1)), Az((size_t)mz * (my + 1) * (mx + 1));
    auto iAx = [&](int z, int y, int x) { return ((size_t)z * (my + 1) + y) * mx + x; };
    auto iAy = [&](int z, int y, int x) { return ((size_t)z * my + y) * (mx + 1) + x; };
    auto iAz = [&](int z, int y, int x) { return ((size_t)z * (my + 1) + y) * (mx + 1) + x; };
    for (int iz = 0; iz < mz + 1; iz++)
      for (int iy = 0; iy < my + 1; iy++)
        for (int ix = 0; ix < mx + 1; ix++) {
          double ta, tb, tc;
          if (ix != mx) apot(px(ix), fy(iy), fz(iz), Ax[iAx(iz, iy, ix)], tb, tc);
          if (iy != my) apot(fx(ix), py(iy), fz(iz), ta, Ay[iAy(iz, iy, ix)], tc);
          if (iz != mz) apot(fx(ix), fy(iy), pz(iz), ta, tb, Az[iAz(iz, iy, ix)]);
        }
    // bfieldi_helper_: B_i = (A_k(j+1) - A_k(j))/dj - (A_j(k+1) - A_j(k))/dk
    V3 fxv = view(b->bfx, mx + 1, my, mz), fyv = view(b->bfy, mx, my + 1, mz),
       fzv = view(b->bfz, mx, my, mz + 1);
    for (int z = 0; z < mz; z++)
      for (int y = 0; y < my; y++)
        for (int x = 0; x < mx + 1; x++)  // dim 0: Aj = Ay, Ak = Az
          fxv.at(x, y, z) = ((Az[iAz(z, y + 1, x)] - Az[iAz(z, y, x)]) / dy -
                             (Ay[iAy(z + 1, y, x)] - Ay[iAy(z, y, x)]) / dz);
    for (int z = 0; z < mz; z++)
      for (int y = 0; y < my + 1; y++)
        for (int x = 0; x < mx; x++)  // dim 1: Aj = Az, Ak = Ax
          fyv.at(x, y, z) = ((Ax[iAx(z + 1, y, x)] - Ax[iAx(z, y, x)]) / dz -
                             (Az[iAz(z, y, x + 1)] - Az[iAz(z, y, x)]) / dx);
    for (int z = 0; z < mz + 1; z++)
      for (int y = 0; y < my; y++)
        for (int x = 0; x < mx; x++)  // dim 2: Aj = Ax, Ak = Ay
          fzv.at(x, y, z) = ((Ay[iAy(z, y, x + 1)] - Ay[iAy(z, y, x)]) / dx -
                             (Ax[iAx(z, y + 1, x)] - Ax[iAx(z, y, x)]) / dy);
    OracleParams dummy{};
    Ctx c;
    setup_ctx(c, &dummy, b);
    center_bfield(c, 0, view(b->bx, mx, my, mz), fxv, 0);
    center_bfield(c, 1, view(b->by, mx, my, mz), fyv, 0);
    center_bfield(c, 2, view(b->bz, mx, my, mz), fzv, 0);
  }

  // setup_fluid_, conserved form (:380-410) with build_linear_HD_inits_
  for (int iz = 0; iz < mz; iz++)
    for (int iy = 0; iy < my; iy++)
      for (int ix = 0; ix < mx; ix++) {
        double x = px(ix), y = py(iy), z = pz(iz);
        double x0, x1, x2;
        R.rot(x, y, z, x0, x1, x2);
        double rho = lin_scalar(density_back, density_ev, amplitude, lambda, x0);
        size_t id = ((size_t)iz * my + iy) * mx + ix;
        b->rho[id] = rho;
        // RotatedVectorInit(LinearVectorInit) (:180-215)
        double tmp = x0 * 2. * PI / lambda;
        double trig = (1 * std::cos(tmp) + (1 - 1) * std::sin(tmp));
        double r0 = mom0_back + amplitude * mom0_ev * trig;
        double r1 = mom1_back + amplitude * mom1_ev * trig;
        double r2 = mom2_back + amplitude * mom2_ev * trig;
        double mpx, mpy, mpz;
        R.inv_rot(r0, r1, r2, mpx, mpy, mpz);
        b->vx[id] = mpx / rho;
        b->vy[id] = mpy / rho;
        b->vz[id] = mpz / rho;
        double etot_dens = lin_scalar(etot_back, etot_ev, amplitude, lambda, x0);
        b->etot[id] = etot_dens / rho;
      }
  if (b->eint) {  // setup_eint_ (:325-372)
    for (int id = 0; id < mx * my * mz; id++) {
      double kinetic = 0.5 * (b->vx[id] * b->vx[id] + b->vy[id] * b->vy[id] +
                              b->vz[id] * b->vz[id]);
      double magnetic = 0.;
      if (mhd_wave)
        magnetic = 0.5 * (b->bx[id] * b->bx[id] + b->by[id] * b->by[id] +
                          b->bz[id] * b->bz[id]) / b->rho[id];
      b->eint[id] = b->etot[id] - kinetic - magnetic;
    }
  }
  return 0;
}

// Cello's cycle for one periodic block (src/Cello/control_charm.cpp:50-150,
// control_stopping.cpp:44-140, control_compute.cpp:57-157): the timestep is
// evaluated on the current (not yet refreshed) ghosts, then the ghosts are
// refreshed and the method computes.
extern "C" int oracle_evolve_periodic(const OracleParams* p, OracleBlock* b,
                                      double stop_time, int max_cycles) {
  double time = 0.0;
  int cycle = 0;
  while (cycle < max_cycles) {
    double dt = oracle_timestep(p, b);
    dt = smin(dt, stop_time - time);
    if (!(time < stop_time)) break;
    oracle_fill_ghosts_periodic(b);
    oracle_step(p, b, dt);
    time += dt;
    cycle++;
  }
  return cycle;
}
