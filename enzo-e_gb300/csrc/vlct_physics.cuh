// vlct_physics.cuh -- device-side physics of the VL+CT step: ideal-gas EOS,
// PLM slope limiters and the HLLE / HLLC / HLLD Riemann solvers.
//
// Every formula keeps the reference's floating-point operation order so that
// the FP64 instantiation (compiled with --fmad=false) reproduces Enzo-E's CPU
// results bit for bit.  The FP32 instantiation uses the same code in float.
// Reference: src/Enzo/fluid-props/EnzoEOSIdeal.hpp,
// src/Enzo/hydro-mhd/toolkit/EnzoReconstructorPLM.hpp,
// src/Enzo/hydro-mhd/riemann/EnzoRiemann{HLL,HLLC,HLLD,Utils}.hpp.
#pragma once
#include <cuda_runtime.h>

namespace vlct {

enum Solver { SOLVER_HLLE = 0, SOLVER_HLLC = 1, SOLVER_HLLD = 2 };
enum Recon { RECON_NN = 0, RECON_PLM = 1, RECON_PLM_ATHENA = 2 };

// Face-frame ordering of the 8 primitives / fluxes (riemann/EnzoRiemannImpl.hpp:
// 40-56, MHDLUT): rho, B_i, B_j, B_k, v_i, v_j, v_k, p (or etot for fluxes).
enum { L_RHO = 0, L_BI = 1, L_BJ = 2, L_BK = 3, L_VI = 4, L_VJ = 5, L_VK = 6,
       L_E = 7 };

// std::min / std::max semantics of the reference (first argument on ties).
template <class R> __device__ __forceinline__ R smin(R a, R b) {
  return (b < a) ? b : a;
}
template <class R> __device__ __forceinline__ R smax(R a, R b) {
  return (a < b) ? b : a;
}
// enzo_utils::min of three values (utils.hpp:82-89)
template <class R> __device__ __forceinline__ R min3(R a, R b, R c) {
  if (a < b) return (c < a) ? c : a;
  return (c < b) ? c : b;
}
template <class R> __device__ __forceinline__ R sqmag(R i, R j, R k) {
  return ((i * i) + ((j * j) + (k * k)));
}

// ---------------------------------------------------------------- EOS ----
template <class R> __device__ __forceinline__ R cs2(R g, R d, R p) {
  return g * p / d;
}
// fast_magnetosonic_speed, generic cos^2 branch (EnzoEOSIdeal.hpp:133-139)
template <class R>
__device__ __forceinline__ R cfast(R g, R d, R p, R bi, R bj, R bk) {
  const R B2 = sqmag(bi, bj, bk);
  const R c2 = cs2(g, d, p);
  const R inv_density = R(1.0) / d;
  const R va2 = B2 * inv_density;
  const R va2_cos2 = (bi * bi) * inv_density;
  const R s = c2 + va2;
  return sqrt(R(0.5) * (va2 + c2 + sqrt(s * s - R(4.) * c2 * va2_cos2)));
}
// specific internal energy p / ((gamma-1) rho) (EnzoEOSIdeal.hpp:79-82)
template <class R> __device__ __forceinline__ R specific_eint(R g, R d, R p) {
  return p / ((g - R(1.0)) * d);
}
// passive upwinding of the internal energy (EnzoRiemannUtils.hpp:224-249)
template <class R>
__device__ __forceinline__ R eint_flux(R g, R dl, R pl, R dr, R pr, R fd) {
  const R el = specific_eint(g, dl, pl);
  const R er = specific_eint(g, dr, pr);
  const R up = ((fd > R(0)) ? R(1) : R(0)) * el + ((fd <= R(0)) ? R(1) : R(0)) * er;
  return up * fd;
}

// ------------------------------------------------------------ limiters ----
// PLM_EnzoRKLimiter (EnzoReconstructorPLM.hpp:287-302)
template <class R>
__device__ __forceinline__ R limiter_enzo_rk(R vm1, R v, R vp1, R theta) {
  R dv_c = R(0.5) * (vp1 - vm1);
  R dv_l = (v - vm1) * theta;
  R dv_r = (vp1 - v) * theta;
  // sign(dv) in {-1, 0, 1} (the reference's (0 < x) - (x < 0)) as selects,
  // with no integer-to-float conversion
  R sl = (R(0.0) < dv_l) ? R(1.0) : ((dv_l < R(0.0)) ? R(-1.0) : R(0.0));
  R sr = (R(0.0) < dv_r) ? R(1.0) : ((dv_r < R(0.0)) ? R(-1.0) : R(0.0));
  return (R(0.5) * (sl + sr)) * min3(fabs(dv_l), fabs(dv_r), fabs(dv_c));
}
// The same limiter in FP32 with fewer instructions: 0.5 (sgn dl + sgn dr) is
// +-1 when the two one-sided differences share a sign and 0 otherwise (a zero
// difference makes the minimum zero), so the slope is the minimum magnitude
// carrying dl's sign when dl dr > 0, else 0 -- the same value, as sign times
// minimum is exact either way (a product dl dr below the FP32 range flushes
// to 0 under -ftz, as do such differences themselves).
template <>
__device__ __forceinline__ float limiter_enzo_rk<float>(float vm1, float v, float vp1,
                                                        float theta) {
  const float dv_c = 0.5f * (vp1 - vm1);
  const float dv_l = (v - vm1) * theta;
  const float dv_r = (vp1 - v) * theta;
  const float m = fminf(fminf(fabsf(dv_l), fabsf(dv_r)), fabsf(dv_c));
  return (dv_l * dv_r > 0.f) ? copysignf(m, dv_l) : 0.f;
}
// PLM_AthenaLimiter (EnzoReconstructorPLM.hpp:337-345)
template <class R>
__device__ __forceinline__ R limiter_athena(R vm1, R v, R vp1) {
  R dv_l = (v - vm1);
  R dv_r = (vp1 - v);
  R temp = dv_l * dv_r;
  if (temp <= R(0.)) return R(0.);
  return R(2.) * temp / (dv_l + dv_r);
}

// ------------------------------------------------------ Riemann solvers ----
// Output of one face solve, in the face frame: 8 fluxes (flux[L_BI] == 0),
// the passive internal-energy flux and the interface velocity v_i-bar.
template <class R> struct FaceFlux {
  R f[8];
  R eflux;
  R vbar;
};

// HLLD (riemann/EnzoRiemannHLLD.hpp:40-448)
template <class R>
__device__ __forceinline__ void hlld(R g, const R* wli, const R* wri,
                                     FaceFlux<R>& out) {
  const R SMALL = R(1.0e-8);
  const R igm1 = R(1.0) / (g - R(1.0));
  const R pressure_l = wli[L_E], pressure_r = wri[L_E];
  const R bxi = wli[L_BI];
  const R bxsq = bxi * bxi;
  const R pbl = R(0.5) * (bxsq + (wli[L_BJ] * wli[L_BJ] + wli[L_BK] * wli[L_BK]));
  const R pbr = R(0.5) * (bxsq + (wri[L_BJ] * wri[L_BJ] + wri[L_BK] * wri[L_BK]));
  const R kel = R(0.5) * wli[L_RHO] *
                (wli[L_VI] * wli[L_VI] +
                 (wli[L_VJ] * wli[L_VJ] + wli[L_VK] * wli[L_VK]));
  const R ker = R(0.5) * wri[L_RHO] *
                (wri[L_VI] * wri[L_VI] +
                 (wri[L_VJ] * wri[L_VJ] + wri[L_VK] * wri[L_VK]));
  // conserved L/R states: d, mx, my, mz, e, by, bz
  const R uld = wli[L_RHO], uld_mx = wli[L_VI] * uld, uld_my = wli[L_VJ] * uld,
          uld_mz = wli[L_VK] * uld, ule = pressure_l * igm1 + kel + pbl,
          ulby = wli[L_BJ], ulbz = wli[L_BK];
  const R urd = wri[L_RHO], urd_mx = wri[L_VI] * urd, urd_my = wri[L_VJ] * urd,
          urd_mz = wri[L_VK] * urd, ure = pressure_r * igm1 + ker + pbr,
          urby = wri[L_BJ], urbz = wri[L_BK];

  const R cfl = cfast(g, wli[L_RHO], pressure_l, wli[L_BI], wli[L_BJ], wli[L_BK]);
  const R cfr = cfast(g, wri[L_RHO], pressure_r, wri[L_BI], wri[L_BJ], wri[L_BK]);
  R spd0 = smin(wli[L_VI] - cfl, wri[L_VI] - cfr);
  R spd4 = smax(wli[L_VI] + cfl, wri[L_VI] + cfr);

  const R ptl = pressure_l + pbl;
  const R ptr = pressure_r + pbr;
  const R fld = uld_mx;
  const R flmx = uld_mx * wli[L_VI] + ptl - bxsq;
  const R flmy = uld_my * wli[L_VI] - bxi * ulby;
  const R flmz = uld_mz * wli[L_VI] - bxi * ulbz;
  const R fle = wli[L_VI] * (ule + ptl - bxsq) -
                bxi * (wli[L_VJ] * ulby + wli[L_VK] * ulbz);
  const R flby = ulby * wli[L_VI] - bxi * wli[L_VJ];
  const R flbz = ulbz * wli[L_VI] - bxi * wli[L_VK];
  const R frd = urd_mx;
  const R frmx = urd_mx * wri[L_VI] + ptr - bxsq;
  const R frmy = urd_my * wri[L_VI] - bxi * urby;
  const R frmz = urd_mz * wri[L_VI] - bxi * urbz;
  const R fre = wri[L_VI] * (ure + ptr - bxsq) -
                bxi * (wri[L_VJ] * urby + wri[L_VK] * urbz);
  const R frby = urby * wri[L_VI] - bxi * wri[L_VJ];
  const R frbz = urbz * wri[L_VI] - bxi * wri[L_VK];

  const R sdl = spd0 - wli[L_VI];
  const R sdr = spd4 - wri[L_VI];
  const R spd2 = (sdr * urd_mx - sdl * uld_mx + (ptl - ptr)) /
                 (sdr * urd - sdl * uld);
  const R sdml = spd0 - spd2;
  const R sdmr = spd4 - spd2;
  const R sdml_inv = R(1.0) / sdml;
  const R sdmr_inv = R(1.0) / sdmr;
  R lst_d = uld * sdl * sdml_inv;
  R rst_d = urd * sdr * sdmr_inv;
  const R lst_d_inv = R(1.0) / lst_d;
  const R rst_d_inv = R(1.0) / rst_d;
  const R sqrtdl = sqrt(lst_d);
  const R sqrtdr = sqrt(rst_d);
  const R spd1 = spd2 - fabs(bxi) / sqrtdl;
  const R spd3 = spd2 + fabs(bxi) / sqrtdr;

  const R ptstl = ptl + uld * sdl * (spd2 - wli[L_VI]);
  const R ptstr = ptr + urd * sdr * (spd2 - wri[L_VI]);
  const R ptst = R(0.5) * (ptstr + ptstl);

  R lst_mx = lst_d * spd2, lst_my, lst_mz, lst_by, lst_bz;
  if (fabs(uld * sdl * sdml - bxsq) < SMALL * ptst) {
    lst_my = lst_d * wli[L_VJ];
    lst_mz = lst_d * wli[L_VK];
    lst_by = ulby;
    lst_bz = ulbz;
  } else {
    R tmp = bxi * (sdl - sdml) / (uld * sdl * sdml - bxsq);
    lst_my = lst_d * (wli[L_VJ] - ulby * tmp);
    lst_mz = lst_d * (wli[L_VK] - ulbz * tmp);
    tmp = (uld * (sdl * sdl) - bxsq) / (uld * sdl * sdml - bxsq);
    lst_by = ulby * tmp;
    lst_bz = ulbz * tmp;
  }
  const R vbstl = (lst_mx * bxi + (lst_my * lst_by + lst_mz * lst_bz)) * lst_d_inv;
  R lst_e = (sdl * ule - ptl * wli[L_VI] + ptst * spd2 +
             bxi * (wli[L_VI] * bxi + (wli[L_VJ] * ulby + wli[L_VK] * ulbz) -
                    vbstl)) *
            sdml_inv;

  R rst_mx = rst_d * spd2, rst_my, rst_mz, rst_by, rst_bz;
  if (fabs(urd * sdr * sdmr - bxsq) < SMALL * ptst) {
    rst_my = rst_d * wri[L_VJ];
    rst_mz = rst_d * wri[L_VK];
    rst_by = urby;
    rst_bz = urbz;
  } else {
    R tmp = bxi * (sdr - sdmr) / (urd * sdr * sdmr - bxsq);
    rst_my = rst_d * (wri[L_VJ] - urby * tmp);
    rst_mz = rst_d * (wri[L_VK] - urbz * tmp);
    tmp = (urd * (sdr * sdr) - bxsq) / (urd * sdr * sdmr - bxsq);
    rst_by = urby * tmp;
    rst_bz = urbz * tmp;
  }
  const R vbstr = (rst_mx * bxi + (rst_my * rst_by + rst_mz * rst_bz)) * rst_d_inv;
  R rst_e = (sdr * ure - ptr * wri[L_VI] + ptst * spd2 +
             bxi * (wri[L_VI] * bxi + (wri[L_VJ] * urby + wri[L_VK] * urbz) -
                    vbstr)) *
            sdmr_inv;

  R ldst_d, ldst_mx, ldst_my, ldst_mz, ldst_e, ldst_by, ldst_bz;
  R rdst_d, rdst_mx, rdst_my, rdst_mz, rdst_e, rdst_by, rdst_bz;
  if (R(0.5) * bxsq < SMALL * ptst) {
    ldst_d = lst_d; ldst_mx = lst_mx; ldst_my = lst_my; ldst_mz = lst_mz;
    ldst_e = lst_e; ldst_by = lst_by; ldst_bz = lst_bz;
    rdst_d = rst_d; rdst_mx = rst_mx; rdst_my = rst_my; rdst_mz = rst_mz;
    rdst_e = rst_e; rdst_by = rst_by; rdst_bz = rst_bz;
  } else {
    const R invsumd = R(1.0) / (sqrtdl + sqrtdr);
    const R bxsig = (bxi > R(0.0) ? R(1.0) : R(-1.0));
    ldst_d = lst_d;
    rdst_d = rst_d;
    ldst_mx = lst_mx;
    rdst_mx = rst_mx;
    R tmp = invsumd * (sqrtdl * (lst_my * lst_d_inv) +
                       sqrtdr * (rst_my * rst_d_inv) + bxsig * (rst_by - lst_by));
    ldst_my = ldst_d * tmp;
    rdst_my = rdst_d * tmp;
    tmp = invsumd * (sqrtdl * (lst_mz * lst_d_inv) +
                     sqrtdr * (rst_mz * rst_d_inv) + bxsig * (rst_bz - lst_bz));
    ldst_mz = ldst_d * tmp;
    rdst_mz = rdst_d * tmp;
    tmp = invsumd * (sqrtdl * rst_by + sqrtdr * lst_by +
                     bxsig * sqrtdl * sqrtdr *
                         ((rst_my * rst_d_inv) - (lst_my * lst_d_inv)));
    ldst_by = rdst_by = tmp;
    tmp = invsumd * (sqrtdl * rst_bz + sqrtdr * lst_bz +
                     bxsig * sqrtdl * sqrtdr *
                         ((rst_mz * rst_d_inv) - (lst_mz * lst_d_inv)));
    ldst_bz = rdst_bz = tmp;
    tmp = spd2 * bxi + (ldst_my * ldst_by + ldst_mz * ldst_bz) / ldst_d;
    ldst_e = lst_e - sqrtdl * bxsig * (vbstl - tmp);
    rdst_e = rst_e + sqrtdr * bxsig * (vbstr - tmp);
  }

  // jump terms S*(U* - U) (step 6, :308-339)
  const R jl2_d = spd1 * (ldst_d - lst_d), jl2_mx = spd1 * (ldst_mx - lst_mx),
          jl2_my = spd1 * (ldst_my - lst_my), jl2_mz = spd1 * (ldst_mz - lst_mz),
          jl2_e = spd1 * (ldst_e - lst_e), jl2_by = spd1 * (ldst_by - lst_by),
          jl2_bz = spd1 * (ldst_bz - lst_bz);
  const R jl1_d = spd0 * (lst_d - uld), jl1_mx = spd0 * (lst_mx - uld_mx),
          jl1_my = spd0 * (lst_my - uld_my), jl1_mz = spd0 * (lst_mz - uld_mz),
          jl1_e = spd0 * (lst_e - ule), jl1_by = spd0 * (lst_by - ulby),
          jl1_bz = spd0 * (lst_bz - ulbz);
  const R jr2_d = spd3 * (rdst_d - rst_d), jr2_mx = spd3 * (rdst_mx - rst_mx),
          jr2_my = spd3 * (rdst_my - rst_my), jr2_mz = spd3 * (rdst_mz - rst_mz),
          jr2_e = spd3 * (rdst_e - rst_e), jr2_by = spd3 * (rdst_by - rst_by),
          jr2_bz = spd3 * (rdst_bz - rst_bz);
  const R jr1_d = spd4 * (rst_d - urd), jr1_mx = spd4 * (rst_mx - urd_mx),
          jr1_my = spd4 * (rst_my - urd_my), jr1_mz = spd4 * (rst_mz - urd_mz),
          jr1_e = spd4 * (rst_e - ure), jr1_by = spd4 * (rst_by - urby),
          jr1_bz = spd4 * (rst_bz - urbz);

  R* f = out.f;
  if (spd0 >= R(0.0)) {
    f[L_RHO] = fld; f[L_VI] = flmx; f[L_VJ] = flmy; f[L_VK] = flmz;
    f[L_E] = fle; f[L_BJ] = flby; f[L_BK] = flbz;
  } else if (spd4 <= R(0.0)) {
    f[L_RHO] = frd; f[L_VI] = frmx; f[L_VJ] = frmy; f[L_VK] = frmz;
    f[L_E] = fre; f[L_BJ] = frby; f[L_BK] = frbz;
  } else if (spd1 >= R(0.0)) {
    f[L_RHO] = fld + jl1_d; f[L_VI] = flmx + jl1_mx; f[L_VJ] = flmy + jl1_my;
    f[L_VK] = flmz + jl1_mz; f[L_E] = fle + jl1_e; f[L_BJ] = flby + jl1_by;
    f[L_BK] = flbz + jl1_bz;
  } else if (spd2 >= R(0.0)) {
    f[L_RHO] = fld + jl1_d + jl2_d; f[L_VI] = flmx + jl1_mx + jl2_mx;
    f[L_VJ] = flmy + jl1_my + jl2_my; f[L_VK] = flmz + jl1_mz + jl2_mz;
    f[L_E] = fle + jl1_e + jl2_e; f[L_BJ] = flby + jl1_by + jl2_by;
    f[L_BK] = flbz + jl1_bz + jl2_bz;
  } else if (spd3 > R(0.0)) {
    f[L_RHO] = frd + jr1_d + jr2_d; f[L_VI] = frmx + jr1_mx + jr2_mx;
    f[L_VJ] = frmy + jr1_my + jr2_my; f[L_VK] = frmz + jr1_mz + jr2_mz;
    f[L_E] = fre + jr1_e + jr2_e; f[L_BJ] = frby + jr1_by + jr2_by;
    f[L_BK] = frbz + jr1_bz + jr2_bz;
  } else {
    f[L_RHO] = frd + jr1_d; f[L_VI] = frmx + jr1_mx; f[L_VJ] = frmy + jr1_my;
    f[L_VK] = frmz + jr1_mz; f[L_E] = fre + jr1_e; f[L_BJ] = frby + jr1_by;
    f[L_BK] = frbz + jr1_bz;
  }
  f[L_BI] = R(0.0);
  out.eflux = eint_flux(g, wli[L_RHO], pressure_l, wri[L_RHO], pressure_r,
                        f[L_RHO]);
  const R l_coef = (spd0 - wli[L_VI]) / (spd0 - spd2);
  const R r_coef = (spd4 - wri[L_VI]) / (spd4 - spd2);
  if (spd0 > R(0)) {
    out.vbar = wli[L_VI];
  } else if (spd4 < R(0)) {
    out.vbar = wri[L_VI];
  } else if (spd2 >= R(0)) {
    out.vbar = spd2 * l_coef;
  } else {
    out.vbar = spd2 * r_coef;
  }
}

// HLLD in FP32 (EnzoRiemannHLLD.hpp:40-448): the same states, wave speeds
// and flux as the FP64 form, with fewer instructions.  The left and right
// states ride in the two lanes of packed FP32 arithmetic (float2: fadd2 /
// fmul2 / ffma2 on sm_100+), so every side-wise operation is one
// instruction for both sides; each shared denominator is inverted once
// (rsqrt for 1/sqrt(rho*)); the flux is F_side + c1 (U* - U) + c2 (U** - U*)
// with the coefficients chosen in the reference's case order.  Differences
// from the FP64 form lie only in rounding.
namespace packed {
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 s2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b as one fused operation: b * -1 + a is exact before its one rounding
__device__ __forceinline__ float2 sub(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
}
}  // namespace packed

template <>
__device__ __forceinline__ void hlld<float>(float g, const float* wli, const float* wri,
                                            FaceFlux<float>& out) {
  using namespace packed;
  const float SMALL = 1.0e-8f;
  const float igm1 = 1.0f / (g - 1.0f);
  const float bxi = wli[L_BI], bxsq = bxi * bxi;
  const float2 BXSQ = s2(bxsq), BXI = s2(bxi), HALF = s2(0.5f);
  const float2 p = f2(wli[L_E], wri[L_E]);
  const float2 d = f2(wli[L_RHO], wri[L_RHO]);
  const float2 u = f2(wli[L_VI], wri[L_VI]);
  const float2 vj = f2(wli[L_VJ], wri[L_VJ]), vk = f2(wli[L_VK], wri[L_VK]);
  const float2 by = f2(wli[L_BJ], wri[L_BJ]), bz = f2(wli[L_BK], wri[L_BK]);
  const float2 inv_d = f2(1.0f / d.x, 1.0f / d.y);
  const float2 bt = fma(by, by, mul(bz, bz));
  const float2 b2 = add(BXSQ, bt);
  const float2 pb = mul(HALF, b2);
  const float2 ke = mul(mul(HALF, d), fma(u, u, fma(vj, vj, mul(vk, vk))));
  const float2 ue = add(fma(p, s2(igm1), ke), pb);
  // fast speeds (EnzoEOSIdeal.hpp:133-139)
  const float2 c2 = mul(mul(s2(g), p), inv_d);
  const float2 va2 = mul(b2, inv_d);
  const float2 vac2 = mul(BXSQ, inv_d);
  const float2 q = add(c2, va2);
  const float2 disc = fma(q, q, mul(mul(s2(-4.0f), c2), vac2));
  const float2 inner = add(q, f2(sqrtf(disc.x), sqrtf(disc.y)));
  const float2 cfh = mul(HALF, inner);
  const float2 cf = f2(sqrtf(cfh.x), sqrtf(cfh.y));
  const float2 um = sub(u, cf), up = add(u, cf);
  const float spd0 = fminf(um.x, um.y);
  const float spd4 = fmaxf(up.x, up.y);
  const float2 pt = add(p, pb);
  // side fluxes: d, mx, my, mz, e, by, bz
  const float2 du = mul(d, u);
  const float2 vbt = fma(vj, by, mul(vk, bz));
  const float2 ptb = sub(pt, BXSQ);
  const float2 F[7] = {du, fma(du, u, ptb), sub(mul(du, vj), mul(BXI, by)),
                       sub(mul(du, vk), mul(BXI, bz)), sub(mul(u, add(ue, ptb)), mul(BXI, vbt)),
                       sub(mul(by, u), mul(BXI, vj)), sub(mul(bz, u), mul(BXI, vk))};
  const float2 S04 = f2(spd0, spd4);
  const float2 sd = sub(S04, u);
  const float2 sdd = mul(sd, d);
  const float2 sddu = mul(sdd, u);
  const float spd2 = (sddu.y - sddu.x + (pt.x - pt.y)) / (sdd.y - sdd.x);
  const float2 SPD2 = s2(spd2);
  const float2 sdm = sub(S04, SPD2);
  const float2 st_d = f2(sdd.x / sdm.x, sdd.y / sdm.y);
  const float2 isq = f2(rsqrtf(st_d.x), rsqrtf(st_d.y));
  const float2 sqrtd = mul(st_d, isq);
  const float2 st_d_inv = mul(isq, isq);
  const float spd1 = spd2 - fabsf(bxi) * isq.x;
  const float spd3 = spd2 + fabsf(bxi) * isq.y;
  const float2 ptw = fma(sdd, sub(SPD2, u), pt);
  const float ptst = 0.5f * (ptw.y + ptw.x);
  // single-star states, both sides at once: d, mx, my, mz, e, by, bz; a
  // side whose |d s (s - s_M) - B_x^2| is below SMALL p* keeps its
  // transverse B and velocity (t1 = 0, t2 = 1)
  const float2 den = sub(mul(sdd, sdm), BXSQ);
  const float thr = SMALL * ptst;
  const bool degl = fabsf(den.x) < thr, degr = fabsf(den.y) < thr;
  const float2 iden = f2(1.0f / den.x, 1.0f / den.y);
  float2 t1 = mul(mul(BXI, sub(sd, sdm)), iden);
  float2 t2 = mul(sub(mul(sdd, sd), BXSQ), iden);
  t1 = f2(degl ? 0.0f : t1.x, degr ? 0.0f : t1.y);
  t2 = f2(degl ? 1.0f : t2.x, degr ? 1.0f : t2.y);
  float2 Us[7];
  Us[0] = st_d;
  Us[1] = mul(st_d, SPD2);
  Us[2] = mul(st_d, sub(vj, mul(by, t1)));
  Us[3] = mul(st_d, sub(vk, mul(bz, t1)));
  Us[5] = mul(by, t2);
  Us[6] = mul(bz, t2);
  const float2 vbst = mul(fma(Us[1], BXI, fma(Us[2], Us[5], mul(Us[3], Us[6]))), st_d_inv);
  const float2 e_num =
      add(fma(SPD2, s2(ptst), sub(mul(sd, ue), mul(pt, u))), mul(BXI, sub(fma(u, BXI, vbt), vbst)));
  Us[4] = f2(e_num.x / sdm.x, e_num.y / sdm.y);
  // double-star states
  float2 Ud[7];
#pragma unroll
  for (int k = 0; k < 7; k++) Ud[k] = Us[k];
  if (!(0.5f * bxsq < SMALL * ptst)) {
    const float invsumd = 1.0f / (sqrtd.x + sqrtd.y);
    const float bxsig = bxi > 0.0f ? 1.0f : -1.0f;
    const float2 vy = mul(Us[2], st_d_inv), vz = mul(Us[3], st_d_inv);
    const float2 wvy = mul(sqrtd, vy), wvz = mul(sqrtd, vz);
    const float ty = invsumd * (wvy.x + wvy.y + bxsig * (Us[5].y - Us[5].x));
    const float tz = invsumd * (wvz.x + wvz.y + bxsig * (Us[6].y - Us[6].x));
    Ud[2] = mul(Us[0], s2(ty));
    Ud[3] = mul(Us[0], s2(tz));
    const float sq = bxsig * sqrtd.x * sqrtd.y;
    const float byd = invsumd * (sqrtd.x * Us[5].y + sqrtd.y * Us[5].x + sq * (vy.y - vy.x));
    const float bzd = invsumd * (sqrtd.x * Us[6].y + sqrtd.y * Us[6].x + sq * (vz.y - vz.x));
    Ud[5] = s2(byd);
    Ud[6] = s2(bzd);
    // v** . B** from the left side's values for both (as the scalar form)
    const float tl = spd2 * bxi + (Ud[2].x * byd + Ud[3].x * bzd) * st_d_inv.x;
    const float2 sg = mul(sqrtd, f2(-bxsig, bxsig));
    Ud[4] = fma(sg, sub(vbst, s2(tl)), Us[4]);
  }
  // F = F_side + c1 (U* - U) + c2 (U** - U*), the cases in the reference's
  // order: F_L (spd0 >= 0), F_R (spd4 <= 0), then by the signs of spd1..spd3
  const bool outer = spd0 >= 0.0f || spd4 <= 0.0f;
  const bool left = spd0 >= 0.0f || (!(spd4 <= 0.0f) && spd2 >= 0.0f);
  const float c1 = outer ? 0.0f : (left ? spd0 : spd4);
  const float c2v = outer ? 0.0f : (left ? (spd1 >= 0.0f ? 0.0f : spd1)
                                         : (spd3 > 0.0f ? spd3 : 0.0f));
  const float2 U[7] = {d, du, mul(d, vj), mul(d, vk), ue, by, bz};
  float Fo[7];
#pragma unroll
  for (int k = 0; k < 7; k++) {
    const float Fk = left ? F[k].x : F[k].y, Uk = left ? U[k].x : U[k].y;
    const float Usk = left ? Us[k].x : Us[k].y, Udk = left ? Ud[k].x : Ud[k].y;
    Fo[k] = Fk + c1 * (Usk - Uk) + c2v * (Udk - Usk);
  }
  out.f[L_RHO] = Fo[0]; out.f[L_VI] = Fo[1]; out.f[L_VJ] = Fo[2]; out.f[L_VK] = Fo[3];
  out.f[L_E] = Fo[4]; out.f[L_BJ] = Fo[5]; out.f[L_BK] = Fo[6];
  out.f[L_BI] = 0.0f;
  out.eflux = eint_flux(g, d.x, p.x, d.y, p.y, out.f[L_RHO]);
  if (spd0 > 0.0f) out.vbar = u.x;
  else if (spd4 < 0.0f) out.vbar = u.y;
  else out.vbar = spd2 * (spd2 >= 0.0f ? sd.x / sdm.x : sd.y / sdm.y);
}

// conserved state from primitives (EnzoRiemannUtils.hpp:48-82)
template <class R, bool MHD>
__device__ __forceinline__ void conserved(R g, const R* w, R* u) {
  u[L_RHO] = w[L_RHO];
  u[L_BI] = w[L_BI]; u[L_BJ] = w[L_BJ]; u[L_BK] = w[L_BK];
  u[L_VI] = w[L_VI] * w[L_RHO];
  u[L_VJ] = w[L_VJ] * w[L_RHO];
  u[L_VK] = w[L_VK] * w[L_RHO];
  const R density = w[L_RHO], pressure = w[L_E];
  const R internal_edens = pressure / (g - R(1.0));
  const R kinetic_edens = R(0.5) * density * sqmag(w[L_VI], w[L_VJ], w[L_VK]);
  const R magnetic_edens = MHD ? R(0.5) * sqmag(w[L_BI], w[L_BJ], w[L_BK])
                               : R(0.5) * sqmag(R(0), R(0), R(0));
  u[L_E] = internal_edens + kinetic_edens + magnetic_edens;
}

// ideal-MHD fluxes (EnzoRiemannUtils.hpp:111-149)
template <class R, bool MHD>
__device__ __forceinline__ void physical_flux(const R* w, const R* u, R pressure,
                                              R* f) {
  const R vi = w[L_VI], vj = w[L_VJ], vk = w[L_VK];
  const R Bi = MHD ? w[L_BI] : R(0), Bj = MHD ? w[L_BJ] : R(0),
          Bk = MHD ? w[L_BK] : R(0);
  const R etot = u[L_E];
  const R ptot = pressure + R(0.5) * sqmag(Bi, Bj, Bk);
  const R mom_i = u[L_VI];
  f[L_RHO] = mom_i;
  f[L_VI] = mom_i * vi - Bi * Bi + ptot;
  f[L_VJ] = mom_i * vj - Bj * Bi;
  f[L_VK] = mom_i * vk - Bk * Bi;
  f[L_E] = ((etot + ptot) * vi - (Bi * vi + (Bj * vj + Bk * vk)) * Bi);
  f[L_BI] = R(0);
  f[L_BJ] = Bj * vi - Bi * vj;
  f[L_BK] = Bk * vi - Bi * vk;
}

// Einfeldt wave speeds with Roe averages (EnzoRiemannHLL.hpp:44-172)
template <class R, bool MHD>
__device__ __forceinline__ void einfeldt(R g, const R* wl, const R* wr,
                                         const R* Ul, const R* Ur, R pl, R pr,
                                         R* bp, R* bm) {
  R c_l, c_r;
  if (MHD) {
    c_l = cfast(g, wl[L_RHO], pl, wl[L_BI], wl[L_BJ], wl[L_BK]);
    c_r = cfast(g, wr[L_RHO], pr, wr[L_BI], wr[L_BJ], wr[L_BK]);
  } else {
    c_l = sqrt(cs2(g, wl[L_RHO], pl));
    c_r = sqrt(cs2(g, wr[L_RHO], pr));
  }
  const R left_speed = (wl[L_VI] - c_l);
  const R right_speed = (wr[L_VI] + c_r);
  const R sqrtrho_l = sqrt(wl[L_RHO]);
  const R sqrtrho_r = sqrt(wr[L_RHO]);
  const R inv_tot = R(1.0) / (sqrtrho_l + sqrtrho_r);
  const R vi_roe = (sqrtrho_l * wl[L_VI] + sqrtrho_r * wr[L_VI]) * inv_tot;
  const R vj_roe = (sqrtrho_l * wl[L_VJ] + sqrtrho_r * wr[L_VJ]) * inv_tot;
  const R vk_roe = (sqrtrho_l * wl[L_VK] + sqrtrho_r * wr[L_VK]) * inv_tot;
  const R v_roe2 = vi_roe * vi_roe + vj_roe * vj_roe + vk_roe * vk_roe;
  R ptot_l = pl, ptot_r = pr;
  if (MHD) {
    ptot_l += R(0.5) * sqmag(wl[L_BI], wl[L_BJ], wl[L_BK]);
    ptot_r += R(0.5) * sqmag(wr[L_BI], wr[L_BJ], wr[L_BK]);
  }
  const R h_l = (Ul[L_E] + ptot_l) / wl[L_RHO];
  const R h_r = (Ur[L_E] + ptot_r) / wr[L_RHO];
  const R h_roe = (sqrtrho_l * h_l + sqrtrho_r * h_r) * inv_tot;
  R c_roe;
  if (MHD) {  // roe_cfast_ (:134-172)
    const R rho_roe = sqrtrho_l * sqrtrho_r;
    const R bi_roe = wl[L_BI];
    const R bj_roe = (sqrtrho_l * wr[L_BJ] + sqrtrho_r * wl[L_BJ]) * inv_tot;
    const R bk_roe = (sqrtrho_l * wr[L_BK] + sqrtrho_r * wl[L_BK]) * inv_tot;
    const R b_roe2 = bi_roe * bi_roe + bj_roe * bj_roe + bk_roe * bk_roe;
    const R gamma_prime = g - R(1.);
    const R dbj = wl[L_BJ] - wr[L_BJ];
    const R dbk = wl[L_BK] - wr[L_BK];
    const R x_prime =
        ((dbj * dbj + dbk * dbk) * R(0.5) * (gamma_prime - R(1)) * inv_tot);
    const R y_prime =
        ((gamma_prime - R(1)) * (wl[L_RHO] + wr[L_RHO]) * R(0.5) / rho_roe);
    const R tilde_a2 =
        (gamma_prime * (h_roe - R(0.5) * v_roe2 - b_roe2 / rho_roe) - x_prime);
    const R tilde_vai2 = bi_roe * bi_roe / rho_roe;
    const R tilde_va2 = (tilde_vai2 + (gamma_prime - y_prime) *
                                          (bj_roe * bj_roe + bk_roe * bk_roe) /
                                          rho_roe);
    const R s = tilde_a2 + tilde_va2;
    c_roe = sqrt(R(0.5) * (tilde_a2 + tilde_va2 +
                           sqrt(s * s - R(4) * tilde_a2 * tilde_vai2)));
  } else {  // roe_cs_ (:123-130)
    const R temp = h_roe - R(0.5) * v_roe2;
    c_roe = sqrt((g - R(1)) * smax(temp, R(0.)));
  }
  *bp = fmax(vi_roe + c_roe, right_speed);
  *bm = fmin(vi_roe - c_roe, left_speed);
}

// HLLE for MHD (EnzoRiemannHLL.hpp:238-345)
template <class R>
__device__ __forceinline__ void hlle(R g, const R* wl, const R* wr,
                                     FaceFlux<R>& out) {
  const R pl = wl[L_E], pr = wr[L_E];
  R Ul[8], Ur[8], Fl[8], Fr[8];
  conserved<R, true>(g, wl, Ul);
  conserved<R, true>(g, wr, Ur);
  physical_flux<R, true>(wl, Ul, pl, Fl);
  physical_flux<R, true>(wr, Ur, pr, Fr);
  R bp, bm;
  einfeldt<R, true>(g, wl, wr, Ul, Ur, pl, pr, &bp, &bm);
  bp = fmax(bp, R(0.0));
  bm = fmin(bm, R(0.0));
  const R inv_speed_diff = R(1.) / (bp - bm);
#pragma unroll
  for (int k = 0; k < 8; k++) {
    out.f[k] = ((bp * Fl[k] - bm * Fr[k] + (Ur[k] - Ul[k]) * bp * bm) *
                inv_speed_diff);
  }
  out.eflux = eint_flux(g, wl[L_RHO], pl, wr[L_RHO], pr, out.f[L_RHO]);
  out.vbar = (bp * wl[L_VI] - bm * wr[L_VI]) * inv_speed_diff;
}

// HLLC for hydrodynamics (EnzoRiemannHLLC.hpp:34-172)
template <class R>
__device__ __forceinline__ void hllc(R g, const R* wl, const R* wr,
                                     FaceFlux<R>& out) {
  const R pl = wl[L_E], pr = wr[L_E];
  R Ul[8], Ur[8];
  conserved<R, false>(g, wl, Ul);
  conserved<R, false>(g, wr, Ur);
  R cs_l, cs_r;
  einfeldt<R, false>(g, wl, wr, Ul, Ur, pl, pr, &cs_r, &cs_l);
  const R bm = fmin(cs_l, R(0.0));
  const R bp = fmax(cs_r, R(0.0));
  const R tl = (pl - (cs_l - wl[L_VI]) * wl[L_RHO] * wl[L_VI]);
  const R tr = (pr - (cs_r - wr[L_VI]) * wr[L_RHO] * wr[L_VI]);
  const R dl = wl[L_RHO] * (cs_l - wl[L_VI]);
  const R dr = -wr[L_RHO] * (cs_r - wr[L_VI]);
  const R q1 = R(1.0) / (dl + dr);
  const R cw = (tr - tl) * q1;
  R cp = (dl * tr + dr * tl) * q1;
  R sl, sr, sm;
  if (cw >= R(0.)) {
    sl = cw / (cw - bm);
    sr = R(0.);
    sm = -bm / (cw - bm);
  } else {
    sl = R(0.);
    sr = -cw / (bp - cw);
    sm = bp / (bp - cw);
  }
  cp = smax(cp, R(0.));
  const R momentumi_l = Ul[L_VI], momentumi_r = Ur[L_VI];
  const R dfl = momentumi_l - bm * wl[L_RHO];
  const R dfr = momentumi_r - bp * wr[L_RHO];
  const R ufl = momentumi_l * (wl[L_VI] - bm) + pl;
  const R ufr = momentumi_r * (wr[L_VI] - bp) + pr;
  const R vfl = (wl[L_RHO] * wl[L_VJ] * (wl[L_VI] - bm));
  const R vfr = (wr[L_RHO] * wr[L_VJ] * (wr[L_VI] - bp));
  const R wfl = (wl[L_RHO] * wl[L_VK] * (wl[L_VI] - bm));
  const R wfr = (wr[L_RHO] * wr[L_VK] * (wr[L_VI] - bp));
  const R efl = (Ul[L_E] * (wl[L_VI] - bm) + pl * wl[L_VI]);
  const R efr = (Ur[L_E] * (wr[L_VI] - bp) + pr * wr[L_VI]);
  out.f[L_RHO] = sl * dfl + sr * dfr;
  out.f[L_VI] = sl * ufl + sr * ufr;
  out.f[L_VJ] = sl * vfl + sr * vfr;
  out.f[L_VK] = sl * wfl + sr * wfr;
  out.f[L_E] = sl * efl + sr * efr;
  out.f[L_VI] += (sm * cp);
  out.f[L_E] += (sm * cp * cw);
  out.f[L_BI] = out.f[L_BJ] = out.f[L_BK] = R(0);
  out.eflux = eint_flux(g, wl[L_RHO], pl, wr[L_RHO], pr, out.f[L_RHO]);
  out.vbar = (sl * (wl[L_VI] - bm) + sr * (wr[L_VI] - bp));
}

// HLLE in FP32 (EnzoRiemannHLL.hpp:44-345): the same states, Einfeldt
// speeds and flux as the FP64 form, the left and right states in the two
// lanes of packed FP32 arithmetic.  Differences from the FP64 form lie only
// in rounding.
template <>
__device__ __forceinline__ void hlle<float>(float g, const float* wl, const float* wr,
                                            FaceFlux<float>& out) {
  using namespace packed;
  const float2 HALF = s2(0.5f);
  const float2 p = f2(wl[L_E], wr[L_E]);
  const float2 d = f2(wl[L_RHO], wr[L_RHO]);
  const float2 u = f2(wl[L_VI], wr[L_VI]);
  const float2 vj = f2(wl[L_VJ], wr[L_VJ]), vk = f2(wl[L_VK], wr[L_VK]);
  const float2 bi = f2(wl[L_BI], wr[L_BI]);
  const float2 bj = f2(wl[L_BJ], wr[L_BJ]), bk = f2(wl[L_BK], wr[L_BK]);
  const float2 inv_d = f2(1.0f / d.x, 1.0f / d.y);
  const float gm1 = g - 1.0f;
  // conserved states and physical fluxes (EnzoRiemannUtils.hpp:48-149)
  const float2 mi = mul(u, d), mj = mul(vj, d), mk = mul(vk, d);
  const float2 b2 = fma(bi, bi, fma(bj, bj, mul(bk, bk)));
  const float2 v2 = fma(u, u, fma(vj, vj, mul(vk, vk)));
  const float2 E = add(fma(p, s2(1.0f / gm1), mul(mul(HALF, d), v2)), mul(HALF, b2));
  const float2 pt = fma(HALF, b2, p);
  const float2 vb = fma(bi, u, fma(bj, vj, mul(bk, vk)));
  float2 F[8], U[8];
  U[L_RHO] = d;
  U[L_BI] = bi;
  U[L_BJ] = bj;
  U[L_BK] = bk;
  U[L_VI] = mi;
  U[L_VJ] = mj;
  U[L_VK] = mk;
  U[L_E] = E;
  F[L_RHO] = mi;
  F[L_BI] = s2(0.0f);
  F[L_BJ] = sub(mul(bj, u), mul(bi, vj));
  F[L_BK] = sub(mul(bk, u), mul(bi, vk));
  F[L_VI] = fma(mi, u, sub(pt, mul(bi, bi)));
  F[L_VJ] = sub(mul(mi, vj), mul(bj, bi));
  F[L_VK] = sub(mul(mi, vk), mul(bk, bi));
  F[L_E] = sub(mul(add(E, pt), u), mul(vb, bi));
  // Einfeldt speeds: fast speeds, Roe averages, Roe fast speed
  const float2 c2 = mul(mul(s2(g), p), inv_d);
  const float2 va2 = mul(b2, inv_d);
  const float2 vac2 = mul(mul(bi, bi), inv_d);
  const float2 sfs = add(c2, va2);
  const float2 disc = fma(sfs, sfs, mul(mul(s2(-4.0f), c2), vac2));
  const float2 cfh = mul(HALF, add(sfs, f2(sqrtf(disc.x), sqrtf(disc.y))));
  const float left_speed = u.x - sqrtf(cfh.x), right_speed = u.y + sqrtf(cfh.y);
  const float2 sq = f2(sqrtf(d.x), sqrtf(d.y));
  const float inv_tot = 1.0f / (sq.x + sq.y);
  const float2 su = mul(sq, u), sv = mul(sq, vj), sw = mul(sq, vk);
  const float vi_roe = (su.x + su.y) * inv_tot;
  const float vj_roe = (sv.x + sv.y) * inv_tot;
  const float vk_roe = (sw.x + sw.y) * inv_tot;
  const float v_roe2 = vi_roe * vi_roe + vj_roe * vj_roe + vk_roe * vk_roe;
  const float2 sh = mul(sq, mul(add(E, pt), inv_d));
  const float h_roe = (sh.x + sh.y) * inv_tot;
  const float rho_roe = sq.x * sq.y;
  const float inv_rho_roe = 1.0f / rho_roe;
  const float bi_roe = bi.x;
  const float bj_roe = (sq.x * bj.y + sq.y * bj.x) * inv_tot;
  const float bk_roe = (sq.x * bk.y + sq.y * bk.x) * inv_tot;
  const float bt_roe2 = bj_roe * bj_roe + bk_roe * bk_roe;
  const float b_roe2 = bi_roe * bi_roe + bt_roe2;
  const float dbj = bj.x - bj.y, dbk = bk.x - bk.y;
  const float x_prime = (dbj * dbj + dbk * dbk) * 0.5f * (gm1 - 1.0f) * inv_tot;
  const float y_prime = (gm1 - 1.0f) * (d.x + d.y) * 0.5f * inv_rho_roe;
  const float tilde_a2 = gm1 * (h_roe - 0.5f * v_roe2 - b_roe2 * inv_rho_roe) - x_prime;
  const float tilde_vai2 = bi_roe * bi_roe * inv_rho_roe;
  const float tilde_va2 = tilde_vai2 + (gm1 - y_prime) * bt_roe2 * inv_rho_roe;
  const float sr = tilde_a2 + tilde_va2;
  const float c_roe =
      sqrtf(0.5f * (tilde_a2 + tilde_va2 + sqrtf(sr * sr - 4.0f * tilde_a2 * tilde_vai2)));
  const float bp = fmaxf(fmaxf(vi_roe + c_roe, right_speed), 0.0f);
  const float bm = fminf(fminf(vi_roe - c_roe, left_speed), 0.0f);
  const float inv_speed_diff = 1.0f / (bp - bm);
  const float bpbm = bp * bm;
  const float2 BPM = f2(bp, -bm);
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const float2 t = mul(BPM, F[k]);
    out.f[k] = ((t.x + t.y) + (U[k].y - U[k].x) * bpbm) * inv_speed_diff;
  }
  out.eflux = eint_flux(g, d.x, p.x, d.y, p.y, out.f[L_RHO]);
  out.vbar = (bp * u.x - bm * u.y) * inv_speed_diff;
}

// HLLC in FP32 (EnzoRiemannHLLC.hpp:34-172 with the Einfeldt speeds of
// EnzoRiemannHLL.hpp:44-172): the same states, speeds and flux as the FP64
// form, the left and right states in the two lanes of packed FP32
// arithmetic.  Differences from the FP64 form lie only in rounding.
template <>
__device__ __forceinline__ void hllc<float>(float g, const float* wl, const float* wr,
                                            FaceFlux<float>& out) {
  using namespace packed;
  const float2 HALF = s2(0.5f);
  const float2 p = f2(wl[L_E], wr[L_E]);
  const float2 d = f2(wl[L_RHO], wr[L_RHO]);
  const float2 u = f2(wl[L_VI], wr[L_VI]);
  const float2 vj = f2(wl[L_VJ], wr[L_VJ]), vk = f2(wl[L_VK], wr[L_VK]);
  const float2 inv_d = f2(1.0f / d.x, 1.0f / d.y);
  const float gm1 = g - 1.0f;
  // conserved momentum and total energy density
  const float2 mom = mul(u, d);
  const float2 v2 = fma(u, u, fma(vj, vj, mul(vk, vk)));
  const float2 E = fma(p, s2(1.0f / gm1), mul(mul(HALF, d), v2));
  // Einfeldt speeds: sound speeds, Roe averages
  const float2 c2 = mul(mul(s2(g), p), inv_d);
  const float left_speed = u.x - sqrtf(c2.x), right_speed = u.y + sqrtf(c2.y);
  const float2 sq = f2(sqrtf(d.x), sqrtf(d.y));
  const float inv_tot = 1.0f / (sq.x + sq.y);
  const float2 su = mul(sq, u), sv = mul(sq, vj), sw = mul(sq, vk);
  const float vi_roe = (su.x + su.y) * inv_tot;
  const float vj_roe = (sv.x + sv.y) * inv_tot;
  const float vk_roe = (sw.x + sw.y) * inv_tot;
  const float v_roe2 = vi_roe * vi_roe + vj_roe * vj_roe + vk_roe * vk_roe;
  const float2 sh = mul(sq, mul(add(E, p), inv_d));
  const float h_roe = (sh.x + sh.y) * inv_tot;
  const float c_roe = sqrtf(gm1 * smax(h_roe - 0.5f * v_roe2, 0.0f));
  const float cs_r = fmaxf(vi_roe + c_roe, right_speed);
  const float cs_l = fminf(vi_roe - c_roe, left_speed);
  const float bm = fminf(cs_l, 0.0f);
  const float bp = fmaxf(cs_r, 0.0f);
  // contact speed and pressure
  const float2 cu = sub(f2(cs_l, cs_r), u);
  const float2 t = sub(p, mul(cu, mom));
  const float2 dd = mul(d, cu);
  const float dl = dd.x, dr = -dd.y;
  const float q1 = 1.0f / (dl + dr);
  const float cw = (t.y - t.x) * q1;
  float cp = (dl * t.y + dr * t.x) * q1;
  float sl, sr, sm;
  if (cw >= 0.0f) {
    sl = cw / (cw - bm);
    sr = 0.0f;
    sm = -bm / (cw - bm);
  } else {
    sl = 0.0f;
    sr = -cw / (bp - cw);
    sm = bp / (bp - cw);
  }
  cp = smax(cp, 0.0f);
  // side fluxes relative to the outer wave speeds
  const float2 B = f2(bm, bp);
  const float2 ub = sub(u, B);
  const float2 df = sub(mom, mul(B, d));
  const float2 uf = fma(mom, ub, p);
  const float2 vf = mul(mul(d, vj), ub);
  const float2 wf = mul(mul(d, vk), ub);
  const float2 ef = fma(E, ub, mul(p, u));
  const float2 SLR = f2(sl, sr);
  const float2 frho = mul(SLR, df), fu = mul(SLR, uf), fv = mul(SLR, vf), fw = mul(SLR, wf),
               fe = mul(SLR, ef), fvb = mul(SLR, ub);
  out.f[L_RHO] = frho.x + frho.y;
  out.f[L_VI] = (fu.x + fu.y) + sm * cp;
  out.f[L_VJ] = fv.x + fv.y;
  out.f[L_VK] = fw.x + fw.y;
  out.f[L_E] = (fe.x + fe.y) + sm * cp * cw;
  out.f[L_BI] = out.f[L_BJ] = out.f[L_BK] = 0.0f;
  out.eflux = eint_flux(g, d.x, p.x, d.y, p.y, out.f[L_RHO]);
  out.vbar = fvb.x + fvb.y;
}

template <int SOLVER, class R>
__device__ __forceinline__ void riemann(R g, const R* wl, const R* wr,
                                        FaceFlux<R>& out) {
  if (SOLVER == SOLVER_HLLD) hlld<R>(g, wl, wr, out);
  else if (SOLVER == SOLVER_HLLE) hlle<R>(g, wl, wr, out);
  else hllc<R>(g, wl, wr, out);
}

}  // namespace vlct
