// surrogate_point.cuh — per-point pieces of the learned surrogate of the
// ICE4_SLOW rates (mode_ice4_slow.F90: RCHONI, RVDEPS, RIAGGS, RIAUTS,
// RVDEPG): the 16 input features and the plain-kernel rates of a micro
// point at its first hard pass, the target encoding, and the decoding of
// the network's outputs.  Host-and-device code.
//
// Features (FP32; the network standardises them with the training-set mean
// and spread):
//   0 T   1 ln p   2 ln rho   3 ln max(rv, 1e-12)   4-8 ln max(r, 1e-14) for
//   rc rr ri rs rg   9 cloud fraction   10 Exner   11 dt   12-14 ln lbda of
//   rain, snow, graupel (0 where the species is absent)   15 ssi
// from the state at the start of the step; the targets are the rates the
// plain kernel evaluates at the first hard pass, after its nucleation /
// RRHONG / RIMLTC adjustments (the network learns that map too).
// Targets per rate k (columns of a 16-wide row): 2k = 1 if the rate is
// nonzero, 2k+1 = asinh(rate / SUR_SCALE) / SUR_AMP; columns 10-14 carry
// the rates themselves (FP32) for error statistics.
#pragma once

#include "rain_ice_point.cuh"

namespace ice3sur {

using namespace ice3pt;

constexpr int NFEAT = 16, NRATE = 5, ROW = 16;
constexpr double SUR_SCALE = 1e-12;   // kg/kg/s: rates far above it are coded logarithmically
constexpr double SUR_AMP = 10.0;

// Per-point constants of the step (rain_ice_point's prologue).
ICE3_HD void point_fix(const Cst &c, const Ice3gbRainIceFields &f, long p, PointFix &pf)
{
  const bool sigm = (int)c.SUBG_AUCV_RC == 1 && (int)c.SUBG_PR_PDF == 0;
  pf.exn = ldp(f.exn, p);
  pf.rho = ldp(f.rhodref, p);
  pf.pres = ldp(f.pabs, p);
  pf.zx = fm::fdiv_rn(c.TT, pf.exn);
  pf.lrho = fm::flog(pf.rho);
  pf.rho_mcexvt = fm::fexp(-c.CEXVT * pf.lrho);
  const double irho = fm::frcp(pf.rho);
  pf.rho_mcexvt1 = pf.rho_mcexvt * irho;
  pf.rcrautc = c.CRIAUTC * irho;
  pf.cf = ldp(f.cldfr, p);
  pf.sigma_rc = sigm ? 2.0 * ldp(f.sigs, p) : 0.0;
}

// The 16 features of grid point p from its state at the start of the step,
// in FP32 (they are stored and consumed in FP32): logarithms of the mixing
// ratios, the slope parameters of rain / snow / graupel as
// mode_ice4_tendencies.F90:389-433 forms them, and the supersaturation over
// ice as :303-306 does.
ICE3_HD void feature_row(const Cst &c, const Derived &d, const Ice3gbRainIceFields &f, long p, double dt,
                         float feat[NFEAT])
{
  const float exn = (float)ldp(f.exn, p), pres = (float)ldp(f.pabs, p), rho = (float)ldp(f.rhodref, p);
  const float t = (float)(ldp(f.tht, p) * ldp(f.exn, p));
  const float rv = (float)ldp(f.rvt, p), rc = (float)ldp(f.rct, p), rr = (float)ldp(f.rrt, p);
  const float ri = (float)ldp(f.rit, p), rs = (float)ldp(f.rst, p), rg = (float)ldp(f.rgt, p);
  const float lrho = logf(rho);
  feat[0] = t;
  feat[1] = logf(pres);
  feat[2] = lrho;
  feat[3] = logf(fmaxf(rv, 1e-12f));
  feat[4] = logf(fmaxf(rc, 1e-14f));
  feat[5] = logf(fmaxf(rr, 1e-14f));
  feat[6] = logf(fmaxf(ri, 1e-14f));
  feat[7] = logf(fmaxf(rs, 1e-14f));
  feat[8] = logf(fmaxf(rg, 1e-14f));
  feat[9] = (float)ldp(f.cldfr, p);
  feat[10] = exn;
  feat[11] = (float)dt;
  feat[12] = rr > 0.0f ? (float)d.lLBR + (float)c.LBEXR * (lrho + logf(fmaxf(rr, (float)c.R_RTMIN))) : 0.0f;
  float ls = 0.0f;
  if (rs > 0.0f) {
    if (c.LSNOW_T != 0.0) {
      const float e = t > 263.15f ? 14.554f - 0.0423f * t : 6.226f - 0.0106f * t;
      const float lb = fmaxf(fminf((float)c.LBDAS_MAX, expf(2.302585093f * e)), (float)c.LBDAS_MIN);
      ls = logf(lb * (float)c.TRANS_MP_GAMMAS);
    } else {
      ls = fminf((float)d.lLBDAS_MAX, (float)d.lLBS + (float)c.LBEXS * (lrho + logf(fmaxf(rs, (float)c.S_RTMIN))));
    }
  }
  feat[13] = ls;
  feat[14] = rg > 0.0f ? (float)d.lLBG + (float)c.LBEXG * (lrho + logf(fmaxf(rg, (float)c.G_RTMIN))) : 0.0f;
  const float esi = expf((float)c.ALPI - (float)c.BETAI / t - (float)c.GAMI * logf(t));
  feat[15] = rv * (pres - esi) / ((float)c.EPSILO * esi) - 1.0f;
}

// Features (and, with RATES, the plain FP64 slow rates of the first hard
// pass) of grid point p; false (nothing written) if p is not a micro point
// of rain_ice.
template <bool RATES>
ICE3_HD bool sample_point(const Cst &c, const Derived &d, const double *__restrict__ lut,
                          const Ice3gbRainIceFields &f, long p, double dt, float feat[NFEAT], double rate[NRATE])
{
  const double th = ldp(f.tht, p), rv = ldp(f.rvt, p), rc = ldp(f.rct, p), rr = ldp(f.rrt, p);
  const double ri = ldp(f.rit, p), rs = ldp(f.rst, p), rg = ldp(f.rgt, p);
  const bool micro = gtp(rc, c.C_RTMIN) || gtp(rr, c.R_RTMIN) || gtp(ri, c.I_RTMIN) || gtp(rs, c.S_RTMIN) ||
                     gtp(rg, c.G_RTMIN);
  if (!micro) return false;
  feature_row(c, d, f, p, dt, feat);
  if (RATES) {
    PointFix pf;
    point_fix(c, f, p, pf);
    // first pass of ICE4_STEPPING (mode_ice4_stepping.F90:212-240)
    const double zdev = (c.CPD + c.CPV * rv + c.CL * (rc + rr) + c.CI * (ri + rs + rg)) * pf.exn;
    const double zzt = th * pf.exn;
    const double lsfact = (c.LSTT + (c.CPV - c.CI) * (zzt - c.TT)) / zdev;
    const double lvfact = (c.LVTT + (c.CPV - c.CL) * (zzt - c.TT)) / zdev;
    const double vart[NV] = {th, rv, rc, rr, ri, rs, rg};
    const bool adju = (int)c.SUBG_AUCV_RC == 2 || (int)c.SUBG_AUCV_RI == 2;
    double hl[4] = {0.0, 0.0, 0.0, 0.0}, hi[4] = {0.0, 0.0, 0.0, 0.0};
    if (adju) {
      hl[0] = f.hlc_hcf[p]; hl[2] = f.hlc_hrc[p]; hi[0] = f.hli_hcf[p]; hi[2] = f.hli_hri[p];
      hl[3] = rc - hl[2];
      hi[3] = ri - hi[2];
      hl[1] = pos(rc) ? pf.cf - hl[0] : 0.;
      hi[1] = pos(ri) ? pf.cf - hi[0] : 0.;
    }
    Rates R;
    for (int k = 0; k < NBU; ++k) R.bu[k] = 0.0;
    for (int k = 0; k < NRS; ++k) R.rs[k] = 0.0;
    for (int k = 0; k < NRG; ++k) R.rg[k] = 0.0;
    R.ssi = 0.0;
    double cit = f.cit[p], rainfr = 1.0, A[NV], B[NV];
    tendencies(c, d, lut, false, pf, lvfact, lsfact, cit, zzt, vart, R, rainfr, hl, hi, A, B);
    for (int k = 0; k < NRATE; ++k) rate[k] = R.bu[B_RCHONI + k];
  }
  return true;
}

// Target row of one point (see the header).
ICE3_HD void encode_targets(const double rate[NRATE], float row[ROW])
{
  for (int k = 0; k < NRATE; ++k) {
    row[2 * k] = rate[k] != 0.0 ? 1.0f : 0.0f;
    row[2 * k + 1] = (float)(asinh(rate[k] / SUR_SCALE) / SUR_AMP);
    row[10 + k] = (float)rate[k];
  }
  row[15] = 0.0f;
}

// Slow rates from one output row of the network (logit, coded value per
// rate): zero where the logit says the rate vanishes.
ICE3_HD void decode_rates(const float *y, double rate[NRATE])
{
  for (int k = 0; k < NRATE; ++k) {
    const float u = fminf(fmaxf(y[2 * k + 1], -4.0f), 4.0f);    // |rate| <= 1.2e5 kg/kg/s
    rate[k] = y[2 * k] > 0.0f ? (double)((float)SUR_SCALE * sinhf((float)SUR_AMP * u)) : 0.0;
  }
}

}  // namespace ice3sur
