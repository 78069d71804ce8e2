// ice_adjust_point.cuh — per-grid-point saturation adjustment (forward) and
// its hand-written reverse-mode derivative; host-and-device code.
//
// Forward: restates src/ice3/jax/stencils/ice_adjust.py:26-398 (IceAdjustJAX)
// for one grid point.  The kernels in ice_adjust.cu (forward) and
// ice_adjust_vjp.cu (adjoint) run it per lane; the tests build it for the
// host as well.
#pragma once

#include "ice3gb_device.cuh"

namespace ice3ia {

struct IaIn {
  double sigqsat, pabs, sigs, th, exn, exn_ref, rho, rv, rc, ri, rr, rs, rg, cf_mf, rc_mf, ri_mf;
  double rvs, rcs, ris, ths;
};
struct IaOut {
  double t, rv_out, rc_out, ri_out, cldfr, hlc_hrc, hlc_hcf, hli_hri, hli_hcf, cph, lv, ls;
  double rvs, rcs, ris, ths;
};
// (the members are also addressed as arrays of 20 / 16 doubles)
static_assert(sizeof(IaIn) == 20 * sizeof(double), "IaIn layout");
static_assert(sizeof(IaOut) == 16 * sizeof(double), "IaOut layout");

// Triangle-PDF subgrid autoconversion (stencils/ice_adjust.py:316-341).
// 1 / max(1e-20, w_dt)^2 is formed only in the branches that read it (with
// no mass flux, w_dt = 0, it would be an IEEE division of 1e-40).
ICE3_HD void triangle_pdf(double w_dt, double crit, double cf_mf, double &hcf, double &hr)
{
  if (fgt(w_dt, crit)) {
    const double inv_w2 = fm::frcp(sq(nmax(1e-20, w_dt)));
    const double cc = crit * cf_mf;
    hcf = 1.0 - 0.5 * sq(cc) * inv_w2;
    hr = w_dt - cc * cc * cc * (inv_w2 * (1.0 / 3.0));
  } else if (fge(crit, 2.0 * w_dt)) {
    hcf = 0.0;
    hr = 0.0;
  } else {
    const double inv_w2 = fm::frcp(sq(nmax(1e-20, w_dt)));
    hcf = 0.5 * sq(2.0 * w_dt - crit) * inv_w2;
    hr = (4.0 * w_dt * w_dt * w_dt - 3.0 * w_dt * sq(crit) + crit * crit * crit) * (inv_w2 * (1.0 / 3.0));
  }
  hcf *= cf_mf;
}

// SRC_1D of condensation.F90:208-214 (index -22..11; the same values as
// src/ice3/phyex_common/lookup_table.py:4-40): s'r_c'/sigma_s^2 of the
// Gaussian subgrid scheme tabulated against 2 q1.
#define ICE3_SRC_1D_VALUES                                                                                      \
  0., 0., 2.0094444e-04, 0.316670e-03, 4.9965648e-04, 0.785956e-03, 1.2341294e-03, 0.193327e-02,            \
      3.0190963e-03, 0.470144e-02, 7.2950651e-03, 0.112759e-01, 1.7350994e-02, 0.265640e-01, 4.0427860e-02,  \
      0.610997e-01, 9.1578111e-02, 0.135888, 0.1991484, 0.230756, 0.2850565, 0.375050, 0.5000000, 0.691489,   \
      0.8413813, 0.933222, 0.9772662, 0.993797, 0.9986521, 0.999768, 0.9999684, 0.999997, 1.0000000, 1.000000
#if defined(__CUDACC__)
static __constant__ double kSrc1dDev[34] = {ICE3_SRC_1D_VALUES};
#endif
static const double kSrc1dHost[34] = {ICE3_SRC_1D_VALUES};

// PSIGRC of condensation.F90:566-571 from q1, times the CB lambda3 factor
// min(3, max(1, 1 - q1)) of :638-647 when LAMBDA3 = CB (0).
ICE3_HD double sigrc_cb(const Cst &c, double q1)
{
  const double x = 2.0 * nmin(100.0, nmax(-100.0, q1));
  const int i = (int)floor(x);
  const int inq1 = i < -22 ? -22 : (i > 10 ? 10 : i);
  const double inc = 2.0 * q1 - inq1;
#if defined(__CUDA_ARCH__)
  const double s0 = kSrc1dDev[inq1 + 22], s1 = kSrc1dDev[inq1 + 23];
#else
  const double s0 = kSrc1dHost[inq1 + 22], s1 = kSrc1dHost[inq1 + 23];
#endif
  double r = nmin(1.0, (1.0 - inc) * s0 + inc * s1);
  if ((int)c.LAMBDA3 == 0) r *= nmin(3.0, nmax(1.0, 1.0 - q1));
  return r;
}

// ---- OCND2 (separate liquid and ice clouds) -----------------------------------
// The TIWMX tables and tiwmx_at() are in ice3gb_device.cuh (shared with the
// rain_ice OCND2 processes).

// Per-point inputs of the OCND2 branch and its extra outputs.
struct Ocnd2In {
  const double *estw, *esti;   // TIWMX tables
  double z, dz;                // height of the level; thickness to the level above (below at the top)
  double ice_cld_wgt;
  bool bottom;                 // k = 0 (condensation.F90:619, JK == IKTB)
};
struct Ocnd2Out {
  double icldfr, wcldfr, ssio, ssiu;
};

// ICECLOUD (micro/mode_icecloud.F90) as CONDENSATION calls it
// (condensation.F90:381-385: PTSTEP = 1, PPBLH = -1, PWCLD = -1, XW2D = 10;
// W2D and RSI are not used): ice cloud fraction and ice super-saturations.
ICE3_HD void icecloud(const Cst &c, double p, double z, double dz, double t, double r, double esw, double esi,
                      double &sifrc, double &ssio, double &ssiu)
{
  const double sigmax = 3.e-4, sigmaz = 1.e-2, xdist = 2500.;
  const double zr = nmax(0.0, r);
  sifrc = 0.0;
  const double za = zr * p / (c.EPSILO + zr);
  const double rhw = za / esw, rhi = za / esi, i2w = esw / esi;
  ssiu = nmin(i2w, rhi);
  ssio = ssiu;
  if (fgt(t, 273.1) || !fgt(zr, 0.0) || fge(esi, p * 0.5)) {
    ssiu = ssiu - 1.0;
    ssio = ssiu;
    return;
  }
  const double rhin = nmax(0.05, nmin(1.0, rhw));
  const double drhdz = rhin * c.GRAVITY0 / (t * c.RD) * (c.EPSILO * c.LVTT / (c.CPD * t) - 1.0);
  const double zz = nmin(1.0, nmax(0.0, z * 0.001));
  double rhdist = sqrt(xdist * sq(sigmax) + xdist * sq(sigmax) + (1.0 - zz) * sq(dz * drhdz) + zz * dz * sq(sigmaz));
  if (fgt(zz, 0.1)) rhdist = rhdist / (1.0 + rhdist);
  const double rhlim = nmax(0.5, nmin(0.99, 1.0 - 0.5 * rhdist));
  double rhdif = 1.0 - sqrt(nmax(0.0, (1.0 - rhw) / (1.0 - rhlim)));
  const double wcld = nmin(1.0, nmax(rhdif, 0.0));
  sifrc = wcld;
  const double rhlimice = 1.0 + i2w * (rhlim - 1.0);
  if (fge(0.999, rhlim)) {
    rhdif = (rhi - rhlimice) * (1.0 / (1.0 - rhlimice));
    if (fge(wcld, 0.0) && fge(0.0, wcld)) sifrc = nmin(1.0, 0.5 * nmax(0.0, rhdif));
    else sifrc = nmin(1.0, wcld + nmin(1.0, (1.0 - 1.0 / i2w) * 0.5 / (1.0 - rhlim)));
  }
  if (fgt(sifrc, 0.01)) {
    ssiu = sifrc + rhlimice * (1.0 - sifrc);
    ssio = (rhi - (1.0 - sifrc) * ssiu) / sifrc;
  } else {
    sifrc = 0.0;
    ssiu = nmax(0.0, sifrc + rhlimice * (1.0 - sifrc) + 2.0 * nmin(0.0, rhi - rhlimice));
  }
  ssio = nmin(i2w, ssio) - 1.0;
  ssiu = nmax(0.0, ssiu) - 1.0;
}

// Constants derived once per thread (divisions of table constants).
struct IaDerived {
  double rdrv, rvrd, irv;   // RD/RV, RV/RD, 1/RV
  double imix;              // the reciprocal of TMAXMIX - TMINMIX that fm::fdiv would form per point
};
ICE3_HD IaDerived ia_derived(const Cst &c)
{
  return {c.RD / c.RV, c.RV / c.RD, 1.0 / c.RV, fm::frcp(c.TMAXMIX - c.TMINMIX)};
}

// srcs (optional): PSRCS of the point (ice_adjust.F90:360, :468).
// OCND2: the separate liquid / ice cloud option of CONDENSATION
// (condensation.F90:373-395, :588-637), with its inputs in *oi and extra
// outputs in *oo (both required then; LSUBG_COND must be set).
template <bool OCND2 = false>
ICE3_HD void ia_point(const Cst &c, const IaDerived &d, double dt, double inv_dt, const IaIn &x, IaOut &o,
                      double *srcs = nullptr, const Ocnd2In *oi = nullptr, Ocnd2Out *oo = nullptr)
{
  const int nrr = (int)c.NRR;
  double t = x.th * x.exn;
  const double lv = c.LVTT + (c.CPV - c.CL) * (t - c.TT);
  const double ls = c.LSTT + (c.CPV - c.CI) * (t - c.TT);
  double cph;
  if (nrr == 5) cph = c.CPD + c.CPV * x.rv + c.CL * (x.rc + x.rr) + c.CI * (x.ri + x.rs);
  else if (nrr == 4) cph = c.CPD + c.CPV * x.rv + c.CL * (x.rc + x.rr);
  else if (nrr == 2) cph = c.CPD + c.CPV * x.rv + c.CL * x.rc + c.CI * x.ri;
  else cph = c.CPD + c.CPV * x.rv + c.CL * (x.rc + x.rr) + c.CI * (x.ri + x.rs + x.rg);
  const double inv_cph = fm::frcp(cph);
  double cldfr = 0.0, rv_out = 0.0, rc_out = 0.0, ri_out = 0.0;
  double hlc_hrc = 0.0, hlc_hcf = 0.0, hli_hri = 0.0, hli_hcf = 0.0;
  if (c.LSUBG_COND != 0.0) {
    // OCND2: ZPRIFACT = 0, the ice is kept out of the total water (condensation.F90:265-273)
    const double rt = OCND2 ? x.rv + x.rc : x.rv + x.rc + x.ri;
    const double it = fm::frcp(t);
    double pv, piv, frac, esw = 0.0;
    if (!OCND2) {
      // es_w and es_i share fm::flog(T) and 1/T (functions/tiwmx.py:18,60)
      const double lt = fm::flog(t);
      // the ice fraction: of the temperature (FRAC_ICE_ADJUST 0, the AROME
      // setting; fm::fdiv's product with the reciprocal formed once), else
      // of the condensate
      const int fmode = (int)c.FRAC_ICE_ADJUST;
      if (fmode == 0) {
        frac = nclip01(fm::mul_(c.TMAXMIX - t, d.imix));
      } else {
        frac = fgt(x.rc + x.ri, 1e-20) ? fm::fdiv(x.rc, x.rc + x.ri) : 0.0;
        if (fmode == 3) frac = nclip01(frac);
      }
      // saturation over water and over ice, each only where the fraction
      // gives it a weight: qsl = (1 - frac) qsl_w + frac qsl_i is qsl_w
      // exactly where frac is 0 and qsl_i where it is 1 (the other term is
      // 0 times a finite value); a NaN fraction keeps both
      pv = piv = 0.0;
      if (fm::bits_(frac) != fm::bits_(1.0)) pv = nmin(fm::fexp(c.ALPW - c.BETAW * it - c.GAMW * lt), 0.99 * x.pabs);
      if (!zerod_(frac)) piv = nmin(fm::fexp(c.ALPI - c.BETAI * it - c.GAMI * lt), 0.99 * x.pabs);
    } else {
      // condensation.F90:375-395: ICECLOUD, then the tabulated saturation
      // pressures; no ice fraction (:412, ZFRAC = 0)
      esw = tiwmx_at(oi->estw, t);
      const double esi = tiwmx_at(oi->esti, t);
      icecloud(c, x.pabs, oi->z, oi->dz, t, x.rv, esw, esi, oo->icldfr, oo->ssio, oo->ssiu);
      pv = nmin(esw, 0.99 * x.pabs);
      piv = nmin(esi, 0.99 * x.pabs);
      frac = 0.0;
    }
    // (OCND2: frac = 0 and qsi feeds the ice cloud factor below)
    double qsl = (OCND2 || fm::bits_(frac) != fm::bits_(1.0)) ? fm::fdiv(d.rdrv * pv, x.pabs - pv) : 0.0;
    const double qsi = (OCND2 || !zerod_(frac)) ? fm::fdiv(d.rdrv * piv, x.pabs - piv) : 0.0;
    qsl = (1.0 - frac) * qsl + frac * qsi;
    const double lvs = (1.0 - frac) * lv + frac * ls;
    const double ah = lvs * qsl * (it * it * d.irv) * (1.0 + qsl * d.rvrd);
    const double a = fm::frcp(1.0 + lvs * inv_cph * ah);
    const double sbar = a * (rt - qsl + ah * lvs * (OCND2 ? x.rc : x.rc + x.ri) * inv_cph);
    // sigma = sqrt(S) as S * S^(-1/2), the reciprocal reused for q1 when the
    // 1e-10 floor leaves sigma alone
    double sigma, isig = 0.0;
    if (c.LSIGMAS != 0.0 && c.LSTATNW == 0.0 && !(fge(x.sigqsat, 0.0) && fge(0.0, x.sigqsat))) {
      const double s2 = sq(2.0 * x.sigs) + sq(x.sigqsat * qsl * a);
      if (fm::frsqrt_ok(s2)) {
        isig = fm::frsqrt(s2);
        sigma = s2 * isig;
      } else {
        sigma = sqrt(s2);
      }
    } else {
      sigma = 2.0 * x.sigs;
    }
    const double sig = nmax(1e-10, sigma);
    const double q1 = (nz(isig) && fm::bits_(sig) == fm::bits_(sigma)) ? sbar * isig : fm::fdiv(sbar, sig);
    sigma = sig;
    if (srcs) *srcs = sigrc_cb(c, q1);
    double cond;
    if (fgt(q1, 0.0)) cond = fge(2.0, q1) ? nmin(0.36787944117144233 + 0.66 * q1 + 0.086 * q1 * q1, 2.0) : q1;
    else cond = fm::fexp(1.2 * q1 - 1.0);
    cond *= sigma;
    cldfr = fge(cond, 1e-12) ? nclip01(0.5 + 0.36 * fm::fatan(1.55 * q1)) : 0.0;
    if (fge(cldfr, 0.0) && fge(0.0, cldfr)) cond = 0.0;
    if (!OCND2) {
      rc_out = (1.0 - frac) * cond;
      ri_out = frac * cond;
      t = t + ((rc_out - x.rc) * lv + (ri_out - x.ri) * ls) * inv_cph;
      rv_out = rt - rc_out - ri_out;
    } else {
      // condensation.F90:588-637.  ZRSW = -9999 (:263) keeps the noise
      // check's sub-saturation branch closed (ZRSDIF = 0): the liquid content
      // is the condensate, and where the check fires (ZRCOLD = PRC_OUT) the
      // temperature keeps its value.  The cloud fraction becomes the
      // radiative one from the water and ice cloud factors.
      rc_out = cond;
      double rcold = x.rc;
      if (fgt(fabs(rc_out - x.rc), 1.0e-12) && fgt(x.pabs * 0.5, esw)) rcold = rc_out;
      oo->wcldfr = cldfr;
      const double sdz = sqrt(oi->dz);
      const double dum1 = nmin(1.0, 20. * rc_out * sdz / qsl);
      const double dum3 = nmax(0.0, oo->icldfr - cldfr);
      const double r_ice = oi->bottom ? x.ri : x.ri + x.rs * 0.5 + x.rg * 0.25;
      const double dum4 = nmax(0.0, nmin(1.0, oi->ice_cld_wgt * r_ice * sdz / qsi));
      const double dum2 = (0.8 * cldfr + 0.2) * nmin(1.0, dum1 + dum4 * cldfr);
      cldfr = nmin(1.0, dum2 + (0.5 * dum3 + 0.5) * dum4);
      ri_out = x.ri;
      t = t + (rc_out - rcold) * lv * inv_cph;
      rv_out = rt - rc_out;
    }
  }
  double rvs = x.rvs, rcs = x.rcs, ris = x.ris, ths = x.ths;
  const double inv_cphex = fm::fdiv(inv_cph, x.exn_ref);
  double w1 = (rc_out - x.rc) * inv_dt, w2 = (ri_out - x.ri) * inv_dt;
  w1 = fgt(0.0, w1) ? nmax(w1, -rcs) : nmin(w1, rvs);
  rvs = rvs - w1;
  rcs = rcs + w1;
  ths = ths + w1 * lv * inv_cphex;
  w2 = fgt(0.0, w2) ? nmax(w2, -ris) : nmin(w2, rvs);
  rvs = rvs - w2;
  ris = ris + w2;
  ths = ths + w2 * ls * inv_cphex;
  if (c.LSUBG_COND == 0.0) {
    cldfr = fgt((rcs + ris) * dt, 1e-12) ? 1.0 : 0.0;
    if (srcs) *srcs = cldfr;
  } else {
    double w1m = x.rc_mf * inv_dt, w2m = x.ri_mf * inv_dt;
    const double tot = w1m + w2m;
    const double scale = fgt(tot, rvs) ? fm::fdiv(rvs, tot) : 1.0;
    w1m *= scale;
    w2m *= scale;
    cldfr = nmin(1.0, cldfr + x.cf_mf);
    rcs = rcs + w1m;
    ris = ris + w2m;
    rvs = rvs - w1m - w2m;
    ths = ths + (w1m * lv + w2m * ls) * inv_cphex;
    const int mfpdf = (int)c.SUBG_MF_PDF;
    if (mfpdf == 0 || mfpdf == 1) {
      // the thresholds enter only as cf_mf * threshold: where cf_mf is +-0
      // that is +-0 whatever their (finite, positive) value, so they are
      // not formed there
      double criaut = 0.0, criaut_i = 0.0;
      if (nz(x.cf_mf)) {
        criaut = fm::fdiv(c.CRIAUTC, x.rho);
        criaut_i = nmin(c.CRIAUTI, fm::fexp10(c.ACRIAUTI * (t - c.TT) + c.BCRIAUTI));
      }
      if (mfpdf == 0) {
        if (fgt(w1m * dt, x.cf_mf * criaut)) { hlc_hrc = w1m * dt; hlc_hcf = nmin(1.0, x.cf_mf); }
        if (fgt(w2m * dt, x.cf_mf * criaut_i)) { hli_hri = w2m * dt; hli_hcf = nmin(1.0, x.cf_mf); }
      } else {
        double hcf, hr;
        triangle_pdf(w1m * dt, x.cf_mf * criaut, x.cf_mf, hcf, hr);
        hlc_hcf = nmin(1.0, hcf);
        hlc_hrc = hr;
        triangle_pdf(w2m * dt, x.cf_mf * criaut_i, x.cf_mf, hcf, hr);
        hli_hcf = nmin(1.0, hcf);
        hli_hri = hr;
      }
    }
  }
  o.t = t; o.rv_out = rv_out; o.rc_out = rc_out; o.ri_out = ri_out; o.cldfr = cldfr;
  o.hlc_hrc = hlc_hrc; o.hlc_hcf = hlc_hcf; o.hli_hri = hli_hri; o.hli_hcf = hli_hcf;
  o.cph = cph; o.lv = lv; o.ls = ls;
  o.rvs = rvs; o.rcs = rcs; o.ris = ris; o.ths = ths;
}

// ---- reverse mode -------------------------------------------------------------
// nmin/nmax that also report whether the first operand was taken (the
// branch the derivative follows).
ICE3_HD double nmin_sel(double a, double b, bool &first)
{
  first = isnan_(a) || (!isnan_(b) && dkey(a) < dkey(b));
  return first ? a : b;
}
ICE3_HD double nmax_sel(double a, double b, bool &first)
{
  first = isnan_(a) || (!isnan_(b) && dkey(a) > dkey(b));
  return first ? a : b;
}
// d nclip01(x)/dx: 1 where the clip left x unchanged.
ICE3_HD bool clip01_pass(double x) { return fgt(x, 0.0) && fgt(1.0, x); }

// Reverse of triangle_pdf: cotangents of hcf (after the factor cf_mf) and hr
// -> accumulated into the cotangents of w_dt, crit and cf_mf.
ICE3_HD void triangle_pdf_vjp(double w_dt, double crit, double cf_mf, double g_hcf, double g_hr, double &b_w,
                              double &b_crit, double &b_cf)
{
  bool w_const;
  const double wmax = nmax_sel(1e-20, w_dt, w_const);
  const double inv_w2 = fm::frcp(sq(wmax));
  double hcf0, b_inv_w2 = 0.0;
  if (fgt(w_dt, crit)) {
    const double cc = crit * cf_mf;
    hcf0 = 1.0 - 0.5 * sq(cc) * inv_w2;
    const double b_hcf0 = cf_mf * g_hcf;
    const double b_cc = -cc * inv_w2 * b_hcf0 - cc * cc * inv_w2 * g_hr;
    b_inv_w2 += -0.5 * cc * cc * b_hcf0 - cc * cc * cc * (1.0 / 3.0) * g_hr;
    b_w += g_hr;
    b_crit += cf_mf * b_cc;
    b_cf += crit * b_cc;
  } else if (fge(crit, 2.0 * w_dt)) {
    hcf0 = 0.0;
  } else {
    const double u = 2.0 * w_dt - crit;
    hcf0 = 0.5 * u * u * inv_w2;
    const double b_hcf0 = cf_mf * g_hcf;
    const double b_u = u * inv_w2 * b_hcf0;
    const double P = 4.0 * w_dt * w_dt * w_dt - 3.0 * w_dt * crit * crit + crit * crit * crit;
    const double b_P = inv_w2 * (1.0 / 3.0) * g_hr;
    b_inv_w2 += 0.5 * u * u * b_hcf0 + P * (1.0 / 3.0) * g_hr;
    b_w += 2.0 * b_u + (12.0 * w_dt * w_dt - 3.0 * crit * crit) * b_P;
    b_crit += -b_u + (-6.0 * w_dt * crit + 3.0 * crit * crit) * b_P;
  }
  b_cf += hcf0 * g_hcf;
  if (!w_const) b_w += -2.0 * inv_w2 / wmax * b_inv_w2;
}

// Reverse-mode derivative of ia_point (hand-written): from the cotangents g
// of the 16 outputs, the gradients gx of the 20 inputs.  The forward
// intermediates are recomputed here, nothing is stored between the passes.
// At kinks (min/max, clips, branch thresholds) the derivative of the branch
// the forward took is returned; the threshold steps (cldfr = 0 below
// cond < 1e-12, the mass-flux PDF cases) are piecewise constant.
ICE3_HD void ia_point_vjp(const Cst &c, const IaDerived &d, double dt, double inv_dt, const IaIn &x, const IaOut &g,
                          IaIn &b)
{
  b = IaIn{};
  // ---- forward, keeping what the reverse pass needs ----
  const int nrr = (int)c.NRR;
  const double t0 = x.th * x.exn;
  const double lv = c.LVTT + (c.CPV - c.CL) * (t0 - c.TT);
  const double ls = c.LSTT + (c.CPV - c.CI) * (t0 - c.TT);
  double cph;
  if (nrr == 5) cph = c.CPD + c.CPV * x.rv + c.CL * (x.rc + x.rr) + c.CI * (x.ri + x.rs);
  else if (nrr == 4) cph = c.CPD + c.CPV * x.rv + c.CL * (x.rc + x.rr);
  else if (nrr == 2) cph = c.CPD + c.CPV * x.rv + c.CL * x.rc + c.CI * x.ri;
  else cph = c.CPD + c.CPV * x.rv + c.CL * (x.rc + x.rr) + c.CI * (x.ri + x.rs + x.rg);
  const double inv_cph = fm::frcp(cph);
  const bool subg = c.LSUBG_COND != 0.0;
  const int fmode = (int)c.FRAC_ICE_ADJUST;
  double rt = 0, lt = 0, it = 0, ew = 0, ei = 0, pv = 0, piv = 0, frac = 0, qsl0 = 0, qsi = 0, qsl = 0, lvs = 0;
  double ah = 0, a = 0, G = 0, sigma0 = 0, sigma = 0, q1 = 0, cond0 = 0, cond = 0, cldfr0 = 0;
  double rc_out = 0, ri_out = 0, t = t0;
  bool pv_first = false, piv_first = false, frac_div = false, frac_pass = false, sig_sqrt = false, sig_const = false;
  bool cond_exp = false, cond_poly = false, poly_pass = false, cld_on = false, cld_pass = false, cld_zero = false;
  if (subg) {
    rt = x.rv + x.rc + x.ri;
    lt = fm::flog(t0);
    it = fm::frcp(t0);
    ew = fm::fexp(c.ALPW - c.BETAW * it - c.GAMW * lt);
    ei = fm::fexp(c.ALPI - c.BETAI * it - c.GAMI * lt);
    pv = nmin_sel(ew, 0.99 * x.pabs, pv_first);
    piv = nmin_sel(ei, 0.99 * x.pabs, piv_first);
    frac_div = fgt(x.rc + x.ri, 1e-20);
    frac = frac_div ? fm::fdiv(x.rc, x.rc + x.ri) : 0.0;
    if (fmode == 3) {
      frac_pass = clip01_pass(frac);
      frac = nclip01(frac);
    } else if (fmode == 0) {
      const double f0 = fm::fdiv(c.TMAXMIX - t0, c.TMAXMIX - c.TMINMIX);
      frac_pass = clip01_pass(f0);
      frac = nclip01(f0);
    } else {
      frac_pass = true;
    }
    qsl0 = fm::fdiv(d.rdrv * pv, x.pabs - pv);
    qsi = fm::fdiv(d.rdrv * piv, x.pabs - piv);
    qsl = (1.0 - frac) * qsl0 + frac * qsi;
    lvs = (1.0 - frac) * lv + frac * ls;
    ah = lvs * qsl * (it * it * d.irv) * (1.0 + qsl * d.rvrd);
    a = fm::frcp(1.0 + lvs * inv_cph * ah);
    G = rt - qsl + ah * lvs * (x.rc + x.ri) * inv_cph;
    const double sbar = a * G;
    if (c.LSIGMAS != 0.0 && c.LSTATNW == 0.0) {
      sig_sqrt = !(fge(x.sigqsat, 0.0) && fge(0.0, x.sigqsat));
      sigma0 = sig_sqrt ? sqrt(sq(2.0 * x.sigs) + sq(x.sigqsat * qsl * a)) : 2.0 * x.sigs;
    } else {
      sigma0 = 2.0 * x.sigs;
    }
    sigma = nmax_sel(1e-10, sigma0, sig_const);
    q1 = fm::fdiv(sbar, sigma);
    if (fgt(q1, 0.0)) {
      if (fge(2.0, q1)) {
        cond_poly = true;
        bool two;
        cond0 = nmin_sel(0.36787944117144233 + 0.66 * q1 + 0.086 * q1 * q1, 2.0, two);
        poly_pass = two;
      } else {
        cond0 = q1;
      }
    } else {
      cond_exp = true;
      cond0 = fm::fexp(1.2 * q1 - 1.0);
    }
    cond = cond0 * sigma;
    cld_on = fge(cond, 1e-12);
    if (cld_on) {
      const double y = 0.5 + 0.36 * fm::fatan(1.55 * q1);
      cld_pass = clip01_pass(y);
      cldfr0 = nclip01(y);
    }
    cld_zero = fge(cldfr0, 0.0) && fge(0.0, cldfr0);
    if (cld_zero) cond = 0.0;
    rc_out = (1.0 - frac) * cond;
    ri_out = frac * cond;
    t = t0 + ((rc_out - x.rc) * lv + (ri_out - x.ri) * ls) * inv_cph;
  }
  const double inv_cphex = fm::fdiv(inv_cph, x.exn_ref);
  const double w1r = (rc_out - x.rc) * inv_dt, w2r = (ri_out - x.ri) * inv_dt;
  const bool neg1 = fgt(0.0, w1r);
  bool w1_first;
  const double w1 = neg1 ? nmax_sel(w1r, -x.rcs, w1_first) : nmin_sel(w1r, x.rvs, w1_first);
  const double rvs1 = x.rvs - w1;
  const bool neg2 = fgt(0.0, w2r);
  bool w2_first;
  const double w2 = neg2 ? nmax_sel(w2r, -x.ris, w2_first) : nmin_sel(w2r, rvs1, w2_first);
  const double rvs2 = rvs1 - w2;

  // ---- reverse ----
  double b_t = g.t, b_rv_out = g.rv_out, b_rc_out = g.rc_out, b_ri_out = g.ri_out, b_lv = g.lv, b_ls = g.ls;
  double b_cph = g.cph, b_inv_cph = 0.0, b_inv_cphex = 0.0;
  // cotangents of the running sources (rvs, rcs, ris, ths after each update)
  double b_rvs = g.rvs, b_rcs = g.rcs, b_ris = g.ris, b_ths = g.ths;
  double b_cldfr0 = 0.0;
  if (subg) {
    const double w1m0 = x.rc_mf * inv_dt, w2m0 = x.ri_mf * inv_dt;
    const double tot = w1m0 + w2m0;
    const bool sc_div = fgt(tot, rvs2);
    const double scale = sc_div ? fm::fdiv(rvs2, tot) : 1.0;
    const double w1m = w1m0 * scale, w2m = w2m0 * scale;
    bool cld1_const;
    nmin_sel(1.0, cldfr0 + x.cf_mf, cld1_const);
    double b_w1m = 0.0, b_w2m = 0.0, b_cf = 0.0;
    const int mfpdf = (int)c.SUBG_MF_PDF;
    if (mfpdf == 0 || mfpdf == 1) {
      const double criaut = fm::fdiv(c.CRIAUTC, x.rho);
      const double p10 = fm::fexp10(c.ACRIAUTI * (t - c.TT) + c.BCRIAUTI);
      bool ci_const;
      const double criaut_i = nmin_sel(c.CRIAUTI, p10, ci_const);
      double b_criaut = 0.0, b_criaut_i = 0.0;
      if (mfpdf == 0) {
        bool one;
        nmin_sel(1.0, x.cf_mf, one);
        if (fgt(w1m * dt, x.cf_mf * criaut)) {
          b_w1m += dt * g.hlc_hrc;
          if (!one) b_cf += g.hlc_hcf;
        }
        if (fgt(w2m * dt, x.cf_mf * criaut_i)) {
          b_w2m += dt * g.hli_hri;
          if (!one) b_cf += g.hli_hcf;
        }
      } else {
        double hcf, hr, b_w = 0.0, b_crit = 0.0;
        bool one;
        triangle_pdf(w1m * dt, x.cf_mf * criaut, x.cf_mf, hcf, hr);
        nmin_sel(1.0, hcf, one);
        triangle_pdf_vjp(w1m * dt, x.cf_mf * criaut, x.cf_mf, one ? 0.0 : g.hlc_hcf, g.hlc_hrc, b_w, b_crit, b_cf);
        b_w1m += dt * b_w;
        b_criaut += x.cf_mf * b_crit;
        b_cf += criaut * b_crit;
        b_w = 0.0;
        b_crit = 0.0;
        triangle_pdf(w2m * dt, x.cf_mf * criaut_i, x.cf_mf, hcf, hr);
        nmin_sel(1.0, hcf, one);
        triangle_pdf_vjp(w2m * dt, x.cf_mf * criaut_i, x.cf_mf, one ? 0.0 : g.hli_hcf, g.hli_hri, b_w, b_crit, b_cf);
        b_w2m += dt * b_w;
        b_criaut_i += x.cf_mf * b_crit;
        b_cf += criaut_i * b_crit;
      }
      b.rho += -criaut / x.rho * b_criaut;
      if (!ci_const) b_t += c.ACRIAUTI * 2.302585092994045684 * p10 * b_criaut_i;
    }
    // ths = ths2 + (w1m lv + w2m ls) inv_cphex; rvs = rvs2 - w1m - w2m; ris = ris1 + w2m; rcs = rcs1 + w1m
    b_w1m += lv * inv_cphex * b_ths - b_rvs + b_rcs;
    b_w2m += ls * inv_cphex * b_ths - b_rvs + b_ris;
    b_lv += w1m * inv_cphex * b_ths;
    b_ls += w2m * inv_cphex * b_ths;
    b_inv_cphex += (w1m * lv + w2m * ls) * b_ths;
    // cldfr = min(1, cldfr0 + cf_mf)
    if (!cld1_const) {
      b_cldfr0 += g.cldfr;
      b_cf += g.cldfr;
    }
    // w1m = w1m0 scale, w2m = w2m0 scale, scale = rvs2 / (w1m0 + w2m0)
    double b_w1m0 = scale * b_w1m, b_w2m0 = scale * b_w2m;
    const double b_scale = w1m0 * b_w1m + w2m0 * b_w2m;
    if (sc_div) {
      const double b_tot = -scale / tot * b_scale;
      b_w1m0 += b_tot;
      b_w2m0 += b_tot;
      b_rvs += b_scale / tot;
    }
    b.rc_mf += inv_dt * b_w1m0;
    b.ri_mf += inv_dt * b_w2m0;
    b.cf_mf += b_cf;
  }
  // ths2 = ths1 + w2 ls inv_cphex; ris1 = ris + w2; rvs2 = rvs1 - w2
  double b_w2 = ls * inv_cphex * b_ths + b_ris - b_rvs;
  b_ls += w2 * inv_cphex * b_ths;
  b_inv_cphex += w2 * ls * b_ths;
  b.ris += b_ris;
  double b_rvs1 = b_rvs;
  double b_w2r = 0.0;
  if (w2_first) b_w2r = b_w2;
  else if (neg2) b.ris -= b_w2;
  else b_rvs1 += b_w2;
  // ths1 = ths + w1 lv inv_cphex; rcs1 = rcs + w1; rvs1 = rvs - w1
  double b_w1 = lv * inv_cphex * b_ths + b_rcs - b_rvs1;
  b_lv += w1 * inv_cphex * b_ths;
  b_inv_cphex += w1 * lv * b_ths;
  b.ths += b_ths;
  b.rcs += b_rcs;
  b.rvs += b_rvs1;
  double b_w1r = 0.0;
  if (w1_first) b_w1r = b_w1;
  else if (neg1) b.rcs -= b_w1;
  else b.rvs += b_w1;
  // w1r = (rc_out - rc) / dt, w2r = (ri_out - ri) / dt
  b_rc_out += inv_dt * b_w1r;
  b.rc -= inv_dt * b_w1r;
  b_ri_out += inv_dt * b_w2r;
  b.ri -= inv_dt * b_w2r;
  // inv_cphex = inv_cph / exn_ref
  b_inv_cph += b_inv_cphex / x.exn_ref;
  b.exn_ref += -inv_cphex / x.exn_ref * b_inv_cphex;
  double b_t0 = 0.0;
  if (subg) {
    // rv_out = rt - rc_out - ri_out
    double b_rt = b_rv_out;
    b_rc_out -= b_rv_out;
    b_ri_out -= b_rv_out;
    // t = t0 + D inv_cph
    const double D = (rc_out - x.rc) * lv + (ri_out - x.ri) * ls;
    b_t0 += b_t;
    const double b_D = inv_cph * b_t;
    b_inv_cph += D * b_t;
    b_rc_out += lv * b_D;
    b.rc -= lv * b_D;
    b_lv += (rc_out - x.rc) * b_D;
    b_ri_out += ls * b_D;
    b.ri -= ls * b_D;
    b_ls += (ri_out - x.ri) * b_D;
    // rc_out = (1 - frac) cond, ri_out = frac cond
    const double b_cond = (1.0 - frac) * b_rc_out + frac * b_ri_out;
    double b_frac = cond * (b_ri_out - b_rc_out);
    const double b_cond1 = cld_zero ? 0.0 : b_cond;
    double b_q1 = 0.0;
    if (cld_on && cld_pass) {
      const double z = 1.55 * q1;
      b_q1 += 0.36 * 1.55 / (1.0 + z * z) * b_cldfr0;
    }
    // cond1 = cond0 sigma
    const double b_cond0 = sigma * b_cond1;
    double b_sigma = cond0 * b_cond1;
    if (cond_exp) b_q1 += 1.2 * cond0 * b_cond0;
    else if (cond_poly) { if (poly_pass) b_q1 += (0.66 + 0.172 * q1) * b_cond0; }
    else b_q1 += b_cond0;
    // q1 = sbar / sigma
    const double b_sbar = b_q1 / sigma;
    b_sigma += -q1 / sigma * b_q1;
    const double b_sigma0 = sig_const ? 0.0 : b_sigma;
    double b_qsl = 0.0, b_a = 0.0;
    if (sig_sqrt) {
      const double u = 2.0 * x.sigs, v = x.sigqsat * qsl * a;
      const double b_u = u / sigma0 * b_sigma0, b_v = v / sigma0 * b_sigma0;
      b.sigs += 2.0 * b_u;
      b.sigqsat += qsl * a * b_v;
      b_qsl += x.sigqsat * a * b_v;
      b_a += x.sigqsat * qsl * b_v;
    } else {
      b.sigs += 2.0 * b_sigma0;
    }
    // sbar = a G, G = rt - qsl + ah lvs (rc + ri) inv_cph
    const double rcri = x.rc + x.ri;
    b_a += G * b_sbar;
    const double b_G = a * b_sbar;
    b_rt += b_G;
    b_qsl -= b_G;
    double b_ah = lvs * rcri * inv_cph * b_G;
    double b_lvs = ah * rcri * inv_cph * b_G;
    b.rc += ah * lvs * inv_cph * b_G;
    b.ri += ah * lvs * inv_cph * b_G;
    b_inv_cph += ah * lvs * rcri * b_G;
    // a = 1 / (1 + lvs inv_cph ah)
    const double b_Dn = -a * a * b_a;
    b_lvs += inv_cph * ah * b_Dn;
    b_inv_cph += lvs * ah * b_Dn;
    b_ah += lvs * inv_cph * b_Dn;
    // ah = lvs qsl K M, K = it^2 / RV, M = 1 + qsl RV / RD
    const double K = it * it * d.irv, M = 1.0 + qsl * d.rvrd;
    b_lvs += qsl * K * M * b_ah;
    b_qsl += lvs * K * M * b_ah + lvs * qsl * K * d.rvrd * b_ah;
    double b_it = 2.0 * it * d.irv * lvs * qsl * M * b_ah;
    // lvs = (1 - frac) lv + frac ls
    b_lv += (1.0 - frac) * b_lvs;
    b_ls += frac * b_lvs;
    b_frac += (ls - lv) * b_lvs;
    // qsl = (1 - frac) qsl0 + frac qsi
    const double b_qsl0 = (1.0 - frac) * b_qsl, b_qsi = frac * b_qsl;
    b_frac += (qsi - qsl0) * b_qsl;
    // qsi = rdrv piv / (pabs - piv), qsl0 = rdrv pv / (pabs - pv)
    const double di = x.pabs - piv, dw = x.pabs - pv;
    const double b_piv = d.rdrv * x.pabs / (di * di) * b_qsi;
    const double b_pv = d.rdrv * x.pabs / (dw * dw) * b_qsl0;
    b.pabs += -d.rdrv * piv / (di * di) * b_qsi - d.rdrv * pv / (dw * dw) * b_qsl0;
    // frac
    if (fmode == 0) {
      if (frac_pass) b_t0 += -b_frac / (c.TMAXMIX - c.TMINMIX);
    } else if (frac_div && frac_pass) {
      const double s2 = rcri * rcri;
      b.rc += x.ri / s2 * b_frac;
      b.ri += -x.rc / s2 * b_frac;
    }
    // pv = min(ew, 0.99 pabs), piv = min(ei, 0.99 pabs)
    double b_ew = 0.0, b_ei = 0.0;
    if (pv_first) b_ew = b_pv; else b.pabs += 0.99 * b_pv;
    if (piv_first) b_ei = b_piv; else b.pabs += 0.99 * b_piv;
    // ew = exp(ALPW - BETAW it - GAMW lt), ei likewise
    b_it += -c.BETAW * ew * b_ew - c.BETAI * ei * b_ei;
    const double b_lt = -c.GAMW * ew * b_ew - c.GAMI * ei * b_ei;
    b_t0 += it * b_lt - it * it * b_it;
    // rt = rv + rc + ri
    b.rv += b_rt;
    b.rc += b_rt;
    b.ri += b_rt;
  } else {
    b_t0 += b_t;
  }
  // inv_cph = 1 / cph
  b_cph += -inv_cph * inv_cph * b_inv_cph;
  if (nrr == 5) {
    b.rv += c.CPV * b_cph; b.rc += c.CL * b_cph; b.rr += c.CL * b_cph; b.ri += c.CI * b_cph; b.rs += c.CI * b_cph;
  } else if (nrr == 4) {
    b.rv += c.CPV * b_cph; b.rc += c.CL * b_cph; b.rr += c.CL * b_cph;
  } else if (nrr == 2) {
    b.rv += c.CPV * b_cph; b.rc += c.CL * b_cph; b.ri += c.CI * b_cph;
  } else {
    b.rv += c.CPV * b_cph; b.rc += c.CL * b_cph; b.rr += c.CL * b_cph;
    b.ri += c.CI * b_cph; b.rs += c.CI * b_cph; b.rg += c.CI * b_cph;
  }
  // lv, ls, t0 = th exn
  b_t0 += (c.CPV - c.CL) * b_lv + (c.CPV - c.CI) * b_ls;
  b.th += x.exn * b_t0;
  b.exn += x.th * b_t0;
}

}  // namespace ice3ia
