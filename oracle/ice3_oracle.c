/*
 * ice3_oracle.c — CPU FP64 restatement of the ICE3 hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the
 * smoke test and the CPU-baseline leg of the benchmark call it to produce the
 * expected outputs and the host-core timing.  The product (the CUDA library
 * under dwarf-p-ice3_gb300/) never links, loads or calls it.
 *
 * Every routine cites the reference lines it restates
 * (maurinl26/dwarf-p-ice3; paths relative to that project):
 *   - ice_adjust: src/ice3/jax/stencils/ice_adjust.py:26-398 (the reference
 *     JAX, which is executed unmodified in FP64 to make the golden vectors);
 *   - sedimentation: src/ice3/jax/stencils/sedimentation.py:58-352 and
 *     PHYEX-IAL_CY50T1/micro/mode_ice4_sedimentation_stat.F90:9-455;
 *   - rain_ice: PHYEX-IAL_CY50T1/micro/rain_ice.F90 (incl. the disabled
 *     tail :758-790), mode_ice4_pack.F90, mode_ice4_stepping.F90,
 *     mode_ice4_tendencies.F90 and the process modules it calls.
 *
 * Parallelised with OpenMP over grid points / columns.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/ice3gb.h"

typedef Ice3gbConstants C;

#define EXPORT __attribute__((visibility("default")))

/* NaN-propagating minimum/maximum, as numpy.minimum/maximum (the reference
 * JAX produces NaN on some degenerate inputs, stencils/ice_adjust.py:293-296). */
static inline double dmin(double a, double b) { return (a < b || a != a) ? a : b; }
static inline double dmax(double a, double b) { return (a > b || a != a) ? a : b; }
static inline double clip01(double x) { return dmin(dmax(x, 0.0), 1.0); }
static inline double sq(double x) { return x * x; }

/* ===================================================================== */
/* ice_adjust (src/ice3/jax/stencils/ice_adjust.py:26-398)               */
/* ===================================================================== */

/* Triangle-PDF subgrid autoconversion, stencils/ice_adjust.py:316-341. */
static void triangle_pdf(double w_dt, double crit, double cf_mf, double *hcf_out, double *hr_out)
{
  const double wmax = dmax(1e-20, w_dt);
  double hcf, hr;
  if (w_dt > crit) {
    hcf = 1.0 - 0.5 * sq(crit * cf_mf / wmax);
    hr = w_dt - pow(crit * cf_mf, 3.0) / (3.0 * sq(wmax));
  } else if (2.0 * w_dt <= crit) {
    hcf = 0.0;
    hr = 0.0;
  } else {
    hcf = sq(2.0 * w_dt - crit) / (2.0 * sq(wmax));
    hr = (4.0 * pow(w_dt, 3.0) - 3.0 * w_dt * sq(crit) + pow(crit, 3.0)) / (3.0 * sq(wmax));
  }
  *hcf_out = hcf * cf_mf;
  *hr_out = hr;
}

/* SRC_1D of condensation.F90:208-214 (index -22..11). */
static const double SRC_1D[34] = {
    0., 0., 2.0094444e-04, 0.316670e-03, 4.9965648e-04, 0.785956e-03, 1.2341294e-03, 0.193327e-02,
    3.0190963e-03, 0.470144e-02, 7.2950651e-03, 0.112759e-01, 1.7350994e-02, 0.265640e-01, 4.0427860e-02,
    0.610997e-01, 9.1578111e-02, 0.135888, 0.1991484, 0.230756, 0.2850565, 0.375050, 0.5000000, 0.691489,
    0.8413813, 0.933222, 0.9772662, 0.993797, 0.9986521, 0.999768, 0.9999684, 0.999997, 1.0000000, 1.000000};

EXPORT double ice3o_src_1d(int i) { return (i >= -22 && i <= 11) ? SRC_1D[i + 22] : 0.0 / 0.0; }

/* PSIGRC from q1 (condensation.F90:566-571) with the CB lambda3 factor
 * (:638-647, NEBN%CLAMBDA3 = 'CB' <-> LAMBDA3 = 0). */
static double sigrc(const C *c, double q1)
{
  int inq1 = (int)floor(dmin(100.0, dmax(-100.0, 2.0 * q1)));
  inq1 = inq1 < -22 ? -22 : (inq1 > 10 ? 10 : inq1);
  const double inc = 2.0 * q1 - inq1;
  double r = dmin(1.0, (1.0 - inc) * SRC_1D[inq1 + 22] + inc * SRC_1D[inq1 + 23]);
  if ((int)c->LAMBDA3 == 0) r *= dmin(3.0, dmax(1.0, 1.0 - q1));
  return r;
}

/* ---- OCND2 (separate liquid and ice clouds) ---------------------------- */

/* TIWMX saturation tables, micro/modd_tiwmx.F90 (XNDEGR = 100, NSTART =
 * 13200, NSTOP = 37316), filled by micro/mode_ini_tiwmx.F90 from
 * micro/mode_tiwmx_fun.F90: ESTABW(j) = ESATW(j/100); ESTABI(j) = the ice
 * formula at and below 273.15 K, the water one above (INI_TIWMX overwrites
 * ESATI's blend there). */
#define TIWMX_NSTART 13200
#define TIWMX_NSTOP 37316
#define TIWMX_N (TIWMX_NSTOP - TIWMX_NSTART + 1)

EXPORT int ice3o_tiwmx_size(void) { return TIWMX_N; }

EXPORT void ice3o_tiwmx_tables(const C *c, double *estw, double *esti)
{
  for (int j = TIWMX_NSTART; j <= TIWMX_NSTOP; ++j) {
    const double t = (double)j / 100.0;
    const double w = exp(c->ALPW - c->BETAW / t - c->GAMW * log(t));
    estw[j - TIWMX_NSTART] = w;
    esti[j - TIWMX_NSTART] = (t > 273.15) ? w : exp(c->ALPI - c->BETAI / t - c->GAMI * log(t));
  }
}

/* The six TIWMX tables OCND2 reads (micro/mode_ini_tiwmx.F90, functions of
 * micro/mode_tiwmx_fun.F90): ESTABW, ESTABI, A2TAB (AA2), BB3TAB (BB3),
 * AM3TAB (AM3, 0 above 273.15 K), REDINTAB (REDIN), each TIWMX_N long. */
enum { TW_ESW, TW_ESI, TW_A2, TW_BB3, TW_AM3, TW_REDIN, TW_N };

static double esatw_fun(const C *c, double t) { return exp(c->ALPW - c->BETAW / t - c->GAMW * log(t)); }
/* ESATI of mode_tiwmx_fun.F90: the water formula at and above TT, the ice one below */
static double esati_fun(const C *c, double t)
{
  return t >= c->TT ? esatw_fun(c, t) : exp(c->ALPI - c->BETAI / t - c->GAMI * log(t));
}

EXPORT void ice3o_tiwmx_all(const C *c, double *tab)
{
  ice3o_tiwmx_tables(c, tab + TW_ESW * TIWMX_N, tab + TW_ESI * TIWMX_N);
  for (int j = TIWMX_NSTART; j <= TIWMX_NSTOP; ++j) {
    const double t = (double)j / 100.0;
    const long i = j - TIWMX_NSTART;
    tab[TW_A2 * TIWMX_N + i] = sq(c->LSTT + (c->CPV - c->CI) * (t - c->TT)) / (2.38e-2 + 0.0071e-2 * (t - c->TT)) /
                               (sq(t) * c->RV);
    tab[TW_BB3 * TIWMX_N + i] = c->RV / (0.211e-4 * pow(t / c->TT, 1.94) * c->P00) * t / esati_fun(c, t);
    tab[TW_AM3 * TIWMX_N + i] =
        t > 273.15 ? 0. : 1000. * exp(12.96 * (esatw_fun(c, t) / esati_fun(c, t) - 1.) - 0.639);
    const double zzt = dmax(0., dmin(1., (c->TT - t) / 20.));
    tab[TW_REDIN * TIWMX_N + i] = 1. - (1. - zzt) / pow(zzt * zzt * zzt + (1. - zzt) * (1. - zzt) * (1. - zzt), .333);
  }
}

/* ESATW / ESATI of micro/mode_tiwmx.F90: TAB(NINT(XNDEGR*T)); the index is
 * clamped to the table (the reference reads out of bounds there). */
static double tiwmx_at(const double *tab, double t)
{
  long j = lround(100.0 * t);
  j = j < TIWMX_NSTART ? TIWMX_NSTART : (j > TIWMX_NSTOP ? TIWMX_NSTOP : j);
  return tab[j - TIWMX_NSTART];
}

/* ICECLOUD, micro/mode_icecloud.F90 (as CONDENSATION calls it,
 * condensation.F90:381-385: PTSTEP = 1, PPBLH = -1, PWCLD = -1, XW2D = PIFR =
 * 10; W2D and RSI are discarded there).  Returns SIFRC (the ice cloud
 * fraction) and the super-saturations SSIO / SSIU. */
static void icecloud(const C *c, double p, double z, double dz, double t, double r, double esw, double esi,
                     double *sifrc_o, double *ssio_o, double *ssiu_o)
{
  const double sigmax = 3.e-4, sigmay = sigmax, sigmaz = 1.e-2, xdist = 2500., ydist = xdist;
  const double zr = dmax(0., r * 1.0);
  double sifrc = 0.;
  double za = zr * p / (c->EPSILO + zr);
  const double rhw = za / esw;
  const double rhi = za / esi;
  const double i2w = esw / esi;
  double ssiu = dmin(i2w, rhi), ssio = ssiu;
  if (t > 273.1 || zr <= 0. || esi >= p * 0.5) {
    ssiu = ssiu - 1.;
    ssio = ssiu;
  } else {
    const double rhin = dmax(0.05, dmin(1., rhw));
    const double drhdz = rhin * c->GRAVITY0 / (t * c->RD) * (c->EPSILO * c->LVTT / (c->CPD * t) - 1.);
    const double zz = dmin(1., dmax(0., z * 0.001));
    double rhdist = sqrt(xdist * sq(sigmax) + ydist * sq(sigmay) + (1. - zz) * sq(dz * drhdz) + zz * dz * sq(sigmaz));
    if (zz > 0.1) rhdist = rhdist / (1. + rhdist);
    const double rhlim = dmax(0.5, dmin(0.99, 1. - 0.5 * rhdist));
    double rhdif = (1. - rhw) / (1.0 - rhlim);
    rhdif = 1. - sqrt(dmax(0., rhdif));
    const double wcld = dmin(1., dmax(rhdif, 0.0));
    sifrc = wcld;
    const double rhlimice = 1. + i2w * (rhlim - 1.);
    if (rhlim <= 0.999) {
      const double rhliminv = 1. / (1. - rhlimice);
      rhdif = (rhi - rhlimice) * rhliminv;
      if (wcld == 0.) {
        sifrc = dmin(1., 0.5 * dmax(0., rhdif));
      } else {
        za = 1. - 1. / i2w;
        sifrc = dmin(1., za * 0.5 / (1. - rhlim));
        sifrc = dmin(1., wcld + sifrc);
      }
    }
    if (sifrc > 0.01) {
      ssiu = sifrc + rhlimice * (1. - sifrc);
      ssio = (rhi - (1. - sifrc) * ssiu) / sifrc;
    } else {
      sifrc = 0.;
      za = dmin(0., rhi - rhlimice);
      ssiu = dmax(0., sifrc + rhlimice * (1. - sifrc) + 2. * za);
    }
    ssio = dmin(i2w, ssio);
    ssiu = dmax(0., ssiu);
    ssiu = ssiu - 1.;
    ssio = ssio - 1.;
  }
  *sifrc_o = sifrc;
  *ssio_o = ssio;
  *ssiu_o = ssiu;
}

EXPORT int ice3o_ice_adjust(const C *c, int nij, int nk, double dt, const Ice3gbIceAdjustFields *f)
{
  if (!c || !f || nij <= 0 || nk <= 0) return ICE3GB_ERR_SHAPE;
  const long n = (long)nij * nk;
  const int nrr = (int)c->NRR;
  const int subg = c->LSUBG_COND != 0.0;
  const int fmode = (int)c->FRAC_ICE_ADJUST;
  const int sigmas = c->LSIGMAS != 0.0 && c->LSTATNW == 0.0;
  const int mfpdf = (int)c->SUBG_MF_PDF;
  const int ocnd2 = c->OCND2 != 0.0;
  if (c->CONDENS != 0.0) return ICE3GB_ERR_UNSUPPORTED;
  if (ocnd2 && (!subg || nk < 2 || !f->zz || !f->ice_cld_wgt)) return ICE3GB_ERR_UNSUPPORTED;
  double *estw = NULL, *esti = NULL;
  if (ocnd2) {
    estw = (double *)malloc(2 * sizeof(double) * TIWMX_N);
    if (!estw) return ICE3GB_ERR_SHAPE;
    esti = estw + TIWMX_N;
    ice3o_tiwmx_tables(c, estw, esti);
  }
#pragma omp parallel for schedule(static)
  for (long p = 0; p < n; ++p) {
    const long col = p % nij;
    const long k = p / nij;
    const double sigqsat = f->sigqsat_3d ? f->sigqsat[p] : f->sigqsat[col];
    const double pabs = f->pabs[p], sigs = f->sigs[p];
    const double rv = f->rv[p], rc = f->rc[p], ri = f->ri[p];
    const double rr = f->rr[p], rs = f->rs[p], rg = f->rg[p];
    double t = f->th[p] * f->exn[p];                                   /* :158 */
    const double lv = c->LVTT + (c->CPV - c->CL) * (t - c->TT);        /* functions/ice_adjust.py:18 */
    const double ls = c->LSTT + (c->CPV - c->CI) * (t - c->TT);        /* functions/ice_adjust.py:70 */
    double cph;                                                        /* :163-172 */
    if (nrr == 5) cph = c->CPD + c->CPV * rv + c->CL * (rc + rr) + c->CI * (ri + rs);
    else if (nrr == 4) cph = c->CPD + c->CPV * rv + c->CL * (rc + rr);
    else if (nrr == 2) cph = c->CPD + c->CPV * rv + c->CL * rc + c->CI * ri;
    else cph = c->CPD + c->CPV * rv + c->CL * (rc + rr) + c->CI * (ri + rs + rg);
    double cldfr = 0.0, rv_out = 0.0, rc_out = 0.0, ri_out = 0.0;
    double hlc_hrc = 0.0, hlc_hcf = 0.0, hli_hri = 0.0, hli_hcf = 0.0;
    double icldfr = 0.0, ssio = 0.0, ssiu = 0.0;
    if (subg) {
      /* OCND2: ZPRIFACT = 0, ice kept out of the total water (condensation.F90:265-273) */
      const double rt = ocnd2 ? rv + rc : rv + rc + ri;                /* :190 */
      double pv, piv, esw = 0.0, dz = 0.0, frac;
      if (!ocnd2) {
        /* es_w/es_i: functions/tiwmx.py:18,60 */
        pv = dmin(exp(c->ALPW - c->BETAW / t - c->GAMW * log(t)), 0.99 * pabs);
        piv = dmin(exp(c->ALPI - c->BETAI / t - c->GAMI * log(t)), 0.99 * pabs);
        frac = (rc + ri > 1e-20) ? rc / (rc + ri) : 0.0;               /* :198-202 */
        if (fmode == 3) frac = clip01(frac);
        else if (fmode == 0) frac = clip01((c->TMAXMIX - t) / (c->TMAXMIX - c->TMINMIX));
      } else {
        /* condensation.F90:375-395: layer thickness to the level above (below
         * at the top), ICECLOUD, tabulated saturation pressures; no ice
         * fraction (:412, ZFRAC = 0) */
        const long kp = k + 1 < nk ? k + 1 : nk - 1;
        dz = f->zz[kp * nij + col] - f->zz[(kp - 1) * nij + col];
        esw = tiwmx_at(estw, t);
        const double esi = tiwmx_at(esti, t);
        icecloud(c, pabs, f->zz[p], dz, t, rv, esw, esi, &icldfr, &ssio, &ssiu);
        pv = dmin(esw, 0.99 * pabs);
        piv = dmin(esi, 0.99 * pabs);
        frac = 0.0;
      }
      double qsl = c->RD / c->RV * pv / (pabs - pv);                   /* :212 */
      const double qsi = c->RD / c->RV * piv / (pabs - piv);
      qsl = (1.0 - frac) * qsl + frac * qsi;
      const double lvs = (1.0 - frac) * lv + frac * ls;
      const double ah = lvs * qsl / (c->RV * sq(t)) * (1.0 + c->RV * qsl / c->RD);
      const double a = 1.0 / (1.0 + lvs / cph * ah);
      const double sbar = a * (rt - qsl + ah * lvs * (ocnd2 ? rc : rc + ri) / cph);
      double sigma;
      if (sigmas)                                                      /* :226-233 */
        sigma = (sigqsat != 0.0) ? sqrt(sq(2.0 * sigs) + sq(sigqsat * qsl * a)) : 2.0 * sigs;
      else
        sigma = 2.0 * sigs;
      sigma = dmax(1e-10, sigma);
      const double q1 = sbar / sigma;
      if (f->srcs) f->srcs[p] = sigrc(c, q1);                          /* ice_adjust.F90:468 */
      double cond;                                                     /* :241-249 */
      if (q1 > 0.0) cond = (q1 <= 2.0) ? dmin(exp(-1.0) + 0.66 * q1 + 0.086 * sq(q1), 2.0) : q1;
      else cond = exp(1.2 * q1 - 1.0);
      cond *= sigma;
      cldfr = (cond >= 1e-12) ? clip01(0.5 + 0.36 * atan(1.55 * q1)) : 0.0;
      if (cldfr == 0.0) cond = 0.0;
      if (!ocnd2) {
        rc_out = (1.0 - frac) * cond;                                  /* :263-266 */
        ri_out = frac * cond;
        t = t + ((rc_out - rc) * lv + (ri_out - ri) * ls) / cph;
        rv_out = rt - rc_out - ri_out;
      } else {
        /* condensation.F90:588-637.  ZRSW = -9999 (:263), so the
         * sub-saturation branch of the noise check is never taken and
         * ZRSDIF = 0: the liquid content is the condensate, and where the
         * check fires the temperature keeps its value (ZRCOLD = PRC_OUT). */
        rc_out = (1.0 - frac) * cond;
        const double lwinc = rc_out - rc;
        double rcold = rc;
        if (fabs(lwinc) > 1.0e-12 && esw < pabs * 0.5) {
          rcold = rc_out;
          rc_out = cond - 0.0;
        }
        const double wcldfr = cldfr;
        const double dum1 = dmin(1.0, 20. * rc_out * sqrt(dz) / qsl);
        const double dum3 = dmax(0., icldfr - wcldfr);
        double dum4 = (k == 0) ? ri : ri + rs * 0.5 + rg * 0.25;
        dum4 = dmax(0., dmin(1., f->ice_cld_wgt[col] * dum4 * sqrt(dz) / qsi));
        const double dum2 = (0.8 * cldfr + 0.2) * dmin(1., dum1 + dum4 * cldfr);
        cldfr = dmin(1., dum2 + (0.5 * dum3 + 0.5) * dum4);
        ri_out = ri;
        t = t + ((rc_out - rcold) * lv + (ri_out - ri) * ls) / cph;
        rv_out = rt - rc_out - ri_out * 0.0;
        if (f->wcldfr) f->wcldfr[p] = wcldfr;
      }
    }
    if (ocnd2) {
      if (f->icldfr) f->icldfr[p] = icldfr;
      if (f->ssio) f->ssio[p] = ssio;
      if (f->ssiu) f->ssiu[p] = ssiu;
      if (f->ifr) f->ifr[p] = 10.;                                     /* condensation.F90:259 */
    }
    double rvs = f->rvs[p], rcs = f->rcs[p], ris = f->ris[p], ths = f->ths[p];
    const double exn_ref = f->exn_ref[p];
    double w1 = (rc_out - rc) / dt, w2 = (ri_out - ri) / dt;           /* :269-281 */
    w1 = (w1 < 0.0) ? dmax(w1, -rcs) : dmin(w1, rvs);
    rvs = rvs - w1;
    rcs = rcs + w1;
    ths = ths + w1 * lv / (cph * exn_ref);
    w2 = (w2 < 0.0) ? dmax(w2, -ris) : dmin(w2, rvs);
    rvs = rvs - w2;
    ris = ris + w2;
    ths = ths + w2 * ls / (cph * exn_ref);
    if (!subg) {
      cldfr = ((rcs + ris) * dt > 1e-12) ? 1.0 : 0.0;                 /* :285 */
      if (f->srcs) f->srcs[p] = cldfr;                                 /* ice_adjust.F90:360 */
    } else {
      const double cf_mf = f->cf_mf[p];                                /* :288-305 */
      double w1m = f->rc_mf[p] / dt, w2m = f->ri_mf[p] / dt;
      const double tot = w1m + w2m;
      const double scale = (tot > rvs) ? rvs / tot : 1.0;
      w1m *= scale;
      w2m *= scale;
      cldfr = dmin(1.0, cldfr + cf_mf);
      rcs = rcs + w1m;
      ris = ris + w2m;
      rvs = rvs - w1m - w2m;
      ths = ths + (w1m * lv + w2m * ls) / (cph * exn_ref);
      const double criaut = c->CRIAUTC / f->rho_dry_ref[p];            /* :308 */
      if (mfpdf == 0) {
        if (w1m * dt > cf_mf * criaut) { hlc_hrc = w1m * dt; hlc_hcf = dmin(1.0, cf_mf); }
      } else if (mfpdf == 1) {
        double hcf, hr;
        triangle_pdf(w1m * dt, cf_mf * criaut, cf_mf, &hcf, &hr);
        hlc_hcf = dmin(1.0, hcf);
        hlc_hrc = hr;
      }
      const double criaut_i = dmin(c->CRIAUTI, pow(10.0, c->ACRIAUTI * (t - c->TT) + c->BCRIAUTI));
      if (mfpdf == 0) {
        if (w2m * dt > cf_mf * criaut_i) { hli_hri = w2m * dt; hli_hcf = dmin(1.0, cf_mf); }
      } else if (mfpdf == 1) {
        double hcf, hr;
        triangle_pdf(w2m * dt, cf_mf * criaut_i, cf_mf, &hcf, &hr);
        hli_hcf = dmin(1.0, hcf);
        hli_hri = hr;
      }
    }
    f->t[p] = t;
    f->rv_out[p] = rv_out;
    f->rc_out[p] = rc_out;
    f->ri_out[p] = ri_out;
    f->cldfr[p] = cldfr;
    f->hlc_hrc[p] = hlc_hrc;
    f->hlc_hcf[p] = hlc_hcf;
    f->hli_hri[p] = hli_hri;
    f->hli_hcf[p] = hli_hcf;
    f->cph[p] = cph;
    f->lv[p] = lv;
    f->ls[p] = ls;
    f->rvs[p] = rvs;
    f->rcs[p] = rcs;
    f->ris[p] = ris;
    f->ths[p] = ths;
  }
  free(estw);
  return ICE3GB_OK;
}

/* ===================================================================== */
/* Statistical sedimentation                                             */
/* ===================================================================== */

/* Terminal velocity of rain/snow/graupel: sedimentation.py:35-43,
 * mode_ice4_sedimentation_stat.F90:408,413. */
static inline double sed_other(double fsed, double exsed, double r, double rho, double cexvt)
{
  return fsed * pow(r, exsed - 1.0) * pow(rho, exsed - cexvt - 1.0);
}

/* Pristine ice velocity: sedimentation.py:46-55, F90:307-319. */
static inline double sed_ice(const C *c, double r, double rho)
{
  return c->FSEDI * pow(rho, -c->CEXVT) *
         pow(dmax(0.05e6, -0.15319e6 - 0.021454e6 * log(rho * r)), c->EXCSEDI);
}

/* Cloud droplet velocity: sedimentation.py:206-214, F90:264-275. */
static inline double sed_cloud(const C *c, double r, double rho, double wlbda, double lbc,
                               double conc, double ray, double fsedc)
{
  const double wlbdc = pow(lbc * conc / (rho * r), c->LBEXC);
  const double cc = c->CC * (1.0 + 1.26 * wlbda * wlbdc / ray);
  return pow(rho, -c->CEXVT) * pow(wlbdc, -c->DC) * cc * fsedc;
}

/* One column, top (k = nk-1) to bottom (k = 0).  `rt` are the sedimenting
 * contents (source * dt), `src` the sources updated in place.  Species order
 * c, r, i, s, g.  fpr (optional) gets the downward flux F_k per level. */
static void sed_column(const C *c, int nij, int nk, double dt, long col, int fortran,
                       const double *rho, const double *dzz, const double *pabs,
                       const double *tht, double sea, double town, int has_sea_town,
                       double *src[5], double *fpr[5], double inpr[5])
{
  const double rtmin[5] = {c->C_RTMIN, c->R_RTMIN, c->I_RTMIN, c->S_RTMIN, c->G_RTMIN};
  /* cloud parameters: sedimentation.py:153-156 / F90:122-127,252-260 */
  double lbc, fsedc, conc, ray;
  if (fortran) {
    const double gac_gc = c->GAC / c->GC, gac2_gc2 = c->GAC2 / c->GC2;
    if (has_sea_town) {
      ray = dmax(1.0, 0.5 * ((1.0 - sea) * gac_gc + sea * gac2_gc2));
      lbc = dmax(dmin(c->LBC_1, c->LBC_2), sea * c->LBC_2 + (1.0 - sea) * c->LBC_1);
      fsedc = dmax(dmin(c->FSEDC_1, c->FSEDC_2), sea * c->FSEDC_2 + (1.0 - sea) * c->FSEDC_1);
      conc = (1.0 - town) * (sea * c->CONC_SEA + (1.0 - sea) * c->CONC_LAND) + town * c->CONC_URBAN;
    } else {
      ray = dmax(1.0, 0.5 * gac_gc);
      lbc = c->LBC_1;
      fsedc = c->FSEDC_1;
      conc = c->CONC_LAND;
    }
  } else {
    ray = 1.0;
    lbc = (1.0 - sea) * c->LBC_1 + sea * c->LBC_2;
    fsedc = (1.0 - sea) * c->FSEDC_1 + sea * c->FSEDC_2;
    conc = (1.0 - town) * ((1.0 - sea) * c->CONC_LAND + sea * c->CONC_SEA) + town * c->CONC_URBAN;
  }
  const double fsed[5] = {0.0, c->FSEDR, 0.0, c->FSEDS, c->FSEDG};
  const double exsed[5] = {0.0, c->EXSEDR, 0.0, c->EXSEDS, c->EXSEDG};
  const double imin = dmax(c->I_RTMIN, 1.0e-7);
  double fabove[5] = {0, 0, 0, 0, 0};
  for (int k = nk - 1; k >= 0; --k) {
    const long p = (long)k * nij + col;
    const double r_rho = rho[p], dz = dzz[p];
    const double tsorhodz = dt / (r_rho * dz);
    const double wlbda = 6.6e-8 * (101325.0 / pabs[p]) * (tht[p] / 293.15);
    double fk[5];
    for (int s = 0; s < 5; ++s) {
      const double rt = src[s][p] * dt;                  /* sedimentation.py:134-138; F90 driver :167-173 */
      const double qp = fabove[s] * tsorhodz;
      double w1 = 0.0, w2 = 0.0;
      if (s == 0) {
        if (fortran && c->LSEDIC == 0.0) { fk[s] = 0.0; continue; }
        if (rt > rtmin[0]) w1 = sed_cloud(c, rt, r_rho, wlbda, lbc, conc, ray, fsedc);
        if (qp > rtmin[0]) w2 = sed_cloud(c, qp, r_rho, wlbda, lbc, conc, ray, fsedc);
      } else if (s == 2) {
        if (rt > imin) w1 = sed_ice(c, rt, r_rho);
        if (qp > imin) w2 = sed_ice(c, qp, r_rho);
      } else {
        if (rt > rtmin[s]) w1 = sed_other(fsed[s], exsed[s], rt, r_rho, c->CEXVT);
        if (qp > rtmin[s]) w2 = sed_other(fsed[s], exsed[s], qp, r_rho, c->CEXVT);
      }
      /* FWSED1/FWSED2: F90:442-453; sedimentation.py:216-223 */
      double flux = dmin(r_rho * dz * rt * (1.0 / dt), w1 * r_rho * rt);
      if (w2 != 0.0) flux += dmax(0.0, 1.0 - dz / (dt * w2)) * fabove[s];
      fk[s] = flux;
    }
    for (int s = 0; s < 5; ++s) {
      /* flux divergence: F90:203-207 (Fortran) vs sedimentation.py:337-341 (JAX) */
      if (fortran)
        src[s][p] = src[s][p] + tsorhodz * (fabove[s] - fk[s]) * (1.0 / dt);
      else
        src[s][p] = src[s][p] + (fabove[s] - fk[s]) / (r_rho * dz * dt);
      if (fpr[s]) fpr[s][p] = fk[s];
      fabove[s] = fk[s];
    }
  }
  for (int s = 0; s < 5; ++s) inpr[s] = fabove[s] / c->RHOLW;   /* :344-348 / F90:213-223 */
}

/* Time-split sedimentation (SEDIM = SPLI) of one column:
 * mode_ice4_sedimentation_split.F90 INTERNAL_SEDIM_SPLI (without electric
 * charges / Beard correction), species in the order c r i s g, then
 * ICE4_CORRECT_NEGATIVITIES with L/cph of the time-t state
 * (mode_ice4_sedimentation.F90:196-229, the factors rain_ice.F90:334-345
 * passes).  rt: mixing ratios at t; returns 0 if a species needed more
 * than max_iter sub-steps. */
/* Hail in ICE4_SEDIMENTATION_STAT (species 7, OTHER_SPECIES with XFSEDH /
 * XEXSEDH, mode_ice4_sedimentation_stat.F90:186-187, 208-222) for one column,
 * on rh = rhs * dt (mode_ice4_sedimentation.F90:179). */
static void sed_hail_column(const C *c, int nij, int nk, double dt, long col, const double *rho,
                            const double *dzz, double *rhs, double *fpr, double *inpr)
{
  double fabove = 0.0;
  for (int k = nk - 1; k >= 0; --k) {
    const long p = (long)k * nij + col;
    const double r_rho = rho[p], dz = dzz[p];
    const double tsorhodz = dt / (r_rho * dz);
    const double rt = rhs[p] * dt;
    const double qp = fabove * tsorhodz;
    double w1 = 0.0, w2 = 0.0;
    if (rt > c->H_RTMIN) w1 = sed_other(c->FSEDH, c->EXSEDH, rt, r_rho, c->CEXVT);
    if (qp > c->H_RTMIN) w2 = sed_other(c->FSEDH, c->EXSEDH, qp, r_rho, c->CEXVT);
    double flux = dmin(r_rho * dz * rt * (1.0 / dt), w1 * r_rho * rt);
    if (w2 != 0.0) flux += dmax(0.0, 1.0 - dz / (dt * w2)) * fabove;
    rhs[p] = rhs[p] + tsorhodz * (fabove - flux) * (1.0 / dt);
    if (fpr) fpr[p] = flux;
    fabove = flux;
  }
  *inpr = fabove / c->RHOLW;
}

static int sed_split_column(const C *c, int nij, int nk, double dt, long col, const double *rho,
                            const double *dzz, const double *pabs, const double *tht, const double *exn,
                            double sea, double town, int has_sea_town, const double *rt[6], const double *rvt,
                            double *src[6], double *rvs, double *ths, double *fpr[6], double inpr[6], int max_iter,
                            int nsp)
{
  /* nsp = 5, or 6 with hail (KRR = 7, species 7 of :340-347: XFSEDH, XEXSEDH) */
  const double rtmin[6] = {c->C_RTMIN, c->R_RTMIN, c->I_RTMIN, c->S_RTMIN, c->G_RTMIN, c->H_RTMIN};
  const double gac_gc = c->GAC / c->GC, gac2_gc2 = c->GAC2 / c->GC2;
  double lbc, fsedc, conc, ray;                                   /* :120-165, rain_ice.F90:396-420 */
  if (has_sea_town) {
    ray = dmax(1.0, 0.5 * ((1.0 - sea) * gac_gc + sea * gac2_gc2));
    lbc = dmax(dmin(c->LBC_1, c->LBC_2), sea * c->LBC_2 + (1.0 - sea) * c->LBC_1);
    fsedc = dmax(dmin(c->FSEDC_1, c->FSEDC_2), sea * c->FSEDC_2 + (1.0 - sea) * c->FSEDC_1);
    conc = (1.0 - town) * (sea * c->CONC_SEA + (1.0 - sea) * c->CONC_LAND) + town * c->CONC_URBAN;
  } else {
    ray = dmax(1.0, 0.5 * gac_gc);
    lbc = c->LBC_1;
    fsedc = c->FSEDC_1;
    conc = c->CONC_LAND;
  }
  const double fsed[6] = {0.0, c->FSEDR, 0.0, c->FSEDS, c->FSEDG, c->FSEDH};
  const double exsed[6] = {0.0, c->EXSEDR, 0.0, c->EXSEDS, c->EXSEDG, c->EXSEDH};
  const double thr[6] = {c->C_RTMIN, c->R_RTMIN, dmax(c->I_RTMIN, 1.0e-7), c->S_RTMIN, c->G_RTMIN, c->H_RTMIN};
  double *rx = (double *)malloc(sizeof(double) * 3 * (size_t)nk);
  double *ext = rx + nk, *w = rx + 2 * nk;
  int ok = 1;
  for (int s = 0; s < nsp; ++s) {
    if (s == 0 && c->LSEDIC == 0.0) {
      inpr[0] = 0.0;
      if (fpr[0]) for (int k = 0; k < nk; ++k) fpr[0][(long)k * nij + col] = 0.0;
      continue;
    }
    for (int k = 0; k < nk; ++k) {                               /* :170-200 */
      const long p = (long)k * nij + col;
      rx[k] = rt[s][p];
      ext[k] = src[s][p] - rt[s][p] / dt;
      if (fpr[s]) fpr[s][p] = 0.0;
    }
    double remaint = dt;
    inpr[s] = 0.0;
    int it = 0;
    while (remaint > 0.0) {
      if (++it > max_iter) { ok = 0; break; }
      for (int k = 0; k < nk; ++k) {                             /* fluxes :500-760 */
        const long p = (long)k * nij + col;
        w[k] = 0.0;
        if (rx[k] > thr[s]) {
          double v;
          if (s == 0) {
            const double t = tht[p] * pow(pabs[p] / c->P00, c->RD / c->CPD);
            const double wlbda = 6.6e-8 * (101325.0 / pabs[p]) * (t / 293.15);
            v = sed_cloud(c, rx[k], rho[p], wlbda, lbc, conc, ray, fsedc);
          } else if (s == 2) {
            v = sed_ice(c, rx[k], rho[p]);
          } else {
            v = sed_other(fsed[s], exsed[s], rx[k], rho[p], c->CEXVT);
          }
          w[k] = v * rho[p] * rx[k];
        }
      }
      double mt = remaint;                                       /* :770-805 */
      for (int k = 0; k < nk; ++k) {
        const long p = (long)k * nij + col;
        if (rx[k] > rtmin[s] && w[k] > 1.e-20) mt = dmin(mt, c->SPLIT_MAXCFL * rho[p] * rx[k] * dzz[p] / w[k]);
      }
      remaint -= mt;
      inpr[s] += w[0] / c->RHOLW * (mt / dt);
      for (int k = 0; k < nk; ++k) {                             /* :806-830 */
        const long p = (long)k * nij + col;
        const double wa = k + 1 < nk ? w[k + 1] : 0.0;
        const double change = mt * (1.0 / (rho[p] * dzz[p])) * (wa - w[k]);
        rx[k] = rx[k] + change + ext[k] * mt;
        src[s][p] += change / dt;
        if (fpr[s]) fpr[s][p] += w[k] * (mt / dt);
      }
    }
  }
  free(rx);
  for (int k = 0; k < nk; ++k) {                                 /* ICE4_CORRECT_NEGATIVITIES */
    const long p = (long)k * nij + col;
    double zice = rt[2][p] + rt[3][p] + rt[4][p];
    if (nsp == 6) zice += rt[5][p];
    const double zdev = c->CPD + c->CPV * rvt[p] + c->CL * (rt[0][p] + rt[1][p]) + c->CI * zice;
    const double t = tht[p] * exn[p];
    const double ls = (c->LSTT + (c->CPV - c->CI) * (t - c->TT)) / zdev;
    const double lv = (c->LVTT + (c->CPV - c->CL) * (t - c->TT)) / zdev;
    double rv = rvs[p], rc = src[0][p], rr = src[1][p], ri = src[2][p], rs = src[3][p], rg = src[4][p];
    double th = ths[p], ww;
    ww = rc - dmax(rc, 0.); rv += ww; th -= ww * lv; rc -= ww;
    ww = rr - dmax(rr, 0.); rv += ww; th -= ww * lv; rr -= ww;
    ww = ri - dmax(ri, 0.); rv += ww; th -= ww * ls; ri -= ww;
    ww = rs - dmax(rs, 0.); rv += ww; th -= ww * ls; rs -= ww;
    ww = rg - dmax(rg, 0.); rv += ww; th -= ww * ls; rg -= ww;
    double rh = nsp == 6 ? src[5][p] : 0.0;
    if (nsp == 6) { ww = rh - dmax(rh, 0.); rv += ww; th -= ww * ls; rh -= ww; }
    ww = dmin(1., dmax(c->V_RTMIN - rv, 0.) / dmax(rc + ri, 1.e-20));
    th -= ww * (rc * lv + ri * ls);
    rv += ww * (rc + ri);
    rc = (1. - ww) * rc;
    ri = (1. - ww) * ri;
    ww = dmin(dmax(rr, 0.), dmax(c->V_RTMIN - rv, 0.)); rv += ww; rr -= ww; th -= ww * lv;
    ww = dmin(dmax(rs, 0.), dmax(c->V_RTMIN - rv, 0.)); rv += ww; rs -= ww; th -= ww * ls;
    ww = dmin(dmax(rg, 0.), dmax(c->V_RTMIN - rv, 0.)); rv += ww; rg -= ww; th -= ww * ls;
    if (nsp == 6) { ww = dmin(dmax(rh, 0.), dmax(c->V_RTMIN - rv, 0.)); rv += ww; rh -= ww; th -= ww * ls; }
    rvs[p] = rv; src[0][p] = rc; src[1][p] = rr; src[2][p] = ri; src[3][p] = rs; src[4][p] = rg; ths[p] = th;
    if (nsp == 6) src[5][p] = rh;
  }
  return ok;
}

/* SPLI sedimentation + negativity correction alone on a rain_ice field set
 * (the ICE4_SEDIMENTATION call of rain_ice with SEDIM = SPLI). */
EXPORT int ice3o_sedimentation_split(const C *c, int nij, int nk, double dt, const Ice3gbRainIceFields *f)
{
  const int has = f->sea != NULL && f->town != NULL;
  int ok = 1;
#pragma omp parallel for schedule(static) reduction(& : ok)
  for (long col = 0; col < nij; ++col) {
    const int nsp = (int)c->NRR == 7 ? 6 : 5;
    double *src[6] = {f->rcs, f->rrs, f->ris, f->rss, f->rgs, f->rhs};
    double *fpr[6] = {f->fpr_c, f->fpr_r, f->fpr_i, f->fpr_s, f->fpr_g, f->fpr_h};
    const double *rt[6] = {f->rct, f->rrt, f->rit, f->rst, f->rgt, f->rht};
    double inpr[6];
    ok &= sed_split_column(c, nij, nk, dt, col, f->rhodref, f->dzz, f->pabs, f->tht, f->exn, has ? f->sea[col] : 0.0,
                           has ? f->town[col] : 0.0, has, rt, f->rvt, src, f->rvs, f->ths, fpr, inpr, 10000, nsp);
    f->inprc[col] = inpr[0]; f->inprr[col] = inpr[1]; f->inpri[col] = inpr[2];
    f->inprs[col] = inpr[3]; f->inprg[col] = inpr[4];
    if (nsp == 6) f->inprh[col] = inpr[5];
  }
  return ok;
}

EXPORT int ice3o_sedimentation(const C *c, int nij, int nk, double dt, const Ice3gbSedimentationFields *f)
{
  if (!c || !f || nij <= 0 || nk <= 0) return ICE3GB_ERR_SHAPE;
  const int fortran = f->fortran_semantics != 0;
  const int has = f->sea != NULL && f->town != NULL;
#pragma omp parallel for schedule(static)
  for (long col = 0; col < nij; ++col) {
    double *src[5] = {f->rcs, f->rrs, f->ris, f->rss, f->rgs};
    double *fpr[5] = {f->fpr_c, f->fpr_r, f->fpr_i, f->fpr_s, f->fpr_g};
    double inpr[5];
    const double sea = f->sea ? f->sea[col] : 0.0, town = f->town ? f->town[col] : 0.0;
    sed_column(c, nij, nk, dt, col, fortran, f->rhodref, f->dzz, f->pabs, f->tht, sea, town,
               has, src, fpr, inpr);
    f->inprc[col] = inpr[0];
    f->inprr[col] = inpr[1];
    f->inpri[col] = inpr[2];
    f->inprs[col] = inpr[3];
    f->inprg[col] = inpr[4];
  }
  return ICE3GB_OK;
}

/* ===================================================================== */
/* ICE4 processes (one grid point)                                       */
/* ===================================================================== */

enum { ITH = 0, IRV = 1, IRC = 2, IRR = 3, IRI = 4, IRS = 5, IRG = 6, NV = 7, IRH = 7, NVH = 8 };
/* NV: the KRR = 6 state (theta + 6 mixing ratios); NVH: with hail (KRR = 7). */

/* Instantaneous/rate budget slots (Fortran IBU* indices, KRR=6 subset). */
enum {
  B_RVHENI_MR, B_RRHONG_MR, B_RIMLTC_MR, B_RSRIMCG_MR,
  B_RCHONI, B_RVDEPS, B_RIAGGS, B_RIAUTS, B_RVDEPG,
  B_RCAUTR, B_RCACCR, B_RREVAV,
  B_RCRIMSS, B_RCRIMSG, B_RSRIMCG, B_RRACCSS, B_RRACCSG, B_RSACCRG, B_RSMLTG, B_RCMLTSR,
  B_RICFRRG, B_RRCFRIG, B_RICFRR, B_RCWETG, B_RIWETG, B_RRWETG, B_RSWETG,
  B_RCDRYG, B_RIDRYG, B_RRDRYG, B_RSDRYG, B_RGMLTR, B_RCBERI,
  /* KRR = 7: graupel -> hail conversion and ICE4_FAST_RH */
  B_RWETGH, B_RWETGH_MR, B_RCWETH, B_RIWETH, B_RSWETH, B_RGWETH, B_RRWETH,
  B_RCDRYH, B_RIDRYH, B_RSDRYH, B_RRDRYH, B_RGDRYH, B_RDRYHG, B_RHMLTR,
  /* OCND2: ICE4_FAST_RI_RS */
  B_RVDEPI, B_RILARS,
  NBU
};
/* fast_rs persistent tendencies (mode_ice4_fast_rs.F90 IRCRIMS..IFREEZ2) */
enum { RS_RCRIMS, RS_RCRIMSS, RS_RSRIMCG, RS_RRACCS, RS_RRACCSS, RS_RSACCRG, RS_FREEZ1, RS_FREEZ2, NRS };
/* fast_rg persistent tendencies (mode_ice4_fast_rg.F90 IRCDRYG..IFREEZ2) */
enum { RG_RCDRYG, RG_RIDRYG, RG_RIWETG, RG_RSDRYG, RG_RSWETG, RG_RRDRYG, RG_FREEZ1, RG_FREEZ2, NRG };
/* fast_rh persistent tendencies (mode_ice4_fast_rh.F90 IRCWETH..IFREEZ2) */
enum { RH_RCWETH, RH_RRWETH, RH_RIDRYH, RH_RIWETH, RH_RSDRYH, RH_RSWETH, RH_RGDRYH, RH_RGWETH, RH_FREEZ1,
       RH_FREEZ2, NRH };

typedef struct {
  double bu[NBU];
  double rs_tend[NRS];
  double rg_tend[NRG];
  double rh_tend[NRH];
  double ssi, ka, dv, ai, cj;
  int tie;    /* a wet/dry growth choice was decided by rounding residuals */
  double esi, colf, acrf;   /* OCND2, hard pass: tabulated es_i, collision factors */
} PointRates;

/* The wet/dry growth choice compares max(0, .) of differences whose exact
 * value is often zero (what the wet growth collects equals its initial
 * estimate); when such a difference cancels two or more non-zero rates, its
 * computed value is a rounding residual and which side wins depends on the
 * last bits of the rates.  nz: the number of non-zero rates cancelled. */
static inline int growth_tie(double a, double b, double scale, int nz)
{
  return nz >= 2 && fabs(a - b) <= 1e-13 * scale;
}
static inline int nonzero(double a, double b, double c, double d, double e)
{
  return (a != 0.) + (b != 0.) + (c != 0.) + (d != 0.) + (e != 0.);
}

static inline double esatw(const C *c, double t) { return exp(c->ALPW - c->BETAW / t - c->GAMW * log(t)); }
static inline double esati(const C *c, double t) { return exp(c->ALPI - c->BETAI / t - c->GAMI * log(t)); }

/* ICE4_NUCLEATION, micro/ice4_nucleation.func.h:69-144 (LOCND2 = .FALSE.). */
static double tiwmx_at(const double *tab, double t);

/* tw != NULL: the OCND2 branch (:127-136): concentration from REDIN, AM3,
 * the height zzz and the ice cloud fraction, no vapour taken (HENI = 0). */
static void ice4_nucleation(const C *c, int ldcompute, double tht, double pabst, double rhodref,
                            double exn, double lsfact, double t, double rvt, double *cit,
                            double *rvheni_mr, double *ssi_out, const double *tw, double zzz, double icldfr)
{
  const int gnegt = ldcompute && t < c->TT && rvt > c->V_RTMIN;
  double zusw = 0.0, zzw = 0.0, zssi = 0.0;
  *rvheni_mr = 0.0;
  if (tw) {
    if (gnegt) {
      const double redin = tiwmx_at(tw + TW_REDIN * TIWMX_N, t);
      const double am3 = tiwmx_at(tw + TW_AM3 * TIWMX_N, dmax(c->FRMIN27, t));
      const double h = (20000. - dmin(20000., zzz)) / 20000.;
      zzw = redin * dmax(0.1, h * h * h * h) * am3 * (0.0001 + 0.9999 * icldfr);
      zzw = dmin(zzw, 50.e3);
      *cit = dmax(zzw + *cit, *cit);
    }
    if (ssi_out) *ssi_out = 0.0;
    return;
  }
  if (gnegt) {
    zzw = log(t);
    zusw = exp(c->ALPW - c->BETAW / t - c->GAMW * zzw);
    zzw = exp(c->ALPI - c->BETAI / t - c->GAMI * zzw);
    zzw = dmin(pabst / 2.0, zzw);
    zssi = rvt * (pabst - zzw) / (c->EPSILO * zzw) - 1.0;
    zusw = dmin(pabst / 2.0, zusw);
    zusw = (zusw / zzw) * ((pabst - zzw) / (pabst - zusw)) - 1.0;
    zssi = dmin(zssi, zusw);
    zzw = 0.0;
    if (t < c->TT - 5.0 && zssi > 0.0) {
      zzw = c->NU20 * exp(c->ALPHA2 * zssi - c->BETA2);
    } else if (t <= c->TT - 2.0 && t >= c->TT - 5.0 && zssi > 0.0) {
      zzw = dmax(c->NU20 * exp(-c->BETA2), c->NU10 * exp(-c->BETA1 * (t - c->TT)) * pow(zssi / zusw, c->ALPHA1));
    }
    zzw = zzw - *cit;
    zzw = dmin(zzw, 50.e3);
    *rvheni_mr = dmax(zzw, 0.0) * c->MNU0 / rhodref;
    *rvheni_mr = dmin(rvt, *rvheni_mr);
    if (c->LFEEDBACKT != 0.0) {
      const double w = dmin(*rvheni_mr, dmax(0.0, (c->TT / exn - tht) / lsfact)) / dmax(*rvheni_mr, 1.e-20);
      *rvheni_mr *= w;
      zzw *= w;
    }
    *cit = dmax(zzw + *cit, *cit);
  }
  if (ssi_out) *ssi_out = zssi;
}

/* ICE4_RRHONG, micro/mode_ice4_rrhong.F90. */
static double ice4_rrhong(const C *c, int ldcompute, double exn, double lvfact, double lsfact,
                          double t, double rrt, double tht)
{
  if (t < c->TT - 35.0 && rrt > c->R_RTMIN && ldcompute) {
    double r = rrt;
    if (c->LFEEDBACKT != 0.0) r = dmin(r, dmax(0.0, ((c->TT - 35.0) / exn - tht) / (lsfact - lvfact)));
    return r;
  }
  return 0.0;
}

/* ICE4_RIMLTC, micro/mode_ice4_rimltc.F90. */
static double ice4_rimltc(const C *c, int ldcompute, double exn, double lvfact, double lsfact,
                          double t, double tht, double rit)
{
  if (rit > 0.0 && t > c->TT && ldcompute) {
    double r = rit;
    if (c->LFEEDBACKT != 0.0) r = dmin(r, dmax(0.0, (tht - c->TT / exn) / (lsfact - lvfact)));
    return r;
  }
  return 0.0;
}

/* Derived fields, mode_ice4_tendencies.F90:303-320 (non-tabulated branch);
 * same formulas as stencils/ice4_tendencies.py:191-245. */
static void ice4_derived(const C *c, double t, double rhodref, double pres, double rv,
                         double *ssi, double *ka, double *dv, double *ai, double *cj)
{
  const double zzw = exp(c->ALPI - c->BETAI / t - c->GAMI * log(t));
  *ssi = rv * (pres - zzw) / (c->EPSILO * zzw) - 1.0;
  *ka = 2.38e-2 + 7.1e-5 * (t - c->TT);
  *dv = 2.11e-5 * pow(t / c->TT, 1.94) * (c->P00 / pres);
  *ai = sq(c->LSTT + (c->CPV - c->CI) * (t - c->TT)) / (*ka * c->RV * sq(t)) + (c->RV * t) / (*dv * zzw);
  *cj = c->SCFAC * pow(rhodref, 0.3) / sqrt(1.718e-5 + 4.9e-8 * (t - c->TT));
}

/* ICE4_COMPUTE_PDF, micro/mode_ice4_compute_pdf.F90 (one point).
 * hl[0..3] = HLC_HCF, HLC_LCF, HLC_HRC, HLC_LRC; hi[0..3] = HLI_HCF, HLI_LCF,
 * HLI_HRI, HLI_LRI (in-out for the ADJU modes).  Returns the rain fraction. */
static double ice4_compute_pdf(const C *c, int ldmicro, double rhodref, double rct, double rit,
                               double cf, double t, double sigma_rc, double hl[4], double hi[4])
{
  const int aucv_rc = (int)c->SUBG_AUCV_RC, aucv_ri = (int)c->SUBG_AUCV_RI, prpdf = (int)c->SUBG_PR_PDF;
  const double rcrautc = ldmicro ? c->CRIAUTC / rhodref : 0.0;
  double hcf = 0, lcf = 0, hrc = 0, lrc = 0;
  if (aucv_rc == 0) {               /* NONE */
    if (rct > rcrautc && ldmicro) { hcf = 1.0; hrc = rct; }
    else if (rct > c->C_RTMIN && ldmicro) { lcf = 1.0; lrc = rct; }
  } else if (aucv_rc == 3) {        /* CLFR */
    if (cf > 0.0 && rct > rcrautc * cf && ldmicro) { hcf = cf; hrc = rct; }
    else if (cf > 0.0 && rct > c->C_RTMIN && ldmicro) { lcf = cf; lrc = rct; }
  } else if (aucv_rc == 2) {        /* ADJU */
    const double sum = ldmicro ? hl[3] + hl[2] : 0.0;
    hcf = hl[0]; lcf = hl[1];
    if (sum > 1.e-20 && ldmicro) { lrc = hl[3] * rct / sum; hrc = hl[2] * rct / sum; }
  } else if (aucv_rc == 1 && prpdf == 0) {  /* PDF + SIGM */
    if (rct > rcrautc + sigma_rc && ldmicro) {
      hcf = 1.0; hrc = rct;
    } else if (rct > rcrautc - sigma_rc && rct <= rcrautc + sigma_rc && ldmicro) {
      hcf = (rct + sigma_rc - rcrautc) / (2.0 * sigma_rc);
      lcf = dmax(0.0, cf - hcf);
      hrc = (rct + sigma_rc - rcrautc) * (rct + sigma_rc + rcrautc) / (4.0 * sigma_rc);
      lrc = dmax(0.0, rct - hrc);
    } else if (rct > c->C_RTMIN && cf > 0.0 && ldmicro) {
      lcf = cf; lrc = rct;
    }
  } else if (aucv_rc == 1) {        /* PDF + HLC*PDF */
    const double coeff = (prpdf == 1 || prpdf == 2) ? 2.0 : (prpdf == 3 ? 3.0 : 4.0);
    const double rcmax = (rct > 0.0 && cf > 0.0 && ldmicro) ? coeff * rct / cf : 0.0;
    double lloc = 0.0, hloc = 0.0;
    const int ok = rct > 0.0 && cf > 0.0 && rcmax > rcrautc && ldmicro;
    if (prpdf == 1) {
      if (ok) { lloc = 0.5 * rcrautc; hloc = (rcmax + rcrautc) / 2.0; }
    } else if (prpdf == 3) {
      if (ok) {
        lloc = (rcrautc * (3.0 * rcmax - 2.0 * rcrautc)) / (3.0 * (2.0 * rcmax - rcrautc));
        hloc = (rcmax + 2.0 * rcrautc) / 3.0;
      }
    } else if (prpdf == 4) {
      if (ok) {
        lloc = (3.0 * pow(rcrautc, 3) - 8.0 * sq(rcrautc) * rcmax + 6.0 * rcrautc * sq(rcmax)) /
               (4.0 * sq(rcrautc) - 12.0 * rcrautc * rcmax + 12.0 * sq(rcmax));
        hloc = (rcmax + 3.0 * rcrautc) / 4.0;
      }
    } else if (prpdf == 2) {
      if (rct <= rcrautc * cf && ok) {
        lloc = (pow(rcmax, 3) - 12.0 * rcmax * sq(rcrautc) + 8.0 * pow(rcrautc, 3)) /
               (6.0 * sq(rcmax) - 24.0 * rcmax * rcrautc + 12.0 * sq(rcrautc));
        hloc = (rcmax + 2.0 * rcrautc) / 3.0;
      } else if (ok) {
        lloc = (2.0 / 3.0) * rcrautc;
        hloc = (3.0 * pow(rcmax, 3) - 8.0 * pow(rcrautc, 3)) / (6.0 * sq(rcmax) - 12.0 * sq(rcrautc));
      }
    }
    if (ok) {
      lcf = cf * (hloc - (rct / cf)) / (hloc - lloc);
      hcf = dmax(0.0, cf - lcf);
      lrc = lloc * lcf;
      hrc = dmax(0.0, rct - lrc);
    } else if (rct > 0.0 && cf > 0.0 && rcmax <= rcrautc && ldmicro) {
      lcf = cf; lrc = rct;
    }
  }
  hl[0] = hcf; hl[1] = lcf; hl[2] = hrc; hl[3] = lrc;
  const double criauti = ldmicro ? dmin(c->CRIAUTI, pow(10.0, c->ACRIAUTI * (t - c->TT) + c->BCRIAUTI)) : 0.0;
  double ihcf = 0, ilcf = 0, ihri = 0, ilri = 0;
  if (aucv_ri == 0) {
    if (rit > criauti && ldmicro) { ihcf = 1.0; ihri = rit; }
    else if (rit > c->I_RTMIN && ldmicro) { ilcf = 1.0; ilri = rit; }
  } else if (aucv_ri == 1) {
    if (cf > 0.0 && rit > criauti * cf && ldmicro) { ihcf = cf; ihri = rit; }
    else if (cf > 0.0 && rit > c->I_RTMIN && ldmicro) { ilcf = cf; ilri = rit; }
  } else if (aucv_ri == 2) {
    const double sum = ldmicro ? hi[3] + hi[2] : 0.0;
    ihcf = hi[0]; ilcf = hi[1];
    if (sum > 1.e-20 && ldmicro) { ilri = hi[3] * rit / sum; ihri = hi[2] * rit / sum; }
  }
  hi[0] = ihcf; hi[1] = ilcf; hi[2] = ihri; hi[3] = ilri;
  return ldmicro ? dmax(hl[0], hi[0]) : 0.0;
}

/* INTERP_MICRO_1D / _2D (packed path), micro/interp_micro.func.h:5-269. */
static inline double lut_index(double x, int knum, double p1, double p2, int *i)
{
  double z = dmax(1.00001, dmin((double)knum - 0.00001, p1 * log(x) + p2));
  *i = (int)z;
  return z - (double)(*i);
}
static inline double lut1d(const double *lt, int i, double f)
{
  return lt[i] * f - lt[i - 1] * (f - 1.0);  /* PLT(I+1)*F - PLT(I)*(F-1) */
}
/* PLT(i1, i2) with Fortran 1-based (i1, i2) = row-major lt[(i1-1)*n2 + (i2-1)] */
static inline double lut2d(const double *lt, int n2, int i1, double f1, int i2, double f2)
{
#define L(a, b) lt[((a) - 1) * n2 + ((b) - 1)]
  return (L(i1 + 1, i2 + 1) * f2 - L(i1 + 1, i2) * (f2 - 1.0)) * f1 -
         (L(i1, i2 + 1) * f2 - L(i1, i2) * (f2 - 1.0)) * (f1 - 1.0);
#undef L
}

/* OCND2 inputs of one point: the TIWMX tables, the ice_adjust OCND2 outputs
 * (super-saturations over ice in the cloudy / clear parts, PIFR, the ice
 * cloud fraction), the level height (rain_ice.F90:386-394) and the cloud
 * droplet concentration (:396-435). */
typedef struct {
  const double *tw;
  double ssio, ssiu, ifr, icldfr, zzz, conc;
} Ocnd2Pt;

/* Per-point context passed to the process routines. */
typedef struct {
  const C *c;
  const Ice3gbLuts *lut;
  int ldsoft, ldcompute;
  double rhodref, pres, exn, lvfact, lsfact, cf, sigma_rc;
  double t;          /* temperature after the instantaneous processes */
  double v[NVH];     /* state after the instantaneous processes       */
  double lbdar, lbdar_rf, lbdas, lbdag, lbdah;
  int hail;          /* KRR = 7                                       */
  /* OCND2 (tw != NULL): TIWMX tables and the per-point inputs */
  const double *tw;
  double ssio, ssiu, ifr, icldfr, zzz, conc;
  double rainfr;     /* PRAINFR (packed, per point)                   */
  double hl[4], hi[4];
} Tctx;

/* ICE4_SLOW, micro/mode_ice4_slow.F90 (LNEWCOEFF = LOCND2 = .FALSE.). */
static void ice4_slow(const Tctx *x, PointRates *pr)
{
  const C *c = x->c;
  const double t = x->t, rho = x->rhodref;
  double *b = pr->bu;
  if (t < c->TT - 35.0 && x->v[IRC] > c->C_RTMIN && x->ldcompute) {
    if (!x->ldsoft) b[B_RCHONI] = dmin(1000., c->HON * rho * x->v[IRC] * exp(c->ALPHA3 * (t - c->TT) - c->BETA3));
  } else b[B_RCHONI] = 0.0;
  if (x->v[IRV] > c->V_RTMIN && x->v[IRS] > c->S_RTMIN && x->ldcompute) {
    if (!x->ldsoft) {
      b[B_RVDEPS] = (pr->ssi / (rho * pr->ai)) *
                    (c->O0DEPS * pow(x->lbdas, c->EX0DEPS) + c->O1DEPS * pr->cj * pow(x->lbdas, c->EX1DEPS));
      if (x->tw) b[B_RVDEPS] = b[B_RVDEPS] * c->FRMIN40;        /* ZREDSN, :92-99, 142 */
    }
  } else b[B_RVDEPS] = 0.0;
  if (x->v[IRI] > c->I_RTMIN && x->v[IRS] > c->S_RTMIN && x->ldcompute) {
    if (!x->ldsoft)
      b[B_RIAGGS] = c->FIAGGS * exp(c->COLEXIS * (t - c->TT)) * x->v[IRI] * pow(x->lbdas, c->EXIAGGS) *
                    pow(rho, -c->CEXVT);
  } else b[B_RIAGGS] = 0.0;
  if (x->hi[2] > c->I_RTMIN && x->ldcompute) {
    if (!x->ldsoft) {
      const double criauti = dmin(c->CRIAUTI, pow(10.0, c->ACRIAUTI * (t - c->TT) + c->BCRIAUTI));
      b[B_RIAUTS] = c->TIMAUTI * exp(c->TEXAUTI * (t - c->TT)) * dmax(x->hi[2] - criauti * x->hi[0], 0.0);
    }
  } else b[B_RIAUTS] = 0.0;
  if (x->v[IRV] > c->V_RTMIN && x->v[IRG] > c->G_RTMIN && x->ldcompute) {
    if (!x->ldsoft) {
      b[B_RVDEPG] = (pr->ssi / (rho * pr->ai)) *
                    (c->O0DEPG * pow(x->lbdag, c->EX0DEPG) + c->O1DEPG * pr->cj * pow(x->lbdag, c->EX1DEPG));
      if (x->tw) b[B_RVDEPG] = b[B_RVDEPG] * c->FRMIN39;        /* ZREDGR, :212 */
    }
  } else b[B_RVDEPG] = 0.0;
}

/* ICE4_WARM, micro/mode_ice4_warm.F90 (LKOGAN = .FALSE.). */
static void ice4_warm(const Tctx *x, PointRates *pr)
{
  const C *c = x->c;
  const double t = x->t, rho = x->rhodref;
  double *b = pr->bu;
  if (c->LWARM == 0.0) { b[B_RCAUTR] = b[B_RCACCR] = b[B_RREVAV] = 0.0; return; }
  if (x->hl[2] > c->C_RTMIN && x->hl[0] > 0.0 && x->ldcompute) {
    if (!x->ldsoft) b[B_RCAUTR] = c->TIMAUTC * dmax(x->hl[2] - x->hl[0] * c->CRIAUTC / rho, 0.0);
  } else b[B_RCAUTR] = 0.0;
  if ((int)c->SUBG_RC_RR_ACCR == 0) {
    if (x->v[IRC] > c->C_RTMIN && x->v[IRR] > c->R_RTMIN && x->ldcompute) {
      if (!x->ldsoft)
        b[B_RCACCR] = c->FCACCR * x->v[IRC] * (x->tw ? pr->acrf : 1.0) /* PACRF */ * pow(x->lbdar, c->EXCACCR) *
                      pow(rho, -c->CEXVT);
    } else b[B_RCACCR] = 0.0;
  } else {
    const int m = x->v[IRC] > c->C_RTMIN && x->v[IRR] > c->R_RTMIN && x->ldcompute;
    const int m1 = m && x->hl[2] > c->C_RTMIN && x->hl[0] > 0.0;
    const int m2 = m && x->hl[3] > c->C_RTMIN && x->hl[1] > 1.e-20;
    if (m1 || m2) {
      if (!x->ldsoft) {
        double r = 0.0;
        if (m1) r = c->FCACCR * x->hl[2] * pow(x->lbdar_rf, c->EXCACCR) * pow(rho, -c->CEXVT);
        if (m2)
          r += c->FCACCR * (x->hl[3] / x->hl[1]) * pow(x->lbdar_rf, c->EXCACCR) * pow(rho, -c->CEXVT) *
               (dmin(x->cf, x->rainfr) - x->hl[0]);
        b[B_RCACCR] = r;
      }
    } else b[B_RCACCR] = 0.0;
  }
  const int evap = (int)c->SUBG_RR_EVAP;
  if (evap == 0) {
    if (x->v[IRR] > c->R_RTMIN && x->v[IRC] <= c->C_RTMIN && x->ldcompute) {
      if (!x->ldsoft) {
        double r = esatw(c, t);
        const double usw = 1. - x->v[IRV] * (x->pres - r) / (c->EPSILO * r);
        r = sq(c->LVTT + (c->CPV - c->CL) * (t - c->TT)) / (pr->ka * c->RV * sq(t)) + (c->RV * t) / (pr->dv * r);
        b[B_RREVAV] = (dmax(0., usw) / (rho * r)) *
                      (c->O0EVAR * pow(x->lbdar, c->EX0EVAR) + c->O1EVAR * pr->cj * pow(x->lbdar, c->EX1EVAR));
      }
    } else b[B_RREVAV] = 0.0;
  } else {
    const double zw4 = (evap == 1) ? 1.0 : x->rainfr;
    const double zw3 = (evap == 1) ? x->lbdar : x->lbdar_rf;
    if (x->v[IRR] > c->R_RTMIN && zw4 > x->cf && x->ldcompute) {
      if (!x->ldsoft) {
        const double tht = x->v[ITH];
        const double thlt = tht - c->LVTT * tht / c->CPD / t * x->v[IRC];
        const double zw2 = thlt * t / tht;
        double r = esatw(c, zw2);
        const double usw = 1.0 - x->v[IRV] * (x->pres - r) / (c->EPSILO * r);
        r = sq(c->LVTT + (c->CPV - c->CL) * (zw2 - c->TT)) / (pr->ka * c->RV * sq(zw2)) + (c->RV * zw2) / (pr->dv * r);
        r = dmax(0., usw) / (rho * r) * (c->O0EVAR * pow(zw3, c->EX0EVAR) + c->O1EVAR * pr->cj * pow(zw3, c->EX1EVAR));
        b[B_RREVAV] = r * (zw4 - x->cf);
      }
    } else b[B_RREVAV] = 0.0;
  }
}

/* Vapour/heat term shared by the freezing-rate and melting computations of
 * fast_rs/fast_rg (mode_ice4_fast_rs.F90 IFREEZ1 / RSMLTG, fast_rg IFREEZ1 / RGMLTR). */
static inline double heat_term(const C *c, double ka, double dv, double t, double rv, double pres, int ice)
{
  double e = rv * pres / (c->EPSILO + rv);
  if (c->LEVLIMIT != 0.0) e = dmin(e, ice ? esati(c, t) : esatw(c, t));
  return ka * (c->TT - t) + (dv * (c->LVTT + (c->CPV - c->CL) * (t - c->TT)) * (c->ESTT - e) / (c->RV * t));
}

/* ICE4_FAST_RS, micro/mode_ice4_fast_rs.F90 (LNEWCOEFF = LOCND2 = .FALSE.). */
static void ice4_fast_rs(const Tctx *x, PointRates *pr)
{
  const C *c = x->c;
  const Ice3gbLuts *lut = x->lut;
  const double t = x->t, rho = x->rhodref, lbdas = x->lbdas, lbdar = x->lbdar;
  double *b = pr->bu, *rs = pr->rs_tend;
  double freez;
  if (x->v[IRS] > c->S_RTMIN && x->ldcompute) {                       /* :100-142 */
    if (!x->ldsoft) {
      double f1 = heat_term(c, pr->ka, pr->dv, t, x->v[IRV], x->pres, 1);
      f1 = f1 * (c->O0DEPS * pow(lbdas, c->EX0DEPS) + c->O1DEPS * pr->cj * pow(lbdas, c->EX1DEPS)) /
           (rho * (c->LMTT - c->CL * (c->TT - t)));
      rs[RS_FREEZ1] = f1;
      rs[RS_FREEZ2] = (rho * (c->LMTT + (c->CI - c->CL) * (c->TT - t))) / (rho * (c->LMTT - c->CL * (c->TT - t)));
    }
    freez = dmax(0., dmax(0., rs[RS_FREEZ1] + rs[RS_FREEZ2] * b[B_RIAGGS]) - b[B_RIAGGS]);
  } else {
    rs[RS_FREEZ1] = rs[RS_FREEZ2] = 0.0;
    freez = 0.0;
  }
  /* riming: :149-274 */
  const int grim = x->v[IRC] > c->C_RTMIN && x->v[IRS] > c->S_RTMIN && x->ldcompute;
  if (!grim) rs[RS_RCRIMS] = rs[RS_RCRIMSS] = rs[RS_RSRIMCG] = 0.0;
  if (!x->ldsoft && grim) {
    int i;
    const double fr = lut_index(lbdas, (int)c->NGAMINC, c->RIMINTP1, c->RIMINTP2, &i);
    const double zw1 = lut1d(lut->gaminc_rim1, i, fr);
    const double zw2 = lut1d(lut->gaminc_rim2, i, fr);
    const double zw3 = lut1d(lut->gaminc_rim4, i, fr);
    const double colf = x->tw ? pr->colf : 1.0;                      /* PCOLF */
    rs[RS_RCRIMSS] = c->CRIMSS * zw1 * x->v[IRC] * colf * pow(lbdas, c->EXCRIMSS) * pow(rho, -c->CEXVT);
    rs[RS_RCRIMS] = c->CRIMSG * x->v[IRC] * colf * pow(lbdas, c->EXCRIMSG) * pow(rho, -c->CEXVT);
    if ((int)c->SNOW_RIMING == 0) { /* M90 */
      const double zzw = rs[RS_RCRIMS] - rs[RS_RCRIMSS];
      double r = c->SRIMCG * pow(lbdas, c->EXSRIMCG) * (1.0 - zw2);
      r = zzw * r / dmax(1.e-20, c->SRIMCG3 * c->SRIMCG2 * pow(lbdas, c->EXSRIMCG2) * (1. - zw3) - c->SRIMCG3 * r);
      rs[RS_RSRIMCG] = r;
    } else rs[RS_RSRIMCG] = 0.0;
  }
  if (grim && t < c->TT) {
    b[B_RCRIMSS] = dmin(freez, rs[RS_RCRIMSS]);
    freez = dmax(0., freez - b[B_RCRIMSS]);
    const double zzw0 = dmin(1., freez / dmax(1.e-20, rs[RS_RCRIMS] - b[B_RCRIMSS]));
    b[B_RCRIMSG] = zzw0 * dmax(0., rs[RS_RCRIMS] - b[B_RCRIMSS]);
    freez = dmax(0., freez - b[B_RCRIMSG]);
    b[B_RSRIMCG] = zzw0 * rs[RS_RSRIMCG];
    b[B_RSRIMCG] *= signbit(b[B_RCRIMSG]) ? 0.0 : 1.0;  /* MAX(0., -SIGN(1., -PRCRIMSG)) */
    b[B_RCRIMSG] = dmax(0., b[B_RCRIMSG]);
  } else {
    b[B_RCRIMSS] = b[B_RCRIMSG] = b[B_RSRIMCG] = 0.0;
  }
  /* accretion of rain on snow: :281-388 */
  const int gacc = x->v[IRR] > c->R_RTMIN && x->v[IRS] > c->S_RTMIN && x->ldcompute;
  if (!gacc) rs[RS_RRACCS] = rs[RS_RRACCSS] = rs[RS_RSACCRG] = 0.0;
  if (!x->ldsoft) {
    rs[RS_RRACCS] = rs[RS_RRACCSS] = rs[RS_RSACCRG] = 0.0;
    if (gacc) {
      int i1, i2;
      const double f1 = lut_index(lbdas, (int)c->NACCLBDAS, c->ACCINTP1S, c->ACCINTP2S, &i1);
      const double f2 = lut_index(lbdar, (int)c->NACCLBDAR, c->ACCINTP1R, c->ACCINTP2R, &i2);
      const double zw1 = lut2d(lut->ker_raccss, ICE3GB_NACCLBDAR, i1, f1, i2, f2);
      const double zw2 = lut2d(lut->ker_raccs, ICE3GB_NACCLBDAR, i1, f1, i2, f2);
      const double zw3 = lut2d(lut->ker_saccrg, ICE3GB_NACCLBDAS, i2, f2, i1, f1);
      const double zzw = c->FRACCSS * pow(lbdas, c->CXS) * pow(rho, -c->CEXVT - 1.) *
                         (c->LBRACCS1 / sq(lbdas) + c->LBRACCS2 / (lbdas * lbdar) + c->LBRACCS3 / sq(lbdar)) /
                         sq(sq(lbdar));
      rs[RS_RRACCSS] = zw1 * zzw;
      if (x->tw) rs[RS_RRACCSS] = rs[RS_RRACCSS] * c->FRMIN7;         /* :327 */
      rs[RS_RRACCS] = zw2 * zzw;
      if (!x->tw || x->v[IRS] > c->FRMIN1)                             /* :347 */
        rs[RS_RSACCRG] = c->FSACCRG * zw3 * pow(lbdas, c->CXS - c->BS) * pow(rho, -c->CEXVT - 1.) *
                         (c->LBSACCR1 / sq(lbdar) + c->LBSACCR2 / (lbdar * lbdas) + c->LBSACCR3 / sq(lbdas)) / lbdar;
    }
  }
  if (gacc && t < c->TT) {
    b[B_RRACCSS] = dmin(freez, rs[RS_RRACCSS]);
    freez = dmax(0., freez - b[B_RRACCSS]);
    const double zzw = dmin(1., freez / dmax(1.e-20, rs[RS_RRACCS] - b[B_RRACCSS]));
    b[B_RRACCSG] = zzw * dmax(0., rs[RS_RRACCS] - b[B_RRACCSS]);
    freez = dmax(0., freez - b[B_RRACCSG]);
    b[B_RSACCRG] = zzw * rs[RS_RSACCRG];
    b[B_RSACCRG] *= signbit(b[B_RRACCSG]) ? 0.0 : 1.0;
    b[B_RRACCSG] = dmax(0., b[B_RRACCSG]);
  } else {
    b[B_RRACCSS] = b[B_RRACCSG] = b[B_RSACCRG] = 0.0;
  }
  /* conversion-melting of snow: :396-441 */
  if (x->v[IRS] > c->S_RTMIN && t > c->TT && x->ldcompute) {
    if (!x->ldsoft) {
      double r = heat_term(c, pr->ka, pr->dv, t, x->v[IRV], x->pres, 0);
      r = c->FSCVMG * dmax(0., (-r * (c->O0DEPS * pow(lbdas, c->EX0DEPS) + c->O1DEPS * pr->cj * pow(lbdas, c->EX1DEPS)) -
                                 (rs[RS_RCRIMS] + rs[RS_RRACCS]) * (rho * c->CL * (c->TT - t))) /
                                (rho * c->LMTT));
      b[B_RSMLTG] = r;
      b[B_RCMLTSR] = rs[RS_RCRIMS];
    }
  } else {
    b[B_RSMLTG] = b[B_RCMLTSR] = 0.0;
  }
}

/* ICE4_FAST_RG, micro/mode_ice4_fast_rg.F90 (KRR = 6, LOCND2 = LNEWCOEFF = .FALSE.). */
static int ice4_fast_rg(const Tctx *x, PointRates *pr, double cit)
{
  const C *c = x->c;
  const Ice3gbLuts *lut = x->lut;
  const double t = x->t, rho = x->rhodref, lbdar = x->lbdar, lbdas = x->lbdas, lbdag = x->lbdag;
  double *b = pr->bu, *rg = pr->rg_tend;
  /* rain contact freezing: :~100-176 */
  if (x->v[IRI] > c->I_RTMIN && x->v[IRR] > c->R_RTMIN && x->ldcompute) {
    if (!x->ldsoft) {
      b[B_RICFRRG] = c->ICFRR * x->v[IRI] * pow(lbdar, c->EXICFRR) * pow(rho, -c->CEXVT);
      b[B_RRCFRIG] = c->RCFRI * cit * pow(lbdar, c->EXRCFRI) * pow(rho, -c->CEXVT - 1.);
      if (c->LCRFLIMIT != 0.0) {
        const double zw = dmax(0., dmin(1., (b[B_RICFRRG] * c->CI + b[B_RRCFRIG] * c->CL) * (c->TT - t) /
                                               dmax(1.e-20, c->LVTT * b[B_RRCFRIG])));
        b[B_RRCFRIG] = zw * b[B_RRCFRIG];
        b[B_RICFRR] = (1. - zw) * b[B_RICFRRG];
        b[B_RICFRRG] = zw * b[B_RICFRRG];
      } else b[B_RICFRR] = 0.0;
    }
  } else {
    b[B_RICFRRG] = b[B_RRCFRIG] = b[B_RICFRR] = 0.0;
  }
  /* cloud/pristine collection: :182-~200 */
  if (x->v[IRG] > c->G_RTMIN && x->v[IRC] > c->C_RTMIN && x->ldcompute) {
    if (!x->ldsoft)
      rg[RG_RCDRYG] = c->FCDRYG * x->v[IRC] * (pow(lbdag, c->CXG - c->DG - 2.) * pow(rho, -c->CEXVT));
  } else rg[RG_RCDRYG] = 0.0;
  if (x->v[IRG] > c->G_RTMIN && x->v[IRI] > c->I_RTMIN && x->ldcompute) {
    if (!x->ldsoft) {
      const double base = pow(lbdag, c->CXG - c->DG - 2.) * pow(rho, -c->CEXVT);
      rg[RG_RIDRYG] = c->FIDRYG * exp(c->COLEXIG * (t - c->TT)) * x->v[IRI] * base;
      rg[RG_RIWETG] = rg[RG_RIDRYG] / (c->COLIG * exp(c->COLEXIG * (t - c->TT)));
    }
  } else rg[RG_RIDRYG] = rg[RG_RIWETG] = 0.0;
  /* snow collection (SDRYG LUT): :203-235 */
  const int gdry_s = x->v[IRS] > c->S_RTMIN && x->v[IRG] > c->G_RTMIN && x->ldcompute;
  if (!gdry_s || x->tw) rg[RG_RSDRYG] = rg[RG_RSWETG] = 0.0;      /* OCND2: no snow-graupel collection */
  if (!x->ldsoft && gdry_s && !x->tw) {
    int i1, i2;
    const double f1 = lut_index(lbdag, (int)c->NDRYLBDAG, c->DRYINTP1G, c->DRYINTP2G, &i1);
    const double f2 = lut_index(lbdas, (int)c->NDRYLBDAS, c->DRYINTP1S, c->DRYINTP2S, &i2);
    const double zw = lut2d(lut->ker_sdryg, ICE3GB_NDRYLBDAS, i1, f1, i2, f2);
    rg[RG_RSWETG] = c->FSDRYG * zw / c->COLSG * pow(lbdas, c->CXS - c->BS) * pow(lbdag, c->CXG) *
                    pow(rho, -c->CEXVT - 1.) *
                    (c->LBSDRYG1 / sq(lbdag) + c->LBSDRYG2 / (lbdag * lbdas) + c->LBSDRYG3 / sq(lbdas));
    rg[RG_RSDRYG] = rg[RG_RSWETG] * c->COLSG * exp(c->COLEXSG * (t - c->TT));
  }
  /* rain collection (RDRYG LUT): :241-271 */
  const int gdry_r = x->v[IRR] > c->R_RTMIN && x->v[IRG] > c->G_RTMIN && x->ldcompute;
  if (!gdry_r) rg[RG_RRDRYG] = 0.0;
  if (!x->ldsoft && gdry_r) {
    int i1, i2;
    const double f1 = lut_index(lbdag, (int)c->NDRYLBDAG, c->DRYINTP1G, c->DRYINTP2G, &i1);
    const double f2 = lut_index(lbdar, (int)c->NDRYLBDAR, c->DRYINTP1R, c->DRYINTP2R, &i2);
    const double zw = lut2d(lut->ker_rdryg, ICE3GB_NDRYLBDAR, i1, f1, i2, f2);
    rg[RG_RRDRYG] = c->FRDRYG * zw / sq(sq(lbdar)) * pow(lbdag, c->CXG) * pow(rho, -c->CEXVT - 1.) *
                    (c->LBRDRYG1 / sq(lbdag) + c->LBRDRYG2 / (lbdag * lbdar) + c->LBRDRYG3 / sq(lbdar));
  }
  const double rdryg_init = rg[RG_RCDRYG] + rg[RG_RIDRYG] + rg[RG_RSDRYG] + rg[RG_RRDRYG];
  /* wet/dry growth selection: :275-338 */
  double rwetg_init = 0.0;
  int ldwetg = 0, lldryg = 0;
  if (x->v[IRG] > c->G_RTMIN && x->ldcompute) {
    if (!x->ldsoft) {
      double f1 = heat_term(c, pr->ka, pr->dv, t, x->v[IRV], x->pres, 1);
      f1 = f1 * (c->O0DEPG * pow(lbdag, c->EX0DEPG) + c->O1DEPG * pr->cj * pow(lbdag, c->EX1DEPG)) /
           (rho * (c->LMTT - c->CL * (c->TT - t)));
      rg[RG_FREEZ1] = f1;
      rg[RG_FREEZ2] = (rho * (c->LMTT + (c->CI - c->CL) * (c->TT - t))) / (rho * (c->LMTT - c->CL * (c->TT - t)));
    }
    const double is = rg[RG_RIWETG] + rg[RG_RSWETG];
    rwetg_init = dmax(is, dmax(0., rg[RG_FREEZ1] + rg[RG_FREEZ2] * is));
    const double wet = dmax(0., rwetg_init - rg[RG_RIWETG] - rg[RG_RSWETG]);
    const double dry = dmax(0., rdryg_init - rg[RG_RIDRYG] - rg[RG_RSDRYG]);
    ldwetg = wet <= dry;
    {
      const int nw = nonzero(rg[RG_RIWETG], rg[RG_RSWETG], 0., 0., 0.);
      const int nd = nonzero(rg[RG_RCDRYG], rg[RG_RIDRYG], rg[RG_RSDRYG], rg[RG_RRDRYG], 0.);
      if (growth_tie(wet, dry, fabs(rwetg_init) + fabs(rdryg_init), nw > nd ? nw : nd)) pr->tie = 1;
    }
    if (c->LNULLWETG != 0.0) ldwetg = ldwetg && rdryg_init > 0.;
    else ldwetg = ldwetg && rwetg_init > 0.;
    if (c->LWETGPOST == 0.0) ldwetg = ldwetg && t < c->TT;
    lldryg = t < c->TT && rdryg_init > 1.e-20 && wet > dry;
  } else {
    rg[RG_FREEZ1] = rg[RG_FREEZ2] = 0.0;
  }
  /* :331-351 part of the wet growth converted into hail (KRR = 7); the
   * graupel sources PRGSI / PRGSI_MR are formed in ICE4_TENDENCIES :510-513 */
  if (x->hail) {
    if (ldwetg) {
      const double rgsi = b[B_RVDEPG] + b[B_RSMLTG] + b[B_RRACCSG] + b[B_RSACCRG] + b[B_RCRIMSG] + b[B_RSRIMCG];
      const double rgsi_mr = b[B_RRHONG_MR] + b[B_RSRIMCG_MR];
      b[B_RWETGH] = (dmax(0., rgsi + b[B_RICFRRG] + b[B_RRCFRIG]) + rwetg_init) * rdryg_init / (rwetg_init + rdryg_init);
      b[B_RWETGH_MR] = dmax(0., rgsi_mr) * rdryg_init / (rwetg_init + rdryg_init);
    } else {
      b[B_RWETGH] = b[B_RWETGH_MR] = 0.0;
    }
  }
  if (ldwetg) {
    b[B_RRWETG] = -(rg[RG_RIWETG] + rg[RG_RSWETG] + rg[RG_RCDRYG] - rwetg_init);
    b[B_RCWETG] = rg[RG_RCDRYG];
    b[B_RIWETG] = rg[RG_RIWETG];
    b[B_RSWETG] = rg[RG_RSWETG];
  } else {
    b[B_RRWETG] = b[B_RCWETG] = b[B_RIWETG] = b[B_RSWETG] = 0.0;
  }
  if (lldryg) {
    b[B_RCDRYG] = rg[RG_RCDRYG];
    b[B_RRDRYG] = rg[RG_RRDRYG];
    b[B_RIDRYG] = rg[RG_RIDRYG];
    b[B_RSDRYG] = rg[RG_RSDRYG];
  } else {
    b[B_RCDRYG] = b[B_RRDRYG] = b[B_RIDRYG] = b[B_RSDRYG] = 0.0;
  }
  /* graupel melting: :390-410 */
  if (x->v[IRG] > c->G_RTMIN && t > c->TT && x->ldcompute) {
    if (!x->ldsoft) {
      double r = heat_term(c, pr->ka, pr->dv, t, x->v[IRV], x->pres, 0);
      r = dmax(0., (-r * (c->O0DEPG * pow(lbdag, c->EX0DEPG) + c->O1DEPG * pr->cj * pow(lbdag, c->EX1DEPG)) -
                    (rg[RG_RCDRYG] + rg[RG_RRDRYG]) * (rho * c->CL * (c->TT - t))) /
                       (rho * c->LMTT));
      b[B_RGMLTR] = r;
    }
  } else b[B_RGMLTR] = 0.0;
  return ldwetg;
}

/* ICE4_FAST_RH, micro/mode_ice4_fast_rh.F90 (LNEWCOEFF = .FALSE.): hail wet
 * and dry growth by collection of cloud, ice, snow, graupel and rain (the
 * snow/graupel/rain kernels tabulated, XKER_SWETH/GWETH/RWETH), the wet/dry
 * choice, the hail -> graupel conversion (LCONVHG) and melting. */
static void ice4_fast_rh(const Tctx *x, PointRates *pr, int ldwetg)
{
  const C *c = x->c;
  const Ice3gbLuts *lut = x->lut;
  const double t = x->t, rho = x->rhodref, lbdar = x->lbdar, lbdas = x->lbdas, lbdag = x->lbdag, lbdah = x->lbdah;
  double *b = pr->bu, *rh = pr->rh_tend;
  const int hh = x->v[IRH] > c->H_RTMIN && x->ldcompute;
  /* :109-131 cloud droplets and pristine ice */
  if (hh && x->v[IRC] > c->C_RTMIN) {
    if (!x->ldsoft) rh[RH_RCWETH] = c->FWETH * x->v[IRC] * (pow(lbdah, c->CXH - c->DH - 2.0) * pow(rho, -c->CEXVT));
  } else rh[RH_RCWETH] = 0.0;
  if (hh && x->v[IRI] > c->I_RTMIN) {
    if (!x->ldsoft) {
      rh[RH_RIWETH] = c->FWETH * x->v[IRI] * (pow(lbdah, c->CXH - c->DH - 2.0) * pow(rho, -c->CEXVT));
      rh[RH_RIDRYH] = rh[RH_RIWETH] * (c->COLIH * exp(c->COLEXIH * (t - c->TT)));
    }
  } else rh[RH_RIWETH] = rh[RH_RIDRYH] = 0.0;
  /* :136-176 snow (XKER_SWETH) */
  int gwet = hh && x->v[IRS] > c->S_RTMIN;
  if (!gwet) rh[RH_RSWETH] = rh[RH_RSDRYH] = 0.0;
  if (!x->ldsoft && gwet) {
    int i1, i2;
    const double f1 = lut_index(lbdah, (int)c->NWETLBDAH, c->WETINTP1H, c->WETINTP2H, &i1);
    const double f2 = lut_index(lbdas, (int)c->NWETLBDAS, c->WETINTP1S, c->WETINTP2S, &i2);
    const double zzw = lut2d(lut->ker_sweth, ICE3GB_NWETLBDAS, i1, f1, i2, f2);
    rh[RH_RSWETH] = c->FSWETH * zzw * (pow(lbdas, c->CXS - c->BS)) * (pow(lbdah, c->CXH)) *
                    (pow(rho, -c->CEXVT - 1.)) *
                    (c->LBSWETH1 / sq(lbdah) + c->LBSWETH2 / (lbdah * lbdas) + c->LBSWETH3 / sq(lbdas));
    rh[RH_RSDRYH] = rh[RH_RSWETH] * (c->COLSH * exp(c->COLEXSH * (t - c->TT)));
  }
  /* :181-213 graupel (XKER_GWETH); dry collection efficiency only where the
   * graupel is not itself in wet growth */
  gwet = hh && x->v[IRG] > c->G_RTMIN;
  if (!gwet) rh[RH_RGWETH] = rh[RH_RGDRYH] = 0.0;
  if (!x->ldsoft && gwet) {
    int i1, i2;
    const double f1 = lut_index(lbdah, (int)c->NWETLBDAH, c->WETINTP1H, c->WETINTP2H, &i1);
    const double f2 = lut_index(lbdag, (int)c->NWETLBDAG, c->WETINTP1G, c->WETINTP2G, &i2);
    const double zzw = lut2d(lut->ker_gweth, ICE3GB_NWETLBDAG, i1, f1, i2, f2);
    rh[RH_RGWETH] = c->FGWETH * zzw * (pow(lbdag, c->CXG - c->BG)) * (pow(lbdah, c->CXH)) *
                    (pow(rho, -c->CEXVT - 1.)) *
                    (c->LBGWETH1 / sq(lbdah) + c->LBGWETH2 / (lbdah * lbdag) + c->LBGWETH3 / sq(lbdag));
    rh[RH_RGDRYH] = rh[RH_RGWETH];
    if (!ldwetg) rh[RH_RGDRYH] = rh[RH_RGDRYH] * (c->COLGH * exp(c->COLEXGH * (t - c->TT)));
  }
  /* :218-245 rain (XKER_RWETH) */
  gwet = hh && x->v[IRR] > c->R_RTMIN;
  if (!gwet) rh[RH_RRWETH] = 0.0;
  if (!x->ldsoft && gwet) {
    int i1, i2;
    const double f1 = lut_index(lbdah, (int)c->NWETLBDAH, c->WETINTP1H, c->WETINTP2H, &i1);
    const double f2 = lut_index(lbdar, (int)c->NWETLBDAR, c->WETINTP1R, c->WETINTP2R, &i2);
    const double zzw = lut2d(lut->ker_rweth, ICE3GB_NWETLBDAR, i1, f1, i2, f2);
    rh[RH_RRWETH] = c->FRWETH * zzw * (pow(lbdar, -4.0)) * (pow(lbdah, c->CXH)) * (pow(rho, -c->CEXVT - 1.)) *
                    (c->LBRWETH1 / sq(lbdah) + c->LBRWETH2 / (lbdah * lbdar) + c->LBRWETH3 / sq(lbdar));
  }
  /* :250-290 freezing rate and growth mode */
  const double rdryh_init = rh[RH_RCWETH] + rh[RH_RIDRYH] + rh[RH_RSDRYH] + rh[RH_RRWETH] + rh[RH_RGDRYH];
  double rweth_init = 0.0;
  int llweth = 0, lldryh = 0;
  if (hh) {
    if (!x->ldsoft) {
      double f1 = heat_term(c, pr->ka, pr->dv, t, x->v[IRV], x->pres, 1);
      f1 = f1 * (c->O0DEPH * pow(lbdah, c->EX0DEPH) + c->O1DEPH * pr->cj * pow(lbdah, c->EX1DEPH)) /
           (rho * (c->LMTT - c->CL * (c->TT - t)));
      rh[RH_FREEZ1] = f1;
      rh[RH_FREEZ2] = (rho * (c->LMTT + (c->CI - c->CL) * (c->TT - t))) / (rho * (c->LMTT - c->CL * (c->TT - t)));
    }
    const double isg = rh[RH_RIWETH] + rh[RH_RSWETH] + rh[RH_RGWETH];
    rweth_init = dmax(isg, dmax(0., rh[RH_FREEZ1] + rh[RH_FREEZ2] * isg));
    const double wet = dmax(0., rweth_init - rh[RH_RIWETH] - rh[RH_RSWETH] - rh[RH_RGWETH]);
    const double dry = dmax(0., rdryh_init - rh[RH_RIDRYH] - rh[RH_RSDRYH] - rh[RH_RGDRYH]);
    llweth = wet <= dry;
    const double wet2 = dmax(0., rweth_init - rh[RH_RIWETH] - rh[RH_RSWETH]);
    const double dry2 = dmax(0., rdryh_init - rh[RH_RIDRYH] - rh[RH_RSDRYH]);
    const int nw = nonzero(rh[RH_RIWETH], rh[RH_RSWETH], rh[RH_RGWETH], 0., 0.);
    const int nd = nonzero(rh[RH_RCWETH], rh[RH_RIDRYH], rh[RH_RSDRYH], rh[RH_RRWETH], rh[RH_RGDRYH]);
    if (growth_tie(wet, dry, fabs(rweth_init) + fabs(rdryh_init), nw > nd ? nw : nd) ||
        growth_tie(wet2, dry2, fabs(rweth_init) + fabs(rdryh_init), nw > nd ? nw : nd))
      pr->tie = 1;
    if (c->LNULLWETH != 0.0) llweth = llweth && rdryh_init > 0.;
    else llweth = llweth && rweth_init > 0.;
    if (c->LWETHPOST == 0.0) llweth = llweth && t < c->TT;
    lldryh = t < c->TT && rdryh_init > 1.e-20 && wet2 > dry2;
  } else {
    rh[RH_FREEZ1] = rh[RH_FREEZ2] = 0.0;
  }
  const double rdryhg = (c->LCONVHG != 0.0 && lldryh) ? rdryh_init * rweth_init / (rdryh_init + rweth_init) : 0.0;
  if (llweth) {
    b[B_RCWETH] = rh[RH_RCWETH];
    b[B_RIWETH] = rh[RH_RIWETH];
    b[B_RSWETH] = rh[RH_RSWETH];
    b[B_RGWETH] = rh[RH_RGWETH];
    b[B_RRWETH] = (rweth_init - rh[RH_RIWETH] - rh[RH_RSWETH] - rh[RH_RGWETH] - rh[RH_RCWETH]);
  } else {
    b[B_RCWETH] = b[B_RIWETH] = b[B_RSWETH] = b[B_RGWETH] = b[B_RRWETH] = 0.0;
  }
  if (lldryh) {
    b[B_RCDRYH] = rh[RH_RCWETH];
    b[B_RIDRYH] = rh[RH_RIDRYH];
    b[B_RSDRYH] = rh[RH_RSDRYH];
    b[B_RRDRYH] = rh[RH_RRWETH];
    b[B_RGDRYH] = rh[RH_RGDRYH];
    b[B_RDRYHG] = rdryhg;
  } else {
    b[B_RCDRYH] = b[B_RIDRYH] = b[B_RSDRYH] = b[B_RRDRYH] = b[B_RGDRYH] = b[B_RDRYHG] = 0.0;
  }
  /* :335-355 melting */
  if (hh && t > c->TT) {
    if (!x->ldsoft) {
      double r = heat_term(c, pr->ka, pr->dv, t, x->v[IRV], x->pres, 0);
      r = dmax(0., (-r * (c->O0DEPH * pow(lbdah, c->EX0DEPH) + c->O1DEPH * pr->cj * pow(lbdah, c->EX1DEPH)) -
                    (rh[RH_RCWETH] + rh[RH_RRWETH]) * (rho * c->CL * (c->TT - t))) /
                       (rho * c->LMTT));
      b[B_RHMLTR] = r;
    }
  } else b[B_RHMLTR] = 0.0;
}

/* ICE4_FAST_RI, micro/mode_ice4_fast_ri.F90. */
static void ice4_fast_ri(const Tctx *x, PointRates *pr, double cit)
{
  const C *c = x->c;
  double *b = pr->bu;
  if (x->tw) { b[B_RCBERI] = 0.0; return; }                        /* mode_ice4_tendencies.F90:568-579 */
  if (pr->ssi > 0. && x->v[IRC] > c->C_RTMIN && x->v[IRI] > c->I_RTMIN && cit > 1.e-20 && x->ldcompute) {
    if (!x->ldsoft) {
      double l = dmin(1.e8, c->LBI * pow(x->rhodref * x->v[IRI] / cit, c->LBEXI));
      b[B_RCBERI] = (pr->ssi / (x->rhodref * pr->ai)) * cit *
                    (c->O0DEPI / l + c->O2DEPI * pr->cj * pr->cj / pow(l, c->DI + 2.0));
    }
  } else b[B_RCBERI] = 0.0;
}

/* ICE4_FAST_RI_RS, micro/mode_ice4_fast_ri_rs.F90 (OCND2, LMODICEDEP =
 * .FALSE.): conversion of large ice crystals to snow (RILARS) and the
 * deposition on ice in the cloudy and clear parts (RVDEPI); zero on soft
 * passes (both are reset on entry and computed only when LDSOFT is false). */
static void ice4_fast_ri_rs(const Tctx *x, PointRates *pr, double cit)
{
  const C *c = x->c;
  double *b = pr->bu;
  const double ztimesc = c->FRMIN14, zdicrit = c->FRMIN15;
  const double rit = x->v[IRI], rho = x->rhodref, t = x->t;
  const double zwcitred = 0.1;
  b[B_RILARS] = 0.;
  b[B_RVDEPI] = 0.;
  if (x->ldsoft) return;
  if (rit > 0.0 && pr->ssi > 0.001)
    b[B_RILARS] = dmin(rit, rit / (87.5 * (zdicrit * zdicrit) * pr->ai / pr->ssi));
  const double zw2d = 1. / (x->ifr * x->icldfr + 1. - x->icldfr);
  if ((x->pres * 0.5 - pr->esi) > 0. && cit > 0. && x->ldcompute) {
    const double xw2d13 = pow(x->ifr, 0.333);
    const double wcitred23 = pow(zwcitred, 0.667);
    const double tc = dmax(-18., dmin(-1., t - c->TT));
    const double hu = dmin(0.15, dmax(0., pr->ssi));
    const double cryssha = 1.1 + 3. * hu * (1. + sin(0.64 * tc - 1.3));
    const double qimax = 366.5 * (zdicrit * zdicrit * zdicrit) * cit * zwcitred / rho;
    double ci2s = 0.;
    if (rit > 1.0e-12 && ztimesc > 0.)
      ci2s = rit * (1. - dmin(1., 0.5 * qimax / rit)) * (1. - x->icldfr) * zw2d / (ztimesc * 0.5);
    const double zzwc = cryssha * 0.878 / pr->ai * pow(cit / rho, 0.667) * pow(dmax(c->I_RTMIN, rit) * zw2d, 0.333);
    if (x->ssio > 0. && x->icldfr > 0.02) b[B_RVDEPI] = b[B_RVDEPI] + zzwc * xw2d13 * x->ssio * x->icldfr;
    if (x->ssiu < 0. && x->icldfr < 0.98) {
      b[B_RILARS] = b[B_RILARS] + ci2s;
      b[B_RVDEPI] = b[B_RVDEPI] + zzwc * wcitred23 * x->ssiu * (1. - x->icldfr);
    }
  }
}

/* The OCND2 parts of the derived fields (mode_ice4_tendencies.F90:303-346,
 * after ice4_derived): tabulated es_i, ssi and ai = AA2 + BB3 p (LLTAB), and
 * the collision factors of cloud water with rain (ACRF) and with snow /
 * graupel (COLF) from the mean droplet radius (LLCOL). */
static void ocnd2_derived(const Tctx *x, PointRates *pr)
{
  const C *c = x->c;
  pr->esi = tiwmx_at(x->tw + TW_ESI * TIWMX_N, x->t);
  pr->ssi = x->v[IRV] * (x->pres - pr->esi) / (c->EPSILO * pr->esi) - 1.0;
  pr->ai = tiwmx_at(x->tw + TW_A2 * TIWMX_N, x->t) + tiwmx_at(x->tw + TW_BB3 * TIWMX_N, x->t) * x->pres;
  const double conc = x->conc * 0.000001;
  pr->colf = 0.00001;
  pr->acrf = 0.00001;
  if (x->v[IRC] > 1.0e-10) {
    const double rcw = 0.1 * pow(0.75 * x->v[IRC] * x->rhodref / (c->PI * conc), 0.333);
    double vt = rcw < 0.0065 ? 1.19e6 * sq(rcw) : 8000. * rcw;
    vt = dmin(10., vt);
    const double st = dmax(0.01, 2. * (100. - vt) * vt / (c->GRAVITY0 * 10.));
    if (st > 0.1) pr->colf = dmax(0.01, dmin(1., 0.939 * pow(st, 2.657)));
    if (x->v[IRR] > 1.0e-10 && rcw > 1.0e-5) {
      const double r20 = exp(rcw * 2000.);
      pr->acrf = (r20 - 1.) / (r20 + 1.);
    }
  }
}

/* Slope parameters, mode_ice4_tendencies.F90:389-433 (LSNOW_T optional). */
static void ice4_slopes(Tctx *x)
{
  const C *c = x->c;
  const double rho = x->rhodref;
  x->lbdar = (x->v[IRR] > 0.) ? c->LBR * pow(rho * dmax(x->v[IRR], c->R_RTMIN), c->LBEXR) : 0.0;
  const int llrfr = (int)c->SUBG_RC_RR_ACCR == 1 || (int)c->SUBG_RR_EVAP == 2;
  if (llrfr)
    x->lbdar_rf = (x->v[IRR] > 0. && x->rainfr > 0.)
                      ? c->LBR * pow(rho * dmax(x->v[IRR] / x->rainfr, c->R_RTMIN), c->LBEXR) : 0.0;
  else
    x->lbdar_rf = x->lbdar;
  if (c->LSNOW_T != 0.0) {
    if (x->v[IRS] > 0. && x->t > 263.15)
      x->lbdas = dmax(dmin(c->LBDAS_MAX, pow(10.0, 14.554 - 0.0423 * x->t)), c->LBDAS_MIN) * c->TRANS_MP_GAMMAS;
    else if (x->v[IRS] > 0. && x->t <= 263.15)
      x->lbdas = dmax(dmin(c->LBDAS_MAX, pow(10.0, 6.226 - 0.0106 * x->t)), c->LBDAS_MIN) * c->TRANS_MP_GAMMAS;
    else x->lbdas = 0.0;
  } else {
    x->lbdas = (x->v[IRS] > 0.) ? dmin(c->LBDAS_MAX, c->LBS * pow(rho * dmax(x->v[IRS], c->S_RTMIN), c->LBEXS)) : 0.0;
  }
  x->lbdag = (x->v[IRG] > 0.) ? c->LBG * pow(rho * dmax(x->v[IRG], c->G_RTMIN), c->LBEXG) : 0.0;
  if (x->hail)                                                        /* :426-432 */
    x->lbdah = (x->v[IRH] > 0.) ? c->LBH * pow(rho * dmax(x->v[IRH], c->H_RTMIN), c->LBEXH) : 0.0;
}

/* ICE4_TENDENCIES (mode_ice4_tendencies.F90:150-717) for one point.
 * `vart` is the state at the start of the pass (PVART), `t` = th*exn.
 * Outputs A (rates) and B (instantaneous increments). */
/* The aggregation of ICE4_TENDENCIES (mode_ice4_tendencies.F90:606-717):
 * the rates b[] of one pass into the tendencies A[] (per second) and the
 * instantaneous changes B[], with the OCND2 rows (RVDEPI, RILARS, the
 * graupel deposition split depg_s / nodepg_s) and the KRR = 7 rows.  The
 * NRR = 6 rows are those of ice4_total_tendencies_update
 * (src/ice3/jax/stencils/ice4_tendencies.py:330-441). */
static void ice4_aggregate(const double *b, double lsfact, double lvfact, int ocnd2, double depg_s,
                           double nodepg_s, int hail, double A[NVH], double B[NVH])
{
  const double lsv = lsfact - lvfact;
  A[ITH] += b[B_RVDEPG] * lsfact;
  A[ITH] += b[B_RCHONI] * lsv;
  A[ITH] += b[B_RVDEPS] * lsfact;
  A[ITH] -= b[B_RREVAV] * lvfact;
  A[ITH] += b[B_RCRIMSS] * lsv;
  A[ITH] += b[B_RCRIMSG] * lsv;
  A[ITH] += b[B_RRACCSS] * lsv;
  A[ITH] += b[B_RRACCSG] * lsv;
  A[ITH] += (b[B_RRCFRIG] - b[B_RICFRR]) * lsv;
  A[ITH] += (b[B_RCWETG] + b[B_RRWETG]) * lsv;
  A[ITH] += (b[B_RCDRYG] + b[B_RRDRYG]) * lsv;
  A[ITH] -= b[B_RGMLTR] * lsv;
  A[ITH] += b[B_RCBERI] * lsv;
  A[IRV] -= b[B_RVDEPG];
  A[IRV] -= b[B_RVDEPS];
  A[IRV] += b[B_RREVAV];
  A[IRC] -= b[B_RCHONI];
  A[IRC] -= b[B_RCAUTR];
  A[IRC] -= b[B_RCACCR];
  A[IRC] -= b[B_RCRIMSS];
  A[IRC] -= b[B_RCRIMSG];
  A[IRC] -= b[B_RCMLTSR];
  A[IRC] -= b[B_RCWETG];
  A[IRC] -= b[B_RCDRYG];
  A[IRC] -= b[B_RCBERI];
  A[IRR] += b[B_RCAUTR];
  A[IRR] += b[B_RCACCR];
  A[IRR] -= b[B_RREVAV];
  A[IRR] -= b[B_RRACCSS];
  A[IRR] -= b[B_RRACCSG];
  A[IRR] += b[B_RCMLTSR];
  A[IRR] = A[IRR] - b[B_RRCFRIG] + b[B_RICFRR];
  A[IRR] -= b[B_RRWETG];
  A[IRR] -= b[B_RRDRYG];
  A[IRR] += b[B_RGMLTR];
  A[IRI] += b[B_RCHONI];
  A[IRI] -= b[B_RIAGGS];
  A[IRI] -= b[B_RIAUTS];
  A[IRI] = A[IRI] - b[B_RICFRRG] - b[B_RICFRR];
  A[IRI] -= b[B_RIWETG];
  A[IRI] -= b[B_RIDRYG];
  A[IRI] += b[B_RCBERI];
  A[IRS] += b[B_RVDEPS];
  A[IRS] += b[B_RIAGGS];
  A[IRS] += b[B_RIAUTS];
  A[IRS] += b[B_RCRIMSS];
  A[IRS] -= b[B_RSRIMCG];
  A[IRS] += b[B_RRACCSS];
  A[IRS] -= b[B_RSACCRG];
  A[IRS] -= b[B_RSMLTG];
  A[IRS] -= b[B_RSWETG];
  A[IRS] -= b[B_RSDRYG];
  A[IRG] += ocnd2 ? b[B_RVDEPG] * nodepg_s : b[B_RVDEPG];         /* :693 */
  A[IRG] += b[B_RCRIMSG] + b[B_RSRIMCG];
  A[IRG] += b[B_RRACCSG] + b[B_RSACCRG];
  A[IRG] += b[B_RSMLTG];
  A[IRG] += b[B_RICFRRG] + b[B_RRCFRIG];
  A[IRG] += b[B_RCWETG] + b[B_RIWETG] + b[B_RSWETG] + b[B_RRWETG];
  A[IRG] += b[B_RCDRYG] + b[B_RIDRYG] + b[B_RSDRYG] + b[B_RRDRYG];
  A[IRG] -= b[B_RGMLTR];
  if (ocnd2) {                                                        /* OCND2 rows */
    A[ITH] += b[B_RVDEPI] * lsfact;                                   /* :625 */
    A[IRV] -= b[B_RVDEPI];                                            /* :630 */
    A[IRI] += b[B_RVDEPI];                                            /* :673-674 */
    A[IRI] -= b[B_RILARS];
    A[IRS] += b[B_RVDEPG] * depg_s;                                   /* :677 */
    A[IRS] += b[B_RILARS];                                            /* :691 */
  }
  if (hail) {                                                         /* KRR = 7 rows */
    A[ITH] += (b[B_RRWETH] + b[B_RCWETH]) * lsv;                      /* :620-622 */
    A[ITH] += (b[B_RCDRYH] + b[B_RRDRYH]) * lsv;
    A[ITH] -= b[B_RHMLTR] * lsv;
    A[IRC] -= b[B_RCWETH];                                            /* :641-642 */
    A[IRC] -= b[B_RCDRYH];
    A[IRR] -= b[B_RRWETH];                                            /* :657-659 */
    A[IRR] -= b[B_RRDRYH];
    A[IRR] += b[B_RHMLTR];
    A[IRI] -= b[B_RIWETH];                                            /* :669-670 */
    A[IRI] -= b[B_RIDRYH];
    A[IRS] -= b[B_RSWETH];                                            /* :688-689 */
    A[IRS] -= b[B_RSDRYH];
    A[IRG] -= b[B_RWETGH];                                            /* :699-700 */
    B[IRG] -= b[B_RWETGH_MR];
    A[IRG] -= b[B_RGWETH];                                            /* :704-705 */
    A[IRG] = A[IRG] - b[B_RGDRYH] + b[B_RDRYHG];
    A[IRH] += b[B_RWETGH];                                            /* :709-715 */
    B[IRH] += b[B_RWETGH_MR];
    A[IRH] = A[IRH] + b[B_RCWETH] + b[B_RIWETH] + b[B_RSWETH] + b[B_RGWETH] + b[B_RRWETH];
    A[IRH] = A[IRH] + b[B_RCDRYH] + b[B_RIDRYH] + b[B_RSDRYH] + b[B_RRDRYH] + b[B_RGDRYH] - b[B_RDRYHG];
    A[IRH] -= b[B_RHMLTR];
  }
}

static void ice4_tendencies(const C *c, const Ice3gbLuts *lut, int ldsoft, int ldcompute,
                            double exn, double rhodref, double lvfact, double lsfact, double pres,
                            double cf, double sigma_rc, double *cit, double t, const double vart[NVH],
                            PointRates *pr, double *rainfr, double hl[4], double hi[4],
                            double A[NVH], double B[NVH], const Ocnd2Pt *oc)
{
  Tctx x;
  x.c = c; x.lut = lut; x.ldsoft = ldsoft; x.ldcompute = ldcompute;
  x.rhodref = rhodref; x.pres = pres; x.exn = exn; x.lvfact = lvfact; x.lsfact = lsfact;
  x.cf = cf; x.sigma_rc = sigma_rc; x.t = t; x.rainfr = *rainfr;
  x.hail = (int)c->NRR == 7;
  x.lbdah = 0.0;
  x.tw = oc ? oc->tw : NULL;
  if (oc) {
    x.ssio = oc->ssio; x.ssiu = oc->ssiu; x.ifr = oc->ifr; x.icldfr = oc->icldfr; x.zzz = oc->zzz;
    x.conc = oc->conc;
  }
  for (int v = 0; v < NVH; ++v) { x.v[v] = (v < NV || x.hail) ? vart[v] : 0.0; A[v] = 0.0; B[v] = 0.0; }
  for (int k = 0; k < 4; ++k) { x.hl[k] = hl[k]; x.hi[k] = hi[k]; }
  double *b = pr->bu;
  if (ldsoft) {
    b[B_RVHENI_MR] = b[B_RRHONG_MR] = b[B_RIMLTC_MR] = b[B_RSRIMCG_MR] = 0.0;
  } else {
    /* :171-183 nucleation */
    ice4_nucleation(c, ldcompute, x.v[ITH], pres, rhodref, exn, lsfact, x.t, x.v[IRV], cit, &b[B_RVHENI_MR], NULL,
                    oc ? oc->tw : NULL, oc ? oc->zzz : 0.0, oc ? oc->icldfr : 0.0);
    x.v[ITH] += b[B_RVHENI_MR] * lsfact;
    x.t = x.v[ITH] * exn;
    x.v[IRV] -= b[B_RVHENI_MR];
    x.v[IRI] += b[B_RVHENI_MR];
    /* :188-201 rrhong */
    b[B_RRHONG_MR] = ice4_rrhong(c, ldcompute, exn, lvfact, lsfact, x.t, x.v[IRR], x.v[ITH]);
    x.v[ITH] += b[B_RRHONG_MR] * (lsfact - lvfact);
    x.t = x.v[ITH] * exn;
    x.v[IRR] -= b[B_RRHONG_MR];
    x.v[IRG] += b[B_RRHONG_MR];
    /* :206-219 rimltc */
    b[B_RIMLTC_MR] = ice4_rimltc(c, ldcompute, exn, lvfact, lsfact, x.t, x.v[ITH], x.v[IRI]);
    x.v[ITH] -= b[B_RIMLTC_MR] * (lsfact - lvfact);
    x.t = x.v[ITH] * exn;
    x.v[IRC] += b[B_RIMLTC_MR];
    x.v[IRI] -= b[B_RIMLTC_MR];
    b[B_RSRIMCG_MR] = 0.0;
    /* :270-295 */
    B[ITH] += b[B_RVHENI_MR] * lsfact;
    B[ITH] += b[B_RRHONG_MR] * (lsfact - lvfact);
    B[ITH] -= b[B_RIMLTC_MR] * (lsfact - lvfact);
    B[IRV] -= b[B_RVHENI_MR];
    B[IRC] += b[B_RIMLTC_MR];
    B[IRR] -= b[B_RRHONG_MR];
    B[IRI] += b[B_RVHENI_MR];
    B[IRI] -= b[B_RIMLTC_MR];
    B[IRS] -= b[B_RSRIMCG_MR];
    B[IRG] += b[B_RRHONG_MR];
    B[IRG] += b[B_RSRIMCG_MR];
    /* :303-320 derived fields */
    ice4_derived(c, x.t, rhodref, pres, x.v[IRV], &pr->ssi, &pr->ka, &pr->dv, &pr->ai, &pr->cj);
    if (oc) ocnd2_derived(&x, pr);
  }
  /* :352 compute_pdf */
  x.rainfr = *rainfr;
  double zrainfr = ice4_compute_pdf(c, ldcompute, rhodref, x.v[IRC], x.v[IRI], cf, x.t, sigma_rc, x.hl, x.hi);
  const int llrfr = (int)c->SUBG_RC_RR_ACCR == 1 || (int)c->SUBG_RR_EVAP == 2;
  if (llrfr) {                                                        /* :357-380 */
    x.rainfr = dmax(x.rainfr, zrainfr);
    int mask = x.v[IRR] > c->R_RTMIN || x.v[IRS] > c->S_RTMIN || x.v[IRG] > c->G_RTMIN;
    if (x.hail) mask = mask || x.v[IRH] > c->H_RTMIN;
    if (mask && x.rainfr == 0.) x.rainfr = 1.;
  } else {
    x.rainfr = 1.;
  }
  ice4_slopes(&x);
  ice4_slow(&x, pr);
  ice4_warm(&x, pr);
  ice4_fast_rs(&x, pr);
  const int ldwetg = ice4_fast_rg(&x, pr, *cit);
  if (x.hail) ice4_fast_rh(&x, pr, ldwetg);                          /* :535-545 */
  ice4_fast_ri(&x, pr, *cit);
  /* :445-458 part of the graupel deposition given to snow; :585-596 RVDEPI, RILARS */
  double depg_s = 0.0, nodepg_s = 1.0;
  if (x.tw) {
    if (c->FRMIN5 > 1.0e-12 && c->FRMIN6 > 0.01) {
      depg_s = dmax(0., dmin(1., (c->FRMIN5 - x.v[IRG] / c->FRMIN5))) * dmax(0., dmin(1., (pr->ssi / c->FRMIN6)));
      nodepg_s = 1. - depg_s;
    }
    ice4_fast_ri_rs(&x, pr, *cit);
  }
  /* :606-717 aggregation */
  ice4_aggregate(b, lsfact, lvfact, x.tw != NULL, depg_s, nodepg_s, x.hail, A, B);
  *rainfr = x.rainfr;
  for (int k = 0; k < 4; ++k) { hl[k] = x.hl[k]; hi[k] = x.hi[k]; }
}

/* The sub-step limits of ICE4_STEPPING.  limit_feedback: with LFEEDBACKT,
 * no sub-step across theta = TT/exn (zx), mode_ice4_stepping.F90:284-299,
 * the temperature part of ice4_step_limiter (src/ice3/jax/stencils/
 * ice4_stepping.py:109-194).  limit_depletion: a species that is present
 * (r > rsmin) and depleting (A < -1e-20) ends the sub-step where it reaches
 * zero, at least MNH_TINY seconds on (:302-311). */
static inline double limit_feedback(double zx, double th, double a, double b, double maxtime)
{
  if ((th - zx) * (th + b - zx) < 0.) maxtime = 0.;
  if (fabs(a) > 1.e-20) {
    const double thr = (zx - b - th) / a;
    if (thr > 0.) maxtime = dmin(maxtime, thr);
  }
  return maxtime;
}

static inline double limit_depletion(double a, double b, double r, double rsmin, double tiny, double maxtime)
{
  if (a < -1.e-20 && r > rsmin) {
    maxtime = dmin(maxtime, -(b + r) / a);
    maxtime = dmax(maxtime, tiny);
  }
  return maxtime;
}

/* The state after a sub-step: x + A dt + B, in that order
 * (mode_ice4_stepping.F90:388-395; state_update of
 * src/ice3/jax/stencils/ice4_stepping.py:232-291). */
static inline void state_update(int nv, double *vart, const double *A, const double *B, double maxtime)
{
  for (int v = 0; v < nv; ++v) vart[v] = vart[v] + A[v] * maxtime + B[v];
}

/* ICE4_STEPPING (mode_ice4_stepping.F90:139-518) restated for one packed
 * point (every packed point is a micro point).  Points of one Fortran call
 * march in lock-step through the same passes; a point only contributes in
 * its own active passes, so its trajectory is the per-point loop below.  The
 * only cross-point coupling kept is PRREVAV = ZBU_INST(:,IRREVAV) after the
 * last pass of the whole call (:514-516), reproduced through `last_key`.
 * Idle passes move a finished point by at most MNH_TINY seconds of its
 * external tendency; that sub-1e-15 relative drift is not reproduced. */
typedef struct {
  double vart[NVH];
  double extpk[NVH];
  double cit, rainfr, rrevav;
  int outer, inner, capped;
  int tie;    /* bit 0: some pass took a growth-mode decision on rounding
               residuals; bit 1: the CIT reset followed an ice residual;
               bit 2: an MRSTEP threshold fell on the chosen sub-step;
               bit 3: a hard pass followed a bit-1 reset;
               bit 4: a depleted species ended a pass at a rounding residual
               whose comparison with XRTMIN decides a MNH_TINY pass */
} StepOut;

/* Depletion ties (StepOut.tie bit 4): a species whose depletion limit was
 * evaluated in a pass (present, A < -1e-20) ends the pass at r + A t + B = 0
 * in exact arithmetic when that limit bound the sub-step; the computed value
 * is a rounding residual, and whether it is above XRTMIN decides whether the
 * next pass is one more MNH_TINY step (mode_ice4_stepping.F90:302-311).  At
 * the 1000/s cap of RCHONI that step moves 2.2e-13 kg/kg, so an evaluation
 * whose rates differ in the last bits (FMA contraction) can land on the other
 * side.  g_depl_flip is a bit mask: with bit k-1 set the oracle takes the
 * other outcome at the k-th such decision of every point (a residual above
 * XRTMIN becomes 0, one at or below it becomes 2 XRTMIN), so that the
 * branches can be enumerated. */
static int g_depl_flip = 0;

EXPORT void ice3o_set_depletion_flip(int k) { g_depl_flip = k; }

static void ice4_stepping_point(const C *c, const Ice3gbLuts *lut, double dt, int max_passes,
                                double exn, double rhodref, double pres, double cf, double sigma_rc,
                                double hlc_hcf, double hlc_hrc, double hli_hcf, double hli_hri,
                                StepOut *s, const Ocnd2Pt *oc)
{
  const double rsmin[NVH] = {0.0, c->V_RTMIN, c->C_RTMIN, c->R_RTMIN, c->I_RTMIN, c->S_RTMIN, c->G_RTMIN,
                             c->H_RTMIN};
  const int hail = (int)c->NRR == 7;
  const int nv = hail ? NVH : NV;                                     /* 0:KRR */
  const double inv_dt = 1.0 / dt;
  PointRates pr;
  memset(&pr, 0, sizeof(pr));
  double hl[4] = {hlc_hcf, 0.0, hlc_hrc, 0.0}, hi[4] = {hli_hcf, 0.0, hli_hri, 0.0};
  if (!hail) s->vart[IRH] = s->extpk[IRH] = 0.0;
  /* :151-158 external tendencies */
  for (int v = 0; v < nv; ++v) s->extpk[v] = s->extpk[v] - s->vart[v] * inv_dt;
  if ((int)c->SUBG_AUCV_RC == 2 || (int)c->SUBG_AUCV_RI == 2) {     /* :170-189 */
    hl[3] = s->vart[IRC] - hlc_hrc;
    hi[3] = s->vart[IRI] - hli_hri;
    hl[1] = (s->vart[IRC] > 0.) ? cf - hlc_hcf : 0.;
    hi[1] = (s->vart[IRI] > 0.) ? cf - hli_hcf : 0.;
  }
  double ztime = 0.0;
  int passes = 0;
  s->outer = 0; s->inner = 0; s->capped = 0; s->rrevav = 0.0; s->tie = 0;
  /* :191-197 time splitting: the maximum number of outer iterations with
   * their own limits, and the sub-step length of TSTEP_TS */
  int nb_iter_max = (int)c->NMAXITER_MICRO;
  double ztstep = 0.0;
  if (c->TSTEP_TS != 0.0) {
    int nb = (int)(dt / c->TSTEP_TS);
    nb = nb > 1 ? nb : 1;
    ztstep = dt / nb;
    nb_iter_max = nb_iter_max > nb ? nb_iter_max : nb;
  }
  double z0rt[NVH], tlast = 0.0;
  int depl_events = 0;
  while (ztime < dt) {                                                /* :204 */
    s->outer++;                                                       /* IITER, :258-266 */
    /* a hard pass after a rounding-decided CIT reset (MRSTEP / TSTEP_TS
     * outer iterations): the reset now reaches every rate of the point */
    if (s->tie & 2) s->tie |= 8;
    int llcompute = 1, lsoft = 0, inner = 0;
    tlast = ztime;                                                    /* ZTIME_LASTCALL */
    for (int v = 0; v < nv; ++v) z0rt[v] = s->vart[v];               /* Z0RT, :409-411 */
    while (llcompute) {                                               /* :227 */
      if (passes >= max_passes) { s->capped = 1; goto done; }
      passes++;
      inner++;
      double zsum2 = s->vart[IRI] + s->vart[IRS] + s->vart[IRG];       /* :276-281 */
      if (hail) zsum2 += s->vart[IRH];
      const double zdev = (c->CPD + c->CPV * s->vart[IRV] + c->CL * (s->vart[IRC] + s->vart[IRR]) + c->CI * zsum2) * exn;
      const double zzt = s->vart[ITH] * exn;
      const double lsfact = (c->LSTT + (c->CPV - c->CI) * (zzt - c->TT)) / zdev;
      const double lvfact = (c->LVTT + (c->CPV - c->CL) * (zzt - c->TT)) / zdev;
      double A[NVH], B[NVH];
      ice4_tendencies(c, lut, lsoft, 1, exn, rhodref, lvfact, lsfact, pres, cf, sigma_rc, &s->cit, zzt,
                      s->vart, &pr, &s->rainfr, hl, hi, A, B, oc);
      s->tie |= pr.tie;
      pr.tie = 0;
      for (int v = 0; v < nv; ++v) A[v] += s->extpk[v];             /* :265-272 */
      double maxtime = dt - ztime;                                    /* :275-282 */
      if (c->LFEEDBACKT != 0.0)                                       /* :284-299 */
        maxtime = limit_feedback(c->TT / exn, s->vart[ITH], A[ITH], B[ITH], maxtime);
      for (int v = 1; v < nv; ++v)                                    /* :302-311 */
        maxtime = limit_depletion(A[v], B[v], s->vart[v], rsmin[v], c->MNH_TINY, maxtime);
      if (ztime + maxtime >= dt) llcompute = 0;                       /* :314-319 */
      if (c->TSTEP_TS != 0.0 && s->outer < nb_iter_max && ztime + maxtime > tlast + ztstep) {  /* :387-397 */
        maxtime = tlast - ztime + ztstep;
        llcompute = 0;
      }
      if (c->MRSTEP != 0.0 && s->outer < nb_iter_max) {              /* :402-453 */
        double maxb = 0.0;
        for (int v = 1; v < nv; ++v) {
          const double thr = fabs(A[v]) > 1.e-20
                                 ? (copysign(1., A[v]) * c->MRSTEP + z0rt[v] - s->vart[v] - B[v]) / A[v] : -1.;
          /* the threshold on a sub-step that does not end the outer
           * iteration yet, up to rounding: a species that grew from zero to
           * MRSTEP in the last outer iteration and now depletes reaches
           * -MRSTEP + Z0RT = 0 together with its depletion time; whether
           * the pass ends the outer iteration (a hard recompute) or
           * continues soft is decided by the last bits of both (a tie,
           * reported with bit 2) */
          if (llcompute && thr >= 0. && fabs(thr - maxtime) <= 1e-12 * maxtime &&
              (s->vart[v] > rsmin[v] || A[v] > 0.))
            s->tie |= 4;
          if (thr >= 0. && thr < maxtime && (s->vart[v] > rsmin[v] || A[v] > 0.)) {
            maxtime = dmin(maxtime, thr);
            llcompute = 0;
          }
          maxb = v == 1 ? fabs(B[v]) : dmax(maxb, fabs(B[v]));
        }
        if (maxb > c->MRSTEP) {
          maxtime = 0.;
          llcompute = 0;
        }
      }
      const double ri0 = s->vart[IRI];
      double rstart[NVH];
      for (int v = 0; v < nv; ++v) rstart[v] = s->vart[v];
      state_update(nv, s->vart, A, B, maxtime);                       /* :388-395 */
      for (int v = 1; v < nv; ++v) {                                  /* depletion ties (bit 4) */
        if (!(A[v] < -1.e-20 && rstart[v] > rsmin[v])) continue;
        const double noise = 4.0 * 2.220446049250313e-16 * (fabs(rstart[v]) + fabs(B[v]) + fabs(A[v] * maxtime));
        if (noise > rsmin[v] && fabs(s->vart[v]) <= noise) {
          s->tie |= 16;
          if (depl_events < 31 && ((g_depl_flip >> depl_events) & 1))
            s->vart[v] = s->vart[v] > rsmin[v] ? 0.0 : 2.0 * rsmin[v];
          ++depl_events;
        }
      }
      /* the ice depleted to a rounding residual: whether CIT is reset below
       * follows the last bits of the pass (a tie, as the growth choice) */
      if (s->cit > 0. && (ri0 != 0. || B[IRI] != 0.) &&
          fabs(s->vart[IRI]) <= 1e-12 * (fabs(ri0) + fabs(B[IRI]) + fabs(A[IRI] * maxtime)))
        s->tie |= 2;
      if (s->vart[IRI] <= 0.) s->cit = 0.;                            /* :398-401 */
      ztime += maxtime;
      s->rrevav = pr.bu[B_RREVAV];
      lsoft = 1;
    }
    s->inner = inner;
  }
done:
  for (int v = 0; v < nv; ++v) s->vart[v] = s->vart[v] - s->extpk[v] * dt;  /* :503-511 */
}

/* ===================================================================== */
/* RAIN_ICE (micro/rain_ice.F90)                                          */
/* ===================================================================== */

EXPORT void ice3o_rainfr_vert(const C *c, int nij, int nk, double *prfr, const double *rr, const double *rs,
                              const double *rg);
static void rainfr_vert_h(const C *c, int nij, int nk, double *prfr, const double *rr, const double *rs,
                          const double *rg, const double *rh);

/* ICE4_SEDIMENTATION of a rain_ice call (mode_ice4_sedimentation.F90:166-229):
 * STAT on the sources x dt, or SPLI on the mixing ratios at t followed by
 * the negativity correction.  Returns 0 if an SPLI column hit its sub-step cap. */
static int rain_ice_sediment(const C *c, int nij, int nk, double dt, int sed_fortran, int has_st,
                             const Ice3gbRainIceFields *f)
{
  int ok = 1;
  const int spli = (int)c->SEDIM == 0;
#pragma omp parallel for schedule(static) reduction(& : ok)
  for (long col = 0; col < nij; ++col) {
    const int hail = (int)c->NRR == 7;
    double *src[6] = {f->rcs, f->rrs, f->ris, f->rss, f->rgs, f->rhs};
    double *fpr[6] = {f->fpr_c, f->fpr_r, f->fpr_i, f->fpr_s, f->fpr_g, f->fpr_h};
    double inpr[6];
    const double sea = f->sea ? f->sea[col] : 0.0, town = f->town ? f->town[col] : 0.0;
    if (spli) {
      const double *rt[6] = {f->rct, f->rrt, f->rit, f->rst, f->rgt, f->rht};
      ok &= sed_split_column(c, nij, nk, dt, col, f->rhodref, f->dzz, f->pabs, f->tht, f->exn, sea, town, has_st,
                             rt, f->rvt, src, f->rvs, f->ths, fpr, inpr, 10000, hail ? 6 : 5);
    } else {
      sed_column(c, nij, nk, dt, col, sed_fortran, f->rhodref, f->dzz, f->pabs, f->tht, sea, town, has_st, src,
                 fpr, inpr);
      if (hail) sed_hail_column(c, nij, nk, dt, col, f->rhodref, f->dzz, f->rhs, f->fpr_h, &inpr[5]);
    }
    f->inprc[col] = inpr[0]; f->inprr[col] = inpr[1]; f->inpri[col] = inpr[2];
    f->inprs[col] = inpr[3]; f->inprg[col] = inpr[4];
    if (hail) f->inprh[col] = inpr[5];
  }
  return ok;
}

/* lsfact / lvfact of RAIN_ICE at time t, without the Exner function
 * (rain_ice.F90:334-345; rain_ice_thermo, src/ice3/jax/stencils/rain_ice.py:95). */
static inline void rain_ice_thermo(const C *c, int hail, double t, double rv, double rc, double rr, double ri,
                                   double rs, double rg, double rh, double *lsf, double *lvf)
{
  const double zrice = hail ? ri + rs + rg + rh : ri + rs + rg;
  const double zdev = c->CPD + c->CPV * rv + c->CL * (rc + rr) + c->CI * zrice;
  *lsf = (c->LSTT + (c->CPV - c->CI) * (t - c->TT)) / zdev;
  *lvf = (c->LVTT + (c->CPV - c->CL) * (t - c->TT)) / zdev;
}

/* LLMICRO without OCND2 (rain_ice.F90:370-381; rain_ice_mask,
 * src/ice3/jax/stencils/rain_ice.py:141). */
static inline int rain_ice_micro(const C *c, int hail, double rc, double rr, double ri, double rs, double rg,
                                 double rh)
{
  return rc > c->C_RTMIN || rr > c->R_RTMIN || ri > c->I_RTMIN || rs > c->S_RTMIN || rg > c->G_RTMIN ||
         (hail && rh > c->H_RTMIN);
}

/* Total tendencies of a micro point (rain_ice.F90:758-790, disabled in the
 * vendored copy; rain_ice_total_tendencies, src/ice3/jax/stencils/
 * rain_ice.py:19-92): (r_end - r_t)/dt per species, theta from L/cph (lvx,
 * lsx: already divided by the reference Exner function), plus the RVHENI
 * taken outside the sub-stepping.  r0: theta and the mixing ratios at t;
 * src: the sources (src[IRH] NULL without hail). */
static void total_tendencies(int hail, double inv, double lvx, double lsx, const double vart[NVH],
                             const double r0[NVH], double zrvheni, double *src[NVH])
{
  const double wv = (vart[IRV] - r0[IRV]) * inv, wc = (vart[IRC] - r0[IRC]) * inv;
  const double wr = (vart[IRR] - r0[IRR]) * inv, wi = (vart[IRI] - r0[IRI]) * inv;
  const double ws = (vart[IRS] - r0[IRS]) * inv, wg = (vart[IRG] - r0[IRG]) * inv;
  const double wh = (vart[IRH] - r0[IRH]) * inv;
  const double wth = (wc + wr) * lvx + (hail ? wi + ws + wg + wh : wi + ws + wg) * lsx;
  *src[ITH] += wth + zrvheni * lsx;
  *src[IRV] += wv - zrvheni;
  *src[IRC] += wc;
  *src[IRR] += wr;
  *src[IRI] += wi + zrvheni;
  *src[IRS] += ws;
  *src[IRG] += wg;
  if (hail) *src[IRH] += wh;
}

/* ICE4_CORRECT_NEGATIVITIES on the sources (mode_ice4_correct_negativities.F90:
 * 9-178): negative hydrometeors go back to vapour with theta compensated
 * (:96-120), then vapour below XRTMIN(1) is refilled from cloud and ice in
 * proportion (:123-136), from rain, snow, graupel and hail (:140-171).
 * x[] = theta, rv, rc, rr, ri, rs, rg, rh sources.  The reference's JAX
 * stencil (src/ice3/jax/stencils/ice4_correct_negativities.py:14) has the
 * first part and only the snow and graupel lines of the second, with the
 * snow / graupel minima as the vapour threshold: `fortran` = 0 runs that
 * form (s_min, g_min its thresholds), 1 the Fortran (s_min = g_min =
 * XRTMIN(1)). */
static void correct_negativities(double s_min, double g_min, int hail, int fortran, double lvx, double lsx,
                                 double x[NVH])
{
  double th = x[ITH], rv = x[IRV], rc = x[IRC], rr = x[IRR], ri = x[IRI], rs = x[IRS], rg = x[IRG];
  double rh = hail ? x[IRH] : 0.0, w;
  w = rc - dmax(rc, 0.); rv += w; th -= w * lvx; rc -= w;
  w = rr - dmax(rr, 0.); rv += w; th -= w * lvx; rr -= w;
  w = ri - dmax(ri, 0.); rv += w; th -= w * lsx; ri -= w;
  w = rs - dmax(rs, 0.); rv += w; th -= w * lsx; rs -= w;
  w = rg - dmax(rg, 0.); rv += w; th -= w * lsx; rg -= w;
  if (hail) { w = rh - dmax(rh, 0.); rv += w; th -= w * lsx; rh -= w; }   /* :115-120 */
  if (fortran) {
    w = dmin(1., dmax(s_min - rv, 0.) / dmax(rc + ri, 1.e-20));
    th -= w * (rc * lvx + ri * lsx);
    rv += w * (rc + ri);
    rc = (1. - w) * rc;
    ri = (1. - w) * ri;
    w = dmin(dmax(rr, 0.), dmax(s_min - rv, 0.)); rv += w; rr -= w; th -= w * lvx;
  }
  w = dmin(dmax(rs, 0.), dmax(s_min - rv, 0.)); rv += w; rs -= w; th -= w * lsx;
  w = dmin(dmax(rg, 0.), dmax(g_min - rv, 0.)); rv += w; rg -= w; th -= w * lsx;
  if (hail) { w = dmin(dmax(rh, 0.), dmax(g_min - rv, 0.)); rv += w; rh -= w; th -= w * lsx; }  /* :165-171 */
  x[ITH] = th; x[IRV] = rv; x[IRC] = rc; x[IRR] = rr; x[IRI] = ri; x[IRS] = rs; x[IRG] = rg;
  if (hail) x[IRH] = rh;
}

/* Fog deposition at the lowest level (rain_ice.F90:876-895; fog_deposition,
 * src/ice3/jax/stencils/rain_ice.py:323): returns the deposit INDEP. */
static inline double fog_deposition(const C *c, double rct, double rhodref, double dzz, double *rcs, double *inprc)
{
  const double indep = c->VDEPOSC * rct * rhodref / c->RHOLW;
  *rcs -= c->VDEPOSC * rct / dzz;
  *inprc += indep;
  return indep;
}

static int rain_ice_supported(const C *c)
{
  if ((int)c->NRR != 6 && (int)c->NRR != 7) return 0;
  if ((int)c->SEDIM != 0 && (int)c->SEDIM != 1) return 0;                    /* SPLI, STAT */
  if ((int)c->SUBG_RC_RR_ACCR != 0 && (int)c->SUBG_RC_RR_ACCR != 1) return 0;  /* NONE, PRFR */
  if ((int)c->SUBG_RR_EVAP < 0 || (int)c->SUBG_RR_EVAP > 2) return 0;          /* NONE, CLFR, PRFR */
  return 1;
}

EXPORT int ice3o_rain_ice_ties(const C *c, const Ice3gbLuts *lut, int nij, int nk, double dt,
                               const Ice3gbRainIceOptions *opt, const Ice3gbRainIceFields *f,
                               uint32_t *status_bits, uint8_t *tie);

EXPORT int ice3o_rain_ice(const C *c, const Ice3gbLuts *lut, int nij, int nk, double dt,
                          const Ice3gbRainIceOptions *opt, const Ice3gbRainIceFields *f,
                          uint32_t *status_bits)
{
  return ice3o_rain_ice_ties(c, lut, nij, nk, dt, opt, f, status_bits, NULL);
}

/* ice3o_rain_ice that also marks (tie[p] != 0, when tie is not NULL) the
 * points whose sub-stepping took a decision on rounding residuals (bit 0: a
 * graupel or hail growth-mode choice; bit 1: the reset of CIT after a pass
 * that depleted the ice to a residual; bit 2: an MRSTEP threshold equal to
 * the sub-step, which decides between a soft pass and a new outer
 * iteration; bit 3: a new outer iteration's hard pass after a bit-1 reset,
 * which carries the reset into every rate); there the reference's own outcome
 * depends on the last bits of the rates. */
EXPORT int ice3o_rain_ice_ties(const C *c, const Ice3gbLuts *lut, int nij, int nk, double dt,
                               const Ice3gbRainIceOptions *opt, const Ice3gbRainIceFields *f,
                               uint32_t *status_bits, uint8_t *tie)
{
  if (!c || !lut || !f || nij <= 0 || nk <= 0) return ICE3GB_ERR_SHAPE;
  if (!rain_ice_supported(c)) return ICE3GB_ERR_UNSUPPORTED;
  const int hail = (int)c->NRR == 7;
  if (hail && (!f->rht || !f->rhs || !f->inprh || (opt && opt->sed_jax > 0))) return ICE3GB_ERR_UNSUPPORTED;
  const int ocnd2 = c->OCND2 != 0.0;
  if (ocnd2 && (!f->ssio || !f->ssiu || !f->ifr || !f->icldfr))
    return ICE3GB_ERR_UNSUPPORTED;
  const long n = (long)nij * nk;
  /* OCND2: TIWMX tables, level heights (rain_ice.F90:386-394: the sum of
   * dzz from the last level IKTE down to the level, minus half its own
   * thickness; with k = 0 at the surface (NKL = 1) IKTE is the top level) and
   * the cloud droplet concentration (:396-435) */
  double *tw = NULL, *zzz = NULL, *conc = NULL;
  if (ocnd2) {
    tw = (double *)malloc(sizeof(double) * TW_N * TIWMX_N);
    zzz = (double *)malloc(sizeof(double) * 2 * n);
    if (!tw || !zzz) { free(tw); free(zzz); return ICE3GB_ERR_RANGE; }
    conc = zzz + n;
    ice3o_tiwmx_all(c, tw);
    const int st = f->sea != NULL && f->town != NULL;
    for (long col = 0; col < nij; ++col) {
      double zsum = 0.;
      for (int k = nk - 1; k >= 0; --k) {
        const long p = (long)k * nij + col;
        zsum = zsum + f->dzz[p];
        zzz[p] = zsum - f->dzz[p] * 0.5;
      }
      const double top = zzz[(long)(nk - 1) * nij + col];
      for (int k = 0; k < nk; ++k) {
        const long p = (long)k * nij + col;
        double cc = c->CONC_LAND;
        if (st && c->FRMIN26 < 0.001) {
          const double tmp = f->sea[col] * c->CONC_SEA + (1. - f->sea[col]) * c->CONC_LAND;
          cc = (1. - f->town[col]) * tmp + f->town[col] * c->CONC_URBAN;
        }
        if (c->FRMIN26 > 0.001) {
          cc = c->FRMIN26 * f->pabs[p] / c->P00;
          if (c->FRMIN22 > 0.001 && st) {
            const double tmp = dmax(0., dmin(1., (zzz[p] - top) / (dmax(0.01, c->FRMIN29 - top))));
            cc = cc * (c->FRMIN22 * (f->sea[col] * c->FRMIN30 + (1. - f->sea[col])) * (1. - tmp) + tmp);
          }
        }
        conc[p] = cc;
      }
    }
  }
  const int lsedim_after = (opt && opt->lsedim_after >= 0) ? opt->lsedim_after : (c->LSEDIM_AFTER != 0.0);
  const int ldeposc = (opt && opt->ldeposc >= 0) ? opt->ldeposc : (c->LDEPOSC != 0.0);
  const int max_passes = (opt && opt->max_passes > 0) ? opt->max_passes : 256;
  const int sed_fortran = !(opt && opt->sed_jax > 0);
  C cc = *c;
  if (opt && opt->lfeedbackt >= 0) cc.LFEEDBACKT = opt->lfeedbackt ? 1.0 : 0.0;
  c = &cc;
  const int has_st = f->sea != NULL && f->town != NULL;
  double *lsf = (double *)malloc(sizeof(double) * n);
  double *lvf = (double *)malloc(sizeof(double) * n);
  double *rvheni = (double *)malloc(sizeof(double) * n);
  int64_t *key = (int64_t *)malloc(sizeof(int64_t) * n);
  if (!lsf || !lvf || !rvheni || !key) {
    free(lsf); free(lvf); free(rvheni); free(key); free(tw); free(zzz);
    return ICE3GB_ERR_RANGE;
  }
  int capped_any = 0;

  /* 2. sedimentation before the microphysics (rain_ice.F90:442-462 -> ICE4_SEDIMENTATION) */
  int sed_capped = 0;
  if (!lsedim_after) sed_capped |= !rain_ice_sediment(c, nij, nk, dt, sed_fortran, has_st, f);

  /* 4.2 precipitation fraction (rain_ice.F90:555-605): with a PRFR option,
   * ICE4_COMPUTE_PDF on the time-t state of the LLMICRO points (its
   * partition overwrites PHLC_HCF/HRC, PHLI_HCF/HRI), then ICE4_RAINFR_VERT
   * down each column; the sub-stepping starts from that fraction. */
  const int llrfr = (int)c->SUBG_RC_RR_ACCR == 1 || (int)c->SUBG_RR_EVAP == 2;
  if (llrfr) {
    const int sigm = (int)c->SUBG_AUCV_RC == 1 && (int)c->SUBG_PR_PDF == 0;
    const int adju = (int)c->SUBG_AUCV_RC == 2 || (int)c->SUBG_AUCV_RI == 2;
#pragma omp parallel for schedule(static)
    for (long p = 0; p < n; ++p) {
      const double rc = f->rct[p], ri = f->rit[p], cf = f->cldfr[p];
      const int micro = rc > c->C_RTMIN || f->rrt[p] > c->R_RTMIN || ri > c->I_RTMIN || f->rst[p] > c->S_RTMIN ||
                        f->rgt[p] > c->G_RTMIN || (hail && f->rht[p] > c->H_RTMIN);
      double hl[4] = {f->hlc_hcf[p], 0.0, f->hlc_hrc[p], 0.0}, hi[4] = {f->hli_hcf[p], 0.0, f->hli_hri[p], 0.0};
      if (adju) {                                                     /* :564-581 */
        hl[3] = rc - hl[2];
        hi[3] = ri - hi[2];
        hl[1] = rc > 0. ? cf - hl[0] : 0.;
        hi[1] = ri > 0. ? cf - hi[0] : 0.;
      }
      const double sigma_rc = sigm ? f->sigs[p] * f->sigs[p] : 0.0;  /* :556-563 */
      const double rf = ice4_compute_pdf(c, micro, f->rhodref[p], rc, ri, cf, f->tht[p] * f->exn[p], sigma_rc, hl, hi);
      f->hlc_hcf[p] = hl[0]; f->hlc_hrc[p] = hl[2]; f->hli_hcf[p] = hi[0]; f->hli_hri[p] = hi[2];
      f->rainfr[p] = rf;
    }
    rainfr_vert_h(c, nij, nk, f->rainfr, f->rrt, f->rst, f->rgt, hail ? f->rht : NULL);
  }

  /* 1., 3., 4., 5. pointwise part */
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : capped_any)
  for (long p = 0; p < n; ++p) {
    const double exn = f->exn[p], rho = f->rhodref[p], pres = f->pabs[p];
    const double th = f->tht[p], rv = f->rvt[p], rc = f->rct[p], rr = f->rrt[p];
    const double ri = f->rit[p], rs = f->rst[p], rg = f->rgt[p], rh = hail ? f->rht[p] : 0.0;
    /* :334-345 lsfact/lvfact without exner */
    const double t = th * exn;
    rain_ice_thermo(c, hail, t, rv, rc, rr, ri, rs, rg, rh, &lsf[p], &lvf[p]);
    /* :370-381 LLMICRO */
    int micro = rain_ice_micro(c, hail, rc, rr, ri, rs, rg, rh);
    Ocnd2Pt oc;
    if (ocnd2) {                                                      /* :347-363 */
      const double m = c->FRMIN13;
      micro = f->ssio[p] > c->FRMIN12 || rc > m || rr > m || ri > m || rs > m || rg > m || (hail && rh > m);
      oc.tw = tw; oc.ssio = f->ssio[p]; oc.ssiu = f->ssiu[p]; oc.ifr = f->ifr[p]; oc.icldfr = f->icldfr[p];
      oc.zzz = zzz[p]; oc.conc = conc[p];
    }
    f->evap3d[p] = 0.0;
    if (!llrfr) f->rainfr[p] = 1.0;  /* :603-605 */
    double cit = f->cit[p];
    double zrvheni = 0.0;
    if (!micro) {
      /* :506-529 nucleation outside LLMICRO points */
      cit = 0.0;
      ice4_nucleation(c, 1, th, pres, rho, exn, lsf[p] / exn, t, rv, &cit, &zrvheni, NULL, ocnd2 ? tw : NULL,
                      ocnd2 ? oc.zzz : 0.0, ocnd2 ? oc.icldfr : 0.0);
    }
    /* :535-539 */
    zrvheni = dmin(f->rvs[p], zrvheni / dt);
    rvheni[p] = zrvheni;
    key[p] = -1;
    if (tie) tie[p] = 0;
    if (micro) {
      /* ICE4_PACK + ICE4_STEPPING (mode_ice4_pack.F90:230-330) */
      StepOut s;
      s.vart[ITH] = th; s.vart[IRV] = rv; s.vart[IRC] = rc; s.vart[IRR] = rr;
      s.vart[IRI] = ri; s.vart[IRS] = rs; s.vart[IRG] = rg;
      s.extpk[ITH] = f->ths[p]; s.extpk[IRV] = f->rvs[p]; s.extpk[IRC] = f->rcs[p]; s.extpk[IRR] = f->rrs[p];
      s.extpk[IRI] = f->ris[p]; s.extpk[IRS] = f->rss[p]; s.extpk[IRG] = f->rgs[p];
      s.vart[IRH] = rh;
      s.extpk[IRH] = hail ? f->rhs[p] : 0.0;
      s.cit = cit;
      s.rainfr = llrfr ? f->rainfr[p] : 1.0;
      const int sigm = (int)c->SUBG_AUCV_RC == 1 && (int)c->SUBG_PR_PDF == 0;
      const double sigma_rc = sigm ? 2.0 * f->sigs[p] : 0.0;  /* pack :266 + stepping :160-166 */
      ice4_stepping_point(c, lut, dt, max_passes, exn, rho, pres, f->cldfr[p], sigma_rc,
                          f->hlc_hcf[p], f->hlc_hrc[p], f->hli_hcf[p], f->hli_hri[p], &s, ocnd2 ? &oc : NULL);
      cit = s.cit;
      if (c->LWARM != 0.0) f->evap3d[p] = s.rrevav;
      f->rainfr[p] = s.rainfr;
      capped_any |= s.capped;
      if (tie) tie[p] = (uint8_t)s.tie;
      key[p] = ((int64_t)s.outer << 32) | (int64_t)s.inner;
      /* 8.1 total tendencies (rain_ice.F90:758-790, disabled in the vendored copy) */
      const double r0[NVH] = {th, rv, rc, rr, ri, rs, rg, rh};
      double *src[NVH] = {&f->ths[p], &f->rvs[p], &f->rcs[p], &f->rrs[p], &f->ris[p], &f->rss[p], &f->rgs[p],
                          hail ? &f->rhs[p] : NULL};
      total_tendencies(hail, 1.0 / dt, lvf[p] / f->exnref[p], lsf[p] / f->exnref[p], s.vart, r0, zrvheni, src);
    } else {
      const double lsx = lsf[p] / f->exnref[p];
      f->ths[p] += zrvheni * lsx;
      f->rvs[p] -= zrvheni;
      f->ris[p] += zrvheni;
    }
    f->cit[p] = cit;
  }
  /* PRREVAV after the last pass of the call (mode_ice4_stepping.F90:514-516) */
  if (c->LWARM != 0.0) {
    int64_t kmax = -1;
    for (long p = 0; p < n; ++p) if (key[p] > kmax) kmax = key[p];
#pragma omp parallel for schedule(static)
    for (long p = 0; p < n; ++p)
      if (key[p] >= 0 && key[p] != kmax) f->evap3d[p] = 0.0;
  }
  /* 8.2 negativity correction on the sources (ICE4_CORRECT_NEGATIVITIES) */
#pragma omp parallel for schedule(static)
  for (long p = 0; p < n; ++p) {
    double x[NVH] = {f->ths[p], f->rvs[p], f->rcs[p], f->rrs[p], f->ris[p], f->rss[p], f->rgs[p],
                     hail ? f->rhs[p] : 0.0};
    correct_negativities(c->V_RTMIN, c->V_RTMIN, hail, 1, lvf[p] / f->exnref[p], lsf[p] / f->exnref[p], x);
    f->ths[p] = x[ITH]; f->rvs[p] = x[IRV]; f->rcs[p] = x[IRC]; f->rrs[p] = x[IRR]; f->ris[p] = x[IRI];
    f->rss[p] = x[IRS]; f->rgs[p] = x[IRG];
    if (hail) f->rhs[p] = x[IRH];
  }
  /* 9. sedimentation after (rain_ice.F90:816-841) */
  if (lsedim_after) sed_capped |= !rain_ice_sediment(c, nij, nk, dt, sed_fortran, has_st, f);
  /* 10. fog deposition (rain_ice.F90:876-895), level k = 0 */
  for (long col = 0; col < nij; ++col) {
    if (ldeposc) {
      const double indep = fog_deposition(c, f->rct[col], f->rhodref[col], f->dzz[col], &f->rcs[col], &f->inprc[col]);
      if (f->indep) f->indep[col] = indep;
    } else if (f->indep) {
      f->indep[col] = 0.0;
    }
  }
  free(lsf); free(lvf); free(rvheni); free(key); free(tw); free(zzz);
  if (status_bits) *status_bits = (capped_any ? ICE3GB_DEV_PASS_CAP : 0u) | (sed_capped ? ICE3GB_DEV_SED_CAP : 0u);
  return ICE3GB_OK;
}

/* ===================================================================== */
/* Per-process entry points (hard pass) used by the golden-vector tests  */
/* ===================================================================== */

EXPORT void ice3o_nucleation(const C *c, long n, const double *tht, const double *pabst, const double *rhodref,
                             const double *exn, const double *lsfact, const double *t, const double *rvt,
                             const uint8_t *ldcompute, double *cit, double *rvheni_mr)
{
  for (long p = 0; p < n; ++p)
    ice4_nucleation(c, ldcompute[p], tht[p], pabst[p], rhodref[p], exn[p], lsfact[p], t[p], rvt[p], &cit[p],
                    &rvheni_mr[p], NULL, NULL, 0.0, 0.0);
}

EXPORT void ice3o_rrhong_rimltc(const C *c, long n, const double *t, const double *exn, const double *lvfact,
                                const double *lsfact, const double *tht, const double *rrt, const double *rit,
                                const uint8_t *ldcompute, double *rrhong, double *rimltc)
{
  for (long p = 0; p < n; ++p) {
    rrhong[p] = ice4_rrhong(c, ldcompute[p], exn[p], lvfact[p], lsfact[p], t[p], rrt[p], tht[p]);
    rimltc[p] = ice4_rimltc(c, ldcompute[p], exn[p], lvfact[p], lsfact[p], t[p], tht[p], rit[p]);
  }
}

EXPORT void ice3o_derived_slopes(const C *c, long n, const double *t, const double *rhodref, const double *pres,
                                 const double *rv, const double *rr, const double *rs, const double *rg,
                                 double *out /* [9][n]: ssi ka dv ai cj lbdar lbdar_rf lbdas lbdag */)
{
  for (long p = 0; p < n; ++p) {
    ice4_derived(c, t[p], rhodref[p], pres[p], rv[p], &out[p], &out[n + p], &out[2 * n + p], &out[3 * n + p],
                 &out[4 * n + p]);
    Tctx x;
    memset(&x, 0, sizeof(x));
    x.c = c; x.rhodref = rhodref[p]; x.t = t[p];
    x.v[IRR] = rr[p]; x.v[IRS] = rs[p]; x.v[IRG] = rg[p];
    ice4_slopes(&x);
    out[5 * n + p] = x.lbdar; out[6 * n + p] = x.lbdar_rf; out[7 * n + p] = x.lbdas; out[8 * n + p] = x.lbdag;
  }
}

EXPORT void ice3o_compute_pdf(const C *c, long n, const uint8_t *ldmicro, const double *rhodref, const double *rct,
                              const double *rit, const double *cf, const double *t, const double *sigma_rc,
                              double *out /* [9][n]: hlc_hcf hlc_lcf hlc_hrc hlc_lrc hli_hcf hli_lcf hli_hri hli_lri rf */)
{
  for (long p = 0; p < n; ++p) {
    double hl[4] = {0, 0, 0, 0}, hi[4] = {0, 0, 0, 0};
    const double rf = ice4_compute_pdf(c, ldmicro[p], rhodref[p], rct[p], rit[p], cf[p], t[p], sigma_rc[p], hl, hi);
    for (int k = 0; k < 4; ++k) { out[k * n + p] = hl[k]; out[(4 + k) * n + p] = hi[k]; }
    out[8 * n + p] = rf;
  }
}

/* Hard-pass rates of the slow/warm/fast processes for given inputs.
 * in: [22][n] = t rhodref pres rv rc rr ri rs rg cit ssi ka dv ai cj hlc_hcf hlc_hrc
 *     hli_hcf hli_hri cf rainfr tht (cf, rainfr, tht: the cloud fraction,
 *     precipitation fraction and theta the CLFR/PRFR warm processes use)
 * out: [NBU][n] budget rates, plus rs_tend [8][n] and rg_tend [8][n]. */
EXPORT int ice3o_process_rates(const C *c, const Ice3gbLuts *lut, long n, const double *in, const uint8_t *ldcompute,
                               double *out_bu, double *out_rs, double *out_rg)
{
  for (long p = 0; p < n; ++p) {
    Tctx x;
    PointRates pr;
    memset(&x, 0, sizeof(x));
    memset(&pr, 0, sizeof(pr));
    x.c = c; x.lut = lut; x.ldsoft = 0; x.ldcompute = ldcompute[p];
    x.t = in[p]; x.rhodref = in[n + p]; x.pres = in[2 * n + p];
    x.v[IRV] = in[3 * n + p]; x.v[IRC] = in[4 * n + p]; x.v[IRR] = in[5 * n + p];
    x.v[IRI] = in[6 * n + p]; x.v[IRS] = in[7 * n + p]; x.v[IRG] = in[8 * n + p];
    const double cit = in[9 * n + p];
    pr.ssi = in[10 * n + p]; pr.ka = in[11 * n + p]; pr.dv = in[12 * n + p]; pr.ai = in[13 * n + p];
    pr.cj = in[14 * n + p];
    x.hl[0] = in[15 * n + p]; x.hl[2] = in[16 * n + p];
    x.hi[0] = in[17 * n + p]; x.hi[2] = in[18 * n + p];
    x.cf = in[19 * n + p]; x.rainfr = in[20 * n + p];
    x.v[ITH] = in[21 * n + p];  /* only used by the CLFR/PRFR evaporation */
    ice4_slopes(&x);
    ice4_slow(&x, &pr);
    ice4_warm(&x, &pr);
    ice4_fast_rs(&x, &pr);
    ice4_fast_rg(&x, &pr, cit);
    ice4_fast_ri(&x, &pr, cit);
    for (int k = 0; k < NBU; ++k) out_bu[k * n + p] = pr.bu[k];
    for (int k = 0; k < NRS; ++k) out_rs[k * n + p] = pr.rs_tend[k];
    for (int k = 0; k < NRG; ++k) out_rg[k * n + p] = pr.rg_tend[k];
  }
  return NBU;
}

/* ICE4_RAINFR_VERT (micro/mode_ice4_rainfr_vert.F90; stencils/rain_ice.py:272-320). */
/* ICE4_RAINFR_VERT with the optional hail (rh NULL for KRR = 6). */
static void rainfr_vert_h(const C *c, int nij, int nk, double *prfr, const double *rr, const double *rs,
                          const double *rg, const double *rh)
{
  for (long col = 0; col < nij; ++col) {
    prfr[(long)(nk - 1) * nij + col] = 0.0;
    for (int k = nk - 2; k >= 0; --k) {
      const long p = (long)k * nij + col;
      int mask = rr[p] > c->R_RTMIN || rs[p] > c->S_RTMIN || rg[p] > c->G_RTMIN;
      if (rh) mask = mask || rh[p] > c->H_RTMIN;
      if (mask) {
        prfr[p] = dmax(prfr[p], prfr[p + nij]);
        if (prfr[p] == 0.) prfr[p] = 1.;
      } else {
        prfr[p] = 0.;
      }
    }
  }
}

EXPORT void ice3o_rainfr_vert(const C *c, int nij, int nk, double *prfr, const double *rr, const double *rs,
                              const double *rg)
{
  for (long col = 0; col < nij; ++col) {
    prfr[(long)(nk - 1) * nij + col] = 0.0;
    for (int k = nk - 2; k >= 0; --k) {
      const long p = (long)k * nij + col;
      const int mask = rr[p] > c->R_RTMIN || rs[p] > c->S_RTMIN || rg[p] > c->G_RTMIN;
      if (mask) {
        prfr[p] = dmax(prfr[p], prfr[p + nij]);
        if (prfr[p] == 0.) prfr[p] = 1.;
      } else {
        prfr[p] = 0.;
      }
    }
  }
}

EXPORT int ice3o_budget_count(void) { return NBU; }

/* The OCND2 pieces of ICE4_TENDENCIES on n points, hard pass, LDCOMPUTE:
 * in = [t, rhodref, pres, rv, rc, rr, ri, rs, rg, cit, ssio, ssiu, ifr,
 * icldfr, zzz, conc] per point (n x 16); out = [cit after the nucleation,
 * es_i, ssi, ai, colf, acrf, rilars, rvdepi] per point (n x 8), with ssi and
 * ai those after the tabulated derived fields (in = state after the
 * instantaneous processes, exn = 1). */
EXPORT void ice3o_ocnd2_rates(const C *c, long n, const double *in, double *out)
{
  double *tw = (double *)malloc(sizeof(double) * TW_N * TIWMX_N);
  if (!tw) return;
  ice3o_tiwmx_all(c, tw);
  for (long p = 0; p < n; ++p) {
    const double *x = in + p * 16;
    Ocnd2Pt oc = {tw, x[10], x[11], x[12], x[13], x[14], x[15]};
    double cit = x[9], rvheni;
    ice4_nucleation(c, 1, x[0], x[2], x[1], 1.0, 1.0, x[0], x[3], &cit, &rvheni, NULL, tw, oc.zzz, oc.icldfr);
    Tctx t;
    memset(&t, 0, sizeof(t));
    t.c = c; t.ldsoft = 0; t.ldcompute = 1; t.t = x[0]; t.rhodref = x[1]; t.pres = x[2];
    t.v[IRV] = x[3]; t.v[IRC] = x[4]; t.v[IRR] = x[5]; t.v[IRI] = x[6]; t.v[IRS] = x[7]; t.v[IRG] = x[8];
    t.tw = tw; t.ssio = oc.ssio; t.ssiu = oc.ssiu; t.ifr = oc.ifr; t.icldfr = oc.icldfr; t.zzz = oc.zzz;
    t.conc = oc.conc;
    PointRates pr;
    memset(&pr, 0, sizeof(pr));
    ice4_derived(c, t.t, t.rhodref, t.pres, t.v[IRV], &pr.ssi, &pr.ka, &pr.dv, &pr.ai, &pr.cj);
    ocnd2_derived(&t, &pr);
    ice4_fast_ri_rs(&t, &pr, cit);
    double *o = out + p * 8;
    o[0] = cit; o[1] = pr.esi; o[2] = pr.ssi; o[3] = pr.ai; o[4] = pr.colf; o[5] = pr.acrf;
    o[6] = pr.bu[B_RILARS]; o[7] = pr.bu[B_RVDEPI];
  }
  free(tw);
}

/* ICE4_FAST_RH alone on n points (hard pass, LDCOMPUTE): in = [t, rhodref,
 * pres, rv, rc, rr, ri, rs, rg, rh] per point (n x 10), ldwetg per point;
 * out = the 10 persistent tendencies PRH_TEND then the 14 hail budget terms
 * (RWETGH .. RHMLTR, the first two left 0) per point (n x 24).  Derived
 * fields and slopes as ICE4_TENDENCIES forms them. */
EXPORT void ice3o_fast_rh(const C *c, const Ice3gbLuts *lut, long n, const double *in, const uint8_t *ldwetg,
                          double *out)
{
  for (long p = 0; p < n; ++p) {
    const double *x = in + p * 10;
    Tctx t;
    memset(&t, 0, sizeof(t));
    t.c = c; t.lut = lut; t.ldsoft = 0; t.ldcompute = 1; t.hail = 1;
    t.t = x[0]; t.rhodref = x[1]; t.pres = x[2];
    t.v[IRV] = x[3]; t.v[IRC] = x[4]; t.v[IRR] = x[5]; t.v[IRI] = x[6]; t.v[IRS] = x[7]; t.v[IRG] = x[8];
    t.v[IRH] = x[9];
    t.rainfr = 1.0;
    PointRates pr;
    memset(&pr, 0, sizeof(pr));
    ice4_derived(c, t.t, t.rhodref, t.pres, t.v[IRV], &pr.ssi, &pr.ka, &pr.dv, &pr.ai, &pr.cj);
    ice4_slopes(&t);
    ice4_fast_rh(&t, &pr, ldwetg[p]);
    double *o = out + p * 24;
    for (int k = 0; k < NRH; ++k) o[k] = pr.rh_tend[k];
    for (int k = 0; k < 14; ++k) o[NRH + k] = pr.bu[B_RWETGH + k];
  }
}

/* ===================================================================== */
/* Chained step: S1 = ice_adjust(x_t, S0); S2 = rain_ice(x_t, S1);        */
/* S3 = ice_adjust(dt*S2, S2)  (same contract as ice3gb_physics_step)       */
/* ===================================================================== */
EXPORT int ice3o_physics_step(const C *c, const Ice3gbLuts *lut, int nij, int nk, double dt,
                              const Ice3gbRainIceOptions *opt, const Ice3gbStepFields *f, uint32_t *bits)
{
  const long n = (long)nij * nk;
  double *buf = (double *)malloc(sizeof(double) * 16 * (size_t)n);
  if (!buf) return ICE3GB_ERR_RANGE;
  double *d[16];
  for (int i = 0; i < 16; ++i) d[i] = buf + (size_t)i * n;
  /* 1. first adjustment; cldfr and hl* into scratch d[0..4], the rest discarded d[5..11] */
  Ice3gbIceAdjustFields a;
  memset(&a, 0, sizeof(a));
  a.sigqsat = f->sigqsat; a.pabs = f->pabs; a.sigs = f->sigs; a.th = f->th; a.exn = f->exn;
  a.exn_ref = f->exnref; a.rho_dry_ref = f->rhodref; a.rv = f->rv; a.rc = f->rc; a.ri = f->ri; a.rr = f->rr;
  a.rs = f->rs; a.rg = f->rg; a.cf_mf = f->cf_mf; a.rc_mf = f->rc_mf; a.ri_mf = f->ri_mf;
  a.rvs = f->rvs; a.rcs = f->rcs; a.ris = f->ris; a.ths = f->ths;
  a.cldfr = d[0]; a.hlc_hrc = d[1]; a.hlc_hcf = d[2]; a.hli_hri = d[3]; a.hli_hcf = d[4];
  a.t = d[5]; a.rv_out = d[6]; a.rc_out = d[7]; a.ri_out = d[8]; a.cph = d[9]; a.lv = d[10]; a.ls = d[11];
  a.sigqsat_3d = 0;
  int rc = ice3o_ice_adjust(c, nij, nk, dt, &a);
  if (rc) { free(buf); return rc; }
  /* 2. rain_ice */
  Ice3gbRainIceFields r;
  memset(&r, 0, sizeof(r));
  r.exn = f->exn; r.dzz = f->dzz; r.rhodref = f->rhodref; r.exnref = f->exnref; r.pabs = f->pabs;
  r.cldfr = d[0]; r.sigs = f->sigs; r.tht = f->th; r.rvt = f->rv; r.rct = f->rc; r.rrt = f->rr;
  r.rit = f->ri; r.rst = f->rs; r.rgt = f->rg; r.sea = f->sea; r.town = f->town; r.cit = f->cit;
  r.hlc_hrc = d[1]; r.hlc_hcf = d[2]; r.hli_hri = d[3]; r.hli_hcf = d[4];
  r.ths = f->ths; r.rvs = f->rvs; r.rcs = f->rcs; r.rrs = f->rrs; r.ris = f->ris; r.rss = f->rss; r.rgs = f->rgs;
  r.evap3d = f->evap3d; r.rainfr = f->rainfr; r.inprc = f->inprc; r.inprr = f->inprr; r.inpri = f->inpri;
  r.inprs = f->inprs; r.inprg = f->inprg;
  rc = ice3o_rain_ice(c, lut, nij, nk, dt, opt, &r, bits);
  if (rc) { free(buf); return rc; }
  /* 3. adjust again the post-microphysics state dt*S2 (d[5..11] reused) */
  double *th2 = d[5], *rv2 = d[6], *rc2 = d[7], *ri2 = d[8], *rr2 = d[9], *rs2 = d[10], *rg2 = d[11];
#pragma omp parallel for schedule(static)
  for (long p = 0; p < n; ++p) {
    th2[p] = dt * f->ths[p];
    rv2[p] = dt * f->rvs[p];
    rc2[p] = dt * f->rcs[p];
    ri2[p] = dt * f->ris[p];
    rr2[p] = dt * f->rrs[p];
    rs2[p] = dt * f->rss[p];
    rg2[p] = dt * f->rgs[p];
  }
  a.th = th2; a.rv = rv2; a.rc = rc2; a.ri = ri2; a.rr = rr2; a.rs = rs2; a.rg = rg2;
  a.t = f->t; a.rv_out = f->rv_out; a.rc_out = f->rc_out; a.ri_out = f->ri_out; a.cldfr = f->cldfr;
  a.hlc_hrc = f->hlc_hrc; a.hlc_hcf = f->hlc_hcf; a.hli_hri = f->hli_hri; a.hli_hcf = f->hli_hcf;
  a.cph = d[12]; a.lv = d[13]; a.ls = d[14];
  rc = ice3o_ice_adjust(c, nij, nk, dt, &a);
  free(buf);
  return rc;
}

/* Per-point ICE4_STEPPING on explicit inputs (test hook for point-level
 * comparisons).  in: exn rho pres th rv rc rr ri rs rg cit ths rvs rcs rrs ris
 * rss rgs cldfr sigs; out: the 7 state values after the step (external
 * tendency removed), cit, rrevav, capped. */
EXPORT int ice3o_stepping_point(const C *c, const Ice3gbLuts *lut, double dt, int max_passes, const double *in,
                                double *out, int *outer, int *inner)
{
  StepOut s;
  for (int v = 0; v < NV; ++v) { s.vart[v] = in[3 + v]; s.extpk[v] = in[11 + v]; }
  s.vart[IRH] = s.extpk[IRH] = 0.0;
  s.cit = in[10];
  s.rainfr = 1.0;
  const int sigm = (int)c->SUBG_AUCV_RC == 1 && (int)c->SUBG_PR_PDF == 0;
  ice4_stepping_point(c, lut, dt, max_passes, in[0], in[1], in[2], in[18], sigm ? 2.0 * in[19] : 0.0,
                      0.0, 0.0, 0.0, 0.0, &s, NULL);
  for (int v = 0; v < NV; ++v) out[v] = s.vart[v];
  out[7] = s.cit; out[8] = s.rrevav; out[9] = s.capped;
  *outer = s.outer; *inner = s.inner;
  return 0;
}

/* ===================================================================== */
/* RAIN_ICE / ICE4_STEPPING pieces for the golden-vector tests            */
/* (each entry point runs the routine the oracle's rain_ice runs)         */
/* ===================================================================== */

/* rain_ice_thermo + rain_ice_mask (NRR = 6): lsfact / lvfact without the
 * Exner function and LLMICRO, from T and the mixing ratios. */
EXPORT void ice3o_rain_ice_thermo(const C *c, long n, const double *t, const double *rv, const double *rc,
                                  const double *rr, const double *ri, const double *rs, const double *rg,
                                  double *lsf, double *lvf, uint8_t *micro)
{
  for (long p = 0; p < n; ++p) {
    rain_ice_thermo(c, 0, t[p], rv[p], rc[p], rr[p], ri[p], rs[p], rg[p], 0.0, &lsf[p], &lvf[p]);
    micro[p] = (uint8_t)rain_ice_micro(c, 0, rc[p], rr[p], ri[p], rs[p], rg[p], 0.0);
  }
}

/* Total tendencies of micro points (NRR = 6).  vend / r0: [7][n] theta and
 * mixing ratios at the end of the sub-stepping / at t; src: [7][n] sources,
 * updated in place. */
EXPORT void ice3o_total_tendencies(long n, double dt, const double *vend, const double *r0, const double *lvx,
                                   const double *lsx, const double *rvheni, double *src)
{
  for (long p = 0; p < n; ++p) {
    double ve[NVH], r[NVH];
    double *s[NVH];
    for (int v = 0; v < NV; ++v) { ve[v] = vend[v * n + p]; r[v] = r0[v * n + p]; s[v] = &src[v * n + p]; }
    ve[IRH] = r[IRH] = 0.0;
    s[IRH] = NULL;
    total_tendencies(0, 1.0 / dt, lvx[p], lsx[p], ve, r, rvheni[p], s);
  }
}

/* The aggregation of one pass (NRR = 6, no OCND2): bu [NBU][n] rates, A
 * [7][n] tendencies out (from zero). */
EXPORT void ice3o_aggregate(long n, const double *bu, const double *lsfact, const double *lvfact, double *A_out)
{
  for (long p = 0; p < n; ++p) {
    double b[NBU], A[NVH] = {0}, B[NVH] = {0};
    for (int k = 0; k < NBU; ++k) b[k] = bu[k * n + p];
    ice4_aggregate(b, lsfact[p], lvfact[p], 0, 0.0, 1.0, 0, A, B);
    for (int v = 0; v < NV; ++v) A_out[v * n + p] = A[v];
  }
}

/* The sub-step length of one pass (NRR = 6): the time left (dt - t_micro,
 * 0 where ldcompute is off), the LFEEDBACKT limit, the depletion limits
 * with the thresholds rsmin[7]; llcompute_out: the pass does not reach dt.
 * vart, A, B: [7][n]. */
EXPORT void ice3o_step_limiter(const C *c, long n, double dt, const double *rsmin, const double *exn,
                               const double *vart, const double *A, const double *B, const double *t_micro,
                               const uint8_t *ldcompute, double *maxtime, uint8_t *llcompute_out)
{
  for (long p = 0; p < n; ++p) {
    double m = ldcompute[p] ? dt - t_micro[p] : 0.0;
    if (c->LFEEDBACKT != 0.0) m = limit_feedback(c->TT / exn[p], vart[p], A[p], B[p], m);
    for (int v = 1; v < NV; ++v) m = limit_depletion(A[v * n + p], B[v * n + p], vart[v * n + p], rsmin[v], c->MNH_TINY, m);
    maxtime[p] = m;
    llcompute_out[p] = (uint8_t)(ldcompute[p] && !(t_micro[p] + m >= dt));
  }
}

/* The state update of one sub-step and the reset of the ice concentration
 * where the ice is gone (mode_ice4_stepping.F90:388-401); vart [7][n] and
 * cit updated in place. */
EXPORT void ice3o_state_update(long n, const double *A, const double *B, const double *dt_micro,
                               const uint8_t *ldmicro, double *vart, double *cit)
{
  for (long p = 0; p < n; ++p) {
    double v[NVH], a[NVH], b[NVH];
    for (int k = 0; k < NV; ++k) { v[k] = vart[k * n + p]; a[k] = A[k * n + p]; b[k] = B[k * n + p]; }
    state_update(NV, v, a, b, dt_micro[p]);
    for (int k = 0; k < NV; ++k) vart[k * n + p] = v[k];
    if (ldmicro[p] && v[IRI] <= 0.) cit[p] = 0.;
  }
}

/* ICE4_CORRECT_NEGATIVITIES (NRR = 6) on x [7][n] in place; fortran = 1:
 * the Fortran form with the vapour threshold XRTMIN(1) (s_min = g_min =
 * V_RTMIN), 0: the reference JAX stencil's form with its thresholds. */
EXPORT void ice3o_correct_negativities(long n, int fortran, double s_min, double g_min, const double *lvx,
                                       const double *lsx, double *x)
{
  for (long p = 0; p < n; ++p) {
    double v[NVH];
    for (int k = 0; k < NV; ++k) v[k] = x[k * n + p];
    v[IRH] = 0.0;
    correct_negativities(s_min, g_min, 0, fortran, lvx[p], lsx[p], v);
    for (int k = 0; k < NV; ++k) x[k * n + p] = v[k];
  }
}

/* Fog deposition on n columns (their lowest level). */
EXPORT void ice3o_fog_deposition(const C *c, long n, const double *rct, const double *rhodref, const double *dzz,
                                 double *rcs, double *inprc)
{
  for (long p = 0; p < n; ++p) (void)fog_deposition(c, rct[p], rhodref[p], dzz[p], &rcs[p], &inprc[p]);
}
