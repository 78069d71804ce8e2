// rain_ice_point.cuh — per-grid-point ICE4 physics of the rain_ice kernel
// (nucleation, compute_pdf, the slow/warm/fast processes, ICE4_TENDENCIES and
// ICE4_STEPPING for one point).  Host-and-device code: the kernel in
// rain_ice.cu runs it per lane; a host build of the same code serves to
// separate algorithmic from math-library differences when comparing with a
// CPU reference.
#pragma once

#include "ice3gb_device.cuh"

namespace ice3pt {


constexpr int RI_THREADS = 256;
constexpr int LUT_N = sizeof(Ice3gbLuts) / sizeof(double);
constexpr int O_RIM1 = 0, O_RIM2 = 80, O_RIM4 = 160, O_RACCSS = 240, O_RACCS = 1840, O_SACCRG = 3440,
              O_RDRYG = 5040, O_SDRYG = 6640;
static_assert(LUT_N == 9840, "Ice3gbLuts layout");

enum { ITH = 0, IRV, IRC, IRR, IRI, IRS, IRG, NV };
enum {
  B_RVHENI_MR, B_RRHONG_MR, B_RIMLTC_MR,
  B_RCHONI, B_RVDEPS, B_RIAGGS, B_RIAUTS, B_RVDEPG,
  B_RCAUTR, B_RCACCR, B_RREVAV,
  B_RCRIMSS, B_RCRIMSG, B_RSRIMCG, B_RRACCSS, B_RRACCSG, B_RSACCRG, B_RSMLTG, B_RCMLTSR,
  B_RICFRRG, B_RRCFRIG, B_RICFRR, B_RCWETG, B_RIWETG, B_RRWETG, B_RSWETG,
  B_RCDRYG, B_RIDRYG, B_RRDRYG, B_RSDRYG, B_RGMLTR, B_RCBERI,
  NBU
};
enum { RS_RCRIMS, RS_RCRIMSS, RS_RSRIMCG, RS_RRACCS, RS_RRACCSS, RS_RSACCRG, RS_FREEZ1, RS_FREEZ2, NRS };
enum { RG_RCDRYG, RG_RIDRYG, RG_RIWETG, RG_RSDRYG, RG_RSWETG, RG_RRDRYG, RG_FREEZ1, RG_FREEZ2, NRG };

// Rates that persist between the hard pass and the following soft passes
// (Fortran ZBU_INST, ZRS_TEND, ZRG_TEND, ZSSI) plus the derived fields.
struct Rates {
  double bu[NBU];
  double rs[NRS];
  double rg[NRG];
  double ssi, ka, dv, ai, cj;
};

// Per-point constants over the whole step.
struct PointFix {
  double rho, lrho, pres, exn, cf, sigma_rc;
  double rho_mcexvt;    // rho**(-CEXVT)
  double rho_mcexvt1;   // rho**(-CEXVT-1)
  double rcrautc;       // CRIAUTC / rho
};

// Per-pass work state (ICE4_TENDENCIES locals).
struct Pass {
  double t;
  double v[NV];
  double lbdar, lbdas, lbdag;        // slope parameters
  double llbdar, llbdas, llbdag;     // their logarithms
  double rainfr;
  double hl[4], hi[4];
};

ICE3_HD double esat_from(double alp, double beta, double gam, double it, double lt)
{
  return fm::fexp(alp - beta * it - gam * lt);
}

// ICE4_NUCLEATION (micro/ice4_nucleation.func.h:69-144, LOCND2 = .FALSE.).
ICE3_HD void nucleation(const Cst &c, bool ld, double tht, double pabst, double rhodref, double exn,
                        double lsfact, double t, double rvt, double &cit, double &rvheni)
{
  rvheni = 0.0;
  if (!(ld && t < c.TT && rvt > c.V_RTMIN)) return;
  const double lt = fm::flog(t), it = 1.0 / t;
  double zusw = esat_from(c.ALPW, c.BETAW, c.GAMW, it, lt);
  double zzw = esat_from(c.ALPI, c.BETAI, c.GAMI, it, lt);
  zzw = fmin(pabst * 0.5, zzw);
  double zssi = rvt * (pabst - zzw) / (c.EPSILO * zzw) - 1.0;
  zusw = fmin(pabst * 0.5, zusw);
  zusw = (zusw / zzw) * ((pabst - zzw) / (pabst - zusw)) - 1.0;
  zssi = fmin(zssi, zusw);
  zzw = 0.0;
  if (t < c.TT - 5.0 && zssi > 0.0) {
    zzw = c.NU20 * fm::fexp(c.ALPHA2 * zssi - c.BETA2);
  } else if (t <= c.TT - 2.0 && t >= c.TT - 5.0 && zssi > 0.0) {
    zzw = fmax(c.NU20 * fm::fexp(-c.BETA2), c.NU10 * fm::fexp(-c.BETA1 * (t - c.TT) + c.ALPHA1 * fm::flog(zssi / zusw)));
  }
  zzw = fmin(zzw - cit, 50.e3);
  rvheni = fmin(rvt, fmax(zzw, 0.0) * c.MNU0 / rhodref);
  if (c.LFEEDBACKT != 0.0) {
    const double w = fmin(rvheni, fmax(0.0, (c.TT / exn - tht) / lsfact)) / fmax(rvheni, 1.e-20);
    rvheni *= w;
    zzw *= w;
  }
  cit = fmax(zzw + cit, cit);
}

// ICE4_COMPUTE_PDF (micro/mode_ice4_compute_pdf.F90), one point; returns RF.
ICE3_HD double compute_pdf(const Cst &c, bool ld, double rcrautc_pt, double rct, double rit, double cf, double t,
                           double sigma_rc, double hl[4], double hi[4])
{
  const int aucv_rc = (int)c.SUBG_AUCV_RC, aucv_ri = (int)c.SUBG_AUCV_RI, prpdf = (int)c.SUBG_PR_PDF;
  const double rcrautc = ld ? rcrautc_pt : 0.0;
  double hcf = 0, lcf = 0, hrc = 0, lrc = 0;
  if (aucv_rc == 0) {
    if (rct > rcrautc && ld) { hcf = 1.0; hrc = rct; }
    else if (rct > c.C_RTMIN && ld) { lcf = 1.0; lrc = rct; }
  } else if (aucv_rc == 3) {
    if (cf > 0.0 && rct > rcrautc * cf && ld) { hcf = cf; hrc = rct; }
    else if (cf > 0.0 && rct > c.C_RTMIN && ld) { lcf = cf; lrc = rct; }
  } else if (aucv_rc == 2) {
    const double sum = ld ? hl[3] + hl[2] : 0.0;
    hcf = hl[0]; lcf = hl[1];
    if (sum > 1.e-20 && ld) { lrc = hl[3] * rct / sum; hrc = hl[2] * rct / sum; }
  } else if (aucv_rc == 1 && prpdf == 0) {
    if (rct > rcrautc + sigma_rc && ld) {
      hcf = 1.0; hrc = rct;
    } else if (rct > rcrautc - sigma_rc && rct <= rcrautc + sigma_rc && ld) {
      const double inv2s = 1.0 / (2.0 * sigma_rc);
      hcf = (rct + sigma_rc - rcrautc) * inv2s;
      lcf = fmax(0.0, cf - hcf);
      hrc = (rct + sigma_rc - rcrautc) * (rct + sigma_rc + rcrautc) * (0.5 * inv2s);
      lrc = fmax(0.0, rct - hrc);
    } else if (rct > c.C_RTMIN && cf > 0.0 && ld) {
      lcf = cf; lrc = rct;
    }
  } else if (aucv_rc == 1) {
    const double coeff = (prpdf == 1 || prpdf == 2) ? 2.0 : (prpdf == 3 ? 3.0 : 4.0);
    const double rcmax = (rct > 0.0 && cf > 0.0 && ld) ? coeff * rct / cf : 0.0;
    double lloc = 0.0, hloc = 0.0;
    const bool ok = rct > 0.0 && cf > 0.0 && rcmax > rcrautc && ld;
    const double a = rcrautc, m = rcmax;
    if (prpdf == 1) {
      if (ok) { lloc = 0.5 * a; hloc = (m + a) / 2.0; }
    } else if (prpdf == 3) {
      if (ok) { lloc = (a * (3.0 * m - 2.0 * a)) / (3.0 * (2.0 * m - a)); hloc = (m + 2.0 * a) / 3.0; }
    } else if (prpdf == 4) {
      if (ok) {
        lloc = (3.0 * a * a * a - 8.0 * a * a * m + 6.0 * a * m * m) / (4.0 * a * a - 12.0 * a * m + 12.0 * m * m);
        hloc = (m + 3.0 * a) / 4.0;
      }
    } else if (prpdf == 2) {
      if (rct <= a * cf && ok) {
        lloc = (m * m * m - 12.0 * m * a * a + 8.0 * a * a * a) / (6.0 * m * m - 24.0 * m * a + 12.0 * a * a);
        hloc = (m + 2.0 * a) / 3.0;
      } else if (ok) {
        lloc = (2.0 / 3.0) * a;
        hloc = (3.0 * m * m * m - 8.0 * a * a * a) / (6.0 * m * m - 12.0 * a * a);
      }
    }
    if (ok) {
      lcf = cf * (hloc - (rct / cf)) / (hloc - lloc);
      hcf = fmax(0.0, cf - lcf);
      lrc = lloc * lcf;
      hrc = fmax(0.0, rct - lrc);
    } else if (rct > 0.0 && cf > 0.0 && rcmax <= rcrautc && ld) {
      lcf = cf; lrc = rct;
    }
  }
  hl[0] = hcf; hl[1] = lcf; hl[2] = hrc; hl[3] = lrc;
  const double criauti = ld ? fmin(c.CRIAUTI, fm::fexp10(c.ACRIAUTI * (t - c.TT) + c.BCRIAUTI)) : 0.0;
  double ihcf = 0, ilcf = 0, ihri = 0, ilri = 0;
  if (aucv_ri == 0) {
    if (rit > criauti && ld) { ihcf = 1.0; ihri = rit; }
    else if (rit > c.I_RTMIN && ld) { ilcf = 1.0; ilri = rit; }
  } else if (aucv_ri == 1) {
    if (cf > 0.0 && rit > criauti * cf && ld) { ihcf = cf; ihri = rit; }
    else if (cf > 0.0 && rit > c.I_RTMIN && ld) { ilcf = cf; ilri = rit; }
  } else if (aucv_ri == 2) {
    const double sum = ld ? hi[3] + hi[2] : 0.0;
    ihcf = hi[0]; ilcf = hi[1];
    if (sum > 1.e-20 && ld) { ilri = hi[3] * rit / sum; ihri = hi[2] * rit / sum; }
  }
  hi[0] = ihcf; hi[1] = ilcf; hi[2] = ihri; hi[3] = ilri;
  return ld ? fmax(hl[0], hi[0]) : 0.0;
}

// INTERP_MICRO (micro/interp_micro.func.h, packed path): index from fm::flog(x).
ICE3_HD double lut_index(double logx, double knum, double p1, double p2, int &i)
{
  const double z = fmax(1.00001, fmin(knum - 0.00001, p1 * logx + p2));
  i = (int)z;
  return z - (double)i;
}
ICE3_HD double lut1d(const double *lt, int i, double f) { return lt[i] * f - lt[i - 1] * (f - 1.0); }
// PLT(i1+1, i2+1) of the 1-based Fortran table is row i1, column i2 of the
// row-major table; lut_index keeps i1 in [1, n1-1] and i2 in [1, n2-1].
ICE3_HD double lut2d(const double *lt, int n2, int i1, double f1, int i2, double f2)
{
  const double *r1 = lt + i1 * n2, *r0 = lt + (i1 - 1) * n2;
  return (r1[i2] * f2 - r1[i2 - 1] * (f2 - 1.0)) * f1 - (r0[i2] * f2 - r0[i2 - 1] * (f2 - 1.0)) * (f1 - 1.0);
}

// Slope parameters, mode_ice4_tendencies.F90:389-433.
ICE3_HD void slopes(const Cst &c, const PointFix &pf, Pass &x)
{
  if (x.v[IRR] > 0.) {
    x.llbdar = fm::flog(c.LBR) + c.LBEXR * (pf.lrho + fm::flog(fmax(x.v[IRR], c.R_RTMIN)));
    x.lbdar = fm::fexp(x.llbdar);
  } else { x.lbdar = 0.0; x.llbdar = -INFINITY; }
  if (c.LSNOW_T != 0.0) {
    if (x.v[IRS] > 0.) {
      const double e = (x.t > 263.15) ? fm::fexp10(14.554 - 0.0423 * x.t) : fm::fexp10(6.226 - 0.0106 * x.t);
      x.lbdas = fmax(fmin(c.LBDAS_MAX, e), c.LBDAS_MIN) * c.TRANS_MP_GAMMAS;
      x.llbdas = fm::flog(x.lbdas);
    } else { x.lbdas = 0.0; x.llbdas = -INFINITY; }
  } else if (x.v[IRS] > 0.) {
    x.llbdas = fmin(fm::flog(c.LBDAS_MAX), fm::flog(c.LBS) + c.LBEXS * (pf.lrho + fm::flog(fmax(x.v[IRS], c.S_RTMIN))));
    x.lbdas = fm::fexp(x.llbdas);
  } else { x.lbdas = 0.0; x.llbdas = -INFINITY; }
  if (x.v[IRG] > 0.) {
    x.llbdag = fm::flog(c.LBG) + c.LBEXG * (pf.lrho + fm::flog(fmax(x.v[IRG], c.G_RTMIN)));
    x.lbdag = fm::fexp(x.llbdag);
  } else { x.lbdag = 0.0; x.llbdag = -INFINITY; }
}

// Heat/vapour term of the freezing and melting rates (fast_rs/fast_rg).
ICE3_HD double heat_term(const Cst &c, const Rates &R, double t, double esat, double rv, double pres)
{
  double e = rv * pres / (c.EPSILO + rv);
  if (c.LEVLIMIT != 0.0) e = fmin(e, esat);
  return R.ka * (c.TT - t) + (R.dv * (c.LVTT + (c.CPV - c.CL) * (t - c.TT)) * (c.ESTT - e) / (c.RV * t));
}

// ICE4_TENDENCIES for one point; see mode_ice4_tendencies.F90 for the order.
ICE3_HD void tendencies(const Cst &c, const double *__restrict__ lut, bool soft, const PointFix &pf,
                        double lvfact, double lsfact, double &cit, double t0, const double vart[NV], Rates &R,
                        double &rainfr, double hl[4], double hi[4], double A[NV], double B[NV])
{
  Pass x;
  x.t = t0;
#pragma unroll
  for (int v = 0; v < NV; ++v) { x.v[v] = vart[v]; A[v] = 0.0; B[v] = 0.0; }
  double *b = R.bu;
  double lt = 0.0, it = 0.0, esw = 0.0, esi = 0.0;
  if (soft) {
    b[B_RVHENI_MR] = b[B_RRHONG_MR] = b[B_RIMLTC_MR] = 0.0;
  } else {
    nucleation(c, true, x.v[ITH], pf.pres, pf.rho, pf.exn, lsfact, x.t, x.v[IRV], cit, b[B_RVHENI_MR]);
    x.v[ITH] += b[B_RVHENI_MR] * lsfact;
    x.t = x.v[ITH] * pf.exn;
    x.v[IRV] -= b[B_RVHENI_MR];
    x.v[IRI] += b[B_RVHENI_MR];
    // RRHONG (mode_ice4_rrhong.F90)
    double r = 0.0;
    if (x.t < c.TT - 35.0 && x.v[IRR] > c.R_RTMIN) {
      r = x.v[IRR];
      if (c.LFEEDBACKT != 0.0) r = fmin(r, fmax(0.0, ((c.TT - 35.0) / pf.exn - x.v[ITH]) / (lsfact - lvfact)));
    }
    b[B_RRHONG_MR] = r;
    x.v[ITH] += r * (lsfact - lvfact);
    x.t = x.v[ITH] * pf.exn;
    x.v[IRR] -= r;
    x.v[IRG] += r;
    // RIMLTC (mode_ice4_rimltc.F90)
    r = 0.0;
    if (x.v[IRI] > 0. && x.t > c.TT) {
      r = x.v[IRI];
      if (c.LFEEDBACKT != 0.0) r = fmin(r, fmax(0.0, (x.v[ITH] - c.TT / pf.exn) / (lsfact - lvfact)));
    }
    b[B_RIMLTC_MR] = r;
    x.v[ITH] -= r * (lsfact - lvfact);
    x.t = x.v[ITH] * pf.exn;
    x.v[IRC] += r;
    x.v[IRI] -= r;
    const double lsv = lsfact - lvfact;
    B[ITH] = b[B_RVHENI_MR] * lsfact + b[B_RRHONG_MR] * lsv - b[B_RIMLTC_MR] * lsv;
    B[IRV] = -b[B_RVHENI_MR];
    B[IRC] = b[B_RIMLTC_MR];
    B[IRR] = -b[B_RRHONG_MR];
    B[IRI] = b[B_RVHENI_MR] - b[B_RIMLTC_MR];
    B[IRG] = b[B_RRHONG_MR];
    // derived fields (mode_ice4_tendencies.F90:303-320)
    lt = fm::flog(x.t);
    it = 1.0 / x.t;
    esi = esat_from(c.ALPI, c.BETAI, c.GAMI, it, lt);
    esw = esat_from(c.ALPW, c.BETAW, c.GAMW, it, lt);
    R.ssi = x.v[IRV] * (pf.pres - esi) / (c.EPSILO * esi) - 1.0;
    R.ka = 2.38e-2 + 7.1e-5 * (x.t - c.TT);
    R.dv = 2.11e-5 * fm::fexp(1.94 * (lt - fm::flog(c.TT))) * (c.P00 / pf.pres);
    R.ai = sq(c.LSTT + (c.CPV - c.CI) * (x.t - c.TT)) / (R.ka * c.RV * x.t * x.t) + (c.RV * x.t) / (R.dv * esi);
    R.cj = c.SCFAC * fm::fexp(0.3 * pf.lrho) / sqrt(1.718e-5 + 4.9e-8 * (x.t - c.TT));
  }
  const double zrainfr = compute_pdf(c, true, pf.rcrautc, x.v[IRC], x.v[IRI], pf.cf, x.t, pf.sigma_rc, hl, hi);
  const bool llrfr = (int)c.SUBG_RC_RR_ACCR == 1 || (int)c.SUBG_RR_EVAP == 2;
  if (llrfr) {
    rainfr = fmax(rainfr, zrainfr);
    if ((x.v[IRR] > c.R_RTMIN || x.v[IRS] > c.S_RTMIN || x.v[IRG] > c.G_RTMIN) && rainfr == 0.) rainfr = 1.;
  } else {
    rainfr = 1.;
  }
  slopes(c, pf, x);
  const double t = x.t, rho = pf.rho;
  const double *v = x.v;

  // ---- ICE4_SLOW (mode_ice4_slow.F90) ----
  if (t < c.TT - 35.0 && v[IRC] > c.C_RTMIN) {
    if (!soft) b[B_RCHONI] = fmin(1000., c.HON * rho * v[IRC] * fm::fexp(c.ALPHA3 * (t - c.TT) - c.BETA3));
  } else b[B_RCHONI] = 0.0;
  if (v[IRV] > c.V_RTMIN && v[IRS] > c.S_RTMIN) {
    if (!soft)
      b[B_RVDEPS] = (R.ssi / (rho * R.ai)) *
                    (c.O0DEPS * fm::fexp(c.EX0DEPS * x.llbdas) + c.O1DEPS * R.cj * fm::fexp(c.EX1DEPS * x.llbdas));
  } else b[B_RVDEPS] = 0.0;
  if (v[IRI] > c.I_RTMIN && v[IRS] > c.S_RTMIN) {
    if (!soft)
      b[B_RIAGGS] = c.FIAGGS * fm::fexp(c.COLEXIS * (t - c.TT) + c.EXIAGGS * x.llbdas) * v[IRI] * pf.rho_mcexvt;
  } else b[B_RIAGGS] = 0.0;
  if (hi[2] > c.I_RTMIN) {
    if (!soft) {
      const double criauti = fmin(c.CRIAUTI, fm::fexp10(c.ACRIAUTI * (t - c.TT) + c.BCRIAUTI));
      b[B_RIAUTS] = c.TIMAUTI * fm::fexp(c.TEXAUTI * (t - c.TT)) * fmax(hi[2] - criauti * hi[0], 0.0);
    }
  } else b[B_RIAUTS] = 0.0;
  if (v[IRV] > c.V_RTMIN && v[IRG] > c.G_RTMIN) {
    if (!soft)
      b[B_RVDEPG] = (R.ssi / (rho * R.ai)) *
                    (c.O0DEPG * fm::fexp(c.EX0DEPG * x.llbdag) + c.O1DEPG * R.cj * fm::fexp(c.EX1DEPG * x.llbdag));
  } else b[B_RVDEPG] = 0.0;

  // ---- ICE4_WARM (mode_ice4_warm.F90), SUBG_RC_RR_ACCR = SUBG_RR_EVAP = NONE ----
  if (c.LWARM != 0.0) {
    if (hl[2] > c.C_RTMIN && hl[0] > 0.0) {
      if (!soft) b[B_RCAUTR] = c.TIMAUTC * fmax(hl[2] - hl[0] * pf.rcrautc, 0.0);
    } else b[B_RCAUTR] = 0.0;
    if (v[IRC] > c.C_RTMIN && v[IRR] > c.R_RTMIN) {
      if (!soft) b[B_RCACCR] = c.FCACCR * v[IRC] * fm::fexp(c.EXCACCR * x.llbdar) * pf.rho_mcexvt;
    } else b[B_RCACCR] = 0.0;
    if (v[IRR] > c.R_RTMIN && v[IRC] <= c.C_RTMIN) {
      if (!soft) {
        const double usw = 1. - v[IRV] * (pf.pres - esw) / (c.EPSILO * esw);
        const double av = sq(c.LVTT + (c.CPV - c.CL) * (t - c.TT)) / (R.ka * c.RV * t * t) + (c.RV * t) / (R.dv * esw);
        b[B_RREVAV] = (fmax(0., usw) / (rho * av)) *
                      (c.O0EVAR * fm::fexp(c.EX0EVAR * x.llbdar) + c.O1EVAR * R.cj * fm::fexp(c.EX1EVAR * x.llbdar));
      }
    } else b[B_RREVAV] = 0.0;
  } else {
    b[B_RCAUTR] = b[B_RCACCR] = b[B_RREVAV] = 0.0;
  }

  // ---- ICE4_FAST_RS (mode_ice4_fast_rs.F90) ----
  double *rs = R.rs;
  double freez;
  if (v[IRS] > c.S_RTMIN) {
    if (!soft) {
      const double den = 1.0 / (rho * (c.LMTT - c.CL * (c.TT - t)));
      rs[RS_FREEZ1] = heat_term(c, R, t, esi, v[IRV], pf.pres) *
                      (c.O0DEPS * fm::fexp(c.EX0DEPS * x.llbdas) + c.O1DEPS * R.cj * fm::fexp(c.EX1DEPS * x.llbdas)) * den;
      rs[RS_FREEZ2] = (rho * (c.LMTT + (c.CI - c.CL) * (c.TT - t))) * den;
    }
    freez = fmax(0., fmax(0., rs[RS_FREEZ1] + rs[RS_FREEZ2] * b[B_RIAGGS]) - b[B_RIAGGS]);
  } else {
    rs[RS_FREEZ1] = rs[RS_FREEZ2] = 0.0;
    freez = 0.0;
  }
  const bool grim = v[IRC] > c.C_RTMIN && v[IRS] > c.S_RTMIN;
  if (!grim) rs[RS_RCRIMS] = rs[RS_RCRIMSS] = rs[RS_RSRIMCG] = 0.0;
  if (!soft && grim) {
    int i;
    const double fr = lut_index(x.llbdas, c.NGAMINC, c.RIMINTP1, c.RIMINTP2, i);
    const double zw1 = lut1d(lut + O_RIM1, i, fr);
    const double zw2 = lut1d(lut + O_RIM2, i, fr);
    const double zw3 = lut1d(lut + O_RIM4, i, fr);
    rs[RS_RCRIMSS] = c.CRIMSS * zw1 * v[IRC] * fm::fexp(c.EXCRIMSS * x.llbdas) * pf.rho_mcexvt;
    rs[RS_RCRIMS] = c.CRIMSG * v[IRC] * fm::fexp(c.EXCRIMSG * x.llbdas) * pf.rho_mcexvt;
    if ((int)c.SNOW_RIMING == 0) {
      const double zzw = rs[RS_RCRIMS] - rs[RS_RCRIMSS];
      const double r = c.SRIMCG * fm::fexp(c.EXSRIMCG * x.llbdas) * (1.0 - zw2);
      rs[RS_RSRIMCG] = zzw * r / fmax(1.e-20, c.SRIMCG3 * c.SRIMCG2 * fm::fexp(c.EXSRIMCG2 * x.llbdas) * (1. - zw3) -
                                                 c.SRIMCG3 * r);
    } else rs[RS_RSRIMCG] = 0.0;
  }
  if (grim && t < c.TT) {
    b[B_RCRIMSS] = fmin(freez, rs[RS_RCRIMSS]);
    freez = fmax(0., freez - b[B_RCRIMSS]);
    const double zzw0 = fmin(1., freez / fmax(1.e-20, rs[RS_RCRIMS] - b[B_RCRIMSS]));
    b[B_RCRIMSG] = zzw0 * fmax(0., rs[RS_RCRIMS] - b[B_RCRIMSS]);
    freez = fmax(0., freez - b[B_RCRIMSG]);
    b[B_RSRIMCG] = zzw0 * rs[RS_RSRIMCG] * (signbit(b[B_RCRIMSG]) ? 0.0 : 1.0);
    b[B_RCRIMSG] = fmax(0., b[B_RCRIMSG]);
  } else {
    b[B_RCRIMSS] = b[B_RCRIMSG] = b[B_RSRIMCG] = 0.0;
  }
  const bool gacc = v[IRR] > c.R_RTMIN && v[IRS] > c.S_RTMIN;
  if (!gacc) rs[RS_RRACCS] = rs[RS_RRACCSS] = rs[RS_RSACCRG] = 0.0;
  if (!soft) {
    rs[RS_RRACCS] = rs[RS_RRACCSS] = rs[RS_RSACCRG] = 0.0;
    if (gacc) {
      int i1, i2;
      const double f1 = lut_index(x.llbdas, c.NACCLBDAS, c.ACCINTP1S, c.ACCINTP2S, i1);
      const double f2 = lut_index(x.llbdar, c.NACCLBDAR, c.ACCINTP1R, c.ACCINTP2R, i2);
      const double zw1 = lut2d(lut + O_RACCSS, ICE3GB_NACCLBDAR, i1, f1, i2, f2);
      const double zw2 = lut2d(lut + O_RACCS, ICE3GB_NACCLBDAR, i1, f1, i2, f2);
      const double zw3 = lut2d(lut + O_SACCRG, ICE3GB_NACCLBDAS, i2, f2, i1, f1);
      const double ilr = 1.0 / x.lbdar, ils = 1.0 / x.lbdas;
      const double zzw = c.FRACCSS * fm::fexp(c.CXS * x.llbdas) * pf.rho_mcexvt1 *
                         (c.LBRACCS1 * ils * ils + c.LBRACCS2 * ils * ilr + c.LBRACCS3 * ilr * ilr) * sq(sq(ilr));
      rs[RS_RRACCSS] = zw1 * zzw;
      rs[RS_RRACCS] = zw2 * zzw;
      rs[RS_RSACCRG] = c.FSACCRG * zw3 * fm::fexp((c.CXS - c.BS) * x.llbdas) * pf.rho_mcexvt1 *
                       (c.LBSACCR1 * ilr * ilr + c.LBSACCR2 * ilr * ils + c.LBSACCR3 * ils * ils) * ilr;
    }
  }
  if (gacc && t < c.TT) {
    b[B_RRACCSS] = fmin(freez, rs[RS_RRACCSS]);
    freez = fmax(0., freez - b[B_RRACCSS]);
    const double zzw = fmin(1., freez / fmax(1.e-20, rs[RS_RRACCS] - b[B_RRACCSS]));
    b[B_RRACCSG] = zzw * fmax(0., rs[RS_RRACCS] - b[B_RRACCSS]);
    freez = fmax(0., freez - b[B_RRACCSG]);
    b[B_RSACCRG] = zzw * rs[RS_RSACCRG] * (signbit(b[B_RRACCSG]) ? 0.0 : 1.0);
    b[B_RRACCSG] = fmax(0., b[B_RRACCSG]);
  } else {
    b[B_RRACCSS] = b[B_RRACCSG] = b[B_RSACCRG] = 0.0;
  }
  if (v[IRS] > c.S_RTMIN && t > c.TT) {
    if (!soft) {
      const double h = heat_term(c, R, t, esw, v[IRV], pf.pres);
      b[B_RSMLTG] = c.FSCVMG * fmax(0., (-h * (c.O0DEPS * fm::fexp(c.EX0DEPS * x.llbdas) +
                                               c.O1DEPS * R.cj * fm::fexp(c.EX1DEPS * x.llbdas)) -
                                         (rs[RS_RCRIMS] + rs[RS_RRACCS]) * (rho * c.CL * (c.TT - t))) /
                                            (rho * c.LMTT));
      b[B_RCMLTSR] = rs[RS_RCRIMS];
    }
  } else {
    b[B_RSMLTG] = b[B_RCMLTSR] = 0.0;
  }

  // ---- ICE4_FAST_RG (mode_ice4_fast_rg.F90, KRR = 6) ----
  double *rg = R.rg;
  if (v[IRI] > c.I_RTMIN && v[IRR] > c.R_RTMIN) {
    if (!soft) {
      b[B_RICFRRG] = c.ICFRR * v[IRI] * fm::fexp(c.EXICFRR * x.llbdar) * pf.rho_mcexvt;
      b[B_RRCFRIG] = c.RCFRI * cit * fm::fexp(c.EXRCFRI * x.llbdar) * pf.rho_mcexvt1;
      if (c.LCRFLIMIT != 0.0) {
        const double zw = fmax(0., fmin(1., (b[B_RICFRRG] * c.CI + b[B_RRCFRIG] * c.CL) * (c.TT - t) /
                                                fmax(1.e-20, c.LVTT * b[B_RRCFRIG])));
        b[B_RRCFRIG] = zw * b[B_RRCFRIG];
        b[B_RICFRR] = (1. - zw) * b[B_RICFRRG];
        b[B_RICFRRG] = zw * b[B_RICFRRG];
      } else b[B_RICFRR] = 0.0;
    }
  } else {
    b[B_RICFRRG] = b[B_RRCFRIG] = b[B_RICFRR] = 0.0;
  }
  const double base_g = fm::fexp((c.CXG - c.DG - 2.) * x.llbdag) * pf.rho_mcexvt;
  if (v[IRG] > c.G_RTMIN && v[IRC] > c.C_RTMIN) {
    if (!soft) rg[RG_RCDRYG] = c.FCDRYG * v[IRC] * base_g;
  } else rg[RG_RCDRYG] = 0.0;
  if (v[IRG] > c.G_RTMIN && v[IRI] > c.I_RTMIN) {
    if (!soft) {
      const double e = fm::fexp(c.COLEXIG * (t - c.TT));
      rg[RG_RIDRYG] = c.FIDRYG * e * v[IRI] * base_g;
      rg[RG_RIWETG] = rg[RG_RIDRYG] / (c.COLIG * e);
    }
  } else rg[RG_RIDRYG] = rg[RG_RIWETG] = 0.0;
  const bool gdry_s = v[IRS] > c.S_RTMIN && v[IRG] > c.G_RTMIN;
  if (!gdry_s) rg[RG_RSDRYG] = rg[RG_RSWETG] = 0.0;
  if (!soft && gdry_s) {
    int i1, i2;
    const double f1 = lut_index(x.llbdag, c.NDRYLBDAG, c.DRYINTP1G, c.DRYINTP2G, i1);
    const double f2 = lut_index(x.llbdas, c.NDRYLBDAS, c.DRYINTP1S, c.DRYINTP2S, i2);
    const double zw = lut2d(lut + O_SDRYG, ICE3GB_NDRYLBDAS, i1, f1, i2, f2);
    const double ilg = 1.0 / x.lbdag, ils = 1.0 / x.lbdas;
    rg[RG_RSWETG] = c.FSDRYG * zw / c.COLSG * fm::fexp((c.CXS - c.BS) * x.llbdas + c.CXG * x.llbdag) * pf.rho_mcexvt1 *
                    (c.LBSDRYG1 * ilg * ilg + c.LBSDRYG2 * ilg * ils + c.LBSDRYG3 * ils * ils);
    rg[RG_RSDRYG] = rg[RG_RSWETG] * c.COLSG * fm::fexp(c.COLEXSG * (t - c.TT));
  }
  const bool gdry_r = v[IRR] > c.R_RTMIN && v[IRG] > c.G_RTMIN;
  if (!gdry_r) rg[RG_RRDRYG] = 0.0;
  if (!soft && gdry_r) {
    int i1, i2;
    const double f1 = lut_index(x.llbdag, c.NDRYLBDAG, c.DRYINTP1G, c.DRYINTP2G, i1);
    const double f2 = lut_index(x.llbdar, c.NDRYLBDAR, c.DRYINTP1R, c.DRYINTP2R, i2);
    const double zw = lut2d(lut + O_RDRYG, ICE3GB_NDRYLBDAR, i1, f1, i2, f2);
    const double ilg = 1.0 / x.lbdag, ilr = 1.0 / x.lbdar;
    rg[RG_RRDRYG] = c.FRDRYG * zw * sq(sq(ilr)) * fm::fexp(c.CXG * x.llbdag) * pf.rho_mcexvt1 *
                    (c.LBRDRYG1 * ilg * ilg + c.LBRDRYG2 * ilg * ilr + c.LBRDRYG3 * ilr * ilr);
  }
  const double rdryg_init = rg[RG_RCDRYG] + rg[RG_RIDRYG] + rg[RG_RSDRYG] + rg[RG_RRDRYG];
  double rwetg_init = 0.0;
  bool ldwetg = false, lldryg = false;
  if (v[IRG] > c.G_RTMIN) {
    if (!soft) {
      const double den = 1.0 / (rho * (c.LMTT - c.CL * (c.TT - t)));
      rg[RG_FREEZ1] = heat_term(c, R, t, esi, v[IRV], pf.pres) *
                      (c.O0DEPG * fm::fexp(c.EX0DEPG * x.llbdag) + c.O1DEPG * R.cj * fm::fexp(c.EX1DEPG * x.llbdag)) * den;
      rg[RG_FREEZ2] = (rho * (c.LMTT + (c.CI - c.CL) * (c.TT - t))) * den;
    }
    const double is = rg[RG_RIWETG] + rg[RG_RSWETG];
    rwetg_init = fmax(is, fmax(0., rg[RG_FREEZ1] + rg[RG_FREEZ2] * is));
    const double wet = fmax(0., rwetg_init - rg[RG_RIWETG] - rg[RG_RSWETG]);
    const double dry = fmax(0., rdryg_init - rg[RG_RIDRYG] - rg[RG_RSDRYG]);
    ldwetg = wet <= dry;
    if (c.LNULLWETG != 0.0) ldwetg = ldwetg && rdryg_init > 0.;
    else ldwetg = ldwetg && rwetg_init > 0.;
    if (c.LWETGPOST == 0.0) ldwetg = ldwetg && t < c.TT;
    lldryg = t < c.TT && rdryg_init > 1.e-20 && wet > dry;
  } else {
    rg[RG_FREEZ1] = rg[RG_FREEZ2] = 0.0;
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
  if (v[IRG] > c.G_RTMIN && t > c.TT) {
    if (!soft) {
      const double h = heat_term(c, R, t, esw, v[IRV], pf.pres);
      b[B_RGMLTR] = fmax(0., (-h * (c.O0DEPG * fm::fexp(c.EX0DEPG * x.llbdag) + c.O1DEPG * R.cj * fm::fexp(c.EX1DEPG * x.llbdag)) -
                              (rg[RG_RCDRYG] + rg[RG_RRDRYG]) * (rho * c.CL * (c.TT - t))) /
                                 (rho * c.LMTT));
    }
  } else b[B_RGMLTR] = 0.0;

  // ---- ICE4_FAST_RI (mode_ice4_fast_ri.F90) ----
  if (R.ssi > 0. && v[IRC] > c.C_RTMIN && v[IRI] > c.I_RTMIN && cit > 1.e-20) {
    if (!soft) {
      const double l = fmin(1.e8, c.LBI * fm::fexp(c.LBEXI * fm::flog(rho * v[IRI] / cit)));
      b[B_RCBERI] = (R.ssi / (rho * R.ai)) * cit * (c.O0DEPI / l + c.O2DEPI * R.cj * R.cj * fm::fexp(-(c.DI + 2.0) * fm::flog(l)));
    }
  } else b[B_RCBERI] = 0.0;

  // ---- aggregation (mode_ice4_tendencies.F90:606-717, KRR = 6) ----
  const double lsv = lsfact - lvfact;
  A[ITH] = b[B_RVDEPG] * lsfact + b[B_RCHONI] * lsv + b[B_RVDEPS] * lsfact - b[B_RREVAV] * lvfact +
           b[B_RCRIMSS] * lsv + b[B_RCRIMSG] * lsv + b[B_RRACCSS] * lsv + b[B_RRACCSG] * lsv +
           (b[B_RRCFRIG] - b[B_RICFRR]) * lsv + (b[B_RCWETG] + b[B_RRWETG]) * lsv +
           (b[B_RCDRYG] + b[B_RRDRYG]) * lsv - b[B_RGMLTR] * lsv + b[B_RCBERI] * lsv;
  A[IRV] = -b[B_RVDEPG] - b[B_RVDEPS] + b[B_RREVAV];
  A[IRC] = -b[B_RCHONI] - b[B_RCAUTR] - b[B_RCACCR] - b[B_RCRIMSS] - b[B_RCRIMSG] - b[B_RCMLTSR] - b[B_RCWETG] -
           b[B_RCDRYG] - b[B_RCBERI];
  A[IRR] = b[B_RCAUTR] + b[B_RCACCR] - b[B_RREVAV] - b[B_RRACCSS] - b[B_RRACCSG] + b[B_RCMLTSR] - b[B_RRCFRIG] +
           b[B_RICFRR] - b[B_RRWETG] - b[B_RRDRYG] + b[B_RGMLTR];
  A[IRI] = b[B_RCHONI] - b[B_RIAGGS] - b[B_RIAUTS] - b[B_RICFRRG] - b[B_RICFRR] - b[B_RIWETG] - b[B_RIDRYG] +
           b[B_RCBERI];
  A[IRS] = b[B_RVDEPS] + b[B_RIAGGS] + b[B_RIAUTS] + b[B_RCRIMSS] - b[B_RSRIMCG] + b[B_RRACCSS] - b[B_RSACCRG] -
           b[B_RSMLTG] - b[B_RSWETG] - b[B_RSDRYG];
  A[IRG] = b[B_RVDEPG] + b[B_RCRIMSG] + b[B_RSRIMCG] + b[B_RRACCSG] + b[B_RSACCRG] + b[B_RSMLTG] + b[B_RICFRRG] +
           b[B_RRCFRIG] + b[B_RCWETG] + b[B_RIWETG] + b[B_RSWETG] + b[B_RRWETG] + b[B_RCDRYG] + b[B_RIDRYG] +
           b[B_RSDRYG] + b[B_RRDRYG] - b[B_RGMLTR];
}

// ICE4_STEPPING for one micro point (mode_ice4_stepping.F90:139-518).
// Returns the pass key (outer << 16 | inner-of-last-outer), 0 if capped.
ICE3_HD unsigned int stepping(const Cst &c, const double *__restrict__ lut, const PointFix &pf, double dt,
                              int max_passes, double vart[NV], const double ext[NV], double &cit,
                              double &rainfr, double &rrevav, double hl[4], double hi[4], bool &capped)
{
  const double rsmin[NV] = {0.0, c.V_RTMIN, c.C_RTMIN, c.R_RTMIN, c.I_RTMIN, c.S_RTMIN, c.G_RTMIN};
  Rates R;
#pragma unroll
  for (int k = 0; k < NBU; ++k) R.bu[k] = 0.0;
#pragma unroll
  for (int k = 0; k < NRS; ++k) R.rs[k] = 0.0;
#pragma unroll
  for (int k = 0; k < NRG; ++k) R.rg[k] = 0.0;
  R.ssi = R.ka = R.dv = R.ai = R.cj = 0.0;
  double ztime = 0.0;
  int passes = 0, outer = 0, inner = 0;
  rrevav = 0.0;
  capped = false;
  while (ztime < dt) {
    ++outer;
    inner = 0;
    bool llcompute = true, soft = false;
    while (llcompute) {
      if (passes >= max_passes) { capped = true; return 0u; }
      ++passes;
      ++inner;
      const double zsum2 = vart[IRI] + vart[IRS] + vart[IRG];
      const double zdev = (c.CPD + c.CPV * vart[IRV] + c.CL * (vart[IRC] + vart[IRR]) + c.CI * zsum2) * pf.exn;
      const double zzt = vart[ITH] * pf.exn;
      const double izdev = 1.0 / zdev;
      const double lsfact = (c.LSTT + (c.CPV - c.CI) * (zzt - c.TT)) * izdev;
      const double lvfact = (c.LVTT + (c.CPV - c.CL) * (zzt - c.TT)) * izdev;
      double A[NV], B[NV];
      tendencies(c, lut, soft, pf, lvfact, lsfact, cit, zzt, vart, R, rainfr, hl, hi, A, B);
#pragma unroll
      for (int v = 0; v < NV; ++v) A[v] += ext[v];
      double maxtime = dt - ztime;
      if (c.LFEEDBACKT != 0.0) {
        const double zx = c.TT / pf.exn;
        if ((vart[ITH] - zx) * (vart[ITH] + B[ITH] - zx) < 0.) maxtime = 0.;
        if (fabs(A[ITH]) > 1.e-20) {
          const double thr = (zx - B[ITH] - vart[ITH]) / A[ITH];
          if (thr > 0.) maxtime = fmin(maxtime, thr);
        }
      }
#pragma unroll
      for (int v = 1; v < NV; ++v) {
        if (A[v] < -1.e-20 && vart[v] > rsmin[v]) {
          maxtime = fmin(maxtime, -(B[v] + vart[v]) / A[v]);
          maxtime = fmax(maxtime, c.MNH_TINY);
        }
      }
      if (ztime + maxtime >= dt) llcompute = false;
      // State update with separately rounded product and sums (no FMA
      // contraction): after a species is depleted, v + A*t + B leaves a
      // rounding residual, and whether it exceeds XRTMIN decides whether the
      // next pass is taken with a MNH_TINY step (:302-311).  At the 1000/s
      // cap of RCHONI that quantum moves 2.2e-13 kg/kg, so the rounding must
      // follow the un-contracted evaluation of the Fortran (and of the CPU
      // reference) rather than a fused multiply-add.
#pragma unroll
      for (int v = 0; v < NV; ++v) vart[v] = add_rn(add_rn(vart[v], mul_rn(A[v], maxtime)), B[v]);
      if (vart[IRI] <= 0.) cit = 0.;
      ztime += maxtime;
      rrevav = R.bu[B_RREVAV];
      soft = true;
    }
  }
  return ((unsigned)outer << 16) | (unsigned)inner;
}


}  // namespace ice3pt
