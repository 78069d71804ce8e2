// rain_ice_point.cuh — per-grid-point ICE4 physics of the rain_ice kernel
// (nucleation, compute_pdf, the slow/warm/fast processes, ICE4_TENDENCIES and
// ICE4_STEPPING for one point).  Host-and-device code; the kernel in
// rain_ice.cu runs it per lane.
//
// FP64 economy (GB300 issues FP64 at 1/64 of the FP32 rate; an FP64 compare
// costs as much as an FMA, integer work is nearly free):
//  * exp/log/exp10 are the table-driven versions of fastmath.cuh;
//  * threshold tests and clamps run on the IEEE bit patterns (integer pipe),
//    see gtp/pos/dmin/dmax in ice3gb_device.cuh;
//  * what several processes share is computed once per hard pass: the
//    ventilation factors of snow and graupel (deposition, freezing and
//    melting all use O0DEP lbda^EX0DEP + O1DEP cj lbda^EX1DEP), the
//    vapour/heat term of the freezing and melting rates, the reciprocal
//    slopes, ssi/(rho ai), the collision-freezing denominator, and the ice
//    autoconversion threshold that compute_pdf also needs;
//  * soft passes (rates frozen at their hard-pass values) skip the slope
//    parameters, which only the hard-pass rates use;
//  * logs of table constants are computed once per block (Derived).
#pragma once

#include "ice3gb_device.cuh"

namespace ice3pt {

// Threads per block of the rain_ice point kernels (one block per SM: the 16
// warps share one copy of the lookup tables and keep in step, see
// rain_ice_kernel.cuh).
#ifndef ICE3GB_RI_THREADS
#define ICE3GB_RI_THREADS 512
#endif
constexpr int RI_THREADS = ICE3GB_RI_THREADS;
// The tables of Ice3gbLuts staged in shared memory (all but the hail
// kernels, which the NRR = 7 instantiation reads from global memory).
constexpr int LUT_N = 9840;
constexpr int O_RIM1 = 0, O_RIM2 = 80, O_RIM4 = 160, O_RACCSS = 240, O_RACCS = 1840, O_SACCRG = 3440,
              O_RDRYG = 5040, O_SDRYG = 6640;
constexpr int O_SWETH = 9840, O_GWETH = 13040, O_RWETH = 14640, LUT_ALL = 16240;
static_assert(offsetof(Ice3gbLuts, ker_sweth) == sizeof(double) * O_SWETH, "Ice3gbLuts layout");
static_assert(offsetof(Ice3gbLuts, ker_gweth) == sizeof(double) * O_GWETH, "Ice3gbLuts layout");
static_assert(offsetof(Ice3gbLuts, ker_rweth) == sizeof(double) * O_RWETH, "Ice3gbLuts layout");
static_assert(sizeof(Ice3gbLuts) == sizeof(double) * LUT_ALL, "Ice3gbLuts layout");

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
// hail (NRR = 7): the eighth state variable, the graupel -> hail conversion
// and the ICE4_FAST_RH rates (mode_ice4_fast_rh.F90 IRCWETH..IFREEZ2)
constexpr int IRH = NV, NVH = NV + 1;
enum {
  BH_RWETGH, BH_RWETGH_MR, BH_RCWETH, BH_RIWETH, BH_RSWETH, BH_RGWETH, BH_RRWETH, BH_RCDRYH, BH_RIDRYH, BH_RSDRYH,
  BH_RRDRYH, BH_RGDRYH, BH_RDRYHG, BH_RHMLTR, NBH
};
enum { RH_RCWETH, RH_RRWETH, RH_RIDRYH, RH_RIWETH, RH_RSDRYH, RH_RSWETH, RH_RGDRYH, RH_RGWETH, RH_FREEZ1,
       RH_FREEZ2, NRH };
struct HailRates {
  double b[NBH];
  double t[NRH];
};
// OCND2 (separate liquid and ice clouds): the per-point inputs (the TIWMX
// tables, the ice_adjust OCND2 outputs of the state, the level height and the
// cloud droplet concentration of rain_ice.F90:386-435) and the hard-pass
// quantities of ICE4_TENDENCIES it adds (tabulated es_i, collision factors,
// ICE4_FAST_RI_RS's RVDEPI / RILARS).
struct OcndPt {
  const double *tw;
  double ssio, ssiu, ifr, icldfr, zzz, conc;
};
struct OcndRates {
  double esi, colf, acrf, rvdepi, rilars;
};

// Constants derived from the table once per block (kept in shared memory).
struct Derived {
  double lLBR, lLBS, lLBG, lLBDAS_MAX, lTT;   // logs of table constants
  double nu20_eb2;                            // NU20 * exp(-BETA2)
  double irv;                                 // 1/RV
  // exponent identities of the table, tested once so that a power already
  // computed is reused (AROME: EX0DEPS = 0, EXCRIMSG = EXCRIMSS,
  // EXSRIMCG2 = 2 EXSRIMCG, CXS = 1, EXICFRR = EXCACCR, EX0EVAR = -2)
  int ex0deps_zero, ex0depg_zero, crims_same, srimcg2_twice, cxs_one, icfrr_caccr, ex0evar_m2;
  // the option switches of the table as integers, so that no lane converts
  // or compares the FP64 table entries
  int aucv_rc, aucv_ri, prpdf, accr, evap, snow_riming;
  int lwarm, lfeedbackt, lsnow_t, lcrflimit, llrfr;
  // differences of table constants, formed once per block (the same IEEE
  // values as formed in place)
  double cpv_cl, cpv_ci, ci_cl, tt_m35, tt_m5, tt_m2;
  double cxs_bs, cxg_dg2, cxh_dh2, cxg_bg, srimcg32;
};

ICE3_HD void make_derived(const Cst &c, Derived &d)
{
  d.lLBR = fm::flog(c.LBR);
  d.lLBS = fm::flog(c.LBS);
  d.lLBG = fm::flog(c.LBG);
  d.lLBDAS_MAX = fm::flog(c.LBDAS_MAX);
  d.lTT = fm::flog(c.TT);
  d.nu20_eb2 = c.NU20 * fm::fexp(-c.BETA2);
  d.irv = 1.0 / c.RV;
  d.ex0deps_zero = c.EX0DEPS == 0.0;
  d.ex0depg_zero = c.EX0DEPG == 0.0;
  d.crims_same = c.EXCRIMSG == c.EXCRIMSS;
  d.srimcg2_twice = c.EXSRIMCG2 == 2.0 * c.EXSRIMCG;
  d.cxs_one = c.CXS == 1.0;
  d.icfrr_caccr = c.EXICFRR == c.EXCACCR;
  d.ex0evar_m2 = c.EX0EVAR == -2.0;
  d.aucv_rc = (int)c.SUBG_AUCV_RC;
  d.aucv_ri = (int)c.SUBG_AUCV_RI;
  d.prpdf = (int)c.SUBG_PR_PDF;
  d.accr = (int)c.SUBG_RC_RR_ACCR;
  d.evap = (int)c.SUBG_RR_EVAP;
  d.snow_riming = (int)c.SNOW_RIMING;
  d.lwarm = c.LWARM != 0.0;
  d.lfeedbackt = c.LFEEDBACKT != 0.0;
  d.lsnow_t = c.LSNOW_T != 0.0;
  d.lcrflimit = c.LCRFLIMIT != 0.0;
  d.llrfr = d.accr == 1 || d.evap == 2;
  d.cpv_cl = c.CPV - c.CL;
  d.cpv_ci = c.CPV - c.CI;
  d.ci_cl = c.CI - c.CL;
  d.tt_m35 = c.TT - 35.0;
  d.tt_m5 = c.TT - 5.0;
  d.tt_m2 = c.TT - 2.0;
  d.cxs_bs = c.CXS - c.BS;
  d.cxg_dg2 = c.CXG - c.DG - 2.;
  d.cxh_dh2 = c.CXH - c.DH - 2.0;
  d.cxg_bg = c.CXG - c.BG;
  d.srimcg32 = c.SRIMCG3 * c.SRIMCG2;
}

// Rates that persist between the hard pass and the following soft passes
// (Fortran ZBU_INST, ZRS_TEND, ZRG_TEND, ZSSI).
struct Rates {
  double bu[NBU];
  double rs[NRS];
  double rg[NRG];
  double ssi;
};

// Per-point constants over the whole step.
struct PointFix {
  double rho, lrho, pres, exn, cf, sigma_rc;
  double rho_mcexvt;    // rho**(-CEXVT)
  double rho_mcexvt1;   // rho**(-CEXVT-1)
  double rcrautc;       // CRIAUTC / rho
  double zx;            // TT / exn (IEEE division: where th stops at the T = TT limit)
};

ICE3_HD double esat_from(double alp, double beta, double gam, double it, double lt)
{
  return fm::fexp(alp - beta * it - gam * lt);
}

// The OCND2 branch of ICE4_NUCLEATION (ice4_nucleation.func.h:127-136): the
// concentration from REDIN, AM3, the height and the ice cloud fraction; no
// vapour is taken (RVHENI = 0).
ICE3_HD void nucleation_ocnd2(const Cst &c, const OcndPt &o, double t, double rvt, double &cit, double &rvheni)
{
  rvheni = 0.0;
  if (!(ltp(t, c.TT) && gtp(rvt, c.V_RTMIN))) return;
  const double redin = tiwmx_at(o.tw + TW_REDIN * kTiwmxN, t);
  const double am3 = tiwmx_at(o.tw + TW_AM3 * kTiwmxN, dmax(c.FRMIN27, t));
  const double h = (20000. - dmin(20000., o.zzz)) * (1.0 / 20000.);
  const double zzw = dmin(redin * dmax(0.1, (h * h) * (h * h)) * am3 * (0.0001 + 0.9999 * o.icldfr), 50.e3);
  cit = dmax(zzw + cit, cit);
}

// The level heights and cloud droplet concentrations of one column for OCND2
// (rain_ice.F90:386-435): the height is the sum of dzz from the last level
// down to the level minus half its thickness (with k = 0 at the surface the
// last level is the top), the concentration the land / sea / town blend or
// the pressure form of XFRMIN(26).
ICE3_HD void ocnd2_column(const Cst &c, const Ice3gbRainIceFields &f, long nij, int nk, long col, double *zzz,
                          double *conc)
{
  double zsum = 0.0;
  for (int k = nk - 1; k >= 0; --k) {
    const long p = (long)k * nij + col;
    const double dz = f.dzz[p];
    zsum = zsum + dz;
    zzz[p] = zsum - dz * 0.5;
  }
  const bool st = f.sea && f.town;
  const double sea = st ? f.sea[col] : 0.0, town = st ? f.town[col] : 0.0;
  const double top = zzz[(long)(nk - 1) * nij + col];
  for (int k = 0; k < nk; ++k) {
    const long p = (long)k * nij + col;
    double cc = c.CONC_LAND;
    if (st && c.FRMIN26 < 0.001) cc = (1. - town) * (sea * c.CONC_SEA + (1. - sea) * c.CONC_LAND) + town * c.CONC_URBAN;
    if (c.FRMIN26 > 0.001) {
      cc = c.FRMIN26 * f.pabs[p] / c.P00;
      if (c.FRMIN22 > 0.001 && st) {
        const double tmp = dmax(0., dmin(1., (zzz[p] - top) / dmax(0.01, c.FRMIN29 - top)));
        cc = cc * (c.FRMIN22 * (sea * c.FRMIN30 + (1. - sea)) * (1. - tmp) + tmp);
      }
    }
    conc[p] = cc;
  }
}

// x == 0 or -0, on the bit pattern.
ICE3_HD bool zerod(double x) { return (opaque_bits(x) << 1) == 0; }

// The T-dependent terms of a hard pass that nucleation computes and the
// rates of the same pass reuse while T keeps its bit pattern (no HENI,
// RRHONG or RIMLTC change in between): log T, 1/T, es_w and es_i.
struct TTerms {
  double t, lt, it, esw, esi;
  bool set, esw_set;   // esw only where the nucleation needed it
};

// ICE4_NUCLEATION (micro/ice4_nucleation.func.h:69-144, LOCND2 = .FALSE.);
// zx = TT/exn (IEEE division).
ICE3_HD void nucleation(const Cst &c, const Derived &d, double tht, double pabst, double rhodref, double zx,
                        double lsfact, double t, double rvt, double &cit, double &rvheni, TTerms *tt = nullptr)
{
  rvheni = 0.0;
  if (!(ltp(t, c.TT) && gtp(rvt, c.V_RTMIN))) return;
  const double lt = fm::flog(t), it = fm::frcp(t);
  double zzw = esat_from(c.ALPI, c.BETAI, c.GAMI, it, lt);
  if (tt) { tt->t = t; tt->lt = lt; tt->it = it; tt->esi = zzw; tt->set = true; tt->esw_set = false; }
  zzw = dmin(pabst * 0.5, zzw);
  double zssi = fm::fdiv(rvt * (pabst - zzw), c.EPSILO * zzw) - 1.0;
  // Not supersaturated over ice: the MIN with the water term below is not
  // positive either, no crystal nucleates, and with cit >= 0 the rest leaves
  // rvheni = 0 and cit as they are (zzw = MIN(-cit, 5e4) <= 0): es_w is not
  // needed.  (A negative cit goes the full way: it is reset to 0 there.)
  if (!pos(zssi) && !negd(cit)) return;
  double zusw = esat_from(c.ALPW, c.BETAW, c.GAMW, it, lt);
  if (tt) { tt->esw = zusw; tt->esw_set = true; }
  zusw = dmin(pabst * 0.5, zusw);
  zusw = fm::fdiv(zusw * (pabst - zzw), zzw * (pabst - zusw)) - 1.0;
  zssi = dmin(zssi, zusw);
  zzw = 0.0;
  if (ltp(t, d.tt_m5) && pos(zssi)) {
    zzw = c.NU20 * fm::fexp(c.ALPHA2 * zssi - c.BETA2);
  } else if (!gtp(t, d.tt_m2) && !ltp(t, d.tt_m5) && pos(zssi)) {
    zzw = dmax(d.nu20_eb2, c.NU10 * fm::fexp(-c.BETA1 * (t - c.TT) + c.ALPHA1 * fm::flog(fm::fdiv(zssi, zusw))));
  }
  zzw = dmin(zzw - cit, 50.e3);
  rvheni = dmin(rvt, fm::fdiv(pmax0(zzw) * c.MNU0, rhodref));
  if (d.lfeedbackt) {
    // w = MIN(rvheni, MAX(0, (TT/exn - th) / lsfact)) / MAX(rvheni, 1e-20)
    // with IEEE divisions, as the Fortran: the limit puts th exactly on
    // TT/exn, and the next T < TT test must see the same rounding.  Where
    // the limit cannot bind the quotient is not formed: w = 0 for rvheni = +0
    // (0 / 1e-20), w = 1 for rvheni > 1e-20 (rvheni / rvheni).
    const double num = zx - tht;
    double w;
    if (opaque_bits(rvheni) == 0) w = 0.0;
    else if (gtp(rvheni, 1.e-20) && quot_above(num, lsfact, rvheni)) w = 1.0;
    else w = dmin(rvheni, pmax0(num / lsfact)) / dmax(rvheni, 1.e-20);
    rvheni *= w;
    zzw *= w;
  }
  cit = dmax(zzw + cit, cit);
}

// ICE4_COMPUTE_PDF (micro/mode_ice4_compute_pdf.F90), one point; returns RF.
// `criauti` receives MIN(CRIAUTI, 10**(ACRIAUTI (T-TT) + BCRIAUTI)), which
// the ice autoconversion of the same pass uses too.
ICE3_HD double compute_pdf(const Cst &c, const Derived &d, double rcrautc, double rct, double rit, double cf,
                           double t, double sigma_rc, double hl[4], double hi[4], double &criauti, bool soft = false)
{
  const int aucv_rc = d.aucv_rc, aucv_ri = d.aucv_ri, prpdf = d.prpdf;
  double hcf = 0, lcf = 0, hrc = 0, lrc = 0;
  if (aucv_rc == 0) {
    if (gtd(rct, rcrautc)) { hcf = 1.0; hrc = rct; }
    else if (gtp(rct, c.C_RTMIN)) { lcf = 1.0; lrc = rct; }
  } else if (aucv_rc == 3) {
    if (pos(cf) && gtd(rct, rcrautc * cf)) { hcf = cf; hrc = rct; }
    else if (pos(cf) && gtp(rct, c.C_RTMIN)) { lcf = cf; lrc = rct; }
  } else if (aucv_rc == 2) {
    const double sum = hl[3] + hl[2];
    hcf = hl[0]; lcf = hl[1];
    if (gtp(sum, 1.e-20)) { lrc = hl[3] * rct / sum; hrc = hl[2] * rct / sum; }
  } else if (aucv_rc == 1 && prpdf == 0) {
    if (gtd(rct, rcrautc + sigma_rc)) {
      hcf = 1.0; hrc = rct;
    } else if (gtd(rct, rcrautc - sigma_rc)) {
      const double inv2s = fm::frcp(2.0 * sigma_rc);
      hcf = (rct + sigma_rc - rcrautc) * inv2s;
      lcf = pmax0(cf - hcf);
      hrc = (rct + sigma_rc - rcrautc) * (rct + sigma_rc + rcrautc) * (0.5 * inv2s);
      lrc = pmax0(rct - hrc);
    } else if (gtp(rct, c.C_RTMIN) && pos(cf)) {
      lcf = cf; lrc = rct;
    }
  } else if (aucv_rc == 1) {
    const double coeff = (prpdf == 1 || prpdf == 2) ? 2.0 : (prpdf == 3 ? 3.0 : 4.0);
    const double rcmax = (pos(rct) && pos(cf)) ? coeff * rct / cf : 0.0;
    double lloc = 0.0, hloc = 0.0;
    const bool ok = pos(rct) && pos(cf) && gtd(rcmax, rcrautc);
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
      if (!gtd(rct, a * cf) && ok) {
        lloc = (m * m * m - 12.0 * m * a * a + 8.0 * a * a * a) / (6.0 * m * m - 24.0 * m * a + 12.0 * a * a);
        hloc = (m + 2.0 * a) / 3.0;
      } else if (ok) {
        lloc = (2.0 / 3.0) * a;
        hloc = (3.0 * m * m * m - 8.0 * a * a * a) / (6.0 * m * m - 12.0 * a * a);
      }
    }
    if (ok) {
      lcf = cf * (hloc - (rct / cf)) / (hloc - lloc);
      hcf = pmax0(cf - lcf);
      lrc = lloc * lcf;
      hrc = pmax0(rct - lrc);
    } else if (pos(rct) && pos(cf) && !gtd(rcmax, rcrautc)) {
      lcf = cf; lrc = rct;
    }
  }
  hl[0] = hcf; hl[1] = lcf; hl[2] = hrc; hl[3] = lrc;
  // the ice threshold matters where the ice is present, or with the CLFR ice
  // partition (criauti * cf); with NONE and no ice it is never read
  criauti = c.CRIAUTI;
  bool ice_high = false;
  if (soft && aucv_ri == 0) {
    // a soft pass reads only rit > MIN(CRIAUTI, 10**x) = rit > CRIAUTI or
    // rit > 10**x, decided from an FP32 estimate of 10**x (within 1e-5)
    // unless rit is within 2^-14 of it
    ice_high = gtd(rit, c.CRIAUTI);
    const bool open = !ice_high && gtp(rit, c.I_RTMIN);
    double x = 0.0, ea = 0.0;
    if (warp_any(open)) {
      x = c.ACRIAUTI * (t - c.TT) + c.BCRIAUTI;
      ea = fm::to_f64(exp2f(fm::to_f32(x) * 3.32192809488736235f));
    }
    const bool near = open && !gtd(rit, ea + ea * 0x1p-14) && !ltd(rit, ea - ea * 0x1p-14);
    if (open && gtd(rit, ea + ea * 0x1p-14)) ice_high = true;
    if (warp_any(near) && near) ice_high = gtd(rit, fm::fexp10(x));
  } else if (warp_any(aucv_ri != 0 || gtp(rit, c.I_RTMIN))) {
    criauti = dmin(c.CRIAUTI, fm::fexp10(c.ACRIAUTI * (t - c.TT) + c.BCRIAUTI));
  }
  double ihcf = 0, ilcf = 0, ihri = 0, ilri = 0;
  if (aucv_ri == 0) {
    if (soft ? ice_high : gtd(rit, criauti)) { ihcf = 1.0; ihri = rit; }
    else if (gtp(rit, c.I_RTMIN)) { ilcf = 1.0; ilri = rit; }
  } else if (aucv_ri == 1) {
    if (pos(cf) && gtd(rit, criauti * cf)) { ihcf = cf; ihri = rit; }
    else if (pos(cf) && gtp(rit, c.I_RTMIN)) { ilcf = cf; ilri = rit; }
  } else if (aucv_ri == 2) {
    const double sum = hi[3] + hi[2];
    ihcf = hi[0]; ilcf = hi[1];
    if (gtp(sum, 1.e-20)) { ilri = hi[3] * rit / sum; ihri = hi[2] * rit / sum; }
  }
  hi[0] = ihcf; hi[1] = ilcf; hi[2] = ihri; hi[3] = ilri;
  return dmax(hl[0], hi[0]);
}

// INTERP_MICRO (micro/interp_micro.func.h, packed path): index from log(x).
// floor(z) is taken from z truncated to FP32 (never above z; one below
// floor(z) only within 2^-23 z above an integer, fixed by the f >= 1 test),
// so that no FP64 <-> integer conversion is issued; same i and f as
// (int)z, z - (double)(int)z.
ICE3_HD double lut_index(double logx, double knum, double p1, double p2, int &i)
{
  const double z = dmax(1.00001, dmin(knum - 0.00001, p1 * logx + p2));
  i = (int)fm::to_f32(z);
  double f = z - fm::i2d(i);
  if (!ltp(f, 1.0)) {
    ++i;
    f = z - fm::i2d(i);
  }
  return f;
}
ICE3_HD double lut1d(const double *lt, int i, double f) { return lt[i] * f - lt[i - 1] * (f - 1.0); }
// PLT(i1+1, i2+1) of the 1-based Fortran table is row i1, column i2 of the
// row-major table; lut_index keeps i1 in [1, n1-1] and i2 in [1, n2-1].
ICE3_HD double lut2d(const double *lt, int n2, int i1, double f1, int i2, double f2)
{
  const double *r1 = lt + i1 * n2, *r0 = lt + (i1 - 1) * n2;
  return (r1[i2] * f2 - r1[i2 - 1] * (f2 - 1.0)) * f1 - (r0[i2] * f2 - r0[i2 - 1] * (f2 - 1.0)) * (f1 - 1.0);
}

// Slope parameters (mode_ice4_tendencies.F90:389-433): lbda and log(lbda) per
// precipitating species, zero / -inf where the species is absent.
struct Slopes {
  double lbdar, lbdas, lbdag, lbdah;
  double llbdar, llbdas, llbdag, llbdah;
};

ICE3_HD void slopes(const Cst &c, const Derived &d, double lrho, double t, const double v[NV], Slopes &s)
{
  if (pos(v[IRR])) {
    s.llbdar = d.lLBR + c.LBEXR * (lrho + fm::flog(dmax(v[IRR], c.R_RTMIN)));
    s.lbdar = fm::fexp(s.llbdar);
  } else { s.lbdar = 0.0; s.llbdar = -INFINITY; }
  if (d.lsnow_t) {
    if (pos(v[IRS])) {
      const double e = gtp(t, 263.15) ? fm::fexp10(14.554 - 0.0423 * t) : fm::fexp10(6.226 - 0.0106 * t);
      s.lbdas = dmax(dmin(c.LBDAS_MAX, e), c.LBDAS_MIN) * c.TRANS_MP_GAMMAS;
      s.llbdas = fm::flog(s.lbdas);
    } else { s.lbdas = 0.0; s.llbdas = -INFINITY; }
  } else if (pos(v[IRS])) {
    s.llbdas = dmin(d.lLBDAS_MAX, d.lLBS + c.LBEXS * (lrho + fm::flog(dmax(v[IRS], c.S_RTMIN))));
    s.lbdas = fm::fexp(s.llbdas);
  } else { s.lbdas = 0.0; s.llbdas = -INFINITY; }
  if (pos(v[IRG])) {
    s.llbdag = d.lLBG + c.LBEXG * (lrho + fm::flog(dmax(v[IRG], c.G_RTMIN)));
    s.lbdag = fm::fexp(s.llbdag);
  } else { s.lbdag = 0.0; s.llbdag = -INFINITY; }
}

// hail slope (mode_ice4_tendencies.F90:426-432)
ICE3_HD void slope_h(const Cst &c, double lrho, double rh, Slopes &s)
{
  if (pos(rh)) {
    s.llbdah = fm::flog(c.LBH) + c.LBEXH * (lrho + fm::flog(dmax(rh, c.H_RTMIN)));
    s.lbdah = fm::fexp(s.llbdah);
  } else { s.lbdah = 0.0; s.llbdah = -INFINITY; }
}

// log of the rain slope parameter within the precipitation fraction
// (mode_ice4_tendencies.F90:395-405, LLRFR): -inf where rr or rainfr is 0.
ICE3_HD double llbdar_rf(const Cst &c, const Derived &d, double lrho, double rr, double rainfr)
{
  if (!(pos(rr) && pos(rainfr))) return -INFINITY;
  return d.lLBR + c.LBEXR * (lrho + fm::flog(dmax(rr / rainfr, c.R_RTMIN)));
}

// The subgrid forms of RCACCR (SUBG_RC_RR_ACCR = PRFR: accretion in the high
// and low cloud parts within the precipitation fraction) and RREVAV
// (SUBG_RR_EVAP = CLFR / PRFR: evaporation in the clear part of the grid or
// of the precipitation fraction, at the liquid-water temperature), hard
// pass (mode_ice4_warm.F90).
ICE3_HD void warm_subgrid(const Cst &c, const Derived &d, const PointFix &pf, double t, const double v[NV],
                          const double hl[4], double ka, double dv, double cj, const Slopes &s, double rainfr,
                          double e_caccr, Rates &R, const double *acrf = nullptr)
{
  double *b = R.bu;
  const bool has_c = gtp(v[IRC], c.C_RTMIN), has_r = gtp(v[IRR], c.R_RTMIN);
  const int accr = d.accr, evap = d.evap;
  const bool llrfr = accr == 1 || evap == 2;
  const double llrf = llrfr ? llbdar_rf(c, d, pf.lrho, v[IRR], rainfr) : s.llbdar;
  if (accr == 0) {
    // OCND2: the collision factor PACRF (mode_ice4_warm.F90:128)
    b[B_RCACCR] = (has_c && has_r) ? (acrf ? c.FCACCR * v[IRC] * *acrf * e_caccr * pf.rho_mcexvt
                                           : c.FCACCR * v[IRC] * e_caccr * pf.rho_mcexvt)
                                   : 0.0;
  } else {
    const bool m = has_c && has_r;
    const bool m1 = m && gtp(hl[2], c.C_RTMIN) && pos(hl[0]);
    const bool m2 = m && gtp(hl[3], c.C_RTMIN) && gtp(hl[1], 1.e-20);
    double r = 0.0;
    if (m1 || m2) {
      const double k = c.FCACCR * fm::fexp(c.EXCACCR * llrf) * pf.rho_mcexvt;
      if (m1) r = k * hl[2];
      if (m2) r += k * fm::fdiv(hl[3], hl[1]) * (dmin(pf.cf, rainfr) - hl[0]);
    }
    b[B_RCACCR] = r;
  }
  if (evap == 0) {
    if (has_r && !has_c) {
      const double esw = esat_from(c.ALPW, c.BETAW, c.GAMW, fm::frcp(t), fm::flog(t));
      const double usw = 1. - fm::fdiv(v[IRV] * (pf.pres - esw), c.EPSILO * esw);
      const double av = fm::fdiv(sq(c.LVTT + d.cpv_cl * (t - c.TT)), ka * c.RV * t * t) +
                        fm::fdiv(c.RV * t, dv * esw);
      b[B_RREVAV] = fm::fdiv(pmax0(usw), pf.rho * av) *
                    (c.O0EVAR * fm::fexp(c.EX0EVAR * s.llbdar) + c.O1EVAR * cj * fm::fexp(c.EX1EVAR * s.llbdar));
    } else b[B_RREVAV] = 0.0;
  } else {
    const double zw4 = evap == 1 ? 1.0 : rainfr;
    const double lz3 = evap == 1 ? s.llbdar : llrf;
    if (has_r && gtd(zw4, pf.cf)) {
      const double tht = v[ITH];
      const double thlt = tht - fm::fdiv(c.LVTT * tht, c.CPD * t) * v[IRC];
      const double zw2 = fm::fdiv(thlt * t, tht);
      const double esw = esat_from(c.ALPW, c.BETAW, c.GAMW, fm::frcp(zw2), fm::flog(zw2));
      const double usw = 1.0 - fm::fdiv(v[IRV] * (pf.pres - esw), c.EPSILO * esw);
      const double av = fm::fdiv(sq(c.LVTT + d.cpv_cl * (zw2 - c.TT)), ka * c.RV * zw2 * zw2) +
                        fm::fdiv(c.RV * zw2, dv * esw);
      b[B_RREVAV] = fm::fdiv(pmax0(usw), pf.rho * av) *
                    (c.O0EVAR * fm::fexp(c.EX0EVAR * lz3) + c.O1EVAR * cj * fm::fexp(c.EX1EVAR * lz3)) *
                    (zw4 - pf.cf);
    } else b[B_RREVAV] = 0.0;
  }
}

// The hard-pass rates of ICE4_TENDENCIES after nucleation, RRHONG and RIMLTC
// (mode_ice4_tendencies.F90:303-600): derived fields, slopes, ICE4_SLOW,
// ICE4_WARM and the rate parts of ICE4_FAST_RS/RG/RI.  The parts that depend
// on the current freezing budget (riming/accretion split, wet/dry growth
// choice) are left to aggregate(), which every pass runs.
// H (NRR = 7): also the rate parts of ICE4_FAST_RH into *hr, from the hail
// kernels at hlut (global memory); v then holds NVH values.
// O (OCND2): the tabulated derived fields, collision factors, tuning factors
// and ICE4_FAST_RI_RS of the LOCND2 branches, with the point inputs *op; the
// hard-pass OCND2 quantities go to *orr.
template <bool SUR = false, bool SUBG = false, bool H = false, bool O = false>
ICE3_HD void hard_rates(const Cst &c, const Derived &d, const double *__restrict__ lut, const PointFix &pf,
                        double t, const double *v, double cit, const double hl[4], const double hi[4],
                        double criauti, Rates &R, bool learned_slow = false, double rainfr = 1.0,
                        HailRates *hr = nullptr, const double *__restrict__ hlut = nullptr,
                        const OcndPt *op = nullptr, OcndRates *orr = nullptr, const TTerms *tt = nullptr)
{
  double *b = R.bu, *rs = R.rs, *rg = R.rg;
  const double rho = pf.rho;
  // derived fields (mode_ice4_tendencies.F90:303-320; OCND2: es_i and ai
  // from the TIWMX tables, :304-309); es_i of the freezing heat terms stays
  // the formula, OCND2 takes the table for ssi, ai and ICE4_FAST_RI_RS only.
  // The nucleation of the same pass has formed them already if T is unchanged.
  // es_w serves the melting heat term (T > TT) and the evaporation of rain
  // without cloud only; it is not formed for the other points
  const bool need_esw = gtp(t, c.TT) || (gtp(v[IRR], c.R_RTMIN) && !gtp(v[IRC], c.C_RTMIN));
  double lt, it, esi_f, esw = 0.0;
  if (tt && tt->set && fm::bits_(tt->t) == fm::bits_(t)) {
    lt = tt->lt; it = tt->it; esi_f = tt->esi;
    if (tt->esw_set) esw = tt->esw;
    else if (need_esw) esw = esat_from(c.ALPW, c.BETAW, c.GAMW, it, lt);
  } else {
    lt = fm::flog(t); it = fm::frcp(t);
    esi_f = esat_from(c.ALPI, c.BETAI, c.GAMI, it, lt);
    if (need_esw) esw = esat_from(c.ALPW, c.BETAW, c.GAMW, it, lt);
  }
  const double esi = O ? tiwmx_at(op->tw + TW_ESI * kTiwmxN, t) : esi_f;
  R.ssi = fm::fdiv(v[IRV] * (pf.pres - esi), c.EPSILO * esi) - 1.0;
  const bool has_v = gtp(v[IRV], c.V_RTMIN), has_c = gtp(v[IRC], c.C_RTMIN), has_r = gtp(v[IRR], c.R_RTMIN);
  const bool has_i = gtp(v[IRI], c.I_RTMIN), has_s = gtp(v[IRS], c.S_RTMIN), has_g = gtp(v[IRG], c.G_RTMIN);
  const bool has_h = H && gtp(v[IRH], c.H_RTMIN);
  const bool warm = gtp(t, c.TT);
  // The diffusion / conduction terms (ka, dv, ai), the ventilation
  // coefficient cj and ssi / (rho ai) serve the processes of snow, graupel
  // and hail (deposition, heat terms), the evaporation of rain, the
  // Bergeron process and the OCND2 ice processes only; points with none of
  // them (cloud and / or ice alone) do not form them.
  const bool need_dep = O || SUBG || has_s || has_g || has_h || (d.lwarm && has_r && !has_c) ||
                        (pos(R.ssi) && has_c && has_i && gtp(cit, 1.e-20));
  double ka = 0.0, dv = 0.0, ika = 0.0, idv = 0.0, ai = 0.0;
  if (need_dep) {
    ka = 2.38e-2 + 7.1e-5 * (t - c.TT);
    dv = 2.11e-5 * fm::fexp(1.94 * (lt - d.lTT)) * fm::fdiv(c.P00, pf.pres);
    ika = fm::frcp(ka);
    idv = fm::frcp(dv);
    ai = O ? tiwmx_at(op->tw + TW_A2 * kTiwmxN, t) + tiwmx_at(op->tw + TW_BB3 * kTiwmxN, t) * pf.pres
           : sq(c.LSTT + d.cpv_ci * (t - c.TT)) * (ika * d.irv * it * it) + (c.RV * t) * fm::fdiv(idv, esi);
  }
  double colf = 1.0, acrf = 1.0;
  if (O) {
    // collision factors from the mean droplet radius (:322-346, LLCOL)
    orr->esi = esi;
    colf = acrf = 0.00001;
    if (gtp(v[IRC], 1.0e-10)) {
      const double rcw = 0.1 * fm::fexp(0.333 * fm::flog(fm::fdiv(0.75 * v[IRC] * rho, c.PI * (op->conc * 0.000001))));
      double vt = ltp(rcw, 0.0065) ? 1.19e6 * sq(rcw) : 8000. * rcw;
      vt = dmin(10., vt);
      const double st = dmax(0.01, fm::fdiv(2. * (100. - vt) * vt, c.GRAVITY0 * 10.));
      if (gtp(st, 0.1)) colf = dmax(0.01, dmin(1., 0.939 * fm::fexp(2.657 * fm::flog(st))));
      if (gtp(v[IRR], 1.0e-10) && gtp(rcw, 1.0e-5)) {
        const double r20 = fm::fexp(rcw * 2000.);
        acrf = fm::fdiv(r20 - 1., r20 + 1.);
      }
    }
    orr->colf = colf;
    orr->acrf = acrf;
  }
  double cj = 0.0, ssi_rai = 0.0;
  if (need_dep) {
    cj = c.SCFAC * fm::fexp(0.3 * pf.lrho) * fm::frsqrt(1.718e-5 + 4.9e-8 * (t - c.TT));
    ssi_rai = fm::fdiv(R.ssi, rho * ai);
  }
  Slopes s;
  slopes(c, d, pf.lrho, t, v, s);
  if (H) slope_h(c, pf.lrho, v[IRH], s);
  // ventilation factors shared by deposition, freezing and melting
  const double vent_s = has_s ? c.O0DEPS * (d.ex0deps_zero ? 1.0 : fm::fexp(c.EX0DEPS * s.llbdas)) +
                                    c.O1DEPS * cj * fm::fexp(c.EX1DEPS * s.llbdas)
                              : 0.0;
  const double vent_g = has_g ? c.O0DEPG * (d.ex0depg_zero ? 1.0 : fm::fexp(c.EX0DEPG * s.llbdag)) +
                                    c.O1DEPG * cj * fm::fexp(c.EX1DEPG * s.llbdag)
                              : 0.0;
  const double ilr = has_r ? fm::frcp(s.lbdar) : 0.0, ils = has_s ? fm::frcp(s.lbdas) : 0.0;
  const double ilg = has_g ? fm::frcp(s.lbdag) : 0.0;
  // lbdar^EXCACCR, shared by RCACCR and (EXICFRR = EXCACCR) RICFRRG
  const double e_caccr = (has_r && (has_c || (has_i && d.icfrr_caccr))) ? fm::fexp(c.EXCACCR * s.llbdar) : 0.0;
  // lbdas^(CXS-BS) (RSACCRG, RSWETG) and lbdag^CXG (RSWETG, RRDRYG)
  const double e_cxsbs = (has_s && (has_r || has_g || has_h)) ? fm::fexp(d.cxs_bs * s.llbdas) : 0.0;
  const double e_cxg = (has_g && (has_s || has_r)) ? fm::fexp(c.CXG * s.llbdag) : 0.0;
  // vapour/heat term of the freezing and melting rates (mode_ice4_fast_rs.F90
  // IFREEZ1/RSMLTG, mode_ice4_fast_rg.F90 IFREEZ1/RGMLTR), e limited by the
  // saturation pressure over ice (freezing) or over water (melting)
  double heat_i = 0.0, heat_w = 0.0;
  if (has_s || has_g || has_h) {
    const double ev = fm::fdiv(v[IRV] * pf.pres, c.EPSILO + v[IRV]);
    const double ei = c.LEVLIMIT != 0.0 ? dmin(ev, esi_f) : ev;
    const double ew = c.LEVLIMIT != 0.0 ? dmin(ev, esw) : ev;
    const double kt = ka * (c.TT - t);
    const double dl = dv * (c.LVTT + d.cpv_cl * (t - c.TT));
    const double irt = it * d.irv;
    heat_i = kt + (dl * (c.ESTT - ei) * irt);
    heat_w = kt + (dl * (c.ESTT - ew) * irt);
  }

  // ---- ICE4_SLOW (mode_ice4_slow.F90); taken from the surrogate instead
  // where it supplies them (slow_rates_from) ----
  if (!(SUR && learned_slow)) {
    b[B_RCHONI] = (ltp(t, d.tt_m35) && has_c)
                      ? dmin(1000., c.HON * rho * v[IRC] * fm::fexp(c.ALPHA3 * (t - c.TT) - c.BETA3))
                      : 0.0;
    b[B_RVDEPS] = (has_v && has_s) ? (O ? ssi_rai * vent_s * c.FRMIN40 : ssi_rai * vent_s) : 0.0;
    b[B_RIAGGS] = (has_i && has_s)
                      ? c.FIAGGS * fm::fexp(c.COLEXIS * (t - c.TT) + c.EXIAGGS * s.llbdas) * v[IRI] * pf.rho_mcexvt
                      : 0.0;
    b[B_RIAUTS] = gtp(hi[2], c.I_RTMIN)
                      ? c.TIMAUTI * fm::fexp(c.TEXAUTI * (t - c.TT)) * pmax0(hi[2] - criauti * hi[0])
                      : 0.0;
    b[B_RVDEPG] = (has_v && has_g) ? (O ? ssi_rai * vent_g * c.FRMIN39 : ssi_rai * vent_g) : 0.0;
  }

  // ---- ICE4_WARM (mode_ice4_warm.F90) ----
  if (SUBG && d.lwarm && (d.accr != 0 || d.evap != 0)) {
    b[B_RCAUTR] = (gtp(hl[2], c.C_RTMIN) && pos(hl[0])) ? c.TIMAUTC * pmax0(hl[2] - hl[0] * pf.rcrautc) : 0.0;
    warm_subgrid(c, d, pf, t, v, hl, ka, dv, cj, s, rainfr, e_caccr, R, O ? &acrf : nullptr);
  } else if (d.lwarm) {
    // SUBG_RC_RR_ACCR = SUBG_RR_EVAP = NONE
    b[B_RCAUTR] = (gtp(hl[2], c.C_RTMIN) && pos(hl[0])) ? c.TIMAUTC * pmax0(hl[2] - hl[0] * pf.rcrautc) : 0.0;
    b[B_RCACCR] = (has_c && has_r) ? (O ? c.FCACCR * v[IRC] * acrf * e_caccr * pf.rho_mcexvt
                                        : c.FCACCR * v[IRC] * e_caccr * pf.rho_mcexvt)
                                   : 0.0;
    if (has_r && !has_c) {
      const double usw = 1. - fm::fdiv(v[IRV] * (pf.pres - esw), c.EPSILO * esw);
      const double av = sq(c.LVTT + d.cpv_cl * (t - c.TT)) * (ika * d.irv * it * it) + (c.RV * t) * fm::fdiv(idv, esw);
      b[B_RREVAV] = fm::fdiv(pmax0(usw), rho * av) *
                    (c.O0EVAR * (d.ex0evar_m2 ? ilr * ilr : fm::fexp(c.EX0EVAR * s.llbdar)) +
                     c.O1EVAR * cj * fm::fexp(c.EX1EVAR * s.llbdar));
    } else b[B_RREVAV] = 0.0;
  } else {
    b[B_RCAUTR] = b[B_RCACCR] = b[B_RREVAV] = 0.0;
  }

  // ---- ICE4_FAST_RS rates (mode_ice4_fast_rs.F90) ----
  // collision-freezing denominator, shared with ICE4_FAST_RG
  const double den = (has_s || has_g || has_h) ? fm::frcp(rho * (c.LMTT - c.CL * (c.TT - t))) : 0.0;
  const double freez2 = (rho * (c.LMTT + d.ci_cl * (c.TT - t))) * den;
  rs[RS_FREEZ1] = has_s ? heat_i * vent_s * den : 0.0;
  rs[RS_FREEZ2] = has_s ? freez2 : 0.0;
  if (has_c && has_s) {
    int i;
    const double fr = lut_index(s.llbdas, c.NGAMINC, c.RIMINTP1, c.RIMINTP2, i);
    const double zw1 = lut1d(lut + O_RIM1, i, fr);
    const double zw2 = lut1d(lut + O_RIM2, i, fr);
    const double zw3 = lut1d(lut + O_RIM4, i, fr);
    const double e_crimss = fm::fexp(c.EXCRIMSS * s.llbdas);
    const double rcc = O ? v[IRC] * colf : v[IRC];                 // PCOLF
    rs[RS_RCRIMSS] = O ? c.CRIMSS * zw1 * v[IRC] * colf * e_crimss * pf.rho_mcexvt
                       : c.CRIMSS * zw1 * v[IRC] * e_crimss * pf.rho_mcexvt;
    rs[RS_RCRIMS] = c.CRIMSG * rcc * (d.crims_same ? e_crimss : fm::fexp(c.EXCRIMSG * s.llbdas)) * pf.rho_mcexvt;
    if (d.snow_riming == 0) {
      const double zzw = rs[RS_RCRIMS] - rs[RS_RCRIMSS];
      const double e_srimcg = fm::fexp(c.EXSRIMCG * s.llbdas);
      const double e_srimcg2 = d.srimcg2_twice ? e_srimcg * e_srimcg : fm::fexp(c.EXSRIMCG2 * s.llbdas);
      const double r = c.SRIMCG * e_srimcg * (1.0 - zw2);
      rs[RS_RSRIMCG] = fm::fdiv(zzw * r, dmax(1.e-20, d.srimcg32 * e_srimcg2 * (1. - zw3) - c.SRIMCG3 * r));
    } else rs[RS_RSRIMCG] = 0.0;
  } else {
    rs[RS_RCRIMS] = rs[RS_RCRIMSS] = rs[RS_RSRIMCG] = 0.0;
  }
  if (has_r && has_s) {
    int i1, i2;
    const double f1 = lut_index(s.llbdas, c.NACCLBDAS, c.ACCINTP1S, c.ACCINTP2S, i1);
    const double f2 = lut_index(s.llbdar, c.NACCLBDAR, c.ACCINTP1R, c.ACCINTP2R, i2);
    const double zw1 = lut2d(lut + O_RACCSS, ICE3GB_NACCLBDAR, i1, f1, i2, f2);
    const double zw2 = lut2d(lut + O_RACCS, ICE3GB_NACCLBDAR, i1, f1, i2, f2);
    const double zw3 = lut2d(lut + O_SACCRG, ICE3GB_NACCLBDAS, i2, f2, i1, f1);
    const double zzw = c.FRACCSS * (d.cxs_one ? s.lbdas : fm::fexp(c.CXS * s.llbdas)) * pf.rho_mcexvt1 *
                       (c.LBRACCS1 * ils * ils + c.LBRACCS2 * ils * ilr + c.LBRACCS3 * ilr * ilr) * sq(sq(ilr));
    rs[RS_RRACCSS] = O ? zw1 * zzw * c.FRMIN7 : zw1 * zzw;        // OCND2: XFRMIN(7), fast_rs :327
    rs[RS_RRACCS] = zw2 * zzw;
    rs[RS_RSACCRG] = (!O || gtp(v[IRS], c.FRMIN1))                 // OCND2: rs > XFRMIN(1), :347
                         ? c.FSACCRG * zw3 * e_cxsbs * pf.rho_mcexvt1 *
                               (c.LBSACCR1 * ilr * ilr + c.LBSACCR2 * ilr * ils + c.LBSACCR3 * ils * ils) * ilr
                         : 0.0;
  } else {
    rs[RS_RRACCS] = rs[RS_RRACCSS] = rs[RS_RSACCRG] = 0.0;
  }
  if (has_s && warm) {
    b[B_RSMLTG] = c.FSCVMG * pmax0(fm::fdiv(-heat_w * vent_s - (rs[RS_RCRIMS] + rs[RS_RRACCS]) * (rho * c.CL * (c.TT - t)),
                                            rho * c.LMTT));
    b[B_RCMLTSR] = rs[RS_RCRIMS];
  } else {
    b[B_RSMLTG] = b[B_RCMLTSR] = 0.0;
  }

  // ---- ICE4_FAST_RG rates (mode_ice4_fast_rg.F90, KRR = 6) ----
  if (has_i && has_r) {
    b[B_RICFRRG] = c.ICFRR * v[IRI] * (d.icfrr_caccr ? e_caccr : fm::fexp(c.EXICFRR * s.llbdar)) * pf.rho_mcexvt;
    b[B_RRCFRIG] = c.RCFRI * cit * fm::fexp(c.EXRCFRI * s.llbdar) * pf.rho_mcexvt1;
    if (d.lcrflimit) {
      const double zw = pmax0(dmin(1., fm::fdiv((b[B_RICFRRG] * c.CI + b[B_RRCFRIG] * c.CL) * (c.TT - t),
                                                  dmax(1.e-20, c.LVTT * b[B_RRCFRIG]))));
      b[B_RRCFRIG] = zw * b[B_RRCFRIG];
      b[B_RICFRR] = (1. - zw) * b[B_RICFRRG];
      b[B_RICFRRG] = zw * b[B_RICFRRG];
    } else b[B_RICFRR] = 0.0;
  } else {
    b[B_RICFRRG] = b[B_RRCFRIG] = b[B_RICFRR] = 0.0;
  }
  const double base_g = (has_g && (has_c || has_i)) ? fm::fexp(d.cxg_dg2 * s.llbdag) * pf.rho_mcexvt : 0.0;
  rg[RG_RCDRYG] = (has_g && has_c) ? c.FCDRYG * v[IRC] * base_g : 0.0;
  if (has_g && has_i) {
    const double e = fm::fexp(c.COLEXIG * (t - c.TT));
    rg[RG_RIDRYG] = c.FIDRYG * e * v[IRI] * base_g;
    rg[RG_RIWETG] = fm::fdiv(rg[RG_RIDRYG], c.COLIG * e);
  } else rg[RG_RIDRYG] = rg[RG_RIWETG] = 0.0;
  if (has_s && has_g && !O) {             // OCND2: no snow-graupel collection (fast_rg :183-189, :207)
    int i1, i2;
    const double f1 = lut_index(s.llbdag, c.NDRYLBDAG, c.DRYINTP1G, c.DRYINTP2G, i1);
    const double f2 = lut_index(s.llbdas, c.NDRYLBDAS, c.DRYINTP1S, c.DRYINTP2S, i2);
    const double zw = lut2d(lut + O_SDRYG, ICE3GB_NDRYLBDAS, i1, f1, i2, f2);
    rg[RG_RSWETG] = fm::fdiv(c.FSDRYG * zw, c.COLSG) * (e_cxsbs * e_cxg) * pf.rho_mcexvt1 *
                    (c.LBSDRYG1 * ilg * ilg + c.LBSDRYG2 * ilg * ils + c.LBSDRYG3 * ils * ils);
    rg[RG_RSDRYG] = rg[RG_RSWETG] * c.COLSG * fm::fexp(c.COLEXSG * (t - c.TT));
  } else rg[RG_RSDRYG] = rg[RG_RSWETG] = 0.0;
  if (has_r && has_g) {
    int i1, i2;
    const double f1 = lut_index(s.llbdag, c.NDRYLBDAG, c.DRYINTP1G, c.DRYINTP2G, i1);
    const double f2 = lut_index(s.llbdar, c.NDRYLBDAR, c.DRYINTP1R, c.DRYINTP2R, i2);
    const double zw = lut2d(lut + O_RDRYG, ICE3GB_NDRYLBDAR, i1, f1, i2, f2);
    rg[RG_RRDRYG] = c.FRDRYG * zw * sq(sq(ilr)) * e_cxg * pf.rho_mcexvt1 *
                    (c.LBRDRYG1 * ilg * ilg + c.LBRDRYG2 * ilg * ilr + c.LBRDRYG3 * ilr * ilr);
  } else rg[RG_RRDRYG] = 0.0;
  rg[RG_FREEZ1] = has_g ? heat_i * vent_g * den : 0.0;
  rg[RG_FREEZ2] = has_g ? freez2 : 0.0;
  if (has_g && warm) {
    b[B_RGMLTR] = pmax0(fm::fdiv(-heat_w * vent_g - (rg[RG_RCDRYG] + rg[RG_RRDRYG]) * (rho * c.CL * (c.TT - t)),
                                 rho * c.LMTT));
  } else b[B_RGMLTR] = 0.0;

  // ---- ICE4_FAST_RH rates (mode_ice4_fast_rh.F90, NRR = 7); the dry
  // collection efficiency of graupel and the wet/dry choice are applied in
  // aggregate() ----
  if (H) {
    double *ht = hr->t;
    const double base_h = (has_h && (has_c || has_i)) ? fm::fexp(d.cxh_dh2 * s.llbdah) * pf.rho_mcexvt
                                                      : 0.0;
    ht[RH_RCWETH] = (has_h && has_c) ? c.FWETH * v[IRC] * base_h : 0.0;
    if (has_h && has_i) {
      ht[RH_RIWETH] = c.FWETH * v[IRI] * base_h;
      ht[RH_RIDRYH] = ht[RH_RIWETH] * (c.COLIH * fm::fexp(c.COLEXIH * (t - c.TT)));
    } else ht[RH_RIWETH] = ht[RH_RIDRYH] = 0.0;
    const double e_cxh = (has_h && (has_s || has_g || has_r)) ? fm::fexp(c.CXH * s.llbdah) : 0.0;
    const double ilh = has_h ? fm::frcp(s.lbdah) : 0.0;
    if (has_h && has_s) {
      int i1, i2;
      const double f1 = lut_index(s.llbdah, c.NWETLBDAH, c.WETINTP1H, c.WETINTP2H, i1);
      const double f2 = lut_index(s.llbdas, c.NWETLBDAS, c.WETINTP1S, c.WETINTP2S, i2);
      const double zw = lut2d(hlut + O_SWETH, ICE3GB_NWETLBDAS, i1, f1, i2, f2);
      ht[RH_RSWETH] = c.FSWETH * zw * e_cxsbs * e_cxh * pf.rho_mcexvt1 *
                      (c.LBSWETH1 * ilh * ilh + c.LBSWETH2 * ilh * ils + c.LBSWETH3 * ils * ils);
      ht[RH_RSDRYH] = ht[RH_RSWETH] * (c.COLSH * fm::fexp(c.COLEXSH * (t - c.TT)));
    } else ht[RH_RSWETH] = ht[RH_RSDRYH] = 0.0;
    if (has_h && has_g) {
      int i1, i2;
      const double f1 = lut_index(s.llbdah, c.NWETLBDAH, c.WETINTP1H, c.WETINTP2H, i1);
      const double f2 = lut_index(s.llbdag, c.NWETLBDAG, c.WETINTP1G, c.WETINTP2G, i2);
      const double zw = lut2d(hlut + O_GWETH, ICE3GB_NWETLBDAG, i1, f1, i2, f2);
      ht[RH_RGWETH] = c.FGWETH * zw * fm::fexp(d.cxg_bg * s.llbdag) * e_cxh * pf.rho_mcexvt1 *
                      (c.LBGWETH1 * ilh * ilh + c.LBGWETH2 * ilh * ilg + c.LBGWETH3 * ilg * ilg);
      ht[RH_RGDRYH] = ht[RH_RGWETH];
    } else ht[RH_RGWETH] = ht[RH_RGDRYH] = 0.0;
    if (has_h && has_r) {
      int i1, i2;
      const double f1 = lut_index(s.llbdah, c.NWETLBDAH, c.WETINTP1H, c.WETINTP2H, i1);
      const double f2 = lut_index(s.llbdar, c.NWETLBDAR, c.WETINTP1R, c.WETINTP2R, i2);
      const double zw = lut2d(hlut + O_RWETH, ICE3GB_NWETLBDAR, i1, f1, i2, f2);
      ht[RH_RRWETH] = c.FRWETH * zw * sq(sq(ilr)) * e_cxh * pf.rho_mcexvt1 *
                      (c.LBRWETH1 * ilh * ilh + c.LBRWETH2 * ilh * ilr + c.LBRWETH3 * ilr * ilr);
    } else ht[RH_RRWETH] = 0.0;
    const double vent_h = has_h ? c.O0DEPH * fm::fexp(c.EX0DEPH * s.llbdah) +
                                      c.O1DEPH * cj * fm::fexp(c.EX1DEPH * s.llbdah)
                                : 0.0;
    ht[RH_FREEZ1] = has_h ? heat_i * vent_h * den : 0.0;
    ht[RH_FREEZ2] = has_h ? freez2 : 0.0;
    hr->b[BH_RHMLTR] = (has_h && warm) ? pmax0(fm::fdiv(-heat_w * vent_h - (ht[RH_RCWETH] + ht[RH_RRWETH]) *
                                                                            (rho * c.CL * (c.TT - t)),
                                                        rho * c.LMTT))
                                       : 0.0;
  }

  // ---- OCND2: ICE4_FAST_RI_RS (mode_ice4_fast_ri_rs.F90, LMODICEDEP = .FALSE.)
  // in place of ICE4_FAST_RI (mode_ice4_tendencies.F90:568-596) ----
  if (O) {
    b[B_RCBERI] = 0.0;
    const double ri = v[IRI], dicrit = c.FRMIN15, timesc = c.FRMIN14;
    double rilars = (pos(ri) && gtp(R.ssi, 0.001)) ? dmin(ri, fm::fdiv(ri, fm::fdiv(87.5 * (dicrit * dicrit) * ai, R.ssi)))
                                                  : 0.0;
    double rvdepi = 0.0;
    if (pos(pf.pres * 0.5 - esi) && pos(cit)) {
      const double w2d = fm::frcp(op->ifr * op->icldfr + 1. - op->icldfr);
      const double xw2d13 = fm::fexp(0.333 * fm::flog(op->ifr));
      const double wcitred23 = fm::fexp(0.667 * fm::flog(0.1));
      const double tc = dmax(-18., dmin(-1., t - c.TT));
      const double hu = dmin(0.15, pmax0(R.ssi));
      const double cryssha = 1.1 + 3. * hu * (1. + sin(0.64 * tc - 1.3));
      const double qimax = fm::fdiv(366.5 * (dicrit * dicrit * dicrit) * cit * 0.1, rho);
      double ci2s = 0.;
      if (gtp(ri, 1.0e-12) && pos(timesc))
        ci2s = fm::fdiv(ri * (1. - dmin(1., fm::fdiv(0.5 * qimax, ri))) * (1. - op->icldfr) * w2d, timesc * 0.5);
      const double zzwc = fm::fdiv(cryssha * 0.878, ai) * fm::fexp(0.667 * fm::flog(fm::fdiv(cit, rho))) *
                          fm::fexp(0.333 * fm::flog(dmax(c.I_RTMIN, ri) * w2d));
      if (pos(op->ssio) && gtp(op->icldfr, 0.02)) rvdepi = rvdepi + zzwc * xw2d13 * op->ssio * op->icldfr;
      if (negd(op->ssiu) && ltp(op->icldfr, 0.98)) {
        rilars = rilars + ci2s;
        rvdepi = rvdepi + zzwc * wcitred23 * op->ssiu * (1. - op->icldfr);
      }
    }
    orr->rilars = rilars;
    orr->rvdepi = rvdepi;
    return;
  }
  // ---- ICE4_FAST_RI (mode_ice4_fast_ri.F90) ----
  if (pos(R.ssi) && has_c && has_i && gtp(cit, 1.e-20)) {
    const double l = dmin(1.e8, c.LBI * fm::fexp(c.LBEXI * fm::flog(fm::fdiv(rho * v[IRI], cit))));
    b[B_RCBERI] = ssi_rai * cit * (fm::fdiv(c.O0DEPI, l) + c.O2DEPI * cj * cj * fm::fexp(-(c.DI + 2.0) * fm::flog(l)));
  } else b[B_RCBERI] = 0.0;
}

// Rates of a soft pass: the hard-pass values where their condition still
// holds on the current state, zero elsewhere (the ELSE branches of the
// process routines under LDSOFT).
template <bool SUBG = false, bool H = false, bool O = false>
ICE3_HD void soft_rates(const Cst &c, const Derived &d, double t, const double *v, double cit, const double hl[4],
                        const double hi[4], Rates &R, double cf = 0.0, double rainfr = 1.0, HailRates *hr = nullptr,
                        OcndRates *orr = nullptr)
{
  if (O) orr->rvdepi = orr->rilars = 0.0;   // ICE4_FAST_RI_RS resets both and computes them on hard passes only
  double *b = R.bu, *rs = R.rs, *rg = R.rg;
  const bool has_v = gtp(v[IRV], c.V_RTMIN), has_c = gtp(v[IRC], c.C_RTMIN), has_r = gtp(v[IRR], c.R_RTMIN);
  const bool has_i = gtp(v[IRI], c.I_RTMIN), has_s = gtp(v[IRS], c.S_RTMIN), has_g = gtp(v[IRG], c.G_RTMIN);
  const bool warm = gtp(t, c.TT);
  if (!(ltp(t, d.tt_m35) && has_c)) b[B_RCHONI] = 0.0;
  if (!(has_v && has_s)) b[B_RVDEPS] = 0.0;
  if (!(has_i && has_s)) b[B_RIAGGS] = 0.0;
  if (!gtp(hi[2], c.I_RTMIN)) b[B_RIAUTS] = 0.0;
  if (!(has_v && has_g)) b[B_RVDEPG] = 0.0;
  if (SUBG && d.lwarm && (d.accr != 0 || d.evap != 0)) {
    if (!(gtp(hl[2], c.C_RTMIN) && pos(hl[0]))) b[B_RCAUTR] = 0.0;
    if (d.accr == 0) {
      if (!(has_c && has_r)) b[B_RCACCR] = 0.0;
    } else {
      const bool m = has_c && has_r;
      if (!((m && gtp(hl[2], c.C_RTMIN) && pos(hl[0])) || (m && gtp(hl[3], c.C_RTMIN) && gtp(hl[1], 1.e-20))))
        b[B_RCACCR] = 0.0;
    }
    const int evap = d.evap;
    if (evap == 0) {
      if (!(has_r && !has_c)) b[B_RREVAV] = 0.0;
    } else if (!(has_r && gtd(evap == 1 ? 1.0 : rainfr, cf))) {
      b[B_RREVAV] = 0.0;
    }
  } else if (d.lwarm) {
    if (!(gtp(hl[2], c.C_RTMIN) && pos(hl[0]))) b[B_RCAUTR] = 0.0;
    if (!(has_c && has_r)) b[B_RCACCR] = 0.0;
    if (!(has_r && !has_c)) b[B_RREVAV] = 0.0;
  } else {
    b[B_RCAUTR] = b[B_RCACCR] = b[B_RREVAV] = 0.0;
  }
  if (!has_s) rs[RS_FREEZ1] = rs[RS_FREEZ2] = 0.0;
  if (!(has_c && has_s)) rs[RS_RCRIMS] = rs[RS_RCRIMSS] = rs[RS_RSRIMCG] = 0.0;
  if (!(has_r && has_s)) rs[RS_RRACCS] = rs[RS_RRACCSS] = rs[RS_RSACCRG] = 0.0;
  if (!(has_s && warm)) b[B_RSMLTG] = b[B_RCMLTSR] = 0.0;
  if (!(has_i && has_r)) b[B_RICFRRG] = b[B_RRCFRIG] = b[B_RICFRR] = 0.0;
  if (!(has_g && has_c)) rg[RG_RCDRYG] = 0.0;
  if (!(has_g && has_i)) rg[RG_RIDRYG] = rg[RG_RIWETG] = 0.0;
  if (!(has_s && has_g)) rg[RG_RSDRYG] = rg[RG_RSWETG] = 0.0;
  if (!(has_r && has_g)) rg[RG_RRDRYG] = 0.0;
  if (!has_g) rg[RG_FREEZ1] = rg[RG_FREEZ2] = 0.0;
  if (!(has_g && warm)) b[B_RGMLTR] = 0.0;
  if (!(pos(R.ssi) && has_c && has_i && gtp(cit, 1.e-20))) b[B_RCBERI] = 0.0;
  if (H) {
    double *ht = hr->t;
    const bool has_h = gtp(v[IRH], c.H_RTMIN);
    if (!(has_h && has_c)) ht[RH_RCWETH] = 0.0;
    if (!(has_h && has_i)) ht[RH_RIWETH] = ht[RH_RIDRYH] = 0.0;
    if (!(has_h && has_s)) ht[RH_RSWETH] = ht[RH_RSDRYH] = 0.0;
    if (!(has_h && has_g)) ht[RH_RGWETH] = ht[RH_RGDRYH] = 0.0;
    if (!(has_h && has_r)) ht[RH_RRWETH] = 0.0;
    if (!has_h) ht[RH_FREEZ1] = ht[RH_FREEZ2] = 0.0;
    if (!(has_h && warm)) hr->b[BH_RHMLTR] = 0.0;
  }
}

// Freezing-budget split of riming/accretion and the wet/dry growth choice
// (mode_ice4_fast_rs.F90:144-176, :188-219; mode_ice4_fast_rg.F90:180-260),
// evaluated on every pass, then the aggregation into the tendency A (per
// second), mode_ice4_tendencies.F90:606-717 (KRR = 6).
// H (NRR = 7): also the graupel -> hail conversion (mode_ice4_fast_rg.F90:
// 331-351), the hail growth mode of ICE4_FAST_RH (mode_ice4_fast_rh.F90:
// 205-213, 250-325; the graupel dry-collection factor on a hard pass) and
// the hail rows of the aggregation, which also move B (RWETGH_MR).
// O (OCND2): the part of the graupel deposition given to snow
// (mode_ice4_tendencies.F90:445-458) and the RVDEPI / RILARS rows.
template <bool H = false, bool O = false>
ICE3_HD void aggregate(const Cst &c, double t, const double *v, double lvfact, double lsfact, Rates &R,
                       double *A, bool soft = false, HailRates *hr = nullptr, double *B = nullptr,
                       const OcndRates *orr = nullptr, const double *ext = nullptr)
{
  double *b = R.bu;
  const double *rs = R.rs, *rg = R.rg;
  const bool has_c = gtp(v[IRC], c.C_RTMIN), has_r = gtp(v[IRR], c.R_RTMIN), has_s = gtp(v[IRS], c.S_RTMIN);
  const bool has_g = gtp(v[IRG], c.G_RTMIN), cold = ltp(t, c.TT);
  double freez = has_s ? pmax0(pmax0(rs[RS_FREEZ1] + rs[RS_FREEZ2] * b[B_RIAGGS]) - b[B_RIAGGS]) : 0.0;
  if (has_c && has_s && cold) {
    b[B_RCRIMSS] = dmin(freez, rs[RS_RCRIMSS]);
    freez = pmax0(freez - b[B_RCRIMSS]);
    const double zzw0 = dmin(1., fm::fdiv(freez, dmax(1.e-20, rs[RS_RCRIMS] - b[B_RCRIMSS])));
    b[B_RCRIMSG] = zzw0 * pmax0(rs[RS_RCRIMS] - b[B_RCRIMSS]);
    freez = pmax0(freez - b[B_RCRIMSG]);
    b[B_RSRIMCG] = zzw0 * rs[RS_RSRIMCG] * (signbit(b[B_RCRIMSG]) ? 0.0 : 1.0);
    b[B_RCRIMSG] = pmax0(b[B_RCRIMSG]);
  } else {
    b[B_RCRIMSS] = b[B_RCRIMSG] = b[B_RSRIMCG] = 0.0;
  }
  if (has_r && has_s && cold) {
    b[B_RRACCSS] = dmin(freez, rs[RS_RRACCSS]);
    freez = pmax0(freez - b[B_RRACCSS]);
    const double zzw = dmin(1., fm::fdiv(freez, dmax(1.e-20, rs[RS_RRACCS] - b[B_RRACCSS])));
    b[B_RRACCSG] = zzw * pmax0(rs[RS_RRACCS] - b[B_RRACCSS]);
    freez = pmax0(freez - b[B_RRACCSG]);
    b[B_RSACCRG] = zzw * rs[RS_RSACCRG] * (signbit(b[B_RRACCSG]) ? 0.0 : 1.0);
    b[B_RRACCSG] = pmax0(b[B_RRACCSG]);
  } else {
    b[B_RRACCSS] = b[B_RRACCSG] = b[B_RSACCRG] = 0.0;
  }
  // the dry-growth sum is read only where graupel is present (and by the hail rows)
  double rdryg_init = 0.0;
  if (H || warp_any(has_g)) rdryg_init = rg[RG_RCDRYG] + rg[RG_RIDRYG] + rg[RG_RSDRYG] + rg[RG_RRDRYG];
  bool ldwetg = false, lldryg = false;
  double rwetg_init = 0.0;
  if (has_g) {
    const double is = rg[RG_RIWETG] + rg[RG_RSWETG];
    rwetg_init = dmax(is, pmax0(rg[RG_FREEZ1] + rg[RG_FREEZ2] * is));
    const double wet = pmax0(rwetg_init - rg[RG_RIWETG] - rg[RG_RSWETG]);
    const double dry = pmax0(rdryg_init - rg[RG_RIDRYG] - rg[RG_RSDRYG]);
    ldwetg = !gtd(wet, dry);
    if (c.LNULLWETG != 0.0) ldwetg = ldwetg && pos(rdryg_init);
    else ldwetg = ldwetg && pos(rwetg_init);
    if (c.LWETGPOST == 0.0) ldwetg = ldwetg && cold;
    lldryg = cold && gtp(rdryg_init, 1.e-20) && gtd(wet, dry);
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
  const double lsv = lsfact - lvfact;
  // The aggregation (mode_ice4_tendencies.F90:606-717) written as transfers:
  // every rate moves water from one species to another (and theta by L/cph),
  // one block per group of processes; a block runs when a lane of the warp
  // has a nonzero rate in it (on a pass about 3 of the 29 rates are nonzero,
  // and the points of a warp share their regime).
  double depg_s = 0.0, nodepg_s = 1.0;
  if (O && gtd(c.FRMIN5, 1.0e-12) && gtd(c.FRMIN6, 0.01)) {
    depg_s = dmax(0., dmin(1., (c.FRMIN5 - fm::fdiv(v[IRG], c.FRMIN5)))) * dmax(0., dmin(1., fm::fdiv(R.ssi, c.FRMIN6)));
    nodepg_s = 1. - depg_s;
  }
  // the sums start from the external tendencies (ICE4_STEPPING adds them to
  // the microphysical ones, mode_ice4_stepping.F90:265-272)
  double ath = 0.0, av = 0.0, ac = 0.0, ar = 0.0, ai = 0.0, as = 0.0, ag = 0.0;
  if (ext) {
    ath = ext[ITH]; av = ext[IRV]; ac = ext[IRC]; ar = ext[IRR]; ai = ext[IRI]; as = ext[IRS]; ag = ext[IRG];
  }
  if (warp_any(nz(b[B_RVDEPG]))) {                                  // vapour -> graupel (and snow, OCND2)
    const double x = b[B_RVDEPG];
    ath += x * lsfact;
    av -= x;
    if (O) { ag += x * nodepg_s; as += x * depg_s; }
    else ag += x;
  }
  if (warp_any(nz(b[B_RVDEPS]))) {                                  // vapour -> snow
    const double x = b[B_RVDEPS];
    ath += x * lsfact;
    av -= x;
    as += x;
  }
  if (warp_any(nz(b[B_RREVAV]))) {                                  // rain -> vapour
    const double x = b[B_RREVAV];
    ath -= x * lvfact;
    av += x;
    ar -= x;
  }
  if (warp_any(nz(b[B_RCHONI]) || nz(b[B_RCBERI]))) {               // cloud -> ice
    const double x = b[B_RCHONI] + b[B_RCBERI];
    ath += x * lsv;
    ac -= x;
    ai += x;
  }
  if (warp_any(nz(b[B_RCAUTR]) || nz(b[B_RCACCR]) || nz(b[B_RCMLTSR]))) {   // cloud -> rain
    const double x = b[B_RCAUTR] + b[B_RCACCR] + b[B_RCMLTSR];
    ac -= x;
    ar += x;
  }
  if (warp_any(nz(b[B_RIAGGS]) || nz(b[B_RIAUTS]))) {               // ice -> snow
    const double x = b[B_RIAGGS] + b[B_RIAUTS];
    ai -= x;
    as += x;
  }
  if (warp_any(nz(b[B_RCRIMSS]) || nz(b[B_RCRIMSG]) || nz(b[B_RSRIMCG]))) {  // riming
    const double x = b[B_RCRIMSS] + b[B_RCRIMSG];
    ath += x * lsv;
    ac -= x;
    as += b[B_RCRIMSS] - b[B_RSRIMCG];
    ag += b[B_RCRIMSG] + b[B_RSRIMCG];
  }
  if (warp_any(nz(b[B_RRACCSS]) || nz(b[B_RRACCSG]) || nz(b[B_RSACCRG]))) {  // rain accretion on snow
    const double x = b[B_RRACCSS] + b[B_RRACCSG];
    ath += x * lsv;
    ar -= x;
    as += b[B_RRACCSS] - b[B_RSACCRG];
    ag += b[B_RRACCSG] + b[B_RSACCRG];
  }
  if (warp_any(nz(b[B_RICFRRG]) || nz(b[B_RRCFRIG]) || nz(b[B_RICFRR]))) {   // rain contact freezing
    ath += (b[B_RRCFRIG] - b[B_RICFRR]) * lsv;
    ar += b[B_RICFRR] - b[B_RRCFRIG];
    ai -= b[B_RICFRRG] + b[B_RICFRR];
    ag += b[B_RICFRRG] + b[B_RRCFRIG];
  }
  if (warp_any(nz(b[B_RCWETG]) || nz(b[B_RRWETG]) || nz(b[B_RIWETG]) || nz(b[B_RSWETG]))) {  // graupel wet growth
    ath += (b[B_RCWETG] + b[B_RRWETG]) * lsv;
    ac -= b[B_RCWETG];
    ar -= b[B_RRWETG];
    ai -= b[B_RIWETG];
    as -= b[B_RSWETG];
    ag += b[B_RCWETG] + b[B_RIWETG] + b[B_RSWETG] + b[B_RRWETG];
  }
  if (warp_any(nz(b[B_RCDRYG]) || nz(b[B_RRDRYG]) || nz(b[B_RIDRYG]) || nz(b[B_RSDRYG]))) {  // graupel dry growth
    ath += (b[B_RCDRYG] + b[B_RRDRYG]) * lsv;
    ac -= b[B_RCDRYG];
    ar -= b[B_RRDRYG];
    ai -= b[B_RIDRYG];
    as -= b[B_RSDRYG];
    ag += b[B_RCDRYG] + b[B_RIDRYG] + b[B_RSDRYG] + b[B_RRDRYG];
  }
  if (warp_any(nz(b[B_RSMLTG]))) {                                  // snow -> graupel (melting conversion)
    as -= b[B_RSMLTG];
    ag += b[B_RSMLTG];
  }
  if (warp_any(nz(b[B_RGMLTR]))) {                                  // graupel -> rain
    const double x = b[B_RGMLTR];
    ath -= x * lsv;
    ar += x;
    ag -= x;
  }
  A[ITH] = ath; A[IRV] = av; A[IRC] = ac; A[IRR] = ar; A[IRI] = ai; A[IRS] = as; A[IRG] = ag;
  if (O) {
    // OCND2 rows (mode_ice4_tendencies.F90:625, 630, 673-674, 691; the
    // graupel deposition given to snow, :677, is in the block above)
    A[ITH] += orr->rvdepi * lsfact;
    A[IRV] -= orr->rvdepi;
    A[IRI] += orr->rvdepi;
    A[IRI] -= orr->rilars;
    A[IRS] += orr->rilars;
  }
  if (H) {
    double *hb = hr->b, *ht = hr->t;
    if (ldwetg) {
      const double rgsi = b[B_RVDEPG] + b[B_RSMLTG] + b[B_RRACCSG] + b[B_RSACCRG] + b[B_RCRIMSG] + b[B_RSRIMCG];
      hb[BH_RWETGH] = fm::fdiv((pmax0(rgsi + b[B_RICFRRG] + b[B_RRCFRIG]) + rwetg_init) * rdryg_init,
                               rwetg_init + rdryg_init);
      hb[BH_RWETGH_MR] = fm::fdiv(pmax0(b[B_RRHONG_MR]) * rdryg_init, rwetg_init + rdryg_init);
    } else {
      hb[BH_RWETGH] = hb[BH_RWETGH_MR] = 0.0;
    }
    const bool has_h = gtp(v[IRH], c.H_RTMIN);
    if (!soft && has_h && has_g && !ldwetg) ht[RH_RGDRYH] = ht[RH_RGDRYH] * (c.COLGH * fm::fexp(c.COLEXGH * (t - c.TT)));
    const double rdryh_init = ht[RH_RCWETH] + ht[RH_RIDRYH] + ht[RH_RSDRYH] + ht[RH_RRWETH] + ht[RH_RGDRYH];
    bool llweth = false, lldryh = false;
    double rweth_init = 0.0;
    if (has_h) {
      const double isg = ht[RH_RIWETH] + ht[RH_RSWETH] + ht[RH_RGWETH];
      rweth_init = dmax(isg, pmax0(ht[RH_FREEZ1] + ht[RH_FREEZ2] * isg));
      const double wet = pmax0(rweth_init - ht[RH_RIWETH] - ht[RH_RSWETH] - ht[RH_RGWETH]);
      const double dry = pmax0(rdryh_init - ht[RH_RIDRYH] - ht[RH_RSDRYH] - ht[RH_RGDRYH]);
      llweth = !gtd(wet, dry);
      if (c.LNULLWETH != 0.0) llweth = llweth && pos(rdryh_init);
      else llweth = llweth && pos(rweth_init);
      if (c.LWETHPOST == 0.0) llweth = llweth && cold;
      lldryh = cold && gtp(rdryh_init, 1.e-20) &&
               gtd(pmax0(rweth_init - ht[RH_RIWETH] - ht[RH_RSWETH]), pmax0(rdryh_init - ht[RH_RIDRYH] - ht[RH_RSDRYH]));
    }
    if (llweth) {
      hb[BH_RCWETH] = ht[RH_RCWETH];
      hb[BH_RIWETH] = ht[RH_RIWETH];
      hb[BH_RSWETH] = ht[RH_RSWETH];
      hb[BH_RGWETH] = ht[RH_RGWETH];
      hb[BH_RRWETH] = rweth_init - ht[RH_RIWETH] - ht[RH_RSWETH] - ht[RH_RGWETH] - ht[RH_RCWETH];
    } else {
      hb[BH_RCWETH] = hb[BH_RIWETH] = hb[BH_RSWETH] = hb[BH_RGWETH] = hb[BH_RRWETH] = 0.0;
    }
    if (lldryh) {
      hb[BH_RCDRYH] = ht[RH_RCWETH];
      hb[BH_RIDRYH] = ht[RH_RIDRYH];
      hb[BH_RSDRYH] = ht[RH_RSDRYH];
      hb[BH_RRDRYH] = ht[RH_RRWETH];
      hb[BH_RGDRYH] = ht[RH_RGDRYH];
      hb[BH_RDRYHG] = c.LCONVHG != 0.0 ? fm::fdiv(rdryh_init * rweth_init, rdryh_init + rweth_init) : 0.0;
    } else {
      hb[BH_RCDRYH] = hb[BH_RIDRYH] = hb[BH_RSDRYH] = hb[BH_RRDRYH] = hb[BH_RGDRYH] = hb[BH_RDRYHG] = 0.0;
    }
    // hail rows of mode_ice4_tendencies.F90:619-715
    A[ITH] += (hb[BH_RRWETH] + hb[BH_RCWETH]) * lsv;
    A[ITH] += (hb[BH_RCDRYH] + hb[BH_RRDRYH]) * lsv;
    A[ITH] -= hb[BH_RHMLTR] * lsv;
    A[IRC] -= hb[BH_RCWETH];
    A[IRC] -= hb[BH_RCDRYH];
    A[IRR] -= hb[BH_RRWETH];
    A[IRR] -= hb[BH_RRDRYH];
    A[IRR] += hb[BH_RHMLTR];
    A[IRI] -= hb[BH_RIWETH];
    A[IRI] -= hb[BH_RIDRYH];
    A[IRS] -= hb[BH_RSWETH];
    A[IRS] -= hb[BH_RSDRYH];
    A[IRG] -= hb[BH_RWETGH];
    B[IRG] -= hb[BH_RWETGH_MR];
    A[IRG] -= hb[BH_RGWETH];
    A[IRG] = A[IRG] - hb[BH_RGDRYH] + hb[BH_RDRYHG];
    A[IRH] = ext ? ext[IRH] + hb[BH_RWETGH] : hb[BH_RWETGH];
    B[IRH] += hb[BH_RWETGH_MR];
    A[IRH] = A[IRH] + hb[BH_RCWETH] + hb[BH_RIWETH] + hb[BH_RSWETH] + hb[BH_RGWETH] + hb[BH_RRWETH];
    A[IRH] = A[IRH] + hb[BH_RCDRYH] + hb[BH_RIDRYH] + hb[BH_RSDRYH] + hb[BH_RRDRYH] + hb[BH_RGDRYH] - hb[BH_RDRYHG];
    A[IRH] -= hb[BH_RHMLTR];
  }
}

// The five ICE4_SLOW rates of a hard pass taken from the learned surrogate
// (sur: RCHONI, RVDEPS, RIAGGS, RIAUTS, RVDEPG): each process keeps its exact
// activity condition of mode_ice4_slow.F90 and the physical sign and cap of
// its rate; only the magnitude comes from the network.
ICE3_HD void slow_rates_from(const Cst &c, double t, const double v[NV], const double hi[4], const double *sur,
                             Rates &R)
{
  double *b = R.bu;
  const bool has_v = gtp(v[IRV], c.V_RTMIN), has_c = gtp(v[IRC], c.C_RTMIN), has_i = gtp(v[IRI], c.I_RTMIN);
  const bool has_s = gtp(v[IRS], c.S_RTMIN), has_g = gtp(v[IRG], c.G_RTMIN);
  b[B_RCHONI] = (ltp(t, c.TT - 35.0) && has_c) ? dmin(1000., pmax0(sur[0])) : 0.0;
  b[B_RVDEPS] = (has_v && has_s) ? sur[1] : 0.0;
  b[B_RIAGGS] = (has_i && has_s) ? pmax0(sur[2]) : 0.0;
  b[B_RIAUTS] = gtp(hi[2], c.I_RTMIN) ? pmax0(sur[3]) : 0.0;
  b[B_RVDEPG] = (has_v && has_g) ? sur[4] : 0.0;
}

// The state adjustments of a hard pass (mode_ice4_tendencies.F90:166-300):
// nucleation (HENI), RRHONG and RIMLTC with their T-feedback limits; v and
// t are updated in place, the increments go to b and B.
template <bool O = false>
ICE3_HD void hard_adjust(const Cst &c, const Derived &d, const PointFix &pf, double lvfact, double lsfact,
                         double &cit, double &t, double v[NV], double *b, double B[NV], const OcndPt *op = nullptr,
                         TTerms *tt = nullptr)
{
  if (O) nucleation_ocnd2(c, *op, t, v[IRV], cit, b[B_RVHENI_MR]);
  else nucleation(c, d, v[ITH], pf.pres, pf.rho, pf.zx, lsfact, t, v[IRV], cit, b[B_RVHENI_MR], tt);
  // each adjustment below moves the state only where its amount is nonzero
  // (x + 0 = x), and a warp skips the updates when none of its lanes has one
  const double lsv = lsfact - lvfact;
  if (warp_any(nz(b[B_RVHENI_MR]))) {
    v[ITH] += b[B_RVHENI_MR] * lsfact;
    t = v[ITH] * pf.exn;
    v[IRV] -= b[B_RVHENI_MR];
    v[IRI] += b[B_RVHENI_MR];
  }
  // RRHONG (mode_ice4_rrhong.F90)
  double r = 0.0;
  if (ltp(t, d.tt_m35) && gtp(v[IRR], c.R_RTMIN)) {
    r = v[IRR];
    if (d.lfeedbackt) {
      // the IEEE quotients only where the limit can bind: (TT - 35)/exn
      // estimated within 2^-22 and taken 2^-20 low, so that the estimated
      // quotient is below the true one
      const double zq = quot_est(d.tt_m35, pf.exn);
      if (!quot_above(zq - fabs(zq) * 0x1p-20 - v[ITH], lsv, r))
        r = dmin(r, pmax0((d.tt_m35 / pf.exn - v[ITH]) / lsv));
    }
  }
  b[B_RRHONG_MR] = r;
  if (warp_any(nz(r))) {
    v[ITH] += r * lsv;
    t = v[ITH] * pf.exn;
    v[IRR] -= r;
    v[IRG] += r;
  }
  // RIMLTC (mode_ice4_rimltc.F90)
  r = 0.0;
  if (pos(v[IRI]) && gtp(t, c.TT)) {
    r = v[IRI];
    if (d.lfeedbackt) {
      // the IEEE quotient only where it can be below r
      const double num = v[ITH] - pf.zx;
      if (!quot_above(num, lsv, r)) r = dmin(r, pmax0(num / lsv));
    }
  }
  b[B_RIMLTC_MR] = r;
  if (warp_any(nz(r))) {
    v[ITH] -= r * lsv;
    t = v[ITH] * pf.exn;
    v[IRC] += r;
    v[IRI] -= r;
  }
  // B stays zero (as tendencies() set it) where all three amounts are zero
  if (warp_any(nz(b[B_RVHENI_MR]) || nz(b[B_RRHONG_MR]) || nz(b[B_RIMLTC_MR]))) {
    B[ITH] = b[B_RVHENI_MR] * lsfact + b[B_RRHONG_MR] * lsv - b[B_RIMLTC_MR] * lsv;
    B[IRV] = -b[B_RVHENI_MR];
    B[IRC] = b[B_RIMLTC_MR];
    B[IRR] = -b[B_RRHONG_MR];
    B[IRI] = b[B_RVHENI_MR] - b[B_RIMLTC_MR];
    B[IRG] = b[B_RRHONG_MR];
  }
}

// ICE4_TENDENCIES for one point (mode_ice4_tendencies.F90): on a hard pass
// nucleation, RRHONG and RIMLTC adjust the state (their increments go to B)
// and all rates are computed; a soft pass keeps the hard-pass rates.
template <bool SUR = false, bool SUBG = false, bool H = false, bool O = false>
ICE3_HD void tendencies(const Cst &c, const Derived &d, const double *__restrict__ lut, bool soft,
                        const PointFix &pf, double lvfact, double lsfact, double &cit, double t0,
                        const double *vart, Rates &R, double &rainfr, double hl[4], double hi[4], double *A,
                        double *B, const double *sur = nullptr, HailRates *hr = nullptr,
                        const double *__restrict__ hlut = nullptr, const OcndPt *op = nullptr,
                        OcndRates *orr = nullptr, const double *ext = nullptr)
{
  constexpr int NVT = H ? NVH : NV;
  double v[NVT];
  double t = t0;
#pragma unroll
  for (int k = 0; k < NVT; ++k) { v[k] = vart[k]; B[k] = 0.0; }
  double *b = R.bu;
  TTerms tt;
  tt.set = tt.esw_set = false;
  if (!soft) {
    hard_adjust<O>(c, d, pf, lvfact, lsfact, cit, t, v, b, B, op, &tt);
  } else {
    b[B_RVHENI_MR] = b[B_RRHONG_MR] = b[B_RIMLTC_MR] = 0.0;
  }
  double criauti;
  const double zrainfr = compute_pdf(c, d, pf.rcrautc, v[IRC], v[IRI], pf.cf, t, pf.sigma_rc, hl, hi, criauti, soft);
  const bool llrfr = d.llrfr;
  if (llrfr) {
    rainfr = dmax(rainfr, zrainfr);
    bool mask = gtp(v[IRR], c.R_RTMIN) || gtp(v[IRS], c.S_RTMIN) || gtp(v[IRG], c.G_RTMIN);
    if (H) mask = mask || gtp(v[NVT - 1], c.H_RTMIN);
    if (mask && zerod(rainfr)) rainfr = 1.;
  } else {
    rainfr = 1.;
  }
  if (!soft)
    hard_rates<SUR, SUBG, H, O>(c, d, lut, pf, t, v, cit, hl, hi, criauti, R, sur != nullptr, rainfr, hr, hlut, op,
                                orr, &tt);
  else soft_rates<SUBG, H, O>(c, d, t, v, cit, hl, hi, R, pf.cf, rainfr, hr, orr);
  if (SUR && !soft && sur) slow_rates_from(c, t, v, hi, sur, R);
  aggregate<H, O>(c, t, v, lvfact, lsfact, R, A, soft, hr, B, orr, ext);
}

// ICE4_STEPPING for one micro point (mode_ice4_stepping.F90:139-518).
// Returns the pass key (outer << 16 | inner-of-last-outer), 0 if capped.
// TS: the MRSTEP / TSTEP_TS time splitting (mode_ice4_stepping.F90:191-197,
// :387-453): per outer iteration (IITER) the state and time at its start; a
// pass ends early when the TSTEP_TS sub-step is used up or a mixing ratio has
// moved by MRSTEP since the start, for the first INB_ITER_MAX iterations.
template <bool SUR = false, bool SUBG = false, bool H = false, bool O = false, bool TS = false>
ICE3_HD unsigned int stepping(const Cst &c, const Derived &d, const double *__restrict__ lut, const PointFix &pf,
                              double dt, int max_passes, double *vart, const double *ext, double &cit,
                              double &rainfr, double &rrevav, double hl[4], double hi[4], bool &capped,
                              const double *sur = nullptr, const double *__restrict__ hlut = nullptr,
                              const OcndPt *op = nullptr)
{
  OcndRates OR{0.0, 1.0, 1.0, 0.0, 0.0};
  int nb_iter_max = 0;
  double ztstep = 0.0, tlast = 0.0;
  double z0rt[H ? NVH : NV];
  if (TS) {
    nb_iter_max = (int)c.NMAXITER_MICRO;
    if (c.TSTEP_TS != 0.0) {
      int nb = (int)(dt / c.TSTEP_TS);
      nb = nb > 1 ? nb : 1;
      ztstep = dt / nb;
      nb_iter_max = nb_iter_max > nb ? nb_iter_max : nb;
    }
  }
  constexpr int NVT = H ? NVH : NV;
  const double rsmin[NVH] = {0.0, c.V_RTMIN, c.C_RTMIN, c.R_RTMIN, c.I_RTMIN, c.S_RTMIN, c.G_RTMIN, c.H_RTMIN};
  HailRates HR;
  if (H) {
#pragma unroll
    for (int k = 0; k < NBH; ++k) HR.b[k] = 0.0;
#pragma unroll
    for (int k = 0; k < NRH; ++k) HR.t[k] = 0.0;
  }
  Rates R;
#pragma unroll
  for (int k = 0; k < NBU; ++k) R.bu[k] = 0.0;
#pragma unroll
  for (int k = 0; k < NRS; ++k) R.rs[k] = 0.0;
#pragma unroll
  for (int k = 0; k < NRG; ++k) R.rg[k] = 0.0;
  R.ssi = 0.0;
  double ztime = 0.0;
  int passes = 0, outer = 0, inner = 0;
  rrevav = 0.0;
  capped = false;
  // TT/exn, lsfact and lvfact are the IEEE quotients, as the Fortran's (the
  // LFEEDBACKT sub-step ends with th on TT/exn, and which side of TT the next
  // pass sees is decided by their rounding), formed by fm::fdiv_rn(2)
  const double zx = pf.zx;
  while (ltd(ztime, dt)) {
    ++outer;
    inner = 0;
    bool llcompute = true, soft = false;
    if (TS) {
      tlast = ztime;
#pragma unroll
      for (int v = 0; v < (H ? NVH : NV); ++v) z0rt[v] = vart[v];
    }
    while (llcompute) {
      if (passes >= max_passes) { capped = true; return 0u; }
      ++passes;
      ++inner;
      double zsum2 = vart[IRI] + vart[IRS] + vart[IRG];
      if (H) zsum2 += vart[IRH];
      const double zdev = (c.CPD + c.CPV * vart[IRV] + c.CL * (vart[IRC] + vart[IRR]) + c.CI * zsum2) * pf.exn;
      const double zzt = vart[ITH] * pf.exn;
      double lsfact, lvfact;     // the IEEE quotients (fdiv_rn2: one reciprocal, checked)
      fm::fdiv_rn2(c.LSTT + d.cpv_ci * (zzt - c.TT), c.LVTT + d.cpv_cl * (zzt - c.TT), zdev, lsfact, lvfact);
      double A[NVT], B[NVT];
      tendencies<SUR, SUBG, H, O>(c, d, lut, soft, pf, lvfact, lsfact, cit, zzt, vart, R, rainfr, hl, hi, A, B, sur,
                                  &HR, hlut, op, &OR, ext);    // A includes the external tendencies
      if (SUR) sur = nullptr;          // learned slow rates: first hard pass only
      double maxtime = dt - ztime;
      // B (the instantaneous changes) is zero on soft passes: no theta jump
      // across TT/exn, no B in the depletion limits and the state update
      if (d.lfeedbackt) {
        if (!soft && negd((vart[ITH] - zx) * (vart[ITH] + B[ITH] - zx))) maxtime = 0.;
        if (abs_gtp(A[ITH], 1.e-20)) {
          // the IEEE quotient only where it can be positive and below maxtime
          const double num = zx - B[ITH] - vart[ITH];
          const double e = quot_est(num, A[ITH]);
          if (!negd(e) && !est_above(e, maxtime)) {
            const double thr = fm::fdiv_rn(num, A[ITH]);
            if (pos(thr)) maxtime = dmin(maxtime, thr);
          }
        }
      }
      // MAX(MIN(maxtime, time to deplete), MNH_TINY) per limited species is
      // MAX(MIN over all of them, MNH_TINY); a species' IEEE quotient is only
      // formed where it can be below the running minimum
      bool limited = false;
      double mt_hi = maxtime + fabs(maxtime) * 0x1p-18;   // est_above's bound, updated with maxtime
#pragma unroll
      for (int v = 1; v < NVT; ++v) {
        if (ltd(A[v], -1.e-20) && gtp(vart[v], rsmin[v])) {
          limited = true;
          const double num = -(B[v] + vart[v]);
          if (!gtd(quot_est(num, A[v]), mt_hi)) {
            maxtime = dmin(maxtime, fm::fdiv_rn(num, A[v]));
            mt_hi = maxtime + fabs(maxtime) * 0x1p-18;
          }
        }
      }
      if (limited) maxtime = dmax(maxtime, c.MNH_TINY);
      if (!ltd(ztime + maxtime, dt)) llcompute = false;
      if (TS && outer < nb_iter_max) {
        if (c.TSTEP_TS != 0.0 && gtd(ztime + maxtime, tlast + ztstep)) {
          maxtime = tlast - ztime + ztstep;
          llcompute = false;
        }
        if (c.MRSTEP != 0.0) {
          double maxb = 0.0;
#pragma unroll
          for (int v = 1; v < (H ? NVH : NV); ++v) {
            const double thr = abs_gtp(A[v], 1.e-20) ? (copysign(1., A[v]) * c.MRSTEP + z0rt[v] - vart[v] - B[v]) / A[v]
                                                    : -1.;
            if (!negd(thr) && ltd(thr, maxtime) && (gtp(vart[v], rsmin[v]) || gtd(A[v], 0.0))) {
              maxtime = dmin(maxtime, thr);
              llcompute = false;
            }
            maxb = v == 1 ? fabs(B[v]) : dmax(maxb, fabs(B[v]));
          }
          if (gtd(maxb, c.MRSTEP)) {
            maxtime = 0.;
            llcompute = false;
          }
        }
      }
      // State update with separately rounded product and sums (no FMA
      // contraction): after a species is depleted, v + A*t + B leaves a
      // rounding residual, and whether it exceeds XRTMIN decides whether the
      // next pass is taken with a MNH_TINY step (:302-311).  At the 1000/s
      // cap of RCHONI that quantum moves 2.2e-13 kg/kg, so the rounding must
      // follow the un-contracted evaluation of the Fortran (and of the CPU
      // reference) rather than a fused multiply-add.
      if (soft) {
#pragma unroll
        for (int v = 0; v < NVT; ++v) vart[v] = add_rn(vart[v], mul_rn(A[v], maxtime));
      } else {
#pragma unroll
        for (int v = 0; v < NVT; ++v) vart[v] = add_rn(add_rn(vart[v], mul_rn(A[v], maxtime)), B[v]);
      }
      if (!pos(vart[IRI])) cit = 0.;
      ztime += maxtime;
      rrevav = R.bu[B_RREVAV];
      soft = true;
    }
  }
  return ((unsigned)outer << 16) | (unsigned)inner;
}

// Load of a read-only field (the read-only data path on the device).
ICE3_HD double ldp(const double *p, long i)
{
#if defined(__CUDA_ARCH__)
  return __ldg(p + i);
#else
  return p[i];
#endif
}

// One grid point of RAIN_ICE (rain_ice.F90:334-652 and the disabled tail
// :758-790): L/cph and LLMICRO, nucleation outside micro points, the ICE4
// sub-stepping, total tendencies and ICE4_CORRECT_NEGATIVITIES on the
// sources, written back in place.  Returns the pass key (0 for points
// outside LLMICRO or capped); `capped` reports a point that hit max_passes.
// H (NRR = 7): with hail (rht / rhs; the hail kernels at hlut).
// O (OCND2): the LOCND2 branches, with the TIWMX tables tw and the level
// heights / droplet concentrations of ocnd2_column() at ozz / oconc.
// TS: the MRSTEP / TSTEP_TS time splitting.
template <bool SUR = false, bool SUBG = false, bool H = false, bool O = false, bool TS = false>
ICE3_HD unsigned int rain_ice_point(const Cst &c, const Derived &d, const double *__restrict__ lut,
                                    const Ice3gbRainIceFields &f, long p, double dt, int max_passes, bool &capped,
                                    const double *sur = nullptr, const double *__restrict__ hlut = nullptr,
                                    const double *tw = nullptr, const double *ozz = nullptr,
                                    const double *oconc = nullptr)
{
  constexpr int NVT = H ? NVH : NV;
  const double inv_dt = 1.0 / dt;
  const bool lwarm = d.lwarm;
  const bool sigm = d.aucv_rc == 1 && d.prpdf == 0;
  const bool adju = d.aucv_rc == 2 || d.aucv_ri == 2;
  unsigned int key = 0u;
  capped = false;
  PointFix pf;
  pf.exn = ldp(f.exn, p);
  pf.rho = ldp(f.rhodref, p);
  pf.pres = ldp(f.pabs, p);
  pf.zx = fm::fdiv_rn(c.TT, pf.exn);
  const double th = ldp(f.tht, p), rv = ldp(f.rvt, p), rc = ldp(f.rct, p), rr = ldp(f.rrt, p);
  const double ri = ldp(f.rit, p), rs = ldp(f.rst, p), rg = ldp(f.rgt, p);
  const double exnref = ldp(f.exnref, p);
  double ths = f.ths[p], rvs = f.rvs[p], rcs = f.rcs[p], rrs = f.rrs[p], ris = f.ris[p], rss = f.rss[p],
         rgs = f.rgs[p];
  double cit = f.cit[p];
  const double rh = H ? ldp(f.rht, p) : 0.0;
  double rhs = H ? f.rhs[p] : 0.0;
  // rain_ice.F90:334-345 (L/cph without exner) and :370-381 (LLMICRO)
  const double zdev = c.CPD + c.CPV * rv + c.CL * (rc + rr) + c.CI * (H ? ri + rs + rg + rh : ri + rs + rg);
  const double t = th * pf.exn;
  // L_s / cph and L_v / cph for the total tendencies (one reciprocal for
  // both); the IEEE lsfact that nucleation's T-feedback limit needs outside
  // micro points is formed there
  const double ls_num = c.LSTT + d.cpv_ci * (t - c.TT), lv_num = c.LVTT + d.cpv_cl * (t - c.TT);
  OcndPt op;
  if (O) {
    op.tw = tw;
    op.ssio = ldp(f.ssio, p); op.ssiu = ldp(f.ssiu, p); op.ifr = ldp(f.ifr, p); op.icldfr = ldp(f.icldfr, p);
    op.zzz = ozz[p];
    op.conc = oconc[p];
  }
  // LLMICRO (OCND2: rain_ice.F90:347-363, the XFRMIN(12) / XFRMIN(13) thresholds)
  const bool micro = O ? (gtp(op.ssio, c.FRMIN12) || gtp(rc, c.FRMIN13) || gtp(rr, c.FRMIN13) || gtp(ri, c.FRMIN13) ||
                          gtp(rs, c.FRMIN13) || gtp(rg, c.FRMIN13) || (H && gtp(rh, c.FRMIN13)))
                       : (gtp(rc, c.C_RTMIN) || gtp(rr, c.R_RTMIN) || gtp(ri, c.I_RTMIN) || gtp(rs, c.S_RTMIN) ||
                          gtp(rg, c.G_RTMIN) || (H && gtp(rh, c.H_RTMIN)));
  const double izx = fm::frcp(zdev) * fm::frcp(exnref);
  const double lsx = ls_num * izx, lvx = lv_num * izx;
  // with a PRFR option the sub-stepping starts from the precipitation
  // fraction of prfr_column (rain_ice.F90:555-602, ICE4_PACK :326)
  const bool llrfr = d.llrfr;
  double evap = 0.0, rainfr = (SUBG && llrfr) ? f.rainfr[p] : 1.0;
  double zrvheni = 0.0;
  if (!micro) {
    cit = 0.0;
    if (O) nucleation_ocnd2(c, op, t, rv, cit, zrvheni);
    else nucleation(c, d, th, pf.pres, pf.rho, pf.zx, fm::fdiv_rn(fm::fdiv_rn(ls_num, zdev), pf.exn), t, rv, cit, zrvheni);
  }
  zrvheni = dmin(rvs, zrvheni * inv_dt);
  if (micro) {
    pf.lrho = fm::flog(pf.rho);
    pf.rho_mcexvt = fm::fexp(-c.CEXVT * pf.lrho);
    const double irho = fm::frcp(pf.rho);
    pf.rho_mcexvt1 = pf.rho_mcexvt * irho;
    pf.rcrautc = c.CRIAUTC * irho;
    pf.cf = ldp(f.cldfr, p);
    pf.sigma_rc = sigm ? 2.0 * ldp(f.sigs, p) : 0.0;
    double vart[NVT], ext[NVT];
    vart[ITH] = th; vart[IRV] = rv; vart[IRC] = rc; vart[IRR] = rr; vart[IRI] = ri; vart[IRS] = rs; vart[IRG] = rg;
    ext[ITH] = ths - th * inv_dt; ext[IRV] = rvs - rv * inv_dt; ext[IRC] = rcs - rc * inv_dt;
    ext[IRR] = rrs - rr * inv_dt; ext[IRI] = ris - ri * inv_dt; ext[IRS] = rss - rs * inv_dt;
    ext[IRG] = rgs - rg * inv_dt;
    if (H) {
      vart[NVT - 1] = rh;
      ext[NVT - 1] = rhs - rh * inv_dt;
    }
    double hl[4] = {0.0, 0.0, 0.0, 0.0}, hi[4] = {0.0, 0.0, 0.0, 0.0};
    if (adju) {
      hl[0] = f.hlc_hcf[p]; hl[2] = f.hlc_hrc[p]; hi[0] = f.hli_hcf[p]; hi[2] = f.hli_hri[p];
      hl[3] = rc - hl[2];
      hi[3] = ri - hi[2];
      hl[1] = pos(rc) ? pf.cf - hl[0] : 0.;
      hi[1] = pos(ri) ? pf.cf - hi[0] : 0.;
    }
    double rrevav;
    key = stepping<SUR, SUBG, H, O, TS>(c, d, lut, pf, dt, max_passes, vart, ext, cit, rainfr, rrevav, hl, hi,
                                        capped, sur, hlut, &op);
#pragma unroll
    for (int v = 0; v < NVT; ++v) vart[v] -= ext[v] * dt;
    evap = lwarm ? rrevav : 0.0;
    // total tendencies (rain_ice.F90:758-790).  The state at t and the
    // sources are read again here instead of being kept live across the
    // sub-stepping (the point's inputs are unchanged until its results are
    // written below): 13 values the register allocator would otherwise spill.
    const double rv0 = ldp(f.rvt, p), rc0 = ldp(f.rct, p), rr0 = ldp(f.rrt, p);
    const double ri0 = ldp(f.rit, p), rs0 = ldp(f.rst, p), rg0 = ldp(f.rgt, p);
    ths = f.ths[p]; rvs = f.rvs[p]; rcs = f.rcs[p]; rrs = f.rrs[p]; ris = f.ris[p]; rss = f.rss[p]; rgs = f.rgs[p];
    if (H) rhs = f.rhs[p];
    const double wv = (vart[IRV] - rv0) * inv_dt, wc = (vart[IRC] - rc0) * inv_dt;
    const double wr = (vart[IRR] - rr0) * inv_dt, wi = (vart[IRI] - ri0) * inv_dt;
    const double ws = (vart[IRS] - rs0) * inv_dt, wg = (vart[IRG] - rg0) * inv_dt;
    const double wh = H ? (vart[NVT - 1] - ldp(f.rht, p)) * inv_dt : 0.0;
    ths += (wc + wr) * lvx + (H ? wi + ws + wg + wh : wi + ws + wg) * lsx + zrvheni * lsx;
    if (H) rhs += wh;
    rvs += wv - zrvheni;
    rcs += wc;
    rrs += wr;
    ris += wi + zrvheni;
    rss += ws;
    rgs += wg;
  } else {
    ths += zrvheni * lsx;
    rvs -= zrvheni;
    ris += zrvheni;
  }
  // ICE4_CORRECT_NEGATIVITIES (mode_ice4_correct_negativities.F90) on the
  // sources, in blocks a warp skips when every lane would move nothing: the
  // negative sources back to vapour, one species at a time (a warp holds
  // negative sources of about 1.6 of the 5 species); cloud and ice to vapour
  // while the vapour source is below XRTMIN(1); then rain, snow, graupel
  double w;
  if (warp_any(negd(rcs))) { w = rcs - pmax0(rcs); rvs += w; ths -= w * lvx; rcs -= w; }
  if (warp_any(negd(rrs))) { w = rrs - pmax0(rrs); rvs += w; ths -= w * lvx; rrs -= w; }
  if (warp_any(negd(ris))) { w = ris - pmax0(ris); rvs += w; ths -= w * lsx; ris -= w; }
  if (warp_any(negd(rss))) { w = rss - pmax0(rss); rvs += w; ths -= w * lsx; rss -= w; }
  if (warp_any(negd(rgs))) { w = rgs - pmax0(rgs); rvs += w; ths -= w * lsx; rgs -= w; }
  if (H && warp_any(negd(rhs))) { w = rhs - pmax0(rhs); rvs += w; ths -= w * lsx; rhs -= w; }
  if (warp_any(ltd(rvs, c.V_RTMIN))) {
    w = dmin(1., fm::fdiv(pmax0(c.V_RTMIN - rvs), dmax(rcs + ris, 1.e-20)));
    ths -= w * (rcs * lvx + ris * lsx);
    rvs += w * (rcs + ris);
    rcs = (1. - w) * rcs;
    ris = (1. - w) * ris;
    if (warp_any(ltd(rvs, c.V_RTMIN))) {
      w = dmin(pmax0(rrs), pmax0(c.V_RTMIN - rvs)); rvs += w; rrs -= w; ths -= w * lvx;
      w = dmin(pmax0(rss), pmax0(c.V_RTMIN - rvs)); rvs += w; rss -= w; ths -= w * lsx;
      w = dmin(pmax0(rgs), pmax0(c.V_RTMIN - rvs)); rvs += w; rgs -= w; ths -= w * lsx;
      if (H) { w = dmin(pmax0(rhs), pmax0(c.V_RTMIN - rvs)); rvs += w; rhs -= w; ths -= w * lsx; }
    }
  }
  f.ths[p] = ths; f.rvs[p] = rvs; f.rcs[p] = rcs; f.rrs[p] = rrs; f.ris[p] = ris; f.rss[p] = rss;
  f.rgs[p] = rgs;
  if (H) f.rhs[p] = rhs;
  f.cit[p] = cit;
  f.evap3d[p] = evap;
  f.rainfr[p] = rainfr;
  return key;
}

// The precipitation fraction a rain_ice call with a PRFR option starts from
// (rain_ice.F90:555-605), for one column: ICE4_COMPUTE_PDF on the time-t
// state of each micro point (its partition overwrites hlc_hcf / hlc_hrc /
// hli_hcf / hli_hri, as the Fortran's INOUT arguments; outside micro points
// the masked form: zeros, ADJU keeps the fractions), then ICE4_RAINFR_VERT
// from the top level down (mode_ice4_rainfr_vert.F90: 0 at the top, the
// maximum with the level above where rain, snow or graupel is present, 1 if
// that is 0, else 0).  Writes f.rainfr of the column.
template <bool H = false>
ICE3_HD void prfr_column(const Cst &c, const Ice3gbRainIceFields &f, long nij, int nk, long col)
{
  Derived d;
  make_derived(c, d);
  const int aucv_rc = d.aucv_rc, aucv_ri = d.aucv_ri;
  const bool sigm = aucv_rc == 1 && (int)c.SUBG_PR_PDF == 0;
  const bool adju = aucv_rc == 2 || aucv_ri == 2;
  double above = 0.0;
  for (int k = nk - 1; k >= 0; --k) {
    const long p = (long)k * nij + col;
    const double rc = ldp(f.rct, p), rr = ldp(f.rrt, p), ri = ldp(f.rit, p), rs = ldp(f.rst, p);
    const double rg = ldp(f.rgt, p), cf = ldp(f.cldfr, p);
    const bool has_h = H && gtp(ldp(f.rht, p), c.H_RTMIN);
    const bool micro = gtp(rc, c.C_RTMIN) || gtp(rr, c.R_RTMIN) || gtp(ri, c.I_RTMIN) || gtp(rs, c.S_RTMIN) ||
                       gtp(rg, c.G_RTMIN) || has_h;
    double hl[4] = {f.hlc_hcf[p], 0.0, f.hlc_hrc[p], 0.0}, hi[4] = {f.hli_hcf[p], 0.0, f.hli_hri[p], 0.0};
    if (adju) {                                                    // rain_ice.F90:564-581
      hl[3] = rc - hl[2];
      hi[3] = ri - hi[2];
      hl[1] = pos(rc) ? cf - hl[0] : 0.;
      hi[1] = pos(ri) ? cf - hi[0] : 0.;
    }
    double rf = 0.0;
    if (micro) {
      const double sig = sigm ? ldp(f.sigs, p) : 0.0;
      const double rho = ldp(f.rhodref, p);
      double criauti;
      rf = compute_pdf(c, d, c.CRIAUTC / rho, rc, ri, cf, ldp(f.tht, p) * ldp(f.exn, p), sig * sig, hl, hi, criauti);
    } else {
      if (aucv_rc != 2) hl[0] = 0.0;
      hl[2] = 0.0;
      if (aucv_ri != 2) hi[0] = 0.0;
      hi[2] = 0.0;
    }
    f.hlc_hcf[p] = hl[0]; f.hlc_hrc[p] = hl[2]; f.hli_hcf[p] = hi[0]; f.hli_hri[p] = hi[2];
    double pr = 0.0;
    if (k < nk - 1 && (gtp(rr, c.R_RTMIN) || gtp(rs, c.S_RTMIN) || gtp(rg, c.G_RTMIN) || has_h)) {
      pr = dmax(rf, above);
      if (zerod(pr)) pr = 1.0;
    }
    f.rainfr[p] = pr;
    above = pr;
  }
}

}  // namespace ice3pt
