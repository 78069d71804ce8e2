// ice_adjust.cu — saturation adjustment with CB02 subgrid condensation.
//
// Restates src/ice3/jax/stencils/ice_adjust.py:26-398 (IceAdjustJAX) for one
// grid point per lane; each thread owns two consecutive points so every field
// moves with one 128-bit load/store (LDG.128/STG.128).  Pure map over the
// nij*nk points: 19 3-D fields read (+ sigqsat per column), 16 written,
// 280 algorithmic bytes per point.
#include "ice3gb_device.cuh"
#include "ice3gb_kernels.h"

namespace {

struct IaIn {
  double sigqsat, pabs, sigs, th, exn, exn_ref, rho, rv, rc, ri, rr, rs, rg, cf_mf, rc_mf, ri_mf;
  double rvs, rcs, ris, ths;
};
struct IaOut {
  double t, rv_out, rc_out, ri_out, cldfr, hlc_hrc, hlc_hcf, hli_hri, hli_hcf, cph, lv, ls;
  double rvs, rcs, ris, ths;
};

// Triangle-PDF subgrid autoconversion (stencils/ice_adjust.py:316-341).
ICE3_HD void triangle_pdf(double w_dt, double crit, double cf_mf, double &hcf, double &hr)
{
  const double wmax = nmax(1e-20, w_dt);
  const double inv_w2 = fm::frcp(sq(wmax));
  if (fgt(w_dt, crit)) {
    const double cc = crit * cf_mf;
    hcf = 1.0 - 0.5 * sq(cc) * inv_w2;
    hr = w_dt - cc * cc * cc * (inv_w2 * (1.0 / 3.0));
  } else if (fge(crit, 2.0 * w_dt)) {
    hcf = 0.0;
    hr = 0.0;
  } else {
    hcf = 0.5 * sq(2.0 * w_dt - crit) * inv_w2;
    hr = (4.0 * w_dt * w_dt * w_dt - 3.0 * w_dt * sq(crit) + crit * crit * crit) * (inv_w2 * (1.0 / 3.0));
  }
  hcf *= cf_mf;
}

// Constants derived once per thread (divisions of table constants).
struct IaDerived {
  double rdrv, rvrd, irv;   // RD/RV, RV/RD, 1/RV
};
ICE3_HD IaDerived ia_derived(const Cst &c) { return {c.RD / c.RV, c.RV / c.RD, 1.0 / c.RV}; }

ICE3_HD void ia_point(const Cst &c, const IaDerived &d, double dt, double inv_dt, const IaIn &x, IaOut &o)
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
    const double rt = x.rv + x.rc + x.ri;
    // es_w and es_i share fm::flog(T) and 1/T (functions/tiwmx.py:18,60)
    const double lt = fm::flog(t), it = fm::frcp(t);
    const double pv = nmin(fm::fexp(c.ALPW - c.BETAW * it - c.GAMW * lt), 0.99 * x.pabs);
    const double piv = nmin(fm::fexp(c.ALPI - c.BETAI * it - c.GAMI * lt), 0.99 * x.pabs);
    double frac = fgt(x.rc + x.ri, 1e-20) ? fm::fdiv(x.rc, x.rc + x.ri) : 0.0;
    const int fmode = (int)c.FRAC_ICE_ADJUST;
    if (fmode == 3) frac = nclip01(frac);
    else if (fmode == 0) frac = nclip01(fm::fdiv(c.TMAXMIX - t, c.TMAXMIX - c.TMINMIX));
    double qsl = fm::fdiv(d.rdrv * pv, x.pabs - pv);
    const double qsi = fm::fdiv(d.rdrv * piv, x.pabs - piv);
    qsl = (1.0 - frac) * qsl + frac * qsi;
    const double lvs = (1.0 - frac) * lv + frac * ls;
    const double ah = lvs * qsl * (it * it * d.irv) * (1.0 + qsl * d.rvrd);
    const double a = fm::frcp(1.0 + lvs * inv_cph * ah);
    const double sbar = a * (rt - qsl + ah * lvs * (x.rc + x.ri) * inv_cph);
    double sigma;
    if (c.LSIGMAS != 0.0 && c.LSTATNW == 0.0)
      sigma = !(fge(x.sigqsat, 0.0) && fge(0.0, x.sigqsat)) ? sqrt(sq(2.0 * x.sigs) + sq(x.sigqsat * qsl * a))
                                                             : 2.0 * x.sigs;
    else
      sigma = 2.0 * x.sigs;
    sigma = nmax(1e-10, sigma);
    const double q1 = fm::fdiv(sbar, sigma);
    double cond;
    if (fgt(q1, 0.0)) cond = fge(2.0, q1) ? nmin(0.36787944117144233 + 0.66 * q1 + 0.086 * q1 * q1, 2.0) : q1;
    else cond = fm::fexp(1.2 * q1 - 1.0);
    cond *= sigma;
    cldfr = fge(cond, 1e-12) ? nclip01(0.5 + 0.36 * fm::fatan(1.55 * q1)) : 0.0;
    if (fge(cldfr, 0.0) && fge(0.0, cldfr)) cond = 0.0;
    rc_out = (1.0 - frac) * cond;
    ri_out = frac * cond;
    t = t + ((rc_out - x.rc) * lv + (ri_out - x.ri) * ls) * inv_cph;
    rv_out = rt - rc_out - ri_out;
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
      const double criaut = fm::fdiv(c.CRIAUTC, x.rho);
      const double criaut_i = nmin(c.CRIAUTI, fm::fexp10(c.ACRIAUTI * (t - c.TT) + c.BCRIAUTI));
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

// Two points per thread, double2 loads/stores; requires an even point count
// and 16-byte aligned fields (checked by the host).  ADV: the state adjusted
// is adv_dt times the sources (th = dt*ths, r = dt*rs, the state after the
// microphysics in the chained physics step) instead of th/rv/.../rg, which
// are then not read; rrs/rss/rgs are read instead.  Output pointers may be
// NULL in the internal chained use (store skipped).
template <bool ADV>
__global__ void __launch_bounds__(256) ice_adjust_v2_kernel(const __grid_constant__ Cst c,
                                                            const __grid_constant__ IaKernelFields kf,
                                                            long npairs, int nij, double dt)
{
  const Ice3gbIceAdjustFields &f = kf.f;
  const double inv_dt = 1.0 / dt;
  const IaDerived d = ia_derived(c);
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < npairs; q += (long)gridDim.x * blockDim.x) {
    const long p = 2 * q;
    IaIn x0, x1;
#define LD2(field, name)                 \
  {                                      \
    const double2 v = ld2(f.field, p);   \
    x0.name = v.x;                       \
    x1.name = v.y;                       \
  }
    LD2(pabs, pabs) LD2(sigs, sigs) LD2(exn, exn) LD2(exn_ref, exn_ref) LD2(rho_dry_ref, rho)
    LD2(cf_mf, cf_mf) LD2(rc_mf, rc_mf) LD2(ri_mf, ri_mf)
    LD2(rvs, rvs) LD2(rcs, rcs) LD2(ris, ris) LD2(ths, ths)
    if (ADV) {
      const double a = kf.adv_dt;
      const double2 vr = ld2(kf.rrs, p), vs = ld2(kf.rss, p), vg = ld2(kf.rgs, p);
      x0.th = a * x0.ths; x1.th = a * x1.ths;
      x0.rv = a * x0.rvs; x1.rv = a * x1.rvs;
      x0.rc = a * x0.rcs; x1.rc = a * x1.rcs;
      x0.ri = a * x0.ris; x1.ri = a * x1.ris;
      x0.rr = a * vr.x;   x1.rr = a * vr.y;
      x0.rs = a * vs.x;   x1.rs = a * vs.y;
      x0.rg = a * vg.x;   x1.rg = a * vg.y;
    } else {
      LD2(th, th) LD2(rv, rv) LD2(rc, rc) LD2(ri, ri) LD2(rr, rr) LD2(rs, rs) LD2(rg, rg)
    }
#undef LD2
    if (f.sigqsat_3d) {
      const double2 v = ld2(f.sigqsat, p);
      x0.sigqsat = v.x;
      x1.sigqsat = v.y;
    } else {
      x0.sigqsat = ld1(f.sigqsat, p % nij);
      x1.sigqsat = ld1(f.sigqsat, (p + 1) % nij);
    }
    IaOut o0, o1;
    ia_point(c, d, dt, inv_dt, x0, o0);
    ia_point(c, d, dt, inv_dt, x1, o1);
#define ST2(field) if (f.field) st2(f.field, p, o0.field, o1.field);
    ST2(t) ST2(rv_out) ST2(rc_out) ST2(ri_out) ST2(cldfr) ST2(hlc_hrc) ST2(hlc_hcf) ST2(hli_hri) ST2(hli_hcf)
    ST2(cph) ST2(lv) ST2(ls) ST2(rvs) ST2(rcs) ST2(ris) ST2(ths)
#undef ST2
  }
}

// Scalar path: odd point counts or unaligned fields.
template <bool ADV>
__global__ void __launch_bounds__(256) ice_adjust_v1_kernel(const __grid_constant__ Cst c,
                                                            const __grid_constant__ IaKernelFields kf,
                                                            long n, int nij, double dt)
{
  const Ice3gbIceAdjustFields &f = kf.f;
  const double inv_dt = 1.0 / dt;
  const IaDerived d = ia_derived(c);
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < n; p += (long)gridDim.x * blockDim.x) {
    IaIn x;
    x.sigqsat = f.sigqsat_3d ? ld1(f.sigqsat, p) : ld1(f.sigqsat, p % nij);
    x.pabs = ld1(f.pabs, p); x.sigs = ld1(f.sigs, p); x.exn = ld1(f.exn, p);
    x.exn_ref = ld1(f.exn_ref, p); x.rho = ld1(f.rho_dry_ref, p);
    x.cf_mf = ld1(f.cf_mf, p); x.rc_mf = ld1(f.rc_mf, p); x.ri_mf = ld1(f.ri_mf, p);
    x.rvs = f.rvs[p]; x.rcs = f.rcs[p]; x.ris = f.ris[p]; x.ths = f.ths[p];
    if (ADV) {
      const double a = kf.adv_dt;
      x.th = a * x.ths; x.rv = a * x.rvs; x.rc = a * x.rcs; x.ri = a * x.ris;
      x.rr = a * ld1(kf.rrs, p); x.rs = a * ld1(kf.rss, p); x.rg = a * ld1(kf.rgs, p);
    } else {
      x.th = ld1(f.th, p); x.rv = ld1(f.rv, p); x.rc = ld1(f.rc, p); x.ri = ld1(f.ri, p);
      x.rr = ld1(f.rr, p); x.rs = ld1(f.rs, p); x.rg = ld1(f.rg, p);
    }
    IaOut o;
    ia_point(c, d, dt, inv_dt, x, o);
#define ST1(field) if (f.field) f.field[p] = o.field;
    ST1(t) ST1(rv_out) ST1(rc_out) ST1(ri_out) ST1(cldfr) ST1(hlc_hrc) ST1(hlc_hcf) ST1(hli_hri) ST1(hli_hcf)
    ST1(cph) ST1(lv) ST1(ls) ST1(rvs) ST1(rcs) ST1(ris) ST1(ths)
#undef ST1
  }
}

}  // namespace

cudaError_t launch_ice_adjust(const Cst &c, const IaKernelFields &kf, int nij, int nk, double dt, bool vec2,
                              int num_sms, cudaStream_t s)
{
  const long n = (long)nij * nk;
  const int threads = 256;
  const long cap = (long)num_sms * 64;
  const bool adv = kf.adv_dt != 0.0;
  if (vec2) {
    const long npairs = n / 2;
    long blocks = (npairs + threads - 1) / threads;
    if (blocks > cap) blocks = cap;
    if (adv) ice_adjust_v2_kernel<true><<<(unsigned)blocks, threads, 0, s>>>(c, kf, npairs, nij, dt);
    else ice_adjust_v2_kernel<false><<<(unsigned)blocks, threads, 0, s>>>(c, kf, npairs, nij, dt);
  } else {
    long blocks = (n + threads - 1) / threads;
    if (blocks > cap) blocks = cap;
    if (adv) ice_adjust_v1_kernel<true><<<(unsigned)blocks, threads, 0, s>>>(c, kf, n, nij, dt);
    else ice_adjust_v1_kernel<false><<<(unsigned)blocks, threads, 0, s>>>(c, kf, n, nij, dt);
  }
  return cudaGetLastError();
}
