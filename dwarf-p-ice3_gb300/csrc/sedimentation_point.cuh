// sedimentation_point.cuh — fall speeds and cloud parameters of the
// statistical sedimentation (ICE4_SEDIMENTATION_STAT,
// mode_ice4_sedimentation_stat.F90 and src/ice3/jax/stencils/sedimentation.py),
// shared by the forward sweep (sedimentation.cu), its adjoint
// (sedimentation_vjp.cu) and the host builds of the tests.
#pragma once

#include "ice3gb_device.cuh"

namespace ice3sed {

struct CloudPar {
  double log_lbc_conc, ray_inv, fsedc;
};

ICE3_HD CloudPar cloud_params(const Cst &c, bool fortran, bool has_st, double sea, double town)
{
  double lbc, fsedc, conc, ray;
  if (fortran) {
    const double gac_gc = c.GAC / c.GC, gac2_gc2 = c.GAC2 / c.GC2;
    if (has_st) {
      ray = fmax(1.0, 0.5 * ((1.0 - sea) * gac_gc + sea * gac2_gc2));
      lbc = fmax(fmin(c.LBC_1, c.LBC_2), sea * c.LBC_2 + (1.0 - sea) * c.LBC_1);
      fsedc = fmax(fmin(c.FSEDC_1, c.FSEDC_2), sea * c.FSEDC_2 + (1.0 - sea) * c.FSEDC_1);
      conc = (1.0 - town) * (sea * c.CONC_SEA + (1.0 - sea) * c.CONC_LAND) + town * c.CONC_URBAN;
    } else {
      ray = fmax(1.0, 0.5 * gac_gc);
      lbc = c.LBC_1;
      fsedc = c.FSEDC_1;
      conc = c.CONC_LAND;
    }
  } else {
    ray = 1.0;
    lbc = (1.0 - sea) * c.LBC_1 + sea * c.LBC_2;
    fsedc = (1.0 - sea) * c.FSEDC_1 + sea * c.FSEDC_2;
    conc = (1.0 - town) * ((1.0 - sea) * c.CONC_LAND + sea * c.CONC_SEA) + town * c.CONC_URBAN;
  }
  CloudPar p;
  p.log_lbc_conc = fm::flog(lbc * conc);
  p.ray_inv = 1.0 / ray;
  p.fsedc = fsedc;
  return p;
}

// The exponents (EXSED - 1, EXSED - CEXVT - 1) of rain, snow, graupel and
// hail at [2 s], [2 s + 1] (the others unused), formed once per block by
// the device sweep instead of per fall speed; the same values as in place.
ICE3_HD void fall_exponents(const Cst &c, double fx[12])
{
  const double ex[6] = {0.0, c.EXSEDR, 0.0, c.EXSEDS, c.EXSEDG, c.EXSEDH};
  for (int s = 0; s < 6; ++s) {
    fx[2 * s] = ex[s] - 1.0;
    fx[2 * s + 1] = ex[s] - c.CEXVT - 1.0;
  }
}

// The power-law fall speed F r^a rho^b = F exp(a log r + b log rho) of rain,
// snow, graupel and hail (a = EXSED - 1, b = EXSED - CEXVT - 1), the sum of
// products fused as fma(a, log r, b log rho) wherever it is formed.
ICE3_HD double power_speed(double f, double a, double b, double lr, double lrho)
{
  return f * fm::fexp(fm::fma_(a, lr, b * lrho));
}

// Fall speed for content r (> threshold checked by the caller); lrho = log(rho).
// fx: the exponents of fall_exponents, or null to form them here.
ICE3_HD double fall_speed(const Cst &c, int s, double r, double lrho, double wlbda, const CloudPar &cp,
                          const double *fx = nullptr)
{
  const double lr = fm::flog(r);
  switch (s) {
    case 0: {  // cloud droplets: sedimentation.py:206-209, F90:264-267
      const double lwlbdc = c.LBEXC * (cp.log_lbc_conc - lrho - lr);
      const double cc = c.CC * (1.0 + 1.26 * wlbda * fm::fexp(lwlbdc) * cp.ray_inv);
      return fm::fexp(-c.CEXVT * lrho - c.DC * lwlbdc) * cc * cp.fsedc;
    }
    case 1:  // rain
      return power_speed(c.FSEDR, fx ? fx[2] : c.EXSEDR - 1.0, fx ? fx[3] : c.EXSEDR - c.CEXVT - 1.0, lr, lrho);
    case 2: {  // pristine ice: sedimentation.py:46-55, F90:307-311
      const double dmax_ = dmax(0.05e6, -0.15319e6 - 0.021454e6 * (lrho + lr));
      return c.FSEDI * fm::fexp(-c.CEXVT * lrho + c.EXCSEDI * fm::flog(dmax_));
    }
    case 3:  // snow
      return power_speed(c.FSEDS, fx ? fx[6] : c.EXSEDS - 1.0, fx ? fx[7] : c.EXSEDS - c.CEXVT - 1.0, lr, lrho);
    case 5:  // hail (NRR = 7): OTHER_SPECIES with XFSEDH / XEXSEDH, F90:186-187
      return power_speed(c.FSEDH, fx ? fx[10] : c.EXSEDH - 1.0, fx ? fx[11] : c.EXSEDH - c.CEXVT - 1.0, lr, lrho);
    default:  // graupel
      return power_speed(c.FSEDG, fx ? fx[8] : c.EXSEDG - 1.0, fx ? fx[9] : c.EXSEDG - c.CEXVT - 1.0, lr, lrho);
  }
}


// Fall speed as fall_speed() (same operations, same value) with its partial
// derivatives with respect to log r, log rho and wlbda.
ICE3_HD double fall_speed_d(const Cst &c, int s, double r, double lrho, double wlbda, const CloudPar &cp, double &d_lr,
                            double &d_lrho, double &d_wl)
{
  const double lr = fm::flog(r);
  d_wl = 0.0;
  switch (s) {
    case 0: {
      const double lwlbdc = c.LBEXC * (cp.log_lbc_conc - lrho - lr);
      const double e2 = fm::fexp(lwlbdc);
      const double cc = c.CC * (1.0 + 1.26 * wlbda * e2 * cp.ray_inv);
      const double e1 = fm::fexp(-c.CEXVT * lrho - c.DC * lwlbdc);
      const double v = e1 * cc * cp.fsedc;
      // dv/dlwlbdc = e1 fsedc CC (-DC (1 + 1.26 wlbda e2 ray_inv) + 1.26 wlbda e2 ray_inv)
      const double d_lw = e1 * cp.fsedc * c.CC * (-c.DC * (1.0 + 1.26 * wlbda * e2 * cp.ray_inv) +
                                                  1.26 * wlbda * e2 * cp.ray_inv);
      d_lr = -c.LBEXC * d_lw;
      d_lrho = -c.CEXVT * v - c.LBEXC * d_lw;
      d_wl = e1 * cp.fsedc * c.CC * 1.26 * e2 * cp.ray_inv;
      return v;
    }
    case 2: {
      bool first;
      const double arg = -0.15319e6 - 0.021454e6 * (lrho + lr);
      first = gtd(0.05e6, arg);
      const double dmax_ = first ? 0.05e6 : arg;
      const double v = c.FSEDI * fm::fexp(-c.CEXVT * lrho + c.EXCSEDI * fm::flog(dmax_));
      const double dld = first ? 0.0 : -0.021454e6 / dmax_;
      d_lr = v * c.EXCSEDI * dld;
      d_lrho = v * (-c.CEXVT + c.EXCSEDI * dld);
      return v;
    }
    default: {
      double fsed, ex;
      if (s == 1) { fsed = c.FSEDR; ex = c.EXSEDR; }
      else if (s == 3) { fsed = c.FSEDS; ex = c.EXSEDS; }
      else { fsed = c.FSEDG; ex = c.EXSEDG; }
      const double v = power_speed(fsed, ex - 1.0, ex - c.CEXVT - 1.0, lr, lrho);
      d_lr = (ex - 1.0) * v;
      d_lrho = (ex - c.CEXVT - 1.0) * v;
      return v;
    }
  }
}

// Fields of one sedimentation sweep; element (k, col) at k * nij + col.
struct SedColumnIO {
  const double *rhodref, *dzz, *pabs, *tht;
  const double *src_in[5];   // sources read (rcs, rrs, ris, rss, rgs)
  double *src_out[5];        // updated sources (may alias src_in), or NULL
  double *fpr[5];            // fluxes F_k, or NULL
  double *inpr[5];           // [nij] surface precipitation, or NULL
  long nij;
  int nk;
};

ICE3_HD double sed_rtmin(const Cst &c, int s)
{
  return (s == 0) ? c.C_RTMIN : (s == 1) ? c.R_RTMIN : (s == 2) ? dmax(c.I_RTMIN, 1.0e-7) : (s == 3) ? c.S_RTMIN
                                                                                     : (s == 4) ? c.G_RTMIN
                                                                                                : c.H_RTMIN;
}

ICE3_HD double sed_load(const double *p, long i)
{
#if defined(__CUDA_ARCH__)
  return __ldg(p + i);
#else
  return p[i];
#endif
}

// Top-down sweep of one column (mode_ice4_sedimentation_stat.F90:143-229,
// sedimentation.py:58-352): the five species side by side, the flux from the
// level above carried in a register.  skip_c: PHYEX's LSEDIC = .FALSE.
// (cloud not sedimented, its outputs left to the caller).
ICE3_HD void sed_column_forward(const Cst &c, bool fortran, bool skip_c, const CloudPar &cp, double dt,
                                const SedColumnIO &io, long col)
{
  const double inv_dt = 1.0 / dt;
  double rtmin[5];
#pragma unroll
  for (int s = 0; s < 5; ++s) rtmin[s] = sed_rtmin(c, s);
  double fabove[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int k = io.nk - 1; k >= 0; --k) {
    const long p = (long)k * io.nij + col;
    const double rho = sed_load(io.rhodref, p), dz = sed_load(io.dzz, p);
    const double rhodz = rho * dz;
    const double tsorhodz = fm::fdiv(dt, rhodz);
    double src[5], rt[5], qp[5];
    bool c1[5], c2[5];
    bool any = false;
#pragma unroll
    for (int s = 0; s < 5; ++s) {
      if (s == 0 && skip_c) { c1[s] = c2[s] = false; src[s] = rt[s] = qp[s] = 0.0; continue; }
      src[s] = io.src_in[s][p];
      rt[s] = src[s] * dt;
      qp[s] = fabove[s] * tsorhodz;
      c1[s] = gtp(rt[s], rtmin[s]);
      c2[s] = gtp(qp[s], rtmin[s]);
      any = any || c1[s] || c2[s];
    }
    const double lrho = any ? fm::flog(rho) : 0.0;
    const double wlbda =
        (c1[0] || c2[0]) ? 6.6e-8 * fm::fdiv(101325.0, sed_load(io.pabs, p)) * (sed_load(io.tht, p) * (1.0 / 293.15))
                         : 0.0;
#pragma unroll
    for (int s = 0; s < 5; ++s) {
      if (s == 0 && skip_c) continue;
      const double w1 = c1[s] ? fall_speed(c, s, rt[s], lrho, wlbda, cp) : 0.0;
      const double w2 = c2[s] ? fall_speed(c, s, qp[s], lrho, wlbda, cp) : 0.0;
      double flux = dmin(rhodz * rt[s] * inv_dt, w1 * rho * rt[s]);
      if (!zerod_(w2)) flux += pmax0(1.0 - fm::fdiv(dz, dt * w2)) * fabove[s];
      if (io.src_out[s]) {
        if (fortran) io.src_out[s][p] = src[s] + tsorhodz * (fabove[s] - flux) * inv_dt;
        else io.src_out[s][p] = src[s] + fm::fdiv(fabove[s] - flux, rhodz * dt);
      }
      if (io.fpr[s]) io.fpr[s][p] = flux;
      fabove[s] = flux;
    }
  }
#pragma unroll
  for (int s = 0; s < 5; ++s)
    if (!(s == 0 && skip_c) && io.inpr[s]) io.inpr[s][col] = fabove[s] / c.RHOLW;
}

// Hail in the statistical sweep (NRR = 7; species 7 of
// mode_ice4_sedimentation_stat.F90:186-222, Fortran semantics) for one
// column: the hail content is rhs * dt (mode_ice4_sedimentation.F90:179).
ICE3_HD void sed_hail_column(const Cst &c, double dt, const double *rhodref, const double *dzz, double *rhs,
                             double *fpr, double *inpr, long nij, int nk, long col)
{
  const double inv_dt = 1.0 / dt;
  const CloudPar cp{};
  double fabove = 0.0;
  for (int k = nk - 1; k >= 0; --k) {
    const long p = (long)k * nij + col;
    const double rho = sed_load(rhodref, p), dz = sed_load(dzz, p);
    const double rhodz = rho * dz;
    const double tsorhodz = fm::fdiv(dt, rhodz);
    const double src = rhs[p], rt = src * dt, qp = fabove * tsorhodz;
    const bool c1 = gtp(rt, c.H_RTMIN), c2 = gtp(qp, c.H_RTMIN);
    const double lrho = (c1 || c2) ? fm::flog(rho) : 0.0;
    const double w1 = c1 ? fall_speed(c, 5, rt, lrho, 0.0, cp) : 0.0;
    const double w2 = c2 ? fall_speed(c, 5, qp, lrho, 0.0, cp) : 0.0;
    double flux = dmin(rhodz * rt * inv_dt, w1 * rho * rt);
    if (!zerod_(w2)) flux += pmax0(1.0 - fm::fdiv(dz, dt * w2)) * fabove;
    rhs[p] = src + tsorhodz * (fabove - flux) * inv_dt;
    if (fpr) fpr[p] = flux;
    fabove = flux;
  }
  inpr[col] = fabove / c.RHOLW;
}

// Cotangents of the sweep's outputs (NULL = zero) and the wanted gradients
// of its inputs (NULL = not wanted), same layouts as SedColumnIO.
struct SedCotangents {
  const double *src[5];      // updated sources
  const double *inpr[5];     // [nij]
  const double *fpr[5];      // fluxes
};
struct SedGradients {
  double *src[5];            // input sources
  double *rhodref, *dzz, *pabs, *tht;
};

// Reverse sweep of one column (hand-written adjoint of sed_column_forward):
// bottom-up, carrying the cotangent of the flux entering each level from
// above.  `flux` holds the forward fluxes F_k of the column (io.fpr layout),
// recomputed by sed_column_forward just before.  Derivatives of the branch
// the forward took at the kinks (the min of the two flux bounds, the
// max(0, .) of the transfer factor, the thresholds rt, qp > XRTMIN).
ICE3_HD void sed_column_vjp(const Cst &c, bool fortran, bool skip_c, const CloudPar &cp, double dt,
                            const SedColumnIO &io, double *const flux[5], const SedCotangents &g,
                            const SedGradients &gx, long col)
{
  const double inv_dt = 1.0 / dt;
  double rtmin[5];
#pragma unroll
  for (int s = 0; s < 5; ++s) rtmin[s] = sed_rtmin(c, s);
  // cotangent of F_k (flux leaving level k downward), starting at the surface
  double bF[5];
#pragma unroll
  for (int s = 0; s < 5; ++s) bF[s] = (g.inpr[s] && !(s == 0 && skip_c)) ? g.inpr[s][col] / c.RHOLW : 0.0;
  for (int k = 0; k < io.nk; ++k) {
    const long p = (long)k * io.nij + col;
    const long pa = p + io.nij;                    // level above
    const double rho = sed_load(io.rhodref, p), dz = sed_load(io.dzz, p);
    const double rhodz = rho * dz;
    const double tsorhodz = fm::fdiv(dt, rhodz);
    double src[5], rt[5], qp[5], fa[5], fk[5];
    bool c1[5], c2[5];
    bool any = false;
#pragma unroll
    for (int s = 0; s < 5; ++s) {
      if (s == 0 && skip_c) { c1[s] = c2[s] = false; src[s] = rt[s] = qp[s] = fa[s] = fk[s] = 0.0; continue; }
      src[s] = io.src_in[s][p];
      rt[s] = src[s] * dt;
      fa[s] = (k + 1 < io.nk) ? flux[s][pa] : 0.0;
      fk[s] = flux[s][p];
      qp[s] = fa[s] * tsorhodz;
      c1[s] = gtp(rt[s], rtmin[s]);
      c2[s] = gtp(qp[s], rtmin[s]);
      any = any || c1[s] || c2[s];
    }
    const double lrho = any ? fm::flog(rho) : 0.0;
    const bool cloud = c1[0] || c2[0];
    const double pabs = cloud ? sed_load(io.pabs, p) : 1.0, tht = cloud ? sed_load(io.tht, p) : 0.0;
    const double wlbda = cloud ? 6.6e-8 * fm::fdiv(101325.0, pabs) * (tht * (1.0 / 293.15)) : 0.0;
    double b_rho = 0.0, b_dz = 0.0, b_rhodz = 0.0, b_tso = 0.0, b_lrho = 0.0, b_wl = 0.0;
#pragma unroll
    for (int s = 0; s < 5; ++s) {
      const double gS = g.src[s] ? g.src[s][p] : 0.0;
      if (s == 0 && skip_c) {                       // sources passed through unchanged
        if (gx.src[s]) gx.src[s][p] = gS;
        continue;
      }
      if (g.fpr[s]) bF[s] += g.fpr[s][p];
      double d1_lr = 0.0, d1_lrho = 0.0, d1_wl = 0.0, d2_lr = 0.0, d2_lrho = 0.0, d2_wl = 0.0;
      const double w1 = c1[s] ? fall_speed_d(c, s, rt[s], lrho, wlbda, cp, d1_lr, d1_lrho, d1_wl) : 0.0;
      const double w2 = c2[s] ? fall_speed_d(c, s, qp[s], lrho, wlbda, cp, d2_lr, d2_lrho, d2_wl) : 0.0;
      const double a1 = rhodz * rt[s] * inv_dt, a2 = w1 * rho * rt[s];
      const bool sel1 = !gtd(a1, a2);
      double Bv = 0.0, u = 0.0;
      const bool nz2 = !zerod_(w2);
      if (nz2) {
        u = 1.0 - fm::fdiv(dz, dt * w2);
        Bv = pmax0(u);
      }
      // source update
      double b_src = gS, b_fa = 0.0, bFt;
      if (fortran) {
        const double coef = tsorhodz * inv_dt;
        b_fa += coef * gS;
        bFt = bF[s] - coef * gS;
        b_tso += (fa[s] - fk[s]) * inv_dt * gS;
      } else {
        const double den = rhodz * dt;
        b_fa += gS / den;
        bFt = bF[s] - gS / den;
        b_rhodz += -(fa[s] - fk[s]) * dt / (den * den) * gS;
      }
      // F_k = min(a1, a2) + Bv F_{k+1}
      b_fa += Bv * bFt;
      const double b_B = fa[s] * bFt;
      double b_rt = 0.0;
      if (sel1) {
        b_rt += rhodz * inv_dt * bFt;
        b_rhodz += rt[s] * inv_dt * bFt;
      } else {
        const double b_w1 = rho * rt[s] * bFt;
        b_rho += w1 * rt[s] * bFt;
        b_rt += w1 * rho * bFt;
        if (c1[s]) {
          b_rt += d1_lr / rt[s] * b_w1;
          b_lrho += d1_lrho * b_w1;
          b_wl += d1_wl * b_w1;
        }
      }
      if (nz2 && pos(u)) {
        const double b_w2 = dz / (dt * w2 * w2) * b_B;
        b_dz += -1.0 / (dt * w2) * b_B;
        if (c2[s]) {
          const double b_qp = d2_lr / qp[s] * b_w2;
          b_lrho += d2_lrho * b_w2;
          b_wl += d2_wl * b_w2;
          b_fa += tsorhodz * b_qp;
          b_tso += fa[s] * b_qp;
        }
      }
      b_src += dt * b_rt;
      if (gx.src[s]) gx.src[s][p] = b_src;
      bF[s] = b_fa;                                 // cotangent of F_{k+1}, used at level k + 1
    }
    // level quantities shared by the species
    b_rhodz += -tsorhodz / rhodz * b_tso;
    b_rho += dz * b_rhodz + (any ? b_lrho / rho : 0.0);
    b_dz += rho * b_rhodz;
    if (gx.rhodref) gx.rhodref[p] = b_rho;
    if (gx.dzz) gx.dzz[p] = b_dz;
    if (gx.pabs) gx.pabs[p] = cloud ? -wlbda / pabs * b_wl : 0.0;
    if (gx.tht) gx.tht[p] = cloud ? wlbda / tht * b_wl : 0.0;
  }
}

// ---- time-split sedimentation (SEDIM = SPLI) ------------------------------
// mode_ice4_sedimentation_split.F90 (INTERNAL_SEDIM_SPLI, without the
// electric charges and the Beard velocity correction) and the negativity
// correction that ICE4_SEDIMENTATION applies after it
// (mode_ice4_sedimentation.F90:196-229).  Per species, in CFL-limited
// sub-steps until the time step is used up: the flux of each level from the
// temporary mixing ratio (initialised with the value at t), the column's
// sub-step = min(remaining time, SPLIT_MAXCFL rho r dz / flux), then the
// temporary mixing ratio moves by the flux divergence plus its external
// tendency (source - r_t / dt) over the sub-step and the source by the flux
// divergence.
struct SplitColumnIO {
  const double *rhodref, *dzz, *pabs, *tht, *exn;
  const double *rt[6];       // mixing ratios at t: rc rr ri rs rg (rh)
  const double *rvt;
  double *src[6];            // in-out sources rcs rrs ris rss rgs (rhs)
  double *rvs, *ths;         // in-out (negativity correction)
  double *fpr[6];            // accumulated fluxes, or NULL
  double *inpr[6];           // [nij]
  double *rtmp, *ext;        // [nk][nij] scratch: temporary mixing ratio, external tendency
  long nij;
  int nk;
  int nsp;                   // 5, or 6 with hail (NRR = 7, species 7 of :340-347)
};

// Flux rho r v(r) of species s at content r (0 below the species' threshold;
// ice: max(XRTMIN, 1e-7)), INTERNAL_SEDIM_SPLI :500-700.
ICE3_HD double split_flux(const Cst &c, int s, double r, double rho, double lrho, double p, double th,
                          const CloudPar &cp)
{
  if (!gtp(r, sed_rtmin(c, s))) return 0.0;
  double wlbda = 0.0;
  if (s == 0) {
    // ZZT = theta (p / P00)^(RD/CPD): the temperature (:520)
    const double t = th * fm::fexp((c.RD / c.CPD) * fm::flog(fm::fdiv(p, c.P00)));
    wlbda = 6.6e-8 * fm::fdiv(101325.0, p) * (t * (1.0 / 293.15));
  }
  return fall_speed(c, s, r, lrho, wlbda, cp) * rho * r;
}

// ICE4_CORRECT_NEGATIVITIES on the sources (mode_ice4_correct_negativities.F90)
// with the latent-heat factors lv / ls.
ICE3_HD void correct_negativities(const Cst &c, double lv, double ls, double &ths, double &rvs, double &rcs,
                                  double &rrs, double &ris, double &rss, double &rgs, double *rhs = nullptr)
{
  double w;
  w = rcs - pmax0(rcs); rvs += w; ths -= w * lv; rcs -= w;
  w = rrs - pmax0(rrs); rvs += w; ths -= w * lv; rrs -= w;
  w = ris - pmax0(ris); rvs += w; ths -= w * ls; ris -= w;
  w = rss - pmax0(rss); rvs += w; ths -= w * ls; rss -= w;
  w = rgs - pmax0(rgs); rvs += w; ths -= w * ls; rgs -= w;
  if (rhs) { w = *rhs - pmax0(*rhs); rvs += w; ths -= w * ls; *rhs -= w; }   // :115-120
  w = dmin(1., fm::fdiv(pmax0(c.V_RTMIN - rvs), dmax(rcs + ris, 1.e-20)));
  ths -= w * (rcs * lv + ris * ls);
  rvs += w * (rcs + ris);
  rcs = (1. - w) * rcs;
  ris = (1. - w) * ris;
  w = dmin(pmax0(rrs), pmax0(c.V_RTMIN - rvs)); rvs += w; rrs -= w; ths -= w * lv;
  w = dmin(pmax0(rss), pmax0(c.V_RTMIN - rvs)); rvs += w; rss -= w; ths -= w * ls;
  w = dmin(pmax0(rgs), pmax0(c.V_RTMIN - rvs)); rvs += w; rgs -= w; ths -= w * ls;
  if (rhs) { w = dmin(pmax0(*rhs), pmax0(c.V_RTMIN - rvs)); rvs += w; *rhs -= w; ths -= w * ls; }   // :165-171
}

// One column; returns false if a species needed more than max_iter sub-steps
// (the sub-stepping then stops for that species).
ICE3_HD bool sed_split_column(const Cst &c, const CloudPar &cp, double dt, const SplitColumnIO &io, long col,
                              int max_iter)
{
  const double inv_dt = 1.0 / dt;
  bool ok = true;
  for (int s = 0; s < io.nsp; ++s) {
    if (s == 0 && c.LSEDIC == 0.0) {          // GSEDIC = .FALSE.: cloud not sedimented
      if (io.inpr[0]) io.inpr[0][col] = 0.0;
      if (io.fpr[0])
        for (int k = 0; k < io.nk; ++k) io.fpr[0][(long)k * io.nij + col] = 0.0;
      continue;
    }
    const double rtmin = s == 0 ? c.C_RTMIN : s == 1 ? c.R_RTMIN : s == 2 ? c.I_RTMIN : s == 3 ? c.S_RTMIN
                                                                                  : s == 4 ? c.G_RTMIN : c.H_RTMIN;
    for (int k = 0; k < io.nk; ++k) {
      const long p = (long)k * io.nij + col;
      const double r = sed_load(io.rt[s], p);
      io.rtmp[p] = r;
      io.ext[p] = io.src[s][p] - r * inv_dt;    // ZPR.S (:180-190)
      if (io.fpr[s]) io.fpr[s][p] = 0.0;
    }
    double remaint = dt, inpr = 0.0;
    int it = 0;
    while (gtp(remaint, 0.0)) {
      if (++it > max_iter) { ok = false; break; }
      // the column's sub-step (:780-805)
      double mt = remaint;
      for (int k = 0; k < io.nk; ++k) {
        const long p = (long)k * io.nij + col;
        const double r = io.rtmp[p];
        if (!gtp(r, rtmin)) continue;
        const double rho = sed_load(io.rhodref, p);
        const double w = split_flux(c, s, r, rho, fm::flog(rho), sed_load(io.pabs, p), sed_load(io.tht, p), cp);
        if (gtp(w, 1.e-20)) mt = dmin(mt, fm::fdiv(c.SPLIT_MAXCFL * rho * r * sed_load(io.dzz, p), w));
      }
      remaint -= mt;
      // update, top-down with the flux of the level above (:806-830)
      const double frac = mt * inv_dt;
      double wa = 0.0;
      for (int k = io.nk - 1; k >= 0; --k) {
        const long p = (long)k * io.nij + col;
        const double r = io.rtmp[p];
        const double rho = sed_load(io.rhodref, p);
        const double w = gtp(r, sed_rtmin(c, s))
                             ? split_flux(c, s, r, rho, fm::flog(rho), sed_load(io.pabs, p), sed_load(io.tht, p), cp)
                             : 0.0;
        const double change = mt * fm::fdiv(1.0, rho * sed_load(io.dzz, p)) * (wa - w);
        io.rtmp[p] = r + change + io.ext[p] * mt;
        io.src[s][p] += change * inv_dt;
        if (io.fpr[s]) io.fpr[s][p] += w * frac;
        if (k == 0) inpr += w / c.RHOLW * frac;
        wa = w;
      }
    }
    if (io.inpr[s]) io.inpr[s][col] = inpr;
  }
  // ICE4_CORRECT_NEGATIVITIES with L/cph of the time-t state (rain_ice.F90:334-345)
  for (int k = 0; k < io.nk; ++k) {
    const long p = (long)k * io.nij + col;
    const double rv = sed_load(io.rvt, p), rc = sed_load(io.rt[0], p), rr = sed_load(io.rt[1], p);
    const double ri = sed_load(io.rt[2], p), rs = sed_load(io.rt[3], p), rg = sed_load(io.rt[4], p);
    const bool hail = io.nsp == 6;
    const double zice = hail ? ri + rs + rg + sed_load(io.rt[5], p) : ri + rs + rg;
    const double zdev = c.CPD + c.CPV * rv + c.CL * (rc + rr) + c.CI * zice;
    const double t = sed_load(io.tht, p) * sed_load(io.exn, p);
    const double ls = (c.LSTT + (c.CPV - c.CI) * (t - c.TT)) / zdev;
    const double lv = (c.LVTT + (c.CPV - c.CL) * (t - c.TT)) / zdev;
    double ths = io.ths[p], rvs = io.rvs[p], rcs = io.src[0][p], rrs = io.src[1][p], ris = io.src[2][p];
    double rss = io.src[3][p], rgs = io.src[4][p];
    double rhs = hail ? io.src[5][p] : 0.0;
    correct_negativities(c, lv, ls, ths, rvs, rcs, rrs, ris, rss, rgs, hail ? &rhs : nullptr);
    io.ths[p] = ths; io.rvs[p] = rvs; io.src[0][p] = rcs; io.src[1][p] = rrs; io.src[2][p] = ris;
    io.src[3][p] = rss; io.src[4][p] = rgs;
    if (hail) io.src[5][p] = rhs;
  }
  return ok;
}

}  // namespace ice3sed
