// sedimentation.cu — statistical sedimentation, one column sweep per thread.
//
// Restates ICE4_SEDIMENTATION_STAT (PHYEX-IAL_CY50T1/micro/
// mode_ice4_sedimentation_stat.F90:143-229) and the reference JAX
// sedimentation_stat (src/ice3/jax/stencils/sedimentation.py:58-352), the two
// differing in the cloud mean-radius factor and the flux-divergence scaling
// (selected by `fortran`).  A thread owns one column and walks k from the top
// level to the surface with the five species side by side, keeping each
// species' incoming flux F_{k+1} in a register; consecutive threads own
// consecutive columns, so every level access is coalesced.  What the species
// share at a level (rho, dz, rho dz, dt/(rho dz) and log rho, computed only
// when a species sediments there) is computed once; threshold tests and
// clamps run on the integer pipe (GB300's FP64 pipe is the bound).
#include "ice3gb_device.cuh"
#include "ice3gb_kernels.h"

namespace {

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

// Fall speed for content r (> threshold checked by the caller); lrho = log(rho).
ICE3_HD double fall_speed(const Cst &c, int s, double r, double lrho, double wlbda, const CloudPar &cp)
{
  const double lr = fm::flog(r);
  switch (s) {
    case 0: {  // cloud droplets: sedimentation.py:206-209, F90:264-267
      const double lwlbdc = c.LBEXC * (cp.log_lbc_conc - lrho - lr);
      const double cc = c.CC * (1.0 + 1.26 * wlbda * fm::fexp(lwlbdc) * cp.ray_inv);
      return fm::fexp(-c.CEXVT * lrho - c.DC * lwlbdc) * cc * cp.fsedc;
    }
    case 1:  // rain
      return c.FSEDR * fm::fexp((c.EXSEDR - 1.0) * lr + (c.EXSEDR - c.CEXVT - 1.0) * lrho);
    case 2: {  // pristine ice: sedimentation.py:46-55, F90:307-311
      const double dmax_ = dmax(0.05e6, -0.15319e6 - 0.021454e6 * (lrho + lr));
      return c.FSEDI * fm::fexp(-c.CEXVT * lrho + c.EXCSEDI * fm::flog(dmax_));
    }
    case 3:  // snow
      return c.FSEDS * fm::fexp((c.EXSEDS - 1.0) * lr + (c.EXSEDS - c.CEXVT - 1.0) * lrho);
    default:  // graupel
      return c.FSEDG * fm::fexp((c.EXSEDG - 1.0) * lr + (c.EXSEDG - c.CEXVT - 1.0) * lrho);
  }
}

__global__ void __launch_bounds__(128) sedimentation_kernel(const __grid_constant__ Cst c, SedArgs a)
{
  const long col = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (col >= a.nij) return;
  // PHYEX skips the cloud species when LSEDIC is off
  const bool skip_c = a.fortran && c.LSEDIC == 0.0;
  if (skip_c) {
    if (a.fpr[0])
      for (int k = 0; k < a.nk; ++k) a.fpr[0][(long)k * a.nij + col] = 0.0;
    a.inpr[0][col] = 0.0;
  }
  const double rtmin[5] = {c.C_RTMIN, c.R_RTMIN, dmax(c.I_RTMIN, 1.0e-7), c.S_RTMIN, c.G_RTMIN};
  CloudPar cp;
  {
    const bool has_st = a.sea != nullptr && a.town != nullptr;
    const double sea = a.sea ? a.sea[col] : 0.0, town = a.town ? a.town[col] : 0.0;
    cp = cloud_params(c, a.fortran, has_st, sea, town);
  }
  const double dt = a.dt, inv_dt = 1.0 / a.dt;
  double fabove[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int k = a.nk - 1; k >= 0; --k) {
    const long p = (long)k * a.nij + col;
    const double rho = ld1(a.rhodref, p), dz = ld1(a.dzz, p);
    const double rhodz = rho * dz;
    const double tsorhodz = fm::fdiv(dt, rhodz);
    double src[5], rt[5], qp[5];
    bool c1[5], c2[5];
    bool any = false;
#pragma unroll
    for (int s = 0; s < 5; ++s) {
      if (s == 0 && skip_c) { c1[s] = c2[s] = false; src[s] = rt[s] = qp[s] = 0.0; continue; }
      src[s] = a.src[s][p];
      rt[s] = src[s] * dt;
      qp[s] = fabove[s] * tsorhodz;
      c1[s] = gtp(rt[s], rtmin[s]);
      c2[s] = gtp(qp[s], rtmin[s]);
      any = any || c1[s] || c2[s];
    }
    const double lrho = any ? fm::flog(rho) : 0.0;
    const double wlbda = (c1[0] || c2[0]) ? 6.6e-8 * fm::fdiv(101325.0, ld1(a.pabs, p)) * (ld1(a.tht, p) * (1.0 / 293.15)) : 0.0;
#pragma unroll
    for (int s = 0; s < 5; ++s) {
      if (s == 0 && skip_c) continue;
      const double w1 = c1[s] ? fall_speed(c, s, rt[s], lrho, wlbda, cp) : 0.0;
      const double w2 = c2[s] ? fall_speed(c, s, qp[s], lrho, wlbda, cp) : 0.0;
      double flux = dmin(rhodz * rt[s] * inv_dt, w1 * rho * rt[s]);
      if (!zerod_(w2)) flux += pmax0(1.0 - fm::fdiv(dz, dt * w2)) * fabove[s];
      if (a.fortran) a.src[s][p] = src[s] + tsorhodz * (fabove[s] - flux) * inv_dt;
      else a.src[s][p] = src[s] + fm::fdiv(fabove[s] - flux, rhodz * dt);
      if (a.fpr[s]) a.fpr[s][p] = flux;
      fabove[s] = flux;
    }
  }
#pragma unroll
  for (int s = 0; s < 5; ++s)
    if (!(s == 0 && skip_c)) a.inpr[s][col] = fabove[s] / c.RHOLW;
}

// Fog deposition on the lowest level (rain_ice.F90:876-895).
__global__ void fog_deposition_kernel(const __grid_constant__ Cst c, FogArgs a)
{
  const long col = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (col >= a.nij) return;
  if (a.enabled) {
    const double rct = a.rct[col];
    const double indep = c.VDEPOSC * rct * a.rhodref[col] / c.RHOLW;
    a.rcs[col] -= c.VDEPOSC * rct / a.dzz[col];
    a.inprc[col] += indep;
    if (a.indep) a.indep[col] = indep;
  } else if (a.indep) {
    a.indep[col] = 0.0;
  }
}

}  // namespace

cudaError_t launch_sedimentation(const Cst &c, const SedArgs &a, cudaStream_t s)
{
  const long n = a.nij;
  const int threads = 128;
  sedimentation_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, s>>>(c, a);
  return cudaGetLastError();
}

cudaError_t launch_fog_deposition(const Cst &c, const FogArgs &a, cudaStream_t s)
{
  const int threads = 256;
  fog_deposition_kernel<<<(unsigned)((a.nij + threads - 1) / threads), threads, 0, s>>>(c, a);
  return cudaGetLastError();
}
