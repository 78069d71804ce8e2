// ice_adjust.cu — saturation adjustment with CB02 subgrid condensation.
//
// Restates src/ice3/jax/stencils/ice_adjust.py:26-398 (IceAdjustJAX) for one
// grid point per lane; each thread owns two consecutive points so every field
// moves with one 128-bit load/store (LDG.128/STG.128).  Pure map over the
// nij*nk points: 19 3-D fields read (+ sigqsat per column), 16 written,
// 280 algorithmic bytes per point.
#include <cmath>

#include "ice3gb_device.cuh"
#include "ice3gb_kernels.h"
#include "ice_adjust_point.cuh"

namespace {
using namespace ice3ia;

// Two points per thread, double2 loads/stores; requires an even point count
// and 16-byte aligned fields (checked by the host).  ADV: the state adjusted
// is adv_dt times the sources (th = dt*ths, r = dt*rs, the state after the
// microphysics in the chained physics step) instead of th/rv/.../rg, which
// are then not read; rrs/rss/rgs are read instead.  Output pointers may be
// NULL in the internal chained use (store skipped).
// Blocks of 256 per SM the registers are capped for: the default leaves
// 158-162 registers (one block, 8 warps per SM); two blocks (128 registers)
// measured 35.67 against 35.58 ms per launch at 1024x1024x90, three (80
// registers, spilling) 39.95 against 39.43 ms before the saturation terms
// were skipped by their weight.
#ifndef IA_MIN_BLOCKS
#define IA_MIN_BLOCKS 1
#endif
template <bool ADV, bool SRC>
__global__ void __launch_bounds__(256, IA_MIN_BLOCKS) ice_adjust_v2_kernel(const __grid_constant__ Cst c,
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
    double s0 = 0.0, s1 = 0.0;
    ia_point(c, d, dt, inv_dt, x0, o0, SRC ? &s0 : nullptr);
    ia_point(c, d, dt, inv_dt, x1, o1, SRC ? &s1 : nullptr);
    if (SRC) st2(f.srcs, p, s0, s1);
#define ST2(field) if (f.field) st2(f.field, p, o0.field, o1.field);
    ST2(t) ST2(rv_out) ST2(rc_out) ST2(ri_out) ST2(cldfr) ST2(hlc_hrc) ST2(hlc_hcf) ST2(hli_hri) ST2(hli_hcf)
    ST2(cph) ST2(lv) ST2(ls) ST2(rvs) ST2(rcs) ST2(ris) ST2(ths)
#undef ST2
  }
}

// Scalar path: odd point counts or unaligned fields.
template <bool ADV, bool SRC>
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
    double s0 = 0.0;
    ia_point(c, d, dt, inv_dt, x, o, SRC ? &s0 : nullptr);
    if (SRC) f.srcs[p] = s0;
#define ST1(field) if (f.field) f.field[p] = o.field;
    ST1(t) ST1(rv_out) ST1(rc_out) ST1(ri_out) ST1(cldfr) ST1(hlc_hrc) ST1(hlc_hcf) ST1(hli_hri) ST1(hli_hcf)
    ST1(cph) ST1(lv) ST1(ls) ST1(rvs) ST1(rcs) ST1(ris) ST1(ths)
#undef ST1
  }
}

// OCND2 (separate liquid and ice clouds): one point per thread; the level
// above (below at the top) gives the layer thickness of ICECLOUD.
template <bool SRC>
__global__ void __launch_bounds__(256) ice_adjust_ocnd2_kernel(const __grid_constant__ Cst c,
                                                               const __grid_constant__ IaKernelFields kf, long n,
                                                               int nij, int nk, double dt)
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
    x.th = ld1(f.th, p); x.rv = ld1(f.rv, p); x.rc = ld1(f.rc, p); x.ri = ld1(f.ri, p);
    x.rr = ld1(f.rr, p); x.rs = ld1(f.rs, p); x.rg = ld1(f.rg, p);
    const long k = p / nij, col = p - k * nij;
    const long kp = k + 1 < nk ? k + 1 : nk - 1;
    Ocnd2In oi;
    oi.estw = kf.tiwmx;
    oi.esti = kf.tiwmx + kTiwmxN;
    oi.z = ld1(f.zz, p);
    oi.dz = ld1(f.zz, kp * nij + col) - ld1(f.zz, (kp - 1) * nij + col);
    oi.ice_cld_wgt = ld1(f.ice_cld_wgt, col);
    oi.bottom = k == 0;
    IaOut o;
    Ocnd2Out oo;
    double s0 = 0.0;
    ia_point<true>(c, d, dt, inv_dt, x, o, SRC ? &s0 : nullptr, &oi, &oo);
    if (SRC) f.srcs[p] = s0;
#define ST1(field) if (f.field) f.field[p] = o.field;
    ST1(t) ST1(rv_out) ST1(rc_out) ST1(ri_out) ST1(cldfr) ST1(hlc_hrc) ST1(hlc_hcf) ST1(hli_hri) ST1(hli_hcf)
    ST1(cph) ST1(lv) ST1(ls) ST1(rvs) ST1(rcs) ST1(ris) ST1(ths)
#undef ST1
    if (f.icldfr) f.icldfr[p] = oo.icldfr;
    if (f.wcldfr) f.wcldfr[p] = oo.wcldfr;
    if (f.ssio) f.ssio[p] = oo.ssio;
    if (f.ssiu) f.ssiu[p] = oo.ssiu;
    if (f.ifr) f.ifr[p] = 10.0;   // PIFR, condensation.F90:259
  }
}

}  // namespace

static_assert(kTiwmxTableN == kTiwmxN && kTiwmxTables == TW_N, "TIWMX table size");

void tiwmx_tables(const Cst &c, double *tab)
{
  // mode_tiwmx_fun.F90 ESATW / ESATI / AA2 / BB3 / AM3 / REDIN as INI_TIWMX
  // fills its tables (the water values above 273.15 K for ESTABI, AM3TAB = 0 there)
  for (int j = kTiwmxStart; j <= kTiwmxStop; ++j) {
    const double t = (double)j / 100.0;
    const long i = j - kTiwmxStart;
    const double w = std::exp(c.ALPW - c.BETAW / t - c.GAMW * std::log(t));
    const double ei = t >= c.TT ? w : std::exp(c.ALPI - c.BETAI / t - c.GAMI * std::log(t));  // ESATI
    tab[TW_ESW * kTiwmxN + i] = w;
    tab[TW_ESI * kTiwmxN + i] = t > 273.15 ? w : std::exp(c.ALPI - c.BETAI / t - c.GAMI * std::log(t));
    const double l = c.LSTT + (c.CPV - c.CI) * (t - c.TT);
    tab[TW_A2 * kTiwmxN + i] = l * l / (2.38e-2 + 0.0071e-2 * (t - c.TT)) / (t * t * c.RV);
    tab[TW_BB3 * kTiwmxN + i] = c.RV / (0.211e-4 * std::pow(t / c.TT, 1.94) * c.P00) * t / ei;
    tab[TW_AM3 * kTiwmxN + i] = t > 273.15 ? 0.0 : 1000. * std::exp(12.96 * (w / ei - 1.) - 0.639);
    const double z = std::fmax(0., std::fmin(1., (c.TT - t) / 20.));
    tab[TW_REDIN * kTiwmxN + i] = 1. - (1. - z) / std::pow(z * z * z + (1. - z) * (1. - z) * (1. - z), .333);
  }
}

cudaError_t launch_ice_adjust(const Cst &c, const IaKernelFields &kf, int nij, int nk, double dt, bool vec2,
                              int num_sms, cudaStream_t s)
{
  const long n = (long)nij * nk;
  const int threads = 256;
  const long cap = (long)num_sms * 64;
  const bool adv = kf.adv_dt != 0.0;
  const bool src = kf.f.srcs != nullptr;
  if (c.OCND2 != 0.0) {   // (the host rejects OCND2 with adv_dt)
    long blocks = (n + threads - 1) / threads;
    if (blocks > cap) blocks = cap;
    if (src) ice_adjust_ocnd2_kernel<true><<<(unsigned)blocks, threads, 0, s>>>(c, kf, n, nij, nk, dt);
    else ice_adjust_ocnd2_kernel<false><<<(unsigned)blocks, threads, 0, s>>>(c, kf, n, nij, nk, dt);
  } else if (vec2) {
    const long npairs = n / 2;
    long blocks = (npairs + threads - 1) / threads;
    if (blocks > cap) blocks = cap;
    if (src) {
      if (adv) ice_adjust_v2_kernel<true, true><<<(unsigned)blocks, threads, 0, s>>>(c, kf, npairs, nij, dt);
      else ice_adjust_v2_kernel<false, true><<<(unsigned)blocks, threads, 0, s>>>(c, kf, npairs, nij, dt);
    } else {
      if (adv) ice_adjust_v2_kernel<true, false><<<(unsigned)blocks, threads, 0, s>>>(c, kf, npairs, nij, dt);
      else ice_adjust_v2_kernel<false, false><<<(unsigned)blocks, threads, 0, s>>>(c, kf, npairs, nij, dt);
    }
  } else {
    long blocks = (n + threads - 1) / threads;
    if (blocks > cap) blocks = cap;
    if (src) {
      if (adv) ice_adjust_v1_kernel<true, true><<<(unsigned)blocks, threads, 0, s>>>(c, kf, n, nij, dt);
      else ice_adjust_v1_kernel<false, true><<<(unsigned)blocks, threads, 0, s>>>(c, kf, n, nij, dt);
    } else {
      if (adv) ice_adjust_v1_kernel<true, false><<<(unsigned)blocks, threads, 0, s>>>(c, kf, n, nij, dt);
      else ice_adjust_v1_kernel<false, false><<<(unsigned)blocks, threads, 0, s>>>(c, kf, n, nij, dt);
    }
  }
  return cudaGetLastError();
}
