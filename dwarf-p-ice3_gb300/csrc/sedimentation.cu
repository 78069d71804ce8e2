// sedimentation.cu — statistical sedimentation, one column sweep per thread.
//
// Restates ICE4_SEDIMENTATION_STAT (PHYEX-IAL_CY50T1/micro/
// mode_ice4_sedimentation_stat.F90:143-229) and the reference JAX
// sedimentation_stat (src/ice3/jax/stencils/sedimentation.py:58-352), the two
// differing in the cloud mean-radius factor and the flux-divergence scaling
// (selected by `fortran`).  A thread owns one column and walks k from the top
// level to the surface with the five species side by side, keeping each
// species' incoming flux F_{k+1} in a register; consecutive threads own
// consecutive columns, so every level access is coalesced.  The fall speeds a
// warp needs at a level are evaluated together, with every lane busy: those
// of rain, snow and graupel pooled across the three species
// (warp_power_speeds), cloud and ice per species (warp_fall_speeds).  What
// the species share at a level (rho, dz, rho dz, dt/(rho dz) and log rho,
// computed only when a species sediments there) is computed once; threshold
// tests and clamps run on the integer pipe (GB300's FP64 pipe is the bound).
#include "ice3gb_device.cuh"
#include "ice3gb_kernels.h"
#include "sedimentation_point.cuh"

namespace {
using namespace ice3sed;

// The fall speeds of species s at one level for the whole warp.  A lane
// needs w1 (content r1 above its threshold, c1) and / or w2 (the flux from
// above, r2, c2); about half of these requests are live, and evaluating them
// in place would run each fall-speed formula for all 32 lanes whenever one
// lane needs it.  The requests are dealt out to consecutive lanes instead
// (the inputs fetched with shuffles), evaluated 32 at a time with every lane
// busy, and the speeds shuffled back to the lanes that asked.  Same function
// on the same arguments: the values are those of the per-lane evaluation.
__device__ __forceinline__ void warp_fall_speeds(const Cst &c, int s, bool c1, double r1, bool c2, double r2,
                                                 double lrho, double wlbda, const CloudPar &cp, const double *fx,
                                                 double &w1, double &w2)
{
  const unsigned full = 0xffffffffu, lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
  const unsigned m1 = __ballot_sync(full, c1), m2 = __ballot_sync(full, c2);
  const int n1 = __popc(m1), ntot = n1 + __popc(m2);
  const int i1 = __popc(m1 & lt), i2 = n1 + __popc(m2 & lt);   // this lane's request numbers
  w1 = w2 = 0.0;
  for (int base = 0; base < ntot; base += 32) {                  // uniform over the warp
    const int j = base + (int)lane;                              // the request this lane evaluates
    const bool first = j < n1;
    int owner = 0;
    if (j < ntot) owner = (int)(first ? __fns(m1, 0u, j + 1) : __fns(m2, 0u, j - n1 + 1));
    const double ra = __shfl_sync(full, r1, owner), rb = __shfl_sync(full, r2, owner);
    const double lr = __shfl_sync(full, lrho, owner);
    double wl = 0.0;
    CloudPar cq = cp;
    if (s == 0) {                                                // the cloud speed: per-column parameters
      wl = __shfl_sync(full, wlbda, owner);
      cq.log_lbc_conc = __shfl_sync(full, cp.log_lbc_conc, owner);
      cq.ray_inv = __shfl_sync(full, cp.ray_inv, owner);
      cq.fsedc = __shfl_sync(full, cp.fsedc, owner);
    }
    double v = 0.0;
    if (j < ntot) v = fall_speed(c, s, first ? ra : rb, lr, wl, cq, fx);
    const double v1 = __shfl_sync(full, v, (unsigned)(i1 - base) & 31u);
    const double v2 = __shfl_sync(full, v, (unsigned)(i2 - base) & 31u);
    if (c1 && i1 >= base && i1 < base + 32) w1 = v1;
    if (c2 && i2 >= base && i2 < base + 32) w2 = v2;
  }
}

// The power-law fall speeds of rain, snow and graupel (species 1, 3, 4) at
// one level for the whole warp, with the requests of the three species
// numbered together (in six slots: species x content / incoming flux) and
// evaluated 32 at a time, so that a round of the exp / log is shared across
// species instead of each species rounding its own requests up to a full
// warp.  Same function (power_speed) on the same arguments as fall_speed.
// live[s]: species s has a request in some lane (its warp is not skipped).
__device__ __forceinline__ void warp_power_speeds(const Cst &c, const bool live[5], const bool c1[5],
                                                  const double r1[5], const bool c2[5], const double r2[5],
                                                  double lrho, const double *fx, double w1[5], double w2[5])
{
  constexpr int SP[3] = {1, 3, 4};
  const unsigned full = 0xffffffffu, lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
  unsigned m[6];
  int off[7];
  off[0] = 0;
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const int s = SP[q >> 1];
    m[q] = live[s] ? __ballot_sync(full, (q & 1) ? c2[s] : c1[s]) : 0u;
    off[q + 1] = off[q] + __popc(m[q]);
  }
  const int ntot = off[6];
  int mine[6];                                                   // this lane's request numbers
#pragma unroll
  for (int q = 0; q < 6; ++q) mine[q] = off[q] + __popc(m[q] & lt);
#pragma unroll
  for (int k = 0; k < 3; ++k) w1[SP[k]] = w2[SP[k]] = 0.0;
  for (int base = 0; base < ntot; base += 32) {                  // uniform over the warp
    const int j = base + (int)lane;                              // the request this lane evaluates
    int q = 0;
    unsigned mq = m[0];
    int oq = 0;
#pragma unroll
    for (int t = 1; t < 6; ++t)
      if (j >= off[t]) { q = t; mq = m[t]; oq = off[t]; }     // selects, not an indexed local array
    const int owner = j < ntot ? (int)__fns(mq, 0u, j - oq + 1) : 0;
    double arg = 0.0;
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      const int s = SP[t >> 1];
      const double x = __shfl_sync(full, (t & 1) ? r2[s] : r1[s], owner);
      if (q == t) arg = x;
    }
    const double lr = __shfl_sync(full, lrho, owner);
    double v = 0.0;
    if (j < ntot) {
      const int k = q >> 1, s = k == 0 ? 1 : k + 2;
      const double f = k == 0 ? c.FSEDR : (k == 1 ? c.FSEDS : c.FSEDG);
      v = power_speed(f, fx[2 * s], fx[2 * s + 1], fm::flog(arg), lr);
    }
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      const int s = SP[t >> 1];
      const double x = __shfl_sync(full, v, (unsigned)(mine[t] - base) & 31u);
      const bool asked = (t & 1) ? c2[s] : c1[s];
      if (live[s] && asked && mine[t] >= base && mine[t] < base + 32) {
        if (t & 1) w2[s] = x;
        else w1[s] = x;
      }
    }
  }
}

// sed_column_forward with the warp's fall speeds evaluated together
// (warp_fall_speeds); every lane of the warp runs the level loop, lanes
// past the last column (valid = false) without loads, stores or requests.
__device__ void sed_column_forward_warp(const Cst &c, bool fortran, bool skip_c, const CloudPar &cp, double dt,
                                        const SedColumnIO &io, long col, bool valid, const double *fx)
{
  const double inv_dt = 1.0 / dt;
  double rtmin[5];
#pragma unroll
  for (int s = 0; s < 5; ++s) rtmin[s] = sed_rtmin(c, s);
  double fabove[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int k = io.nk - 1; k >= 0; --k) {
    const long p = (long)k * io.nij + col;
    const double rho = valid ? sed_load(io.rhodref, p) : 1.0, dz = valid ? sed_load(io.dzz, p) : 1.0;
    const double rhodz = rho * dz;
    const double tsorhodz = fm::fdiv(dt, rhodz);
    // per-level factors of the species' fluxes and sources (formed once
    // instead of per species)
    const double rhodz_idt = rhodz * inv_dt, tso_idt = tsorhodz * inv_dt, dz_idt = dz * inv_dt;
    double src[5], rt[5], qp[5];
    bool c1[5], c2[5];
    bool any = false;
#pragma unroll
    for (int s = 0; s < 5; ++s) {
      if (s == 0 && skip_c) { c1[s] = c2[s] = false; src[s] = rt[s] = qp[s] = 0.0; continue; }
      src[s] = valid ? io.src_in[s][p] : 0.0;
      rt[s] = src[s] * dt;
      qp[s] = fabove[s] * tsorhodz;
      c1[s] = valid && gtp(rt[s], rtmin[s]);
      c2[s] = valid && gtp(qp[s], rtmin[s]);
      any = any || c1[s] || c2[s];
    }
    const double lrho = any ? fm::flog(rho) : 0.0;
    const double wlbda =
        (c1[0] || c2[0]) ? 6.6e-8 * fm::fdiv(101325.0, sed_load(io.pabs, p)) * (sed_load(io.tht, p) * (1.0 / 293.15))
                         : 0.0;
    // a species that no lane of the warp moves at this level (content at or
    // below its threshold and not negative, nothing falling in) has a zero
    // flux and keeps its source; the warp skips its arithmetic
    bool live[5];
#pragma unroll
    for (int s = 0; s < 5; ++s)
      live[s] = !(s == 0 && skip_c) && !__all_sync(0xffffffffu, !c1[s] && !c2[s] && !negd(rt[s]) && zerod_(fabove[s]));
    double w1[5], w2[5];
    warp_power_speeds(c, live, c1, rt, c2, qp, lrho, fx, w1, w2);
    if (live[0]) warp_fall_speeds(c, 0, c1[0], rt[0], c2[0], qp[0], lrho, wlbda, cp, fx, w1[0], w2[0]);
    if (live[2]) warp_fall_speeds(c, 2, c1[2], rt[2], c2[2], qp[2], lrho, wlbda, cp, fx, w1[2], w2[2]);
#pragma unroll
    for (int s = 0; s < 5; ++s) {
      if (s == 0 && skip_c) continue;
      if (!live[s]) {
        if (valid) {
          if (io.src_out[s] && io.src_out[s] != io.src_in[s]) io.src_out[s][p] = src[s];
          if (io.fpr[s]) io.fpr[s][p] = 0.0;
        }
        fabove[s] = 0.0;
        continue;
      }
      double flux = dmin(rhodz_idt * rt[s], w1[s] * rho * rt[s]);
      if (!zerod_(w2[s])) flux += pmax0(1.0 - dz_idt * fm::frcp(w2[s])) * fabove[s];
      if (valid) {
        if (io.src_out[s]) {
          if (fortran) io.src_out[s][p] = src[s] + tso_idt * (fabove[s] - flux);
          else io.src_out[s][p] = src[s] + fm::fdiv(fabove[s] - flux, rhodz * dt);
        }
        if (io.fpr[s]) io.fpr[s][p] = flux;
      }
      fabove[s] = flux;
    }
  }
#pragma unroll
  for (int s = 0; s < 5; ++s)
    if (valid && !(s == 0 && skip_c) && io.inpr[s]) io.inpr[s][col] = fabove[s] / c.RHOLW;
}

// 128 threads, ~148 registers: 3 blocks per SM; capping the registers for
// 4 or 5 blocks (SED_MIN_BLOCKS: 128 / 96 registers) measured 39.7 / 44.0
// against 38.0 ms at 1024x1024 columns.
#ifndef SED_MIN_BLOCKS
#define SED_MIN_BLOCKS 1
#endif
__global__ void __launch_bounds__(128, SED_MIN_BLOCKS) sedimentation_kernel(const __grid_constant__ Cst c, SedArgs a)
{
  const long col = blockIdx.x * (long)blockDim.x + threadIdx.x;
  __shared__ double fx[12];
  if (threadIdx.x == 0) fall_exponents(c, fx);
  __syncthreads();
  // whole warps run the sweep (they share the fall-speed evaluations); a
  // warp entirely past the last column leaves
  const bool valid = col < a.nij;
  if (__all_sync(0xffffffffu, !valid)) return;
  // PHYEX skips the cloud species when LSEDIC is off
  const bool skip_c = a.fortran && c.LSEDIC == 0.0;
  if (skip_c && valid) {
    if (a.fpr[0])
      for (int k = 0; k < a.nk; ++k) a.fpr[0][(long)k * a.nij + col] = 0.0;
    a.inpr[0][col] = 0.0;
  }
  const bool has_st = a.sea != nullptr && a.town != nullptr;
  const double sea = (a.sea && valid) ? a.sea[col] : 0.0, town = (a.town && valid) ? a.town[col] : 0.0;
  const CloudPar cp = cloud_params(c, a.fortran, has_st, sea, town);
  SedColumnIO io;
  io.rhodref = a.rhodref; io.dzz = a.dzz; io.pabs = a.pabs; io.tht = a.tht;
  for (int s = 0; s < 5; ++s) {
    io.src_in[s] = a.src[s];
    io.src_out[s] = a.src[s];
    io.fpr[s] = a.fpr[s];
    io.inpr[s] = a.inpr[s];
  }
  io.nij = a.nij;
  io.nk = a.nk;
  sed_column_forward_warp(c, a.fortran, skip_c, cp, a.dt, io, col, valid, fx);
  // hail (NRR = 7), an independent species: its own sweep of the column
  if (a.hsrc && valid) sed_hail_column(c, a.dt, a.rhodref, a.dzz, a.hsrc, a.hfpr, a.hinpr, a.nij, a.nk, col);
}

// Fog deposition on the lowest level (rain_ice.F90:876-895).
// SEDIM = SPLI: one column per thread (sed_split_column).
__global__ void __launch_bounds__(128) sedimentation_split_kernel(const __grid_constant__ Cst c,
                                                                  const __grid_constant__ SplitArgs a)
{
  const long col = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (col >= a.sed.nij) return;
  const bool has_st = a.sed.sea != nullptr && a.sed.town != nullptr;
  const double sea = has_st ? a.sed.sea[col] : 0.0, town = has_st ? a.sed.town[col] : 0.0;
  const CloudPar cp = cloud_params(c, true, has_st, sea, town);
  const long n = (long)a.sed.nij * a.sed.nk;
  SplitColumnIO io;
  io.rhodref = a.sed.rhodref; io.dzz = a.sed.dzz; io.pabs = a.sed.pabs; io.tht = a.sed.tht; io.exn = a.exn;
  io.rvt = a.rvt; io.rvs = a.rvs; io.ths = a.ths;
  for (int s = 0; s < 5; ++s) {
    io.rt[s] = a.rt[s];
    io.src[s] = a.sed.src[s];
    io.fpr[s] = a.sed.fpr[s];
    io.inpr[s] = a.sed.inpr[s];
  }
  io.nsp = a.rht ? 6 : 5;
  io.rt[5] = a.rht;
  io.src[5] = a.sed.hsrc;
  io.fpr[5] = a.sed.hfpr;
  io.inpr[5] = a.sed.hinpr;
  io.rtmp = a.scratch;
  io.ext = a.scratch + n;
  io.nij = a.sed.nij;
  io.nk = a.sed.nk;
  if (!sed_split_column(c, cp, a.sed.dt, io, col, a.max_iter)) atomicOr(a.status, ICE3GB_DEV_SED_CAP);
}

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

cudaError_t launch_sedimentation_split(const Cst &c, const SplitArgs &a, cudaStream_t s)
{
  const long n = a.sed.nij;
  const int threads = 128;
  sedimentation_split_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, s>>>(c, a);
  return cudaGetLastError();
}

cudaError_t launch_fog_deposition(const Cst &c, const FogArgs &a, cudaStream_t s)
{
  const int threads = 256;
  fog_deposition_kernel<<<(unsigned)((a.nij + threads - 1) / threads), threads, 0, s>>>(c, a);
  return cudaGetLastError();
}
