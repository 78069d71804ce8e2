// Host build of the rain_ice kernel's per-point code (the same
// rain_ice_point() the device runs), exported for tests/test_rain_ice_host.py.
#include <vector>

#include "../dwarf-p-ice3_gb300/csrc/rain_ice_point.cuh"

extern "C" int rain_ice_points_host(const Ice3gbConstants *c, const Ice3gbLuts *luts, int nij, int nk, double dt,
                                    int max_passes, const Ice3gbRainIceFields *f, unsigned int *keys)
{
  ice3pt::Derived d;
  ice3pt::make_derived(*c, d);
  int capped_any = 0;
  for (long p = 0; p < (long)nij * nk; ++p) {
    bool capped;
    keys[p] = ice3pt::rain_ice_point(*c, d, reinterpret_cast<const double *>(luts), *f, p, dt, max_passes, capped);
    capped_any |= capped;
  }
  return capped_any;
}

// The same with the subgrid warm-process options (SUBG_RC_RR_ACCR /
// SUBG_RR_EVAP): the precipitation fraction of each column first when a
// PRFR option is set (prfr_column), then the points.
extern "C" int rain_ice_points_host_subg(const Ice3gbConstants *c, const Ice3gbLuts *luts, int nij, int nk,
                                         double dt, int max_passes, const Ice3gbRainIceFields *f,
                                         unsigned int *keys)
{
  ice3pt::Derived d;
  ice3pt::make_derived(*c, d);
  if ((int)c->SUBG_RC_RR_ACCR == 1 || (int)c->SUBG_RR_EVAP == 2)
    for (long col = 0; col < nij; ++col) ice3pt::prfr_column(*c, *f, nij, nk, col);
  int capped_any = 0;
  for (long p = 0; p < (long)nij * nk; ++p) {
    bool capped;
    keys[p] = ice3pt::rain_ice_point<false, true>(*c, d, reinterpret_cast<const double *>(luts), *f, p, dt,
                                                  max_passes, capped);
    capped_any |= capped;
  }
  return capped_any;
}

// With hail (NRR = 7, the kernel's H instantiation; the hail kernels read
// from the full table), any warm-process options.
extern "C" int rain_ice_points_host_hail(const Ice3gbConstants *c, const Ice3gbLuts *luts, int nij, int nk,
                                         double dt, int max_passes, const Ice3gbRainIceFields *f,
                                         unsigned int *keys)
{
  ice3pt::Derived d;
  ice3pt::make_derived(*c, d);
  const double *lt = reinterpret_cast<const double *>(luts);
  const bool subg = (int)c->SUBG_RC_RR_ACCR != 0 || (int)c->SUBG_RR_EVAP != 0;
  if ((int)c->SUBG_RC_RR_ACCR == 1 || (int)c->SUBG_RR_EVAP == 2)
    for (long col = 0; col < nij; ++col) ice3pt::prfr_column<true>(*c, *f, nij, nk, col);
  int capped_any = 0;
  for (long p = 0; p < (long)nij * nk; ++p) {
    bool capped;
    keys[p] = subg ? ice3pt::rain_ice_point<false, true, true>(*c, d, lt, *f, p, dt, max_passes, capped, nullptr, lt)
                   : ice3pt::rain_ice_point<false, false, true>(*c, d, lt, *f, p, dt, max_passes, capped, nullptr, lt);
    capped_any |= capped;
  }
  return capped_any;
}

// With OCND2 (the kernel's O instantiation, with any warm option and the
// time splitting): the precipitation fraction of a PRFR option and the column
// heights and droplet concentrations first (prfr_column, ocnd2_column), then
// the points; tw = the six TIWMX tables (ice3o_tiwmx_all layout).
extern "C" int rain_ice_points_host_ocnd2(const Ice3gbConstants *c, const Ice3gbLuts *luts, int nij, int nk,
                                          double dt, int max_passes, const Ice3gbRainIceFields *f, const double *tw,
                                          unsigned int *keys)
{
  ice3pt::Derived d;
  ice3pt::make_derived(*c, d);
  const double *lt = reinterpret_cast<const double *>(luts);
  const long n = (long)nij * nk;
  std::vector<double> ocs(2 * (size_t)n);
  const bool subg = (int)c->SUBG_RC_RR_ACCR != 0 || (int)c->SUBG_RR_EVAP != 0;
  const bool ts = c->MRSTEP != 0.0 || c->TSTEP_TS != 0.0;
  if ((int)c->SUBG_RC_RR_ACCR == 1 || (int)c->SUBG_RR_EVAP == 2)
    for (long col = 0; col < nij; ++col) ice3pt::prfr_column(*c, *f, nij, nk, col);
  for (long col = 0; col < nij; ++col) ice3pt::ocnd2_column(*c, *f, nij, nk, col, ocs.data(), ocs.data() + n);
  int capped_any = 0;
  double *zz = ocs.data(), *conc = ocs.data() + n;
  for (long p = 0; p < n; ++p) {
    bool capped;
    using namespace ice3pt;
    if (subg)
      keys[p] = ts ? rain_ice_point<false, true, false, true, true>(*c, d, lt, *f, p, dt, max_passes, capped, nullptr,
                                                                    lt, tw, zz, conc)
                   : rain_ice_point<false, true, false, true>(*c, d, lt, *f, p, dt, max_passes, capped, nullptr, lt,
                                                              tw, zz, conc);
    else
      keys[p] = ts ? rain_ice_point<false, false, false, true, true>(*c, d, lt, *f, p, dt, max_passes, capped, nullptr,
                                                                     lt, tw, zz, conc)
                   : rain_ice_point<false, false, false, true>(*c, d, lt, *f, p, dt, max_passes, capped, nullptr, lt,
                                                               tw, zz, conc);
    capped_any |= capped;
  }
  return capped_any;
}

// With the MRSTEP / TSTEP_TS time splitting (the kernel's TS instantiation),
// any warm option, with or without hail.
extern "C" int rain_ice_points_host_ts(const Ice3gbConstants *c, const Ice3gbLuts *luts, int nij, int nk, double dt,
                                       int max_passes, const Ice3gbRainIceFields *f, unsigned int *keys)
{
  ice3pt::Derived d;
  ice3pt::make_derived(*c, d);
  const double *lt = reinterpret_cast<const double *>(luts);
  const bool subg = (int)c->SUBG_RC_RR_ACCR != 0 || (int)c->SUBG_RR_EVAP != 0;
  const bool hail = (int)c->NRR == 7;
  if ((int)c->SUBG_RC_RR_ACCR == 1 || (int)c->SUBG_RR_EVAP == 2)
    for (long col = 0; col < nij; ++col) {
      if (hail) ice3pt::prfr_column<true>(*c, *f, nij, nk, col);
      else ice3pt::prfr_column<false>(*c, *f, nij, nk, col);
    }
  int capped_any = 0;
  for (long p = 0; p < (long)nij * nk; ++p) {
    bool capped;
    unsigned int k;
    if (hail)
      k = subg ? ice3pt::rain_ice_point<false, true, true, false, true>(*c, d, lt, *f, p, dt, max_passes, capped, nullptr, lt)
               : ice3pt::rain_ice_point<false, false, true, false, true>(*c, d, lt, *f, p, dt, max_passes, capped, nullptr, lt);
    else
      k = subg ? ice3pt::rain_ice_point<false, true, false, false, true>(*c, d, lt, *f, p, dt, max_passes, capped)
               : ice3pt::rain_ice_point<false, false, false, false, true>(*c, d, lt, *f, p, dt, max_passes, capped);
    keys[p] = k;
    capped_any |= capped;
  }
  return capped_any;
}

// Host build of the surrogate's feature / target sampling (surrogate_point.cuh):
// per grid point the 16 features and the five plain slow rates of a micro
// point at its first hard pass; micro[p] = 0 elsewhere.
#include "../dwarf-p-ice3_gb300/csrc/surrogate_point.cuh"

extern "C" long sur_sample_host(const Ice3gbConstants *c, const Ice3gbLuts *luts, int nij, int nk, double dt,
                                const Ice3gbRainIceFields *f, float *feat, double *rate, unsigned char *micro)
{
  ice3pt::Derived d;
  ice3pt::make_derived(*c, d);
  long cnt = 0;
  for (long p = 0; p < (long)nij * nk; ++p) {
    const bool m = ice3sur::sample_point<true>(*c, d, reinterpret_cast<const double *>(luts), *f, p, dt, feat + 16 * p,
                                         rate + 5 * p);
    micro[p] = m ? 1 : 0;
    cnt += m;
  }
  return cnt;
}
