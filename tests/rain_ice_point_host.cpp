// Host build of the rain_ice kernel's per-point code (the same
// rain_ice_point() the device runs), exported for tests/test_rain_ice_host.py.
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
