// Host build of the ice_adjust per-point forward and its hand-written
// reverse-mode derivative (the functions the device kernels run), exported
// for tests/test_adjoint_host.py.  Fields are passed as arrays of n values in
// the order of IaIn (20 inputs) and IaOut (16 outputs).
#include "../dwarf-p-ice3_gb300/csrc/ice_adjust_point.cuh"

using namespace ice3ia;

static void gather_in(const double *const *in, long p, IaIn &x)
{
  double *v = &x.sigqsat;
  for (int k = 0; k < 20; ++k) v[k] = in[k][p];
}

extern "C" void ia_forward_host(const Ice3gbConstants *c, double dt, long n, const double *const *in, double *const *out)
{
  const IaDerived d = ia_derived(*c);
  for (long p = 0; p < n; ++p) {
    IaIn x;
    gather_in(in, p, x);
    IaOut o;
    ia_point(*c, d, dt, 1.0 / dt, x, o);
    const double *v = &o.t;
    for (int k = 0; k < 16; ++k) out[k][p] = v[k];
  }
}

extern "C" void ia_vjp_host(const Ice3gbConstants *c, double dt, long n, const double *const *in,
                            const double *const *gout, double *const *gin)
{
  const IaDerived d = ia_derived(*c);
  for (long p = 0; p < n; ++p) {
    IaIn x, b;
    gather_in(in, p, x);
    IaOut g;
    double *gv = &g.t;
    for (int k = 0; k < 16; ++k) gv[k] = gout[k] ? gout[k][p] : 0.0;
    ia_point_vjp(*c, d, dt, 1.0 / dt, x, g, b);
    const double *bv = &b.sigqsat;
    for (int k = 0; k < 20; ++k) gin[k][p] = bv[k];
  }
}

// PSRCS (s'r_c'/sigma_s^2) of each point, as the forward kernel's SRC
// instantiation writes it.
extern "C" void ia_srcs_host(const Ice3gbConstants *c, double dt, long n, const double *const *in, double *srcs)
{
  const IaDerived d = ia_derived(*c);
  for (long p = 0; p < n; ++p) {
    IaIn x;
    gather_in(in, p, x);
    IaOut o;
    ia_point(*c, d, dt, 1.0 / dt, x, o, srcs + p);
  }
}
