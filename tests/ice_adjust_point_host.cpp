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

// OCND2 forward on a [nk][nij] grid, as ice_adjust_ocnd2_kernel runs it:
// in = the 20 IaIn fields (sigqsat per point), zz [nk][nij], ice_cld_wgt
// [nij], tiwmx = ESTABW then ESTABI; out = the 16 IaOut fields, out2 =
// icldfr, wcldfr, ssio, ssiu.
extern "C" void ia_ocnd2_host(const Ice3gbConstants *c, double dt, long nij, long nk, const double *const *in,
                              const double *zz, const double *wgt, const double *tiwmx, double *const *out,
                              double *const *out2)
{
  const IaDerived d = ia_derived(*c);
  for (long p = 0; p < nij * nk; ++p) {
    IaIn x;
    gather_in(in, p, x);
    const long k = p / nij, col = p - k * nij;
    const long kp = k + 1 < nk ? k + 1 : nk - 1;
    Ocnd2In oi;
    oi.estw = tiwmx;
    oi.esti = tiwmx + kTiwmxN;
    oi.z = zz[p];
    oi.dz = zz[kp * nij + col] - zz[(kp - 1) * nij + col];
    oi.ice_cld_wgt = wgt[col];
    oi.bottom = k == 0;
    IaOut o;
    Ocnd2Out oo;
    ia_point<true>(*c, d, dt, 1.0 / dt, x, o, nullptr, &oi, &oo);
    const double *v = &o.t;
    for (int j = 0; j < 16; ++j) out[j][p] = v[j];
    out2[0][p] = oo.icldfr;
    out2[1][p] = oo.wcldfr;
    out2[2][p] = oo.ssio;
    out2[3][p] = oo.ssiu;
  }
}
