// Host build of the sedimentation column sweep and its hand-written adjoint
// (the functions the device kernels run), exported for
// tests/test_adjoint_host.py.  sea = town = 0 (no land/sea weighting).
#include "../dwarf-p-ice3_gb300/csrc/sedimentation_point.cuh"

using namespace ice3sed;

static SedColumnIO io_of(int nij, int nk, const double *rho, const double *dz, const double *pabs, const double *tht,
                         const double *const *src)
{
  SedColumnIO io;
  io.rhodref = rho; io.dzz = dz; io.pabs = pabs; io.tht = tht;
  for (int s = 0; s < 5; ++s) {
    io.src_in[s] = src[s];
    io.src_out[s] = nullptr;
    io.fpr[s] = nullptr;
    io.inpr[s] = nullptr;
  }
  io.nij = nij;
  io.nk = nk;
  return io;
}

extern "C" void sed_forward_host(const Ice3gbConstants *c, int nij, int nk, double dt, int fortran, const double *rho,
                                 const double *dz, const double *pabs, const double *tht, const double *const *src,
                                 double *const *src_out, double *const *inpr)
{
  const bool skip_c = fortran && c->LSEDIC == 0.0;
  const CloudPar cp = cloud_params(*c, fortran != 0, false, 0.0, 0.0);
  SedColumnIO io = io_of(nij, nk, rho, dz, pabs, tht, src);
  for (int s = 0; s < 5; ++s) { io.src_out[s] = src_out[s]; io.inpr[s] = inpr[s]; }
  for (long col = 0; col < nij; ++col) sed_column_forward(*c, fortran != 0, skip_c, cp, dt, io, col);
}

extern "C" void sed_vjp_host(const Ice3gbConstants *c, int nij, int nk, double dt, int fortran, const double *rho,
                             const double *dz, const double *pabs, const double *tht, const double *const *src,
                             const double *const *g_src, const double *const *g_inpr, double *const *gx_src,
                             double *grho, double *gdz, double *gpabs, double *gtht, double *flux_scratch)
{
  const bool skip_c = fortran && c->LSEDIC == 0.0;
  const CloudPar cp = cloud_params(*c, fortran != 0, false, 0.0, 0.0);
  SedColumnIO io = io_of(nij, nk, rho, dz, pabs, tht, src);
  double *flux[5];
  for (int s = 0; s < 5; ++s) {
    flux[s] = flux_scratch + (long)s * nij * nk;
    io.fpr[s] = flux[s];
  }
  SedCotangents g;
  SedGradients gx;
  for (int s = 0; s < 5; ++s) {
    g.src[s] = g_src[s];
    g.inpr[s] = g_inpr[s];
    g.fpr[s] = nullptr;
    gx.src[s] = gx_src[s];
  }
  gx.rhodref = grho; gx.dzz = gdz; gx.pabs = gpabs; gx.tht = gtht;
  for (long col = 0; col < nij; ++col) {
    sed_column_forward(*c, fortran != 0, skip_c, cp, dt, io, col);
    sed_column_vjp(*c, fortran != 0, skip_c, cp, dt, io, flux, g, gx, col);
  }
}
