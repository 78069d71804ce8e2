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

// Host build of the time-split sedimentation (SEDIM = SPLI) and its
// negativity correction on a rain_ice field set; scratch: 2 nij nk doubles.
extern "C" int sed_split_host(const Ice3gbConstants *c, int nij, int nk, double dt, const Ice3gbRainIceFields *f,
                              double *scratch)
{
  const bool has_st = f->sea && f->town;
  int ok = 1;
  for (long col = 0; col < nij; ++col) {
    const CloudPar cp = cloud_params(*c, true, has_st, has_st ? f->sea[col] : 0.0, has_st ? f->town[col] : 0.0);
    SplitColumnIO io;
    io.rhodref = f->rhodref; io.dzz = f->dzz; io.pabs = f->pabs; io.tht = f->tht; io.exn = f->exn;
    io.rt[0] = f->rct; io.rt[1] = f->rrt; io.rt[2] = f->rit; io.rt[3] = f->rst; io.rt[4] = f->rgt;
    io.rvt = f->rvt; io.rvs = f->rvs; io.ths = f->ths;
    io.src[0] = f->rcs; io.src[1] = f->rrs; io.src[2] = f->ris; io.src[3] = f->rss; io.src[4] = f->rgs;
    io.fpr[0] = f->fpr_c; io.fpr[1] = f->fpr_r; io.fpr[2] = f->fpr_i; io.fpr[3] = f->fpr_s; io.fpr[4] = f->fpr_g;
    io.inpr[0] = f->inprc; io.inpr[1] = f->inprr; io.inpr[2] = f->inpri; io.inpr[3] = f->inprs; io.inpr[4] = f->inprg;
    const bool hail = (int)c->NRR == 7;
    io.nsp = hail ? 6 : 5;
    io.rt[5] = hail ? f->rht : nullptr;
    io.src[5] = hail ? f->rhs : nullptr;
    io.fpr[5] = hail ? f->fpr_h : nullptr;
    io.inpr[5] = hail ? f->inprh : nullptr;
    io.rtmp = scratch;
    io.ext = scratch + (long)nij * nk;
    io.nij = nij;
    io.nk = nk;
    ok &= sed_split_column(*c, cp, dt, io, col, 10000) ? 1 : 0;
  }
  return ok;
}

// The statistical sweep of a rain_ice call (Fortran semantics, sea/town
// weighting, hail when NRR = 7), as the rain_ice entry points launch it.
extern "C" void sed_stat_rain_ice_host(const Ice3gbConstants *c, int nij, int nk, double dt,
                                       const Ice3gbRainIceFields *f)
{
  const bool has_st = f->sea && f->town;
  const bool skip_c = c->LSEDIC == 0.0;
  const bool hail = (int)c->NRR == 7;
  for (long col = 0; col < nij; ++col) {
    const CloudPar cp = cloud_params(*c, true, has_st, has_st ? f->sea[col] : 0.0, has_st ? f->town[col] : 0.0);
    SedColumnIO io;
    io.rhodref = f->rhodref; io.dzz = f->dzz; io.pabs = f->pabs; io.tht = f->tht;
    double *src[5] = {f->rcs, f->rrs, f->ris, f->rss, f->rgs};
    double *fpr[5] = {f->fpr_c, f->fpr_r, f->fpr_i, f->fpr_s, f->fpr_g};
    double *inpr[5] = {f->inprc, f->inprr, f->inpri, f->inprs, f->inprg};
    for (int s = 0; s < 5; ++s) {
      io.src_in[s] = src[s];
      io.src_out[s] = src[s];
      io.fpr[s] = fpr[s];
      io.inpr[s] = inpr[s];
    }
    io.nij = nij;
    io.nk = nk;
    if (skip_c) {
      f->inprc[col] = 0.0;
      if (f->fpr_c)
        for (int k = 0; k < nk; ++k) f->fpr_c[(long)k * nij + col] = 0.0;
    }
    sed_column_forward(*c, true, skip_c, cp, dt, io, col);
    if (hail) sed_hail_column(*c, dt, f->rhodref, f->dzz, f->rhs, f->fpr_h, f->inprh, nij, nk, col);
  }
}
