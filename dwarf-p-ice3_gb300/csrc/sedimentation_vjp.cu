// sedimentation_vjp.cu — adjoint (vector-Jacobian product) of the
// statistical sedimentation sweep.
//
// One thread per column: sed_column_forward recomputes the column's fluxes
// F_k of the five species into a scratch array (nothing is kept from the
// forward call), then sed_column_vjp (sedimentation_point.cuh) runs the
// hand-written reverse sweep bottom-up.  Consecutive threads own consecutive
// columns, so every level access is coalesced.
#include "ice3gb_device.cuh"
#include "ice3gb_kernels.h"
#include "sedimentation_point.cuh"

namespace {
using namespace ice3sed;

__global__ void __launch_bounds__(128) sedimentation_vjp_kernel(const __grid_constant__ Cst c,
                                                                const __grid_constant__ SedVjpArgs a)
{
  const long col = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (col >= a.nij) return;
  const bool skip_c = a.fortran && c.LSEDIC == 0.0;
  const bool has_st = a.sea != nullptr && a.town != nullptr;
  const double sea = a.sea ? a.sea[col] : 0.0, town = a.town ? a.town[col] : 0.0;
  const CloudPar cp = cloud_params(c, a.fortran, has_st, sea, town);
  SedColumnIO io;
  io.rhodref = a.rhodref; io.dzz = a.dzz; io.pabs = a.pabs; io.tht = a.tht;
  double *flux[5];
  for (int s = 0; s < 5; ++s) {
    io.src_in[s] = a.src[s];
    io.src_out[s] = nullptr;
    io.inpr[s] = nullptr;
    flux[s] = a.flux + (long)s * a.nij * a.nk;
    io.fpr[s] = flux[s];
  }
  io.nij = a.nij;
  io.nk = a.nk;
  SedCotangents g;
  SedGradients gx;
  for (int s = 0; s < 5; ++s) {
    g.src[s] = a.g.src[s];
    g.inpr[s] = a.g.inpr[s];
    g.fpr[s] = a.g.fpr[s];
    gx.src[s] = a.gx.src[s];
  }
  gx.rhodref = a.gx.rhodref; gx.dzz = a.gx.dzz; gx.pabs = a.gx.pabs; gx.tht = a.gx.tht;
  sed_column_forward(c, a.fortran, skip_c, cp, a.dt, io, col);
  sed_column_vjp(c, a.fortran, skip_c, cp, a.dt, io, flux, g, gx, col);
}

}  // namespace

cudaError_t launch_sedimentation_vjp(const Ice3gbConstants &c, const SedVjpArgs &a, cudaStream_t s)
{
  const int threads = 128;
  sedimentation_vjp_kernel<<<(unsigned)((a.nij + threads - 1) / threads), threads, 0, s>>>(c, a);
  return cudaGetLastError();
}
