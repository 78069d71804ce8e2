// ice_adjust_vjp.cu — adjoint (vector-Jacobian product) of ice_adjust.
//
// One grid point per thread (grid-stride loop): the inputs and the output
// cotangents are loaded, ia_point_vjp (ice_adjust_point.cuh) recomputes the
// forward intermediates in registers and runs the hand-written reverse pass,
// and the wanted input gradients are stored.  Nothing from the forward call
// is kept (recompute-forward).  A per-column sigqsat has its gradient summed
// over the levels by a second kernel (a fixed-order sum: deterministic).
#include "ice3gb_device.cuh"
#include "ice3gb_kernels.h"
#include "ice_adjust_point.cuh"

namespace {
using namespace ice3ia;

__device__ __forceinline__ double ldz(const double *p, long i) { return p ? __ldg(p + i) : 0.0; }

__global__ void __launch_bounds__(256) ice_adjust_vjp_kernel(const __grid_constant__ Cst c,
                                                             const __grid_constant__ IaVjpArgs a)
{
  const IaDerived d = ia_derived(c);
  const double inv_dt = 1.0 / a.dt;
  const long n = (long)a.nij * a.nk;
  const Ice3gbIceAdjustFields &f = a.f;
  const Ice3gbIceAdjustCotangents &g = a.g;
  const Ice3gbIceAdjustGradients &gx = a.gx;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < n; p += (long)gridDim.x * blockDim.x) {
    IaIn x;
    x.sigqsat = f.sigqsat_3d ? ld1(f.sigqsat, p) : ld1(f.sigqsat, p % a.nij);
    x.pabs = ld1(f.pabs, p); x.sigs = ld1(f.sigs, p); x.th = ld1(f.th, p); x.exn = ld1(f.exn, p);
    x.exn_ref = ld1(f.exn_ref, p); x.rho = ld1(f.rho_dry_ref, p);
    x.rv = ld1(f.rv, p); x.rc = ld1(f.rc, p); x.ri = ld1(f.ri, p); x.rr = ld1(f.rr, p); x.rs = ld1(f.rs, p);
    x.rg = ld1(f.rg, p); x.cf_mf = ld1(f.cf_mf, p); x.rc_mf = ld1(f.rc_mf, p); x.ri_mf = ld1(f.ri_mf, p);
    x.rvs = ld1(f.rvs, p); x.rcs = ld1(f.rcs, p); x.ris = ld1(f.ris, p); x.ths = ld1(f.ths, p);
    IaOut gy;
    gy.t = ldz(g.t, p); gy.rv_out = ldz(g.rv_out, p); gy.rc_out = ldz(g.rc_out, p); gy.ri_out = ldz(g.ri_out, p);
    gy.cldfr = ldz(g.cldfr, p); gy.hlc_hrc = ldz(g.hlc_hrc, p); gy.hlc_hcf = ldz(g.hlc_hcf, p);
    gy.hli_hri = ldz(g.hli_hri, p); gy.hli_hcf = ldz(g.hli_hcf, p); gy.cph = ldz(g.cph, p);
    gy.lv = ldz(g.lv, p); gy.ls = ldz(g.ls, p); gy.rvs = ldz(g.rvs, p); gy.rcs = ldz(g.rcs, p);
    gy.ris = ldz(g.ris, p); gy.ths = ldz(g.ths, p);
    IaIn b;
    ia_point_vjp(c, d, a.dt, inv_dt, x, gy, b);
#define ST(field, member) if (gx.field) gx.field[p] = b.member;
    ST(pabs, pabs) ST(sigs, sigs) ST(th, th) ST(exn, exn) ST(exn_ref, exn_ref) ST(rho_dry_ref, rho)
    ST(rv, rv) ST(rc, rc) ST(ri, ri) ST(rr, rr) ST(rs, rs) ST(rg, rg) ST(cf_mf, cf_mf) ST(rc_mf, rc_mf)
    ST(ri_mf, ri_mf) ST(rvs, rvs) ST(rcs, rcs) ST(ris, ris) ST(ths, ths)
#undef ST
    if (a.sigqsat_out) a.sigqsat_out[p] = b.sigqsat;
  }
}

// out[ij] = sum over k of in[k][ij], k ascending.
__global__ void column_sum_kernel(const double *__restrict__ in, double *__restrict__ out, int nij, int nk)
{
  const long col = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (col >= nij) return;
  double s = 0.0;
  for (int k = 0; k < nk; ++k) s += in[(long)k * nij + col];
  out[col] = s;
}

}  // namespace

cudaError_t launch_ice_adjust_vjp(const Ice3gbConstants &c, const IaVjpArgs &a, int num_sms, cudaStream_t s)
{
  const long n = (long)a.nij * a.nk;
  long blocks = (n + 255) / 256;
  if (blocks > (long)num_sms * 32) blocks = (long)num_sms * 32;
  ice_adjust_vjp_kernel<<<(unsigned)blocks, 256, 0, s>>>(c, a);
  return cudaGetLastError();
}

cudaError_t launch_column_sum(const double *in, double *out, int nij, int nk, cudaStream_t s)
{
  column_sum_kernel<<<(unsigned)((nij + 127) / 128), 128, 0, s>>>(in, out, nij, nk);
  return cudaGetLastError();
}
