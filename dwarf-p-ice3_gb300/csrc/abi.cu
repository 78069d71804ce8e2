// abi.cu — extern "C" entry points of libice3gb.so (declared in include/ice3gb.h).
//
// Handle = one immutable constants table + its lookup tables on one device,
// plus a sticky device status word.  Every rain_ice call takes its scratch
// (work counter, pass keys) from the stream-ordered allocator on the caller's
// stream, so concurrent calls on distinct streams share nothing but the
// atomically updated status word.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "ice3gb_device.cuh"
#include "ice3gb_kernels.h"

namespace {

constexpr uint32_t kMagic = 0x1CE3B300u;
constexpr long kMaxPoints = 1L << 40;

// Resources of the slab pipeline of ice3gb_physics_step_host (created on
// first use, grow-only): a copy-in stream, two compute streams (slabs
// alternate between them, so that one slab's kernels fill the SMs the tail
// of the other's leaves idle), a copy-out stream, NB rotating sets of slab
// buffers, and the full-size evap3d / pass-key arrays whose fix-up needs the
// maximum pass key over all slabs.
struct HostPipe {
  static constexpr int NB = 4, NC = 2;
  bool ready = false;
  cudaStream_t s_in = nullptr, s_cmp[NC] = {}, s_out = nullptr;
  cudaEvent_t in_done[NB] = {}, cmp_done[NB] = {}, out_done[NB] = {};
  cudaEvent_t start = nullptr, fix_done = nullptr, cleared = nullptr, cmp_end[NC] = {};
  char *buf[NB] = {};
  size_t buf_cap = 0;              // bytes per slab set
  double *evap_all = nullptr;      // [n] evap3d, slab after slab
  unsigned int *keys_all = nullptr;  // 4 control words + [n] pass keys
  size_t all_cap = 0;              // points
};

struct Handle {
  uint32_t magic;
  Ice3gbConstants c;
  double *d_luts;
  double *d_tiwmx;   // OCND2 TIWMX tables (six, see ice3gb_device.cuh)
  unsigned int *d_status;
  int device, num_sms;
  bool rain_ice_ok;
  std::string rain_ice_why;
  // staging buffers of the _host entry points (grow-only)
  double *d_stage;
  size_t stage_cap;
  HostPipe pipe;
  std::mutex mu;
  char err[512];
  // per-kernel timing (ice3gb_profile_*)
  bool profiling;
  std::mutex prof_mu;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> events;
};

enum {
  K_ICE_ADJUST = 0, K_SEDIM, K_RAIN_ICE, K_EVAP_FIXUP, K_FOG, K_ORDER, K_IA_VJP, K_SED_VJP, K_SUR_SAMPLE, K_SUR_MLP,
  K_SUR_RAIN_ICE, K_PRFR, K_COUNT
};
const char *kKernelNames[K_COUNT] = {"ice_adjust", "sedimentation", "rain_ice", "rain_ice_evap_fixup",
                                     "fog_deposition", "rain_ice_order", "ice_adjust_vjp", "sedimentation_vjp",
                                     "surrogate_sample", "surrogate_mlp", "rain_ice_surrogate",
                                     "rain_ice_precip_fraction"};

// Brackets one launch with events when the handle is profiling.
struct ProfScope {
  Handle *h;
  int id;
  cudaStream_t s;
  cudaEvent_t a = nullptr, b = nullptr;
  ProfScope(Handle *h_, int id_, cudaStream_t s_) : h(h_), id(id_), s(s_)
  {
    if (h->profiling && cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess)
      cudaEventRecord(a, s);
  }
  ~ProfScope()
  {
    if (a && b) {
      cudaEventRecord(b, s);
      std::lock_guard<std::mutex> lock(h->prof_mu);
      h->events.push_back({id, {a, b}});
    }
  }
};

thread_local char g_err[512] = "";

int fail(Handle *h, int code, const char *fmt, ...) __attribute__((format(printf, 3, 4)));
int fail(Handle *h, int code, const char *fmt, ...)
{
  char *dst = h ? h->err : g_err;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(dst, 512, fmt, ap);
  va_end(ap);
  if (h) snprintf(g_err, sizeof(g_err), "%s", h->err);
  return code;
}

int cuda_fail(Handle *h, cudaError_t e, const char *where)
{
  return fail(h, ICE3GB_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

Handle *as_handle(void *p)
{
  Handle *h = static_cast<Handle *>(p);
  if (!h || h->magic != kMagic) return nullptr;
  return h;
}

int check_device(Handle *h)
{
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaGetDevice");
  if (dev != h->device)
    return fail(h, ICE3GB_ERR_HANDLE, "handle created on device %d, current device is %d", h->device, dev);
  return ICE3GB_OK;
}

int check_shape(Handle *h, int nij, int nk)
{
  if (nij <= 0 || nk <= 0) return fail(h, ICE3GB_ERR_SHAPE, "nij=%d nk=%d must be positive", nij, nk);
  if ((long)nij * nk > kMaxPoints) return fail(h, ICE3GB_ERR_SHAPE, "nij*nk too large");
  return ICE3GB_OK;
}

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

#define REQUIRE(ptr)                                                              \
  do {                                                                            \
    if (!(ptr)) return fail(h, ICE3GB_ERR_NULL, "required field %s is NULL", #ptr); \
  } while (0)

int validate_ice_adjust(Handle *h, const Ice3gbIceAdjustFields *f, int nk)
{
  if (!f) return fail(h, ICE3GB_ERR_NULL, "fields pointer is NULL");
  REQUIRE(f->sigqsat); REQUIRE(f->pabs); REQUIRE(f->sigs); REQUIRE(f->th); REQUIRE(f->exn);
  REQUIRE(f->exn_ref); REQUIRE(f->rho_dry_ref); REQUIRE(f->rv); REQUIRE(f->rc); REQUIRE(f->ri);
  REQUIRE(f->rr); REQUIRE(f->rs); REQUIRE(f->rg); REQUIRE(f->cf_mf); REQUIRE(f->rc_mf); REQUIRE(f->ri_mf);
  REQUIRE(f->rvs); REQUIRE(f->rcs); REQUIRE(f->ris); REQUIRE(f->ths);
  REQUIRE(f->t); REQUIRE(f->rv_out); REQUIRE(f->rc_out); REQUIRE(f->ri_out); REQUIRE(f->cldfr);
  REQUIRE(f->hlc_hrc); REQUIRE(f->hlc_hcf); REQUIRE(f->hli_hri); REQUIRE(f->hli_hcf);
  REQUIRE(f->cph); REQUIRE(f->lv); REQUIRE(f->ls);
  if (h->c.CONDENS != 0.0) return fail(h, ICE3GB_ERR_UNSUPPORTED, "CONDENS=%g (only CB02=0)", h->c.CONDENS);
  if (h->c.OCND2 != 0.0) {
    if (h->c.LSUBG_COND == 0.0)
      return fail(h, ICE3GB_ERR_UNSUPPORTED, "OCND2 needs LSUBG_COND (subgrid condensation)");
    if (nk < 2) return fail(h, ICE3GB_ERR_SHAPE, "OCND2 needs nk >= 2 (layer thickness), got %d", nk);
    REQUIRE(f->zz); REQUIRE(f->ice_cld_wgt);
  }
  return ICE3GB_OK;
}

bool ia_vec2_ok(const Ice3gbIceAdjustFields *f, long n)
{
  if (n % 2) return false;
  const void *ptrs[] = {f->pabs, f->sigs, f->th, f->exn, f->exn_ref, f->rho_dry_ref, f->rv, f->rc, f->ri, f->rr,
                        f->rs, f->rg, f->cf_mf, f->rc_mf, f->ri_mf, f->rvs, f->rcs, f->ris, f->ths, f->t,
                        f->rv_out, f->rc_out, f->ri_out, f->cldfr, f->hlc_hrc, f->hlc_hcf, f->hli_hri, f->hli_hcf,
                        f->cph, f->lv, f->ls};
  for (const void *p : ptrs)
    if (!aligned16(p)) return false;
  if (f->sigqsat_3d && !aligned16(f->sigqsat)) return false;
  if (f->srcs && !aligned16(f->srcs)) return false;
  return true;
}

int validate_sed(Handle *h, const Ice3gbSedimentationFields *f)
{
  if (!f) return fail(h, ICE3GB_ERR_NULL, "fields pointer is NULL");
  REQUIRE(f->rhodref); REQUIRE(f->dzz); REQUIRE(f->pabs); REQUIRE(f->tht);
  REQUIRE(f->rcs); REQUIRE(f->rrs); REQUIRE(f->ris); REQUIRE(f->rss); REQUIRE(f->rgs);
  REQUIRE(f->inprc); REQUIRE(f->inprr); REQUIRE(f->inpri); REQUIRE(f->inprs); REQUIRE(f->inprg);
  if ((f->sea == nullptr) != (f->town == nullptr))
    return fail(h, ICE3GB_ERR_NULL, "sea and town must be both given or both NULL");
  return ICE3GB_OK;
}

int validate_rain_ice(Handle *h, const Ice3gbRainIceFields *f)
{
  if (!f) return fail(h, ICE3GB_ERR_NULL, "fields pointer is NULL");
  REQUIRE(f->exn); REQUIRE(f->dzz); REQUIRE(f->rhodref); REQUIRE(f->exnref); REQUIRE(f->pabs);
  REQUIRE(f->cldfr); REQUIRE(f->sigs); REQUIRE(f->tht); REQUIRE(f->rvt); REQUIRE(f->rct); REQUIRE(f->rrt);
  REQUIRE(f->rit); REQUIRE(f->rst); REQUIRE(f->rgt); REQUIRE(f->cit);
  REQUIRE(f->ths); REQUIRE(f->rvs); REQUIRE(f->rcs); REQUIRE(f->rrs); REQUIRE(f->ris); REQUIRE(f->rss);
  REQUIRE(f->rgs); REQUIRE(f->evap3d); REQUIRE(f->rainfr);
  REQUIRE(f->inprc); REQUIRE(f->inprr); REQUIRE(f->inpri); REQUIRE(f->inprs); REQUIRE(f->inprg);
  if ((int)h->c.SUBG_AUCV_RC == 2 || (int)h->c.SUBG_AUCV_RI == 2) {
    REQUIRE(f->hlc_hrc); REQUIRE(f->hlc_hcf); REQUIRE(f->hli_hri); REQUIRE(f->hli_hcf);
  }
  if ((f->sea == nullptr) != (f->town == nullptr))
    return fail(h, ICE3GB_ERR_NULL, "sea and town must be both given or both NULL");
  if (!h->rain_ice_ok) return fail(h, ICE3GB_ERR_UNSUPPORTED, "%s", h->rain_ice_why.c_str());
  if ((int)h->c.NRR == 7) {  // hail
    REQUIRE(f->rht); REQUIRE(f->rhs); REQUIRE(f->inprh);
  }
  if (h->c.OCND2 != 0.0) {   // the ice_adjust OCND2 outputs of the same state
    REQUIRE(f->ssio); REQUIRE(f->ssiu); REQUIRE(f->ifr); REQUIRE(f->icldfr);
  }
  return ICE3GB_OK;
}

SedArgs sed_args(const Ice3gbSedimentationFields &f, int nij, int nk, double dt, int fortran)
{
  SedArgs a;
  a.rhodref = f.rhodref; a.dzz = f.dzz; a.pabs = f.pabs; a.tht = f.tht; a.sea = f.sea; a.town = f.town;
  a.src[0] = f.rcs; a.src[1] = f.rrs; a.src[2] = f.ris; a.src[3] = f.rss; a.src[4] = f.rgs;
  a.fpr[0] = f.fpr_c; a.fpr[1] = f.fpr_r; a.fpr[2] = f.fpr_i; a.fpr[3] = f.fpr_s; a.fpr[4] = f.fpr_g;
  a.inpr[0] = f.inprc; a.inpr[1] = f.inprr; a.inpr[2] = f.inpri; a.inpr[3] = f.inprs; a.inpr[4] = f.inprg;
  a.nij = nij; a.nk = nk; a.dt = dt; a.fortran = fortran;
  a.hsrc = a.hfpr = a.hinpr = nullptr;
  return a;
}

// Scratch of one rain_ice launch sequence (device words).
struct RiScratch {
  unsigned int *chunk;     // work counter, cleared here
  unsigned int *key_max;   // max pass key; cleared here unless shared across calls
  unsigned int *keys;      // [n] pass key per point
  unsigned int *order;     // [n] processing order, or NULL (index order)
  bool clear_key_max;      // false: the caller cleared it once for several calls
  bool evap_fixup;         // false: the caller runs the fix-up after the last call
  bool may_alloc = true;   // false: no stream-ordered allocation (SPLI sedimentation refused)
};

// The learned slow rates of a surrogate-assisted rain_ice call.
struct SurCall {
  void *mlp;
  const Ice3gbSurrogateNorm *norm;
  uint64_t *stats;   // host [ICE3GB_SUR_NSTATS] or NULL
};

int check_surrogate(Handle *h, const SurCall &sur, long n)
{
  int n_in = 0, n_out = 0;
  if (!mlp_dims(sur.mlp, &n_in, &n_out)) return fail(h, ICE3GB_ERR_HANDLE, "surrogate: not an MLP handle");
  if (n_in != ICE3GB_SUR_NFEAT || n_out != ICE3GB_SUR_NOUT)
    return fail(h, ICE3GB_ERR_SHAPE, "surrogate: the MLP maps %d -> %d, expected %d -> %d", n_in, n_out,
                ICE3GB_SUR_NFEAT, ICE3GB_SUR_NOUT);
  if (!sur.norm) return fail(h, ICE3GB_ERR_NULL, "surrogate: normalisation is NULL");
  if ((int)h->c.SUBG_RC_RR_ACCR != 0 || (int)h->c.SUBG_RR_EVAP != 0)
    return fail(h, ICE3GB_ERR_UNSUPPORTED, "surrogate: trained with SUBG_RC_RR_ACCR = SUBG_RR_EVAP = NONE only");
  if ((int)h->c.NRR != 6) return fail(h, ICE3GB_ERR_UNSUPPORTED, "surrogate: trained for NRR = 6 (no hail)");
  if (h->c.OCND2 != 0.0) return fail(h, ICE3GB_ERR_UNSUPPORTED, "surrogate: trained without OCND2");
  if (h->c.MRSTEP != 0.0 || h->c.TSTEP_TS != 0.0)
    return fail(h, ICE3GB_ERR_UNSUPPORTED, "surrogate: no MRSTEP / TSTEP_TS time splitting");
  if (n > 2147483647L) return fail(h, ICE3GB_ERR_RANGE, "surrogate: at most 2^31 - 1 points per call");
  return ICE3GB_OK;
}

// Features -> network -> rain_ice with the learned slow rates.  Synchronises
// the stream once to size the network's batch and once at the end (device
// error flag of the tensor-core kernels, counters).
int run_surrogate_points(Handle *h, const Ice3gbConstants &c, const RainIceArgs &a, const SurCall &sur,
                         cudaStream_t s)
{
  const long n = (long)a.nij * a.nk;
  const size_t fb = ((sizeof(float) * 16 * (size_t)n + 255) / 256) * 256;
  const size_t yb = ((sizeof(float) * ICE3GB_SUR_NOUT * (size_t)n + 255) / 256) * 256;
  const size_t rb = ((sizeof(int) * (size_t)n + 255) / 256) * 256;
  char *scr = nullptr;
  cudaError_t e = cudaMallocAsync(&scr, fb + yb + rb + 256, s);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaMallocAsync");
  float *feat = reinterpret_cast<float *>(scr), *y = reinterpret_cast<float *>(scr + fb);
  int *row_of_point = reinterpret_cast<int *>(scr + fb + yb);
  unsigned long long *ctr = reinterpret_cast<unsigned long long *>(scr + fb + yb + rb);
  int rc = ICE3GB_OK;
  e = cudaMemsetAsync(ctr, 0, sizeof(unsigned long long) * (1 + ICE3GB_SUR_NSTATS), s);
  if (e == cudaSuccess) {
    SurSampleArgs sa;
    std::memset(&sa, 0, sizeof(sa));
    sa.f = a.f; sa.luts = a.luts; sa.nij = a.nij; sa.nk = a.nk; sa.dt = a.dt;
    sa.norm_on = 1; sa.norm = *sur.norm;
    sa.feat = feat; sa.row_of_point = row_of_point; sa.count = ctr; sa.stats = ctr + 1; sa.cap = n;
    ProfScope ps(h, K_SUR_SAMPLE, s);
    e = launch_surrogate_sample(c, sa, h->num_sms, s);
  }
  unsigned long long rows = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&rows, ctr, sizeof(rows), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) rc = cuda_fail(h, e, "surrogate sampling");
  if (rc == ICE3GB_OK && rows > 0) {
    ProfScope ps(h, K_SUR_MLP, s);
    e = mlp_infer(sur.mlp, (long)(rows < (unsigned long long)n ? rows : n), feat, y, s);
    if (e != cudaSuccess) rc = cuda_fail(h, e, "surrogate network");
  }
  if (rc == ICE3GB_OK) {
    SurRainIceArgs ra;
    ra.ri = a; ra.y = y; ra.ldy = ICE3GB_SUR_NOUT; ra.row_of_point = row_of_point; ra.stats = ctr + 1;
    ProfScope ps(h, K_SUR_RAIN_ICE, s);
    e = launch_rain_ice_surrogate(c, ra, h->num_sms, s);
    if (e != cudaSuccess) rc = cuda_fail(h, e, "rain_ice surrogate launch");
  }
  unsigned long long st[ICE3GB_SUR_NSTATS] = {};
  if (rc == ICE3GB_OK) {
    e = cudaMemcpyAsync(st, ctr + 1, sizeof(st), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = cuda_fail(h, e, "surrogate counters");
  }
  if (rc == ICE3GB_OK && mlp_device_error(sur.mlp))
    rc = fail(h, ICE3GB_ERR_DEVICE, "surrogate network: a tensor-core barrier timed out");
  if (rc == ICE3GB_OK && sur.stats)
    for (int i = 0; i < ICE3GB_SUR_NSTATS; ++i) sur.stats[i] = st[i];
  cudaFreeAsync(scr, s);
  return rc;
}

// Launch sequence of one rain_ice call (sur: with the learned slow rates).
int run_rain_ice_core(Handle *h, int nij, int nk, double dt, const Ice3gbRainIceOptions *opt,
                      const Ice3gbRainIceFields *f, const RiScratch &rs, cudaStream_t s,
                      const SurCall *sur = nullptr)
{
  const int lsedim_after = (opt && opt->lsedim_after >= 0) ? opt->lsedim_after : (h->c.LSEDIM_AFTER != 0.0);
  const int ldeposc = (opt && opt->ldeposc >= 0) ? opt->ldeposc : (h->c.LDEPOSC != 0.0);
  const int max_passes = (opt && opt->max_passes > 0) ? opt->max_passes : 256;
  if (max_passes > 65535) return fail(h, ICE3GB_ERR_RANGE, "max_passes=%d above 65535", max_passes);
  const int sed_fortran = !(opt && opt->sed_jax > 0);
  Ice3gbConstants c = h->c;
  if (opt && opt->lfeedbackt >= 0) c.LFEEDBACKT = opt->lfeedbackt ? 1.0 : 0.0;
  Ice3gbSedimentationFields sf;
  std::memset(&sf, 0, sizeof(sf));
  sf.rhodref = f->rhodref; sf.dzz = f->dzz; sf.pabs = f->pabs; sf.tht = f->tht; sf.sea = f->sea; sf.town = f->town;
  sf.rcs = f->rcs; sf.rrs = f->rrs; sf.ris = f->ris; sf.rss = f->rss; sf.rgs = f->rgs;
  sf.inprc = f->inprc; sf.inprr = f->inprr; sf.inpri = f->inpri; sf.inprs = f->inprs; sf.inprg = f->inprg;
  sf.fpr_c = f->fpr_c; sf.fpr_r = f->fpr_r; sf.fpr_i = f->fpr_i; sf.fpr_s = f->fpr_s; sf.fpr_g = f->fpr_g;
  SedArgs sa = sed_args(sf, nij, nk, dt, sed_fortran);
  const bool hail = (int)h->c.NRR == 7;
  if (hail) {
    if (!sed_fortran) return fail(h, ICE3GB_ERR_UNSUPPORTED, "hail (NRR = 7) with the Fortran sedimentation only");
    sa.hsrc = f->rhs;
    sa.hfpr = f->fpr_h;
    sa.hinpr = f->inprh;
  }
  cudaError_t e;
  // SEDIM: 1 = STAT (statistical), 0 = SPLI (time-split, needs 2 n doubles of scratch)
  const bool spli = (int)c.SEDIM == 0;
  const bool ocnd2 = c.OCND2 != 0.0;
  // both refusals come before the first launch: a refused call leaves every field untouched
  if (spli && !rs.may_alloc)
    return fail(h, ICE3GB_ERR_UNSUPPORTED, "SEDIM=SPLI needs scratch memory: not available in this entry point");
  if (ocnd2 && !rs.may_alloc)
    return fail(h, ICE3GB_ERR_UNSUPPORTED, "OCND2 needs scratch memory: not available in this entry point");
  auto sediment = [&]() -> int {
    ProfScope ps(h, K_SEDIM, s);
    if (!spli) {
      cudaError_t e2 = launch_sedimentation(c, sa, s);
      return e2 == cudaSuccess ? ICE3GB_OK : cuda_fail(h, e2, "sedimentation launch");
    }
    SplitArgs sp;
    sp.sed = sa;
    sp.rt[0] = f->rct; sp.rt[1] = f->rrt; sp.rt[2] = f->rit; sp.rt[3] = f->rst; sp.rt[4] = f->rgt;
    sp.rvt = f->rvt; sp.exn = f->exn; sp.rvs = f->rvs; sp.ths = f->ths;
    sp.rht = hail ? f->rht : nullptr;
    sp.status = h->d_status;
    sp.max_iter = 10000;
    double *scr = nullptr;
    cudaError_t e2 = cudaMallocAsync(&scr, sizeof(double) * 2 * (size_t)nij * nk, s);
    if (e2 != cudaSuccess) return cuda_fail(h, e2, "cudaMallocAsync");
    sp.scratch = scr;
    e2 = launch_sedimentation_split(c, sp, s);
    cudaFreeAsync(scr, s);
    return e2 == cudaSuccess ? ICE3GB_OK : cuda_fail(h, e2, "sedimentation (SPLI) launch");
  };
  if (!lsedim_after) {
    const int rc = sediment();
    if (rc != ICE3GB_OK) return rc;
  }
  if ((e = cudaMemsetAsync(rs.chunk, 0, sizeof(unsigned int), s)) != cudaSuccess ||
      (rs.clear_key_max && (e = cudaMemsetAsync(rs.key_max, 0, sizeof(unsigned int), s)) != cudaSuccess))
    return cuda_fail(h, e, "cudaMemsetAsync");
  RainIceArgs a;
  a.f = *f;
  a.luts = h->d_luts;
  a.scr.status = h->d_status;
  a.scr.chunk_counter = rs.chunk;
  a.scr.key_max = rs.key_max;
  a.scr.keys = rs.keys;
  a.order = rs.order;
  a.nij = nij; a.nk = nk; a.dt = dt; a.max_passes = max_passes; a.lfeedbackt = (int)c.LFEEDBACKT;
  a.tw = nullptr;
  a.ocs = nullptr;
  if (ocnd2) {
    // level heights and droplet concentrations of the OCND2 processes (2 n doubles)
    if ((e = cudaMallocAsync(&a.ocs, sizeof(double) * 2 * (size_t)nij * nk, s)) != cudaSuccess)
      return cuda_fail(h, e, "cudaMallocAsync");
    a.tw = h->d_tiwmx;
    if ((e = launch_rain_ice_ocnd2_columns(c, a, s)) != cudaSuccess) {
      cudaFreeAsync(a.ocs, s);
      return cuda_fail(h, e, "rain_ice OCND2 columns");
    }
  }
  struct OcsFree {   // the OCND2 scratch goes back to the pool on every return below
    double *p;
    cudaStream_t s;
    ~OcsFree() { if (p) cudaFreeAsync(p, s); }
  } ocs_free{a.ocs, s};
  if ((int)c.SUBG_RC_RR_ACCR == 1 || (int)c.SUBG_RR_EVAP == 2) {
    ProfScope ps(h, K_PRFR, s);
    if ((e = launch_rain_ice_prfr(c, a, s)) != cudaSuccess) return cuda_fail(h, e, "rain_ice precipitation fraction");
  }
  if (rs.order) {
    ProfScope ps(h, K_ORDER, s);
    if ((e = launch_rain_ice_order(c, a, s)) != cudaSuccess) return cuda_fail(h, e, "rain_ice order launch");
  }
  if (sur) {
    const int rc = run_surrogate_points(h, c, a, *sur, s);
    if (rc != ICE3GB_OK) return rc;
    e = cudaSuccess;
  } else {
    ProfScope ps(h, K_RAIN_ICE, s);
    e = launch_rain_ice_points(c, a, h->num_sms, s);
  }
  if (e == cudaSuccess && rs.evap_fixup) {
    ProfScope ps(h, K_EVAP_FIXUP, s);
    e = launch_rain_ice_evap_fixup(a, s);
  }
  if (e != cudaSuccess) return cuda_fail(h, e, "rain_ice launch");
  if (lsedim_after) {
    const int rc = sediment();
    if (rc != ICE3GB_OK) return rc;
  }
  if (ldeposc || f->indep) {
    ProfScope ps(h, K_FOG, s);
    FogArgs fa;
    fa.rct = f->rct; fa.rhodref = f->rhodref; fa.dzz = f->dzz; fa.rcs = f->rcs; fa.inprc = f->inprc;
    fa.indep = f->indep; fa.nij = nij; fa.enabled = ldeposc;
    if ((e = launch_fog_deposition(c, fa, s)) != cudaSuccess) return cuda_fail(h, e, "fog launch");
  }
  return ICE3GB_OK;
}

// rain_ice with per-call scratch from the stream-ordered allocator: control
// words, pass keys and (below 2^32 points) the processing order.
int run_rain_ice(Handle *h, int nij, int nk, double dt, const Ice3gbRainIceOptions *opt,
                 const Ice3gbRainIceFields *f, cudaStream_t s, const SurCall *sur = nullptr)
{
  const long n = (long)nij * nk;
  const bool ordered = n < 4294967296L;
  unsigned int *scr = nullptr;
  const size_t bytes = sizeof(unsigned int) * (4 + (size_t)n * (ordered ? 2 : 1));
  cudaError_t e = cudaMallocAsync(&scr, bytes, s);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaMallocAsync");
  const RiScratch rs = {scr, scr + 1, scr + 4, ordered ? scr + 4 + n : nullptr, true, true};
  const int rc = run_rain_ice_core(h, nij, nk, dt, opt, f, rs, s, sur);
  cudaFreeAsync(scr, s);
  return rc;
}

int validate_step(Handle *h, const Ice3gbStepFields *f)
{
  if (!f) return fail(h, ICE3GB_ERR_NULL, "fields pointer is NULL");
  REQUIRE(f->sigqsat); REQUIRE(f->pabs); REQUIRE(f->exn); REQUIRE(f->exnref); REQUIRE(f->rhodref);
  REQUIRE(f->dzz); REQUIRE(f->sigs); REQUIRE(f->th); REQUIRE(f->rv); REQUIRE(f->rc); REQUIRE(f->ri);
  REQUIRE(f->rr); REQUIRE(f->rs); REQUIRE(f->rg); REQUIRE(f->cf_mf); REQUIRE(f->rc_mf); REQUIRE(f->ri_mf);
  REQUIRE(f->ths); REQUIRE(f->rvs); REQUIRE(f->rcs); REQUIRE(f->rrs); REQUIRE(f->ris); REQUIRE(f->rss);
  REQUIRE(f->rgs); REQUIRE(f->cit); REQUIRE(f->t); REQUIRE(f->rv_out); REQUIRE(f->rc_out); REQUIRE(f->ri_out);
  REQUIRE(f->cldfr); REQUIRE(f->hlc_hrc); REQUIRE(f->hlc_hcf); REQUIRE(f->hli_hri); REQUIRE(f->hli_hcf);
  REQUIRE(f->evap3d); REQUIRE(f->rainfr); REQUIRE(f->inprc); REQUIRE(f->inprr); REQUIRE(f->inpri);
  REQUIRE(f->inprs); REQUIRE(f->inprg);
  if ((f->sea == nullptr) != (f->town == nullptr))
    return fail(h, ICE3GB_ERR_NULL, "sea and town must be both given or both NULL");
  if (h->c.CONDENS != 0.0 || h->c.OCND2 != 0.0)
    return fail(h, ICE3GB_ERR_UNSUPPORTED, "ice_adjust: only CONDENS=CB02 without OCND2");
  if (!h->rain_ice_ok) return fail(h, ICE3GB_ERR_UNSUPPORTED, "%s", h->rain_ice_why.c_str());
  if ((int)h->c.NRR != 6)
    return fail(h, ICE3GB_ERR_UNSUPPORTED, "physics step: NRR = 6 only (the step fields carry no hail)");
  return ICE3GB_OK;
}

int run_physics_step(Handle *h, int nij, int nk, double dt, const Ice3gbRainIceOptions *opt,
                     const Ice3gbStepFields *f, cudaStream_t s, const RiScratch *ri_scr = nullptr,
                     const SurCall *sur = nullptr)
{
  const long n = (long)nij * nk;
  double *scr = nullptr;
  cudaError_t e = cudaMallocAsync(&scr, sizeof(double) * 5 * (size_t)n, s);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaMallocAsync");
  double *cldfr1 = scr, *hlc_hrc1 = scr + n, *hlc_hcf1 = scr + 2 * n, *hli_hri1 = scr + 3 * n,
         *hli_hcf1 = scr + 4 * n;
  // 1. first adjustment: S0 -> S1, cloud fraction and subgrid partition to scratch
  IaKernelFields k1;
  std::memset(&k1, 0, sizeof(k1));
  Ice3gbIceAdjustFields &a = k1.f;
  a.sigqsat = f->sigqsat; a.pabs = f->pabs; a.sigs = f->sigs; a.th = f->th; a.exn = f->exn;
  a.exn_ref = f->exnref; a.rho_dry_ref = f->rhodref; a.rv = f->rv; a.rc = f->rc; a.ri = f->ri; a.rr = f->rr;
  a.rs = f->rs; a.rg = f->rg; a.cf_mf = f->cf_mf; a.rc_mf = f->rc_mf; a.ri_mf = f->ri_mf;
  a.rvs = f->rvs; a.rcs = f->rcs; a.ris = f->ris; a.ths = f->ths;
  a.cldfr = cldfr1; a.hlc_hrc = hlc_hrc1; a.hlc_hcf = hlc_hcf1; a.hli_hri = hli_hri1; a.hli_hcf = hli_hcf1;
  a.sigqsat_3d = 0;
  int rc = ICE3GB_OK;
  {
    ProfScope ps(h, K_ICE_ADJUST, s);
    e = launch_ice_adjust(h->c, k1, nij, nk, dt, ia_vec2_ok(&a, n), h->num_sms, s);
  }
  if (e != cudaSuccess) rc = cuda_fail(h, e, "ice_adjust launch");
  // 2. rain_ice on the time-t state with S1
  if (rc == ICE3GB_OK) {
    Ice3gbRainIceFields r;
    std::memset(&r, 0, sizeof(r));
    r.exn = f->exn; r.dzz = f->dzz; r.rhodref = f->rhodref; r.exnref = f->exnref; r.pabs = f->pabs;
    r.cldfr = cldfr1; r.sigs = f->sigs; r.tht = f->th; r.rvt = f->rv; r.rct = f->rc; r.rrt = f->rr;
    r.rit = f->ri; r.rst = f->rs; r.rgt = f->rg; r.sea = f->sea; r.town = f->town; r.cit = f->cit;
    r.hlc_hrc = hlc_hrc1; r.hlc_hcf = hlc_hcf1; r.hli_hri = hli_hri1; r.hli_hcf = hli_hcf1;
    r.ths = f->ths; r.rvs = f->rvs; r.rcs = f->rcs; r.rrs = f->rrs; r.ris = f->ris; r.rss = f->rss;
    r.rgs = f->rgs; r.evap3d = f->evap3d; r.rainfr = f->rainfr; r.inprc = f->inprc; r.inprr = f->inprr;
    r.inpri = f->inpri; r.inprs = f->inprs; r.inprg = f->inprg;
    rc = ri_scr ? run_rain_ice_core(h, nij, nk, dt, opt, &r, *ri_scr, s, sur)
                : run_rain_ice(h, nij, nk, dt, opt, &r, s, sur);
  }
  // 3. final adjustment on the post-microphysics state dt*S2 with S2 -> S3
  if (rc == ICE3GB_OK) {
    IaKernelFields k2 = k1;
    Ice3gbIceAdjustFields &b = k2.f;
    b.t = f->t; b.rv_out = f->rv_out; b.rc_out = f->rc_out; b.ri_out = f->ri_out; b.cldfr = f->cldfr;
    b.hlc_hrc = f->hlc_hrc; b.hlc_hcf = f->hlc_hcf; b.hli_hri = f->hli_hri; b.hli_hcf = f->hli_hcf;
    k2.rrs = f->rrs; k2.rss = f->rss; k2.rgs = f->rgs;
    k2.adv_dt = dt;
    const bool v2 = ia_vec2_ok(&b, n) && aligned16(f->rrs) && aligned16(f->rss) && aligned16(f->rgs);
    ProfScope ps(h, K_ICE_ADJUST, s);
    e = launch_ice_adjust(h->c, k2, nij, nk, dt, v2, h->num_sms, s);
    if (e != cudaSuccess) rc = cuda_fail(h, e, "ice_adjust launch");
  }
  cudaFreeAsync(scr, s);
  return rc;
}

// ---- host staging -----------------------------------------------------------
int ensure_stage(Handle *h, size_t bytes)
{
  if (h->stage_cap >= bytes) return ICE3GB_OK;
  if (h->d_stage) cudaFree(h->d_stage);
  h->d_stage = nullptr;
  h->stage_cap = 0;
  cudaError_t e = cudaMalloc(&h->d_stage, bytes);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaMalloc(staging)");
  h->stage_cap = bytes;
  return ICE3GB_OK;
}


// ---- slab pipeline of the chained step on host buffers -----------------------
// Columns are independent, so ice3gb_physics_step_host runs the step on
// column slabs: pitched copies of slab i+1 in (host [nk][nij] -> compact
// device [nk][w]) and of slab i-1 out overlap the kernels of slab i; the
// slabs alternate between two compute streams, so that the kernels of two
// slabs overlap as well (streams ordered by events).  evap3d keeps PRREVAV
// only at points active in the last pass of the whole call, so the slabs
// share one maximum-pass-key word and write evap3d and the pass keys to
// full-size arrays; one fix-up after the last slab and a final copy-out of
// evap3d give the same result as ice3gb_physics_step on the whole grid.
int pipe_init(Handle *h)
{
  HostPipe &P = h->pipe;
  if (P.ready) return ICE3GB_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&P.s_in, cudaStreamNonBlocking);
  for (int k = 0; k < HostPipe::NC && e == cudaSuccess; ++k) {
    e = cudaStreamCreateWithFlags(&P.s_cmp[k], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P.cmp_end[k], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&P.s_out, cudaStreamNonBlocking);
  for (int b = 0; b < HostPipe::NB && e == cudaSuccess; ++b) {
    e = cudaEventCreateWithFlags(&P.in_done[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P.cmp_done[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P.out_done[b], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P.start, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P.fix_done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P.cleared, cudaEventDisableTiming);
  if (e != cudaSuccess) return cuda_fail(h, e, "slab pipeline streams/events");
  P.ready = true;
  return ICE3GB_OK;
}

void pipe_free(Handle *h)
{
  HostPipe &P = h->pipe;
  if (!P.ready) return;
  cudaStreamSynchronize(P.s_in);
  for (int k = 0; k < HostPipe::NC; ++k) cudaStreamSynchronize(P.s_cmp[k]);
  cudaStreamSynchronize(P.s_out);
  for (int b = 0; b < HostPipe::NB; ++b) {
    cudaEventDestroy(P.in_done[b]);
    cudaEventDestroy(P.cmp_done[b]);
    cudaEventDestroy(P.out_done[b]);
    if (P.buf[b]) cudaFree(P.buf[b]);
  }
  cudaEventDestroy(P.start);
  cudaEventDestroy(P.fix_done);
  cudaEventDestroy(P.cleared);
  for (int k = 0; k < HostPipe::NC; ++k) {
    cudaEventDestroy(P.cmp_end[k]);
    cudaStreamDestroy(P.s_cmp[k]);
  }
  cudaStreamDestroy(P.s_in);
  cudaStreamDestroy(P.s_out);
  if (P.evap_all) cudaFree(P.evap_all);
  if (P.keys_all) cudaFree(P.keys_all);
  P = HostPipe();
}

// Column boundaries of the slabs: slabs of w_max columns, the first and the
// last ones graded (w_max / 4, w_max / 4, w_max / 2 at each end, multiples of
// 64 columns) when the grid holds at least 6 of them, because the first
// slab's copy-in and the last slab's copy-out overlap no kernel.
std::vector<long> slab_cuts(long nij, long w_max)
{
  std::vector<long> widths;
  const long q = (w_max / 4 + 63) / 64 * 64, hlf = (w_max / 2 + 63) / 64 * 64;
  long left = nij;
  const bool graded = nij >= 6 * w_max && q >= 64;
  if (graded) {
    for (long w : {q, q, hlf}) { widths.push_back(w); left -= w; }
    left -= 2 * q + hlf;                             // the trailing ones
  }
  while (left > 0) {
    const long w = left < w_max ? left : w_max;
    widths.push_back(w);
    left -= w;
  }
  if (graded)
    for (long w : {hlf, q, q}) widths.push_back(w);
  std::vector<long> cuts(1, 0);
  for (long w : widths) cuts.push_back(cuts.back() + w);
  return cuts;
}

#ifndef ICE3GB_HOST_SLABS
#define ICE3GB_HOST_SLABS 8
#endif

int run_physics_step_pipelined(Handle *h, int nij, int nk, double dt, const Ice3gbRainIceOptions *opt,
                               const Ice3gbStepFields *f, cudaStream_t s)
{
  int rc;
  if ((rc = pipe_init(h))) return rc;
  HostPipe &P = h->pipe;
  // slab width: about ICE3GB_HOST_SLABS slabs, at least 4096 columns, a multiple of 64
  long w_max = ((long)nij / ICE3GB_HOST_SLABS + 63) / 64 * 64;
  if (w_max < 4096) w_max = 4096;
  if (w_max > nij) w_max = nij;
  const long n_all = (long)nij * nk;
  const size_t b3 = (size_t)w_max * nk * sizeof(double), b2 = (size_t)w_max * sizeof(double);
  const size_t b3p = (b3 + 255) & ~(size_t)255, b2p = (b2 + 255) & ~(size_t)255;
  const size_t bo = ((size_t)w_max * nk * sizeof(unsigned int) + 255) & ~(size_t)255;
  // per set: 16 inputs + 8 in-out + 10 outputs (evap3d goes to evap_all) 3-D; sigqsat, sea, town + 5 2-D;
  // the processing order of rain_ice
  const size_t set_bytes = 34 * b3p + 8 * b2p + bo;
  cudaError_t e = cudaSuccess;
  if (P.buf_cap < set_bytes) {
    for (int b = 0; b < HostPipe::NB; ++b) {
      if (P.buf[b]) cudaFree(P.buf[b]);
      P.buf[b] = nullptr;
    }
    P.buf_cap = 0;
    for (int b = 0; b < HostPipe::NB && e == cudaSuccess; ++b) e = cudaMalloc(&P.buf[b], set_bytes);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaMalloc(slab buffers)");
    P.buf_cap = set_bytes;
  }
  if (P.all_cap < (size_t)n_all) {
    if (P.evap_all) cudaFree(P.evap_all);
    if (P.keys_all) cudaFree(P.keys_all);
    P.evap_all = nullptr;
    P.keys_all = nullptr;
    P.all_cap = 0;
    e = cudaMalloc(&P.evap_all, sizeof(double) * (size_t)n_all);
    if (e == cudaSuccess) e = cudaMalloc(&P.keys_all, sizeof(unsigned int) * (4 + (size_t)n_all));
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaMalloc(evap3d/keys)");
    P.all_cap = (size_t)n_all;
  }
  // order after the caller's earlier work on its stream; clear the control
  // words (work counters of the two compute streams at 0 and 2, the shared
  // key_max at 1) before either compute stream starts
  if ((e = cudaEventRecord(P.start, s)) != cudaSuccess || (e = cudaStreamWaitEvent(P.s_in, P.start, 0)) != cudaSuccess ||
      (e = cudaStreamWaitEvent(P.s_cmp[0], P.start, 0)) != cudaSuccess ||
      (e = cudaMemsetAsync(P.keys_all, 0, 4 * sizeof(unsigned int), P.s_cmp[0])) != cudaSuccess ||
      (e = cudaEventRecord(P.cleared, P.s_cmp[0])) != cudaSuccess ||
      (e = cudaStreamWaitEvent(P.s_cmp[1], P.cleared, 0)) != cudaSuccess)
    return cuda_fail(h, e, "slab pipeline start");
  const size_t hp = (size_t)nij * sizeof(double);   // host row pitch of 3-D fields
  const std::vector<long> cuts = slab_cuts(nij, w_max);
  const long nslab = (long)cuts.size() - 1;
  long pt_off = 0;                                   // offset of the slab in evap_all / keys
  for (long i = 0; i < nslab && rc == ICE3GB_OK; ++i) {
    const int b = (int)(i % HostPipe::NB);
    const long col0 = cuts[i];
    const long w = cuts[i + 1] - cuts[i];
    const size_t wb = (size_t)w * sizeof(double);
    char *base = P.buf[b];
    size_t off = 0;
    auto take = [&](size_t bp) { double *p = reinterpret_cast<double *>(base + off); off += bp; return p; };
    // ---- copy in
    if (i >= HostPipe::NB && (e = cudaStreamWaitEvent(P.s_in, P.out_done[b], 0)) != cudaSuccess) break;
    auto up3 = [&](const double *src) -> double * {
      double *p = take(b3p);
      if (src && e == cudaSuccess)
        e = cudaMemcpy2DAsync(p, wb, src + col0, hp, wb, (size_t)nk, cudaMemcpyHostToDevice, P.s_in);
      return src ? p : nullptr;
    };
    auto up2 = [&](const double *src) -> double * {
      double *p = take(b2p);
      if (src && e == cudaSuccess) e = cudaMemcpyAsync(p, src + col0, wb, cudaMemcpyHostToDevice, P.s_in);
      return src ? p : nullptr;
    };
    Ice3gbStepFields d;
    std::memset(&d, 0, sizeof(d));
    d.sigqsat = up2(f->sigqsat);
    d.pabs = up3(f->pabs); d.exn = up3(f->exn); d.exnref = up3(f->exnref); d.rhodref = up3(f->rhodref);
    d.dzz = up3(f->dzz); d.sigs = up3(f->sigs); d.th = up3(f->th); d.rv = up3(f->rv); d.rc = up3(f->rc);
    d.ri = up3(f->ri); d.rr = up3(f->rr); d.rs = up3(f->rs); d.rg = up3(f->rg);
    d.cf_mf = up3(f->cf_mf); d.rc_mf = up3(f->rc_mf); d.ri_mf = up3(f->ri_mf);
    d.sea = up2(f->sea); d.town = up2(f->town);
    d.ths = up3(f->ths); d.rvs = up3(f->rvs); d.rcs = up3(f->rcs); d.rrs = up3(f->rrs); d.ris = up3(f->ris);
    d.rss = up3(f->rss); d.rgs = up3(f->rgs); d.cit = up3(f->cit);
    d.t = take(b3p); d.rv_out = take(b3p); d.rc_out = take(b3p); d.ri_out = take(b3p); d.cldfr = take(b3p);
    d.hlc_hrc = take(b3p); d.hlc_hcf = take(b3p); d.hli_hri = take(b3p); d.hli_hcf = take(b3p);
    d.rainfr = take(b3p);
    d.inprc = take(b2p); d.inprr = take(b2p); d.inpri = take(b2p); d.inprs = take(b2p); d.inprg = take(b2p);
    unsigned int *order = reinterpret_cast<unsigned int *>(base + off);
    d.evap3d = P.evap_all + pt_off;
    if (e == cudaSuccess) e = cudaEventRecord(P.in_done[b], P.s_in);
    if (e != cudaSuccess) break;
    // ---- compute on the slab's compute stream, with that stream's work
    // counter (the fix-up of evap3d waits for both streams)
    const int k = (int)(i % HostPipe::NC);
    cudaStream_t sc = P.s_cmp[k];
    if ((e = cudaStreamWaitEvent(sc, P.in_done[b], 0)) != cudaSuccess) break;
    const RiScratch rs = {P.keys_all + 2 * k, P.keys_all + 1, P.keys_all + 4 + pt_off, order, false, false};
    if ((rc = run_physics_step(h, (int)w, nk, dt, opt, &d, sc, &rs))) break;
    if ((e = cudaEventRecord(P.cmp_done[b], sc)) != cudaSuccess) break;
    // ---- copy out (everything but evap3d)
    if ((e = cudaStreamWaitEvent(P.s_out, P.cmp_done[b], 0)) != cudaSuccess) break;
    struct Out { double *dst; const double *src; bool three_d; };
    const Out outs[] = {
        {f->ths, d.ths, true}, {f->rvs, d.rvs, true}, {f->rcs, d.rcs, true}, {f->rrs, d.rrs, true},
        {f->ris, d.ris, true}, {f->rss, d.rss, true}, {f->rgs, d.rgs, true}, {f->cit, d.cit, true},
        {f->t, d.t, true}, {f->rv_out, d.rv_out, true}, {f->rc_out, d.rc_out, true}, {f->ri_out, d.ri_out, true},
        {f->cldfr, d.cldfr, true}, {f->hlc_hrc, d.hlc_hrc, true}, {f->hlc_hcf, d.hlc_hcf, true},
        {f->hli_hri, d.hli_hri, true}, {f->hli_hcf, d.hli_hcf, true}, {f->rainfr, d.rainfr, true},
        {f->inprc, d.inprc, false}, {f->inprr, d.inprr, false}, {f->inpri, d.inpri, false},
        {f->inprs, d.inprs, false}, {f->inprg, d.inprg, false}};
    for (const Out &o : outs) {
      if (e != cudaSuccess) break;
      e = o.three_d ? cudaMemcpy2DAsync(o.dst + col0, hp, o.src, wb, wb, (size_t)nk, cudaMemcpyDeviceToHost, P.s_out)
                    : cudaMemcpyAsync(o.dst + col0, o.src, wb, cudaMemcpyDeviceToHost, P.s_out);
    }
    if (e == cudaSuccess) e = cudaEventRecord(P.out_done[b], P.s_out);
    if (e != cudaSuccess) break;
    pt_off += w * nk;
  }
  if (rc == ICE3GB_OK && e == cudaSuccess) {
    // evap3d: zero it where the point was not active in the last pass of the call
    RainIceArgs a;
    std::memset(&a, 0, sizeof(a));
    a.f.evap3d = P.evap_all;
    a.scr.keys = P.keys_all + 4;
    a.scr.key_max = P.keys_all + 1;
    a.nij = nij;
    a.nk = nk;
    if ((e = cudaEventRecord(P.cmp_end[1], P.s_cmp[1])) == cudaSuccess)
      e = cudaStreamWaitEvent(P.s_cmp[0], P.cmp_end[1], 0);
    if (e == cudaSuccess) {
      ProfScope ps(h, K_EVAP_FIXUP, P.s_cmp[0]);
      e = launch_rain_ice_evap_fixup(a, P.s_cmp[0]);
    }
    if (e == cudaSuccess) e = cudaEventRecord(P.fix_done, P.s_cmp[0]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(P.s_out, P.fix_done, 0);
    long off_pts = 0;
    for (long i = 0; i < nslab && e == cudaSuccess; ++i) {
      const long col0 = cuts[i];
      const long w = cuts[i + 1] - cuts[i];
      const size_t wb = (size_t)w * sizeof(double);
      e = cudaMemcpy2DAsync(f->evap3d + col0, hp, P.evap_all + off_pts, wb, wb, (size_t)nk, cudaMemcpyDeviceToHost,
                            P.s_out);
      off_pts += w * nk;
    }
  }
  // drain all streams before returning (the call is synchronous)
  const cudaError_t e1 = cudaStreamSynchronize(P.s_in);
  cudaError_t e2 = cudaStreamSynchronize(P.s_cmp[0]);
  const cudaError_t e2b = cudaStreamSynchronize(P.s_cmp[1]);
  if (e2 == cudaSuccess) e2 = e2b;
  const cudaError_t e3 = cudaStreamSynchronize(P.s_out);
  if (rc != ICE3GB_OK) return rc;
  if (e == cudaSuccess) e = e1 != cudaSuccess ? e1 : e2 != cudaSuccess ? e2 : e3;
  if (e != cudaSuccess) return cuda_fail(h, e, "slab pipeline");
  return ICE3GB_OK;
}

}  // namespace

// Validation + launch sequence with caller-provided scratch (used by the
// entry point of rain_ice_noalloc.cu, which owns its static scratch: four
// control words, then scratch_points pass keys, then scratch_points order
// words).
int ice3gb_internal_rain_ice_with_scratch(void *handle, int nij, int nk, double dt,
                                          const Ice3gbRainIceOptions *opt, const Ice3gbRainIceFields *f,
                                          unsigned int *scratch, long scratch_points, void *stream)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "invalid handle");
  int rc;
  if ((rc = check_shape(h, nij, nk))) return rc;
  if ((long)nij * nk > scratch_points)
    return fail(h, ICE3GB_ERR_RANGE, "nij*nk = %ld grid points exceeds the %ld-point static scratch",
                (long)nij * nk, scratch_points);
  if ((rc = validate_rain_ice(h, f)) || (rc = check_device(h))) return rc;
  if (!scratch) return fail(h, ICE3GB_ERR_CUDA, "static scratch address unavailable");
  // control words [0, 4), pass keys [4, 4 + nij*nk), processing order from 4 + scratch_points
  const RiScratch rs = {scratch, scratch + 1, scratch + 4, scratch + 4 + scratch_points, true, true, false};
  return run_rain_ice_core(h, nij, nk, dt, opt, f, rs, static_cast<cudaStream_t>(stream));
}

// Records a CUDA error on the handle (or globally) for the other translation units.
int ice3gb_internal_cuda_fail(void *handle, cudaError_t e, const char *where)
{
  return cuda_fail(as_handle(handle), e, where);
}

extern "C" {

int ice3gb_version(void) { return ICE3GB_VERSION; }

static const char *kNames[] = {
#define ICE3GB_X_NAME(name) #name,
    ICE3GB_CONSTANTS(ICE3GB_X_NAME)
#undef ICE3GB_X_NAME
};

int ice3gb_constant_count(void) { return (int)(sizeof(kNames) / sizeof(kNames[0])); }

const char *ice3gb_constant_name(int i)
{
  if (i < 0 || i >= ice3gb_constant_count()) return nullptr;
  return kNames[i];
}

int ice3gb_create(const Ice3gbConstants *c, const Ice3gbLuts *luts, void **handle)
{
  if (!c || !luts || !handle) return fail(nullptr, ICE3GB_ERR_NULL, "ice3gb_create: NULL argument");
  *handle = nullptr;
  if ((int)c->NGAMINC != ICE3GB_NGAMINC || (int)c->NACCLBDAS != ICE3GB_NACCLBDAS ||
      (int)c->NACCLBDAR != ICE3GB_NACCLBDAR || (int)c->NDRYLBDAG != ICE3GB_NDRYLBDAG ||
      (int)c->NDRYLBDAS != ICE3GB_NDRYLBDAS || (int)c->NDRYLBDAR != ICE3GB_NDRYLBDAR ||
      (int)c->NWETLBDAH != ICE3GB_NWETLBDAH || (int)c->NWETLBDAS != ICE3GB_NWETLBDAS ||
      (int)c->NWETLBDAG != ICE3GB_NWETLBDAG || (int)c->NWETLBDAR != ICE3GB_NWETLBDAR)
    return fail(nullptr, ICE3GB_ERR_RANGE, "lookup-table sizes differ from the compiled ones");
  Handle *h = new Handle();
  h->magic = kMagic;
  h->c = *c;
  h->d_luts = nullptr;
  h->d_tiwmx = nullptr;
  h->d_status = nullptr;
  h->d_stage = nullptr;
  h->stage_cap = 0;
  h->err[0] = 0;
  h->profiling = false;
  cudaError_t e = cudaGetDevice(&h->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
  if (e == cudaSuccess) e = cudaMalloc(&h->d_luts, sizeof(Ice3gbLuts));
  if (e == cudaSuccess) e = cudaMemcpy(h->d_luts, luts, sizeof(Ice3gbLuts), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&h->d_status, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMemset(h->d_status, 0, sizeof(unsigned int));
  if (e == cudaSuccess && c->OCND2 != 0.0) {
    std::vector<double> tab((size_t)kTiwmxTables * kTiwmxTableN);
    tiwmx_tables(*c, tab.data());
    e = cudaMalloc(&h->d_tiwmx, sizeof(double) * tab.size());
    if (e == cudaSuccess)
      e = cudaMemcpy(h->d_tiwmx, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    int rc = cuda_fail(nullptr, e, "ice3gb_create");
    if (h->d_luts) cudaFree(h->d_luts);
    if (h->d_tiwmx) cudaFree(h->d_tiwmx);
    if (h->d_status) cudaFree(h->d_status);
    h->magic = 0;
    delete h;
    return rc;
  }
  h->rain_ice_ok = true;
  char why[256] = "";
  if ((int)c->NRR != 6 && (int)c->NRR != 7)
    snprintf(why, sizeof(why), "rain_ice supports NRR = 6 or 7 (hail), got %g", c->NRR);
  else if ((int)c->SEDIM != 0 && (int)c->SEDIM != 1)
    snprintf(why, sizeof(why), "rain_ice: SEDIM must be SPLI (0) or STAT (1), got %g", c->SEDIM);
  else if (((int)c->SUBG_RC_RR_ACCR != 0 && (int)c->SUBG_RC_RR_ACCR != 1) ||
           (int)c->SUBG_RR_EVAP < 0 || (int)c->SUBG_RR_EVAP > 2)
    snprintf(why, sizeof(why), "rain_ice: SUBG_RC_RR_ACCR must be NONE or PRFR, SUBG_RR_EVAP NONE, CLFR or PRFR");
  if (why[0]) {
    h->rain_ice_ok = false;
    h->rain_ice_why = why;
  }
  *handle = h;
  return ICE3GB_OK;
}

static void drop_events(Handle *h)
{
  std::lock_guard<std::mutex> lock(h->prof_mu);
  for (auto &ev : h->events) {
    cudaEventDestroy(ev.second.first);
    cudaEventDestroy(ev.second.second);
  }
  h->events.clear();
}

int ice3gb_profile_enable(void *handle, int enable)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_profile_enable: invalid handle");
  drop_events(h);
  h->profiling = enable != 0;
  return ICE3GB_OK;
}

int ice3gb_profile_read(void *handle, int kernel_id, int *launches, double *total_ms)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_profile_read: invalid handle");
  if (kernel_id < 0 || kernel_id >= K_COUNT) return fail(h, ICE3GB_ERR_RANGE, "kernel id %d", kernel_id);
  std::lock_guard<std::mutex> lock(h->prof_mu);
  int cnt = 0;
  double tot = 0.0;
  for (auto &ev : h->events) {
    if (ev.first != kernel_id) continue;
    float ms = 0.f;
    cudaError_t e = cudaEventSynchronize(ev.second.second);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev.second.first, ev.second.second);
    if (e != cudaSuccess) return cuda_fail(h, e, "ice3gb_profile_read");
    ++cnt;
    tot += ms;
  }
  if (launches) *launches = cnt;
  if (total_ms) *total_ms = tot;
  return ICE3GB_OK;
}

const char *ice3gb_kernel_name(int kernel_id)
{
  return (kernel_id >= 0 && kernel_id < K_COUNT) ? kKernelNames[kernel_id] : nullptr;
}

int ice3gb_destroy(void *handle)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_destroy: invalid handle");
  drop_events(h);
  pipe_free(h);
  cudaFree(h->d_luts);
  if (h->d_tiwmx) cudaFree(h->d_tiwmx);
  cudaFree(h->d_status);
  if (h->d_stage) cudaFree(h->d_stage);
  h->magic = 0;
  delete h;
  return ICE3GB_OK;
}

int ice3gb_last_error(void *handle, char *buf, size_t n)
{
  Handle *h = as_handle(handle);
  const char *src = h ? h->err : g_err;
  if (buf && n) snprintf(buf, n, "%s", src);
  return (int)strlen(src);
}

int ice3gb_status(void *handle, void *stream, uint32_t *bits)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_status: invalid handle");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned int v = 0;
  cudaError_t e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaMemcpy(&v, h->d_status, sizeof(v), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(h->d_status, 0, sizeof(unsigned int));
  if (e != cudaSuccess) return cuda_fail(h, e, "ice3gb_status");
  if (bits) *bits = v;
  if (v) return fail(h, ICE3GB_ERR_DEVICE, "device status 0x%x%s", v,
                     (v & ICE3GB_DEV_PASS_CAP) ? " (sub-step pass cap reached)" : "");
  return ICE3GB_OK;
}

int ice3gb_ice_adjust(void *handle, int nij, int nk, double dt, const Ice3gbIceAdjustFields *f, void *stream)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_ice_adjust: invalid handle");
  int rc;
  if ((rc = check_shape(h, nij, nk)) || (rc = validate_ice_adjust(h, f, nk)) || (rc = check_device(h))) return rc;
  const long n = (long)nij * nk;
  IaKernelFields kf;
  kf.f = *f;
  kf.rrs = kf.rss = kf.rgs = nullptr;
  kf.adv_dt = 0.0;
  kf.tiwmx = h->d_tiwmx;
  cudaError_t e;
  {
    ProfScope ps(h, K_ICE_ADJUST, static_cast<cudaStream_t>(stream));
    e = launch_ice_adjust(h->c, kf, nij, nk, dt, ia_vec2_ok(f, n), h->num_sms, static_cast<cudaStream_t>(stream));
  }
  if (e != cudaSuccess) return cuda_fail(h, e, "ice_adjust launch");
  return ICE3GB_OK;
}

int ice3gb_sedimentation(void *handle, int nij, int nk, double dt, const Ice3gbSedimentationFields *f,
                         void *stream)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_sedimentation: invalid handle");
  int rc;
  if ((rc = check_shape(h, nij, nk)) || (rc = validate_sed(h, f)) || (rc = check_device(h))) return rc;
  cudaError_t e;
  {
    ProfScope ps(h, K_SEDIM, static_cast<cudaStream_t>(stream));
    e = launch_sedimentation(h->c, sed_args(*f, nij, nk, dt, f->fortran_semantics != 0),
                             static_cast<cudaStream_t>(stream));
  }
  if (e != cudaSuccess) return cuda_fail(h, e, "sedimentation launch");
  return ICE3GB_OK;
}

int ice3gb_ice_adjust_vjp(void *handle, int nij, int nk, double dt, const Ice3gbIceAdjustFields *f,
                          const Ice3gbIceAdjustCotangents *g, const Ice3gbIceAdjustGradients *gx, void *stream)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_ice_adjust_vjp: invalid handle");
  int rc;
  if ((rc = check_shape(h, nij, nk))) return rc;
  if (!f || !g || !gx) return fail(h, ICE3GB_ERR_NULL, "fields, cotangents or gradients pointer is NULL");
  REQUIRE(f->sigqsat); REQUIRE(f->pabs); REQUIRE(f->sigs); REQUIRE(f->th); REQUIRE(f->exn);
  REQUIRE(f->exn_ref); REQUIRE(f->rho_dry_ref); REQUIRE(f->rv); REQUIRE(f->rc); REQUIRE(f->ri);
  REQUIRE(f->rr); REQUIRE(f->rs); REQUIRE(f->rg); REQUIRE(f->cf_mf); REQUIRE(f->rc_mf); REQUIRE(f->ri_mf);
  REQUIRE(f->rvs); REQUIRE(f->rcs); REQUIRE(f->ris); REQUIRE(f->ths);
  if (h->c.CONDENS != 0.0) return fail(h, ICE3GB_ERR_UNSUPPORTED, "CONDENS=%g (only CB02=0)", h->c.CONDENS);
  if (h->c.OCND2 != 0.0) return fail(h, ICE3GB_ERR_UNSUPPORTED, "OCND2 is not supported");
  if ((rc = check_device(h))) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long n = (long)nij * nk;
  IaVjpArgs a;
  a.f = *f;
  a.g = *g;
  a.gx = *gx;
  a.nij = nij;
  a.nk = nk;
  a.dt = dt;
  a.sigqsat_out = nullptr;
  double *scr = nullptr;
  cudaError_t e = cudaSuccess;
  if (gx->sigqsat) {
    if (f->sigqsat_3d) {
      a.sigqsat_out = gx->sigqsat;
    } else {
      if ((e = cudaMallocAsync(&scr, sizeof(double) * (size_t)n, s)) != cudaSuccess)
        return cuda_fail(h, e, "cudaMallocAsync");
      a.sigqsat_out = scr;
    }
  }
  {
    ProfScope ps(h, K_IA_VJP, s);
    e = launch_ice_adjust_vjp(h->c, a, h->num_sms, s);
  }
  if (e == cudaSuccess && scr) e = launch_column_sum(scr, gx->sigqsat, nij, nk, s);
  if (scr) cudaFreeAsync(scr, s);
  if (e != cudaSuccess) return cuda_fail(h, e, "ice_adjust_vjp launch");
  return ICE3GB_OK;
}

int ice3gb_sedimentation_vjp(void *handle, int nij, int nk, double dt, const Ice3gbSedimentationFields *f,
                             const Ice3gbSedimentationCotangents *g, const Ice3gbSedimentationGradients *gx,
                             void *stream)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_sedimentation_vjp: invalid handle");
  int rc;
  if ((rc = check_shape(h, nij, nk))) return rc;
  if (!f || !g || !gx) return fail(h, ICE3GB_ERR_NULL, "fields, cotangents or gradients pointer is NULL");
  REQUIRE(f->rhodref); REQUIRE(f->dzz); REQUIRE(f->pabs); REQUIRE(f->tht);
  REQUIRE(f->rcs); REQUIRE(f->rrs); REQUIRE(f->ris); REQUIRE(f->rss); REQUIRE(f->rgs);
  if ((f->sea == nullptr) != (f->town == nullptr))
    return fail(h, ICE3GB_ERR_NULL, "sea and town must be both given or both NULL");
  if ((rc = check_device(h))) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long n = (long)nij * nk;
  SedVjpArgs a;
  std::memset(&a, 0, sizeof(a));
  a.rhodref = f->rhodref; a.dzz = f->dzz; a.pabs = f->pabs; a.tht = f->tht; a.sea = f->sea; a.town = f->town;
  a.src[0] = f->rcs; a.src[1] = f->rrs; a.src[2] = f->ris; a.src[3] = f->rss; a.src[4] = f->rgs;
  a.nij = nij; a.nk = nk; a.dt = dt; a.fortran = f->fortran_semantics ? 1 : 0;
  a.g.src[0] = g->rcs; a.g.src[1] = g->rrs; a.g.src[2] = g->ris; a.g.src[3] = g->rss; a.g.src[4] = g->rgs;
  a.g.inpr[0] = g->inprc; a.g.inpr[1] = g->inprr; a.g.inpr[2] = g->inpri; a.g.inpr[3] = g->inprs;
  a.g.inpr[4] = g->inprg;
  a.g.fpr[0] = g->fpr_c; a.g.fpr[1] = g->fpr_r; a.g.fpr[2] = g->fpr_i; a.g.fpr[3] = g->fpr_s; a.g.fpr[4] = g->fpr_g;
  a.gx.src[0] = gx->rcs; a.gx.src[1] = gx->rrs; a.gx.src[2] = gx->ris; a.gx.src[3] = gx->rss;
  a.gx.src[4] = gx->rgs;
  a.gx.rhodref = gx->rhodref; a.gx.dzz = gx->dzz; a.gx.pabs = gx->pabs; a.gx.tht = gx->tht;
  cudaError_t e = cudaMallocAsync(&a.flux, sizeof(double) * 5 * (size_t)n, s);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaMallocAsync");
  {
    ProfScope ps(h, K_SED_VJP, s);
    e = launch_sedimentation_vjp(h->c, a, s);
  }
  cudaFreeAsync(a.flux, s);
  if (e != cudaSuccess) return cuda_fail(h, e, "sedimentation_vjp launch");
  return ICE3GB_OK;
}

int ice3gb_physics_step(void *handle, int nij, int nk, double dt, const Ice3gbRainIceOptions *opt,
                        const Ice3gbStepFields *f, void *stream)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_physics_step: invalid handle");
  int rc;
  if ((rc = check_shape(h, nij, nk)) || (rc = validate_step(h, f)) || (rc = check_device(h))) return rc;
  return run_physics_step(h, nij, nk, dt, opt, f, static_cast<cudaStream_t>(stream));
}

int ice3gb_physics_step_host(void *handle, int nij, int nk, double dt, const Ice3gbRainIceOptions *opt,
                             const Ice3gbStepFields *f, void *stream)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_physics_step_host: invalid handle");
  int rc;
  if ((rc = check_shape(h, nij, nk)) || (rc = validate_step(h, f)) || (rc = check_device(h))) return rc;
  std::lock_guard<std::mutex> lock(h->mu);
  return run_physics_step_pipelined(h, nij, nk, dt, opt, f, static_cast<cudaStream_t>(stream));
}

int ice3gb_rain_ice(void *handle, int nij, int nk, double dt, const Ice3gbRainIceOptions *opt,
                    const Ice3gbRainIceFields *f, void *stream)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_rain_ice: invalid handle");
  int rc;
  if ((rc = check_shape(h, nij, nk)) || (rc = validate_rain_ice(h, f)) || (rc = check_device(h))) return rc;
  return run_rain_ice(h, nij, nk, dt, opt, f, static_cast<cudaStream_t>(stream));
}

// ---- learned surrogate of the ICE4_SLOW rates ------------------------------

int ice3gb_surrogate_sample(void *handle, int nij, int nk, double dt, const Ice3gbRainIceFields *f,
                            const Ice3gbSurrogateNorm *norm, int64_t cap, float *features, float *targets,
                            int64_t *point_of_row, int32_t *row_of_point, uint64_t *counters, void *stream)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_surrogate_sample: invalid handle");
  int rc;
  if ((rc = check_shape(h, nij, nk)) || (rc = validate_rain_ice(h, f)) || (rc = check_device(h))) return rc;
  if (!features || !counters) return fail(h, ICE3GB_ERR_NULL, "ice3gb_surrogate_sample: features or counters NULL");
  if (cap < 0 || cap > 2147483647L) return fail(h, ICE3GB_ERR_RANGE, "ice3gb_surrogate_sample: cap %lld", (long long)cap);
  if (!aligned16(features) || (targets && !aligned16(targets)))
    return fail(h, ICE3GB_ERR_ALIGN, "ice3gb_surrogate_sample: features/targets not 16-byte aligned");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(counters, 0, sizeof(uint64_t) * (1 + ICE3GB_SUR_NSTATS), s);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemsetAsync");
  SurSampleArgs sa;
  std::memset(&sa, 0, sizeof(sa));
  sa.f = *f; sa.luts = h->d_luts; sa.nij = nij; sa.nk = nk; sa.dt = dt;
  sa.norm_on = norm != nullptr;
  if (norm) sa.norm = *norm;
  sa.feat = features; sa.targets = targets;
  sa.point_of_row = reinterpret_cast<long long *>(point_of_row);
  sa.row_of_point = row_of_point;
  sa.count = reinterpret_cast<unsigned long long *>(counters);
  sa.stats = reinterpret_cast<unsigned long long *>(counters) + 1;
  sa.cap = (long)cap;
  ProfScope ps(h, K_SUR_SAMPLE, s);
  if ((e = launch_surrogate_sample(h->c, sa, h->num_sms, s)) != cudaSuccess) return cuda_fail(h, e, "surrogate sample");
  return ICE3GB_OK;
}

int ice3gb_rain_ice_surrogate(void *handle, void *mlp, int nij, int nk, double dt, const Ice3gbRainIceOptions *opt,
                              const Ice3gbRainIceFields *f, const Ice3gbSurrogateNorm *norm, uint64_t *stats,
                              void *stream)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_rain_ice_surrogate: invalid handle");
  int rc;
  if ((rc = check_shape(h, nij, nk)) || (rc = validate_rain_ice(h, f)) || (rc = check_device(h))) return rc;
  const SurCall sur = {mlp, norm, stats};
  if ((rc = check_surrogate(h, sur, (long)nij * nk))) return rc;
  return run_rain_ice(h, nij, nk, dt, opt, f, static_cast<cudaStream_t>(stream), &sur);
}

int ice3gb_physics_step_surrogate(void *handle, void *mlp, int nij, int nk, double dt,
                                  const Ice3gbRainIceOptions *opt, const Ice3gbStepFields *f,
                                  const Ice3gbSurrogateNorm *norm, uint64_t *stats, void *stream)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_physics_step_surrogate: invalid handle");
  int rc;
  if ((rc = check_shape(h, nij, nk)) || (rc = validate_step(h, f)) || (rc = check_device(h))) return rc;
  const SurCall sur = {mlp, norm, stats};
  if ((rc = check_surrogate(h, sur, (long)nij * nk))) return rc;
  return run_physics_step(h, nij, nk, dt, opt, f, static_cast<cudaStream_t>(stream), nullptr, &sur);
}

// ---- host-buffer entry points ---------------------------------------------

int ice3gb_ice_adjust_host(void *handle, int nij, int nk, double dt, const Ice3gbIceAdjustFields *f,
                           void *stream)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_ice_adjust_host: invalid handle");
  int rc;
  if ((rc = check_shape(h, nij, nk)) || (rc = validate_ice_adjust(h, f, nk)) || (rc = check_device(h))) return rc;
  std::lock_guard<std::mutex> lock(h->mu);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = (size_t)nij * nk, b3 = n * sizeof(double);
  const size_t bq = (f->sigqsat_3d ? n : (size_t)nij) * sizeof(double);
  const size_t bq_pad = (bq + 255) & ~(size_t)255, b3_pad = (b3 + 255) & ~(size_t)255;
  // 15 inputs + 4 in-out + 12 outputs (+ srcs) (+ OCND2: zz, ice_cld_wgt and 5 outputs)
  const int nsrc = f->srcs ? 1 : 0;
  const bool ocnd2 = h->c.OCND2 != 0.0;
  const size_t bw_pad = (((size_t)nij * sizeof(double)) + 255) & ~(size_t)255;
  if ((rc = ensure_stage(h, bq_pad + (31 + nsrc + (ocnd2 ? 6 : 0)) * b3_pad + (ocnd2 ? bw_pad : 0)))) return rc;
  char *base = reinterpret_cast<char *>(h->d_stage);
  Ice3gbIceAdjustFields d;
  std::memset(&d, 0, sizeof(d));
  d.sigqsat = reinterpret_cast<double *>(base);
  d.sigqsat_3d = f->sigqsat_3d;
  double *slot = reinterpret_cast<double *>(base + bq_pad);
  const size_t step = b3_pad / sizeof(double);
  const double *const *in_src[] = {&f->pabs, &f->sigs, &f->th, &f->exn, &f->exn_ref, &f->rho_dry_ref, &f->rv,
                                   &f->rc, &f->ri, &f->rr, &f->rs, &f->rg, &f->cf_mf, &f->rc_mf, &f->ri_mf};
  const double **in_dst[] = {&d.pabs, &d.sigs, &d.th, &d.exn, &d.exn_ref, &d.rho_dry_ref, &d.rv,
                             &d.rc, &d.ri, &d.rr, &d.rs, &d.rg, &d.cf_mf, &d.rc_mf, &d.ri_mf};
  double *const *io_src[] = {&f->rvs, &f->rcs, &f->ris, &f->ths};
  double **io_dst[] = {&d.rvs, &d.rcs, &d.ris, &d.ths};
  double *const *out_src[] = {&f->t, &f->rv_out, &f->rc_out, &f->ri_out, &f->cldfr, &f->hlc_hrc, &f->hlc_hcf,
                              &f->hli_hri, &f->hli_hcf, &f->cph, &f->lv, &f->ls};
  double **out_dst[] = {&d.t, &d.rv_out, &d.rc_out, &d.ri_out, &d.cldfr, &d.hlc_hrc, &d.hlc_hcf,
                        &d.hli_hri, &d.hli_hcf, &d.cph, &d.lv, &d.ls};
  cudaError_t e = cudaMemcpyAsync((void *)d.sigqsat, f->sigqsat, bq, cudaMemcpyHostToDevice, s);
  for (int i = 0; i < 15 && e == cudaSuccess; ++i, slot += step) {
    *in_dst[i] = slot;
    e = cudaMemcpyAsync(slot, *in_src[i], b3, cudaMemcpyHostToDevice, s);
  }
  for (int i = 0; i < 4 && e == cudaSuccess; ++i, slot += step) {
    *io_dst[i] = slot;
    e = cudaMemcpyAsync(slot, *io_src[i], b3, cudaMemcpyHostToDevice, s);
  }
  for (int i = 0; i < 12; ++i, slot += step) *out_dst[i] = slot;
  if (nsrc) {
    d.srcs = slot;
    slot += step;
  }
  double *const *o2_src[] = {&f->icldfr, &f->wcldfr, &f->ssio, &f->ssiu, &f->ifr};
  double **o2_dst[] = {&d.icldfr, &d.wcldfr, &d.ssio, &d.ssiu, &d.ifr};
  if (ocnd2) {
    if (e == cudaSuccess) {
      d.zz = slot;
      e = cudaMemcpyAsync(slot, f->zz, b3, cudaMemcpyHostToDevice, s);
      slot += step;
    }
    for (int i = 0; i < 5; ++i, slot += step)
      if (*o2_src[i]) *o2_dst[i] = slot;
    if (e == cudaSuccess) {
      d.ice_cld_wgt = slot;
      e = cudaMemcpyAsync(slot, f->ice_cld_wgt, (size_t)nij * sizeof(double), cudaMemcpyHostToDevice, s);
    }
  }
  if (e != cudaSuccess) return cuda_fail(h, e, "host->device copy");
  IaKernelFields kf;
  kf.f = d;
  kf.rrs = kf.rss = kf.rgs = nullptr;
  kf.adv_dt = 0.0;
  kf.tiwmx = h->d_tiwmx;
  {
    ProfScope ps(h, K_ICE_ADJUST, s);
    e = launch_ice_adjust(h->c, kf, nij, nk, dt, ia_vec2_ok(&d, (long)n), h->num_sms, s);
  }
  if (e != cudaSuccess) return cuda_fail(h, e, "ice_adjust launch");
  for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaMemcpyAsync(*io_src[i], *io_dst[i], b3, cudaMemcpyDeviceToHost, s);
  for (int i = 0; i < 12 && e == cudaSuccess; ++i)
    e = cudaMemcpyAsync(*out_src[i], *out_dst[i], b3, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && nsrc) e = cudaMemcpyAsync(f->srcs, d.srcs, b3, cudaMemcpyDeviceToHost, s);
  for (int i = 0; i < 5 && ocnd2 && e == cudaSuccess; ++i)
    if (*o2_src[i]) e = cudaMemcpyAsync(*o2_src[i], *o2_dst[i], b3, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(h, e, "device->host copy");
  return ICE3GB_OK;
}

int ice3gb_rain_ice_host(void *handle, int nij, int nk, double dt, const Ice3gbRainIceOptions *opt,
                         const Ice3gbRainIceFields *f, void *stream)
{
  Handle *h = as_handle(handle);
  if (!h) return fail(nullptr, ICE3GB_ERR_HANDLE, "ice3gb_rain_ice_host: invalid handle");
  int rc;
  if ((rc = check_shape(h, nij, nk)) || (rc = validate_rain_ice(h, f)) || (rc = check_device(h))) return rc;
  std::lock_guard<std::mutex> lock(h->mu);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = (size_t)nij * nk, b3 = n * sizeof(double), b2 = (size_t)nij * sizeof(double);
  const size_t b3p = (b3 + 255) & ~(size_t)255, b2p = (b2 + 255) & ~(size_t)255;
  const bool adju = (int)h->c.SUBG_AUCV_RC == 2 || (int)h->c.SUBG_AUCV_RI == 2;
  const bool st = f->sea != nullptr;
  const bool fpr = f->fpr_c || f->fpr_r || f->fpr_i || f->fpr_s || f->fpr_g;
  const bool hail = (int)h->c.NRR == 7, ocnd2 = h->c.OCND2 != 0.0;
  // 14 in + cit + (4 hl/hi) + 7 sources + 2 out 3-D (+5 fpr) (+ hail: rht, rhs, fpr_h)
  // (+ OCND2: ssio, ssiu, ifr, icldfr); 2-D: sea town + 6 out (+ inprh)
  const size_t n3 = 14 + 1 + (adju ? 4 : 0) + 7 + 2 + (fpr ? 5 : 0) + (hail ? 3 : 0) + (ocnd2 ? 4 : 0);
  if ((rc = ensure_stage(h, n3 * b3p + 9 * b2p))) return rc;
  char *base = reinterpret_cast<char *>(h->d_stage);
  size_t off = 0;
  auto take3 = [&]() { double *p = reinterpret_cast<double *>(base + off); off += b3p; return p; };
  auto take2 = [&]() { double *p = reinterpret_cast<double *>(base + off); off += b2p; return p; };
  Ice3gbRainIceFields d;
  std::memset(&d, 0, sizeof(d));
  cudaError_t e = cudaSuccess;
  auto up3 = [&](const double *src) -> double * {
    double *p = take3();
    if (e == cudaSuccess) e = cudaMemcpyAsync(p, src, b3, cudaMemcpyHostToDevice, s);
    return p;
  };
  d.exn = up3(f->exn); d.dzz = up3(f->dzz); d.rhodref = up3(f->rhodref); d.exnref = up3(f->exnref);
  d.pabs = up3(f->pabs); d.cldfr = up3(f->cldfr); d.sigs = up3(f->sigs); d.tht = up3(f->tht);
  d.rvt = up3(f->rvt); d.rct = up3(f->rct); d.rrt = up3(f->rrt); d.rit = up3(f->rit); d.rst = up3(f->rst);
  d.rgt = up3(f->rgt); d.cit = up3(f->cit);
  if (adju) {
    d.hlc_hrc = up3(f->hlc_hrc); d.hlc_hcf = up3(f->hlc_hcf); d.hli_hri = up3(f->hli_hri);
    d.hli_hcf = up3(f->hli_hcf);
  }
  d.ths = up3(f->ths); d.rvs = up3(f->rvs); d.rcs = up3(f->rcs); d.rrs = up3(f->rrs); d.ris = up3(f->ris);
  d.rss = up3(f->rss); d.rgs = up3(f->rgs);
  d.evap3d = take3(); d.rainfr = take3();
  if (fpr) { d.fpr_c = take3(); d.fpr_r = take3(); d.fpr_i = take3(); d.fpr_s = take3(); d.fpr_g = take3(); }
  if (st) {
    double *ps = take2(), *pt = take2();
    if (e == cudaSuccess) e = cudaMemcpyAsync(ps, f->sea, b2, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(pt, f->town, b2, cudaMemcpyHostToDevice, s);
    d.sea = ps; d.town = pt;
  } else {
    take2(); take2();
  }
  d.inprc = take2(); d.inprr = take2(); d.inpri = take2(); d.inprs = take2(); d.inprg = take2();
  d.indep = f->indep ? take2() : nullptr;
  if (hail) {
    d.rht = up3(f->rht);
    d.rhs = up3(f->rhs);
    d.fpr_h = f->fpr_h ? take3() : nullptr;
    d.inprh = take2();
  }
  if (ocnd2) {
    d.ssio = up3(f->ssio); d.ssiu = up3(f->ssiu); d.ifr = up3(f->ifr); d.icldfr = up3(f->icldfr);
  }
  if (e != cudaSuccess) return cuda_fail(h, e, "host->device copy");
  if ((rc = run_rain_ice(h, nij, nk, dt, opt, &d, s))) return rc;
  struct Pair { double *dst; const double *src; size_t bytes; };
  const Pair back[] = {
      {f->cit, d.cit, b3}, {f->ths, d.ths, b3}, {f->rvs, d.rvs, b3}, {f->rcs, d.rcs, b3}, {f->rrs, d.rrs, b3},
      {f->ris, d.ris, b3}, {f->rss, d.rss, b3}, {f->rgs, d.rgs, b3}, {f->evap3d, d.evap3d, b3},
      {f->rainfr, d.rainfr, b3}, {f->inprc, d.inprc, b2}, {f->inprr, d.inprr, b2}, {f->inpri, d.inpri, b2},
      {f->inprs, d.inprs, b2}, {f->inprg, d.inprg, b2}, {f->indep, d.indep, b2},
      {f->fpr_c, d.fpr_c, b3}, {f->fpr_r, d.fpr_r, b3}, {f->fpr_i, d.fpr_i, b3}, {f->fpr_s, d.fpr_s, b3},
      {f->fpr_g, d.fpr_g, b3}, {hail ? f->rhs : nullptr, d.rhs, b3}, {hail ? f->inprh : nullptr, d.inprh, b2},
      {hail ? f->fpr_h : nullptr, d.fpr_h, b3}};
  for (const Pair &p : back)
    if (p.dst && p.src && e == cudaSuccess) e = cudaMemcpyAsync(p.dst, p.src, p.bytes, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(h, e, "device->host copy");
  return ICE3GB_OK;
}

}  // extern "C"
