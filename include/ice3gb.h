/*
 * ice3gb.h — C ABI of the GB300-native ICE3 one-moment microphysics hot path
 * (saturation adjustment `ice_adjust`, the ICE4 `rain_ice` step and the
 * statistical sedimentation sweep), FP64, one GPU.
 *
 * Reference interfaces this ABI replaces (maurinl26/dwarf-p-ice3):
 *   - Fortran/C bridge `c_ice_adjust`    PHYEX-IAL_CY50T1/bridge/phyex_bridge.F90:27
 *   - Fortran/C bridge `c_ini_rain_ice`  PHYEX-IAL_CY50T1/bridge/phyex_bridge.F90:215
 *   - Fortran/C bridge `c_rain_ice`      PHYEX-IAL_CY50T1/bridge/phyex_bridge.F90:242
 *   - Python components `IceAdjustJAX.__call__` src/ice3/jax/ice_adjust.py:139
 *     and `RainIceJAX.__call__` src/ice3/jax/rain_ice.py:181
 *   - `sedimentation_stat` src/ice3/jax/stencils/sedimentation.py:58
 *
 * Conventions (same memory order as the Fortran bridge's (nlon, nlev) arrays):
 *   - every 3-D field is contiguous [nk][nij] (horizontal index fastest),
 *     FP64, element (ij, k) at offset k*nij + ij; k = 0 is the lowest level
 *     (ground-to-space ordering, PHYEX D%NKL = 1);
 *   - 2-D (per column) fields are [nij];
 *   - the device entry points take DEVICE pointers and run asynchronously on
 *     `stream` (a cudaStream_t passed as void*; NULL = legacy default stream);
 *     the `_host` entry points take HOST pointers, stage through device
 *     buffers owned by the handle and return after the results are back;
 *   - callers own all field memory; in-out fields are read then overwritten;
 *   - every call returns ICE3GB_OK (0) or a negative ICE3GB_ERR_* code, no
 *     exception or abort crosses the ABI; `ice3gb_last_error` gives the text.
 *
 * A handle holds one immutable constants table (the reference's
 * `Phyex(...).to_externals()` flattened into Ice3gbConstants + Ice3gbLuts),
 * so, unlike the Fortran module state set by `c_ini_rain_ice`, several tables
 * can live side by side.  Concurrent calls on one handle must use distinct
 * streams and are then safe, except the `_host` calls, which share the
 * handle's staging buffers and must be serialised by the caller.
 */
#ifndef ICE3GB_H
#define ICE3GB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ICE3GB_VERSION 10000 /* 1.0.0 */

/* ---- status codes ------------------------------------------------------ */
#define ICE3GB_OK               0
#define ICE3GB_ERR_NULL        -1  /* required pointer is NULL            */
#define ICE3GB_ERR_SHAPE       -2  /* nij/nk out of range                  */
#define ICE3GB_ERR_ALIGN       -3  /* field not 16-byte aligned            */
#define ICE3GB_ERR_CUDA        -4  /* CUDA runtime error                   */
#define ICE3GB_ERR_UNSUPPORTED -5  /* option value not implemented         */
#define ICE3GB_ERR_DEVICE      -6  /* device-side status word set          */
#define ICE3GB_ERR_HANDLE      -7  /* invalid handle                       */
#define ICE3GB_ERR_RANGE       -8  /* size beyond a fixed limit            */

/* Device status word bits (read by ice3gb_status). */
#define ICE3GB_DEV_PASS_CAP     1u /* a point hit the sub-step pass cap     */
#define ICE3GB_DEV_SED_CAP      2u /* a column hit the SPLI sub-step cap    */

/*
 * Constants table: every field is a double (switches stored as 0.0/1.0,
 * enumerations as their integer value).  Names are the keys of
 * `Phyex(program).to_externals()` (src/ice3/phyex_common/phyex.py:307).
 * `ice3gb_constant_name(i)` returns the i-th name, so hosts fill by name.
 */
#define ICE3GB_CONSTANTS(X)                                                   \
  /* physical constants (modd_cst) */                                         \
  X(TT) X(CPD) X(CPV) X(CL) X(CI) X(RD) X(RV) X(LVTT) X(LSTT) X(LMTT)         \
  X(ESTT) X(ALPW) X(BETAW) X(GAMW) X(ALPI) X(BETAI) X(GAMI) X(EPSILO)         \
  X(P00) X(RHOLW) X(MNH_TINY) X(GRAVITY0) X(PI)                               \
  /* subgrid condensation (modd_nebn) */                                      \
  X(TMAXMIX) X(TMINMIX) X(LSUBG_COND) X(LSIGMAS) X(LSTATNW)                   \
  X(FRAC_ICE_ADJUST) X(CONDENS) X(OCND2) X(NRR) X(LAMBDA3)                    \
  /* ICE3/ICE4 switches (modd_param_icen) */                                  \
  X(LWARM) X(LSEDIC) X(LDEPOSC) X(VDEPOSC) X(SEDIM) X(LFEEDBACKT)             \
  X(LEVLIMIT) X(LNULLWETG) X(LWETGPOST) X(SNOW_RIMING) X(LCRFLIMIT)           \
  X(NMAXITER_MICRO) X(MRSTEP) X(TSTEP_TS) X(SUBG_RC_RR_ACCR) X(SUBG_RR_EVAP)  \
  X(SUBG_PR_PDF) X(SUBG_AUCV_RC) X(SUBG_AUCV_RI) X(SUBG_MF_PDF)               \
  X(LSEDIM_AFTER) X(LSNOW_T) X(SPLIT_MAXCFL)                                  \
  /* hydrometeor descriptors (modd_rain_ice_descrn) */                        \
  X(CEXVT) X(V_RTMIN) X(C_RTMIN) X(R_RTMIN) X(I_RTMIN) X(S_RTMIN) X(G_RTMIN)  \
  X(CC) X(DC) X(LBEXC) X(LBC_1) X(LBC_2) X(LBR) X(LBEXR) X(LBI) X(LBEXI)      \
  X(DI) X(LBS) X(LBEXS) X(LBG) X(LBEXG) X(CXS) X(BS) X(CXG) X(DG)             \
  X(LBDAS_MAX) X(LBDAS_MIN) X(TRANS_MP_GAMMAS) X(CONC_SEA) X(CONC_LAND)       \
  X(CONC_URBAN) X(FVELOS) X(ALPHAS) X(NUS) X(GAC) X(GC) X(GAC2) X(GC2)        \
  /* rate constants (modd_rain_ice_paramn) */                                 \
  X(FSEDC_1) X(FSEDC_2) X(FSEDR) X(EXSEDR) X(FSEDI) X(EXCSEDI) X(FSEDS)       \
  X(EXSEDS) X(FSEDG) X(EXSEDG) X(NU10) X(ALPHA1) X(BETA1) X(NU20) X(ALPHA2)   \
  X(BETA2) X(MNU0) X(ALPHA3) X(BETA3) X(HON) X(SCFAC) X(O0EVAR) X(O1EVAR)     \
  X(EX0EVAR) X(EX1EVAR) X(O0DEPI) X(O2DEPI) X(O0DEPS) X(O1DEPS) X(EX0DEPS)    \
  X(EX1DEPS) X(O0DEPG) X(O1DEPG) X(EX0DEPG) X(EX1DEPG) X(TIMAUTI) X(TEXAUTI)  \
  X(CRIAUTI) X(ACRIAUTI) X(BCRIAUTI) X(FIAGGS) X(COLEXIS) X(EXIAGGS)          \
  X(TIMAUTC) X(CRIAUTC) X(FCACCR) X(EXCACCR) X(CRIMSS) X(EXCRIMSS) X(CRIMSG)  \
  X(EXCRIMSG) X(SRIMCG) X(EXSRIMCG) X(SRIMCG2) X(EXSRIMCG2) X(SRIMCG3)        \
  X(RIMINTP1) X(RIMINTP2) X(NGAMINC) X(FRACCSS) X(LBRACCS1) X(LBRACCS2)       \
  X(LBRACCS3) X(FSACCRG) X(LBSACCR1) X(LBSACCR2) X(LBSACCR3) X(ACCINTP1S)     \
  X(ACCINTP2S) X(ACCINTP1R) X(ACCINTP2R) X(NACCLBDAS) X(NACCLBDAR) X(FSCVMG)  \
  X(RCFRI) X(EXRCFRI) X(ICFRR) X(EXICFRR) X(FCDRYG) X(COLIG) X(COLEXIG)       \
  X(FIDRYG) X(COLSG) X(COLEXSG) X(FSDRYG) X(LBSDRYG1) X(LBSDRYG2)             \
  X(LBSDRYG3) X(FRDRYG) X(LBRDRYG1) X(LBRDRYG2) X(LBRDRYG3) X(DRYINTP1R)      \
  X(DRYINTP2R) X(DRYINTP1S) X(DRYINTP2S) X(DRYINTP1G) X(DRYINTP2G)            \
  X(NDRYLBDAR) X(NDRYLBDAS) X(NDRYLBDAG)                                      \
  /* hail, NRR = 7 (mode_ini_rain_ice.F90 2.5, 5, 9; modd_param_icen) */      \
  X(H_RTMIN) X(LBH) X(LBEXH) X(CXH) X(DH) X(BG) X(FSEDH) X(EXSEDH)            \
  X(O0DEPH) X(O1DEPH) X(EX0DEPH) X(EX1DEPH) X(FWETH) X(COLIH) X(COLEXIH)      \
  X(FSWETH) X(LBSWETH1) X(LBSWETH2) X(LBSWETH3) X(COLSH) X(COLEXSH)           \
  X(FGWETH) X(LBGWETH1) X(LBGWETH2) X(LBGWETH3) X(COLGH) X(COLEXGH)           \
  X(FRWETH) X(LBRWETH1) X(LBRWETH2) X(LBRWETH3) X(WETINTP1H) X(WETINTP2H)     \
  X(WETINTP1S) X(WETINTP2S) X(WETINTP1G) X(WETINTP2G) X(WETINTP1R)            \
  X(WETINTP2R) X(NWETLBDAH) X(NWETLBDAS) X(NWETLBDAG) X(NWETLBDAR)            \
  X(LNULLWETH) X(LWETHPOST) X(LCONVHG)                                        \
  /* XFRMIN(1:40), the OCND2 tuning vector (modd_param_icen.F90:366-395) */     \
  X(FRMIN1) X(FRMIN2) X(FRMIN3) X(FRMIN4) X(FRMIN5) X(FRMIN6) X(FRMIN7)       \
  X(FRMIN8) X(FRMIN9) X(FRMIN10) X(FRMIN11) X(FRMIN12) X(FRMIN13)             \
  X(FRMIN14) X(FRMIN15) X(FRMIN16) X(FRMIN17) X(FRMIN18) X(FRMIN19)           \
  X(FRMIN20) X(FRMIN21) X(FRMIN22) X(FRMIN23) X(FRMIN24) X(FRMIN25)           \
  X(FRMIN26) X(FRMIN27) X(FRMIN28) X(FRMIN29) X(FRMIN30) X(FRMIN31)           \
  X(FRMIN32) X(FRMIN33) X(FRMIN34) X(FRMIN35) X(FRMIN36) X(FRMIN37)           \
  X(FRMIN38) X(FRMIN39) X(FRMIN40)

typedef struct Ice3gbConstants {
#define ICE3GB_X_FIELD(name) double name;
  ICE3GB_CONSTANTS(ICE3GB_X_FIELD)
#undef ICE3GB_X_FIELD
} Ice3gbConstants;

/* Lookup tables of the ICE4 collection kernels, FP64.  Two-dimensional
 * tables are row-major: ker_x[i*n2 + j] is the Fortran XKER_X(i+1, j+1)
 * (micro/mode_ini_rain_ice.F90:768-890, data in src/ice3/phyex_common/xker_*.py). */
#define ICE3GB_NGAMINC   80
#define ICE3GB_NACCLBDAS 40
#define ICE3GB_NACCLBDAR 40
#define ICE3GB_NDRYLBDAG 40
#define ICE3GB_NDRYLBDAS 80
#define ICE3GB_NDRYLBDAR 40
#define ICE3GB_NWETLBDAH 40   /* hail tables (NRR = 7 only)               */
#define ICE3GB_NWETLBDAS 80
#define ICE3GB_NWETLBDAG 40
#define ICE3GB_NWETLBDAR 40
typedef struct Ice3gbLuts {
  double gaminc_rim1[ICE3GB_NGAMINC];
  double gaminc_rim2[ICE3GB_NGAMINC];
  double gaminc_rim4[ICE3GB_NGAMINC];
  double ker_raccss[ICE3GB_NACCLBDAS * ICE3GB_NACCLBDAR]; /* (lbdas, lbdar) */
  double ker_raccs[ICE3GB_NACCLBDAS * ICE3GB_NACCLBDAR];  /* (lbdas, lbdar) */
  double ker_saccrg[ICE3GB_NACCLBDAR * ICE3GB_NACCLBDAS]; /* (lbdar, lbdas) */
  double ker_rdryg[ICE3GB_NDRYLBDAG * ICE3GB_NDRYLBDAR];  /* (lbdag, lbdar) */
  double ker_sdryg[ICE3GB_NDRYLBDAG * ICE3GB_NDRYLBDAS];  /* (lbdag, lbdas) */
  /* hail collection kernels XKER_SWETH / GWETH / RWETH
     (micro/mode_read_xker_sweth.F90, _gweth, _rweth)                       */
  double ker_sweth[ICE3GB_NWETLBDAH * ICE3GB_NWETLBDAS];  /* (lbdah, lbdas) */
  double ker_gweth[ICE3GB_NWETLBDAH * ICE3GB_NWETLBDAG];  /* (lbdah, lbdag) */
  double ker_rweth[ICE3GB_NWETLBDAH * ICE3GB_NWETLBDAR];  /* (lbdah, lbdar) */
} Ice3gbLuts;

/* ---- ice_adjust -------------------------------------------------------- */
/* Arguments of IceAdjustJAX.__call__ (src/ice3/jax/ice_adjust.py:139-160)
 * and of c_ice_adjust (phyex_bridge.F90:27-35); outputs are the 16-tuple of
 * src/ice3/jax/stencils/ice_adjust.py:381-398, written in place. */
typedef struct Ice3gbIceAdjustFields {
  const double *sigqsat;            /* [nij], or [nk][nij] if sigqsat_3d  */
  const double *pabs, *sigs, *th, *exn, *exn_ref, *rho_dry_ref;
  const double *rv, *rc, *ri, *rr, *rs, *rg;
  const double *cf_mf, *rc_mf, *ri_mf;
  double *rvs, *rcs, *ris, *ths;    /* in-out sources                    */
  double *t, *rv_out, *rc_out, *ri_out, *cldfr;
  double *hlc_hrc, *hlc_hcf, *hli_hri, *hli_hcf;
  double *cph, *lv, *ls;
  int64_t sigqsat_3d;               /* 0: per column, 1: full 3-D field   */
  double *srcs;                     /* optional out (NULL: not computed):
                                       PSRCS = s'r_c'/sigma_s^2 of
                                       ice_adjust.F90:360,468 and
                                       condensation.F90:566-571, :638-647  */
  /* OCND2 = 1 only (separate liquid and ice clouds, condensation.F90:373-395,
   * :588-637, mode_icecloud.F90); ignored otherwise:                       */
  const double *zz;                 /* [nk][nij] height of the levels (m),
                                       k = 0 at the surface; nk >= 2        */
  const double *ice_cld_wgt;        /* [nij] PICE_CLD_WGT                  */
  double *icldfr, *wcldfr;          /* out: ice / water cloud fraction     */
  double *ssio, *ssiu;              /* out: ice super-saturation in the
                                       cloudy / clear part                 */
  double *ifr;                      /* out: PIFR (10 everywhere)           */
} Ice3gbIceAdjustFields;

/* ---- statistical sedimentation ---------------------------------------- */
/* Arguments of sedimentation_stat (src/ice3/jax/stencils/sedimentation.py:58)
 * ~ ICE4_SEDIMENTATION_STAT (micro/mode_ice4_sedimentation_stat.F90:9).
 * The two reference implementations differ, `fortran_semantics` selects:
 *   0: reference JAX — cloud mean-radius factor 1 (sedimentation.py:156) and
 *      flux divergence divided by rho*dz*dt (sedimentation.py:337-341);
 *   1: PHYEX Fortran — factor MAX(1, 0.5*Gamma(NUC+1/ALPHAC)/Gamma(NUC))
 *      weighted by sea (mode_ice4_sedimentation_stat.F90:123-127, 253) and
 *      divergence divided by rho*dz (:203-207). */
typedef struct Ice3gbSedimentationFields {
  const double *rhodref, *dzz, *pabs, *tht;
  const double *sea, *town;         /* [nij], optional (NULL -> 0)        */
  double *rcs, *rrs, *ris, *rss, *rgs;            /* in-out sources       */
  double *inprc, *inprr, *inpri, *inprs, *inprg;  /* out [nij]            */
  double *fpr_c, *fpr_r, *fpr_i, *fpr_s, *fpr_g;  /* out, optional        */
  int64_t fortran_semantics;
} Ice3gbSedimentationFields;

/* ---- rain_ice ---------------------------------------------------------- */
/* Arguments of c_rain_ice (phyex_bridge.F90:242-254) / RAIN_ICE
 * (micro/rain_ice.F90) and of the RainIceJAX state dict
 * (src/ice3/jax/rain_ice.py:181).  The handle's SUBG_RC_RR_ACCR (NONE,
 * PRFR) and SUBG_RR_EVAP (NONE, CLFR, PRFR) select the warm-process forms;
 * with a PRFR option the call first forms the precipitation fraction from
 * the time-t state (rain_ice.F90:555-605), which rewrites hlc_hcf, hlc_hrc,
 * hli_hcf and hli_hri with ICE4_COMPUTE_PDF's partition, as the Fortran's
 * INOUT arguments; rainfr returns the precipitation fraction (1 everywhere
 * without a PRFR option). */
typedef struct Ice3gbRainIceFields {
  const double *exn, *dzz, *rhodref, *exnref, *pabs, *cldfr, *sigs;
  const double *tht, *rvt, *rct, *rrt, *rit, *rst, *rgt;
  const double *sea, *town;         /* [nij], optional                    */
  double *cit;                      /* in-out pristine ice concentration  */
  double *hlc_hrc, *hlc_hcf, *hli_hri, *hli_hcf;  /* in-out               */
  double *ths, *rvs, *rcs, *rrs, *ris, *rss, *rgs; /* in-out sources      */
  double *evap3d, *rainfr;          /* out [nk][nij]                      */
  double *inprc, *inprr, *inpri, *inprs, *inprg, *indep; /* out [nij]     */
  double *fpr_c, *fpr_r, *fpr_i, *fpr_s, *fpr_g;  /* out, optional        */
  /* hail (NRR = 7 only; ignored otherwise)                                 */
  const double *rht;                /* hail mixing ratio at t             */
  double *rhs;                      /* in-out hail source                 */
  double *inprh;                    /* out [nij] hail precipitation rate  */
  double *fpr_h;                    /* out, optional                      */
  /* OCND2 only (ignored otherwise): the ice_adjust OCND2 outputs of the
   * same state (Ice3gbIceAdjustFields ssio, ssiu, ifr, icldfr)           */
  const double *ssio, *ssiu, *ifr, *icldfr;
} Ice3gbRainIceFields;

/* Per-call overrides of RainIceJAX.__call__ keywords
 * (src/ice3/jax/rain_ice.py:181-190); a negative value keeps the table's. */
typedef struct Ice3gbRainIceOptions {
  int32_t lsedim_after;   /* LSEDIM_AFTER                                   */
  int32_t ldeposc;        /* LDEPOSC (fog deposition)                       */
  int32_t lfeedbackt;     /* LFEEDBACKT                                     */
  int32_t max_passes;     /* cap on tendency passes per point (default 256) */
  int32_t sed_jax;        /* 1: reference-JAX sedimentation semantics,
                             0 (default): Fortran (see Ice3gbSedimentationFields) */
} Ice3gbRainIceOptions;

/* ---- chained physics step --------------------------------------------- */
/* One AROME-style microphysics step on a time-t state, fused on the device:
 *   S1 = ice_adjust(x_t, S0)
 *   S2 = rain_ice(x_t, S1, cloud fraction and hl* of the first adjustment)
 *   S3 = ice_adjust(dt*S2, S2)
 * Sources are PHYEX total sources (x_{t+dt}/dt), so dt*S2 is the state after
 * the microphysics; the order follows PHYEX's adjustment before and after the
 * microphysics (micro/ice_adjust.F90, micro/rain_ice.F90).  In-out sources go
 * S0 -> S3 (rrs/rss/rgs end as S2); the outputs are those of the final
 * adjustment plus the rain_ice diagnostics.  No counterpart entry point exists
 * in the reference; it chains the two reference interfaces above. */
typedef struct Ice3gbStepFields {
  const double *sigqsat;            /* [nij]                                */
  const double *pabs, *exn, *exnref, *rhodref, *dzz, *sigs;
  const double *th, *rv, *rc, *ri, *rr, *rs, *rg;
  const double *cf_mf, *rc_mf, *ri_mf;
  const double *sea, *town;         /* [nij], optional                    */
  double *ths, *rvs, *rcs, *rrs, *ris, *rss, *rgs, *cit;  /* in-out        */
  double *t, *rv_out, *rc_out, *ri_out, *cldfr;
  double *hlc_hrc, *hlc_hcf, *hli_hri, *hli_hcf;
  double *evap3d, *rainfr;          /* out [nk][nij]                      */
  double *inprc, *inprr, *inpri, *inprs, *inprg;  /* out [nij]            */
} Ice3gbStepFields;

/* ---- library / handle -------------------------------------------------- */
int         ice3gb_version(void);
int         ice3gb_constant_count(void);
const char *ice3gb_constant_name(int i);
/* Replaces c_ini_rain_ice (phyex_bridge.F90:215): validates the table,
 * uploads the lookup tables to the current device, returns a handle. */
int ice3gb_create(const Ice3gbConstants *c, const Ice3gbLuts *luts, void **handle);
int ice3gb_destroy(void *handle);
/* Text of the last error on this handle (or of the last global error when
 * handle is NULL); returns the message length. */
int ice3gb_last_error(void *handle, char *buf, size_t n);
/* Synchronises `stream`, reads and clears the device status word; returns
 * ICE3GB_OK or ICE3GB_ERR_DEVICE (bits in *bits when non-NULL). */
int ice3gb_status(void *handle, void *stream, uint32_t *bits);

/* ---- device entry points (async on stream) ----------------------------- */
/* Replaces c_ice_adjust (phyex_bridge.F90:27) / IceAdjustJAX.__call__. */
int ice3gb_ice_adjust(void *handle, int nij, int nk, double dt,
                      const Ice3gbIceAdjustFields *f, void *stream);
/* Replaces sedimentation_stat (stencils/sedimentation.py:58); the statistical
 * scheme whatever the table's SEDIM. */
int ice3gb_sedimentation(void *handle, int nij, int nk, double dt,
                         const Ice3gbSedimentationFields *f, void *stream);
/* Replaces c_rain_ice (phyex_bridge.F90:242) / RainIceJAX.__call__.  NRR = 7
 * adds hail (rht, rhs, inprh required; ICE4_FAST_RH and the hail species).  The
 * table's SEDIM picks the sedimentation: STAT (1) or SPLI (0, time-split,
 * micro/mode_ice4_sedimentation_split.F90, followed by
 * ICE4_CORRECT_NEGATIVITIES, micro/mode_ice4_sedimentation.F90:196-229;
 * allocates 2 nij*nk doubles of stream-ordered scratch). */
int ice3gb_rain_ice(void *handle, int nij, int nk, double dt,
                    const Ice3gbRainIceOptions *opt,
                    const Ice3gbRainIceFields *f, void *stream);

/* Chained ice_adjust -> rain_ice -> ice_adjust step (see Ice3gbStepFields). */
int ice3gb_physics_step(void *handle, int nij, int nk, double dt, const Ice3gbRainIceOptions *opt,
                        const Ice3gbStepFields *f, void *stream);

/* ---- adjoint of ice_adjust ---------------------------------------------- */
/* Cotangents of the 16 outputs of ice3gb_ice_adjust (NULL = zero), same
 * names and shapes as in Ice3gbIceAdjustFields. */
typedef struct Ice3gbIceAdjustCotangents {
  const double *t, *rv_out, *rc_out, *ri_out, *cldfr;
  const double *hlc_hrc, *hlc_hcf, *hli_hri, *hli_hcf;
  const double *cph, *lv, *ls;
  const double *rvs, *rcs, *ris, *ths;
} Ice3gbIceAdjustCotangents;

/* Gradients of the 20 inputs (NULL = not wanted; written, not accumulated).
 * sigqsat is [nij] when the forward's sigqsat is per column (its gradient is
 * then summed over the levels), [nk][nij] otherwise. */
typedef struct Ice3gbIceAdjustGradients {
  double *sigqsat, *pabs, *sigs, *th, *exn, *exn_ref, *rho_dry_ref;
  double *rv, *rc, *ri, *rr, *rs, *rg;
  double *cf_mf, *rc_mf, *ri_mf;
  double *rvs, *rcs, *ris, *ths;
} Ice3gbIceAdjustGradients;

/* Vector-Jacobian product of ice3gb_ice_adjust at the inputs of `f` (its
 * output pointers are not used): gradients of <cotangents, outputs> with
 * respect to every input.  Hand-written reverse mode that recomputes the
 * forward intermediates per point; at kinks (min/max, clips) the derivative
 * of the branch the forward takes.  No counterpart in the reference (which
 * relies on jax.vjp of IceAdjustJAX, src/ice3/jax/ice_adjust.py:139). */
int ice3gb_ice_adjust_vjp(void *handle, int nij, int nk, double dt, const Ice3gbIceAdjustFields *f,
                          const Ice3gbIceAdjustCotangents *g, const Ice3gbIceAdjustGradients *gx, void *stream);

/* ---- adjoint of the sedimentation sweep ---------------------------------- */
/* Cotangents of the outputs of ice3gb_sedimentation (NULL = zero): the
 * updated sources [nk][nij], the surface precipitation [nij] and the
 * fluxes fpr_* [nk][nij]. */
typedef struct Ice3gbSedimentationCotangents {
  const double *rcs, *rrs, *ris, *rss, *rgs;
  const double *inprc, *inprr, *inpri, *inprs, *inprg;
  const double *fpr_c, *fpr_r, *fpr_i, *fpr_s, *fpr_g;
} Ice3gbSedimentationCotangents;

/* Gradients of the inputs (NULL = not wanted): the sources before the sweep
 * and rhodref, dzz, pabs, tht [nk][nij]. */
typedef struct Ice3gbSedimentationGradients {
  double *rcs, *rrs, *ris, *rss, *rgs;
  double *rhodref, *dzz, *pabs, *tht;
} Ice3gbSedimentationGradients;

/* Vector-Jacobian product of ice3gb_sedimentation at the inputs of `f` (its
 * rcs..rgs are read as the sources before the sweep and not modified; its
 * output pointers are not used).  Hand-written reverse sweep (bottom-up)
 * that recomputes the column fluxes first.  No counterpart in the reference
 * (sedimentation_stat, src/ice3/jax/stencils/sedimentation.py:58). */
int ice3gb_sedimentation_vjp(void *handle, int nij, int nk, double dt, const Ice3gbSedimentationFields *f,
                             const Ice3gbSedimentationCotangents *g, const Ice3gbSedimentationGradients *gx,
                             void *stream);

/* ---- BF16 tensor-core MLP (the slow-process surrogate) ------------------ */
/* A per-point MLP n_in -> n_hidden (GELU) x n_hidden_layers -> n_out with
 * BF16 weights and activations on the tcgen05 tensor cores (FP32
 * accumulation), FP32 master weights and Adam; hand-written backward pass.
 * Limits: n_in <= 256, 16 <= n_hidden <= 256, n_hidden_layers <= 8, n_out
 * even and <= 16.  Parameters: a flat FP32 vector, per layer W [out][in]
 * then b [out].  Arrays are device FP32: x [n][n_in], y [n][n_out], targets
 * [n][16] (per rate r: 2r = 1 if the rate is nonzero, 2r + 1 = transformed
 * value).  No counterpart exists in the reference. */
typedef struct Ice3gbMlpShape {
  int32_t n_in, n_hidden, n_hidden_layers, n_out;
} Ice3gbMlpShape;
int     ice3gb_mlp_create(const Ice3gbMlpShape *shape, uint64_t seed, void **mlp);
int     ice3gb_mlp_destroy(void *mlp);
int64_t ice3gb_mlp_param_count(void *mlp);
int     ice3gb_mlp_get_params(void *mlp, float *host);
int     ice3gb_mlp_set_params(void *mlp, const float *host);
/* Inference.  The surrogate's shape (16 -> 256 x 3 -> <= 16) with 16-byte
 * aligned x runs one fused persistent kernel (weights streamed from L2,
 * activations kept on chip); other shapes, and ice3gb_mlp_forward_layered
 * always, run one tensor-core GEMM launch per layer (the training forward).
 * Both give the same values bit for bit. */
int     ice3gb_mlp_forward(void *mlp, int n, const float *x, float *y, void *stream);
int     ice3gb_mlp_forward_layered(void *mlp, int n, const float *x, float *y, void *stream);
/* Loss (binary cross-entropy of the activity logits + squared error of the
 * values where active, mean over the n rows) and its gradient (device
 * [param_count] or NULL) for one batch. */
int     ice3gb_mlp_loss_grad(void *mlp, int n, const float *x, const float *targets, float *grad, float *loss,
                             void *stream);
/* One Adam step (lr, beta 0.9 / 0.999) on one batch; loss: device float or NULL. */
int     ice3gb_mlp_train_step(void *mlp, int n, const float *x, const float *targets, float lr, float *loss,
                              void *stream);
/* ICE3GB_ERR_DEVICE if a tensor-core kernel of this MLP timed out on its barrier. */
int     ice3gb_mlp_error(void *mlp);
/* The GEMM building block: C[m][n] (FP32, row stride ldc) = sum_k A(m,k) B(n,k)
 * with BF16 A(m,k) = A[m*sam + k*sak], B(n,k) = B[n*sbn + k*sbk], N <= 256. */
int     ice3gb_tc_gemm_bf16(int M, int N, int K, const void *A, int64_t sam, int64_t sak, const void *B, int64_t sbn,
                            int64_t sbk, float *C, int64_t ldc, int *err, void *stream);

/* ---- learned surrogate of the ICE4_SLOW rates ----------------------------- */
/* The MLP (16 features -> 10 outputs: per slow rate RCHONI, RVDEPS, RIAGGS,
 * RIAUTS, RVDEPG a logit "nonzero" and asinh(rate / 1e-12) / 10) stands in
 * for the five ICE4_SLOW rates (PHYEX mode_ice4_slow.F90, reached from the
 * reference's rain_ice through src/ice3/jax/rain_ice.py:181) at the first
 * hard pass of each micro point.  Features: T, ln p, ln rho, ln rv, ln rc,
 * ln rr, ln ri, ln rs, ln rg, cloud fraction, Exner, dt, ln lbda of rain /
 * snow / graupel, ssi, taken where the plain kernel evaluates the rates.
 * Standardised as (x - mean) * inv_std; points whose standardised features
 * leave [lo, hi] run the plain path.  No counterpart exists in the
 * reference. */
#define ICE3GB_SUR_NFEAT 16
#define ICE3GB_SUR_NOUT 10
typedef struct Ice3gbSurrogateNorm {
  float mean[16], inv_std[16], lo[16], hi[16];
} Ice3gbSurrogateNorm;
/* counters of a surrogate call (uint64 each) */
enum {
  ICE3GB_SUR_MICRO = 0,           /* micro points of rain_ice */
  ICE3GB_SUR_OUTSIDE = 1,         /* micro points outside the envelope (plain path) */
  ICE3GB_SUR_OVER_CAP = 2,        /* accepted points beyond the row capacity (plain path) */
  ICE3GB_SUR_USED = 3,            /* points that kept the learned slow rates */
  ICE3GB_SUR_FIXUP_FALLBACK = 4,  /* points recomputed by the plain path after the fix-up check */
  ICE3GB_SUR_NSTATS = 8
};
/* Features (and, if targets != NULL, the plain kernel's slow rates encoded
 * as training targets: per rate k, column 2k = 1 if nonzero, 2k+1 = coded
 * value, 10 + k = the rate) of the micro points of one rain_ice call,
 * compacted to rows in an unspecified order: point_of_row / row_of_point
 * (either may be NULL) map rows to grid points (-1: no row).  norm = NULL:
 * raw features, no envelope.  counters: device uint64[1 + ICE3GB_SUR_NSTATS]
 * = rows handed out, then the counters; zeroed by the call.  features and
 * targets: 16-byte aligned device float [cap][16]; cap <= 2^31 - 1.  The
 * fields are only read. */
int ice3gb_surrogate_sample(void *handle, int nij, int nk, double dt, const Ice3gbRainIceFields *f,
                            const Ice3gbSurrogateNorm *norm, int64_t cap, float *features, float *targets,
                            int64_t *point_of_row, int32_t *row_of_point, uint64_t *counters, void *stream);
/* ice3gb_rain_ice with the network's slow rates (mlp: ice3gb_mlp_create
 * handle with n_in 16, n_out 10) where a point is inside the envelope and
 * passes the fix-up check, the plain path elsewhere, in the same launch.
 * stats: host uint64[ICE3GB_SUR_NSTATS] or NULL (NULL avoids the final
 * synchronisation; the call synchronises once on the stream to size the
 * network's batch). */
int ice3gb_rain_ice_surrogate(void *handle, void *mlp, int nij, int nk, double dt, const Ice3gbRainIceOptions *opt,
                              const Ice3gbRainIceFields *f, const Ice3gbSurrogateNorm *norm, uint64_t *stats,
                              void *stream);
/* ice3gb_physics_step with the surrogate-assisted rain_ice. */
int ice3gb_physics_step_surrogate(void *handle, void *mlp, int nij, int nk, double dt,
                                  const Ice3gbRainIceOptions *opt, const Ice3gbStepFields *f,
                                  const Ice3gbSurrogateNorm *norm, uint64_t *stats, void *stream);

/* ---- allocation-free rain_ice ------------------------------------------- */
/* Same computation and arguments as ice3gb_rain_ice, for callers that must
 * not allocate device memory during the call (a model that gives the GPU's
 * memory to its own pool at start-up, or runs under a device-memory cap set
 * outside the library).  Its scratch is a static device array
 * inside the library, sized for ICE3GB_NOALLOC_MAX_POINTS grid points (32 MiB:
 * a pass key and a processing-order word per point, held on every GPU that
 * loads the library, until exit); nij*nk above that is rejected with
 * ICE3GB_ERR_RANGE.  The points run in the same regime order as in
 * ice3gb_rain_ice.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress), so make it before any stream capture; a
 * cudaDeviceReset between calls is not supported.  Calls that overlap on the
 * GPU share the array and race: serialise them.  Refused with
 * ICE3GB_ERR_UNSUPPORTED before any launch (the fields are left untouched):
 * a table with SEDIM = SPLI (0), whose time-split sedimentation needs
 * 2 nij*nk doubles of stream-ordered scratch, and a table with OCND2, whose
 * level heights and droplet concentrations need as much.  No counterpart
 * exists in the reference. */
#define ICE3GB_NOALLOC_MAX_POINTS 4194304
int ice3gb_rain_ice_noalloc(void *handle, int nij, int nk, double dt, const Ice3gbRainIceOptions *opt,
                            const Ice3gbRainIceFields *f, void *stream);

/* ---- per-kernel timing -------------------------------------------------- */
/* While enabled, every kernel launch of the handle is bracketed by CUDA
 * events recorded on the caller's stream.  ice3gb_profile_read synchronises
 * those events and returns, per kernel id, the number of launches and their
 * summed device time since the last enable.  Kernel ids: 0 ice_adjust,
 * 1 sedimentation, 2 rain_ice (pointwise sub-stepping), 3 rain_ice evap3d
 * fix-up, 4 fog deposition, 5 rain_ice point ordering (regime sort),
 * 6 ice_adjust adjoint, 7 sedimentation adjoint, 8 surrogate feature
 * sampling, 9 surrogate network (all its tensor-core launches of one call),
 * 10 rain_ice with the learned slow rates, 11 rain_ice precipitation
 * fraction (PRFR options). */
#define ICE3GB_NKERNELS 12
int         ice3gb_profile_enable(void *handle, int enable);
int         ice3gb_profile_read(void *handle, int kernel_id, int *launches, double *total_ms);
const char *ice3gb_kernel_name(int kernel_id);

/* ---- host-buffer entry points (synchronous) ---------------------------- */
/* Same as above with HOST pointers, as c_ice_adjust / c_rain_ice take them:
 * host->device copies, the kernels and device->host copies all run on
 * `stream`; the call returns when the outputs are in host memory.
 * ice3gb_physics_step_host runs the step in column slabs on the handle's
 * own streams (copy-in, two compute, copy-out; ordered after the caller's
 * earlier work on `stream`), so that the copies of one slab overlap the
 * kernels of others; its outputs equal ice3gb_physics_step's bit for bit. */
int ice3gb_ice_adjust_host(void *handle, int nij, int nk, double dt,
                           const Ice3gbIceAdjustFields *f, void *stream);
int ice3gb_rain_ice_host(void *handle, int nij, int nk, double dt,
                         const Ice3gbRainIceOptions *opt,
                         const Ice3gbRainIceFields *f, void *stream);
int ice3gb_physics_step_host(void *handle, int nij, int nk, double dt, const Ice3gbRainIceOptions *opt,
                             const Ice3gbStepFields *f, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* ICE3GB_H */
