// ice3gb_kernels.h — host-side launchers of the ICE3 kernels (internal).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <cuda_bf16.h>

#include "../../include/ice3gb.h"

struct SedArgs {
  const double *rhodref, *dzz, *pabs, *tht, *sea, *town;
  double *src[5];   // rcs rrs ris rss rgs (in-out)
  double *fpr[5];   // optional flux outputs
  double *inpr[5];  // [nij] outputs
  int nij, nk;
  double dt;
  int fortran;
  double *hsrc, *hfpr, *hinpr;   // hail (NRR = 7): rhs, its flux, inprh; NULL otherwise
};

// Time-split sedimentation (SEDIM = SPLI) of a rain_ice call.
struct SplitArgs {
  SedArgs sed;                     // geometry, sources, outputs, sea/town
  const double *rt[5], *rvt, *exn; // mixing ratios at t, exner
  const double *rht;               // hail at t (NRR = 7), else NULL
  double *rvs, *ths;               // in-out (negativity correction)
  double *scratch;                 // 2 * nij * nk doubles
  unsigned int *status;            // ICE3GB_DEV_SED_CAP
  int max_iter;
};

struct FogArgs {
  const double *rct, *rhodref, *dzz;
  double *rcs, *inprc, *indep;
  int nij, enabled;
};

// Scratch words of one rain_ice call (device memory, zeroed before launch).
struct RainIceScratch {
  unsigned int *status;            // ICE3GB_DEV_* bits
  unsigned int *chunk_counter;     // dynamic work distribution
  unsigned int *key_max;           // max over points of (outer << 16 | inner)
  unsigned int *keys;              // [n] per-point pass key, 0 = not a micro point
};

struct RainIceArgs {
  Ice3gbRainIceFields f;
  const double *luts;  // Ice3gbLuts on the device
  const double *tw;    // OCND2: the TIWMX tables, else NULL
  double *ocs;         // OCND2: [2][nk][nij] level heights then droplet concentrations, else NULL
  RainIceScratch scr;
  unsigned int *order; // [n] processing order of the grid points, or NULL (index order)
  int nij, nk;
  double dt;
  int max_passes;
  int lfeedbackt;
};

// Surrogate feature sampling (surrogate_rain_ice.cu).
struct SurSampleArgs {
  Ice3gbRainIceFields f;
  const double *luts;
  int nij, nk;
  double dt;
  int norm_on;                      // standardise + envelope check
  Ice3gbSurrogateNorm norm;
  float *feat;                      // [cap][16]
  float *targets;                   // [cap][16] or NULL
  long long *point_of_row;          // [cap] or NULL
  int *row_of_point;                // [n] or NULL
  unsigned long long *count;        // rows handed out (may exceed cap)
  unsigned long long *stats;        // ICE3GB_SUR_* counters
  long cap;
};

// rain_ice with the learned slow rates.
struct SurRainIceArgs {
  RainIceArgs ri;
  const float *y;                   // network outputs, row stride ldy
  int ldy;
  const int *row_of_point;          // [n], -1: plain path
  unsigned long long *stats;
};

// ice_adjust kernel arguments: the public fields plus the optional
// "advance the state by adv_dt * sources first" extension of the chained step.
struct IaKernelFields {
  Ice3gbIceAdjustFields f;
  const double *rrs, *rss, *rgs;
  double adv_dt;
  const double *tiwmx;   // OCND2: the six TIWMX tables (6 x 24117 doubles)
};

// ice_adjust adjoint arguments; sigqsat_out receives the per-point sigqsat
// gradient ([nk][nij]: the 3-D gradient itself, or the terms of the column sum).
struct IaVjpArgs {
  Ice3gbIceAdjustFields f;
  Ice3gbIceAdjustCotangents g;
  Ice3gbIceAdjustGradients gx;
  double *sigqsat_out;
  int nij, nk;
  double dt;
};

// sedimentation adjoint arguments (the cotangent / gradient pointer sets
// mirror Ice3gbSedimentationCotangents / Ice3gbSedimentationGradients);
// flux is a [5][nk][nij] scratch for the recomputed forward fluxes.
struct SedVjpArgs {
  const double *rhodref, *dzz, *pabs, *tht, *sea, *town;
  const double *src[5];
  double *flux;
  int nij, nk;
  double dt;
  int fortran;
  struct {
    const double *src[5], *inpr[5], *fpr[5];
  } g;
  struct {
    double *src[5];
    double *rhodref, *dzz, *pabs, *tht;
  } gx;
};
cudaError_t launch_sedimentation_vjp(const Ice3gbConstants &c, const SedVjpArgs &a, cudaStream_t s);

cudaError_t launch_ice_adjust_vjp(const Ice3gbConstants &c, const IaVjpArgs &a, int num_sms, cudaStream_t s);
cudaError_t launch_column_sum(const double *in, double *out, int nij, int nk, cudaStream_t s);
// BF16 tensor-core GEMM (mlp.cu): C[m][n] = sum_k A(m, k) B(n, k) with
// A(m, k) = A[m * sam + k * sak], B(n, k) = B[n * sbn + k * sbk]; N <= 256.
enum { EPI_STORE = 0, EPI_BIAS_GELU = 1, EPI_BIAS = 2, EPI_DGELU = 3 };
struct TcGemmArgs {
  const __nv_bfloat16 *A;
  long sam, sak;
  const __nv_bfloat16 *B;
  long sbn, sbk;
  int M, N, K, k_split;
  int epi;
  float *C;                 // EPI_STORE (split partials), EPI_BIAS, EPI_DGELU (f32 dZ, optional)
  long ldc;
  const float *bias;        // EPI_BIAS_GELU, EPI_BIAS
  const float *Zin;         // EPI_DGELU
  float *Zout;              // EPI_BIAS_GELU (optional)
  long ldz;
  __nv_bfloat16 *H;         // EPI_BIAS_GELU, EPI_DGELU
  long ldh;
  int *err;
};
cudaError_t launch_tc_gemm(const TcGemmArgs &a, cudaStream_t s);
// Fused inference of the 16 -> 256 x 3 (GELU) -> n_out <= 16 MLP (mlp.cu).
struct MlpFusedArgs {
  const float *x;           // [n][16]
  float *y;                 // [n][n_out]
  long n;
  int n_out;
  const __nv_bfloat16 *w1, *w2, *w3, *w4;   // packed by launch_mlp_pack
  const float *b1, *b2, *b3, *b4;
  int *err;
};
constexpr long MLP_PACKED_ELEMS = 4096 + 65536 + 65536 + 4096;
cudaError_t launch_mlp_pack(const float *p, long w1, long w2, long w3, long w4, int n_out, __nv_bfloat16 *out,
                            cudaStream_t s);
cudaError_t launch_mlp_fused(const MlpFusedArgs &a, int num_sms, cudaStream_t s);
cudaError_t launch_sum_splits(const float *part, float *out, long n, int splits, cudaStream_t s);
cudaError_t launch_col_sum(const float *x, float *out, int rows, int cols, long ld, cudaStream_t s);
cudaError_t launch_surrogate_loss(const float *y, const float *tgt, int rows, int nrates, __nv_bfloat16 *dy, float *dyf,
                                  float *loss, cudaStream_t s);
cudaError_t launch_adam(float *w, const float *g, float *m1, float *m2, __nv_bfloat16 *w16, long n, float lr, float b1,
                        float b2, float eps, int step, cudaStream_t s);
cudaError_t launch_to_bf16(const float *x, __nv_bfloat16 *y, long n, cudaStream_t s);

// OCND2 TIWMX tables (micro/mode_ini_tiwmx.F90), filled on the host: six
// tables of 24,117 entries at T = j/100 K (ice_adjust.cu; the layout of
// ice3gb_device.cuh).
constexpr int kTiwmxTableN = 24117, kTiwmxTables = 6;
void tiwmx_tables(const Ice3gbConstants &c, double *tab);

cudaError_t launch_ice_adjust(const Ice3gbConstants &c, const IaKernelFields &kf, int nij, int nk, double dt,
                              bool vec2, int num_sms, cudaStream_t s);
cudaError_t launch_sedimentation(const Ice3gbConstants &c, const SedArgs &a, cudaStream_t s);
cudaError_t launch_fog_deposition(const Ice3gbConstants &c, const FogArgs &a, cudaStream_t s);
cudaError_t launch_rain_ice_points(const Ice3gbConstants &c, const RainIceArgs &a, int num_sms, cudaStream_t s);
cudaError_t launch_rain_ice_evap_fixup(const RainIceArgs &a, cudaStream_t s);
cudaError_t launch_rain_ice_order(const Ice3gbConstants &c, const RainIceArgs &a, cudaStream_t s);
size_t rain_ice_smem_bytes();

cudaError_t launch_sedimentation_split(const Ice3gbConstants &c, const SplitArgs &a, cudaStream_t s);
// Precipitation fraction of a rain_ice call with a PRFR option (before the point kernel).
cudaError_t launch_rain_ice_points_ts(const Ice3gbConstants &c, const RainIceArgs &a, int num_sms, cudaStream_t s);
cudaError_t launch_rain_ice_ocnd2_columns(const Ice3gbConstants &c, const RainIceArgs &a, cudaStream_t s);
cudaError_t launch_rain_ice_prfr(const Ice3gbConstants &c, const RainIceArgs &a, cudaStream_t s);
cudaError_t launch_surrogate_sample(const Ice3gbConstants &c, const SurSampleArgs &a, int num_sms, cudaStream_t s);
cudaError_t launch_rain_ice_surrogate(const Ice3gbConstants &c, const SurRainIceArgs &a, int num_sms, cudaStream_t s);
// Forward pass of an MLP handle (ice3gb_mlp_create) over n rows in chunks,
// without keeping activations; cudaErrorInvalidValue for a bad handle.
cudaError_t mlp_infer(void *mlp, long n, const float *x, float *y, cudaStream_t s);
// n_in / n_out of an MLP handle; false for a bad handle.
bool mlp_dims(void *mlp, int *n_in, int *n_out);
// 1 if a tensor-core kernel of the MLP timed out (device flag, synchronous read).
int mlp_device_error(void *mlp);
