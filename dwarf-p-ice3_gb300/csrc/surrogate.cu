// surrogate.cu — the per-point MLP (C ABI) and the slow-process surrogate.
//
// MLP: n_in -> n_hidden (GELU) x n_hidden_layers -> n_out, BF16 weights and
// activations on the tensor cores (tc_gemm_kernel, FP32 accumulation in
// TMEM), FP32 master weights, biases and Adam state.  The backward pass is
// written by hand from the same GEMM with transposed operand staging:
//   dW_l = dZ_l^T H_{l-1} (split over the batch, partials summed in a fixed
//   order), db_l = column sums of dZ_l, dZ_{l-1} = (dZ_l W_l) * GELU'(Z_{l-1}).
// Parameters are a flat FP32 vector: per layer W [out][in] then b [out].
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <random>
#include <vector>

#include "ice3gb_kernels.h"

namespace {

constexpr uint32_t kMlpMagic = 0x4D4C5033u;

struct Mlp {
  uint32_t magic = kMlpMagic;
  int n_in, n_hid, n_layers, n_out;   // n_layers hidden layers
  int nl;                             // n_layers + 1 weight layers
  std::vector<int> din, dout;         // per weight layer
  std::vector<long> woff, boff;       // offsets in the flat parameter vector
  long nparam = 0;
  float *p = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;  // [nparam]
  std::vector<__nv_bfloat16 *> w16;   // BF16 copies of W
  int *err = nullptr;
  float *loss = nullptr;
  // activation buffers for `cap` rows
  long cap = 0;
  __nv_bfloat16 *xb = nullptr, *dyb = nullptr, *dzb[2] = {nullptr, nullptr};
  std::vector<__nv_bfloat16 *> H;     // [n_layers] [cap][n_hid]
  std::vector<float *> Z;             // [n_layers] [cap][n_hid]
  float *y = nullptr, *dyf = nullptr, *dzf = nullptr, *part = nullptr;
  long part_cap = 0;
  // inference buffers for INFER_CHUNK rows (no activations kept)
  __nv_bfloat16 *xi = nullptr, *hi[2] = {nullptr, nullptr};
  // packed BF16 weights of the fused inference kernel, valid for version pk_version
  __nv_bfloat16 *wpk = nullptr;
  long version = 0, pk_version = -1;
  int num_sms = 0;
  int step = 0;
  std::mutex mu;
};

constexpr long INFER_CHUNK = 1L << 21;

Mlp *as_mlp(void *p)
{
  Mlp *m = static_cast<Mlp *>(p);
  return (m && m->magic == kMlpMagic) ? m : nullptr;
}

void free_acts(Mlp *m)
{
  cudaFree(m->xb); cudaFree(m->dyb); cudaFree(m->dzb[0]); cudaFree(m->dzb[1]);
  for (auto *h : m->H) cudaFree(h);
  for (auto *z : m->Z) cudaFree(z);
  cudaFree(m->y); cudaFree(m->dyf); cudaFree(m->dzf);
  m->H.clear(); m->Z.clear();
  m->xb = m->dyb = m->dzb[0] = m->dzb[1] = nullptr;
  m->y = m->dyf = m->dzf = nullptr;
  m->cap = 0;
}

cudaError_t ensure_acts(Mlp *m, long n)
{
  if (m->cap >= n) return cudaSuccess;
  free_acts(m);
  const long c = ((n + 127) / 128) * 128;
  cudaError_t e = cudaMalloc(&m->xb, sizeof(__nv_bfloat16) * c * m->n_in);
  if (e == cudaSuccess) e = cudaMalloc(&m->dyb, sizeof(__nv_bfloat16) * c * 16);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaMalloc(&m->dzb[i], sizeof(__nv_bfloat16) * c * m->n_hid);
  m->H.assign(m->n_layers, nullptr);
  m->Z.assign(m->n_layers, nullptr);
  for (int l = 0; l < m->n_layers && e == cudaSuccess; ++l) {
    e = cudaMalloc(&m->H[l], sizeof(__nv_bfloat16) * c * m->n_hid);
    if (e == cudaSuccess) e = cudaMalloc(&m->Z[l], sizeof(float) * c * m->n_hid);
  }
  if (e == cudaSuccess) e = cudaMalloc(&m->y, sizeof(float) * c * 16);
  if (e == cudaSuccess) e = cudaMalloc(&m->dyf, sizeof(float) * c * 16);
  if (e == cudaSuccess) e = cudaMalloc(&m->dzf, sizeof(float) * c * m->n_hid);
  if (e == cudaSuccess) m->cap = c;
  return e;
}

cudaError_t ensure_infer(Mlp *m)
{
  if (m->xi) return cudaSuccess;
  cudaError_t e = cudaMalloc(&m->xi, sizeof(__nv_bfloat16) * INFER_CHUNK * m->n_in);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaMalloc(&m->hi[i], sizeof(__nv_bfloat16) * INFER_CHUNK * m->n_hid);
  if (e != cudaSuccess) {
    cudaFree(m->xi); cudaFree(m->hi[0]); cudaFree(m->hi[1]);
    m->xi = m->hi[0] = m->hi[1] = nullptr;
  }
  return e;
}

void free_infer(Mlp *m)
{
  cudaFree(m->xi); cudaFree(m->hi[0]); cudaFree(m->hi[1]);
  m->xi = m->hi[0] = m->hi[1] = nullptr;
}

TcGemmArgs gemm(const __nv_bfloat16 *A, long sam, long sak, const __nv_bfloat16 *B, long sbn, long sbk, int M, int N,
                int K, int epi, int *err)
{
  TcGemmArgs a;
  std::memset(&a, 0, sizeof(a));
  a.A = A; a.sam = sam; a.sak = sak; a.B = B; a.sbn = sbn; a.sbk = sbk;
  a.M = M; a.N = N; a.K = K; a.k_split = 1; a.epi = epi; a.err = err;
  return a;
}

// Forward of n rows already in m->xb; keeps Z and H of the hidden layers.
cudaError_t mlp_forward_dev(Mlp *m, int n, float *y_out, long ldy, cudaStream_t s)
{
  cudaError_t e = cudaSuccess;
  const __nv_bfloat16 *in = m->xb;
  long ldin = m->n_in;
  for (int l = 0; l < m->n_layers && e == cudaSuccess; ++l) {
    TcGemmArgs a = gemm(in, ldin, 1, m->w16[l], m->din[l], 1, n, m->dout[l], m->din[l], EPI_BIAS_GELU, m->err);
    a.bias = m->p + m->boff[l];
    a.Zout = m->Z[l]; a.ldz = m->n_hid;
    a.H = m->H[l]; a.ldh = m->n_hid;
    e = launch_tc_gemm(a, s);
    in = m->H[l];
    ldin = m->n_hid;
  }
  if (e == cudaSuccess) {
    const int L = m->nl - 1;
    TcGemmArgs a = gemm(in, ldin, 1, m->w16[L], m->din[L], 1, n, m->dout[L], m->din[L], EPI_BIAS, m->err);
    a.bias = m->p + m->boff[L];
    a.C = y_out; a.ldc = ldy;
    e = launch_tc_gemm(a, s);
  }
  return e;
}

bool fused_shape(const Mlp *m) { return m->n_in == 16 && m->n_hid == 256 && m->n_layers == 3 && m->n_out <= 16; }

// Forward through the fused kernel (surrogate shape): packs the weights when
// they changed since the last pack.
cudaError_t mlp_infer_fused(Mlp *m, long n, const float *x, float *y, cudaStream_t s)
{
  cudaError_t e = cudaSuccess;
  if (!m->wpk) e = cudaMalloc(&m->wpk, sizeof(__nv_bfloat16) * MLP_PACKED_ELEMS);
  if (e == cudaSuccess && m->pk_version != m->version) {
    e = launch_mlp_pack(m->p, m->woff[0], m->woff[1], m->woff[2], m->woff[3], m->n_out, m->wpk, s);
    if (e == cudaSuccess) m->pk_version = m->version;
  }
  if (e != cudaSuccess) return e;
  MlpFusedArgs a;
  a.x = x; a.y = y; a.n = n; a.n_out = m->n_out;
  a.w1 = m->wpk; a.w2 = m->wpk + 4096; a.w3 = m->wpk + 4096 + 65536; a.w4 = m->wpk + 4096 + 131072;
  a.b1 = m->p + m->boff[0]; a.b2 = m->p + m->boff[1]; a.b3 = m->p + m->boff[2]; a.b4 = m->p + m->boff[3];
  a.err = m->err;
  return launch_mlp_fused(a, m->num_sms, s);
}

// Forward of n rows of x (f32 [n][n_in]) into y (f32 [n][n_out]) with one
// GEMM launch per layer, chunk by chunk through ping-pong BF16 activation
// buffers (any shape; the training path's forward).
cudaError_t mlp_infer_layered(Mlp *m, long n, const float *x, float *y, cudaStream_t s)
{
  cudaError_t e = ensure_infer(m);
  for (long r0 = 0; r0 < n && e == cudaSuccess; r0 += INFER_CHUNK) {
    const int rows = (int)(n - r0 < INFER_CHUNK ? n - r0 : INFER_CHUNK);
    e = launch_to_bf16(x + r0 * m->n_in, m->xi, (long)rows * m->n_in, s);
    const __nv_bfloat16 *in = m->xi;
    long ldin = m->n_in;
    for (int l = 0; l < m->n_layers && e == cudaSuccess; ++l) {
      TcGemmArgs a = gemm(in, ldin, 1, m->w16[l], m->din[l], 1, rows, m->dout[l], m->din[l], EPI_BIAS_GELU, m->err);
      a.bias = m->p + m->boff[l];
      a.H = m->hi[l & 1]; a.ldh = m->n_hid;
      e = launch_tc_gemm(a, s);
      in = m->hi[l & 1];
      ldin = m->n_hid;
    }
    if (e == cudaSuccess) {
      const int L = m->nl - 1;
      TcGemmArgs a = gemm(in, ldin, 1, m->w16[L], m->din[L], 1, rows, m->dout[L], m->din[L], EPI_BIAS, m->err);
      a.bias = m->p + m->boff[L];
      a.C = y + r0 * m->n_out; a.ldc = m->n_out;
      e = launch_tc_gemm(a, s);
    }
  }
  return e;
}

cudaError_t mlp_infer_dev(Mlp *m, long n, const float *x, float *y, cudaStream_t s)
{
  if ((((uintptr_t)x) & 15) == 0 && fused_shape(m)) return mlp_infer_fused(m, n, x, y, s);
  return mlp_infer_layered(m, n, x, y, s);
}

int split_for(int n) { int sp = n / 512; return sp < 1 ? 1 : (sp > 32 ? 32 : sp); }

cudaError_t ensure_part(Mlp *m, long words)
{
  if (m->part_cap >= words) return cudaSuccess;
  cudaFree(m->part);
  m->part = nullptr;
  m->part_cap = 0;
  cudaError_t e = cudaMalloc(&m->part, sizeof(float) * words);
  if (e == cudaSuccess) m->part_cap = words;
  return e;
}

// dW (dout x din) = dZ^T (dout x n) * X (n x din), split over n, into g.
cudaError_t weight_grad(Mlp *m, const __nv_bfloat16 *dz, long lddz, const __nv_bfloat16 *x, long ldx, int n, int dout,
                        int din, float *gw, cudaStream_t s)
{
  const int sp = split_for(n);
  cudaError_t e = ensure_part(m, (long)sp * dout * din);
  if (e != cudaSuccess) return e;
  TcGemmArgs a = gemm(dz, 1, lddz, x, 1, ldx, dout, din, n, EPI_STORE, m->err);
  a.k_split = sp;
  a.C = m->part; a.ldc = din;
  e = launch_tc_gemm(a, s);
  if (e == cudaSuccess) e = launch_sum_splits(m->part, gw, (long)dout * din, sp, s);
  return e;
}

// Loss and gradient (into m->g) of n rows: x (device f32 [n][n_in]), tgt [n][16].
cudaError_t mlp_loss_grad(Mlp *m, int n, const float *x, const float *tgt, cudaStream_t s)
{
  cudaError_t e = ensure_acts(m, n);
  if (e == cudaSuccess) e = launch_to_bf16(x, m->xb, (long)n * m->n_in, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->loss, 0, sizeof(float), s);
  if (e == cudaSuccess) e = mlp_forward_dev(m, n, m->y, 16, s);
  if (e == cudaSuccess) e = launch_surrogate_loss(m->y, tgt, n, m->n_out / 2, m->dyb, m->dyf, m->loss, s);
  if (e != cudaSuccess) return e;
  // output layer: dW = dY^T H_last, db = column sums of dY
  const int L = m->nl - 1;
  e = weight_grad(m, m->dyb, 16, m->H[m->n_layers - 1], m->n_hid, n, m->dout[L], m->din[L], m->g + m->woff[L], s);
  if (e == cudaSuccess) e = launch_col_sum(m->dyf, m->g + m->boff[L], n, m->dout[L], 16, s);
  if (e != cudaSuccess) return e;
  int cur = 0;
  const __nv_bfloat16 *dnext = m->dyb;
  long ldnext = 16;
  for (int l = m->n_layers - 1; l >= 0 && e == cudaSuccess; --l) {
    // dZ_l = (dZ_{l+1} W_{l+1}) * GELU'(Z_l)
    const int lw = l + 1;  // weight layer consuming H_l
    TcGemmArgs a = gemm(dnext, ldnext, 1, m->w16[lw], 1, m->din[lw], n, m->dout[l], m->dout[lw], EPI_DGELU, m->err);
    a.Zin = m->Z[l]; a.ldz = m->n_hid;
    a.H = m->dzb[cur]; a.ldh = m->n_hid;
    a.C = m->dzf; a.ldc = m->n_hid;
    e = launch_tc_gemm(a, s);
    if (e == cudaSuccess) e = launch_col_sum(m->dzf, m->g + m->boff[l], n, m->dout[l], m->n_hid, s);
    const __nv_bfloat16 *xin = l > 0 ? m->H[l - 1] : m->xb;
    const long ldx = l > 0 ? m->n_hid : m->n_in;
    if (e == cudaSuccess) e = weight_grad(m, m->dzb[cur], m->n_hid, xin, ldx, n, m->dout[l], m->din[l], m->g + m->woff[l], s);
    dnext = m->dzb[cur];
    ldnext = m->n_hid;
    cur ^= 1;
  }
  return e;
}

}  // namespace

cudaError_t mlp_infer(void *mlp, long n, const float *x, float *y, cudaStream_t s)
{
  Mlp *m = as_mlp(mlp);
  if (!m || n < 0) return cudaErrorInvalidValue;
  std::lock_guard<std::mutex> lock(m->mu);
  return mlp_infer_dev(m, n, x, y, s);
}

bool mlp_dims(void *mlp, int *n_in, int *n_out)
{
  Mlp *m = as_mlp(mlp);
  if (!m) return false;
  *n_in = m->n_in;
  *n_out = m->n_out;
  return true;
}

int mlp_device_error(void *mlp)
{
  Mlp *m = as_mlp(mlp);
  int err = 0;
  if (!m || cudaMemcpy(&err, m->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
  return err != 0;
}

extern "C" {

int ice3gb_mlp_create(const Ice3gbMlpShape *shape, uint64_t seed, void **out)
{
  if (!shape || !out) return ICE3GB_ERR_NULL;
  *out = nullptr;
  if (shape->n_in < 1 || shape->n_in > 256 || shape->n_hidden < 16 || shape->n_hidden > 256 ||
      shape->n_hidden_layers < 1 || shape->n_hidden_layers > 8 || shape->n_out < 2 || shape->n_out > 16 ||
      (shape->n_out % 2) != 0)
    return ICE3GB_ERR_RANGE;
  Mlp *m = new Mlp();
  m->n_in = shape->n_in; m->n_hid = shape->n_hidden; m->n_layers = shape->n_hidden_layers; m->n_out = shape->n_out;
  m->nl = m->n_layers + 1;
  long off = 0;
  for (int l = 0; l < m->nl; ++l) {
    const int din = l == 0 ? m->n_in : m->n_hid;
    const int dout = l == m->nl - 1 ? m->n_out : m->n_hid;
    m->din.push_back(din);
    m->dout.push_back(dout);
    m->woff.push_back(off);
    off += (long)din * dout;
    m->boff.push_back(off);
    off += dout;
  }
  m->nparam = off;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || m->num_sms < 1)
    m->num_sms = 1;
  // He-normal hidden weights, scaled-down output weights, zero biases
  std::vector<float> host(off, 0.0f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < m->nl; ++l) {
    const float sd = (l == m->nl - 1 ? 0.5f : 1.0f) * std::sqrt(2.0f / (float)m->din[l]);
    std::normal_distribution<float> nd(0.0f, sd);
    for (long i = 0; i < (long)m->din[l] * m->dout[l]; ++i) host[m->woff[l] + i] = nd(rng);
  }
  cudaError_t e = cudaMalloc(&m->p, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMalloc(&m->g, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMalloc(&m->m1, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMalloc(&m->m2, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMalloc(&m->err, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&m->loss, sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(m->p, host.data(), sizeof(float) * off, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->m1, 0, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMemset(m->m2, 0, sizeof(float) * off);
  if (e == cudaSuccess) e = cudaMemset(m->err, 0, sizeof(int));
  m->w16.assign(m->nl, nullptr);
  for (int l = 0; l < m->nl && e == cudaSuccess; ++l) {
    e = cudaMalloc(&m->w16[l], sizeof(__nv_bfloat16) * (size_t)m->din[l] * m->dout[l]);
    if (e == cudaSuccess) e = launch_to_bf16(m->p + m->woff[l], m->w16[l], (long)m->din[l] * m->dout[l], nullptr);
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    free_acts(m);
    cudaFree(m->p); cudaFree(m->g); cudaFree(m->m1); cudaFree(m->m2); cudaFree(m->err); cudaFree(m->loss);
    for (auto *w : m->w16) cudaFree(w);
    delete m;
    return ICE3GB_ERR_CUDA;
  }
  *out = m;
  return ICE3GB_OK;
}

int ice3gb_mlp_destroy(void *mlp)
{
  Mlp *m = as_mlp(mlp);
  if (!m) return ICE3GB_ERR_HANDLE;
  free_acts(m);
  free_infer(m);
  cudaFree(m->wpk);
  cudaFree(m->p); cudaFree(m->g); cudaFree(m->m1); cudaFree(m->m2); cudaFree(m->err); cudaFree(m->loss);
  cudaFree(m->part);
  for (auto *w : m->w16) cudaFree(w);
  m->magic = 0;
  delete m;
  return ICE3GB_OK;
}

int64_t ice3gb_mlp_param_count(void *mlp)
{
  Mlp *m = as_mlp(mlp);
  return m ? m->nparam : ICE3GB_ERR_HANDLE;
}

int ice3gb_mlp_get_params(void *mlp, float *host)
{
  Mlp *m = as_mlp(mlp);
  if (!m) return ICE3GB_ERR_HANDLE;
  if (!host) return ICE3GB_ERR_NULL;
  return cudaMemcpy(host, m->p, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost) == cudaSuccess ? ICE3GB_OK
                                                                                                  : ICE3GB_ERR_CUDA;
}

int ice3gb_mlp_set_params(void *mlp, const float *host)
{
  Mlp *m = as_mlp(mlp);
  if (!m) return ICE3GB_ERR_HANDLE;
  if (!host) return ICE3GB_ERR_NULL;
  cudaError_t e = cudaMemcpy(m->p, host, sizeof(float) * m->nparam, cudaMemcpyHostToDevice);
  for (int l = 0; l < m->nl && e == cudaSuccess; ++l)
    e = launch_to_bf16(m->p + m->woff[l], m->w16[l], (long)m->din[l] * m->dout[l], nullptr);
  if (e == cudaSuccess) e = cudaMemset(m->m1, 0, sizeof(float) * m->nparam);
  if (e == cudaSuccess) e = cudaMemset(m->m2, 0, sizeof(float) * m->nparam);
  m->step = 0;
  m->version += 1;
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return e == cudaSuccess ? ICE3GB_OK : ICE3GB_ERR_CUDA;
}

int ice3gb_mlp_forward(void *mlp, int n, const float *x, float *y, void *stream)
{
  Mlp *m = as_mlp(mlp);
  if (!m) return ICE3GB_ERR_HANDLE;
  if (!x || !y) return ICE3GB_ERR_NULL;
  if (n < 1) return ICE3GB_ERR_SHAPE;
  std::lock_guard<std::mutex> lock(m->mu);
  return mlp_infer_dev(m, n, x, y, static_cast<cudaStream_t>(stream)) == cudaSuccess ? ICE3GB_OK : ICE3GB_ERR_CUDA;
}

int ice3gb_mlp_forward_layered(void *mlp, int n, const float *x, float *y, void *stream)
{
  Mlp *m = as_mlp(mlp);
  if (!m) return ICE3GB_ERR_HANDLE;
  if (!x || !y) return ICE3GB_ERR_NULL;
  if (n < 1) return ICE3GB_ERR_SHAPE;
  std::lock_guard<std::mutex> lock(m->mu);
  return mlp_infer_layered(m, n, x, y, static_cast<cudaStream_t>(stream)) == cudaSuccess ? ICE3GB_OK
                                                                                           : ICE3GB_ERR_CUDA;
}

int ice3gb_mlp_loss_grad(void *mlp, int n, const float *x, const float *tgt, float *grad, float *loss, void *stream)
{
  Mlp *m = as_mlp(mlp);
  if (!m) return ICE3GB_ERR_HANDLE;
  if (!x || !tgt) return ICE3GB_ERR_NULL;
  if (n < 1) return ICE3GB_ERR_SHAPE;
  std::lock_guard<std::mutex> lock(m->mu);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = mlp_loss_grad(m, n, x, tgt, s);
  if (e == cudaSuccess && grad) e = cudaMemcpyAsync(grad, m->g, sizeof(float) * m->nparam, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToDevice, s);
  return e == cudaSuccess ? ICE3GB_OK : ICE3GB_ERR_CUDA;
}

int ice3gb_mlp_train_step(void *mlp, int n, const float *x, const float *tgt, float lr, float *loss, void *stream)
{
  Mlp *m = as_mlp(mlp);
  if (!m) return ICE3GB_ERR_HANDLE;
  if (!x || !tgt) return ICE3GB_ERR_NULL;
  if (n < 1) return ICE3GB_ERR_SHAPE;
  std::lock_guard<std::mutex> lock(m->mu);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = mlp_loss_grad(m, n, x, tgt, s);
  m->step += 1;
  m->version += 1;
  for (int l = 0; l < m->nl && e == cudaSuccess; ++l) {
    const long nw = (long)m->din[l] * m->dout[l];
    e = launch_adam(m->p + m->woff[l], m->g + m->woff[l], m->m1 + m->woff[l], m->m2 + m->woff[l], m->w16[l], nw, lr,
                    0.9f, 0.999f, 1e-8f, m->step, s);
    if (e == cudaSuccess)
      e = launch_adam(m->p + m->boff[l], m->g + m->boff[l], m->m1 + m->boff[l], m->m2 + m->boff[l], nullptr,
                      m->dout[l], lr, 0.9f, 0.999f, 1e-8f, m->step, s);
  }
  if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToDevice, s);
  return e == cudaSuccess ? ICE3GB_OK : ICE3GB_ERR_CUDA;
}

int ice3gb_mlp_error(void *mlp)
{
  Mlp *m = as_mlp(mlp);
  if (!m) return ICE3GB_ERR_HANDLE;
  int err = 0;
  if (cudaMemcpy(&err, m->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return ICE3GB_ERR_CUDA;
  return err ? ICE3GB_ERR_DEVICE : ICE3GB_OK;
}

int ice3gb_tc_gemm_bf16(int M, int N, int K, const void *A, int64_t sam, int64_t sak, const void *B, int64_t sbn,
                        int64_t sbk, float *C, int64_t ldc, int *err, void *stream)
{
  if (!A || !B || !C || !err) return ICE3GB_ERR_NULL;
  if (M < 1 || N < 1 || N > 256 || K < 1) return ICE3GB_ERR_SHAPE;
  TcGemmArgs a;
  std::memset(&a, 0, sizeof(a));
  a.A = static_cast<const __nv_bfloat16 *>(A); a.sam = sam; a.sak = sak;
  a.B = static_cast<const __nv_bfloat16 *>(B); a.sbn = sbn; a.sbk = sbk;
  a.M = M; a.N = N; a.K = K; a.k_split = 1; a.epi = EPI_STORE; a.C = C; a.ldc = ldc; a.err = err;
  return launch_tc_gemm(a, static_cast<cudaStream_t>(stream)) == cudaSuccess ? ICE3GB_OK : ICE3GB_ERR_CUDA;
}

}  // extern "C"
