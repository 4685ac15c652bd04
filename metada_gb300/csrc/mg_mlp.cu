// Learned column observation operator.
//
// The plain operator maps a column of nlev temperatures T_l (K) and specific
// humidities q_l to nch channel values
//     y_c = sum_l w[c,l] exp(-tau_c sum_{m<=l} q_m) T_l^4 / 1e8
// (CUDA expf).  The surrogate is an MLP nin -> nh -> nh -> nout with SiLU,
// BF16 weights and FP32 accumulation, trained by Adam on columns the plain
// operator labels.  Everything here is hand-written CUDA: the column kernels,
// the three GEMM shapes of forward and backward propagation, the activation
// and bias-gradient epilogues, the loss, and Adam.
//
// Column features for the MLP: [(T_l - 255)/30 for l < nlev,
// 100 q_l for l < nlev, 0 ... 0] padded to nin (the operator depends on q
// through its running sum, so q enters linearly); outputs are
// standardised per channel (y - out_shift)/out_scale.
#include <cuda_bf16.h>

#include <cub/device/device_radix_sort.cuh>

#include <memory>
#include <vector>

#include "mg_internal.h"

struct mg_mlp {
  int nin = 0, nh = 0, nout = 0;
  int64_t nparam = 0;
  // FP32 master parameters, Adam moments, gradients, BF16 working weights.
  float* master = nullptr;
  float* m1 = nullptr;
  float* m2 = nullptr;
  float* grad = nullptr;
  __nv_bfloat16* wbf = nullptr;
  float* out_shift = nullptr;
  float* out_scale = nullptr;
  int64_t step = 0;
  // activations for a batch of up to cap rows
  int64_t cap = 0;
  float* Z1 = nullptr;
  float* H1 = nullptr;
  float* Z2 = nullptr;
  float* H2 = nullptr;
  float* Y = nullptr;
  float* dY = nullptr;
  float* dA = nullptr;  // nh-wide scratch
  float* dB = nullptr;
  float* loss = nullptr;
  // BF16 activations of the tensor-core inference path, up to tc_cap rows,
  // and its error flag (a bounded wait that gave up).
  int64_t tc_cap = 0;
  __nv_bfloat16* Xb = nullptr;
  __nv_bfloat16* H1b = nullptr;
  __nv_bfloat16* H2b = nullptr;
  int* tc_err = nullptr;
  // parameter offsets: W1 (nh x nin), b1, W2 (nh x nh), b2, W3 (nout x nh), b3
  int64_t oW1 = 0, ob1 = 0, oW2 = 0, ob2 = 0, oW3 = 0, ob3 = 0;
};

namespace {

constexpr int kThreads = 256;
constexpr int BM = 64, BN = 64, BK = 16;

__device__ __forceinline__ float sigmoidf_(float z) { return 1.0f / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigmoidf_(z); }
__device__ __forceinline__ float silu_grad(float z) {
  const float s = sigmoidf_(z);
  return s * (1.0f + z * (1.0f - s));
}

template <typename T>
__device__ __forceinline__ float ld(const T* p) { return static_cast<float>(*p); }
template <>
__device__ __forceinline__ float ld<__nv_bfloat16>(const __nv_bfloat16* p) { return __bfloat162float(*p); }

// C[m, n] = sum_k opA(m, k) opB(k, n) with
//   opA(m, k) = TA ? A[k*lda + m] : A[m*lda + k]
//   opB(k, n) = TB ? B[k*ldb + n] : B[n*ldb + k]
// then epi(m, n, acc).  64 x 64 tiles, 16-deep K steps, 4 x 4 per thread.
template <bool TA, bool TB, typename TAe, typename TBe, typename Epi>
__global__ void __launch_bounds__(kThreads) gemm_kernel(int M, int N, int K, const TAe* __restrict__ A, int lda,
                                                        const TBe* __restrict__ B, int ldb, Epi epi) {
  __shared__ float As[BK][BM + 4];
  __shared__ float Bs[BK][BN + 4];
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int e = tid; e < BM * BK; e += kThreads) {
      int m, k;
      if (TA) { m = e % BM; k = e / BM; } else { k = e % BK; m = e / BK; }
      const int gm = m0 + m, gk = k0 + k;
      As[k][m] = (gm < M && gk < K) ? ld(TA ? &A[(int64_t)gk * lda + gm] : &A[(int64_t)gm * lda + gk]) : 0.0f;
    }
    for (int e = tid; e < BN * BK; e += kThreads) {
      int n, k;
      if (TB) { n = e % BN; k = e / BN; } else { k = e % BK; n = e / BK; }
      const int gn = n0 + n, gk = k0 + k;
      Bs[k][n] = (gn < N && gk < K) ? ld(TB ? &B[(int64_t)gk * ldb + gn] : &B[(int64_t)gn * ldb + gk]) : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
      if (m < M && n < N) epi(m, n, acc[i][j]);
    }
}

// Epilogues.
struct EpiBiasSilu {  // Z = acc + b, H = SiLU(Z)
  const float* b;
  float* Z;
  float* H;
  int ld;
  __device__ void operator()(int m, int n, float acc) const {
    const float z = acc + b[n];
    Z[(int64_t)m * ld + n] = z;
    H[(int64_t)m * ld + n] = silu(z);
  }
};
struct EpiBias {  // Y = acc + b
  const float* b;
  float* Y;
  int ld;
  __device__ void operator()(int m, int n, float acc) const { Y[(int64_t)m * ld + n] = acc + b[n]; }
};
struct EpiSiluGrad {  // dZ = acc * SiLU'(Z)
  const float* Z;
  float* dZ;
  int ld;
  __device__ void operator()(int m, int n, float acc) const {
    dZ[(int64_t)m * ld + n] = acc * silu_grad(Z[(int64_t)m * ld + n]);
  }
};
struct EpiStore {  // G = acc
  float* G;
  int ld;
  __device__ void operator()(int m, int n, float acc) const { G[(int64_t)m * ld + n] = acc; }
};

template <bool TA, bool TB, typename TAe, typename TBe, typename Epi>
cudaError_t gemm(cudaStream_t s, int M, int N, int K, const TAe* A, int lda, const TBe* B, int ldb, Epi epi) {
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
  gemm_kernel<TA, TB, TAe, TBe, Epi><<<grid, kThreads, 0, s>>>(M, N, K, A, lda, B, ldb, epi);
  MG_COUNT_LAUNCH();
  return cudaGetLastError();
}

// Column sums of a B x N matrix into out (bias gradients).
__global__ void colsum_kernel(const float* __restrict__ D, int64_t B, int N, float* __restrict__ out) {
  const int n = blockIdx.x;
  float s = 0.0f;
  for (int64_t b = threadIdx.x; b < B; b += blockDim.x) s += D[b * N + n];
  __shared__ float red[kThreads];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = red[0];
}

// dY = 2 (Y - (Yt - shift)/scale) / (B nout); loss += sum of squares.
__global__ void loss_grad_kernel(const float* __restrict__ Y, const float* __restrict__ Yt, int64_t B, int nout,
                                 const float* __restrict__ shift, const float* __restrict__ scale,
                                 float* __restrict__ dY, float* __restrict__ loss) {
  const int64_t total = B * nout;
  float acc = 0.0f;
  const float inv = 2.0f / (float)total;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e % nout);
    const float t = (Yt[e] - shift[c]) / scale[c];
    const float r = Y[e] - t;
    dY[e] = inv * r;
    acc += r * r;
  }
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

__global__ void adam_kernel(float* __restrict__ w, float* __restrict__ m1, float* __restrict__ m2,
                            const float* __restrict__ g, int64_t n, float lr, float b1, float b2, float eps,
                            float c1, float c2, __nv_bfloat16* __restrict__ wbf) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.0f - b1) * gi;
    const float v = b2 * m2[i] + (1.0f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = v;
    const float wi = w[i] - lr * (a / c1) / (sqrtf(v / c2) + eps);
    w[i] = wi;
    wbf[i] = __float2bfloat16_rn(wi);
  }
}

__global__ void to_bf16_kernel(const float* __restrict__ w, int64_t n, __nv_bfloat16* __restrict__ wbf) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    wbf[i] = __float2bfloat16_rn(w[i]);
}

__global__ void bf16_to_float_kernel(const __nv_bfloat16* __restrict__ wbf, int64_t n, float* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = __bfloat162float(wbf[i]);
}

// Plain column operator: one thread per column.
__global__ void column_op_kernel(const float* __restrict__ T, const float* __restrict__ q, int64_t ncol, int nlev,
                                 const float* __restrict__ w, const float* __restrict__ tau, int nch,
                                 float* __restrict__ y) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncol; c += (int64_t)gridDim.x * blockDim.x) {
    float acc[32];
    for (int ch = 0; ch < nch; ++ch) acc[ch] = 0.0f;
    float Q = 0.0f;
    for (int l = 0; l < nlev; ++l) {
      Q += q[c * nlev + l];
      const float t = T[c * nlev + l];
      const float t4 = (t * t) * (t * t) / 1e8f;
      for (int ch = 0; ch < nch; ++ch) acc[ch] += w[ch * nlev + l] * expf(-tau[ch] * Q) * t4;
    }
    for (int ch = 0; ch < nch; ++ch) y[c * nch + ch] = acc[ch];
  }
}

// Column features (see file comment) from T and q columns.
__global__ void column_features_kernel(const float* __restrict__ T, const float* __restrict__ q, int64_t ncol,
                                       int nlev, int nin, float* __restrict__ X) {
  const int64_t total = ncol * nin;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = e / nin;
    const int f = (int)(e - c * nin);
    float v = 0.0f;
    if (f < nlev) v = (T[c * nlev + f] - 255.0f) / 30.0f;
    else if (f < 2 * nlev) v = 100.0f * q[c * nlev + f - nlev];
    X[e] = v;
  }
}

// Column obs on a member-major state laid out ((v*nlev + l)*ncol + col),
// v = 0: T (K), v = 1: ln q.  One thread per (obs, member): the column of
// member i at obs o, either labelled by the plain operator (channel obs_ch[o]
// into HX) or turned into MLP features (row o*k + i of X).
// Obs in column order: keys = obs_col (as 32-bit), values = obs index.
__global__ void obs_sort_keys_kernel(const int64_t* __restrict__ obs_col, int64_t p, uint32_t* __restrict__ keys,
                                     int32_t* __restrict__ vals) {
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < p; o += (int64_t)gridDim.x * blockDim.x) {
    keys[o] = (uint32_t)obs_col[o];
    vals[o] = (int32_t)o;
  }
}

// One thread per (member, obs) of a slice of p obs taken in column order
// (perm: slice rank -> obs index): consecutive threads read the same member
// at neighbouring columns, so a warp's loads share sectors (a thread per
// (obs, member) in obs order read one 32-byte sector per value).  The plain
// operator writes HX[o k + i]; the feature rows are slice-local in thread
// order (row i p + r), so a warp writes neighbouring rows.
__global__ void hx_column_kernel(const double* __restrict__ Xs, int k, int64_t ld, int64_t ncol, int nlev,
                                 const int64_t* __restrict__ obs_col, const int32_t* __restrict__ obs_ch,
                                 int64_t p, const int32_t* __restrict__ perm, const float* __restrict__ w,
                                 const float* __restrict__ tau, double* __restrict__ HX, float* __restrict__ feat,
                                 int nin, __nv_bfloat16* __restrict__ featb = nullptr) {
  const int64_t total = p * k;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / p);
    const int64_t r = e - (int64_t)i * p;
    const int64_t o = perm[r];
    const double* x = Xs + (int64_t)i * ld + obs_col[o];
    if (HX) {
      const int ch = obs_ch[o];
      float Q = 0.0f, acc = 0.0f;
      for (int l = 0; l < nlev; ++l) {
        const float t = (float)x[(int64_t)l * ncol];
        Q += expf((float)x[(int64_t)(nlev + l) * ncol]);
        acc += w[ch * nlev + l] * expf(-tau[ch] * Q) * ((t * t) * (t * t) / 1e8f);
      }
      HX[o * k + i] = acc;
    } else if (featb) {
      // the row in registers, written as 16-byte chunks (nin % 8 == 0 here)
      __nv_bfloat16* f = featb + e * nin;
      for (int c0 = 0; c0 < nin; c0 += 8) {
        __align__(16) __nv_bfloat16 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int j = c0 + u;
          float val = 0.0f;
          if (j < nlev)
            val = ((float)x[(int64_t)j * ncol] - 255.0f) / 30.0f;
          else if (j < 2 * nlev)
            val = 100.0f * expf((float)x[(int64_t)j * ncol]);
          v[u] = __float2bfloat16_rn(val);
        }
        *reinterpret_cast<uint4*>(f + c0) = *reinterpret_cast<const uint4*>(v);
      }
    } else {
      float* f = feat + e * nin;
      for (int l = 0; l < nlev; ++l) {
        f[l] = ((float)x[(int64_t)l * ncol] - 255.0f) / 30.0f;
        f[nlev + l] = 100.0f * expf((float)x[(int64_t)(nlev + l) * ncol]);
      }
      for (int j = 2 * nlev; j < nin; ++j) f[j] = 0.0f;
    }
  }
}

// HX[o k + i] = Y[(i p + r) nout + obs_ch[o]] * scale + shift (de-standardise),
// o = perm[r], for the slice's network output rows (feature row order).
__global__ void pick_channel_kernel(const float* __restrict__ Y, int64_t p, int k, int nout,
                                    const int32_t* __restrict__ perm, const int32_t* __restrict__ obs_ch,
                                    const float* __restrict__ shift, const float* __restrict__ scale,
                                    double* __restrict__ HX) {
  const int64_t total = p * k;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / p, r = e - i * p, o = perm[r];
    const int ch = obs_ch[o];
    HX[o * k + i] = (double)(Y[e * nout + ch] * scale[ch] + shift[ch]);
  }
}

inline unsigned grid_for(int64_t n, int threads = kThreads) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return (unsigned)b;
}

int ensure_capacity(mg_context* ctx, mg_mlp* m, int64_t B) {
  if (B <= m->cap) return MG_OK;
  float* bufs[] = {m->Z1, m->H1, m->Z2, m->H2, m->Y, m->dY, m->dA, m->dB};
  for (float* p : bufs)
    if (p) cudaFree(p);
  const int64_t hw = (int64_t)B * m->nh, ow = (int64_t)B * m->nout;
  float** targets[] = {&m->Z1, &m->H1, &m->Z2, &m->H2, &m->dA, &m->dB};
  for (float** t : targets) {
    if (cudaMalloc(t, sizeof(float) * hw) != cudaSuccess) {
      cudaGetLastError();
      return mg::fail(ctx, MG_ERR_NOMEM, "mg_mlp: activation allocation failed");
    }
  }
  if (cudaMalloc(&m->Y, sizeof(float) * ow) != cudaSuccess || cudaMalloc(&m->dY, sizeof(float) * ow) != cudaSuccess) {
    cudaGetLastError();
    return mg::fail(ctx, MG_ERR_NOMEM, "mg_mlp: activation allocation failed");
  }
  m->cap = B;
  return MG_OK;
}

// Forward pass on a batch (bf16 weights, FP32 accumulation): fills Z1, H1,
// Z2, H2 and Y (standardised outputs).
int forward(mg_context* ctx, mg_mlp* m, const float* X, int64_t B) {
  cudaStream_t s = ctx->stream;
  const __nv_bfloat16* W = m->wbf;
  const float* P = m->master;
  const int nin = m->nin, nh = m->nh, no = m->nout;
  MG_TRY_CUDA((gemm<false, false>(s, (int)B, nh, nin, X, nin, W + m->oW1, nin, EpiBiasSilu{P + m->ob1, m->Z1, m->H1, nh})));
  MG_TRY_CUDA((gemm<false, false>(s, (int)B, nh, nh, m->H1, nh, W + m->oW2, nh, EpiBiasSilu{P + m->ob2, m->Z2, m->H2, nh})));
  MG_TRY_CUDA((gemm<false, false>(s, (int)B, no, nh, m->H2, nh, W + m->oW3, nh, EpiBias{P + m->ob3, m->Y, no})));
  return MG_OK;
}

// The tensor-core inference path needs K (nin, nh) a multiple of 8 and
// N (nh, nout) at most 256; those sizes also keep every weight block of the
// BF16 parameter vector 16-byte aligned.
bool tc_shapes_ok(const mg_mlp* m) { return m->nin % 8 == 0 && m->nh % 8 == 0 && m->nh <= 256 && m->nout <= 256; }

int ensure_tc_capacity(mg_context* ctx, mg_mlp* m, int64_t B) {
  if (B <= m->tc_cap) return MG_OK;
  void* old[] = {m->Xb, m->H1b, m->H2b};
  for (void* p : old)
    if (p) cudaFree(p);
  m->Xb = m->H1b = m->H2b = nullptr;
  m->tc_cap = 0;
  if (cudaMalloc(&m->Xb, sizeof(__nv_bfloat16) * B * m->nin) != cudaSuccess ||
      cudaMalloc(&m->H1b, sizeof(__nv_bfloat16) * B * m->nh) != cudaSuccess ||
      cudaMalloc(&m->H2b, sizeof(__nv_bfloat16) * B * m->nh) != cudaSuccess ||
      (!m->tc_err && cudaMalloc(&m->tc_err, sizeof(int)) != cudaSuccess)) {
    cudaGetLastError();
    return mg::fail(ctx, MG_ERR_NOMEM, "mg_mlp: activation allocation failed");
  }
  m->tc_cap = B;
  return MG_OK;
}

// Inference on the tensor cores: m->Xb (B x nin, BF16) -> m->Y (B x nout,
// standardised, FP32); hidden activations are rounded to BF16 between layers.
int forward_tc(mg_context* ctx, mg_mlp* m, int64_t B) {
  const __nv_bfloat16* W = m->wbf;
  const float* P = m->master;
  const int Bi = (int)B, nin = m->nin, nh = m->nh, no = m->nout;
  int rc;
  if ((rc = mg::tc_gemm_bf16(ctx, m->Xb, W + m->oW1, Bi, nh, nin, P + m->ob1, 1, nullptr, m->H1b, nh, m->tc_err)))
    return rc;
  if ((rc = mg::tc_gemm_bf16(ctx, m->H1b, W + m->oW2, Bi, nh, nh, P + m->ob2, 1, nullptr, m->H2b, nh, m->tc_err)))
    return rc;
  return mg::tc_gemm_bf16(ctx, m->H2b, W + m->oW3, Bi, no, nh, P + m->ob3, 0, m->Y, nullptr, no, m->tc_err);
}

// Gradients of the mean squared (standardised) error into m->grad.
int backward(mg_context* ctx, mg_mlp* m, const float* X, const float* Yt, int64_t B) {
  cudaStream_t s = ctx->stream;
  const __nv_bfloat16* W = m->wbf;
  float* G = m->grad;
  const int nin = m->nin, nh = m->nh, no = m->nout;
  MG_TRY_CUDA(cudaMemsetAsync(m->loss, 0, sizeof(float), s));
  loss_grad_kernel<<<grid_for(B * no), kThreads, 0, s>>>(m->Y, Yt, B, no, m->out_shift, m->out_scale, m->dY, m->loss);
  MG_COUNT_LAUNCH();
  // layer 3: dW3 = dY^T H2, db3 = colsum dY, dH2 = dY W3 (then * SiLU'(Z2))
  MG_TRY_CUDA((gemm<true, true>(s, no, nh, (int)B, m->dY, no, m->H2, nh, EpiStore{G + m->oW3, nh})));
  colsum_kernel<<<no, kThreads, 0, s>>>(m->dY, B, no, G + m->ob3);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA((gemm<false, true>(s, (int)B, nh, no, m->dY, no, W + m->oW3, nh, EpiSiluGrad{m->Z2, m->dA, nh})));
  // layer 2
  MG_TRY_CUDA((gemm<true, true>(s, nh, nh, (int)B, m->dA, nh, m->H1, nh, EpiStore{G + m->oW2, nh})));
  colsum_kernel<<<nh, kThreads, 0, s>>>(m->dA, B, nh, G + m->ob2);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA((gemm<false, true>(s, (int)B, nh, nh, m->dA, nh, W + m->oW2, nh, EpiSiluGrad{m->Z1, m->dB, nh})));
  // layer 1
  MG_TRY_CUDA((gemm<true, true>(s, nh, nin, (int)B, m->dB, nh, X, nin, EpiStore{G + m->oW1, nin})));
  colsum_kernel<<<nh, kThreads, 0, s>>>(m->dB, B, nh, G + m->ob1);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

// perm[r] = the obs at rank r in column order (CUB radix sort on the
// column index); tmp is column_sort_bytes(p) bytes of device workspace.
size_t column_sort_bytes(int64_t p) {
  size_t b = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, b, (const uint32_t*)nullptr, (uint32_t*)nullptr, (const int32_t*)nullptr,
                                  (int32_t*)nullptr, (int)p);
  return b + 256 + 2 * sizeof(uint32_t) * (size_t)p + sizeof(int32_t) * (size_t)p + 1024;
}

cudaError_t sort_obs_by_column(const int64_t* obs_col, int64_t p, int32_t* perm, void* tmp, cudaStream_t s) {
  char* t = static_cast<char*>(tmp);
  auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
  uint32_t* keys = reinterpret_cast<uint32_t*>(t);
  uint32_t* keys_out = reinterpret_cast<uint32_t*>(t + align(sizeof(uint32_t) * p));
  int32_t* vals = reinterpret_cast<int32_t*>(t + 2 * align(sizeof(uint32_t) * p));
  void* sort_tmp = t + 2 * align(sizeof(uint32_t) * p) + align(sizeof(int32_t) * p);
  size_t sb = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, sb, (const uint32_t*)nullptr, (uint32_t*)nullptr, (const int32_t*)nullptr,
                                  (int32_t*)nullptr, (int)p);
  obs_sort_keys_kernel<<<grid_for(p), kThreads, 0, s>>>(obs_col, p, keys, vals);
  MG_COUNT_LAUNCH();
  return cub::DeviceRadixSort::SortPairs(sort_tmp, sb, keys, keys_out, vals, perm, (int)p, 0, 32, s);
}

}  // namespace

extern "C" {

int mg_column_op(mg_context* ctx, const float* T, const float* q, int64_t ncol, int32_t nlev, const float* w,
                 const float* tau, int32_t nch, float* y) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(T && q && w && tau && y && ncol >= 0 && nlev > 0 && nch > 0 && nch <= 32,
               "mg_column_op: bad arguments (nch <= 32)");
  if (ncol == 0) return MG_OK;
  column_op_kernel<<<grid_for(ncol), kThreads, 0, ctx->stream>>>(T, q, ncol, nlev, w, tau, nch, y);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

int mg_column_features(mg_context* ctx, const float* T, const float* q, int64_t ncol, int32_t nlev, int32_t nin,
                       float* X) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(T && q && X && ncol >= 0 && nlev > 0 && nin >= 2 * nlev, "mg_column_features: bad arguments");
  if (ncol == 0) return MG_OK;
  column_features_kernel<<<grid_for(ncol * nin), kThreads, 0, ctx->stream>>>(T, q, ncol, nlev, nin, X);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

int mg_hx_column(mg_context* ctx, const double* X, int32_t k, int64_t ld, int64_t ncol, int32_t nlev,
                 const int64_t* obs_col, const int32_t* obs_ch, int64_t p, const float* w, const float* tau,
                 int32_t nch, double* HX) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(X && obs_col && obs_ch && w && tau && HX && k > 0 && ncol > 0 && nlev > 0 && nch > 0 &&
                   ld >= 2 * (int64_t)nlev * ncol,
               "mg_hx_column: bad arguments");
  if (p == 0) return MG_OK;
  MG_CHECK_ARG(p < ((int64_t)1 << 31) && ncol < ((int64_t)1 << 32), "mg_hx_column: too many obs or columns");
  mg::Carver cv;
  cv.reserve<int32_t>(p);
  cv.reserve<char>(column_sort_bytes(p));
  void* ws = mg::workspace(ctx, cv.off);
  if (!ws) return MG_ERR_NOMEM;
  cv = mg::Carver{static_cast<char*>(ws), 0};
  int32_t* perm = cv.take<int32_t>(p);
  void* stmp = cv.take<char>(column_sort_bytes(p));
  MG_TRY_CUDA(sort_obs_by_column(obs_col, p, perm, stmp, ctx->stream));
  hx_column_kernel<<<grid_for(p * k), kThreads, 0, ctx->stream>>>(X, k, ld, ncol, nlev, obs_col, obs_ch, p, perm, w,
                                                                   tau, HX, nullptr, 0);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

int mg_mlp_create(mg_context* ctx, int32_t nin, int32_t nh, int32_t nout, mg_mlp** out) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(out && nin > 0 && nh > 0 && nout > 0 && nout <= 32, "mg_mlp_create: bad sizes");
  auto m = std::make_unique<mg_mlp>();
  m->nin = nin;
  m->nh = nh;
  m->nout = nout;
  m->oW1 = 0;
  m->ob1 = m->oW1 + (int64_t)nh * nin;
  m->oW2 = m->ob1 + nh;
  m->ob2 = m->oW2 + (int64_t)nh * nh;
  m->oW3 = m->ob2 + nh;
  m->ob3 = m->oW3 + (int64_t)nout * nh;
  m->nparam = m->ob3 + nout;
  const size_t pb = sizeof(float) * m->nparam;
  if (cudaMalloc(&m->master, pb) != cudaSuccess || cudaMalloc(&m->m1, pb) != cudaSuccess ||
      cudaMalloc(&m->m2, pb) != cudaSuccess || cudaMalloc(&m->grad, pb) != cudaSuccess ||
      cudaMalloc(&m->wbf, sizeof(__nv_bfloat16) * m->nparam) != cudaSuccess ||
      cudaMalloc(&m->out_shift, sizeof(float) * nout) != cudaSuccess ||
      cudaMalloc(&m->out_scale, sizeof(float) * nout) != cudaSuccess ||
      cudaMalloc(&m->loss, sizeof(float) * 2) != cudaSuccess) {
    cudaGetLastError();
    return mg::fail(ctx, MG_ERR_NOMEM, "mg_mlp_create: allocation failed");
  }
  MG_TRY_CUDA(cudaMemset(m->master, 0, pb));
  MG_TRY_CUDA(cudaMemset(m->m1, 0, pb));
  MG_TRY_CUDA(cudaMemset(m->m2, 0, pb));
  std::vector<float> zero(nout, 0.0f), one(nout, 1.0f);
  MG_TRY_CUDA(cudaMemcpy(m->out_shift, zero.data(), sizeof(float) * nout, cudaMemcpyHostToDevice));
  MG_TRY_CUDA(cudaMemcpy(m->out_scale, one.data(), sizeof(float) * nout, cudaMemcpyHostToDevice));
  *out = m.release();
  return MG_OK;
}

void mg_mlp_destroy(mg_mlp* m) {
  if (!m) return;
  void* ps[] = {m->master, m->m1, m->m2, m->grad, m->wbf, m->out_shift, m->out_scale, m->loss,
                m->Z1, m->H1, m->Z2, m->H2, m->Y, m->dY, m->dA, m->dB,
                m->Xb, m->H1b, m->H2b, m->tc_err};
  for (void* p : ps)
    if (p) cudaFree(p);
  delete m;
}

int64_t mg_mlp_num_params(const mg_mlp* m) { return m ? m->nparam : 0; }

int mg_mlp_set_params(mg_context* ctx, mg_mlp* m, const float* params, const float* out_shift,
                      const float* out_scale) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(m && params, "mg_mlp_set_params: bad arguments");
  MG_TRY_CUDA(cudaMemcpyAsync(m->master, params, sizeof(float) * m->nparam, cudaMemcpyDeviceToDevice, ctx->stream));
  if (out_shift)
    MG_TRY_CUDA(cudaMemcpyAsync(m->out_shift, out_shift, sizeof(float) * m->nout, cudaMemcpyDeviceToDevice, ctx->stream));
  if (out_scale)
    MG_TRY_CUDA(cudaMemcpyAsync(m->out_scale, out_scale, sizeof(float) * m->nout, cudaMemcpyDeviceToDevice, ctx->stream));
  MG_TRY_CUDA(cudaMemsetAsync(m->m1, 0, sizeof(float) * m->nparam, ctx->stream));
  MG_TRY_CUDA(cudaMemsetAsync(m->m2, 0, sizeof(float) * m->nparam, ctx->stream));
  m->step = 0;
  to_bf16_kernel<<<grid_for(m->nparam), kThreads, 0, ctx->stream>>>(m->master, m->nparam, m->wbf);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  return MG_OK;
}

int mg_mlp_get_params(mg_context* ctx, const mg_mlp* m, float* params, int32_t bf16_rounded) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(m && params, "mg_mlp_get_params: bad arguments");
  if (bf16_rounded) {
    bf16_to_float_kernel<<<grid_for(m->nparam), kThreads, 0, ctx->stream>>>(m->wbf, m->nparam, params);
    MG_COUNT_LAUNCH();
    MG_TRY_CUDA(cudaGetLastError());
  } else {
    MG_TRY_CUDA(cudaMemcpyAsync(params, m->master, sizeof(float) * m->nparam, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return MG_OK;
}

int mg_mlp_forward(mg_context* ctx, mg_mlp* m, const float* X, int64_t B, float* Y) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(m && X && Y && B > 0 && B < (int64_t)1 << 31, "mg_mlp_forward: bad arguments");
  int rc = ensure_capacity(ctx, m, B);
  if (rc != MG_OK) return rc;
  if ((rc = forward(ctx, m, X, B)) != MG_OK) return rc;
  MG_TRY_CUDA(cudaMemcpyAsync(Y, m->Y, sizeof(float) * B * m->nout, cudaMemcpyDeviceToDevice, ctx->stream));
  return MG_OK;
}

int mg_mlp_gradients(mg_context* ctx, mg_mlp* m, const float* X, const float* Yt, int64_t B, float* grad,
                     float* loss) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(m && X && Yt && B > 0 && B < (int64_t)1 << 31, "mg_mlp_gradients: bad arguments");
  int rc = ensure_capacity(ctx, m, B);
  if (rc != MG_OK) return rc;
  if ((rc = forward(ctx, m, X, B)) != MG_OK) return rc;
  if ((rc = backward(ctx, m, X, Yt, B)) != MG_OK) return rc;
  if (grad)
    MG_TRY_CUDA(cudaMemcpyAsync(grad, m->grad, sizeof(float) * m->nparam, cudaMemcpyDeviceToDevice, ctx->stream));
  if (loss) {
    float h = 0.0f;
    MG_TRY_CUDA(cudaMemcpyAsync(&h, m->loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    MG_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
    *loss = h / (float)(B * m->nout);
  }
  return MG_OK;
}

int mg_mlp_train_step(mg_context* ctx, mg_mlp* m, const float* X, const float* Yt, int64_t B, float lr,
                      float* loss) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(m && X && Yt && B > 0 && lr > 0.0f, "mg_mlp_train_step: bad arguments");
  int rc = ensure_capacity(ctx, m, B);
  if (rc != MG_OK) return rc;
  if ((rc = forward(ctx, m, X, B)) != MG_OK) return rc;
  if ((rc = backward(ctx, m, X, Yt, B)) != MG_OK) return rc;
  m->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - powf(b1, (float)m->step), c2 = 1.0f - powf(b2, (float)m->step);
  adam_kernel<<<grid_for(m->nparam), kThreads, 0, ctx->stream>>>(m->master, m->m1, m->m2, m->grad, m->nparam, lr, b1,
                                                                 b2, 1e-8f, c1, c2, m->wbf);
  MG_COUNT_LAUNCH();
  MG_TRY_CUDA(cudaGetLastError());
  if (loss) {
    float h = 0.0f;
    MG_TRY_CUDA(cudaMemcpyAsync(&h, m->loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    MG_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
    *loss = h / (float)(B * m->nout);
  }
  return MG_OK;
}

int mg_hx_column_mlp(mg_context* ctx, mg_mlp* m, const double* X, int32_t k, int64_t ld, int64_t ncol, int32_t nlev,
                     const int64_t* obs_col, const int32_t* obs_ch, int64_t p, double* HX) {
  if (!ctx) return MG_ERR_ARG;
  MG_CHECK_ARG(m && X && obs_col && obs_ch && HX && k > 0 && ncol > 0 && nlev > 0 && 2 * nlev <= m->nin &&
                   ld >= 2 * (int64_t)nlev * ncol,
               "mg_hx_column_mlp: bad arguments");
  if (p == 0) return MG_OK;
  MG_CHECK_ARG(p < ((int64_t)1 << 31) && ncol < ((int64_t)1 << 32), "mg_hx_column_mlp: too many obs or columns");
  // Columns are run through the network in slices so activations stay
  // bounded; the obs are taken in column order (sorted once per call).
  const int64_t total = p * k;
  const int64_t slice = std::min<int64_t>(total, (int64_t)1 << 20);
  const bool tc = tc_shapes_ok(m);
  mg::Carver cv;
  cv.reserve<int32_t>(p);
  cv.reserve<char>(column_sort_bytes(p));
  if (!tc) cv.reserve<float>((size_t)slice * m->nin);
  void* ws = mg::workspace(ctx, cv.off);
  if (!ws) return MG_ERR_NOMEM;
  cv = mg::Carver{static_cast<char*>(ws), 0};
  int32_t* perm = cv.take<int32_t>(p);
  void* stmp = cv.take<char>(column_sort_bytes(p));
  float* feat = tc ? nullptr : cv.take<float>((size_t)slice * m->nin);
  MG_TRY_CUDA(sort_obs_by_column(obs_col, p, perm, stmp, ctx->stream));
  if (tc) {
    int rc = ensure_capacity(ctx, m, slice);
    if (rc != MG_OK || (rc = ensure_tc_capacity(ctx, m, slice)) != MG_OK) return rc;
    MG_TRY_CUDA(cudaMemsetAsync(m->tc_err, 0, sizeof(int), ctx->stream));
    for (int64_t o0 = 0; o0 < p; o0 += slice / k) {
      const int64_t np = std::min<int64_t>(p - o0, slice / k);
      hx_column_kernel<<<grid_for(np * k), kThreads, 0, ctx->stream>>>(
          X, k, ld, ncol, nlev, obs_col, obs_ch, np, perm + o0, nullptr, nullptr, nullptr, nullptr, m->nin, m->Xb);
      MG_COUNT_LAUNCH();
      if ((rc = forward_tc(ctx, m, np * k)) != MG_OK) return rc;
      pick_channel_kernel<<<grid_for(np * k), kThreads, 0, ctx->stream>>>(m->Y, np, k, m->nout, perm + o0, obs_ch,
                                                                          m->out_shift, m->out_scale, HX);
      MG_COUNT_LAUNCH();
      MG_TRY_CUDA(cudaGetLastError());
    }
    int h = 0;
    MG_TRY_CUDA(cudaMemcpyAsync(&h, m->tc_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MG_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
    if (h) return mg::fail(ctx, MG_ERR_TIMEOUT, "mg_hx_column_mlp: a tensor-core GEMM wait gave up");
    return MG_OK;
  }
  int rc = ensure_capacity(ctx, m, slice);
  if (rc != MG_OK) return rc;
  for (int64_t o0 = 0; o0 < p; o0 += slice / k) {
    const int64_t np = std::min<int64_t>(p - o0, slice / k);
    hx_column_kernel<<<grid_for(np * k), kThreads, 0, ctx->stream>>>(X, k, ld, ncol, nlev, obs_col, obs_ch, np,
                                                                     perm + o0, nullptr, nullptr, nullptr, feat,
                                                                     m->nin);
    MG_COUNT_LAUNCH();
    if ((rc = forward(ctx, m, feat, np * k)) != MG_OK) return rc;
    pick_channel_kernel<<<grid_for(np * k), kThreads, 0, ctx->stream>>>(m->Y, np, k, m->nout, perm + o0, obs_ch,
                                                                        m->out_shift, m->out_scale, HX);
    MG_COUNT_LAUNCH();
    MG_TRY_CUDA(cudaGetLastError());
  }
  return MG_OK;
}

}  // extern "C"
