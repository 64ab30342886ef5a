// fvs_mlp.cu — the learned warm start: a small MLP trained and evaluated on
// the GPU with the library's own kernels.
//
// Network: n_in -> width (GELU) -> ... -> width (GELU) -> n_out, `depth`
// hidden layers.  Weights are kept in FP32 (Adam master copy) and rounded to
// BF16 for every GEMM; activations enter the GEMMs in BF16; every GEMM
// accumulates in FP32 on the tensor cores: tcgen05.mma with the accumulator in
// tensor memory (fvs_tcgemm.cuh, the default engine), or the warp-level
// mma.sync m16n8k16 kernel below (kept as the comparison engine).
// Training: minibatch Adam on the mean squared error.
//
// GEMM convention: C[m][n] = sum_k A(m,k) B(n,k) (+ bias[n]); each operand is
// either K-major (row m at A + m*lda) or stored transposed (element (m,k) at
// A + k*lda + m), which covers the forward pass (X W^T), the input gradient
// (dZ W) and the weight gradient (dZ^T X) without explicit transposes.
//
// The reference has no learned component; this is the third "AI-systems
// pattern" laid over the drop-in FP64 path, which stays unchanged.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "../../include/fvs2d.h"
#include "fvs_tcgemm.cuh"

namespace {

thread_local std::string g_mlp_error;

typedef __nv_bfloat16 bf16;

constexpr int BM = 128, BN = 128, BK = 32, KPAD = 8;  // smem rows padded to avoid bank conflicts
constexpr int GEMM_THREADS = 256;                       // 8 warps: 4 along M x 2 along N, 32x64 each

enum Epilogue : int { EPI_F32 = 0, EPI_BIAS_F32 = 1, EPI_BIAS_GELU = 2 };

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// tile loader: operand element (row r, col k) of a [rows x K] view into smem
// s[r][k]; out-of-range elements read as zero
template <bool KMAJOR>
__device__ __forceinline__ void load_tile(bf16 (*s)[BK + KPAD], const bf16* g, int ld, int row0, int rows, int k0, int K,
                                          int ntile_rows) {
  const int t = threadIdx.x;
  if (KMAJOR) {
    // 8 contiguous k per load
    for (int i = t; i < ntile_rows * (BK / 8); i += GEMM_THREADS) {
      const int r = i / (BK / 8), kk = (i % (BK / 8)) * 8;
      const int gr = row0 + r, gk = k0 + kk;
#pragma unroll
      for (int j = 0; j < 8; j++)
        s[r][kk + j] = (gr < rows && gk + j < K) ? g[(size_t)gr * ld + gk + j] : __float2bfloat16(0.f);
    }
  } else {
    // element (r, k) at g + k*ld + r: contiguous along r
    for (int i = t; i < ntile_rows * BK; i += GEMM_THREADS) {
      const int kk = i / ntile_rows, r = i % ntile_rows;
      const int gr = row0 + r, gk = k0 + kk;
      s[r][kk] = (gr < rows && gk < K) ? g[(size_t)gk * ld + gr] : __float2bfloat16(0.f);
    }
  }
}

template <bool A_KM, bool B_KM>
__global__ void __launch_bounds__(GEMM_THREADS) k_gemm(const bf16* __restrict__ A, int lda, const bf16* __restrict__ B,
                                                       int ldb, int M, int N, int K, int epi,
                                                       const float* __restrict__ bias, float* __restrict__ C, int ldc,
                                                       bf16* __restrict__ Cact, int ldact) {
  __shared__ __align__(16) bf16 sA[BM][BK + KPAD];
  __shared__ __align__(16) bf16 sB[BN][BK + KPAD];
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = (warp & 3) * 32, wn = (warp >> 2) * 64;
  const int g = lane >> 2, tq = lane & 3;
  float acc[2][8][4];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 8; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[i][j][q] = 0.f;
  for (int k0 = 0; k0 < K; k0 += BK) {
    load_tile<A_KM>(sA, A, lda, m0, M, k0, K, BM);
    load_tile<B_KM>(sB, B, ldb, n0, N, k0, K, BN);
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[2][4], bfr[8][2];
#pragma unroll
      for (int i = 0; i < 2; i++) {
        const int r = wm + 16 * i + g;
        af[i][0] = *reinterpret_cast<const uint32_t*>(&sA[r][kk + 2 * tq]);
        af[i][1] = *reinterpret_cast<const uint32_t*>(&sA[r + 8][kk + 2 * tq]);
        af[i][2] = *reinterpret_cast<const uint32_t*>(&sA[r][kk + 8 + 2 * tq]);
        af[i][3] = *reinterpret_cast<const uint32_t*>(&sA[r + 8][kk + 8 + 2 * tq]);
      }
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int c = wn + 8 * j + g;
        bfr[j][0] = *reinterpret_cast<const uint32_t*>(&sB[c][kk + 2 * tq]);
        bfr[j][1] = *reinterpret_cast<const uint32_t*>(&sB[c][kk + 8 + 2 * tq]);
      }
#pragma unroll
      for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) mma_bf16(acc[i][j], af[i], bfr[j]);
    }
    __syncthreads();
  }
  // epilogue
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 8; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int m = m0 + wm + 16 * i + g + (q >= 2 ? 8 : 0);
        const int n = n0 + wn + 8 * j + 2 * tq + (q & 1);
        if (m >= M || n >= N) continue;
        float z = acc[i][j][q];
        if (epi != EPI_F32 && bias) z += bias[n];
        if (C) C[(size_t)m * ldc + n] = z;
        if (epi == EPI_BIAS_GELU && Cact) Cact[(size_t)m * ldact + n] = __float2bfloat16(gelu(z));
      }
}

__global__ void k_f32_to_bf16(const float* __restrict__ x, bf16* __restrict__ y, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16(x[i]);
}

// rows of the dataset selected by idx, padded to ld columns, as BF16
__global__ void k_gather_rows(const float* __restrict__ x, int ncol, const int* __restrict__ idx, int n, bf16* __restrict__ out,
                              int ld) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * ld) return;
  const int r = i / ld, c = i % ld;
  out[i] = __float2bfloat16(c < ncol ? x[(size_t)idx[r] * ncol + c] : 0.f);
}

__global__ void k_gather_rows_f32(const float* __restrict__ x, int ncol, const int* __restrict__ idx, int n, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * ncol) return;
  const int r = i / ncol, c = i % ncol;
  out[i] = x[(size_t)idx[r] * ncol + c];
}

// dY = 2 (Y - T) / (n * nout) as BF16 (ld = ldg), squared error summed into loss
__global__ void k_mse(const float* __restrict__ Y, int ldy, const float* __restrict__ T, int n, int nout, bf16* __restrict__ dY,
                      int ldg, float* __restrict__ loss_acc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float e2 = 0.f;
  if (i < n * ldg) {
    const int r = i / ldg, c = i % ldg;
    float d = 0.f;
    if (c < nout) {
      d = Y[(size_t)r * ldy + c] - T[(size_t)r * nout + c];
      e2 = d * d;
    }
    dY[i] = __float2bfloat16(2.f * d / float(n * nout));
  }
  for (int o = 16; o > 0; o >>= 1) e2 += __shfl_down_sync(0xffffffffu, e2, o);
  if ((threadIdx.x & 31) == 0 && e2 != 0.f) atomicAdd(loss_acc, e2);
}

// dZ = dA * gelu'(Z) as BF16
__global__ void k_gelu_back(const float* __restrict__ dA, const float* __restrict__ Z, bf16* __restrict__ dZ, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) dZ[i] = __float2bfloat16(dA[i] * gelu_grad(Z[i]));
}

// bias gradient: column sums of a [n x cols] BF16 matrix (ld).  A block of
// 32 x 32 threads takes 32 columns: each thread row sums every 32nd matrix
// row, then the 32 partial sums of a column are added in a fixed order
// (deterministic).
__global__ void __launch_bounds__(1024) k_colsum(const bf16* __restrict__ g, int n, int cols, int ld,
                                                 float* __restrict__ out) {
  __shared__ float part[32][33];
  const int c = blockIdx.x * 32 + threadIdx.x;
  float s = 0.f;
  if (c < cols)
    for (int r = threadIdx.y; r < n; r += 32) s += __bfloat162float(g[(size_t)r * ld + c]);
  part[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && c < cols) {
    float t = 0.f;
    for (int k = 0; k < 32; k++) t += part[k][threadIdx.x];
    out[c] = t;
  }
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v, size_t n,
                       float lr, float b1, float b2, float eps, float bc1, float bc2) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

inline unsigned nblk(size_t n, int b = 256) { return (unsigned)((n + b - 1) / b); }
inline int pad16(int x) { return (x + 15) / 16 * 16; }

}  // namespace

struct fvs_mlp {
  int n_in = 0, width = 0, depth = 0, n_out = 0;
  int in_pad = 0, out_pad = 0;
  int nl = 0;                        // GEMM layers = depth + 1
  std::vector<int> din, dout;        // padded layer dimensions
  std::vector<size_t> woff, boff;    // offsets into the FP32 parameter vector
  size_t nparam = 0;
  std::string err;
  cudaStream_t stream = nullptr;
  float* w = nullptr;                // FP32 master parameters (padded layout)
  float* g = nullptr;                // gradients
  float* am = nullptr;               // Adam moments
  float* av = nullptr;
  bf16* wb = nullptr;                // BF16 copy of the weights
  int cap = 0;                       // rows of the activation buffers
  std::vector<bf16*> act;            // act[l]: input of layer l, [cap][din[l]]
  std::vector<float*> pre;           // pre[l]: layer output before GELU, [cap][dout[l]]
  bf16* dz = nullptr;                // [cap][max dim]
  bf16* dz2 = nullptr;
  float* da = nullptr;               // [cap][max dim]
  float* loss = nullptr;
  int* gemm_err = nullptr;           // set by a tcgen05 GEMM whose bounded wait expired
  float* split_ws = nullptr;         // split-K partial sums of the tcgen05 GEMM
  size_t split_cap = 0;              // floats
  int engine = 0;                    // 0: tcgen05, 1: mma.sync
  int step = 0;
  std::vector<void*> owned;

  ~fvs_mlp() {
    for (void* p : owned) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
  }
  int fail(int code, const std::string& m) {
    err = m;
    return code;
  }
  template <typename V>
  V* dalloc(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, sizeof(V) * std::max<size_t>(n, 1)) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, sizeof(V) * std::max<size_t>(n, 1));
    owned.push_back(p);
    return static_cast<V*>(p);
  }
  bool ensure_cap(int rows) {
    if (rows <= cap) return true;
    const int maxd = std::max(*std::max_element(din.begin(), din.end()), *std::max_element(dout.begin(), dout.end()));
    act.assign(nl + 1, nullptr);
    pre.assign(nl, nullptr);
    for (int l = 0; l <= nl; l++) act[l] = dalloc<bf16>((size_t)rows * (l < nl ? din[l] : dout[nl - 1]));
    for (int l = 0; l < nl; l++) pre[l] = dalloc<float>((size_t)rows * dout[l]);
    dz = dalloc<bf16>((size_t)rows * maxd);
    dz2 = dalloc<bf16>((size_t)rows * maxd);
    da = dalloc<float>((size_t)rows * maxd);
    for (int l = 0; l <= nl; l++) if (!act[l]) return false;
    for (int l = 0; l < nl; l++) if (!pre[l]) return false;
    if (!dz || !dz2 || !da) return false;
    cap = rows;
    return true;
  }
};

namespace {

template <bool A_KM, bool B_KM>
void gemm(fvs_mlp* m, const bf16* A, int lda, const bf16* B, int ldb, int M, int N, int K, int epi,
          const float* bias, float* C, int ldc, bf16* Cact, int ldact) {
  if (m->engine == 0) {
    const int tiles = ((N + tc::BN - 1) / tc::BN) * ((M + tc::BM - 1) / tc::BM);
    const int nk = (K + tc::BK - 1) / tc::BK;
    int nsplit = 1;
    if (epi == EPI_F32 && C && !Cact && tiles < 64 && nk >= 4) {
      // few output tiles and a long K (the weight gradient, K = batch rows):
      // split K so that about one CTA per SM works, then add the partials
      const int want = std::max(1, 148 / tiles);
      const int per = std::max(1, (nk + want - 1) / want);
      nsplit = (nk + per - 1) / per;
      const size_t need = (size_t)nsplit * M * ldc;
      if (nsplit > 1 && need > m->split_cap) {
        float* w = m->dalloc<float>(need);
        if (w) {
          m->split_ws = w;
          m->split_cap = need;
        } else {
          nsplit = 1;
        }
      }
    }
    dim3 grid((unsigned)((N + tc::BN - 1) / tc::BN), (unsigned)((M + tc::BM - 1) / tc::BM), (unsigned)nsplit);
    const size_t stride = (size_t)M * ldc;
    float* out = nsplit > 1 ? m->split_ws : C;
    tc::k_gemm_tc<A_KM, B_KM><<<grid, tc::THREADS, tc::SMEM_BYTES, m->stream>>>(A, lda, B, ldb, M, N, K, epi, bias,
                                                                              out, ldc, Cact, ldact, m->gemm_err,
                                                                              stride);
    if (nsplit > 1)
      tc::k_sum_splits<<<nblk((size_t)M * N), 256, 0, m->stream>>>(m->split_ws, nsplit, stride, M, N, ldc, C);
    return;
  }
  dim3 grid((unsigned)((N + BN - 1) / BN), (unsigned)((M + BM - 1) / BM));
  k_gemm<A_KM, B_KM><<<grid, GEMM_THREADS, 0, m->stream>>>(A, lda, B, ldb, M, N, K, epi, bias, C, ldc, Cact, ldact);
}

// the tcgen05 GEMM uses 64 KB of dynamic shared memory
bool tc_gemm_setup() {
  const int b = tc::SMEM_BYTES;
  return cudaFuncSetAttribute(tc::k_gemm_tc<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) == cudaSuccess &&
         cudaFuncSetAttribute(tc::k_gemm_tc<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) == cudaSuccess &&
         cudaFuncSetAttribute(tc::k_gemm_tc<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) == cudaSuccess &&
         cudaFuncSetAttribute(tc::k_gemm_tc<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) == cudaSuccess;
}

void refresh_bf16(fvs_mlp* m) { k_f32_to_bf16<<<nblk(m->nparam), 256, 0, m->stream>>>(m->w, m->wb, m->nparam); }

// forward over n rows already in act[0]; outputs pre[nl-1]
void forward(fvs_mlp* m, int n) {
  for (int l = 0; l < m->nl; l++) {
    const bool last = l == m->nl - 1;
    gemm<true, true>(m, m->act[l], m->din[l], m->wb + m->woff[l], m->din[l], n, m->dout[l], m->din[l],
                     last ? EPI_BIAS_F32 : EPI_BIAS_GELU, m->w + m->boff[l], m->pre[l], m->dout[l], last ? nullptr : m->act[l + 1],
                     m->dout[l]);
  }
}

// backward from dY (BF16, [n][out_pad]) in dz; gradients into g
void backward(fvs_mlp* m, int n) {
  bf16* dcur = m->dz;
  bf16* dnext = m->dz2;
  for (int l = m->nl - 1; l >= 0; l--) {
    const int di = m->din[l], dn = m->dout[l];
    // dW_l[n][k] = sum_m dZ[m][n] act_l[m][k]
    gemm<false, false>(m, dcur, dn, m->act[l], di, dn, di, n, EPI_F32, nullptr, m->g + m->woff[l], di, nullptr, 0);
    k_colsum<<<(dn + 31) / 32, dim3(32, 32), 0, m->stream>>>(dcur, n, dn, dn, m->g + m->boff[l]);
    if (l == 0) break;
    // dA_{l}[m][k] = sum_n dZ[m][n] W_l[n][k]; dZ_{l-1} = dA * gelu'(pre_{l-1})
    gemm<true, false>(m, dcur, dn, m->wb + m->woff[l], di, n, di, dn, EPI_F32, nullptr, m->da, di, nullptr, 0);
    k_gelu_back<<<nblk((size_t)n * di), 256, 0, m->stream>>>(m->da, m->pre[l - 1], dnext, (size_t)n * di);
    std::swap(dcur, dnext);
  }
}

int check(fvs_mlp* m, const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) return m->fail(FVS_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
  int flag = 0;
  e = cudaMemcpy(&flag, m->gemm_err, sizeof flag, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return m->fail(FVS_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
  if (flag) return m->fail(FVS_ERR_TIMEOUT, std::string(where) + ": a tensor-core GEMM wait ran out of its budget");
  return FVS_OK;
}

}  // namespace

extern "C" {

int fvs_mlp_create(int32_t n_in, int32_t width, int32_t depth, int32_t n_out, uint64_t seed, fvs_mlp** out) {
  if (!out) return FVS_ERR_INVALID;
  *out = nullptr;
  if (n_in <= 0 || n_in > 64 || width <= 0 || width > 1024 || width % 16 || depth < 1 || depth > 16 || n_out <= 0 ||
      n_out > 64) {
    g_mlp_error = "MLP sizes: 1 <= n_in, n_out <= 64; width a multiple of 16 up to 1024; 1 <= depth <= 16";
    return FVS_ERR_INVALID;
  }
  std::unique_ptr<fvs_mlp> m(new fvs_mlp());
  m->n_in = n_in; m->width = width; m->depth = depth; m->n_out = n_out;
  m->in_pad = pad16(n_in);
  m->out_pad = pad16(n_out);
  m->nl = depth + 1;
  for (int l = 0; l < m->nl; l++) {
    m->din.push_back(l == 0 ? m->in_pad : width);
    m->dout.push_back(l == m->nl - 1 ? m->out_pad : width);
  }
  size_t off = 0;
  for (int l = 0; l < m->nl; l++) {
    m->woff.push_back(off);
    off += (size_t)m->din[l] * m->dout[l];
    m->boff.push_back(off);
    off += m->dout[l];
  }
  m->nparam = off;
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) {
    g_mlp_error = "cudaStreamCreate failed";
    return FVS_ERR_CUDA;
  }
  if (!tc_gemm_setup()) {
    g_mlp_error = "tensor-core GEMM setup (dynamic shared memory) failed";
    return FVS_ERR_CUDA;
  }
  m->w = m->dalloc<float>(off);
  m->g = m->dalloc<float>(off);
  m->am = m->dalloc<float>(off);
  m->av = m->dalloc<float>(off);
  m->wb = m->dalloc<bf16>(off);
  m->loss = m->dalloc<float>(4);
  m->gemm_err = m->dalloc<int>(4);
  if (!m->w || !m->g || !m->am || !m->av || !m->wb || !m->loss || !m->gemm_err) {
    g_mlp_error = "MLP device allocation failed";
    return FVS_ERR_NOMEM;
  }
  // He-style init (seeded), zero biases; padded rows/columns stay zero
  std::vector<float> h(off, 0.f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < m->nl; l++) {
    const int fan_in = l == 0 ? n_in : width, rows = l == m->nl - 1 ? n_out : width;
    std::normal_distribution<float> nd(0.f, std::sqrt(2.f / fan_in));
    for (int r = 0; r < rows; r++)
      for (int k = 0; k < fan_in; k++) h[m->woff[l] + (size_t)r * m->din[l] + k] = nd(rng);
  }
  cudaMemcpy(m->w, h.data(), 4 * off, cudaMemcpyHostToDevice);
  refresh_bf16(m.get());
  if (check(m.get(), "MLP init")) {
    g_mlp_error = m->err;
    return FVS_ERR_CUDA;
  }
  *out = m.release();
  return FVS_OK;
}

void fvs_mlp_destroy(fvs_mlp* m) { delete m; }

const char* fvs_mlp_last_error(const fvs_mlp* m) { return m ? m->err.c_str() : g_mlp_error.c_str(); }

// number of parameters in the unpadded layout: per layer W[out][in], b[out]
int fvs_mlp_num_params(const fvs_mlp* m, int64_t* n) {
  if (!m || !n) return FVS_ERR_INVALID;
  int64_t s = 0;
  for (int l = 0; l < m->nl; l++) {
    const int i = l == 0 ? m->n_in : m->width, o = l == m->nl - 1 ? m->n_out : m->width;
    s += (int64_t)i * o + o;
  }
  *n = s;
  return FVS_OK;
}

int fvs_mlp_set_engine(fvs_mlp* m, int32_t engine) {
  if (!m || engine < 0 || engine > 1) return FVS_ERR_INVALID;
  m->engine = engine;
  return FVS_OK;
}

static int copy_params(fvs_mlp* m, float* host, const float* in, int64_t n, bool get, const float* dev_src) {
  int64_t need = 0;
  fvs_mlp_num_params(m, &need);
  if (n < need) return m->fail(FVS_ERR_INVALID, "parameter buffer too small");
  std::vector<float> pad(m->nparam, 0.f);
  if (get && cudaMemcpy(pad.data(), dev_src, 4 * m->nparam, cudaMemcpyDeviceToHost) != cudaSuccess)
    return m->fail(FVS_ERR_CUDA, "parameter download");
  int64_t p = 0;
  for (int l = 0; l < m->nl; l++) {
    const int i = l == 0 ? m->n_in : m->width, o = l == m->nl - 1 ? m->n_out : m->width;
    for (int r = 0; r < o; r++)
      for (int k = 0; k < i; k++, p++) {
        float& dst = pad[m->woff[l] + (size_t)r * m->din[l] + k];
        if (get) host[p] = dst; else dst = in[p];
      }
    for (int r = 0; r < o; r++, p++) {
      float& dst = pad[m->boff[l] + r];
      if (get) host[p] = dst; else dst = in[p];
    }
  }
  if (!get) {
    if (cudaMemcpy(m->w, pad.data(), 4 * m->nparam, cudaMemcpyHostToDevice) != cudaSuccess)
      return m->fail(FVS_ERR_CUDA, "parameter upload");
    cudaMemset(m->am, 0, 4 * m->nparam);
    cudaMemset(m->av, 0, 4 * m->nparam);
    m->step = 0;
    refresh_bf16(m);
    return check(m, "set_params");
  }
  return FVS_OK;
}

int fvs_mlp_get_params(fvs_mlp* m, float* dst, int64_t n) {
  if (!m || !dst) return FVS_ERR_INVALID;
  return copy_params(m, dst, nullptr, n, true, m->w);
}

int fvs_mlp_set_params(fvs_mlp* m, const float* src, int64_t n) {
  if (!m || !src) return FVS_ERR_INVALID;
  return copy_params(m, nullptr, src, n, false, nullptr);
}

// loss and parameter gradients of one batch (no update), for checking
int fvs_mlp_loss_grad(fvs_mlp* m, const float* x, const float* y, int32_t n, float* loss, float* grads) {
  if (!m || !x || !y || n <= 0) return FVS_ERR_INVALID;
  if (!m->ensure_cap(n)) return m->fail(FVS_ERR_NOMEM, "activation allocation");
  float* dx = m->dalloc<float>((size_t)n * m->n_in);
  float* dy = m->dalloc<float>((size_t)n * m->n_out);
  int* di = m->dalloc<int>(n);
  if (!dx || !dy || !di) return m->fail(FVS_ERR_NOMEM, "batch allocation");
  std::vector<int> idx(n);
  for (int i = 0; i < n; i++) idx[i] = i;
  cudaMemcpy(dx, x, 4 * (size_t)n * m->n_in, cudaMemcpyHostToDevice);
  cudaMemcpy(dy, y, 4 * (size_t)n * m->n_out, cudaMemcpyHostToDevice);
  cudaMemcpy(di, idx.data(), 4 * (size_t)n, cudaMemcpyHostToDevice);
  k_gather_rows<<<nblk((size_t)n * m->in_pad), 256, 0, m->stream>>>(dx, m->n_in, di, n, m->act[0], m->in_pad);
  forward(m, n);
  cudaMemsetAsync(m->loss, 0, 4, m->stream);
  k_mse<<<nblk((size_t)n * m->out_pad), 256, 0, m->stream>>>(m->pre[m->nl - 1], m->out_pad, dy, n, m->n_out, m->dz,
                                                            m->out_pad, m->loss);
  cudaMemsetAsync(m->g, 0, 4 * m->nparam, m->stream);
  backward(m, n);
  int rc = check(m, "loss_grad");
  if (rc) return rc;
  float l = 0.f;
  cudaMemcpy(&l, m->loss, 4, cudaMemcpyDeviceToHost);
  if (loss) *loss = l / float(n * m->n_out);
  if (grads) {
    int64_t np = 0;
    fvs_mlp_num_params(m, &np);
    rc = copy_params(m, grads, nullptr, np, true, m->g);
  }
  return rc;
}

// minibatch Adam; loss_per_epoch[epochs] (mean squared error of the epoch)
int fvs_mlp_train(fvs_mlp* m, const float* x, const float* y, int64_t n, int32_t batch, int32_t epochs, float lr,
                  uint64_t seed, float* loss_per_epoch) {
  if (!m || !x || !y || n <= 0 || batch <= 0 || epochs <= 0 || n > (int64_t)1 << 31) return FVS_ERR_INVALID;
  batch = (int)std::min<int64_t>(batch, n);
  if (!m->ensure_cap(batch)) return m->fail(FVS_ERR_NOMEM, "activation allocation");
  float* dx = m->dalloc<float>((size_t)n * m->n_in);
  float* dy = m->dalloc<float>((size_t)n * m->n_out);
  float* ty = m->dalloc<float>((size_t)batch * m->n_out);
  int* didx = m->dalloc<int>(n);
  if (!dx || !dy || !ty || !didx) return m->fail(FVS_ERR_NOMEM, "dataset allocation");
  cudaMemcpy(dx, x, 4 * (size_t)n * m->n_in, cudaMemcpyHostToDevice);
  cudaMemcpy(dy, y, 4 * (size_t)n * m->n_out, cudaMemcpyHostToDevice);
  std::vector<int> idx(n);
  std::mt19937_64 rng(seed);
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int ep = 0; ep < epochs; ep++) {
    for (int64_t i = 0; i < n; i++) idx[i] = (int)i;
    std::shuffle(idx.begin(), idx.end(), rng);
    cudaMemcpyAsync(didx, idx.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, m->stream);
    cudaMemsetAsync(m->loss, 0, 4, m->stream);
    for (int64_t s0 = 0; s0 + batch <= n; s0 += batch) {
      const int* bi = didx + s0;
      k_gather_rows<<<nblk((size_t)batch * m->in_pad), 256, 0, m->stream>>>(dx, m->n_in, bi, batch, m->act[0], m->in_pad);
      k_gather_rows_f32<<<nblk((size_t)batch * m->n_out), 256, 0, m->stream>>>(dy, m->n_out, bi, batch, ty);
      forward(m, batch);
      k_mse<<<nblk((size_t)batch * m->out_pad), 256, 0, m->stream>>>(m->pre[m->nl - 1], m->out_pad, ty, batch, m->n_out, m->dz,
                                                                      m->out_pad, m->loss);
      backward(m, batch);
      m->step++;
      k_adam<<<nblk(m->nparam), 256, 0, m->stream>>>(m->w, m->g, m->am, m->av, m->nparam, lr, b1, b2, eps,
                                                     1.f - std::pow(b1, (float)m->step), 1.f - std::pow(b2, (float)m->step));
      refresh_bf16(m);
    }
    int rc = check(m, "train");
    if (rc) return rc;
    if (loss_per_epoch) {
      float l = 0.f;
      cudaMemcpy(&l, m->loss, 4, cudaMemcpyDeviceToHost);
      loss_per_epoch[ep] = l / float((n / batch) * batch * m->n_out);
    }
  }
  return FVS_OK;
}

int fvs_mlp_predict(fvs_mlp* m, const float* x, int64_t n, float* y) {
  if (!m || !x || !y || n <= 0) return FVS_ERR_INVALID;
  const int chunk = (int)std::min<int64_t>(n, 65536);
  if (!m->ensure_cap(chunk)) return m->fail(FVS_ERR_NOMEM, "activation allocation");
  float* dx = m->dalloc<float>((size_t)chunk * m->n_in);
  int* di = m->dalloc<int>(chunk);
  if (!dx || !di) return m->fail(FVS_ERR_NOMEM, "batch allocation");
  std::vector<int> idx(chunk);
  for (int i = 0; i < chunk; i++) idx[i] = i;
  cudaMemcpy(di, idx.data(), 4 * (size_t)chunk, cudaMemcpyHostToDevice);
  std::vector<float> out((size_t)chunk * m->out_pad);
  for (int64_t s0 = 0; s0 < n; s0 += chunk) {
    const int c = (int)std::min<int64_t>(chunk, n - s0);
    cudaMemcpyAsync(dx, x + s0 * m->n_in, 4 * (size_t)c * m->n_in, cudaMemcpyHostToDevice, m->stream);
    k_gather_rows<<<nblk((size_t)c * m->in_pad), 256, 0, m->stream>>>(dx, m->n_in, di, c, m->act[0], m->in_pad);
    forward(m, c);
    cudaMemcpyAsync(out.data(), m->pre[m->nl - 1], 4 * (size_t)c * m->out_pad, cudaMemcpyDeviceToHost, m->stream);
    int rc = check(m, "predict");
    if (rc) return rc;
    for (int r = 0; r < c; r++)
      for (int k = 0; k < m->n_out; k++) y[(s0 + r) * m->n_out + k] = out[(size_t)r * m->out_pad + k];
  }
  return FVS_OK;
}

}  // extern "C"
