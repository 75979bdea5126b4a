// Learned warm start: a 3-layer perceptron (n_in -> hidden -> hidden ->
// n_out, ReLU) with BF16 weights and activations, FP32 accumulation, FP32
// master weights and Adam.  It maps the data of a parametrised problem
// family to a starting iterate (x0, y0, s0) for the solver (the reference's
// warm-start inputs Data.x/y/s, pdos.h:29-32, common.h:147-161); the solver,
// not the network, produces every reported result.
//
// All products go through one tensor-core kernel, C[M,N] = A[M,K] B[N,K]^T
// with both operands K-contiguous (mma.sync m16n8k16 BF16 -> FP32, ldmatrix
// fragments, cp.async double buffering), with fused epilogues: bias, ReLU,
// multiplication by a ReLU mask, BF16 or FP32 output.  The backward pass
// transposes its operands into that form first.  Every reduction (loss,
// bias gradients) has a fixed order.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "common.cuh"
#include "engine.cuh"

namespace pdosgpu {
namespace mlp {

using bf16 = __nv_bfloat16;

constexpr int BM = 128, BN = 128, BK = 32, KPAD = 8;  // smem rows of BK + KPAD
constexpr int kThreads = 256;                          // 8 warps: 2 (M) x 4 (N)

struct Epi {
  const float *bias;   // [N] or NULL
  const bf16 *mask;    // [M, ldm] or NULL: out *= (mask > 0)
  int ldm;
  int relu;
  float *out_f32;      // one of the two outputs
  bf16 *out_bf16;
  int ldc;
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, bool pred) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  const int n = pred ? 16 : 0;  // zero-fill when out of range
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(s), "l"(gmem), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void ldmatrix_x4(unsigned (&r)[4], const void *smem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(s));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
      "{%8, %9}, {%0, %1, %2, %3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// C[M,N] = A[M,K] B[N,K]^T (+ epilogue).  lda, ldb and K are multiples of 8
// (16-byte rows); rows past M or N and the K tail read as zero.
__global__ void __launch_bounds__(kThreads) gemm_nt_kernel(const bf16 *__restrict__ A, int lda,
                                                           const bf16 *__restrict__ B, int ldb, int M,
                                                           int N, int K, Epi ep) {
  __shared__ __align__(16) bf16 As[2][BM][BK + KPAD];
  __shared__ __align__(16) bf16 Bs[2][BN][BK + KPAD];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 2, wn = warp & 3;  // warp tile 64 x 32
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;

  auto load = [&](int stage, int k0) {
#pragma unroll
    for (int i = 0; i < 2; ++i) {  // 128 rows x 4 chunks of 8 per operand
      const int c = tid + i * kThreads;
      const int row = c >> 2, kc = (c & 3) * 8;
      const int ga = m0 + row, gb = n0 + row, gk = k0 + kc;
      const bool ka = gk < K;
      cp_async16(&As[stage][row][kc], A + (size_t)(ga < M ? ga : 0) * lda + (ka ? gk : 0), ga < M && ka);
      cp_async16(&Bs[stage][row][kc], B + (size_t)(gb < N ? gb : 0) * ldb + (ka ? gk : 0), gb < N && ka);
    }
    cp_async_commit();
  };

  float acc[4][4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int t = 0; t < 4; ++t) acc[i][j][t] = 0.f;

  const int nk = (K + BK - 1) / BK;
  load(0, 0);
  for (int kt = 0; kt < nk; ++kt) {
    const int st = kt & 1;
    cp_async_wait_all();
    __syncthreads();
    if (kt + 1 < nk) load(st ^ 1, (kt + 1) * BK);
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      unsigned a[4][4], b[2][4];
#pragma unroll
      for (int mi = 0; mi < 4; ++mi)
        ldmatrix_x4(a[mi], &As[st][wm * 64 + mi * 16 + (lane & 15)][kk + (lane >> 4) * 8]);
#pragma unroll
      for (int nj = 0; nj < 2; ++nj)
        ldmatrix_x4(b[nj], &Bs[st][wn * 32 + nj * 16 + (lane & 7) + (lane >> 4) * 8][kk + ((lane >> 3) & 1) * 8]);
#pragma unroll
      for (int mi = 0; mi < 4; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
          mma_bf16(acc[mi][ni], a[mi], b[ni >> 1][(ni & 1) * 2], b[ni >> 1][(ni & 1) * 2 + 1]);
    }
  }

  // epilogue: acc[mi][ni] holds rows r, r+8 and columns c, c+1
#pragma unroll
  for (int mi = 0; mi < 4; ++mi) {
#pragma unroll
    for (int ni = 0; ni < 4; ++ni) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = m0 + wm * 64 + mi * 16 + (lane >> 2) + h * 8;
        if (r >= M) continue;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int cidx = n0 + wn * 32 + ni * 8 + (lane & 3) * 2 + e;
          if (cidx >= N) continue;
          float v = acc[mi][ni][h * 2 + e];
          if (ep.bias) v += ep.bias[cidx];
          if (ep.relu) v = v > 0.f ? v : 0.f;
          if (ep.mask && !(__bfloat162float(ep.mask[(size_t)r * ep.ldm + cidx]) > 0.f)) v = 0.f;
          if (ep.out_f32) ep.out_f32[(size_t)r * ep.ldc + cidx] = v;
          else ep.out_bf16[(size_t)r * ep.ldc + cidx] = __float2bfloat16_rn(v);
        }
      }
    }
  }
}

// out[c, r] = in[r, c] for an R x C block of a BF16 matrix.
__global__ void transpose_kernel(const bf16 *in, int ldi, bf16 *out, int ldo, int R, int C) {
  __shared__ bf16 tile[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += 8) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    tile[i][threadIdx.x] = (r < R && c < C) ? in[(size_t)r * ldi + c] : __float2bfloat16_rn(0.f);
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += 8) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (c < C && r < R) out[(size_t)c * ldo + r] = tile[threadIdx.x][i];
  }
}

__global__ void f32_to_bf16_kernel(const float *in, int rows, int cols, int ldi, bf16 *out, int ldo) {
  const int64_t total = (int64_t)rows * ldo;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / ldo), c = (int)(i % ldo);
    out[i] = __float2bfloat16_rn(c < cols ? in[(size_t)r * ldi + c] : 0.f);
  }
}

// dY = 2 (Y - T) / (B * n_valid) as BF16 (zero in padding columns) and the
// per-row squared errors (summed afterwards in a fixed order).
__global__ void loss_grad_kernel(const float *Y, int ldy, const float *T, int ldt, int B, int nvalid,
                                 bf16 *dY, double *row_sq) {
  __shared__ double scratch[256 / 32];
  const int r = blockIdx.x;
  const float scale = 2.f / ((float)B * (float)nvalid);
  double acc = 0.0;
  for (int c = threadIdx.x; c < ldy; c += blockDim.x) {
    float g = 0.f;
    if (c < nvalid) {
      const float d = Y[(size_t)r * ldy + c] - T[(size_t)r * ldt + c];
      acc += (double)d * (double)d;
      g = scale * d;
    }
    dY[(size_t)r * ldy + c] = __float2bfloat16_rn(g);
  }
  acc = block_sum<256>(acc, scratch);
  if (threadIdx.x == 0) row_sq[r] = acc;
}

__global__ void sum_rows_kernel(const double *row_sq, int B, double denom, double *loss) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int r = 0; r < B; ++r) s += row_sq[r];
    *loss = s / denom;
  }
}

// db[c] = sum over rows of d[r, c] (rows in order).
__global__ void colsum_kernel(const bf16 *d, int ld, int B, int N, float *db) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int r = 0; r < B; ++r) s += __bfloat162float(d[(size_t)r * ld + c]);
    db[c] = s;
  }
}

// Adam (Kingma & Ba) on FP32 master weights; refreshes the BF16 copy.
__global__ void adam_kernel(float *w, const float *g, float *m, float *v, bf16 *wb, int64_t count, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16_rn(wi);
  }
}

__global__ void to_bf16_kernel(const float *w, bf16 *wb, int64_t count) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    wb[i] = __float2bfloat16_rn(w[i]);
}

// Network output rows -> stacked starting iterates in double: row b holds
// [x (n) | y (m) | s (m)] in standardised units; value = out * std + mean.
__global__ void scatter_start_kernel(const float *Y, int ldy, int B, int n, int m, const float *mean,
                                     const float *stdv, double *x0, double *y0, double *s0) {
  const int64_t per = (int64_t)n + 2 * (int64_t)m;
  const int64_t total = per * B;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / per, c = i % per;
    const double v = (double)Y[b * ldy + c] * (double)stdv[c] + (double)mean[c];
    if (c < n) x0[b * n + c] = v;
    else if (c < n + m) y0[b * m + (c - n)] = v;
    else s0[b * m + (c - n - m)] = v;
  }
}

inline int pad8(int v) { return (v + 7) & ~7; }

inline int blocks_for(int64_t n, int per = 256) {
  int64_t g = (n + per - 1) / per;
  const int64_t cap = (int64_t)num_sms() * 16;
  return (int)std::max<int64_t>(1, std::min(g, cap));
}

class Net {
 public:
  ~Net() {
    if (stream_) {
      cudaStreamSynchronize(stream_);
      cudaStreamDestroy(stream_);
    }
  }
  int create(int n_in, int hidden, int n_out, int max_batch);
  int set_params(const float *const *w, const float *const *b);
  int get_params(float *const *w, float *const *b, bool grads);
  int forward(const float *x, int B, float *y);
  int train_step(const float *x, const float *t, int B, float lr, double *loss);
  int predict_start(const float *x, int B, const float *mean, const float *stdv, int n, int m, double *x0,
                    double *y0, double *s0);
  int time_forward(int B, int reps, double *ms, double *flops);
  cudaStream_t stream_ = nullptr;
  int64_t launches = 0;

 private:
  int gemm(const bf16 *A, int lda, const bf16 *B, int ldb, int M, int N, int K, const Epi &ep);
  int transpose(const bf16 *in, int ldi, bf16 *out, int ldo, int R, int C);
  int run_forward(int B);
  int dims_[4] = {0, 0, 0, 0};   // n_in, hidden, hidden, n_out
  int ld_[4] = {0, 0, 0, 0};     // padded to multiples of 8
  int max_batch_ = 0;
  int64_t step_ = 0;
  DeviceArena arena_;
  float *w_[3] = {}, *b_[3] = {}, *gw_[3] = {}, *gb_[3] = {};
  float *mw_[3] = {}, *vw_[3] = {}, *mb_[3] = {}, *vb_[3] = {};
  bf16 *wb_[3] = {}, *wt_[3] = {};  // BF16 weights [out, in_pad] and transposes [in, out_pad]
  bf16 *act_[4] = {};               // X0, H1, H2 (BF16), dY (BF16)
  bf16 *dh_[3] = {};                // gradients w.r.t. H1, H2
  bf16 *tr_a_ = nullptr, *tr_b_ = nullptr;  // transposed operands of the weight gradients
  float *y_ = nullptr;              // output [B, ld_out] FP32
  double *row_sq_ = nullptr, *loss_d_ = nullptr;
  float *x_stage_ = nullptr;
};

int Net::gemm(const bf16 *A, int lda, const bf16 *B, int ldb, int M, int N, int K, const Epi &ep) {
  if (M <= 0 || N <= 0) return PDOSGPU_OK;
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
  gemm_nt_kernel<<<grid, kThreads, 0, stream_>>>(A, lda, B, ldb, M, N, K, ep);
  PDOS_CUDA_TRY(cudaGetLastError());
  ++launches;
  return PDOSGPU_OK;
}

int Net::transpose(const bf16 *in, int ldi, bf16 *out, int ldo, int R, int C) {
  dim3 grid((C + 31) / 32, (R + 31) / 32), block(32, 8);
  transpose_kernel<<<grid, block, 0, stream_>>>(in, ldi, out, ldo, R, C);
  PDOS_CUDA_TRY(cudaGetLastError());
  ++launches;
  return PDOSGPU_OK;
}

int Net::create(int n_in, int hidden, int n_out, int max_batch) {
  if (n_in <= 0 || hidden <= 0 || n_out <= 0 || max_batch <= 0)
    return fail(PDOSGPU_EINVAL, "network sizes must be positive");
  dims_[0] = n_in;
  dims_[1] = dims_[2] = hidden;
  dims_[3] = n_out;
  for (int i = 0; i < 4; ++i) ld_[i] = pad8(dims_[i]);
  max_batch_ = pad8(max_batch);
  PDOS_CUDA_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  for (int l = 0; l < 3; ++l) {
    const int64_t rows = ld_[l + 1], cols = ld_[l];  // padded: zero rows / columns stay zero
    const int64_t cnt = rows * cols;
    PDOS_TRY(arena_.alloc(&w_[l], cnt));
    PDOS_TRY(arena_.alloc(&gw_[l], cnt));
    PDOS_TRY(arena_.alloc(&mw_[l], cnt));
    PDOS_TRY(arena_.alloc(&vw_[l], cnt));
    PDOS_TRY(arena_.alloc(&wb_[l], cnt));
    PDOS_TRY(arena_.alloc(&wt_[l], cnt));
    PDOS_TRY(arena_.alloc(&b_[l], rows));
    PDOS_TRY(arena_.alloc(&gb_[l], rows));
    PDOS_TRY(arena_.alloc(&mb_[l], rows));
    PDOS_TRY(arena_.alloc(&vb_[l], rows));
    for (float *p : {w_[l], gw_[l], mw_[l], vw_[l]}) PDOS_CUDA_TRY(cudaMemsetAsync(p, 0, sizeof(float) * cnt, stream_));
    for (float *p : {b_[l], gb_[l], mb_[l], vb_[l]}) PDOS_CUDA_TRY(cudaMemsetAsync(p, 0, sizeof(float) * rows, stream_));
    PDOS_CUDA_TRY(cudaMemsetAsync(wb_[l], 0, sizeof(bf16) * cnt, stream_));
    PDOS_CUDA_TRY(cudaMemsetAsync(wt_[l], 0, sizeof(bf16) * cnt, stream_));
  }
  for (int i = 0; i < 4; ++i) {
    const int ld = i < 3 ? ld_[i] : ld_[3];
    PDOS_TRY(arena_.alloc(&act_[i], (size_t)max_batch_ * ld));
    PDOS_CUDA_TRY(cudaMemsetAsync(act_[i], 0, sizeof(bf16) * (size_t)max_batch_ * ld, stream_));
  }
  for (int i = 1; i < 3; ++i) PDOS_TRY(arena_.alloc(&dh_[i], (size_t)max_batch_ * ld_[i]));
  const int64_t widest = std::max(std::max(ld_[0], ld_[1]), ld_[3]);
  PDOS_TRY(arena_.alloc(&tr_a_, (size_t)max_batch_ * widest));
  PDOS_TRY(arena_.alloc(&tr_b_, (size_t)max_batch_ * widest));
  PDOS_TRY(arena_.alloc(&y_, (size_t)max_batch_ * ld_[3]));
  PDOS_TRY(arena_.alloc(&row_sq_, (size_t)max_batch_));
  PDOS_TRY(arena_.alloc(&loss_d_, 1));
  PDOS_TRY(arena_.alloc(&x_stage_, (size_t)max_batch_ * ld_[0]));
  PDOS_CUDA_TRY(cudaStreamSynchronize(stream_));
  return PDOSGPU_OK;
}

// Host FP32 parameters in their natural shapes (W[l]: dims[l+1] x dims[l]).
int Net::set_params(const float *const *w, const float *const *b) {
  for (int l = 0; l < 3; ++l) {
    const int rows = dims_[l + 1], cols = dims_[l];
    PDOS_CUDA_TRY(cudaMemcpy2DAsync(w_[l], sizeof(float) * ld_[l], w[l], sizeof(float) * cols,
                                    sizeof(float) * cols, rows, cudaMemcpyHostToDevice, stream_));
    PDOS_CUDA_TRY(cudaMemcpyAsync(b_[l], b[l], sizeof(float) * rows, cudaMemcpyHostToDevice, stream_));
    const int64_t cnt = (int64_t)ld_[l + 1] * ld_[l];
    to_bf16_kernel<<<blocks_for(cnt), 256, 0, stream_>>>(w_[l], wb_[l], cnt);
    PDOS_CUDA_TRY(cudaGetLastError());
  }
  PDOS_CUDA_TRY(cudaStreamSynchronize(stream_));
  step_ = 0;
  return PDOSGPU_OK;
}

int Net::get_params(float *const *w, float *const *b, bool grads) {
  for (int l = 0; l < 3; ++l) {
    const int rows = dims_[l + 1], cols = dims_[l];
    const float *ws = grads ? gw_[l] : w_[l];
    const float *bs = grads ? gb_[l] : b_[l];
    if (w[l])
      PDOS_CUDA_TRY(cudaMemcpy2DAsync(w[l], sizeof(float) * cols, ws, sizeof(float) * ld_[l], sizeof(float) * cols,
                                      rows, cudaMemcpyDeviceToHost, stream_));
    if (b[l]) PDOS_CUDA_TRY(cudaMemcpyAsync(b[l], bs, sizeof(float) * rows, cudaMemcpyDeviceToHost, stream_));
  }
  PDOS_CUDA_TRY(cudaStreamSynchronize(stream_));
  return PDOSGPU_OK;
}

int Net::run_forward(int B) {
  // H1 = relu(X0 W1^T + b1), H2 = relu(H1 W2^T + b2), Y = H2 W3^T + b3
  Epi e1{b_[0], nullptr, 0, 1, nullptr, act_[1], ld_[1]};
  PDOS_TRY(gemm(act_[0], ld_[0], wb_[0], ld_[0], B, dims_[1], ld_[0], e1));
  Epi e2{b_[1], nullptr, 0, 1, nullptr, act_[2], ld_[2]};
  PDOS_TRY(gemm(act_[1], ld_[1], wb_[1], ld_[1], B, dims_[2], ld_[1], e2));
  Epi e3{b_[2], nullptr, 0, 0, y_, nullptr, ld_[3]};
  PDOS_TRY(gemm(act_[2], ld_[2], wb_[2], ld_[2], B, dims_[3], ld_[2], e3));
  return PDOSGPU_OK;
}

int Net::forward(const float *x, int B, float *y) {
  if (B <= 0 || B > max_batch_) return fail(PDOSGPU_EINVAL, "batch size out of range");
  f32_to_bf16_kernel<<<blocks_for((int64_t)B * ld_[0]), 256, 0, stream_>>>(x, B, dims_[0], dims_[0], act_[0], ld_[0]);
  PDOS_CUDA_TRY(cudaGetLastError());
  PDOS_TRY(run_forward(B));
  if (y)
    PDOS_CUDA_TRY(cudaMemcpy2DAsync(y, sizeof(float) * dims_[3], y_, sizeof(float) * ld_[3], sizeof(float) * dims_[3],
                                    B, cudaMemcpyDeviceToDevice, stream_));
  return PDOSGPU_OK;
}

int Net::train_step(const float *x, const float *t, int B, float lr, double *loss) {
  if (B <= 0 || B > max_batch_ || (B % 8) != 0)
    return fail(PDOSGPU_EINVAL, "training batch must be a positive multiple of 8 within the maximum");
  PDOS_TRY(forward(x, B, nullptr));
  const int H1 = dims_[1], H2 = dims_[2], NO = dims_[3], NI = dims_[0];
  loss_grad_kernel<<<B, 256, 0, stream_>>>(y_, ld_[3], t, NO, B, NO, act_[3], row_sq_);
  sum_rows_kernel<<<1, 32, 0, stream_>>>(row_sq_, B, (double)B * NO, loss_d_);
  PDOS_CUDA_TRY(cudaGetLastError());
  launches += 2;
  // layer 3: dW3 = dY^T H2, db3 = colsum dY, dH2 = (dY W3) * (H2 > 0)
  PDOS_TRY(transpose(act_[3], ld_[3], tr_a_, B, B, ld_[3]));   // dY^T  [ld3, B]
  PDOS_TRY(transpose(act_[2], ld_[2], tr_b_, B, B, ld_[2]));   // H2^T  [ld2, B]
  Epi g3{nullptr, nullptr, 0, 0, gw_[2], nullptr, ld_[2]};
  PDOS_TRY(gemm(tr_a_, B, tr_b_, B, NO, H2, B, g3));
  colsum_kernel<<<blocks_for(NO), 256, 0, stream_>>>(act_[3], ld_[3], B, NO, gb_[2]);
  PDOS_TRY(transpose(wb_[2], ld_[2], wt_[2], ld_[3], ld_[3], ld_[2]));  // W3^T [ld2, ld3]
  Epi d2{nullptr, act_[2], ld_[2], 0, nullptr, dh_[2], ld_[2]};
  PDOS_TRY(gemm(act_[3], ld_[3], wt_[2], ld_[3], B, H2, ld_[3], d2));
  // layer 2
  PDOS_TRY(transpose(dh_[2], ld_[2], tr_a_, B, B, ld_[2]));    // dH2^T [ld2, B]
  PDOS_TRY(transpose(act_[1], ld_[1], tr_b_, B, B, ld_[1]));   // H1^T  [ld1, B]
  Epi g2{nullptr, nullptr, 0, 0, gw_[1], nullptr, ld_[1]};
  PDOS_TRY(gemm(tr_a_, B, tr_b_, B, H2, H1, B, g2));
  colsum_kernel<<<blocks_for(H2), 256, 0, stream_>>>(dh_[2], ld_[2], B, H2, gb_[1]);
  PDOS_TRY(transpose(wb_[1], ld_[1], wt_[1], ld_[2], ld_[2], ld_[1]));  // W2^T [ld1, ld2]
  Epi d1{nullptr, act_[1], ld_[1], 0, nullptr, dh_[1], ld_[1]};
  PDOS_TRY(gemm(dh_[2], ld_[2], wt_[1], ld_[2], B, H1, ld_[2], d1));
  // layer 1
  PDOS_TRY(transpose(dh_[1], ld_[1], tr_a_, B, B, ld_[1]));    // dH1^T [ld1, B]
  PDOS_TRY(transpose(act_[0], ld_[0], tr_b_, B, B, ld_[0]));   // X0^T  [ld0, B]
  Epi g1{nullptr, nullptr, 0, 0, gw_[0], nullptr, ld_[0]};
  PDOS_TRY(gemm(tr_a_, B, tr_b_, B, H1, NI, B, g1));
  colsum_kernel<<<blocks_for(H1), 256, 0, stream_>>>(dh_[1], ld_[1], B, H1, gb_[0]);
  PDOS_CUDA_TRY(cudaGetLastError());
  launches += 3;
  // Adam
  ++step_;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - powf(b1, (float)step_), c2 = 1.f - powf(b2, (float)step_);
  for (int l = 0; l < 3; ++l) {
    const int64_t cnt = (int64_t)ld_[l + 1] * ld_[l];
    adam_kernel<<<blocks_for(cnt), 256, 0, stream_>>>(w_[l], gw_[l], mw_[l], vw_[l], wb_[l], cnt, lr, b1, b2, eps,
                                                       c1, c2);
    adam_kernel<<<blocks_for(ld_[l + 1]), 256, 0, stream_>>>(b_[l], gb_[l], mb_[l], vb_[l], nullptr, ld_[l + 1], lr,
                                                             b1, b2, eps, c1, c2);
  }
  PDOS_CUDA_TRY(cudaGetLastError());
  launches += 6;
  if (loss) {
    PDOS_CUDA_TRY(cudaMemcpyAsync(loss, loss_d_, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    PDOS_CUDA_TRY(cudaStreamSynchronize(stream_));
  }
  return PDOSGPU_OK;
}

int Net::predict_start(const float *x, int B, const float *mean, const float *stdv, int n, int m, double *x0,
                       double *y0, double *s0) {
  if ((int64_t)n + 2 * (int64_t)m != dims_[3])
    return fail(PDOSGPU_EINVAL, "n + 2m must equal the network's output width");
  PDOS_TRY(forward(x, B, nullptr));
  const int64_t total = (int64_t)B * dims_[3];
  scatter_start_kernel<<<blocks_for(total), 256, 0, stream_>>>(y_, ld_[3], B, n, m, mean, stdv, x0, y0, s0);
  PDOS_CUDA_TRY(cudaGetLastError());
  ++launches;
  return PDOSGPU_OK;
}

// Forward GEMMs alone, `reps` times on the current inputs: *flops = their
// algorithmic FLOPs (2 M N K per product).
int Net::time_forward(int B, int reps, double *ms, double *flops) {
  if (B <= 0 || B > max_batch_ || reps <= 0) return fail(PDOSGPU_EINVAL, "bad timing request");
  cudaEvent_t e0, e1;
  PDOS_CUDA_TRY(cudaEventCreate(&e0));
  PDOS_CUDA_TRY(cudaEventCreate(&e1));
  int rc = run_forward(B);
  cudaEventRecord(e0, stream_);
  for (int r = 0; r < reps && rc == PDOSGPU_OK; ++r) rc = run_forward(B);
  cudaEventRecord(e1, stream_);
  float t = 0.f;
  if (rc == PDOSGPU_OK && cudaEventSynchronize(e1) != cudaSuccess) rc = fail(PDOSGPU_ECUDA, "forward failed");
  if (rc == PDOSGPU_OK) cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  PDOS_TRY(rc);
  *ms = t / reps;
  if (flops)
    *flops = 2.0 * B * ((double)dims_[0] * dims_[1] + (double)dims_[1] * dims_[2] + (double)dims_[2] * dims_[3]);
  return PDOSGPU_OK;
}

}  // namespace mlp
}  // namespace pdosgpu

struct pdosgpu_mlp {
  pdosgpu::mlp::Net net;
};

using namespace pdosgpu;

extern "C" {

int pdosgpu_mlp_create(int n_in, int hidden, int n_out, int max_batch, pdosgpu_mlp **out) {
  if (!out) return fail(PDOSGPU_EINVAL, "NULL argument");
  *out = nullptr;
  int devs = 0;
  if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) return fail(PDOSGPU_ENOTSUP, "no CUDA device");
  auto p = new (std::nothrow) pdosgpu_mlp();
  if (!p) return fail(PDOSGPU_ENOMEM, "host allocation failed");
  const int rc = p->net.create(n_in, hidden, n_out, max_batch);
  if (rc != PDOSGPU_OK) {
    delete p;
    return rc;
  }
  *out = p;
  return PDOSGPU_OK;
}

int pdosgpu_mlp_set_params(pdosgpu_mlp *p, const float *w1, const float *b1, const float *w2, const float *b2,
                           const float *w3, const float *b3) {
  if (!p || !w1 || !b1 || !w2 || !b2 || !w3 || !b3) return fail(PDOSGPU_EINVAL, "NULL argument");
  const float *w[3] = {w1, w2, w3}, *b[3] = {b1, b2, b3};
  return p->net.set_params(w, b);
}

int pdosgpu_mlp_get_params(pdosgpu_mlp *p, int grads, float *w1, float *b1, float *w2, float *b2, float *w3,
                           float *b3) {
  if (!p) return fail(PDOSGPU_EINVAL, "NULL network");
  float *w[3] = {w1, w2, w3}, *b[3] = {b1, b2, b3};
  return p->net.get_params(w, b, grads != 0);
}

int pdosgpu_mlp_forward(pdosgpu_mlp *p, const float *x, int batch, float *y) {
  if (!p || !x) return fail(PDOSGPU_EINVAL, "NULL argument");
  return p->net.forward(x, batch, y);
}

int pdosgpu_mlp_train_step(pdosgpu_mlp *p, const float *x, const float *t, int batch, float lr, double *loss) {
  if (!p || !x || !t) return fail(PDOSGPU_EINVAL, "NULL argument");
  return p->net.train_step(x, t, batch, lr, loss);
}

int pdosgpu_mlp_predict_start(pdosgpu_mlp *p, const float *x, int batch, const float *mean, const float *stdv,
                              int64_t n, int64_t m, double *x0, double *y0, double *s0) {
  if (!p || !x || !mean || !stdv || !x0 || !y0 || !s0) return fail(PDOSGPU_EINVAL, "NULL argument");
  return p->net.predict_start(x, batch, mean, stdv, (int)n, (int)m, x0, y0, s0);
}

int pdosgpu_mlp_time_forward(pdosgpu_mlp *p, int batch, int reps, double *ms, double *flops) {
  if (!p || !ms) return fail(PDOSGPU_EINVAL, "NULL argument");
  return p->net.time_forward(batch, reps, ms, flops);
}

void *pdosgpu_mlp_stream(pdosgpu_mlp *p) { return p ? p->net.stream_ : nullptr; }

int pdosgpu_mlp_sync(pdosgpu_mlp *p) {
  if (!p) return fail(PDOSGPU_EINVAL, "NULL network");
  PDOS_CUDA_TRY(cudaStreamSynchronize(p->net.stream_));
  return PDOSGPU_OK;
}

void pdosgpu_mlp_free(pdosgpu_mlp *p) { delete p; }

}  // extern "C"
