// Learned warm start: a 3-layer perceptron (n_in -> hidden -> hidden ->
// n_out, ReLU) with BF16 weights and activations, FP32 accumulation, FP32
// master weights and Adam.  It maps the data of a parametrised problem
// family to a starting iterate (x0, y0, s0) for the solver (the reference's
// warm-start inputs Data.x/y/s, pdos.h:29-32, common.h:147-161); the solver,
// not the network, produces every reported result.
//
// Every product is C[M,N] = A[M,K] B[N,K]^T with both operands K-contiguous
// and a fused epilogue (bias, ReLU, multiplication by a ReLU mask, BF16 or
// FP32 output), on one of two tensor-core kernels with identical results:
// mma.sync m16n8k16 (ldmatrix fragments, cp.async double buffering; the
// default, faster at these sizes) or tcgen05.mma with accumulators in
// tensor memory (pdosgpu_mlp_set_kernel).  The backward pass transposes its
// operands into that form first.  Every reduction (loss, bias gradients) has
// a fixed order.
#include <cuda.h>
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

// ---------------------------------------------------------------------------
// The same product on the 5th-generation tensor cores: one thread issues
// tcgen05.mma (128 x 256 x 16 per instruction, BF16 in, FP32 accumulators in
// 256 columns of tensor memory) from shared-memory descriptors; tiles arrive
// by cp.async, four stages deep, in the canonical no-swizzle K-major layout
// (8 x 16-byte core matrices, 128 B each); a tcgen05.commit on a per-stage
// mbarrier tells the loaders when a stage is free; the four warps read the
// accumulators back with tcgen05.ld (one row per thread) and apply the same
// epilogue with 16-byte stores.  Every mbarrier wait is bounded: on timeout
// the kernel records an error flag, stops issuing, and still frees its
// tensor memory.
namespace tc {
constexpr int TM = 128, TN = 256, TK = 32;
constexpr int kThreads = 128;
constexpr int kATileBytes = TM * TK * 2;           // 8 KB
constexpr int kBTileBytes = TN * TK * 2;           // 16 KB
constexpr int kStageBytes = kATileBytes + kBTileBytes;
constexpr int kStages = 4;  // 97 KB: two CTAs per SM, 2 x 256 TMEM columns
constexpr int kSmemBytes = kStages * kStageBytes + 1024;  // stages + alignment
constexpr uint32_t kTmemCols = TN;                 // FP32 accumulators: 128 lanes x TN columns
constexpr long long kWaitCycles = 2000000000ll;  // about one second at 2 GHz
// instruction descriptor, kind::f16: FP32 accumulate (bit 4), A and B BF16
// (bits 7, 10), both K-major, N/8 at bit 17, M/16 at bit 24
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                            ((uint32_t)(TM >> 4) << 24);

// shared-memory matrix descriptor, no swizzle: start address, leading
// (K-direction) and stride (8-row direction) byte offsets, version 1
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// probe of an mbarrier phase (may suspend the thread briefly)
__device__ __forceinline__ bool mbar_try_wait(uint32_t addr, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(addr), "r"(parity)
      : "memory");
  return ok != 0;
}

// true if the phase completed within `limit` clock cycles (default about a
// second)
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t addr, uint32_t parity, long long limit = kWaitCycles) {
  const long long t0 = clock64();
  while (!mbar_try_wait(addr, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}

// The fused epilogue of one accumulator row chunk (32 columns starting at
// cb), with 16-byte accesses when the chunk lies inside the matrix.
__device__ __forceinline__ void store_row32(const Epi &ep, int r, int cb, int M, int N, const uint32_t (&v)[32]) {
  if (r < M && cb < N) {
    float x[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) x[j] = __uint_as_float(v[j]);
    const bool full = cb + 32 <= N;  // row chunk in range: 16-byte accesses
    if (ep.bias) {
#pragma unroll
      for (int j = 0; j < 32; ++j)
        if (full || cb + j < N) x[j] += __ldg(ep.bias + cb + j);
    }
    if (ep.relu) {
#pragma unroll
      for (int j = 0; j < 32; ++j) x[j] = x[j] > 0.f ? x[j] : 0.f;
    }
    if (ep.mask) {
      const bf16 *mrow = ep.mask + (size_t)r * ep.ldm + cb;
      if (full) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const uint4 w = *reinterpret_cast<const uint4 *>(mrow + 8 * q);
          const bf16 *h = reinterpret_cast<const bf16 *>(&w);
#pragma unroll
          for (int e = 0; e < 8; ++e)
            if (!(__bfloat162float(h[e]) > 0.f)) x[8 * q + e] = 0.f;
        }
      } else {
        for (int j = 0; j < 32 && cb + j < N; ++j)
          if (!(__bfloat162float(mrow[j]) > 0.f)) x[j] = 0.f;
      }
    }
    if (ep.out_f32) {
      float *o = ep.out_f32 + (size_t)r * ep.ldc + cb;
      if (full) {
#pragma unroll
        for (int q = 0; q < 8; ++q)
          *reinterpret_cast<float4 *>(o + 4 * q) = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
      } else {
        for (int j = 0; j < 32 && cb + j < N; ++j) o[j] = x[j];
      }
    } else {
      bf16 *o = ep.out_bf16 + (size_t)r * ep.ldc + cb;
      if (full) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          uint4 w;
          bf16 *h = reinterpret_cast<bf16 *>(&w);
#pragma unroll
          for (int e = 0; e < 8; ++e) h[e] = __float2bfloat16_rn(x[8 * q + e]);
          *reinterpret_cast<uint4 *>(o + 8 * q) = w;
        }
      } else {
        for (int j = 0; j < 32 && cb + j < N; ++j) o[j] = __float2bfloat16_rn(x[j]);
      }
    }
  }
}

__global__ void __launch_bounds__(kThreads) gemm_nt_tc_kernel(const bf16 *__restrict__ A, int lda,
                                                              const bf16 *__restrict__ B, int ldb, int M,
                                                              int N, int K, Epi ep, int *err) {
  extern __shared__ unsigned char raw[];
  __shared__ uint64_t mbar[kStages];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail;
  unsigned char *base = (unsigned char *)(((uintptr_t)raw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(base);
  const uint32_t mb0 = (uint32_t)__cvta_generic_to_shared(&mbar[0]);
  if (tid == 0) {
    s_fail = 0;
    for (int i = 0; i < kStages; ++i) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb0 + 8 * i));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    const uint32_t slot = (uint32_t)__cvta_generic_to_shared(&tmem_slot);
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  // one 16-byte chunk: row r, K chunk kc of a tile -> core (r/8, kc), row r%8
  auto load = [&](int stage, int k0) {
    const uint32_t a_s = sbase + stage * kStageBytes, b_s = a_s + kATileBytes;
#pragma unroll
    for (int i = 0; i < (TN * TK / 8) / kThreads; ++i) {  // B rows 0..TN-1, A rows 0..TM-1
      const int c = tid + i * kThreads;
      const int r = c / (TK / 8), kc = c % (TK / 8);
      const uint32_t off = (uint32_t)(((r >> 3) * (TK / 8) + kc) * 128 + (r & 7) * 16);
      const int gk = k0 + kc * 8;
      const bool kin = gk < K;
      const int gb = n0 + r;
      const bf16 *pb = B + (size_t)(gb < N ? gb : 0) * ldb + (kin ? gk : 0);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(b_s + off), "l"(pb),
                   "r"((gb < N && kin) ? 16 : 0));
      if (r < TM) {
        const int ga = m0 + r;
        const bf16 *pa = A + (size_t)(ga < M ? ga : 0) * lda + (kin ? gk : 0);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(a_s + off), "l"(pa),
                     "r"((ga < M && kin) ? 16 : 0));
      }
    }
    asm volatile("cp.async.commit_group;");
  };

  // Pipeline: tiles 0..kStages-2 in flight first; at step kt the products of
  // tile kt are issued, then the stage read by tile kt-1 is refilled with
  // tile kt+kStages-1 once those products have completed (its commit).  Every
  // completion of every stage's mbarrier is waited for exactly once, in order.
  const int nk = (K + TK - 1) / TK;
  bool ok = true;
  for (int t = 0; t < kStages - 1; ++t) {
    if (t < nk) load(t, t * TK);
    else asm volatile("cp.async.commit_group;");  // keep one group per tile
  }
  for (int kt = 0; kt < nk; ++kt) {
    const int st = kt % kStages;
    asm volatile("cp.async.wait_group %0;" ::"n"(kStages - 2) : "memory");  // tile kt has landed
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // cp.async data -> async proxy
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a_s = sbase + st * kStageBytes, b_s = a_s + kATileBytes;
#pragma unroll
      for (int s = 0; s < TK / 16; ++s) {  // K = 16 per product: two core matrices
        const uint64_t ad = smem_desc(a_s + s * 256, 128, (TK / 8) * 128);
        const uint64_t bd = smem_desc(b_s + s * 256, 128, (TK / 8) * 128);
        const uint32_t acc = (kt > 0 || s > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(kIdesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       mb0 + 8 * st)
                   : "memory");
    }
    const int nxt = kt + kStages - 1;  // tile refilling the stage of tile kt-1
    if (kt >= 1) {
      const int pt = kt - 1;
      if (tid == 0 && !mbar_wait_bounded(mb0 + 8 * (pt % kStages), (uint32_t)((pt / kStages) & 1))) s_fail = 1;
      __syncthreads();
      if (s_fail) {
        ok = false;
        break;
      }
    }
    if (nxt < nk) load(nxt % kStages, nxt * TK);
    else asm volatile("cp.async.commit_group;");
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  if (ok) {  // the last tile's products (the commit covers all earlier ones)
    const int lt = nk - 1;
    if (tid == 0 && !mbar_wait_bounded(mb0 + 8 * (lt % kStages), (uint32_t)((lt / kStages) & 1))) s_fail = 1;
    __syncthreads();
    ok = !s_fail;
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {  // accumulators: warp w holds rows 32w..32w+31 (TMEM lanes)
    const int r = m0 + warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < TN; c0 += 32) {
      uint32_t v[32];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
          "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
          "[%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
            "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
            "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
            "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      store_row32(ep, r, n0 + c0, M, N, v);
    }
  } else if (tid == 0) {
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}
}  // namespace tc

// ---------------------------------------------------------------------------
// The tcgen05 product fed by the Tensor Memory Accelerator: warp-specialised.
// Thread 0 of warp 0 streams stages with cp.async.bulk.tensor (host-encoded
// 2-D tensor maps of A and B, zero fill outside the matrices); thread 0 of
// warp 1 waits for each full stage, issues tcgen05.mma and commits the stage
// back to the producer; then all four warps drain tensor memory into the
// epilogue.  One TMA box per operand and stage, 64 K-elements (128 bytes)
// wide, lands with the 128-byte swizzle: rows of 128 bytes whose 16-byte
// chunks are permuted within each group of 8 rows (1,024 bytes).  The
// shared-memory descriptors name that layout (swizzle mode 2, 1,024 bytes
// between 8-row groups), and the four 16-deep products of a stage start 32
// bytes apart inside the swizzled rows.  Stages are 1,024-byte aligned.
namespace tma {
constexpr int TM = 128, TN = 256, TK = 64;
constexpr int kThreads = 128;
constexpr int kStages = 4;
constexpr int kABytes = TM * 128, kBBytes = TN * 128;  // 128-byte rows of 64 K-elements
constexpr int kStageBytes = kABytes + kBBytes;         // 48 KB
constexpr int kSmemBytes = kStages * kStageBytes + 1024;
constexpr uint32_t kTmemCols = TN;
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                            ((uint32_t)(TM >> 4) << 24);

// K-major operand in the 128-byte swizzled layout: start address, leading
// byte offset 16 (unused by this layout), 1,024 bytes between 8-row groups,
// version 1, swizzle mode 2 (128-byte).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(mbar)
      : "memory");
}

// test_wait > 0 (failure-path test only): before any copy or product, the
// CTA waits at most test_wait clock cycles on a barrier that nothing
// completes; the wait runs out, the CTA records the timeout in *err, issues
// nothing, frees its tensor memory and leaves its outputs unwritten.
__global__ void __launch_bounds__(kThreads) gemm_nt_tma_kernel(const __grid_constant__ CUtensorMap tmA,
                                                               const __grid_constant__ CUtensorMap tmB, int M,
                                                               int N, int K, Epi ep, int *err, long long test_wait) {
  extern __shared__ unsigned char raw[];
  __shared__ uint64_t full[kStages], empty[kStages], done, never;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail, s_issued;
  unsigned char *base = (unsigned char *)(((uintptr_t)raw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(base);
  const uint32_t fb = (uint32_t)__cvta_generic_to_shared(&full[0]);
  const uint32_t eb = (uint32_t)__cvta_generic_to_shared(&empty[0]);
  const uint32_t db = (uint32_t)__cvta_generic_to_shared(&done);
  if (tid == 0) {
    s_fail = 0;
    s_issued = 0;
    for (int i = 0; i < kStages; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(fb + 8 * i));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(eb + 8 * i));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(db));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t)__cvta_generic_to_shared(&never)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
  }
  if (warp == 2) {
    const uint32_t slot = (uint32_t)__cvta_generic_to_shared(&tmem_slot);
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const int nk = (K + TK - 1) / TK;
  if (test_wait > 0) {  // a wait that nothing completes (failure-path test)
    if (tid == 0 && !tc::mbar_wait_bounded((uint32_t)__cvta_generic_to_shared(&never), 0, test_wait)) s_fail = 1;
    __syncthreads();
  }

  if (warp == 0) {  // producer: lane 0 streams the stages
    if (lane == 0) {
    for (int kt = 0; kt < nk && !*(volatile int *)&s_fail; ++kt) {
      const int st = kt % kStages;
      if (kt >= kStages &&
          !tc::mbar_wait_bounded(eb + 8 * st, (uint32_t)(((kt / kStages) - 1) & 1))) {
        s_fail = 1;
        break;
      }
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb + 8 * st),
                   "r"((uint32_t)kStageBytes)
                   : "memory");
      const uint32_t a_s = sbase + st * kStageBytes, b_s = a_s + kABytes;
      const int x = kt * TK;  // a multiple of 64 elements: 128-byte aligned
      tma_load_2d(a_s, &tmA, x, m0, fb + 8 * st);
      tma_load_2d(b_s, &tmB, x, n0, fb + 8 * st);
      s_issued = kt + 1;
    }
    }
    __syncwarp();
  } else if (warp == 1) {  // products: lane 0 issues
    if (lane == 0) {
    for (int kt = 0; kt < nk && !*(volatile int *)&s_fail; ++kt) {
      const int st = kt % kStages;
      if (!tc::mbar_wait_bounded(fb + 8 * st, (uint32_t)((kt / kStages) & 1))) {
        s_fail = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a_s = sbase + st * kStageBytes, b_s = a_s + kABytes;
#pragma unroll
      for (int s = 0; s < TK / 16; ++s) {  // 16 K-elements (32 bytes) per product
        const uint64_t ad = sw128_desc(a_s + 32 * s);
        const uint64_t bd = sw128_desc(b_s + 32 * s);
        const uint32_t acc = (kt > 0 || s > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(kIdesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(eb + 8 * st)
                   : "memory");
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(db)
                 : "memory");
    }
    __syncwarp();
  }
  // everyone: the last commit covers every product
  // one verdict for the whole CTA: the epilogue's tensor-memory loads need
  // whole warps
  bool ok = __syncthreads_and(tc::mbar_wait_bounded(db, 0)) != 0;
  if (s_fail) ok = false;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    // Each warp passes its 32 x 32 accumulator blocks through a padded
    // shared tile (the operand stages are idle now), so that the epilogue
    // reads masks and writes outputs a row at a time with lane = column:
    // coalesced 128-byte (FP32) or 64-byte (BF16) rows instead of 32 rows
    // touched per store.  The arithmetic per element is store_row32's.
    float *tile = reinterpret_cast<float *>(base) + warp * (32 * 33);
    const int rbase = m0 + warp * 32;
#pragma unroll 1
    for (int c0 = 0; c0 < TN; c0 += 32) {
      uint32_t v[32];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
          "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
          "[%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
            "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
            "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
            "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      const int cb = n0 + c0;
      if (cb >= N) continue;  // uniform over the warp
#pragma unroll
      for (int j = 0; j < 32; ++j) tile[lane * 33 + j] = __uint_as_float(v[j]);
      __syncwarp();
      const int c = cb + lane;
      const bool cok = c < N;
      const float bj = (ep.bias && cok) ? __ldg(ep.bias + c) : 0.f;
      for (int i = 0; i < 32; ++i) {
        const int r = rbase + i;
        if (r >= M) break;  // uniform over the warp
        float x = tile[i * 33 + lane];
        if (ep.bias) x += bj;
        if (ep.relu) x = x > 0.f ? x : 0.f;
        if (cok) {
          if (ep.mask && !(__bfloat162float(ep.mask[(size_t)r * ep.ldm + c]) > 0.f)) x = 0.f;
          if (ep.out_f32) ep.out_f32[(size_t)r * ep.ldc + c] = x;
          else ep.out_bf16[(size_t)r * ep.ldc + c] = __float2bfloat16_rn(x);
        }
      }
      __syncwarp();
    }
  } else if (tid == 0) {
    atomicExch(err, 1);
    // wait (bounded) for the loads still in flight before the CTA leaves
    for (int kt = max(0, s_issued - kStages); kt < s_issued; ++kt)
      tc::mbar_wait_bounded(fb + 8 * (kt % kStages), (uint32_t)((kt / kStages) & 1));
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 2) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}
}  // namespace tma

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
  int set_gemm(int kind);
  int check();
  long long test_wait_ = 0;  // failure-path test of the bounded waits (0: off)
  int encode_map(CUtensorMap *map, const bf16 *p, int ld, int rows, int K, int box_rows);
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
  int *tc_err_ = nullptr;
  int gemm_kind_ = 0;
  float *x_stage_ = nullptr;
};

int Net::gemm(const bf16 *A, int lda, const bf16 *B, int ldb, int M, int N, int K, const Epi &ep) {
  if (M <= 0 || N <= 0) return PDOSGPU_OK;
  if (gemm_kind_ == 2) {
    CUtensorMap ma, mb;
    PDOS_TRY(encode_map(&ma, A, lda, M, K, tma::TM));
    PDOS_TRY(encode_map(&mb, B, ldb, N, K, tma::TN));
    dim3 grid((N + tma::TN - 1) / tma::TN, (M + tma::TM - 1) / tma::TM);
    tma::gemm_nt_tma_kernel<<<grid, tma::kThreads, tma::kSmemBytes, stream_>>>(ma, mb, M, N, K, ep, tc_err_,
                                                                              test_wait_);
  } else if (gemm_kind_ == 1) {
    dim3 grid((N + tc::TN - 1) / tc::TN, (M + tc::TM - 1) / tc::TM);
    tc::gemm_nt_tc_kernel<<<grid, tc::kThreads, tc::kSmemBytes, stream_>>>(A, lda, B, ldb, M, N, K, ep, tc_err_);
  } else {
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
    gemm_nt_kernel<<<grid, kThreads, 0, stream_>>>(A, lda, B, ldb, M, N, K, ep);
  }
  PDOS_CUDA_TRY(cudaGetLastError());
  ++launches;
  return PDOSGPU_OK;
}

// 0: mma.sync kernel, 1: tcgen05 fed by cp.async, 2: tcgen05 fed by TMA.
int Net::set_gemm(int kind) {
  if (kind < 0 || kind > 2) return fail(PDOSGPU_EINVAL, "unknown product kernel");
  if (kind == 1)
    PDOS_CUDA_TRY(cudaFuncSetAttribute(tc::gemm_nt_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       tc::kSmemBytes));
  if (kind == 2)
    PDOS_CUDA_TRY(cudaFuncSetAttribute(tma::gemm_nt_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       tma::kSmemBytes));
  gemm_kind_ = kind;
  return PDOSGPU_OK;
}

// 2-D tensor map of a row-major BF16 matrix (rows x K, leading dimension
// ld elements, a multiple of 8): boxes of 64 K-elements x box_rows rows
// written with the 128-byte swizzle, zero fill outside.
int Net::encode_map(CUtensorMap *map, const bf16 *p, int ld, int rows, int K, int box_rows) {
  if ((reinterpret_cast<uintptr_t>(p) & 15) || (ld & 7) || K <= 0 || rows <= 0)
    return fail(PDOSGPU_EINVAL, "tensor-map operand must be 16-byte aligned with ld a multiple of 8");
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(bf16)};
  const cuuint32_t box[2] = {(cuuint32_t)tma::TK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1u, 1u};
  // The driver entry point is looked up through the runtime, so the library
  // itself does not link libcuda (it loads on machines without a driver).
  using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static const EncodeTiled encode = []() -> EncodeTiled {  // thread-safe one-time look-up
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    return reinterpret_cast<EncodeTiled>(fn);
  }();
  if (!encode) return fail(PDOSGPU_ECUDA, "driver entry point cuTensorMapEncodeTiled not found");
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16 *>(p), dims, strides, box,
                            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(PDOSGPU_ECUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return PDOSGPU_OK;
}

// Nonzero if a tcgen05 product gave up waiting for its tensor cores.
int Net::check() {
  int h = 0;
  PDOS_CUDA_TRY(cudaMemcpyAsync(&h, tc_err_, sizeof(int), cudaMemcpyDeviceToHost, stream_));
  PDOS_CUDA_TRY(cudaStreamSynchronize(stream_));
  if (h) {  // reported once: the flag is cleared for the next products
    PDOS_CUDA_TRY(cudaMemsetAsync(tc_err_, 0, sizeof(int), stream_));
    PDOS_CUDA_TRY(cudaStreamSynchronize(stream_));
    return fail(PDOSGPU_ECUDA, "a tensor-core product timed out waiting for its operands");
  }
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
  PDOS_TRY(set_gemm(2));  // the TMA-fed tcgen05 products by default
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
  PDOS_TRY(arena_.alloc(&tc_err_, 1));
  PDOS_CUDA_TRY(cudaMemsetAsync(tc_err_, 0, sizeof(int), stream_));
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
  return p->net.check();
}

int pdosgpu_mlp_set_kernel(pdosgpu_mlp *p, int kind) {
  if (!p) return fail(PDOSGPU_EINVAL, "NULL network");
  return p->net.set_gemm(kind);
}

int pdosgpu_mlp_test_wait_timeout(pdosgpu_mlp *p, int64_t cycles) {
  if (!p) return fail(PDOSGPU_EINVAL, "NULL network");
  if (cycles < 0) return fail(PDOSGPU_EINVAL, "cycles must be nonnegative");
  PDOS_TRY(p->net.check());
  p->net.test_wait_ = cycles;
  return PDOSGPU_OK;
}

void pdosgpu_mlp_free(pdosgpu_mlp *p) { delete p; }

}  // extern "C"
