// Cone projection that allocates no device memory.
//
// Some callers cannot call cudaMalloc while they solve: a process whose
// device memory is owned by a pool or framework allocator that must not be
// bypassed, code running inside a region that forbids allocation (real-time
// loops, callbacks that must not synchronise the device), or a host that has
// handed all free memory to another component.  For them this file offers one
// entry point, pdosgpu_proj_cone_f64_noalloc, computing the same projection as
// pdosgpu_proj_cone_f64 (projCone, cones.c:5-57) but keeping its scratch --
// cone offsets, per-chunk partial norms and cone heads -- in a fixed-size
// static device array instead of allocating it.
//
// The array below belongs to this file's module.  With CUDA's lazy module
// loading (the default), the driver loads the module, the array (about
// 3 MB) and each kernel into a context when they are first used there, and
// that memory stays until the context is destroyed.  So the first call in a
// context is the one that allocates: make one call per device (or per
// context) that projects at least one second-order cone and one zero or
// nonnegative row, so that every kernel of the projection has run, before
// any region that must not allocate and before any stream capture.  All
// calls share the array and it keeps the last call's contents; every slot a
// call reads is written earlier in the same call, so nothing has to start at
// zero.  Calls whose kernels overlap on the GPU (different streams, or
// different host threads on the same stream ordering) race on the array.
#include <cuda.h>

#include <mutex>

#include "admm_ops.cuh"

namespace pdosgpu {

namespace {

constexpr int kNaMaxCones = 1 << 16;   // second-order cones per call
constexpr int kNaMaxChunks = 1 << 17;  // 4096-row chunks over all cones per call
constexpr int kNaChunk = 4096;         // rows per chunk
constexpr int kNaBlock = 256;
constexpr int kNaScan = 1024;
constexpr int kNaMaxContexts = 64;

// layout of the static scratch (byte offsets)
constexpr size_t kNaQ = 0;                                         // int64 q[kNaMaxCones]
constexpr size_t kNaOff = kNaQ + 8 * (size_t)kNaMaxCones;          // int64 off[kNaMaxCones+1]
constexpr size_t kNaChunk0 = kNaOff + 8 * ((size_t)kNaMaxCones + 8);   // int32 chunk0[kNaMaxCones+1]
constexpr size_t kNaHead = kNaChunk0 + 4 * ((size_t)kNaMaxCones + 8);  // double head[kNaMaxCones]
constexpr size_t kNaSq = kNaHead + 8 * (size_t)kNaMaxCones;        // double chunk_sq[kNaMaxChunks]
constexpr size_t kNaBytes = kNaSq + 8 * (size_t)kNaMaxChunks;

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

namespace {

struct NaView {
  long long *q, *off;
  int *chunk0;
  double *head, *chunk_sq;
};

NaView na_view(unsigned char *base) {
  return NaView{reinterpret_cast<long long *>(base + kNaQ), reinterpret_cast<long long *>(base + kNaOff),
                reinterpret_cast<int *>(base + kNaChunk0), reinterpret_cast<double *>(base + kNaHead),
                reinterpret_cast<double *>(base + kNaSq)};
}

// cone offsets and chunk offsets: one block, sequential tiles of kNaScan
__global__ void __launch_bounds__(kNaScan) na_scan_kernel(NaView s, int ncones, long long row0) {
  __shared__ int warp_tot[kNaScan / 32];
  __shared__ long long warp_tot64[kNaScan / 32];
  __shared__ long long carry_rows;
  __shared__ int carry_chunks;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    carry_rows = row0;
    carry_chunks = 0;
  }
  __syncthreads();
  for (int base = 0; base < ncones; base += kNaScan) {
    const int i = base + threadIdx.x;
    const long long qi = i < ncones ? s.q[i] : 0;
    const int ci = i < ncones ? (int)((qi + kNaChunk - 1) / kNaChunk) : 0;
    long long xr = qi;
    int xc = ci;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long yr = __shfl_up_sync(0xffffffffu, xr, o);
      const int yc = __shfl_up_sync(0xffffffffu, xc, o);
      if (lane >= o) {
        xr += yr;
        xc += yc;
      }
    }
    if (lane == 31) {
      warp_tot64[warp] = xr;
      warp_tot[warp] = xc;
    }
    __syncthreads();
    if (warp == 0) {
      long long wr = warp_tot64[lane];
      int wc = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long yr = __shfl_up_sync(0xffffffffu, wr, o);
        const int yc = __shfl_up_sync(0xffffffffu, wc, o);
        if (lane >= o) {
          wr += yr;
          wc += yc;
        }
      }
      warp_tot64[lane] = wr;
      warp_tot[lane] = wc;
    }
    __syncthreads();
    const long long before_r = (warp > 0 ? warp_tot64[warp - 1] : 0) + xr - qi;
    const int before_c = (warp > 0 ? warp_tot[warp - 1] : 0) + xc - ci;
    if (i < ncones) {
      s.off[i] = carry_rows + before_r;
      s.chunk0[i] = carry_chunks + before_c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      carry_rows += warp_tot64[kNaScan / 32 - 1];
      carry_chunks += warp_tot[kNaScan / 32 - 1];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    s.off[ncones] = carry_rows;
    s.chunk0[ncones] = carry_chunks;
  }
}

__device__ __forceinline__ int na_cone_of_chunk(const NaView &s, int ncones, int c) {
  int lo = 0, hi = ncones;  // largest i with chunk0[i] <= c
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (s.chunk0[mid] <= c) lo = mid; else hi = mid;
  }
  return lo;
}

// per chunk: sum of squares of its tail rows; the cone's first chunk records
// the head value
__global__ void __launch_bounds__(kNaBlock) na_chunk_sq_kernel(NaView s, int ncones, const double *v) {
  __shared__ double scratch[kNaBlock / 32];
  const int c = blockIdx.x;
  const int cone = na_cone_of_chunk(s, ncones, c);
  const long long head = s.off[cone];
  const long long r0 = head + (long long)(c - s.chunk0[cone]) * kNaChunk;
  const long long r1 = min(r0 + kNaChunk, s.off[cone + 1]);
  double acc = 0.0;
  for (long long r = r0 + threadIdx.x; r < r1; r += kNaBlock)
    if (r != head) acc += v[r] * v[r];
  acc = block_sum<kNaBlock>(acc, scratch);
  if (threadIdx.x == 0) {
    s.chunk_sq[c] = acc;
    if (r0 == head) s.head[cone] = v[head];
  }
}

// per chunk: the cone's tail norm from its chunk sums (fixed order), then
// the three-case rule of cones.c:21-47 on the chunk's rows
__global__ void __launch_bounds__(kNaBlock) na_apply_kernel(NaView s, int ncones, double *v) {
  __shared__ double s_tail;
  const int c = blockIdx.x;
  const int cone = na_cone_of_chunk(s, ncones, c);
  if (threadIdx.x < 32) {
    double a = 0.0;
    for (int k = s.chunk0[cone] + threadIdx.x; k < s.chunk0[cone + 1]; k += 32) a += s.chunk_sq[k];
    a = warp_sum(a);
    if (threadIdx.x == 0) s_tail = sqrt(a);
  }
  __syncthreads();
  const double tail = s_tail, hv = s.head[cone];
  const long long head = s.off[cone];
  const long long r0 = head + (long long)(c - s.chunk0[cone]) * kNaChunk;
  const long long r1 = min(r0 + kNaChunk, s.off[cone + 1]);
  for (long long r = r0 + threadIdx.x; r < r1; r += kNaBlock) v[r] = soc_apply(v[r], r == head, hv, tail);
}

// Unique id of the calling thread's current context (cuCtxGetId: never
// reused within a process), or 0 when no context is current yet.  The
// driver functions are looked up through the runtime, so the library does
// not link libcuda.
int current_context_id(unsigned long long *id) {
  using GetCurrent = CUresult (*)(CUcontext *);
  using GetId = CUresult (*)(CUcontext, unsigned long long *);
  struct Fns {
    GetCurrent current = nullptr;
    GetId get_id = nullptr;
  };
  static const Fns fns = []() {  // thread-safe one-time look-up
    Fns f;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      f.current = reinterpret_cast<GetCurrent>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      f.get_id = reinterpret_cast<GetId>(p);
    return f;
  }();
  if (!fns.current || !fns.get_id) return fail(PDOSGPU_ECUDA, "driver entry points cuCtxGetCurrent/cuCtxGetId not found");
  CUcontext ctx = nullptr;
  if (fns.current(&ctx) != CUDA_SUCCESS) return fail(PDOSGPU_ECUDA, "cuCtxGetCurrent failed");
  *id = 0;
  if (ctx && fns.get_id(ctx, id) != CUDA_SUCCESS) return fail(PDOSGPU_ECUDA, "cuCtxGetId failed");
  return PDOSGPU_OK;
}

std::mutex g_na_mutex;
unsigned long long g_na_ctx[kNaMaxContexts] = {};  // context ids, 0 = free slot
void *g_na_ptr[kNaMaxContexts] = {};
int g_na_next = 0;  // slot to reuse once all are taken

// Device address of the static scratch in the current context.  The first
// call in a context looks it up (cudaGetSymbolAddress, which loads this
// module into the context if it is not loaded yet); later calls reuse it.
// The cache is keyed by the context's unique id, so a context destroyed and
// created again (cudaDeviceReset) gets a fresh look-up, never a stale
// address.
int na_scratch(unsigned char **out) {
  unsigned long long id = 0;
  PDOS_TRY(current_context_id(&id));
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (id != 0) {
    for (int i = 0; i < kNaMaxContexts; ++i) {
      if (g_na_ctx[i] == id) {
        *out = static_cast<unsigned char *>(g_na_ptr[i]);
        return PDOSGPU_OK;
      }
    }
  }
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return fail(PDOSGPU_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  if (id == 0) PDOS_TRY(current_context_id(&id));  // the look-up made the primary context current
  if (id != 0) {
    int slot = -1;
    for (int i = 0; i < kNaMaxContexts && slot < 0; ++i)
      if (g_na_ctx[i] == 0) slot = i;
    if (slot < 0) {
      slot = g_na_next;
      g_na_next = (g_na_next + 1) % kNaMaxContexts;
    }
    g_na_ctx[slot] = id;
    g_na_ptr[slot] = p;
  }
  *out = static_cast<unsigned char *>(p);
  return PDOSGPU_OK;
}

}  // namespace
}  // namespace pdosgpu

using namespace pdosgpu;

extern "C" int pdosgpu_proj_cone_f64_noalloc(double *v, int64_t f, int64_t l, int64_t qsize,
                                             const int64_t *q, void *stream) {
  if (f < 0 || l < 0 || qsize < 0 || (qsize > 0 && !q)) return fail(PDOSGPU_EINVAL, "bad cone");
  if (qsize > kNaMaxCones)
    return fail(PDOSGPU_EINVAL, "pdosgpu_proj_cone_f64_noalloc: more than 65536 second-order cones");
  int64_t m = f + l, nchunks = 0;
  for (int64_t i = 0; i < qsize; ++i) {
    if (q[i] <= 0) return fail(PDOSGPU_EINVAL, "cone sizes must be positive");
    m += q[i];
    nchunks += (q[i] + kNaChunk - 1) / kNaChunk;
  }
  if (nchunks > kNaMaxChunks)
    return fail(PDOSGPU_EINVAL,
                "pdosgpu_proj_cone_f64_noalloc: cones need more than 131072 chunks of 4096 rows");
  // the scratch address in this context (looked up by the first call made
  // in the context)
  unsigned char *base = nullptr;
  PDOS_TRY(na_scratch(&base));
  if (m == 0) return PDOSGPU_OK;
  if (!v) return fail(PDOSGPU_EINVAL, "NULL vector");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const NaView s = na_view(base);
  if (f + l > 0) {
    const int g = (int)std::min<int64_t>((f + l + 255) / 256, 4096);
    proj_lin_kernel<double><<<g, 256, 0, st>>>(v, f, l);
  }
  if (qsize > 0) {
    // q is host memory: a pageable q is staged by the driver before this
    // copy returns, so the caller may reuse q at once
    PDOS_CUDA_TRY(cudaMemcpyAsync(s.q, q, sizeof(int64_t) * qsize, cudaMemcpyHostToDevice, st));
    na_scan_kernel<<<1, kNaScan, 0, st>>>(s, (int)qsize, (long long)(f + l));
    na_chunk_sq_kernel<<<(int)nchunks, kNaBlock, 0, st>>>(s, (int)qsize, v);
    na_apply_kernel<<<(int)nchunks, kNaBlock, 0, st>>>(s, (int)qsize, v);
  }
  PDOS_CUDA_TRY(cudaGetLastError());
  return PDOSGPU_OK;
}
