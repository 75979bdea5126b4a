// The C-ABI layer (pdos_gpu.h): workspace life cycle, error reporting and
// the kernel-level entry points on device memory.
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "admm_ops.cuh"
#include "engine.cuh"

struct pdosgpu_work {
  std::unique_ptr<pdosgpu::EngineBase> engine;
  int64_t max_iters = 0;
};

namespace pdosgpu {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg) {
  set_error(msg);
  return code;
}

int device_transpose(int m, int n, int nnz, const int32_t *Ap, const int32_t *Ai, int32_t *Rp,
                     int32_t *perm, int32_t *col_of, DeviceArena &tmp, cudaStream_t st);

namespace setup {
template <typename T>
__global__ void gather_kernel_api(const int32_t *perm, const T *src, T *dst, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    dst[i] = src[perm[i]];
}
__global__ void gather_col_kernel_api(const int32_t *perm, const int32_t *col_of, int32_t *Rj, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    Rj[i] = col_of[perm[i]];
}
}  // namespace setup

// Eight independent FP64 fused multiply-add chains per thread: the device's
// FP64 FMA issue rate, the second ceiling (beside HBM) of the FP64 SpMV,
// which executes one FMA per nonzero.
__global__ void fp64_fma_rate_kernel(double *sink, int iters) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 1e-3 * (threadIdx.x + k);
  const double mul = 0.999999999, add = 1e-12;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], mul, add);
  }
  double t = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) t += a[k];
  if (t == -1.0) *sink = t;  // never true; keeps the chains live
}

static int check_device() {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0)
    return fail(PDOSGPU_ENOTSUP, std::string("no CUDA device: ") + cudaGetErrorString(e));
  return PDOSGPU_OK;
}

template <typename T>
static int spmv_impl(int32_t rows, const int32_t *rowptr, const int32_t *colidx, const T *val,
                     const T *x, T sc, T *y, int accum, cudaStream_t st) {
  if (rows < 0) return fail(PDOSGPU_EINVAL, "rows must be nonnegative");
  if (rows == 0) return PDOSGPU_OK;
  if (!rowptr || !y || !x) return fail(PDOSGPU_EINVAL, "NULL pointer");
  std::vector<int32_t> rp(rows + 1);
  PDOS_CUDA_TRY(cudaMemcpyAsync(rp.data(), rowptr, sizeof(int32_t) * (rows + 1), cudaMemcpyDeviceToHost, st));
  PDOS_CUDA_TRY(cudaStreamSynchronize(st));
  for (int32_t r = 0; r < rows; ++r)
    if (rp[r + 1] < rp[r] || rp[0] != 0) return fail(PDOSGPU_EINVAL, "rowptr is not nondecreasing from 0");
  const int32_t nnz = rp[rows];
  if (nnz > 0 && (!colidx || !val)) return fail(PDOSGPU_EINVAL, "NULL pointer");
  // plan (slices of the caller's rows) and its scratch, freed on return
  DeviceArena arena;
  SellPlan<T> plan;
  PDOS_TRY(plan.build(rp.data(), rows, colidx, val, arena, st));
  GridReduce none{nullptr, nullptr, 0, plan.slots(), 0};
  plan.run(x, nullptr, OpAxpy<T>{x, y, sc, accum}, none, st);
  PDOS_CUDA_TRY(cudaGetLastError());
  PDOS_CUDA_TRY(cudaStreamSynchronize(st));  // before the plan is freed
  return PDOSGPU_OK;
}

}  // namespace pdosgpu

using namespace pdosgpu;

extern "C" {

const char *pdos_gpu_last_error(void) { return g_last_error.c_str(); }

void pdosgpu_default_options(pdosgpu_options *opt) {
  if (!opt) return;
  std::memset(opt, 0, sizeof(*opt));
  opt->precision = PDOSGPU_FP64;
  opt->scaling = PDOSGPU_SCALE_2NORM;
  opt->device = 0;
}

int pdosgpu_setup(const pdosgpu_problem *prob, const pdosgpu_options *opt, pdosgpu_work **out) {
  if (!prob || !out) return fail(PDOSGPU_EINVAL, "NULL argument");
  *out = nullptr;
  PDOS_TRY(check_device());
  pdosgpu_options o;
  pdosgpu_default_options(&o);
  if (opt) o = *opt;
  auto w = new (std::nothrow) pdosgpu_work();
  if (!w) return fail(PDOSGPU_ENOMEM, "host allocation failed");
  int rc = make_engine(*prob, o, w->engine);
  if (rc != PDOSGPU_OK) {
    delete w;
    return rc;
  }
  w->max_iters = prob->max_iters;
  *out = w;
  return PDOSGPU_OK;
}

int pdosgpu_solve(pdosgpu_work *w) {
  if (!w || !w->engine) return fail(PDOSGPU_EINVAL, "NULL workspace");
  return w->engine->iterate(w->max_iters, true);
}

int pdosgpu_iterate(pdosgpu_work *w, int64_t iters) {
  if (!w || !w->engine) return fail(PDOSGPU_EINVAL, "NULL workspace");
  if (iters < 0) return fail(PDOSGPU_EINVAL, "iters must be nonnegative");
  return w->engine->iterate(iters, false);
}

int pdosgpu_reset(pdosgpu_work *w) {
  if (!w || !w->engine) return fail(PDOSGPU_EINVAL, "NULL workspace");
  return w->engine->reset();
}

int pdosgpu_fetch(pdosgpu_work *w, double *x, double *s, double *y, pdosgpu_info *info) {
  if (!w || !w->engine) return fail(PDOSGPU_EINVAL, "NULL workspace");
  return w->engine->fetch(x, s, y, info);
}

void pdosgpu_free(pdosgpu_work *w) { delete w; }

void *pdosgpu_stream(pdosgpu_work *w) { return (w && w->engine) ? w->engine->stream() : nullptr; }

int pdosgpu_fp64_fma_rate(int device, double *fma_per_s) {
  PDOS_TRY(check_device());
  if (!fma_per_s) return fail(PDOSGPU_EINVAL, "NULL output");
  PDOS_CUDA_TRY(cudaSetDevice(device));
  int sms = 0;
  PDOS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  cudaStream_t st = nullptr;
  PDOS_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = PDOSGPU_OK;
  const int blocks = sms * 8, threads = 256, iters = 1 << 14;
  double *sink = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess ||
      cudaMalloc(&sink, sizeof(double)) != cudaSuccess)
    rc = fail(PDOSGPU_ECUDA, "event or buffer creation failed");
  float ms = 0.f;
  if (rc == PDOSGPU_OK) {
    fp64_fma_rate_kernel<<<blocks, threads, 0, st>>>(sink, iters);  // warm-up
    cudaEventRecord(e0, st);
    fp64_fma_rate_kernel<<<blocks, threads, 0, st>>>(sink, iters);
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.f)
      rc = fail(PDOSGPU_ECUDA, "FMA rate kernel failed");
  }
  if (sink) cudaFree(sink);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  PDOS_TRY(rc);
  *fma_per_s = (double)blocks * threads * 8.0 * iters / (ms / 1e3);
  return PDOSGPU_OK;
}

int pdosgpu_time_kernel(pdosgpu_work *w, int which, int reps, double *ms_per_launch) {
  if (!w || !w->engine) return fail(PDOSGPU_EINVAL, "NULL workspace");
  return w->engine->time_kernel(which, reps, ms_per_launch);
}

int pdosgpu_csc_to_csr_f64(int32_t m, int32_t n, int32_t nnz, const int32_t *Ap, const int32_t *Ai,
                           const double *Ax, int32_t *Rp, int32_t *Rj, double *Rx, void *stream) {
  if (m < 0 || n < 0 || nnz < 0) return fail(PDOSGPU_EINVAL, "negative size");
  if (!Rp || (nnz > 0 && (!Ap || !Ai || !Rj))) return fail(PDOSGPU_EINVAL, "NULL pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  DeviceArena tmp;
  int32_t *perm = nullptr, *col_of = nullptr;
  PDOS_TRY(tmp.alloc(&perm, (size_t)nnz));
  PDOS_TRY(tmp.alloc(&col_of, (size_t)nnz));
  PDOS_TRY(device_transpose(m, n, nnz, Ap, Ai, Rp, perm, col_of, tmp, st));
  if (nnz > 0) {
    const int grid = std::min((nnz + 255) / 256, 4096);
    setup::gather_col_kernel_api<<<grid, 256, 0, st>>>(perm, col_of, Rj, nnz);
    if (Rx && Ax) setup::gather_kernel_api<double><<<grid, 256, 0, st>>>(perm, Ax, Rx, nnz);
  }
  PDOS_CUDA_TRY(cudaGetLastError());
  PDOS_CUDA_TRY(cudaStreamSynchronize(st));
  return PDOSGPU_OK;
}

int pdosgpu_spmv_f64(int32_t rows, int32_t cols, const int32_t *rowptr, const int32_t *colidx,
                     const double *val, const double *x, double sc, double *y, int accum, void *stream) {
  (void)cols;
  return spmv_impl<double>(rows, rowptr, colidx, val, x, sc, y, accum, static_cast<cudaStream_t>(stream));
}

int pdosgpu_spmv_f32(int32_t rows, int32_t cols, const int32_t *rowptr, const int32_t *colidx,
                     const float *val, const float *x, float sc, float *y, int accum, void *stream) {
  (void)cols;
  return spmv_impl<float>(rows, rowptr, colidx, val, x, sc, y, accum, static_cast<cudaStream_t>(stream));
}

int pdosgpu_proj_cone_f64(double *v, int64_t f, int64_t l, int64_t qsize, const int64_t *q, void *stream) {
  if (f < 0 || l < 0 || qsize < 0 || (qsize > 0 && !q)) return fail(PDOSGPU_EINVAL, "bad cone");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int64_t m = f + l;
  for (int64_t i = 0; i < qsize; ++i) {
    if (q[i] <= 0) return fail(PDOSGPU_EINVAL, "cone sizes must be positive");
    m += q[i];
  }
  if (m == 0) return PDOSGPU_OK;
  if (!v) return fail(PDOSGPU_EINVAL, "NULL vector");
  if (m > (int64_t)INT32_MAX - 4096) return fail(PDOSGPU_EINVAL, "vector too long");
  std::vector<int32_t> small_off, small_len, row0, row1, cone, head, chunk0, nchunks;
  int64_t off = f + l;
  for (int64_t c = 0; c < qsize; ++c) {
    if (q[c] <= kSmallCone) {
      small_off.push_back((int32_t)off);
      small_len.push_back((int32_t)q[c]);
    } else {
      const int32_t big = (int32_t)head.size();
      head.push_back((int32_t)off);
      chunk0.push_back((int32_t)row0.size());
      int32_t k = 0;
      for (int64_t r = off; r < off + q[c]; r += kConeChunk, ++k) {
        row0.push_back((int32_t)r);
        row1.push_back((int32_t)std::min<int64_t>(off + q[c], r + kConeChunk));
        cone.push_back(big);
      }
      nchunks.push_back(k);
    }
    off += q[c];
  }
  DeviceArena arena;
  ConeTables ct{};
  auto up = [&](const std::vector<int32_t> &h, const int32_t **dst) -> int {
    int32_t *p = nullptr;
    PDOS_TRY(arena.alloc(&p, h.size() + 1));
    if (!h.empty())
      PDOS_CUDA_TRY(cudaMemcpyAsync(p, h.data(), sizeof(int32_t) * h.size(), cudaMemcpyHostToDevice, st));
    *dst = p;
    return PDOSGPU_OK;
  };
  PDOS_TRY(up(small_off, &ct.small_off));
  PDOS_TRY(up(small_len, &ct.small_len));
  PDOS_TRY(up(row0, &ct.chunk_row0));
  PDOS_TRY(up(row1, &ct.chunk_row1));
  PDOS_TRY(up(cone, &ct.chunk_cone));
  PDOS_TRY(up(head, &ct.big_head));
  PDOS_TRY(up(chunk0, &ct.big_chunk0));
  PDOS_TRY(up(nchunks, &ct.big_nchunks));
  ct.n_small = (int32_t)small_off.size();
  ct.n_chunks = (int32_t)row0.size();
  PDOS_TRY(arena.alloc(&ct.chunk_sq, row0.size() + 1));
  PDOS_TRY(arena.alloc(&ct.big_headval, head.size() + 1));
  if (f + l > 0) proj_lin_kernel<double><<<(int)std::min<int64_t>((f + l + 255) / 256, 4096), 256, 0, st>>>(v, f, l);
  if (ct.n_small > 0)
    proj_small_kernel<double, kBlock><<<std::min((ct.n_small + 7) / 8, 4096), kBlock, 0, st>>>(v, ct);
  if (ct.n_chunks > 0) {
    proj_chunk_sq_kernel<double, kBlock><<<ct.n_chunks, kBlock, 0, st>>>(v, ct);
    proj_chunk_apply_kernel<double, kBlock><<<ct.n_chunks, kBlock, 0, st>>>(v, ct);
  }
  PDOS_CUDA_TRY(cudaGetLastError());
  PDOS_CUDA_TRY(cudaStreamSynchronize(st));
  return PDOSGPU_OK;
}

}  // extern "C"
