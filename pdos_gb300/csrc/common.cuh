// Shared helpers of the GB300 PDOS kernels: error plumbing, warp/block
// reductions, the grid-reduction scratch and the device-side solver state.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

#include "../../include/pdos_gpu.h"

namespace pdosgpu {

// ---------------------------------------------------------------- errors
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);

#define PDOS_CUDA_TRY(call)                                                   \
  do {                                                                        \
    cudaError_t err_ = (call);                                                \
    if (err_ != cudaSuccess) {                                                \
      return ::pdosgpu::fail(PDOSGPU_ECUDA, std::string(#call) + ": " +       \
                                                cudaGetErrorString(err_));    \
    }                                                                         \
  } while (0)

#define PDOS_TRY(call)           \
  do {                           \
    int rc_ = (call);            \
    if (rc_ != PDOSGPU_OK) {     \
      return rc_;                \
    }                            \
  } while (0)

constexpr int kWarp = 32;

// ------------------------------------------------------------ reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum of `v` over the whole block, in a fixed tree order (deterministic).
// `scratch` must hold BLOCK/32 doubles; every thread gets the total.
template <int BLOCK>
__device__ __forceinline__ double block_sum(double v, double *scratch) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    t = lane < BLOCK / 32 ? scratch[lane] : 0.0;
    t = warp_sum(t);
    if (lane == 0) scratch[0] = t;
  }
  __syncthreads();
  t = scratch[0];
  __syncthreads();
  return t;
}

// Grid reduction scratch: every block of a reduction site writes NR block
// partials; the last block to arrive (ticket) sums all of them in a fixed
// order, so results are bit-identical run to run for a fixed grid.
struct GridReduce {
  double *partials;      // [slots * NR]
  unsigned int *ticket;  // one counter per site, returns to 0 after use
  int base;              // first slot of this kernel
  int slots_total;       // slots summed by the final block
  int final_kernel;      // 1: this kernel's last block does the final sum
};

// Writes this block's NR partials to slot base+blockIdx.x; returns true in
// the (single) last block of the final kernel, with tot[] = the grid totals.
template <int BLOCK, int NR>
__device__ bool grid_reduce(const GridReduce &g, double (&red)[NR],
                            double (&tot)[NR], double *scratch) {
  __shared__ bool s_last;
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    double v = block_sum<BLOCK>(red[i], scratch);
    if (threadIdx.x == 0) g.partials[(size_t)(g.base + blockIdx.x) * NR + i] = v;
  }
  if (!g.final_kernel) return false;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned prev = atomicAdd(g.ticket, 1u);
    s_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    double acc = 0.0;
    for (int b = threadIdx.x; b < g.slots_total; b += BLOCK)
      acc += __ldcg(&g.partials[(size_t)b * NR + i]);
    tot[i] = block_sum<BLOCK>(acc, scratch);
  }
  if (threadIdx.x == 0) *g.ticket = 0u;
  return true;
}

// ------------------------------------------------------------ solver state
// Scalars of one ADMM solve, resident in device memory.  Kernels read the
// flags at entry and return at once when there is nothing to do, so a
// captured iteration can be replayed past convergence harmlessly.
struct DevState {
  // constants
  double lambda, alpha_relax, eps, pscale, dscale, tol_sq;
  long long max_iters, cg_max;
  // CG scalars (indirect/private.c:31-104)
  double qsold, step, ratio;
  // reductions feeding the stop test (pdos.c:95-107)
  double pres_sq, by;
  // last residuals (reported)
  double p_res, d_res, p_obj, d_obj, eta;
  long long admm_iter, cg_total;
  int cg_iter, cg_active, done, solved, evaluated;
  int cg_skip;  // done || !cg_active, read by the CG SpMV kernels
  int diverged;  // a residual or the gap went non-finite: the solve stopped there
};

}  // namespace pdosgpu
