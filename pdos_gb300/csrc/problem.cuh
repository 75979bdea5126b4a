// Device set-up shared by the single-instance and the batched engines.
//
// A ProblemDesc describes one problem, or a batch of problems stacked
// block-diagonally (instance i owns rows [inst_row0[i], inst_row0[i+1]) and
// columns [inst_col0[i], inst_col0[i+1])).  Second-order cones are given by
// their absolute first row and size.  Everything done here acts on one row,
// one column or one cone at a time, so a stacked batch gets, instance by
// instance, the bits a single solve would get.
#pragma once

#include <cstdint>
#include <vector>

#include "admm_ops.cuh"
#include "engine.cuh"

namespace pdosgpu {

// The x-space ratio applied after equilibration (common.h:185-192): E, c and
// the matrix values are multiplied by it, a warm-start x is divided by it.
constexpr double kXRatio = 1e3;

struct ProblemDesc {
  int64_t n = 0, m = 0, nnz = 0;
  const double *Ax = nullptr;
  const int64_t *Ai = nullptr, *Ap = nullptr;  // CSC, absolute rows
  const double *b = nullptr, *c = nullptr;
  const double *x0 = nullptr, *y0 = nullptr, *s0 = nullptr;  // may be NULL
  std::vector<int64_t> soc_off, soc_len;      // absolute cone rows
  std::vector<int64_t> inst_row0, inst_col0;  // [B+1]
  int normalize = 0;
  int ruiz = 0;            // Ruiz equilibration (one instance only)
  int64_t ruiz_soc0 = 0;   // first cone row (f + l) for the Ruiz passes
};

template <typename T>
struct DeviceProblem {
  int32_t m = 0, n = 0, nnz = 0;
  int32_t *Ap = nullptr, *Ai = nullptr, *Rp = nullptr, *Rj = nullptr;  // padded by 16
  T *Ax = nullptr, *Rx = nullptr;                                      // padded by 16
  double *D64 = nullptr, *E64 = nullptr;  // row / column scaling (E includes x1e3)
  double *Epre64 = nullptr;               // E before the x-space ratio (warm starts)
  T *b = nullptr, *c = nullptr, *D = nullptr, *E = nullptr;
  T *x_init = nullptr, *y_init = nullptr, *s_init = nullptr;
  // per instance: lambda (common.h:182) and the DIMACS denominators of the
  // caller's b and c (pdos.c:76-77)
  std::vector<double> lambda, pscale, dscale;
  std::vector<int32_t> rp_host, ap_host;  // row pointers of A and of A' (host copies)
};

// Host-side checks of one problem (sizes, cone table, parameters).
int validate_problem(const pdosgpu_problem &pr);

// Upload, validate, transpose, equilibrate, scale the warm start, set lambda
// per instance and apply the x-space ratio.  Allocations go to `arena`.
template <typename T>
int setup_problem(const ProblemDesc &d, DeviceArena &arena, cudaStream_t st, DeviceProblem<T> &out);

// Cone tables of the grid projection kernels from absolute cone rows.
int build_cone_tables(const std::vector<int64_t> &off, const std::vector<int64_t> &len,
                      DeviceArena &arena, cudaStream_t st, ConeTables &ct, int *soc_grid,
                      int *socbig_grid);

}  // namespace pdosgpu
