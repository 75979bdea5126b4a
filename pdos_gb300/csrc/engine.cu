// Grid engine: set-up on the device, one captured CUDA graph per ADMM
// iteration, host loop that replays it until the device-side stop flag is
// set.  Instantiated for double (the reference's arithmetic) and float
// (float storage and SpMV, double reductions).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "batch_layout.h"
#include "engine.cuh"
#include "problem.cuh"
#include "setup_kernels.cuh"

namespace pdosgpu {

static thread_local int g_num_sms = 0;

int num_sms() {
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 1;
  }
  return g_num_sms;
}

namespace {

inline int grid1d(int64_t n, int block = 256) {
  int64_t g = (n + block - 1) / block;
  const int64_t cap = (int64_t)num_sms() * 16;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

template <class K>
int persistent_grid(K kernel, int block, size_t smem, int work) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
  if (per_sm < 1) per_sm = 1;
  int g = per_sm * num_sms();
  if (work < g) g = work;
  return g < 1 ? 1 : g;
}



double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

// ----------------------------------------------------------------- scan
int device_excl_scan(const int *in, int n, int *out, bool with_total, DeviceArena &tmp,
                     cudaStream_t st) {
  using namespace setup;
  if (n == 0) {
    if (with_total) PDOS_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(int), st));
    return PDOSGPU_OK;
  }
  const int nb = (n + kScanTile - 1) / kScanTile;
  int *sums = nullptr;
  PDOS_TRY(tmp.alloc(&sums, (size_t)nb + 1));
  scan_tile_sums<<<nb, kScanBlock, 0, st>>>(in, n, sums);
  scan_sums<<<1, kScanBlock, 0, st>>>(sums, nb);
  scan_apply<<<nb, kScanBlock, 0, st>>>(in, n, sums, out, with_total ? 1 : 0);
  PDOS_CUDA_TRY(cudaGetLastError());
  return PDOSGPU_OK;
}

// Stable CSC -> CSR: Rp (m+1) and the permutation perm[k] = CSC position of
// the k-th CSR entry; col_of[p] = column of CSC position p.
int device_transpose(int m, int n, int nnz, const int32_t *Ap, const int32_t *Ai, int32_t *Rp,
                     int32_t *perm, int32_t *col_of, DeviceArena &tmp, cudaStream_t st) {
  using namespace setup;
  int *cnt = nullptr;
  PDOS_TRY(tmp.alloc(&cnt, (size_t)m));
  PDOS_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)m, st));
  if (nnz > 0) count_rows_kernel<<<grid1d(nnz), 256, 0, st>>>(Ai, nnz, cnt);
  PDOS_TRY(device_excl_scan(cnt, m, Rp, true, tmp, st));
  if (nnz == 0) return PDOSGPU_OK;
  col_of_kernel<<<grid1d(nnz), 256, 0, st>>>(Ap, n, nnz, col_of);
  int32_t *ka, *kb, *va, *vb;
  PDOS_TRY(tmp.alloc(&ka, (size_t)nnz));
  PDOS_TRY(tmp.alloc(&kb, (size_t)nnz));
  PDOS_TRY(tmp.alloc(&va, (size_t)nnz));
  vb = perm;
  PDOS_CUDA_TRY(cudaMemcpyAsync(ka, Ai, sizeof(int32_t) * (size_t)nnz, cudaMemcpyDeviceToDevice, st));
  iota_kernel<<<grid1d(nnz), 256, 0, st>>>(va, nnz);
  int bits = 1;
  while (bits < 31 && (1 << bits) < m) ++bits;
  const int passes = (bits + 7) / 8;
  const int nblocks = (nnz + kRadixTile - 1) / kRadixTile;
  int *counts = nullptr;
  PDOS_TRY(tmp.alloc(&counts, (size_t)kRadixBins * nblocks));
  // ping-pong so that the last pass lands in `perm`
  int32_t *bufs_k[2] = {ka, kb};
  int32_t *bufs_v[2] = {va, vb};
  if (passes % 2 == 0) {
    bufs_v[0] = vb;
    bufs_v[1] = va;
    iota_kernel<<<grid1d(nnz), 256, 0, st>>>(vb, nnz);
  }
  for (int pass = 0; pass < passes; ++pass) {
    const int src = pass & 1, dst = src ^ 1;
    radix_hist<<<nblocks, kRadixBlock, 0, st>>>(bufs_k[src], nnz, pass * 8, counts, nblocks);
    PDOS_TRY(device_excl_scan(counts, kRadixBins * nblocks, counts, false, tmp, st));
    radix_scatter<<<nblocks, kRadixBlock, 0, st>>>(bufs_k[src], bufs_v[src], nnz, pass * 8, counts,
                                                     nblocks, bufs_k[dst], bufs_v[dst]);
  }
  PDOS_CUDA_TRY(cudaGetLastError());
  return PDOSGPU_OK;
}

// ============================================================== Engine<T>
template <typename T>
class Engine : public EngineBase {
 public:
  ~Engine() override {
    if (exec_) cudaGraphExecDestroy(exec_);
    for (auto e : extra_exec_)
      if (e) cudaGraphExecDestroy(e);
    if (stream_) {
      cudaStreamSynchronize(stream_);
      cudaStreamDestroy(stream_);
    }
    if (host_state_) cudaFreeHost(host_state_);
  }

  int setup(const pdosgpu_problem &pr, const pdosgpu_options &opt);
  int iterate(int64_t iters, bool until_done) override;
  int reset() override;
  int fetch(double *x, double *s, double *y, pdosgpu_info *info) override;
  int time_kernel(int which, int reps, double *ms) override;
  void *stream() override { return stream_; }

 private:
  int launch_iteration();
  int build_graph();
  int run_prep();
  int read_state();

  // sizes
  int32_t m_ = 0, n_ = 0, nnz_ = 0, f_ = 0, l_ = 0;
  int64_t qsize_ = 0;
  int64_t max_iters_ = 0, cg_max_ = 0;
  int verbose_ = 0;
  double lambda_ = 0, alpha_ = 1, eps_ = 0, tol_sq_ = 0, pscale_ = 1, dscale_ = 1;

  DeviceArena arena_;
  cudaStream_t stream_ = nullptr;
  cudaGraphExec_t exec_ = nullptr;
  std::vector<cudaGraphExec_t> extra_exec_;  // [top, cg block, tail] when split
  int cg_block_ = 0;
  int64_t nodes_main_ = 0, nodes_top_ = 0, nodes_cg_ = 0, nodes_tail_ = 0;
  DevState *S_ = nullptr;
  DevState *host_state_ = nullptr;

  // matrix in both layouts
  int32_t *Rp_ = nullptr, *Rj_ = nullptr, *Ap_ = nullptr, *Ai_ = nullptr;
  T *Rx_ = nullptr, *Ax_ = nullptr;
  SellPlan<T> sellA_, sellT_;  // A x (rows of A) and A' y (rows of A')
  // vectors
  Vecs<T> V_{};
  T *x_init_ = nullptr, *s_init_ = nullptr, *y_init_ = nullptr;
  double *D64_ = nullptr, *E64_ = nullptr, *out_ = nullptr;
  // reductions
  double *partials_ = nullptr;
  unsigned int *tickets_ = nullptr;
  // cones
  ConeTables ct_{};
  int soc_grid_ = 0, socbig_grid_ = 0;
  // grids
  int grid_upd_ = 1;
  int grid_dir_ = 1;
};

// ======================================================== validation
// Host-side checks of one problem (pdos.c:61-71, pdosmodule.c:94-311).
int validate_problem(const pdosgpu_problem &pr) {
  if (pr.n <= 0 || pr.m <= 0) return fail(PDOSGPU_EINVAL, "n and m must be positive");
  if (!pr.Ap || !pr.b || !pr.c) return fail(PDOSGPU_EINVAL, "Ap, b and c must not be NULL");
  const int64_t nnz64 = pr.Ap[pr.n];
  if (nnz64 < 0) return fail(PDOSGPU_EINVAL, "Ap[n] is negative");
  if (nnz64 > 0 && (!pr.Ai || !pr.Ax)) return fail(PDOSGPU_EINVAL, "Ai and Ax must not be NULL");
  const int64_t lim = (int64_t)INT32_MAX - 4096;
  if (pr.m > lim || pr.n > lim || nnz64 > lim)
    return fail(PDOSGPU_EINVAL, "m, n and nnz must each be below 2^31 - 4096");
  if (pr.f < 0 || pr.l < 0 || pr.qsize < 0 || (pr.qsize > 0 && !pr.q))
    return fail(PDOSGPU_EINVAL, "cone sizes must be nonnegative");
  int64_t rows = pr.f + pr.l;
  for (int64_t i = 0; i < pr.qsize; ++i) {
    if (pr.q[i] <= 0) return fail(PDOSGPU_EINVAL, "second-order cone sizes must be positive");
    rows += pr.q[i];
  }
  if (rows != pr.m) return fail(PDOSGPU_EINVAL, "m does not equal f + l + sum(q)");
  if (pr.max_iters < 0 || pr.cg_max_its < 0)
    return fail(PDOSGPU_EINVAL, "MAX_ITERS and CG_MAX_ITS must be nonnegative");
  if (!(pr.eps_abs >= 0) || !std::isfinite(pr.alpha) || !(pr.cg_tol >= 0))
    return fail(PDOSGPU_EINVAL, "EPS_ABS, ALPHA and CG_TOL must be finite and nonnegative");
  return PDOSGPU_OK;
}

// ======================================================== setup_problem
template <typename T>
int setup_problem(const ProblemDesc &d, DeviceArena &arena, cudaStream_t st, DeviceProblem<T> &P) {
  using namespace setup;
  const int m = (int)d.m, n = (int)d.n, nnz = (int)d.nnz;
  const int64_t ninst = (int64_t)d.inst_row0.size() - 1;
  const int64_t ncones = (int64_t)d.soc_off.size();
  if (ninst < 1 || (int64_t)d.inst_col0.size() != ninst + 1)
    return fail(PDOSGPU_EINVAL, "instance ranges are malformed");
  if (d.ruiz && ninst != 1) return fail(PDOSGPU_EINVAL, "Ruiz equilibration takes one instance");
  P.m = m;
  P.n = n;
  P.nnz = nnz;
  {  // DIMACS denominators from the caller's b and c (pdos.c:76-77)
    P.pscale.assign(ninst, 1.0);
    P.dscale.assign(ninst, 1.0);
    batch::parallel_for(ninst, [&](int64_t k) {  // instances in parallel, each summed in order
      double sb = 0.0, sc = 0.0;
      for (int64_t i = d.inst_row0[k]; i < d.inst_row0[k + 1]; ++i) sb += d.b[i] * d.b[i];
      for (int64_t j = d.inst_col0[k]; j < d.inst_col0[k + 1]; ++j) sc += d.c[j] * d.c[j];
      P.pscale[k] = 1.0 + std::sqrt(sb);
      P.dscale[k] = 1.0 + std::sqrt(sc);
    });
  }

  DeviceArena tmp;  // set-up temporaries
  // ---- upload and narrow
  int64_t *Ai64 = nullptr, *Ap64 = nullptr;
  double *Ax0 = nullptr, *b0 = nullptr, *c0 = nullptr;
  int *err = nullptr;
  PDOS_TRY(tmp.alloc(&Ai64, (size_t)nnz));
  PDOS_TRY(tmp.alloc(&Ap64, (size_t)n + 1));
  PDOS_TRY(tmp.alloc(&Ax0, (size_t)nnz));
  PDOS_TRY(tmp.alloc(&b0, (size_t)m));
  PDOS_TRY(tmp.alloc(&c0, (size_t)n));
  PDOS_TRY(tmp.alloc(&err, 1));
  // row pointer, index and value arrays are padded by 16 entries
  PDOS_TRY(arena.alloc(&P.Ap, (size_t)n + 16));
  PDOS_TRY(arena.alloc(&P.Ai, (size_t)nnz + 16));
  PDOS_TRY(arena.alloc(&P.Rp, (size_t)m + 16));
  PDOS_TRY(arena.alloc(&P.Rj, (size_t)nnz + 16));
  PDOS_CUDA_TRY(cudaMemsetAsync(P.Ap, 0, sizeof(int32_t) * ((size_t)n + 16), st));
  PDOS_CUDA_TRY(cudaMemsetAsync(P.Rp, 0, sizeof(int32_t) * ((size_t)m + 16), st));
  PDOS_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
  if (nnz > 0) {
    PDOS_CUDA_TRY(cudaMemcpyAsync(Ai64, d.Ai, sizeof(int64_t) * nnz, cudaMemcpyHostToDevice, st));
    PDOS_CUDA_TRY(cudaMemcpyAsync(Ax0, d.Ax, sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
  }
  PDOS_CUDA_TRY(cudaMemcpyAsync(Ap64, d.Ap, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, st));
  PDOS_CUDA_TRY(cudaMemcpyAsync(b0, d.b, sizeof(double) * m, cudaMemcpyHostToDevice, st));
  PDOS_CUDA_TRY(cudaMemcpyAsync(c0, d.c, sizeof(double) * n, cudaMemcpyHostToDevice, st));
  if (nnz > 0) {
    narrow_rows_kernel<<<grid1d(nnz), 256, 0, st>>>(Ai64, P.Ai, nnz, m, err);
    finite_check_kernel<<<grid1d(nnz), 256, 0, st>>>(Ax0, nnz, err, 4);
  }
  narrow_ptr_kernel<<<grid1d(n + 1), 256, 0, st>>>(Ap64, P.Ap, n, nnz, err);
  finite_check_kernel<<<grid1d(m), 256, 0, st>>>(b0, m, err, 4);
  finite_check_kernel<<<grid1d(n), 256, 0, st>>>(c0, n, err, 4);
  PDOS_CUDA_TRY(cudaGetLastError());
  int herr = 0;
  PDOS_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  PDOS_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr & 1) return fail(PDOSGPU_EINVAL, "row index out of range in Ai");
  if (herr & 2) return fail(PDOSGPU_EINVAL, "Ap is not a valid column pointer array");
  if (herr & 4) return fail(PDOSGPU_EINVAL, "A, b or c holds NaN or Inf");

  // ---- transpose (cs_transpose)
  int32_t *perm = nullptr, *col_of = nullptr;
  PDOS_TRY(tmp.alloc(&perm, (size_t)nnz));
  PDOS_TRY(tmp.alloc(&col_of, (size_t)nnz));
  PDOS_TRY(device_transpose(m, n, nnz, P.Ap, P.Ai, P.Rp, perm, col_of, tmp, st));
  if (nnz > 0) gather_col_kernel<<<grid1d(nnz), 256, 0, st>>>(perm, col_of, P.Rj, nnz);

  // ---- equilibration in double
  double *Aw = nullptr, *bw = nullptr, *cw = nullptr, *xw = nullptr, *yw = nullptr, *sw = nullptr;
  PDOS_TRY(tmp.alloc(&Aw, (size_t)nnz + 16));
  PDOS_TRY(tmp.alloc(&bw, (size_t)m));
  PDOS_TRY(tmp.alloc(&cw, (size_t)n));
  PDOS_TRY(tmp.alloc(&xw, (size_t)n));
  PDOS_TRY(tmp.alloc(&yw, (size_t)m));
  PDOS_TRY(tmp.alloc(&sw, (size_t)m));
  PDOS_TRY(arena.alloc(&P.D64, (size_t)m));
  PDOS_TRY(arena.alloc(&P.E64, (size_t)n));
  double *D64 = P.D64, *E64 = P.E64;
  PDOS_CUDA_TRY(cudaMemsetAsync(xw, 0, sizeof(double) * n, st));
  PDOS_CUDA_TRY(cudaMemsetAsync(yw, 0, sizeof(double) * m, st));
  PDOS_CUDA_TRY(cudaMemsetAsync(sw, 0, sizeof(double) * m, st));
  if (d.x0) PDOS_CUDA_TRY(cudaMemcpyAsync(xw, d.x0, sizeof(double) * n, cudaMemcpyHostToDevice, st));
  if (d.y0) PDOS_CUDA_TRY(cudaMemcpyAsync(yw, d.y0, sizeof(double) * m, cudaMemcpyHostToDevice, st));
  if (d.s0) PDOS_CUDA_TRY(cudaMemcpyAsync(sw, d.s0, sizeof(double) * m, cudaMemcpyHostToDevice, st));

  // cone row tables (host -> device)
  std::vector<int32_t> cone_of_row_h;
  int32_t *cone_of_row = nullptr;
  int64_t *cone_off = nullptr, *cone_len = nullptr;
  if (ncones > 0) {
    cone_of_row_h.assign(m, -1);
    auto fill = [&](int64_t c) {
      for (int64_t i = 0; i < d.soc_len[c]; ++i) cone_of_row_h[d.soc_off[c] + i] = (int32_t)c;
    };
    if (ninst > 1)  // a batch: cones of many instances, in parallel
      batch::parallel_for(ncones, fill);
    else
      for (int64_t c = 0; c < ncones; ++c) fill(c);
    PDOS_TRY(tmp.alloc(&cone_of_row, (size_t)m));
    PDOS_TRY(tmp.alloc(&cone_off, (size_t)ncones));
    PDOS_TRY(tmp.alloc(&cone_len, (size_t)ncones));
    PDOS_CUDA_TRY(cudaMemcpyAsync(cone_of_row, cone_of_row_h.data(), sizeof(int32_t) * m,
                                  cudaMemcpyHostToDevice, st));
    PDOS_CUDA_TRY(cudaMemcpyAsync(cone_off, d.soc_off.data(), sizeof(int64_t) * ncones,
                                  cudaMemcpyHostToDevice, st));
    PDOS_CUDA_TRY(cudaMemcpyAsync(cone_len, d.soc_len.data(), sizeof(int64_t) * ncones,
                                  cudaMemcpyHostToDevice, st));
  }

  const bool ruiz = d.normalize && d.ruiz;
  if (!d.normalize) {
    fill_kernel<<<grid1d(m), 256, 0, st>>>(D64, m, 1.0);
    fill_kernel<<<grid1d(n), 256, 0, st>>>(E64, n, 1.0);
    if (nnz > 0) PDOS_CUDA_TRY(cudaMemcpyAsync(Aw, Ax0, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, st));
  } else if (!ruiz) {
    // common.h:69-137
    double *Rx0 = nullptr;
    PDOS_TRY(tmp.alloc(&Rx0, (size_t)nnz));
    if (nnz > 0) gather_kernel<double><<<grid1d(nnz), 256, 0, st>>>(perm, Ax0, Rx0, nnz);
    row_sumsq_kernel<<<grid1d(m, 128), 128, 0, st>>>(P.Rp, Rx0, m, D64);
    if (ncones > 0) {
      double *mean = nullptr;
      PDOS_TRY(tmp.alloc(&mean, (size_t)ncones));
      cone_mean_kernel<<<grid1d(ncones, 128), 128, 0, st>>>(D64, cone_off, cone_len, (int)ncones, mean);
      cone_broadcast_kernel<<<grid1d(m), 256, 0, st>>>(D64, cone_of_row, mean, 0, m);
    }
    clamp_rsqrt_kernel<<<grid1d(m), 256, 0, st>>>(D64, m);
    if (nnz > 0) {
      PDOS_CUDA_TRY(cudaMemcpyAsync(Aw, Ax0, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, st));
      scale_by_row_kernel<<<grid1d(nnz), 256, 0, st>>>(Aw, P.Ai, D64, nnz);
    }
    col_sumsq_kernel<<<grid1d(n, 128), 128, 0, st>>>(P.Ap, Aw, n, E64);
    clamp_rsqrt_kernel<<<grid1d(n), 256, 0, st>>>(E64, n);
    if (nnz > 0) scale_by_col_kernel<<<grid1d(nnz), 256, 0, st>>>(Aw, col_of, E64, nnz);
  } else {
    // ruiz_equil_common.h:130-245
    const int64_t soc0 = d.ruiz_soc0;
    double *cv = nullptr, *cb = nullptr, *rowmax = nullptr, *colmax = nullptr, *sc = nullptr;
    int32_t *ci = nullptr;
    PDOS_TRY(tmp.alloc(&cv, (size_t)nnz));
    PDOS_TRY(tmp.alloc(&ci, (size_t)nnz));
    PDOS_TRY(tmp.alloc(&cb, (size_t)m));
    PDOS_TRY(tmp.alloc(&rowmax, (size_t)m));
    PDOS_TRY(tmp.alloc(&colmax, (size_t)n));
    PDOS_TRY(tmp.alloc(&sc, 4));
    if (ncones > 0) {
      int *head = nullptr, *run_excl = nullptr;
      PDOS_TRY(tmp.alloc(&head, (size_t)nnz));
      PDOS_TRY(tmp.alloc(&run_excl, (size_t)nnz + 1));
      if (nnz > 0) run_heads_kernel<<<grid1d(nnz), 256, 0, st>>>(P.Ai, cone_of_row, nnz, head);
      PDOS_TRY(device_excl_scan(head, nnz, run_excl, true, tmp, st));
      int nruns = 0;
      PDOS_CUDA_TRY(cudaMemcpyAsync(&nruns, run_excl + nnz, sizeof(int), cudaMemcpyDeviceToHost, st));
      PDOS_CUDA_TRY(cudaStreamSynchronize(st));
      double *runmax = nullptr;
      PDOS_TRY(tmp.alloc(&runmax, (size_t)nruns));
      PDOS_CUDA_TRY(cudaMemsetAsync(runmax, 0, sizeof(double) * (nruns > 0 ? nruns : 1), st));
      if (nnz > 0) {
        run_max_kernel<<<grid1d(nnz), 256, 0, st>>>(P.Ai, cone_of_row, Ax0, run_excl, head, nnz, runmax);
        run_apply_kernel<<<grid1d(nnz), 256, 0, st>>>(P.Ai, cone_of_row, cone_off, Ax0, run_excl, head,
                                                      runmax, nnz, cv, ci);
      }
      double *cmax = nullptr;
      PDOS_TRY(tmp.alloc(&cmax, (size_t)ncones));
      PDOS_CUDA_TRY(cudaMemsetAsync(cmax, 0, sizeof(double) * ncones, st));
      cone_absmax_kernel<<<grid1d(m - soc0), 256, 0, st>>>(b0, cone_of_row, soc0, m, cmax);
      cone_collapse_b_kernel<<<grid1d(m), 256, 0, st>>>(b0, cone_of_row, cmax, m, cb);
    } else {
      if (nnz > 0) {
        PDOS_CUDA_TRY(cudaMemcpyAsync(cv, Ax0, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, st));
        PDOS_CUDA_TRY(cudaMemcpyAsync(ci, P.Ai, sizeof(int32_t) * nnz, cudaMemcpyDeviceToDevice, st));
      }
      PDOS_CUDA_TRY(cudaMemcpyAsync(cb, b0, sizeof(double) * m, cudaMemcpyDeviceToDevice, st));
    }
    fill_kernel<<<grid1d(m), 256, 0, st>>>(D64, m, 1.0);
    fill_kernel<<<grid1d(n), 256, 0, st>>>(E64, n, 1.0);
    PDOS_CUDA_TRY(cudaMemsetAsync(rowmax, 0, sizeof(double) * m, st));
    PDOS_CUDA_TRY(cudaMemsetAsync(colmax, 0, sizeof(double) * n, st));
    const double sc_init[4] = {1.0, 1.0, 0.0, 0.0};
    PDOS_CUDA_TRY(cudaMemcpyAsync(sc, sc_init, sizeof(sc_init), cudaMemcpyHostToDevice, st));
    for (int pass = 0; pass < 3; ++pass) {
      if (nnz > 0) ruiz_rowmax_kernel<<<grid1d(nnz), 256, 0, st>>>(cv, ci, col_of, E64, nnz, rowmax);
      ruiz_lastpi_kernel<<<grid1d(n), 256, 0, st>>>(c0, E64, n, sc);
      ruiz_row_finish_kernel<<<grid1d(m), 256, 0, st>>>(cb, sc, m, rowmax);
      if (ncones > 0)
        ruiz_cone_rows_kernel<<<grid1d(m - soc0), 256, 0, st>>>(cone_of_row, cone_off, soc0, m, rowmax);
      ruiz_update_kernel<<<grid1d(m), 256, 0, st>>>(D64, rowmax, m);
      ruiz_last_kernel<<<1, 32, 0, st>>>(sc, 0);
      ruiz_colmax_kernel<<<grid1d(n, 128), 128, 0, st>>>(P.Ap, cv, ci, D64, c0, sc, n, colmax);
      ruiz_lastdelta_kernel<<<grid1d(m), 256, 0, st>>>(cb, D64, m, sc);
      ruiz_update_kernel<<<grid1d(n), 256, 0, st>>>(E64, colmax, n);
      ruiz_last_kernel<<<1, 32, 0, st>>>(sc, 1);
    }
    if (nnz > 0) ruiz_scale_kernel<<<grid1d(nnz), 256, 0, st>>>(Ax0, P.Ai, col_of, D64, E64, nnz, Aw);
  }
  // c, b and the warm start (common.h:139-161); lambda (common.h:182);
  // x-space ratio (common.h:185-192)
  if (d.normalize) {
    vec_scale_kernel<<<grid1d(n), 256, 0, st>>>(c0, E64, cw, n, 0);
    vec_scale_kernel<<<grid1d(m), 256, 0, st>>>(b0, D64, bw, m, 0);
    vec_scale_kernel<<<grid1d(m), 256, 0, st>>>(yw, D64, yw, m, 1);
    vec_scale_kernel<<<grid1d(n), 256, 0, st>>>(xw, E64, xw, n, 1);
    vec_scale_kernel<<<grid1d(m), 256, 0, st>>>(sw, D64, sw, m, 0);
  } else {
    PDOS_CUDA_TRY(cudaMemcpyAsync(cw, c0, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    PDOS_CUDA_TRY(cudaMemcpyAsync(bw, b0, sizeof(double) * m, cudaMemcpyDeviceToDevice, st));
  }
  {
    // lambda = (guard + ||b||) / (guard + ||c||) on the scaled data of each
    // instance, summed sequentially on the host in the reference's order
    // (common.h:182)
    std::vector<double> hb(m), hc(n);
    PDOS_CUDA_TRY(cudaMemcpyAsync(hb.data(), bw, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
    PDOS_CUDA_TRY(cudaMemcpyAsync(hc.data(), cw, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    PDOS_CUDA_TRY(cudaStreamSynchronize(st));
    const double guard = ruiz ? 1e-6 : 1e-15;
    P.lambda.assign(ninst, 1.0);
    batch::parallel_for(ninst, [&](int64_t k) {
      double sb = 0.0, sc = 0.0;
      for (int64_t i = d.inst_row0[k]; i < d.inst_row0[k + 1]; ++i) sb += hb[i] * hb[i];
      for (int64_t j = d.inst_col0[k]; j < d.inst_col0[k + 1]; ++j) sc += hc[j] * hc[j];
      P.lambda[k] = (guard + std::sqrt(sb)) / (guard + std::sqrt(sc));
    });
  }
  PDOS_TRY(arena.alloc(&P.Epre64, (size_t)n));
  PDOS_CUDA_TRY(cudaMemcpyAsync(P.Epre64, E64, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  scal_kernel<<<grid1d(n), 256, 0, st>>>(E64, n, kXRatio, 0);
  scal_kernel<<<grid1d(n), 256, 0, st>>>(cw, n, kXRatio, 0);
  scal_kernel<<<grid1d(n), 256, 0, st>>>(xw, n, kXRatio, 1);
  if (nnz > 0) scal_kernel<<<grid1d(nnz), 256, 0, st>>>(Aw, nnz, kXRatio, 0);
  PDOS_CUDA_TRY(cudaGetLastError());

  // ---- working arrays in T
  PDOS_TRY(arena.alloc(&P.Ax, (size_t)nnz + 16));
  PDOS_TRY(arena.alloc(&P.Rx, (size_t)nnz + 16));
  PDOS_TRY(arena.alloc(&P.b, (size_t)m));
  PDOS_TRY(arena.alloc(&P.c, (size_t)n));
  PDOS_TRY(arena.alloc(&P.D, (size_t)m));
  PDOS_TRY(arena.alloc(&P.E, (size_t)n));
  if (nnz > 0) {
    double *Rxd = nullptr;
    PDOS_TRY(tmp.alloc(&Rxd, (size_t)nnz));
    gather_kernel<double><<<grid1d(nnz), 256, 0, st>>>(perm, Aw, Rxd, nnz);
    convert_kernel<T><<<grid1d(nnz), 256, 0, st>>>(Aw, P.Ax, nnz);
    convert_kernel<T><<<grid1d(nnz), 256, 0, st>>>(Rxd, P.Rx, nnz);
  }
  convert_kernel<T><<<grid1d(m), 256, 0, st>>>(bw, P.b, m);
  convert_kernel<T><<<grid1d(n), 256, 0, st>>>(cw, P.c, n);
  convert_kernel<T><<<grid1d(m), 256, 0, st>>>(D64, P.D, m);
  convert_kernel<T><<<grid1d(n), 256, 0, st>>>(E64, P.E, n);
  PDOS_TRY(arena.alloc(&P.x_init, (size_t)n));
  PDOS_TRY(arena.alloc(&P.y_init, (size_t)m));
  PDOS_TRY(arena.alloc(&P.s_init, (size_t)m));
  convert_kernel<T><<<grid1d(n), 256, 0, st>>>(xw, P.x_init, n);
  convert_kernel<T><<<grid1d(m), 256, 0, st>>>(yw, P.y_init, m);
  convert_kernel<T><<<grid1d(m), 256, 0, st>>>(sw, P.s_init, m);
  PDOS_CUDA_TRY(cudaGetLastError());

  // ---- host copies of both pointer arrays (for the SpMV layouts)
  P.rp_host.assign((size_t)m + 1, 0);
  P.ap_host.assign((size_t)n + 1, 0);
  PDOS_CUDA_TRY(cudaMemcpyAsync(P.rp_host.data(), P.Rp, sizeof(int32_t) * (m + 1), cudaMemcpyDeviceToHost, st));
  PDOS_CUDA_TRY(cudaStreamSynchronize(st));
  batch::parallel_for((n + 1 + 65535) / 65536, [&](int64_t c) {  // one chunk (no thread) below 65,536
    for (int64_t j = c * 65536; j < std::min<int64_t>(n + 1, (c + 1) * 65536); ++j) P.ap_host[j] = (int32_t)d.Ap[j];
  });
  tmp.release();
  return PDOSGPU_OK;
}

template int setup_problem<double>(const ProblemDesc &, DeviceArena &, cudaStream_t, DeviceProblem<double> &);
template int setup_problem<float>(const ProblemDesc &, DeviceArena &, cudaStream_t, DeviceProblem<float> &);

// Cone tables of the grid projection kernels: cones of at most kSmallCone
// rows go to one warp each, larger ones are cut into kConeChunk-row chunks.
int build_cone_tables(const std::vector<int64_t> &off_in, const std::vector<int64_t> &len_in,
                      DeviceArena &arena, cudaStream_t st, ConeTables &ct, int *soc_grid,
                      int *socbig_grid) {
  std::vector<int32_t> small_off, small_len, chunk_row0, chunk_row1, chunk_cone, big_head, big_chunk0,
      big_nchunks;
  const int64_t ncones = (int64_t)off_in.size();
  for (int64_t c = 0; c < ncones; ++c) {
    const int64_t off = off_in[c], q = len_in[c];
    if (q <= kSmallCone) {
      small_off.push_back((int32_t)off);
      small_len.push_back((int32_t)q);
    } else {
      const int32_t big = (int32_t)big_head.size();
      big_head.push_back((int32_t)off);
      big_chunk0.push_back((int32_t)chunk_row0.size());
      int32_t nch = 0;
      for (int64_t r = off; r < off + q; r += kConeChunk) {
        chunk_row0.push_back((int32_t)r);
        chunk_row1.push_back((int32_t)std::min<int64_t>(off + q, r + kConeChunk));
        chunk_cone.push_back(big);
        ++nch;
      }
      big_nchunks.push_back(nch);
    }
  }
  auto up = [&](const std::vector<int32_t> &v, const int32_t **dst) -> int {
    int32_t *p = nullptr;
    PDOS_TRY(arena.alloc(&p, v.size() + 1));
    if (!v.empty())
      PDOS_CUDA_TRY(cudaMemcpyAsync(p, v.data(), sizeof(int32_t) * v.size(), cudaMemcpyHostToDevice, st));
    *dst = p;
    return PDOSGPU_OK;
  };
  PDOS_TRY(up(small_off, &ct.small_off));
  PDOS_TRY(up(small_len, &ct.small_len));
  PDOS_TRY(up(chunk_row0, &ct.chunk_row0));
  PDOS_TRY(up(chunk_row1, &ct.chunk_row1));
  PDOS_TRY(up(chunk_cone, &ct.chunk_cone));
  PDOS_TRY(up(big_head, &ct.big_head));
  PDOS_TRY(up(big_chunk0, &ct.big_chunk0));
  PDOS_TRY(up(big_nchunks, &ct.big_nchunks));
  ct.n_small = (int32_t)small_off.size();
  ct.n_chunks = (int32_t)chunk_row0.size();
  PDOS_TRY(arena.alloc(&ct.chunk_sq, chunk_row0.size() + 1));
  PDOS_TRY(arena.alloc(&ct.big_headval, big_head.size() + 1));
  const int warps = kBlock / 32;
  ct.small_blocks = ct.n_small > 0 ? std::min((ct.n_small + warps - 1) / warps, num_sms() * 8) : 0;
  *soc_grid = ncones > 0 ? ct.small_blocks + ct.n_chunks : 0;
  *socbig_grid = ct.n_chunks;
  // the host vectors above go out of scope: wait for their copies
  PDOS_CUDA_TRY(cudaStreamSynchronize(st));
  return PDOSGPU_OK;
}

// ============================================================== Engine<T>
template <typename T>
int Engine<T>::setup(const pdosgpu_problem &pr, const pdosgpu_options &opt) {
  const double t0 = now_ms();
  PDOS_TRY(validate_problem(pr));
  const int64_t nnz64 = pr.Ap[pr.n];

  m_ = (int32_t)pr.m;
  n_ = (int32_t)pr.n;
  nnz_ = (int32_t)nnz64;
  f_ = (int32_t)pr.f;
  l_ = (int32_t)pr.l;
  qsize_ = pr.qsize;
  max_iters_ = pr.max_iters;
  cg_max_ = pr.cg_max_its;
  verbose_ = (int)pr.verbose;
  alpha_ = pr.alpha;
  eps_ = pr.eps_abs;
  tol_sq_ = pr.cg_tol * pr.cg_tol;

  ProblemDesc d;
  d.n = pr.n;
  d.m = pr.m;
  d.nnz = nnz64;
  d.Ax = pr.Ax;
  d.Ai = pr.Ai;
  d.Ap = pr.Ap;
  d.b = pr.b;
  d.c = pr.c;
  d.x0 = pr.x0;
  d.y0 = pr.y0;
  d.s0 = pr.s0;
  d.inst_row0 = {0, pr.m};
  d.inst_col0 = {0, pr.n};
  d.normalize = pr.normalize ? 1 : 0;
  d.ruiz = (pr.normalize && opt.scaling == PDOSGPU_SCALE_RUIZ) ? 1 : 0;
  d.ruiz_soc0 = pr.f + pr.l;
  {
    int64_t off = pr.f + pr.l;
    for (int64_t c = 0; c < pr.qsize; ++c) {
      d.soc_off.push_back(off);
      d.soc_len.push_back(pr.q[c]);
      off += pr.q[c];
    }
  }

  PDOS_CUDA_TRY(cudaSetDevice(opt.device));
  g_num_sms = 0;
  PDOS_CUDA_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  cudaStream_t st = stream_;
  const int m = m_, n = n_;

  DeviceProblem<T> P;
  PDOS_TRY(setup_problem<T>(d, arena_, st, P));
  lambda_ = P.lambda[0];
  pscale_ = P.pscale[0];
  dscale_ = P.dscale[0];
  Ap_ = P.Ap;
  Ai_ = P.Ai;
  Rp_ = P.Rp;
  Rj_ = P.Rj;
  Ax_ = P.Ax;
  Rx_ = P.Rx;
  D64_ = P.D64;
  E64_ = P.E64;
  x_init_ = P.x_init;
  y_init_ = P.y_init;
  s_init_ = P.s_init;

  V_.m = m;
  V_.n = n;
  V_.f = f_;
  V_.l = l_;
  V_.b = P.b;
  V_.c = P.c;
  V_.D = P.D;
  V_.E = P.E;
  PDOS_TRY(arena_.alloc(&V_.x, (size_t)n));
  PDOS_TRY(arena_.alloc(&V_.p, (size_t)n));
  PDOS_TRY(arena_.alloc(&V_.q, (size_t)n));
  PDOS_TRY(arena_.alloc(&V_.t, (size_t)n));
  PDOS_TRY(arena_.alloc(&V_.s, (size_t)m));
  PDOS_TRY(arena_.alloc(&V_.y, (size_t)m));
  PDOS_TRY(arena_.alloc(&V_.st, (size_t)m));
  PDOS_TRY(arena_.alloc(&V_.u, (size_t)m));
  PDOS_TRY(arena_.alloc(&V_.ax, (size_t)m));
  PDOS_TRY(arena_.alloc(&out_, (size_t)n + 2 * (size_t)m));
  PDOS_CUDA_TRY(cudaGetLastError());

  // ---- solver state
  PDOS_TRY(arena_.alloc(&S_, 1));
  PDOS_CUDA_TRY(cudaMallocHost(&host_state_, sizeof(DevState)));
  PDOS_CUDA_TRY(cudaMemsetAsync(S_, 0, sizeof(DevState), st));

  // ---- SELL plans of A (rows of A) and A' (columns of A)
  PDOS_TRY(sellA_.build(P.rp_host.data(), m, Rj_, Rx_, arena_, st));
  PDOS_TRY(sellT_.build(P.ap_host.data(), n, Ai_, Ax_, arena_, st));
  PDOS_TRY(build_cone_tables(d.soc_off, d.soc_len, arena_, st, ct_, &soc_grid_, &socbig_grid_));

  // ---- grids and reduction scratch (an SpMV kernel uses grid+1 slots)
  grid_upd_ = persistent_grid(cg_update_kernel<T, kBlock>, kBlock, 0, (n + kBlock - 1) / kBlock);
  grid_dir_ = std::max(1, std::min((n + kBlock - 1) / kBlock, num_sms() * 8));
  size_t slots = 0;
  slots = std::max(slots, (size_t)sellA_.slots() * 2);
  slots = std::max(slots, (size_t)sellT_.slots() * 3);
  slots = std::max(slots, (size_t)grid_upd_);
  slots = std::max(slots, (size_t)(sellA_.slots() + soc_grid_ + socbig_grid_) * 2);
  PDOS_TRY(arena_.alloc(&partials_, slots));
  PDOS_TRY(arena_.alloc(&tickets_, 8));
  PDOS_CUDA_TRY(cudaMemsetAsync(tickets_, 0, sizeof(unsigned) * 8, st));

  PDOS_CUDA_TRY(cudaStreamSynchronize(st));
  PDOS_TRY(reset());
  PDOS_TRY(build_graph());
  PDOS_CUDA_TRY(cudaStreamSynchronize(st));
  setup_ms = now_ms() - t0;
  return PDOSGPU_OK;
}

template <typename T>
int Engine<T>::run_prep() {
  GridReduce gr{partials_, tickets_ + 0, 0, sellA_.slots(), 1};
  sellA_.run(V_.x, nullptr, OpPrep<T>{V_, (T)lambda_, S_}, gr, stream_);
  PDOS_CUDA_TRY(cudaGetLastError());
  launches += 1;
  return PDOSGPU_OK;
}

template <typename T>
int Engine<T>::reset() {
  cudaStream_t st = stream_;
  DevState h{};
  h.lambda = lambda_;
  h.alpha_relax = alpha_;
  h.eps = eps_;
  h.pscale = pscale_;
  h.dscale = dscale_;
  h.tol_sq = tol_sq_;
  h.max_iters = max_iters_;
  h.cg_max = cg_max_;
  h.p_res = h.d_res = h.p_obj = h.d_obj = h.eta = -1.0;
  h.done = max_iters_ <= 0 ? 1 : 0;
  h.cg_skip = 1;
  *host_state_ = h;
  PDOS_CUDA_TRY(cudaMemcpyAsync(S_, host_state_, sizeof(DevState), cudaMemcpyHostToDevice, st));
  PDOS_CUDA_TRY(cudaMemcpyAsync(V_.x, x_init_, sizeof(T) * n_, cudaMemcpyDeviceToDevice, st));
  PDOS_CUDA_TRY(cudaMemcpyAsync(V_.y, y_init_, sizeof(T) * m_, cudaMemcpyDeviceToDevice, st));
  PDOS_CUDA_TRY(cudaMemcpyAsync(V_.s, s_init_, sizeof(T) * m_, cudaMemcpyDeviceToDevice, st));
  PDOS_CUDA_TRY(cudaMemsetAsync(V_.p, 0, sizeof(T) * n_, st));
  PDOS_CUDA_TRY(cudaMemsetAsync(V_.q, 0, sizeof(T) * n_, st));
  PDOS_CUDA_TRY(cudaMemsetAsync(V_.t, 0, sizeof(T) * n_, st));
  PDOS_CUDA_TRY(cudaMemsetAsync(V_.st, 0, sizeof(T) * m_, st));
  PDOS_CUDA_TRY(cudaMemsetAsync(V_.u, 0, sizeof(T) * m_, st));
  PDOS_CUDA_TRY(cudaMemsetAsync(V_.ax, 0, sizeof(T) * m_, st));
  PDOS_TRY(run_prep());
  return PDOSGPU_OK;
}

template <typename T>
int Engine<T>::build_graph() {
  cudaStream_t st = stream_;
  const T lam = (T)lambda_;
  auto top = [&]() {
    GridReduce gr{partials_, tickets_ + 1, 0, sellT_.slots(), 1};
    sellT_.run(V_.y, V_.u, OpTop<T>{V_, lam, S_}, gr, st);
  };
  auto cg = [&]() {
    GridReduce none{partials_, tickets_ + 2, 0, sellA_.slots(), 0};
    sellA_.run(V_.p, nullptr, OpCgA<T>{V_, S_}, none, st);
    GridReduce g2{partials_, tickets_ + 3, 0, sellT_.slots(), 1};
    sellT_.run(V_.u, nullptr, OpCgAt<T>{V_, S_}, g2, st);
    GridReduce g3{partials_, tickets_ + 4, 0, grid_upd_, 1};
    cg_update_kernel<T, kBlock><<<grid_upd_, kBlock, 0, st>>>(V_, S_, g3);
    cg_direction_kernel<T, kBlock><<<grid_dir_, kBlock, 0, st>>>(V_, S_);
  };
  auto tail = [&]() {
    const int gpost = sellA_.slots();
    const int total = gpost + soc_grid_ + socbig_grid_;
    GridReduce g5{partials_, tickets_ + 5, 0, total, qsize_ == 0 ? 1 : 0};
    OpPost<T> op{V_, lam, (T)alpha_, (T)(1.0 - alpha_), S_};
    sellA_.run(V_.x, nullptr, op, g5, st);
    if (qsize_ > 0) {
      GridReduce g6{partials_, tickets_ + 6, gpost, total, socbig_grid_ == 0 ? 1 : 0};
      soc_kernel<T, kBlock><<<soc_grid_, kBlock, 0, st>>>(V_, ct_, lam, S_, g6);
      if (socbig_grid_ > 0) {
        GridReduce g7{partials_, tickets_ + 7, gpost + soc_grid_, total, 1};
        soc_big_kernel<T, kBlock><<<socbig_grid_, kBlock, 0, st>>>(V_, ct_, lam, S_, g7);
      }
    }
  };
  int64_t last_nodes = 0;
  auto capture = [&](auto &&body, cudaGraphExec_t *exec) -> int {
    cudaGraph_t graph = nullptr;
    PDOS_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    body();
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (e != cudaSuccess) return fail(PDOSGPU_ECUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    size_t nodes = 0;
    cudaGraphGetNodes(graph, nullptr, &nodes);
    last_nodes = (int64_t)nodes;
    e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(PDOSGPU_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    return PDOSGPU_OK;
  };
  if (cg_max_ <= 64) {
    PDOS_TRY(capture(
        [&]() {
          top();
          for (int64_t k = 0; k < cg_max_; ++k) cg();
          tail();
        },
        &exec_));
    nodes_main_ = last_nodes;
  } else {
    cg_block_ = 16;
    extra_exec_.assign(3, nullptr);
    PDOS_TRY(capture([&]() { top(); }, &extra_exec_[0]));
    nodes_top_ = last_nodes;
    PDOS_TRY(capture(
        [&]() {
          for (int k = 0; k < cg_block_; ++k) cg();
        },
        &extra_exec_[1]));
    nodes_cg_ = last_nodes;
    PDOS_TRY(capture([&]() { tail(); }, &extra_exec_[2]));
    nodes_tail_ = last_nodes;
  }
  return PDOSGPU_OK;
}

template <typename T>
int Engine<T>::launch_iteration() {
  if (exec_) {
    PDOS_CUDA_TRY(cudaGraphLaunch(exec_, stream_));
    launches += nodes_main_;
  } else {
    PDOS_CUDA_TRY(cudaGraphLaunch(extra_exec_[0], stream_));
    for (int64_t k = 0; k < cg_max_; k += cg_block_) {
      PDOS_CUDA_TRY(cudaGraphLaunch(extra_exec_[1], stream_));
      launches += nodes_cg_;
    }
    PDOS_CUDA_TRY(cudaGraphLaunch(extra_exec_[2], stream_));
    launches += nodes_top_ + nodes_tail_;
  }
  return PDOSGPU_OK;
}

template <typename T>
int Engine<T>::read_state() {
  PDOS_CUDA_TRY(cudaMemcpyAsync(host_state_, S_, sizeof(DevState), cudaMemcpyDeviceToHost, stream_));
  PDOS_CUDA_TRY(cudaStreamSynchronize(stream_));
  return PDOSGPU_OK;
}

static void print_header() {
  printf(" iter |  ||Ax+s-b||    ||A'y+c||       c'x          -b'y          eta    \n");
  printf("==========================================================================\n");
}

static void print_row(long long i, const DevState &s) {
  printf("%5lld | %11.3e   %10.3e   %11.3e   %11.3e   %10.3e   \n", i, s.p_res, s.d_res, s.p_obj,
         s.d_obj, s.eta);
}

template <typename T>
int Engine<T>::iterate(int64_t iters, bool until_done) {
  const double t0 = now_ms();
  PDOS_TRY(read_state());
  if (host_state_->done || iters <= 0) {
    solve_ms = now_ms() - t0;
    return PDOSGPU_OK;
  }
  if (verbose_) {
    printf("lambda: %5.3e\n\n", lambda_);
    print_header();
    int64_t done_iters = 0;
    while (done_iters < iters) {
      const long long before = host_state_->admm_iter;
      PDOS_TRY(launch_iteration());
      PDOS_TRY(read_state());
      ++done_iters;
      const DevState &s = *host_state_;
      if (s.solved || s.done) {
        print_row(s.solved ? before : s.admm_iter, s);
        break;
      }
      if (before % 10 == 0) print_row(before, s);
    }
    printf("Total solve time is %4.8fs\n", (now_ms() - t0) / 1e3);
  } else {
    int64_t launched = 0;
    int64_t batch = 1;
    while (launched < iters) {
      const int64_t nb = std::min<int64_t>(batch, iters - launched);
      for (int64_t i = 0; i < nb; ++i) PDOS_TRY(launch_iteration());
      launched += nb;
      if (until_done || launched >= iters) {
        PDOS_TRY(read_state());
        if (host_state_->done) break;
      }
      if (batch < 16) batch *= 2;
    }
  }
  PDOS_TRY(read_state());
  solve_ms = now_ms() - t0;
  return PDOSGPU_OK;
}

template <typename T>
__global__ void unscale_kernel(const T *x, const T *s, const T *y, const double *D, const double *E,
                               int n, int m, double *out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n + m; i += gridDim.x * blockDim.x) {
    if (i < n) {
      out[i] = E[i] * (double)x[i];  // pdos.c:272-282
    } else {
      const int r = i - n;
      out[n + r] = (double)s[r] / D[r];      // pdos.c:284-294
      out[n + m + r] = D[r] * (double)y[r];  // pdos.c:261-270
    }
  }
}

template <typename T>
int Engine<T>::fetch(double *x, double *s, double *y, pdosgpu_info *info) {
  cudaStream_t st = stream_;
  unscale_kernel<T><<<grid1d(n_ + m_), 256, 0, st>>>(V_.x, V_.s, V_.y, D64_, E64_, n_, m_, out_);
  PDOS_CUDA_TRY(cudaGetLastError());
  if (x) PDOS_CUDA_TRY(cudaMemcpyAsync(x, out_, sizeof(double) * n_, cudaMemcpyDeviceToHost, st));
  if (s) PDOS_CUDA_TRY(cudaMemcpyAsync(s, out_ + n_, sizeof(double) * m_, cudaMemcpyDeviceToHost, st));
  if (y) PDOS_CUDA_TRY(cudaMemcpyAsync(y, out_ + n_ + m_, sizeof(double) * m_, cudaMemcpyDeviceToHost, st));
  PDOS_TRY(read_state());
  if (info) {
    const DevState &h = *host_state_;
    info->admm_iters = h.admm_iter;
    info->cg_iters = h.cg_total;
    info->solved = h.solved;
    info->diverged = h.diverged;
    info->p_res = h.p_res;
    info->d_res = h.d_res;
    info->p_obj = h.p_obj;
    info->d_obj = h.d_obj;
    info->eta = h.eta;
    info->lambda = lambda_;
    info->setup_ms = setup_ms;
    info->solve_ms = solve_ms;
    info->kernel_launches = launches;
  }
  return PDOSGPU_OK;
}

template <typename T>
int Engine<T>::time_kernel(int which, int reps, double *ms) {
  if (reps <= 0 || !ms) return fail(PDOSGPU_EINVAL, "reps must be positive");
  cudaStream_t st = stream_;
  // make every kernel do its full work: not done, CG active
  PDOS_TRY(read_state());
  DevState h = *host_state_;
  h.done = 0;
  h.cg_active = 1;
  h.cg_skip = 0;
  h.ratio = 0.5;
  h.qsold = 1.0;
  h.cg_iter = 0;
  h.max_iters = INT64_MAX / 2;
  *host_state_ = h;
  PDOS_CUDA_TRY(cudaMemcpyAsync(S_, host_state_, sizeof(DevState), cudaMemcpyHostToDevice, st));
  const T lam = (T)lambda_;
  cudaEvent_t e0, e1;
  PDOS_CUDA_TRY(cudaEventCreate(&e0));
  PDOS_CUDA_TRY(cudaEventCreate(&e1));
  auto launch = [&]() {
    switch (which) {
      case 0: {  // CG u = A p
        GridReduce none{partials_, tickets_ + 2, 0, sellA_.slots(), 0};
        sellA_.run(V_.p, nullptr, OpCgA<T>{V_, S_}, none, st);
        break;
      }
      case 1: {  // CG t = p + A'u, p't
        GridReduce g2{partials_, tickets_ + 3, 0, sellT_.slots(), 1};
        sellT_.run(V_.u, nullptr, OpCgAt<T>{V_, S_}, g2, st);
        break;
      }
      case 2: {  // A'(y, u) of the iteration's first pass
        GridReduce gr{partials_, tickets_ + 1, 0, sellT_.slots(), 0};
        sellT_.run(V_.y, V_.u, OpTop<T>{V_, lam, S_}, gr, st);
        break;
      }
      case 3: {  // A x of the iteration's last pass
        GridReduce g5{partials_, tickets_ + 5, 0, sellA_.slots(), 0};
        sellA_.run(V_.x, nullptr, OpPost<T>{V_, lam, (T)alpha_, (T)(1.0 - alpha_), S_}, g5, st);
        break;
      }
      case 4: {  // the SpMV kernel of the CG A pass alone (no split-row combine)
        GridReduce none{partials_, tickets_ + 2, 0, sellA_.slots(), 0};
        sell_spmv_kernel<T, 256, OpCgA<T>><<<sellA_.spmv_grid, 256, 0, st>>>(
            sellA_.dev, V_.p, V_.p, sellA_.vsum, OpCgA<T>{V_, S_}, none);
        break;
      }
      default: {  // the SpMV kernel of the CG A' pass alone
        GridReduce g2{partials_, tickets_ + 3, 0, sellT_.slots(), 0};
        sell_spmv_kernel<T, 256, OpCgAt<T>><<<sellT_.spmv_grid, 256, 0, st>>>(
            sellT_.dev, V_.u, V_.u, sellT_.vsum, OpCgAt<T>{V_, S_}, g2);
      }
    }
  };
  launch();  // warm-up
  PDOS_CUDA_TRY(cudaEventRecord(e0, st));
  for (int r = 0; r < reps; ++r) launch();
  PDOS_CUDA_TRY(cudaEventRecord(e1, st));
  PDOS_CUDA_TRY(cudaGetLastError());
  PDOS_CUDA_TRY(cudaEventSynchronize(e1));
  float total = 0.f;
  PDOS_CUDA_TRY(cudaEventElapsedTime(&total, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  launches += reps + 1;
  *ms = (double)total / reps;
  return PDOSGPU_OK;
}

int make_engine(const pdosgpu_problem &prob, const pdosgpu_options &opt,
                std::unique_ptr<EngineBase> &out) {
  if (opt.precision == PDOSGPU_FP32) {
    auto e = std::make_unique<Engine<float>>();
    PDOS_TRY(e->setup(prob, opt));
    out = std::move(e);
  } else if (opt.precision == PDOSGPU_FP64) {
    auto e = std::make_unique<Engine<double>>();
    PDOS_TRY(e->setup(prob, opt));
    out = std::move(e);
  } else {
    return fail(PDOSGPU_EINVAL, "unknown precision");
  }
  return PDOSGPU_OK;
}

}  // namespace pdosgpu
