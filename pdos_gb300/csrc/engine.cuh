// Grid engine: one PDOS indirect solve spread over the whole GPU.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "admm_ops.cuh"
#include "common.cuh"
#include "sell.cuh"

namespace pdosgpu {

constexpr int kBlock = 256;

int num_sms();

#ifndef PDOS_SELL_BLOCKS_PER_SM
#define PDOS_SELL_BLOCKS_PER_SM 16
#endif

// Device allocations owned by one workspace, released together.
class DeviceArena {
 public:
  ~DeviceArena() { release(); }
  template <typename T>
  int alloc(T **p, size_t count) {
    void *raw = nullptr;
    size_t bytes = (count > 0 ? count : 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&raw, bytes);
    if (e != cudaSuccess) {
      *p = nullptr;
      return fail(PDOSGPU_ENOMEM, std::string("cudaMalloc(") + std::to_string(bytes) +
                                      " B): " + cudaGetErrorString(e));
    }
    ptrs_.push_back(raw);
    *p = static_cast<T *>(raw);
    return PDOSGPU_OK;
  }
  void release() {
    for (void *p : ptrs_)
      if (p) cudaFree(p);
    ptrs_.clear();
  }

 private:
  std::vector<void *> ptrs_;
};

// Device side of a SELL plan (see sell.cuh), built from a host row pointer
// array and the device index / value arrays of the same row-wise matrix.
template <typename T>
struct SellPlan {
  SellDev<T> dev{};
  T *vsum = nullptr;  // [2 * nvr] virtual-row partials (scratch)
  int spmv_grid = 1, combine_rows = 1, combine_grid = 1;

  int build(const int32_t *ptr_h, int32_t rows, const int32_t *idx_d, const T *val_d,
            DeviceArena &arena, cudaStream_t st) {
    SellHost h;
    h.build(ptr_h, rows);
    int32_t *slice_off, *vr_len, *idx, *vr_ptr, *vr_list, *heavy, *slot_src, *vr_row, *split;
    T *val;
    PDOS_TRY(arena.alloc(&slice_off, h.slice_off.size()));
    PDOS_TRY(arena.alloc(&vr_len, h.vr_len.size()));
    PDOS_TRY(arena.alloc(&vr_ptr, h.vr_ptr.size()));
    PDOS_TRY(arena.alloc(&vr_list, h.vr_list.size()));
    PDOS_TRY(arena.alloc(&heavy, h.heavy.size()));
    PDOS_TRY(arena.alloc(&vr_row, h.vr_row.size()));
    PDOS_TRY(arena.alloc(&split, h.split.size()));
    PDOS_TRY(arena.alloc(&idx, (size_t)h.slots));
    PDOS_TRY(arena.alloc(&val, (size_t)h.slots));
    PDOS_TRY(arena.alloc(&vsum, (size_t)2 * h.nvr));
    auto up = [&](int32_t *d, const std::vector<int32_t> &v) -> int {
      if (!v.empty())
        PDOS_CUDA_TRY(cudaMemcpyAsync(d, v.data(), sizeof(int32_t) * v.size(), cudaMemcpyHostToDevice, st));
      return PDOSGPU_OK;
    };
    PDOS_TRY(up(slice_off, h.slice_off));
    PDOS_TRY(up(vr_len, h.vr_len));
    PDOS_TRY(up(vr_ptr, h.vr_ptr));
    PDOS_TRY(up(vr_list, h.vr_list));
    PDOS_TRY(up(heavy, h.heavy));
    PDOS_TRY(up(vr_row, h.vr_row));
    PDOS_TRY(up(split, h.split));
    if (h.slots > 0) {
      DeviceArena tmp;
      PDOS_TRY(tmp.alloc(&slot_src, (size_t)h.slots));
      PDOS_TRY(up(slot_src, h.slot_src));
      const int g = (int)std::min<int64_t>((h.slots + 255) / 256, (int64_t)num_sms() * 16);
      sell_fill_kernel<T><<<g, 256, 0, st>>>(slot_src, h.slots, idx_d, val_d, idx, val);
      PDOS_CUDA_TRY(cudaGetLastError());
      PDOS_CUDA_TRY(cudaStreamSynchronize(st));  // before slot_src is freed
    }
    dev = SellDev<T>{slice_off, vr_len, idx, val, h.nslices, h.nvr, vr_ptr, vr_list, heavy,
                     (int32_t)h.heavy.size(), rows, vr_row, split, (int32_t)h.split.size(),
                     h.ngiant};
    vrow = h.vrow;
    nvr = h.nvr;
    spmv_grid = std::max(1, std::min((h.nslices + 7) / 8, num_sms() * PDOS_SELL_BLOCKS_PER_SM));
    combine_rows = std::max(1, std::min(((int)h.split.size() + 255) / 256, num_sms() * 8));
    combine_grid = combine_rows + h.ngiant + ((int)h.heavy.size() - h.ngiant + 7) / 8;
    return PDOSGPU_OK;
  }
  int vrow = 0, nvr = 0;
  bool has_combine() const { return dev.nsplit + dev.nheavy > 0; }
  // grid-reduction slots used by one run()
  int slots() const { return spmv_grid + (has_combine() ? combine_grid : 0); }
  // y-side of M x (x1 non-NULL: M x0 and M x1 at once), rows handed to `op`.
  // `gr` describes this run's slot range; its final flag applies to the last
  // kernel of the run.
  template <class Op>
  void run(const T *x0, const T *x1, const Op &op, GridReduce gr, cudaStream_t st) const {
    GridReduce g1 = gr;
    if (has_combine()) g1.final_kernel = 0;
    sell_spmv_kernel<T, 256, Op><<<spmv_grid, 256, 0, st>>>(dev, x0, x1 ? x1 : x0, vsum, op, g1);
    if (has_combine()) {
      GridReduce g2 = gr;
      g2.base = gr.base + spmv_grid;
      sell_combine_kernel<T, 256, Op><<<combine_grid, 256, 0, st>>>(dev, vsum, op, g2, combine_rows);
    }
  }
};

class EngineBase {
 public:
  virtual ~EngineBase() {}
  virtual int iterate(int64_t iters, bool until_done) = 0;
  virtual int reset() = 0;
  virtual int fetch(double *x, double *s, double *y, pdosgpu_info *info) = 0;
  virtual int time_kernel(int which, int reps, double *ms) = 0;
  virtual void *stream() = 0;
  double setup_ms = 0, solve_ms = 0;
  int64_t launches = 0;
};

int make_engine(const pdosgpu_problem &prob, const pdosgpu_options &opt,
                std::unique_ptr<EngineBase> &out);

}  // namespace pdosgpu
