// Grid engine: one PDOS indirect solve spread over the whole GPU.
#pragma once

#include <memory>
#include <vector>

#include "admm_ops.cuh"
#include "common.cuh"
#include "spmv.cuh"

namespace pdosgpu {

constexpr int kBlock = 256;
constexpr int kTileNnz = 2048;
constexpr int kMaxTileRows = 4 * kBlock;

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
  void free_one(void *p) {
    for (auto &q : ptrs_)
      if (q == p) {
        cudaFree(q);
        q = nullptr;
      }
  }
  void release() {
    for (void *p : ptrs_)
      if (p) cudaFree(p);
    ptrs_.clear();
  }

 private:
  std::vector<void *> ptrs_;
};

template <typename T>
struct SpmvPlan {
  std::vector<Tile> tiles_h;
  std::vector<LongRow> longs_h;
  int32_t slots = 0;
  Tile *tiles = nullptr;
  LongRow *longs = nullptr;
  T *chunk_partial = nullptr;
  unsigned int *long_ticket = nullptr;
  TilesDev<T> view() const {
    return TilesDev<T>{tiles, (int32_t)tiles_h.size(), longs, chunk_partial, long_ticket};
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
