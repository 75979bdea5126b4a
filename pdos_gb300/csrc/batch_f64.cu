// The FP64 batch engine: BatchEngine<double> and its kernels, in a
// translation unit of their own.
#include "batch_engine.cuh"

namespace pdosgpu {
namespace batch {

std::unique_ptr<BatchBase> make_batch_engine_f64() { return std::make_unique<BatchEngine<double>>(); }

}  // namespace batch
}  // namespace pdosgpu
