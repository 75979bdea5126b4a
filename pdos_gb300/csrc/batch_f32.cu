// The FP32 batch engine: BatchEngine<float> and its kernels, in a
// translation unit of their own.
#include "batch_engine.cuh"

namespace pdosgpu {
namespace batch {

std::unique_ptr<BatchBase> make_batch_engine_f32() { return std::make_unique<BatchEngine<float>>(); }

}  // namespace batch
}  // namespace pdosgpu
