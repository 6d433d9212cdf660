// bgk_inst_f32_f32.cu -- kernels for storage float, compute float.
#include <type_traits>
#include "bgk_instantiate.cuh"

namespace bgk {
KernelTable table_f32_f32() { return inst::make_table<float, float>(); }
}  // namespace bgk
