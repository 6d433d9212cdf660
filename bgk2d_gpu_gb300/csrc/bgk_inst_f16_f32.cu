// bgk_inst_f16_f32.cu -- kernels for storage __half, compute float.
#include <type_traits>
#include "bgk_instantiate.cuh"

namespace bgk {
KernelTable table_f16_f32() { return inst::make_table<__half, float>(); }
}  // namespace bgk
