// bgk_inst_bf16_f32.cu -- kernels for storage __nv_bfloat16, compute float.
#include <type_traits>
#include "bgk_instantiate.cuh"

namespace bgk {
KernelTable table_bf16_f32() { return inst::make_table<__nv_bfloat16, float>(); }
}  // namespace bgk
