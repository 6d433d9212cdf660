// bgk_inst_f32_f64.cu -- kernels for storage float, compute double.
#include <type_traits>
#include "bgk_instantiate.cuh"

namespace bgk {
KernelTable table_f32_f64() { return inst::make_table<float, double>(); }
}  // namespace bgk
