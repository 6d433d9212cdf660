// bgk_inst_f64_f64.cu -- kernels for storage double, compute double.
#include <type_traits>
#include "bgk_instantiate.cuh"

namespace bgk {
KernelTable table_f64_f64() { return inst::make_table<double, double>(); }
}  // namespace bgk
