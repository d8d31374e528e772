// search_f32_d3.cu -- kNN kernels instantiated for float, 3-D records.
#include "search_impl.cuh"

namespace nabo_gb300 {
NABO_SEARCH_INSTANTIATE(float, 3)
}  // namespace nabo_gb300
