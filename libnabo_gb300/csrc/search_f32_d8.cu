// search_f32_d8.cu -- kNN kernels instantiated for float, 8-D records.
#include "search_impl.cuh"

namespace nabo_gb300 {
NABO_SEARCH_INSTANTIATE(float, 8)
}  // namespace nabo_gb300
