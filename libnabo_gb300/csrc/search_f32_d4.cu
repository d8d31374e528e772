// search_f32_d4.cu -- kNN kernels instantiated for float, 4-D records.
#include "search_impl.cuh"

namespace nabo_gb300 {
NABO_SEARCH_INSTANTIATE(float, 4)
}  // namespace nabo_gb300
