// search_f32_d16.cu -- kNN kernels instantiated for float, 16-D records.
#include "search_impl.cuh"

namespace nabo_gb300 {
NABO_SEARCH_INSTANTIATE(float, 16)
}  // namespace nabo_gb300
