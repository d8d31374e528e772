// search_f32_d2.cu -- kNN kernels instantiated for float, 2-D records.
#include "search_impl.cuh"

namespace nabo_gb300 {
NABO_SEARCH_INSTANTIATE(float, 2)
}  // namespace nabo_gb300
