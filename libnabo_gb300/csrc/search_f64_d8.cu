// search_f64_d8.cu -- kNN kernels instantiated for double, 8-D records.
#include "search_impl.cuh"

namespace nabo_gb300 {
NABO_SEARCH_INSTANTIATE(double, 8)
}  // namespace nabo_gb300
