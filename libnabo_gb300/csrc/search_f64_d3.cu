// search_f64_d3.cu -- kNN kernels instantiated for double, 3-D records.
#include "search_impl.cuh"

namespace nabo_gb300 {
NABO_SEARCH_INSTANTIATE(double, 3)
}  // namespace nabo_gb300
