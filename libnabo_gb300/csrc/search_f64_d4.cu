// search_f64_d4.cu -- kNN kernels instantiated for double, 4-D records.
#include "search_impl.cuh"

namespace nabo_gb300 {
NABO_SEARCH_INSTANTIATE(double, 4)
}  // namespace nabo_gb300
