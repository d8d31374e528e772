// search_f64_d2.cu -- kNN kernels instantiated for double, 2-D records.
#include "search_impl.cuh"

namespace nabo_gb300 {
NABO_SEARCH_INSTANTIATE(double, 2)
}  // namespace nabo_gb300
