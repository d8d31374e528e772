// search_f64_d16.cu -- kNN kernels instantiated for double, 16-D records.
#include "search_impl.cuh"

namespace nabo_gb300 {
NABO_SEARCH_INSTANTIATE(double, 16)
}  // namespace nabo_gb300
