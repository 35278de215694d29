// Reduce kernels instantiated for double (see gbk_reduce_impl.cuh).
#include "gbk_reduce_impl.cuh"

namespace gbk {
template int reduce_typed<double>(int, const double*, int64_t, int64_t, void*, Workspace*, const gbk_tuning_t*);
template int mdreduce_typed<double>(int, const double*, const MDBox&, void*, Workspace*, const gbk_tuning_t*);
}  // namespace gbk
