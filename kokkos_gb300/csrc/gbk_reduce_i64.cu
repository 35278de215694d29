// Reduce kernels instantiated for int64_t (see gbk_reduce_impl.cuh).
#include "gbk_reduce_impl.cuh"

namespace gbk {
template int reduce_typed<int64_t>(int, const int64_t*, int64_t, int64_t, void*, Workspace*, const gbk_tuning_t*);
template int mdreduce_typed<int64_t>(int, const int64_t*, const MDBox&, void*, Workspace*, const gbk_tuning_t*);
}  // namespace gbk
