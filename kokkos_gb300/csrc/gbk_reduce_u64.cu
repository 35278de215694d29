// Reduce kernels instantiated for uint64_t (see gbk_reduce_impl.cuh).
#include "gbk_reduce_impl.cuh"

namespace gbk {
template int reduce_typed<uint64_t>(int, const uint64_t*, int64_t, int64_t, void*, Workspace*, const gbk_tuning_t*);
template int mdreduce_typed<uint64_t>(int, const uint64_t*, const MDBox&, void*, Workspace*, const gbk_tuning_t*);
}  // namespace gbk
