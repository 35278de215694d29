// Reduce kernels instantiated for uint32_t (see gbk_reduce_impl.cuh).
#include "gbk_reduce_impl.cuh"

namespace gbk {
template int reduce_typed<uint32_t>(int, const uint32_t*, int64_t, int64_t, void*, Workspace*, const gbk_tuning_t*);
template int mdreduce_typed<uint32_t>(int, const uint32_t*, const MDBox&, void*, Workspace*, const gbk_tuning_t*);
}  // namespace gbk
