// Reduce kernels instantiated for float (see gbk_reduce_impl.cuh).
#include "gbk_reduce_impl.cuh"

namespace gbk {
template int reduce_typed<float>(int, const float*, int64_t, int64_t, void*, Workspace*, const gbk_tuning_t*);
template int mdreduce_typed<float>(int, const float*, const MDBox&, void*, Workspace*, const gbk_tuning_t*);
}  // namespace gbk
