// Comparator for the sort benchmarks, not part of the product: the reference's
// CUDA sort path calls thrust (algorithms/src/sorting/impl/Kokkos_SortImpl.hpp:
// 204-219 thrust::sort; impl/Kokkos_SortByKeyImpl.hpp:125-138
// thrust::sort_by_key), so bench.py times these two calls on the same keys
// and stream as the library's radix sort.  thrust is the CUDA toolkit's CCCL.
#include <cstdint>

#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/execution_policy.h>
#include <thrust/sort.h>

extern "C" {

int gbk_cmp_thrust_sort_u64(uint64_t* keys, int64_t n, void* stream) {
  thrust::device_ptr<uint64_t> k(keys);
  thrust::sort(thrust::cuda::par_nosync.on((cudaStream_t)stream), k, k + n);
  return (int)cudaGetLastError();
}

int gbk_cmp_thrust_sort_by_key_u64_i32(uint64_t* keys, int32_t* vals, int64_t n, void* stream) {
  thrust::device_ptr<uint64_t> k(keys);
  thrust::device_ptr<int32_t> v(vals);
  thrust::sort_by_key(thrust::cuda::par_nosync.on((cudaStream_t)stream), k, k + n, v);
  return (int)cudaGetLastError();
}

}  // extern "C"
