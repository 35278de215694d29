/* Set-up of the GB300 execution space (the role Kokkos_Setup_Cuda.hpp plays
 * for the CUDA space, core/src/setup/Kokkos_Setup_Cuda.hpp): functions marked
 * KOKKOS_FUNCTION and lambdas marked KOKKOS_LAMBDA are compiled for the host
 * and for sm_103a, so user functors and Kokkos' own functors (View
 * initialisation, deep_copy, reducers) run inside this space's kernels. */
#ifndef KOKKOS_SETUP_GB300_HPP_
#define KOKKOS_SETUP_GB300_HPP_

#if !defined(KOKKOS_ENABLE_GB300)
#error "Kokkos_Setup_GB300.hpp included without KOKKOS_ENABLE_GB300"
#endif
#if !defined(__CUDACC__)
#error "the GB300 space is compiled by nvcc (-gencode arch=compute_103a,code=sm_103a)"
#endif

#include <cuda_runtime.h>

#define KOKKOS_LAMBDA [=] __host__ __device__
#define KOKKOS_CLASS_LAMBDA [ =, *this ] __host__ __device__
#define KOKKOS_DEDUCTION_GUIDE __host__ __device__
#define KOKKOS_IMPL_FORCEINLINE_FUNCTION __device__ __host__ __forceinline__
#define KOKKOS_IMPL_FORCEINLINE __forceinline__
#define KOKKOS_IMPL_INLINE_FUNCTION __device__ __host__ inline
#define KOKKOS_IMPL_FUNCTION __device__ __host__
#define KOKKOS_IMPL_HOST_FUNCTION __host__
#define KOKKOS_IMPL_DEVICE_FUNCTION __device__
#define KOKKOS_IMPL_RELOCATABLE_FUNCTION __device__ __host__

#if defined(__CUDA_ARCH__)
#define KOKKOS_IF_ON_DEVICE(CODE) \
  { KOKKOS_IMPL_STRIP_PARENS(CODE) }
#define KOKKOS_IF_ON_HOST(CODE) \
  {}
#else
#define KOKKOS_IF_ON_DEVICE(CODE) \
  {}
#define KOKKOS_IF_ON_HOST(CODE) \
  { KOKKOS_IMPL_STRIP_PARENS(CODE) }
#endif

// Kokkos::abort in device code (core/src/Kokkos_Abort.hpp calls
// Impl::device_abort): the skeleton kernels' abort request, see
// GB300/Kokkos_GB300_Skeletons.hpp.
#include <GB300/Kokkos_GB300_Skeletons.hpp>
namespace Kokkos {
namespace Impl {
__device__ inline void device_abort(const char* const msg) { ::gbk_skel::request_abort(msg); }
}  // namespace Impl
}  // namespace Kokkos

#endif
