/* Forward declarations of the GB300 space (the role of
 * core/src/fwd/Kokkos_Fwd_CUDA.hpp for the CUDA space). */
#ifndef KOKKOS_GB300_FWD_HPP_
#define KOKKOS_GB300_FWD_HPP_
#if defined(KOKKOS_ENABLE_GB300)
namespace Kokkos {
namespace Experimental {
class GB300Space;  ///< device memory of the GPU the space runs on
class GB300;       ///< execution space: one CUDA stream on one GB300
}  // namespace Experimental
}  // namespace Kokkos
#endif
#endif
