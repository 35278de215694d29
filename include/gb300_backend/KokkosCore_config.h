/* Feature macros of a Kokkos build with the Serial host space and the GB300
 * device space (Kokkos::Experimental::GB300), i.e. what the reference's CMake
 * step writes into KokkosCore_config.h (cmake/KokkosCore_config.h.in) for
 * -DKokkos_ENABLE_SERIAL=ON plus the GB300 backend.  Put this directory ahead
 * of the Kokkos sources on the include path:
 *   -I include/gb300_backend -I <kokkos>/core/src -I <kokkos>/containers/src
 *   -I <kokkos>/algorithms/src -I <kokkos>/tpls/desul/include
 *   -I <kokkos>/tpls/mdspan/include
 * and compile every translation unit with nvcc for sm_103a. */
#if !defined(KOKKOS_MACROS_HPP) || defined(KOKKOS_CORE_CONFIG_H)
#error "include Kokkos_Macros.hpp instead of KokkosCore_config.h"
#else
#define KOKKOS_CORE_CONFIG_H
#endif
#define KOKKOS_VERSION 40699
#define KOKKOS_VERSION_MAJOR 4
#define KOKKOS_VERSION_MINOR 6
#define KOKKOS_VERSION_PATCH 99
#define KOKKOS_ENABLE_SERIAL
#define KOKKOS_ENABLE_GB300
#define KOKKOS_ENABLE_DEFAULT_DEVICE_TYPE_SERIAL
#define KOKKOS_ENABLE_CXX17
#define KOKKOS_ENABLE_DEPRECATED_CODE_4
#define KOKKOS_ENABLE_COMPLEX_ALIGN
#define KOKKOS_ENABLE_IMPL_MDSPAN
#define KOKKOS_ENABLE_IMPL_REF_COUNT_BRANCH_UNLIKELY
#define KOKKOS_ENABLE_LIBDL
#define KOKKOS_ENABLE_TUNING
