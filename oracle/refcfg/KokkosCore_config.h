/* Hand-written feature macros for a host-only (OpenMP + Serial) build of the
 * reference Kokkos sources.  Replaces the header the reference's CMake step
 * would generate; only the macros the OpenMP/Serial reduce, scan, ScatterView
 * and sort paths read are set.  Used by oracle/ref.mk (checker only). */
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
#define KOKKOS_ENABLE_OPENMP
#define KOKKOS_ENABLE_CXX17
#define KOKKOS_ENABLE_DEPRECATED_CODE_4
#define KOKKOS_ENABLE_COMPLEX_ALIGN
#define KOKKOS_ENABLE_IMPL_MDSPAN
#define KOKKOS_ENABLE_IMPL_REF_COUNT_BRANCH_UNLIKELY
#define KOKKOS_ENABLE_LIBDL
#define KOKKOS_ENABLE_TUNING
