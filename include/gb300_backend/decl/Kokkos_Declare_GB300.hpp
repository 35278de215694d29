/* Declarations of the GB300 space, included by Kokkos_Core.hpp through
 * KokkosCore_Config_DeclareBackend.hpp (the role of
 * core/src/decl/Kokkos_Declare_CUDA.hpp for the CUDA space). */
#ifndef KOKKOS_DECLARE_GB300_HPP
#define KOKKOS_DECLARE_GB300_HPP

#if defined(KOKKOS_ENABLE_GB300)
#include <GB300/Kokkos_GB300.hpp>
#include <GB300/Kokkos_GB300_Parallel_Range.hpp>
#include <GB300/Kokkos_GB300_Parallel_MDRange.hpp>
#include <GB300/Kokkos_GB300_Parallel_Team.hpp>
#include <GB300/Kokkos_GB300_Hooks.hpp>
#endif

#endif
