/* Backend set-up headers of the Serial + GB300 build: the GB300 space makes
 * KOKKOS_FUNCTION / KOKKOS_LAMBDA host-device functions. */
#ifndef KOKKOS_SETUP_HPP_
#define KOKKOS_SETUP_HPP_
#include <setup/Kokkos_Setup_GB300.hpp>
#endif
