/* Backend declarations of the Serial + GB300 build. */
#ifndef KOKKOS_DECLARE_HPP_
#define KOKKOS_DECLARE_HPP_
#include <decl/Kokkos_Declare_SERIAL.hpp>
#include <decl/Kokkos_Declare_GB300.hpp>
#endif
