/* Backend forward declarations of the Serial + GB300 build (the reference's
 * CMake writes this list from the enabled backends). */
#ifndef KOKKOS_FWD_HPP_
#define KOKKOS_FWD_HPP_
#include <fwd/Kokkos_Fwd_SERIAL.hpp>
#include <fwd/Kokkos_Fwd_GB300.hpp>
#endif
