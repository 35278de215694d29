/* No device backend is set up in the host-only reference build. */
#ifndef KOKKOS_SETUP_HPP_
#define KOKKOS_SETUP_HPP_
#endif
