/* desul atomics configuration for the host-only reference build: no device
 * atomics are enabled (host atomics come from the GCC builtins). */
#ifndef DESUL_ATOMICS_CONFIG_HPP_
#define DESUL_ATOMICS_CONFIG_HPP_
#endif
