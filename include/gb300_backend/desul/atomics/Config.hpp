/* desul atomics configuration of the Serial + GB300 build: device code uses
 * the CUDA atomics (the GB300 space compiles with nvcc, whole-program, no
 * relocatable device code); host code uses the GCC builtins. */
#ifndef DESUL_ATOMICS_CONFIG_HPP_
#define DESUL_ATOMICS_CONFIG_HPP_
#define DESUL_ATOMICS_ENABLE_CUDA
#endif
