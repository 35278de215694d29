"""GB300-native (sm_103a) reduce / scan / scatter / sort path for Kokkos.

The product is the C ABI in include/gbk.h, implemented by libgbk.so
(kokkos_gb300/csrc/*.cu), and the C++ header API over it.  This Python
package holds the build driver (build.py), the ctypes binding (gbk.py) and
the seeded input generator (datagen.py).
"""
__all__ = ["build", "gbk", "datagen"]
