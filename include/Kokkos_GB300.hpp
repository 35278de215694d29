// Kokkos_GB300.hpp — the header-template path of the GB300 reduce / scan /
// scatter / sort library: Kokkos' API for this path (View, RangePolicy,
// MDRangePolicy, TeamPolicy, parallel_for / parallel_reduce /
// parallel_scan with user functors and the built-in reducers, ScatterView,
// atomics, sort / sort_by_key / BinSort, std reduce / scans,
// Experimental::Graph) for one GB300 execution space.  User functors are
// instantiated in the caller's translation unit on the library's kernel
// skeletons; the fixed-type operations go through the C ABI (gbk.h).
//
// Compile with nvcc:  -std=c++17 --extended-lambda
//   -gencode arch=compute_103a,code=sm_103a -I<repo>/include -L<repo>/kokkos_gb300 -lgbk
//
// The names live in namespace gb300k; `namespace Kokkos = gb300k` is
// provided unless GBK_NO_KOKKOS_NAMESPACE is defined (define it when the
// reference Kokkos headers are included in the same translation unit).
#pragma once

#include "gb300/core.hpp"
#include "gb300/reducers.hpp"
#include "gb300/parallel.hpp"
#include "gb300/scan.hpp"
#include "gb300/scatter_sort.hpp"
#include "gb300/algorithms.hpp"
#include "gb300/unordered_map.hpp"

#ifndef GBK_NO_KOKKOS_NAMESPACE
namespace Kokkos = gb300k;
#endif
