// The reference's core/unit_test/TestParallelScanRangePolicy.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestParallelScanRangePolicy.hpp>
