// The reference's algorithms/unit_tests/TestBinSortB.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestBinSortB.hpp>
