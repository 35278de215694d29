// The reference's algorithms/unit_tests/TestBinSortA.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestBinSortA.hpp>
