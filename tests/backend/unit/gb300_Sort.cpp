// The reference's algorithms/unit_tests/TestSort.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestSort.hpp>
