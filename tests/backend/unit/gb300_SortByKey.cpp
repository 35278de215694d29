// The reference's algorithms/unit_tests/TestSortByKey.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestSortByKey.hpp>
