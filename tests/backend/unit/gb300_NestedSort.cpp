// The reference's algorithms/unit_tests/TestNestedSort.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestNestedSort.hpp>
