// The reference's core/unit_test/TestGraph.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestGraph.hpp>
