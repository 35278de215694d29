// The reference's core/unit_test/TestRange.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestRange.hpp>
