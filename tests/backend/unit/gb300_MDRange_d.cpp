// The reference's core/unit_test/TestMDRange_d.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestMDRange_d.hpp>
