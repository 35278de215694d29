// The reference's core/unit_test/TestMDRange_f.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestMDRange_f.hpp>
