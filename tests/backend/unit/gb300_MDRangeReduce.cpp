// The reference's core/unit_test/TestMDRangeReduce.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestMDRangeReduce.hpp>
