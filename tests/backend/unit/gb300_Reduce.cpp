// The reference's core/unit_test/TestReduce.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestReduce.hpp>
