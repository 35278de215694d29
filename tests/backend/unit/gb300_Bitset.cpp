// The reference's containers/unit_tests/TestBitset.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestBitset.hpp>
