// The reference's containers/unit_tests/TestUnorderedMap.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestUnorderedMap.hpp>
