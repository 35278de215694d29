// The reference's core/unit_test/TestReducers_c.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestReducers_c.hpp>
