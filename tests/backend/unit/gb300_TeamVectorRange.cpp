// The reference's core/unit_test/TestTeamVectorRange.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestTeamVectorRange.hpp>
