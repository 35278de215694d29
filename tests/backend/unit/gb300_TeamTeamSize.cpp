// The reference's core/unit_test/TestTeamTeamSize.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestTeamTeamSize.hpp>
