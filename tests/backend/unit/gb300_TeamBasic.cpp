// The reference's core/unit_test/TestTeamBasic.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestTeamBasic.hpp>
