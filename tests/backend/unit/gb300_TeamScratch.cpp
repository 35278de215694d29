// The reference's core/unit_test/TestTeamScratch.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestTeamScratch.hpp>
