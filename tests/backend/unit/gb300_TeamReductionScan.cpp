// The reference's core/unit_test/TestTeamReductionScan.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestTeamReductionScan.hpp>
