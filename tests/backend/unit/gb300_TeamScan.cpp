// The reference's core/unit_test/TestTeamScan.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestTeamScan.hpp>
