// The reference's core/unit_test/TestReductions_DeviceView.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestReductions_DeviceView.hpp>
