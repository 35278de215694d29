// The reference's core/unit_test/TestAtomicOperations_double.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestAtomicOperations_double.hpp>
