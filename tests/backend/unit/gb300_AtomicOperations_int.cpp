// The reference's core/unit_test/TestAtomicOperations_int.hpp on the GB300 space.
#include <TestGB300_Category.hpp>
#include <TestAtomicOperations_int.hpp>
