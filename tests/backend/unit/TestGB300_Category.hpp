// Test category of the reference's own unit tests (core/unit_test,
// containers/unit_tests, algorithms/unit_tests) on the GB300 execution
// space: the same macros the reference's category files define for its
// backends (core/unit_test/category_files/TestCuda_Category.hpp).
#ifndef KOKKOS_TEST_GB300_HPP
#define KOKKOS_TEST_GB300_HPP

#include <gtest/gtest.h>

#define TEST_CATEGORY gb300
#define TEST_CATEGORY_NUMBER 20
#define TEST_CATEGORY_DEATH gb300_DeathTest
#define TEST_EXECSPACE Kokkos::Experimental::GB300
#define TEST_CATEGORY_FIXTURE(name) gb300_##name

#endif
