// The reference's containers/unit_tests/TestScatterView.hpp on the GB300
// space.  As the reference does for its CUDA space (TestScatterView.hpp, the
// KOKKOS_ENABLE_CUDA block before test_scatter_view), the ScatterDuplicated
// configurations are left out on this GPU space: a duplicate per resident
// thread is not a GPU layout, and ScatterView's GB300 default is
// non-duplicated with atomic contributions.
#include <TestGB300_Category.hpp>
#include <Kokkos_Core.hpp>

namespace Test {
template <typename DeviceType, typename ScatterType, typename NumberType>
struct TestDuplicatedScatterView;
template <typename ScatterType, typename NumberType>
struct TestDuplicatedScatterView<Kokkos::Experimental::GB300, ScatterType, NumberType> {
  TestDuplicatedScatterView(int) {}
};
template <typename ScatterType, typename NumberType>
struct TestDuplicatedScatterView<Kokkos::Device<Kokkos::Experimental::GB300, Kokkos::Experimental::GB300Space>,
                                 ScatterType, NumberType> {
  TestDuplicatedScatterView(int) {}
};
}  // namespace Test

#include <TestScatterView.hpp>
