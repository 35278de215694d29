# Builds the reference Kokkos OpenMP + Serial backend directly from its own
# sources (no CMake), for use as a CHECKER only: it generates golden vectors
# and validates the oracle restatement in this container.  Outputs go only to
# oracle/_ref/ (git-ignored).  Nothing in the product links this.
#
#   make -f oracle/ref.mk REF=/path/to/kokkos -j8
#
# The config headers CMake would generate are replaced by the hand-written
# feature-macro headers in oracle/refcfg/.

REF    ?= $(abspath $(dir $(lastword $(MAKEFILE_LIST)))/../../reference)
OUT    ?= oracle/_ref
CXX    ?= g++
CXXFLAGS ?= -O3 -std=c++17 -fopenmp -fPIC
INC = -Ioracle/refcfg -I$(REF)/core/src -I$(REF)/containers/src \
      -I$(REF)/algorithms/src -I$(REF)/simd/src -I$(REF)/tpls/desul/include \
      -I$(REF)/tpls/mdspan/include

CORE_SRCS = $(wildcard $(REF)/core/src/impl/*.cpp) \
            $(REF)/core/src/OpenMP/Kokkos_OpenMP.cpp \
            $(REF)/core/src/OpenMP/Kokkos_OpenMP_Instance.cpp \
            $(REF)/core/src/OpenMP/Kokkos_OpenMP_Task.cpp \
            $(REF)/core/src/Serial/Kokkos_Serial.cpp \
            $(REF)/core/src/Serial/Kokkos_Serial_Task.cpp \
            $(REF)/containers/src/impl/Kokkos_UnorderedMap_impl.cpp
CORE_OBJS = $(patsubst $(REF)/%.cpp,$(OUT)/obj/%.o,$(CORE_SRCS))

all: $(OUT)/libkokkos_ref.a $(OUT)/ref_runner

$(OUT)/obj/%.o: $(REF)/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@

$(OUT)/libkokkos_ref.a: $(CORE_OBJS)
	@mkdir -p $(OUT)
	ar rcs $@ $^

# The runner is this project's own program (oracle/ref_runner.cpp) that calls
# the reference API on inputs read from files and writes the results.
$(OUT)/ref_runner: oracle/ref_runner.cpp $(OUT)/libkokkos_ref.a
	$(CXX) $(CXXFLAGS) $(INC) $< $(OUT)/libkokkos_ref.a -ldl -o $@

clean:
	rm -rf $(OUT)/obj $(OUT)/libkokkos_ref.a $(OUT)/ref_runner

.PHONY: all clean
