# Builds the reference Omega_h library (serial backend) straight from its
# sources with g++, plus the dump driver oracle/ref_driver.cpp, into
# oracle/_ref/.  The reference's own CMake build is not used: the only file
# CMake would generate, an options header of #define lines, is written here
# with every optional backend (MPI, OpenMP, Kokkos, CUDA, zlib) switched off.
#
#   make -f oracle/ref.mk REF=<reference source checkout> -j8
#
# Outputs (git-ignored): oracle/_ref/libomega_h_ref.a, oracle/_ref/ref_driver

ifndef REF
$(error REF must name the reference's source checkout)
endif
OUT := oracle/_ref
CXX ?= g++
CXXFLAGS := -O2 -std=c++17 -ffp-contract=off -fno-fast-math -w \
            -I$(OUT)/include -I$(REF)/src -I$(REF)/tpl -Iomega_h_gb300/csrc

# the library sources of the reference's serial build (src/CMakeLists.txt:1-112),
# minus the optional-dependency front ends that are compiled out anyway
SRC_NAMES := adapt adj align amr amr_topology amr_transfer any approach array \
  array_ops assoc base64 bbox bcast bipart box build build_parser chartab \
  check_collapse class cmdline coarsen coarsen_overshoot coarsen_qualities \
  coarsen_topology collapse_rail comm compare confined conserve dist eigen \
  expr fail fence file filesystem finite_automaton fix future ghost globals \
  grammar graph hilbert histogram indset inertia input int128 int_scan \
  language laplace library linpart malloc map mark math_lang matrix mesh \
  metric metric_input migrate modify owners parser parser_graph pool print \
  profile quality reader recover refine refine_qualities refine_topology \
  regex regress remotes reorder scatterplot shape shared_alloc simplify sort \
  stacktrace surface swap swap2d swap2d_qualities swap2d_topology swap3d \
  swap3d_qualities swap3d_topology tag timer transfer unmap_mesh vector vtk \
  xml xml_lite yaml random coarsen_flip overlay gmsh

OBJS := $(patsubst %,$(OUT)/obj/Omega_h_%.o,$(SRC_NAMES))

all: $(OUT)/ref_driver

$(OUT)/include/Omega_h_config.h:
	mkdir -p $(OUT)/include $(OUT)/obj
	printf '%s\n' '#ifndef OMEGA_H_CONFIG_H' '#define OMEGA_H_CONFIG_H' \
	  '#define OMEGA_H_VERSION_MAJOR 9' '#define OMEGA_H_VERSION_MINOR 34' \
	  '#define OMEGA_H_VERSION_PATCH 13' '#define OMEGA_H_SEMVER "9.34.13"' \
	  '#define OMEGA_H_CXX_FLAGS ""' '#define OMEGA_H_CMAKE_ARGS ""' '#define OMEGA_H_COMMIT ""' \
	  '#endif' > $@

$(OUT)/obj/%.o: $(REF)/src/%.cpp $(OUT)/include/Omega_h_config.h
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/libomega_h_ref.a: $(OBJS)
	ar rcs $@ $^

$(OUT)/ref_driver: oracle/ref_driver.cpp omega_h_gb300/csrc/ohg_workload.hpp $(OUT)/libomega_h_ref.a
	$(CXX) $(CXXFLAGS) -Ioracle oracle/ref_driver.cpp $(OUT)/libomega_h_ref.a -o $@

# The reference's OpenMP backend (the reference's -DOmega_h_USE_OpenMP=ON, with
# CMake's Release flags -O3 -DNDEBUG):
# the same sources with OMEGA_H_USE_OPENMP defined and -fopenmp, into
# oracle/_ref/omp/, for timing the reference's own parallel build.
#   make -f oracle/ref.mk REF=<reference source checkout> omp -j8
OMP := $(OUT)/omp
OMP_CXXFLAGS := -O3 -DNDEBUG -std=c++17 -ffp-contract=off -fno-fast-math -w -fopenmp \
            -I$(OMP)/include -I$(REF)/src -I$(REF)/tpl -Iomega_h_gb300/csrc
OMP_OBJS := $(patsubst %,$(OMP)/obj/Omega_h_%.o,$(SRC_NAMES))

$(OMP)/include/Omega_h_config.h:
	mkdir -p $(OMP)/include $(OMP)/obj
	printf '%s\n' '#ifndef OMEGA_H_CONFIG_H' '#define OMEGA_H_CONFIG_H' \
	  '#define OMEGA_H_VERSION_MAJOR 9' '#define OMEGA_H_VERSION_MINOR 34' \
	  '#define OMEGA_H_VERSION_PATCH 13' '#define OMEGA_H_SEMVER "9.34.13"' \
	  '#define OMEGA_H_USE_OPENMP' \
	  '#define OMEGA_H_CXX_FLAGS ""' '#define OMEGA_H_CMAKE_ARGS ""' '#define OMEGA_H_COMMIT ""' \
	  '#endif' > $@

$(OMP)/obj/%.o: $(REF)/src/%.cpp $(OMP)/include/Omega_h_config.h
	$(CXX) $(OMP_CXXFLAGS) -c $< -o $@

$(OMP)/libomega_h_ref.a: $(OMP_OBJS)
	ar rcs $@ $^

$(OMP)/ref_driver: oracle/ref_driver.cpp omega_h_gb300/csrc/ohg_workload.hpp $(OMP)/libomega_h_ref.a
	$(CXX) $(OMP_CXXFLAGS) -Ioracle oracle/ref_driver.cpp $(OMP)/libomega_h_ref.a -o $@

omp: $(OMP)/ref_driver

.PHONY: all omp
