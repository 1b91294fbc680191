# Recipe: compile the reference's own solver sources (unmodified, read in place) plus
# oracle/ref_shim.cpp into oracle/_ref/libsovereign_ref.so.  Test infrastructure only.
#
#   make -f oracle/ref.mk            (from the repository root)
#
# REF must point at the reference project's solver directory.  When it does not exist
# (for example on a machine without the reference checkout) there is nothing to build.
REF ?= /root/reference/02-software/solver
OUT := oracle/_ref
CXX ?= g++
# -ffp-contract=off keeps products and sums separately rounded on every host, which is
# what the reference's x86-64 Release build does.
CXXFLAGS := -std=c++14 -O3 -fopenmp -fPIC -ffp-contract=off -I$(REF)/include -w

SRCS := solver.cpp mps.cpp milp_v2.cpp qp.cpp qp_admm.cpp qp_dual_newton.cpp \
        sparse_lp.cpp bounded_simplex.cpp accelerated_qp.cpp
OBJS := $(addprefix $(OUT)/,$(SRCS:.cpp=.o)) $(OUT)/ref_shim.o

all: $(OUT)/libsovereign_ref.so

$(OUT):
	mkdir -p $(OUT)

$(OUT)/%.o: $(REF)/src/%.cpp | $(OUT)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/ref_shim.o: oracle/ref_shim.cpp | $(OUT)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/libsovereign_ref.so: $(OBJS)
	$(CXX) -shared -fopenmp -o $@ $(OBJS)

.PHONY: all

# Level-A drop-in check: the reference's library with SOVEREIGN_CUDA defined (so its CPU stub of
# make_cuda_box drops out), the GB300 plugin hypergrey-sih-26_gb300/plugin/cuda_box_gb300.cpp in
# place of src/cuda_box.cu, and the reference's own CLI and scale harness linked against
# libboxqp.so.  Built from the reference's sources where they lie; outputs only into oracle/_ref.
PKG := hypergrey-sih-26_gb300
LIBDIR := $(abspath $(PKG)/boxqp)
LVL_FLAGS := $(CXXFLAGS) -DSOVEREIGN_CUDA=1 -Iinclude
LVL_OBJS := $(addprefix $(OUT)/lvl_,$(SRCS:.cpp=.o)) $(OUT)/lvl_plugin.o

$(OUT)/lvl_%.o: $(REF)/src/%.cpp | $(OUT)
	$(CXX) $(LVL_FLAGS) -c $< -o $@

$(OUT)/lvl_plugin.o: $(PKG)/plugin/cuda_box_gb300.cpp | $(OUT)
	$(CXX) $(LVL_FLAGS) -c $< -o $@

$(OUT)/solver_scale_gb300: $(LVL_OBJS) $(REF)/src/scale_benchmark.cpp
	$(CXX) $(LVL_FLAGS) $(REF)/src/scale_benchmark.cpp $(LVL_OBJS) -L$(LIBDIR) -lboxqp -Wl,-rpath,$(LIBDIR) -o $@

$(OUT)/solver_cli_gb300: $(LVL_OBJS) $(REF)/src/main.cpp
	$(CXX) $(LVL_FLAGS) $(REF)/src/main.cpp $(LVL_OBJS) -L$(LIBDIR) -lboxqp -Wl,-rpath,$(LIBDIR) -o $@

level_a: $(OUT)/solver_scale_gb300 $(OUT)/solver_cli_gb300

.PHONY: level_a

# The reference's CUDA plugin kernels, unmodified, compiled for this GPU into a loadable module
# (device code only; oracle/ref_cuda_harness.c drives it with the reference's host loop).
NVCC ?= nvcc
$(OUT)/cuda_box_sm103a.cubin: $(REF)/src/cuda_box.cu | $(OUT)
	$(NVCC) -cubin -gencode arch=compute_103a,code=sm_103a -O3 -I$(REF)/include -w -o $@ $<

cuda_cubin: $(OUT)/cuda_box_sm103a.cubin

.PHONY: cuda_cubin
