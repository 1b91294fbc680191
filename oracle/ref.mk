# Recipe: build the reference's own solver (unmodified sources) plus oracle/ref_shim.cpp into
# oracle/_ref/libsovereign_ref.so.  Test infrastructure only.
#
#   make -f oracle/ref.mk stage       (from the repository root, where the reference checkout is)
#   make -f oracle/ref.mk             (anywhere the staged copy exists)
#
# `stage` copies the reference files this recipe compiles (solver sources and headers) and the
# reference's two box-QP QPLIB instances with their manifest into oracle/_ref/, which git ignores
# and which travels with the working tree to machines without the reference checkout (the GPU
# host, an aarch64 machine that must compile them itself).  Every other target builds from that
# staged copy.  REF is the reference project's solver directory: BOXQP_REFERENCE_DIR when set,
# else the checkout location of the build container.
REF ?= $(or $(BOXQP_REFERENCE_DIR),/root/reference/02-software/solver)
OUT := oracle/_ref
SRC := $(OUT)/src
CXX ?= g++
# -ffp-contract=off keeps products and sums separately rounded on every host, which is
# what the reference's x86-64 Release build does.
CXXFLAGS := -std=c++14 -O3 -fopenmp -fPIC -ffp-contract=off -I$(SRC)/include -w

SRCS := solver.cpp mps.cpp milp_v2.cpp qp.cpp qp_admm.cpp qp_dual_newton.cpp \
        sparse_lp.cpp bounded_simplex.cpp accelerated_qp.cpp
STAGED_SRCS := $(SRCS) scale_benchmark.cpp main.cpp cuda_box.cu
QPLIB := 8792.qplib 8991.qplib manifest.json
OBJS := $(addprefix $(OUT)/,$(SRCS:.cpp=.o)) $(OUT)/ref_shim.o

all: $(OUT)/libsovereign_ref.so

# Copies only when the reference checkout exists; cp -p keeps the sources' times, so a second
# stage does not trigger rebuilds.
stage:
	@if [ -d "$(REF)/src" ]; then \
	    mkdir -p $(SRC)/src $(SRC)/include $(OUT)/qplib && \
	    for f in $(STAGED_SRCS); do cp -p "$(REF)/src/$$f" $(SRC)/src/; done && \
	    cp -p "$(REF)"/include/*.hpp $(SRC)/include/ && \
	    for f in $(QPLIB); do cp -p "$(REF)/datasets/qplib/$$f" $(OUT)/qplib/; done; \
	fi

$(OUT):
	mkdir -p $(OUT)

$(OUT)/%.o: $(SRC)/src/%.cpp | $(OUT)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/ref_shim.o: oracle/ref_shim.cpp | $(OUT)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/libsovereign_ref.so: $(OBJS)
	$(CXX) -shared -fopenmp -o $@ $(OBJS)

# The reference's own scale harness and JSON CLI, CPU build (their cuda backend reports "No CUDA
# device available" through the reference's stub of make_cuda_box).
$(OUT)/solver_scale_ref: $(OBJS) $(SRC)/src/scale_benchmark.cpp
	$(CXX) $(CXXFLAGS) $(SRC)/src/scale_benchmark.cpp $(addprefix $(OUT)/,$(SRCS:.cpp=.o)) -o $@

.PHONY: all stage

# Level-A drop-in check: the reference's library with SOVEREIGN_CUDA defined (so its CPU stub of
# make_cuda_box drops out), the GB300 plugin hypergrey-sih-26_gb300/plugin/cuda_box_gb300.cpp in
# place of src/cuda_box.cu, and the reference's own CLI and scale harness linked against
# libboxqp.so.  Outputs only into oracle/_ref.
#
# The *_gb300_engine variants link the same unmodified objects with -Wl,--wrap for
# sovereign::solve_accelerated_box: the call from the CLI and the scale harness lands in
# __wrap_ (plugin/engine_route.cpp), which sends cuda = true to the device-resident engine
# (bqp_solve_sync) and everything else to the reference's own function.  It is the link-level
# form of the one-line change to solve_accelerated_box that INTEGRATION.md describes.
PKG := hypergrey-sih-26_gb300
LIBDIR := $(abspath $(PKG)/boxqp)
LVL_FLAGS := $(CXXFLAGS) -DSOVEREIGN_CUDA=1 -Iinclude
# Only accelerated_qp.cpp reads SOVEREIGN_CUDA: the other objects are the library's own.
PLAIN_SRCS := $(filter-out accelerated_qp.cpp,$(SRCS))
LVL_OBJS := $(addprefix $(OUT)/,$(PLAIN_SRCS:.cpp=.o)) $(OUT)/lvl_accelerated_qp.o $(OUT)/lvl_plugin.o
WRAP := -Wl,--wrap=_ZN9sovereign21solve_accelerated_boxERKNS_16QuadraticProblemERKNS_9QpOptionsEb

$(OUT)/lvl_accelerated_qp.o: $(SRC)/src/accelerated_qp.cpp | $(OUT)
	$(CXX) $(LVL_FLAGS) -c $< -o $@

$(OUT)/lvl_plugin.o: $(PKG)/plugin/cuda_box_gb300.cpp | $(OUT)
	$(CXX) $(LVL_FLAGS) -c $< -o $@

$(OUT)/lvl_route.o: $(PKG)/plugin/engine_route.cpp | $(OUT)
	$(CXX) $(LVL_FLAGS) -c $< -o $@

$(OUT)/solver_scale_gb300: $(LVL_OBJS) $(SRC)/src/scale_benchmark.cpp
	$(CXX) $(LVL_FLAGS) $(SRC)/src/scale_benchmark.cpp $(LVL_OBJS) -L$(LIBDIR) -lboxqp -Wl,-rpath,$(LIBDIR) -o $@

$(OUT)/solver_cli_gb300: $(LVL_OBJS) $(SRC)/src/main.cpp
	$(CXX) $(LVL_FLAGS) $(SRC)/src/main.cpp $(LVL_OBJS) -L$(LIBDIR) -lboxqp -Wl,-rpath,$(LIBDIR) -o $@

$(OUT)/solver_scale_gb300_engine: $(LVL_OBJS) $(OUT)/lvl_route.o $(SRC)/src/scale_benchmark.cpp
	$(CXX) $(LVL_FLAGS) $(SRC)/src/scale_benchmark.cpp $(LVL_OBJS) $(OUT)/lvl_route.o $(WRAP) -L$(LIBDIR) -lboxqp \
	    -Wl,-rpath,$(LIBDIR) -o $@

$(OUT)/solver_cli_gb300_engine: $(LVL_OBJS) $(OUT)/lvl_route.o $(SRC)/src/main.cpp
	$(CXX) $(LVL_FLAGS) $(SRC)/src/main.cpp $(LVL_OBJS) $(OUT)/lvl_route.o $(WRAP) -L$(LIBDIR) -lboxqp \
	    -Wl,-rpath,$(LIBDIR) -o $@

level_a: $(OUT)/solver_scale_gb300 $(OUT)/solver_cli_gb300 $(OUT)/solver_scale_gb300_engine \
         $(OUT)/solver_cli_gb300_engine

.PHONY: level_a

# The reference's CUDA plugin kernels, unmodified, compiled for this GPU into a loadable module
# (device code only; oracle/ref_cuda_harness.c drives it with the reference's host loop).
NVCC ?= nvcc
$(OUT)/cuda_box_sm103a.cubin: $(SRC)/src/cuda_box.cu | $(OUT)
	$(NVCC) -cubin -gencode arch=compute_103a,code=sm_103a -O3 -I$(SRC)/include -w -o $@ $<

cuda_cubin: $(OUT)/cuda_box_sm103a.cubin

.PHONY: cuda_cubin
