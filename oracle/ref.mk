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
