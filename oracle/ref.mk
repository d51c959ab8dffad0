# Builds the reference's own pressure-path sources, unmodified and where they
# lie, into oracle/_ref/libvfsref.so: a checker of the oracle restatement
# (test infrastructure; git-ignored output, nothing of the product links it).
#
#   make -f ref.mk REF=<reference checkout>      (from oracle/)
#
# The sources include PETSc 3.2, HYPRE and MPI headers; ref_stub/ provides
# single-rank stand-ins under the same header names.  The compiled files are
# the translation units that define the path's functions: FormMetrics
# (metrics.c), setup_lidx2, PoissonLHSNew, VolumeFlux, Projection,
# UpdatePressure and the multigrid transfers (poisson.c), PoissonRHS2_hypre
# (poisson_hypre.c), Divergence and the run-option globals (main.c),
# Contra2Cart (rhs.c), the global sums (rhs2.c), MG set-up (init.c) and the
# Cmpnts helpers FormMetrics calls (momentum.c).  The reference's makefile builds
# them with mpicxx as C++; here g++ with FP contraction off (the oracle's
# arithmetic).  Functions those files call in other reference files (the rest
# of the solver) are bound to stubs that abort if the checked path ever
# reaches them (_ref/unbound.cpp, generated from the link's undefined list).
REF ?= /root/reference
CXX ?= g++
OUT := _ref
LIB := $(OUT)/libvfsref.so
SRCS := metrics poisson poisson_hypre main rhs rhs2 init momentum
FLAGS := -O2 -ffp-contract=off -fPIC -w -std=gnu++17 -Iref_stub -I$(REF) -Dmain=vfs_ref_unused_main
OBJS := $(SRCS:%=$(OUT)/%.o) $(OUT)/vfs_ref_stub.o $(OUT)/ref_harness.o

all: $(LIB)

$(OUT)/%.o: $(REF)/%.c ref_stub/vfs_ref_stub.h
	@mkdir -p $(OUT)
	$(CXX) $(FLAGS) -x c++ -c $< -o $@

$(OUT)/vfs_ref_stub.o: ref_stub/vfs_ref_stub.cpp ref_stub/vfs_ref_stub.h
	@mkdir -p $(OUT)
	$(CXX) $(FLAGS) -c $< -o $@

$(OUT)/ref_harness.o: ref_harness.cpp ref_stub/vfs_ref_stub.h
	@mkdir -p $(OUT)
	$(CXX) $(FLAGS) -c $< -o $@

# unbound.cpp: one aborting definition per symbol the objects leave undefined
# that neither the C/C++ runtime nor libm provides
$(OUT)/unbound.cpp: $(OBJS) ref_unbound.py
	python3 ref_unbound.py $(OUT)/unbound.cpp $(OBJS)

$(OUT)/unbound.o: $(OUT)/unbound.cpp
	$(CXX) -O0 -fPIC -w -c $< -o $@

$(LIB): $(OBJS) $(OUT)/unbound.o
	$(CXX) -shared -o $@ $^ -lm -Wl,--no-undefined

clean:
	rm -rf $(OUT)

.PHONY: all clean
