# Builds the MAPP reference itself, from its sources where they lie, into
# oracle/_ref/ as the Python module `mapp4py` (test infrastructure only: the
# second oracle that pins oracle.c and the golden fixtures).
#
#   make -f oracle/ref.mk -j16 REF=/path/to/mapp4py
#
# Nothing is copied out of the reference tree.  What makes it build here:
#  - refshim/mpi.h + mpi_shim.c: a single-rank MPI (no MPI library exists on
#    these machines);
#  - refshim/compat.h, forced in with -include: Python 3.12 / NumPy 2
#    compatibility macros (lvalue Py_TYPE/Py_REFCNT, co_varnames);
#  - -DNPY_TARGET_VERSION=NPY_2_0_API_VERSION for PyArray_Descr::elsize;
#  - refshim/ref_probe.cpp: entry points that set exact states and read
#    forces through the reference's ForceFieldMD (see that file).
# -ffp-contract=off keeps the reference's unfused rounding on any host.
# -O0: NewDynamicMD declares `void reset(){};` with an empty body in the
# class (dynamic_md.h:185) while its working body is an explicit
# specialization in dynamic_md.cpp:175,228 that the minimizers' translation
# units never see.  An optimising build inlines (or drops as a pure call)
# the empty body there, so md.min_lbfgs / md.min_cg never rebuild their
# neighbour lists once atoms pass the skin and compute forces on stale
# lists.  Unoptimised, every call goes through the symbol and links to the
# specialization (strong over the weak implicit instantiation), which is
# the behaviour the code intends.  IEEE results are the same at any -O on
# x86-64 (SSE2, no contraction).
REF     ?= /root/reference
HERE    := $(dir $(abspath $(lastword $(MAKEFILE_LIST))))
OUT     := $(HERE)_ref
SHIM    := $(HERE)refshim
PY      ?= python3
PYINC   := $(shell $(PY) -c "import sysconfig; print(sysconfig.get_paths()['include'])")
NPINC   := $(shell $(PY) -c "import numpy; print(numpy.get_include())")
EXT     := $(shell $(PY) -c "import sysconfig; print(sysconfig.get_config_var('EXT_SUFFIX'))")
CXX     ?= g++
CC      ?= gcc
FLAGS   := -O0 -fPIC -w -ffp-contract=off -fno-fast-math
CXXFLAGS_REF := -std=c++11 $(FLAGS) -I$(SHIM) -I$(REF)/src -I$(PYINC) -I$(NPINC) \
                -DNPY_TARGET_VERSION=NPY_2_0_API_VERSION -include $(SHIM)/compat.h

SRCS    := $(wildcard $(REF)/src/*.cpp)
OBJS    := $(patsubst $(REF)/src/%.cpp,$(OUT)/obj/%.o,$(SRCS)) \
           $(OUT)/obj/_ref_probe.o $(OUT)/obj/_mpi_shim.o
LIB     := $(OUT)/mapp4py$(EXT)

all: $(LIB)

$(LIB): $(OBJS)
	$(CXX) -shared -o $@ $(OBJS)

$(OUT)/obj/%.o: $(REF)/src/%.cpp
	@mkdir -p $(OUT)/obj
	$(CXX) $(CXXFLAGS_REF) -c $< -o $@

$(OUT)/obj/_ref_probe.o: $(SHIM)/ref_probe.cpp $(SHIM)/compat.h $(SHIM)/mpi.h
	@mkdir -p $(OUT)/obj
	$(CXX) $(CXXFLAGS_REF) -c $< -o $@

$(OUT)/obj/_mpi_shim.o: $(SHIM)/mpi_shim.c $(SHIM)/mpi.h
	@mkdir -p $(OUT)/obj
	$(CC) $(FLAGS) -c $< -o $@

clean:
	rm -rf $(OUT)

.PHONY: all clean
