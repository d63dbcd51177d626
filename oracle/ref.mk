# Builds the reference OpenMOC C++ library (its src/*.cpp, compiled where they
# lie) twice: FP_PRECISION=float (the CPUSolver being matched) and
# FP_PRECISION=double (the FP64 accuracy oracle). Outputs only go to
# oracle/_ref/, which is git-ignored. Flags follow the reference's own gcc
# build (config.py: -O3 -ffast-math -fopenmp -std=c++11 -fpic, the
# FP_PRECISION / VEC_LENGTH / VEC_ALIGNMENT / SINGLE / GCC / OPENMP macros),
# plus -fno-finite-math-only: the sources compare against infinity (e.g. the
# infinite lattice z-width test in Lattice::getLatZ, src/Universe.cpp:1986),
# which gcc 13 folds away under plain -ffast-math.
#
# Also links oracle/openmoc_run.cpp (OpenMOC run on the benchmark
# configurations: golden files and the timed CPU baseline) against each build.
#
#   make -f oracle/ref.mk REF=<OpenMOC source tree> -j8
ifndef REF
$(error REF must name an OpenMOC source tree (the directory holding src/))
endif
ORACLE := $(patsubst %/,%,$(dir $(lastword $(MAKEFILE_LIST))))
OUT ?= oracle/_ref
CXX ?= g++

SRCS := Cell Cmfd CPUSolver CPULSSolver ExpEvaluator Geometry linalg \
        LocalCoords log Material Matrix Mesh MOCKernel Point Progress \
        Quadrature Region RunTime Solver Surface Timer Track Track3D \
        TrackGenerator TrackGenerator3D TrackTraversingAlgorithms \
        TraverseSegments Universe Vector

COMMON := -O3 -ffast-math -fno-finite-math-only -fopenmp -std=c++11 -fpic -w -DGCC -DOPENMP \
          -DVEC_ALIGNMENT=64
F32DEFS := -DFP_PRECISION=float -DSINGLE -DVEC_LENGTH=8 -DCMFD_PRECISION=float \
           -DLINALG_TOL=1E-7
F64DEFS := -DFP_PRECISION=double -DVEC_LENGTH=4 -DCMFD_PRECISION=double \
           -DLINALG_TOL=1E-15
F32FLAGS := $(COMMON) $(F32DEFS)
F64FLAGS := $(COMMON) $(F64DEFS)
RUNFLAGS := -O2 -fopenmp -std=c++11 -w -DGCC -DOPENMP -DVEC_ALIGNMENT=64 -I$(REF)/src

OBJ32 := $(addprefix $(OUT)/f32/,$(addsuffix .o,$(SRCS)))
OBJ64 := $(addprefix $(OUT)/f64/,$(addsuffix .o,$(SRCS)))
RUN_DEPS := $(ORACLE)/openmoc_run.cpp $(ORACLE)/../openmoc_gb300/adapter/pack_reference.h \
            $(ORACLE)/../openmoc_gb300/csrc/synthetic_xs.h

all: $(OUT)/libopenmoc_f32.a $(OUT)/libopenmoc_f64.a \
     $(OUT)/openmoc_run_f32 $(OUT)/openmoc_run_f64

$(OUT)/f32/%.o: $(REF)/src/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(F32FLAGS) -c $< -o $@

$(OUT)/f64/%.o: $(REF)/src/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(F64FLAGS) -c $< -o $@

$(OUT)/libopenmoc_f32.a: $(OBJ32)
	ar rcs $@ $^

$(OUT)/libopenmoc_f64.a: $(OBJ64)
	ar rcs $@ $^

$(OUT)/openmoc_run_f32: $(RUN_DEPS) $(OUT)/libopenmoc_f32.a
	$(CXX) $(RUNFLAGS) $(F32DEFS) $< $(OUT)/libopenmoc_f32.a -o $@

$(OUT)/openmoc_run_f64: $(RUN_DEPS) $(OUT)/libopenmoc_f64.a
	$(CXX) $(RUNFLAGS) $(F64DEFS) $< $(OUT)/libopenmoc_f64.a -o $@

.PHONY: all
