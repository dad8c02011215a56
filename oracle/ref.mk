# Builds the reference DVM-system runtime (libdvm + libdvmh, host-only, OpenMP host
# handlers) from its own sources, where they lie, into oracle/_ref/.  Test
# infrastructure only: the result is the oracle that pins oracle/restate.c and
# generates tests/golden/.  Nothing in the product links it.
#
# usage:  make -f oracle/ref.mk -j8 REF=<the reference checkout>/dvm_sys
#
# What is compiled (file lists follow rts/src/makefile.uni OBJ_C/OBJ_FTN and
# rts/dvmh/makefile.uni OBJ, written out here; the reference makefiles are not run):
#   libdvm : the nine unity units rts/src/1.c..9.c, the zlib wrappers rts/src/_*.c,
#            rts/src/linitstd.c (the Fortran clfdvm.f is left out: no gfortran);
#   libdvmh: every rts/dvmh/*.cpp and the four rts/dvmh/*.cu compiled as C++
#            without HAVE_CUDA (their CUDA paths compile to error stubs).
# Two small headers are written into oracle/_ref/gen: dvmvers.h (version strings the
# sources expect from the installer) and an empty dynamic_include.h (NVRTC hook).
# Defines = the reference installer's single-process, MPI-stub configuration.

ifndef REF
$(error REF must name the reference dvm_sys source tree)
endif
OUT     ?= oracle/_ref
GEN      = $(OUT)/gen
OBJ_DIR  = $(OUT)/obj

CC      ?= gcc
CXX     ?= g++
DVMOPT   = -D_DVM_MPI_ -DMPICH_IGNORE_CXX_SEEK -DOMPI_SKIP_MPICXX=1 -DMPICH_SKIP_MPICXX=1 \
           -DMPI_NO_CPPBIND -D_MPI_STUBS_ -D_RTS_ZLIB_ -D_UNIX_ -D_F_TIME_ -D_DATA_ALIGN_ACCESS_
CFLAGS_DVM  = -O2 -fopenmp -fPIC -w $(DVMOPT) -D_MPI_PROF_EXT_ -I$(GEN) \
              -I$(REF)/rts/src -I$(REF)/rts/include -I$(REF)/tools/Zlib/src -I$(REF)/tools/Zlib/include
CFLAGS_DVMH = -O2 -fopenmp -fPIC -w -fvisibility=hidden $(DVMOPT) -I$(GEN) \
              -I$(REF)/rts/include -I$(REF)/rts/dvmh/include -I$(REF)/rts/dvmh

DVM_SRC  = $(addprefix $(REF)/rts/src/,1.c 2.c 3.c 4.c 5.c 6.c 7.c 8.c 9.c linitstd.c \
             _adler32.c _compress.c _crc32.c _gzio.c _uncompr.c _deflate.c _trees.c _zutil.c \
             _inflate.c _infblock.c _inftrees.c _infcodes.c _infutil.c _inffast.c)
DVMH_CPP = $(wildcard $(REF)/rts/dvmh/*.cpp)
DVMH_CU  = $(wildcard $(REF)/rts/dvmh/*.cu)

DVM_OBJ  = $(patsubst $(REF)/rts/src/%.c,$(OBJ_DIR)/dvm/%.o,$(DVM_SRC))
DVMH_OBJ = $(patsubst $(REF)/rts/dvmh/%.cpp,$(OBJ_DIR)/dvmh/%.o,$(DVMH_CPP)) \
           $(patsubst $(REF)/rts/dvmh/%.cu,$(OBJ_DIR)/dvmh/%.cu.o,$(DVMH_CU))

all: $(OUT)/libdvm.a $(OUT)/libdvmh.a $(OUT)/pstub.o $(OUT)/ref_driver

# The workload programs (same sources the GPU build uses, without CUDA handlers)
# linked against the reference runtime: the order-exact oracle with DVMH_NUM_THREADS=1.
WL      ?= dvm-snapshot-r6603-fork_gb300/workloads
WL_SRC   = $(WL)/jac2d.c $(WL)/jac3d.c $(WL)/sor3d.c $(WL)/heat.c $(WL)/gsd2d.c $(WL)/genred.c $(WL)/rec2d.c $(WL)/gsd3d.c $(WL)/gs2d.c $(WL)/gen3d.c $(WL)/jacperf.c $(WL)/cdvh2d.c $(WL)/cdvh2d_init.cpp oracle/ref_driver.c
WL_CFLAGS = -O2 -fopenmp -ffp-contract=off -fno-fast-math -DWL_NO_CUDA -I$(REF)/rts/dvmh/include -I$(WL)

$(OUT)/ref_driver: $(WL_SRC) $(WL)/wl_common.h $(OUT)/libdvm.a $(OUT)/libdvmh.a $(OUT)/pstub.o
	$(CC) $(WL_CFLAGS) $(WL_SRC) $(OUT)/pstub.o $(OUT)/libdvmh.a $(OUT)/libdvm.a -lstdc++ -lrt -lm -lpthread -o $@

$(GEN)/dvmvers.h:
	mkdir -p $(GEN)
	printf '#define VERS "oracle"\n#define PLATFORM "gnu_noMPI"\n#define _DVM_Minus_ %s\n' "'-'" > $@
	: > $(GEN)/dynamic_include.h

$(OBJ_DIR)/dvm/%.o: $(REF)/rts/src/%.c $(GEN)/dvmvers.h
	@mkdir -p $(dir $@)
	$(CC) $(CFLAGS_DVM) -c $< -o $@

$(OBJ_DIR)/dvmh/%.o: $(REF)/rts/dvmh/%.cpp $(GEN)/dvmvers.h
	@mkdir -p $(dir $@)
	$(CXX) $(CFLAGS_DVMH) -c $< -o $@

$(OBJ_DIR)/dvmh/%.cu.o: $(REF)/rts/dvmh/%.cu $(GEN)/dvmvers.h
	@mkdir -p $(dir $@)
	$(CXX) $(CFLAGS_DVMH) -x c++ -c $< -o $@

$(OUT)/libdvm.a: $(DVM_OBJ)
	rm -f $@ && ar crs $@ $^

$(OUT)/libdvmh.a: $(DVMH_OBJ)
	rm -f $@ && ar crs $@ $^

# -D_MPI_PROF_EXT_ drops the MPI profiling layer that would define this symbol.
$(OUT)/pstub.o:
	@mkdir -p $(OUT)
	printf 'int PMPI_Finalize(void){return 0;}\n' > $(OUT)/pstub.c
	$(CC) -O2 -c $(OUT)/pstub.c -o $@

.PHONY: all
