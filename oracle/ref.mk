# Builds the unmodified FHedin/mc_cpp reference (scalar FField_MDBAS path) from the sources
# where they lie, plus this repository's own probe driver linked against those objects.
#
#   make -f oracle/ref.mk REF=<directory of the mc_cpp sources>    (run from the repository root)
#
# Outputs go to oracle/_ref/ only (git-ignored).  Nothing here is shipped or measured as the
# product: the probe is test infrastructure used to pin the oracle restatement and to generate
# golden fixtures under tests/golden/.
#
# Deviations from the reference's own CMake build, all outside the reference's arithmetic:
#  * Global_include.hpp is generated here (CMake's configure_file step).
#  * -include cmath -include limits: Move.hpp / Parser.hpp rely on transitive includes that
#    g++ 13 no longer provides.
#  * List_nonBonded.cpp is compiled from a copy in oracle/_ref/patched/ with TOLLIST raised from
#    0.02 to 0.5.  The reference sizes each Verlet row once (List_nonBonded.cpp:827-830) and has
#    its growth check commented out (:885-902), so long MC runs overflow the heap at :904.  TOLLIST
#    only sets row capacity; list contents and energies are unchanged.
#  * -std=c++11 keeps GCC in ISO mode, so no FMA contraction (-ffp-contract=off is implied); the
#    restatement in oracle/mc_oracle.cpp is built the same way so FP64 sums agree bit for bit.

ifeq ($(strip $(REF)),)
$(error REF must name the directory of the FHedin/mc_cpp sources: make -f oracle/ref.mk REF=<dir>)
endif
OUT      := oracle/_ref
CXX      ?= g++
CXXFLAGS := -std=c++11 -O3 -ffp-contract=off -fopenmp -w -include cmath -include limits \
            -I$(OUT)/gen -I$(REF)/include -I$(REF)/include/experimental -I$(REF)/rapidxml-1.13

SRCNAMES := Angle AtomList Bond Bond_UB Dihedral Dihedral_improper Ensemble Ens_NVT FField \
            FField_MDBAS IO IO_MDBAS List_Moves MC MC_metropolis Parser PerConditions Selection
OBJS     := $(addprefix $(OUT)/obj/,$(addsuffix .o,$(SRCNAMES))) $(OUT)/obj/List_nonBonded.o

all: $(OUT)/ref_probe $(OUT)/mc_cpp $(OUT)/libcharmmene.so

$(OUT)/gen/Global_include.hpp:
	@mkdir -p $(OUT)/gen
	printf '#ifndef GLOBAL_INCLUDE_H\n#define GLOBAL_INCLUDE_H\n#define VERSION_MAJOR 0\n#define VERSION_MINOR 2\n#define PROGRAM_NAME "mc_cpp"\n#endif\n' > $@

$(OUT)/patched/List_nonBonded.cpp: $(REF)/src/List_nonBonded.cpp
	@mkdir -p $(OUT)/patched
	sed 's/TOLLIST = 0\.02;/TOLLIST = 0.5;/' $< > $@
	grep -q 'TOLLIST = 0.5;' $@

$(OUT)/obj/%.o: $(REF)/src/%.cpp $(OUT)/gen/Global_include.hpp
	@mkdir -p $(OUT)/obj
	$(CXX) $(CXXFLAGS) -fPIC -c $< -o $@

$(OUT)/obj/List_nonBonded.o: $(OUT)/patched/List_nonBonded.cpp $(OUT)/gen/Global_include.hpp
	@mkdir -p $(OUT)/obj
	$(CXX) $(CXXFLAGS) -fPIC -c $< -o $@

$(OUT)/obj/mc_cpp_main.o: $(REF)/src/mc_cpp.cpp $(OUT)/gen/Global_include.hpp
	@mkdir -p $(OUT)/obj
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/obj/FORTRAN_interface.o: $(REF)/src/FORTRAN_interface.cpp $(OUT)/gen/Global_include.hpp
	@mkdir -p $(OUT)/obj
	$(CXX) $(CXXFLAGS) -fPIC -c $< -o $@

$(OUT)/mc_cpp: $(OBJS) $(OUT)/obj/mc_cpp_main.o
	$(CXX) $(CXXFLAGS) $^ -o $@

$(OUT)/libcharmmene.so: $(OBJS) $(OUT)/obj/FORTRAN_interface.o
	$(CXX) $(CXXFLAGS) -shared $^ -o $@

$(OUT)/ref_probe: oracle/ref_probe.cpp $(OBJS)
	$(CXX) $(CXXFLAGS) oracle/ref_probe.cpp $(OBJS) -o $@

# FField_CUDA (mc_cpp_gb300/adapter/) compiled with the reference's headers and flags and linked
# with the reference objects and libmcgpu.so: the drop-in as a maintainer would build it.
LIBDIR   := mc_cpp_gb300/_lib
$(OUT)/adapter_check: oracle/adapter_check.cpp mc_cpp_gb300/adapter/FField_CUDA.cpp mc_cpp_gb300/adapter/FField_CUDA.hpp \
                      include/mcg.h $(OBJS) $(LIBDIR)/libmcgpu.so
	$(CXX) $(CXXFLAGS) -Wall -Imc_cpp_gb300/adapter -Iinclude oracle/adapter_check.cpp mc_cpp_gb300/adapter/FField_CUDA.cpp \
	    $(OBJS) -L$(LIBDIR) -lmcgpu -Wl,-rpath,$(abspath $(LIBDIR)) -o $@

# exit status 0 when the reference sources are where REF points
ref-present:
	@test -f $(REF)/src/FField_MDBAS.cpp

clean:
	rm -rf $(OUT)

.PHONY: all clean ref-present
