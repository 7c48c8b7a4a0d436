# Builds the reference pinning harness (test infrastructure) from the reference
# sources where they lie: g++ on lib_ensembles/source/gpudte.cu (device code
# compiled as host code through ref_shim/), and on the host-side sources of
# lib_core, lib_data and lib_parsing.  The reference's own CMake build is not
# used.  Output: oracle/_ref/libref.so (git-ignored).  REF names the reference
# tree; oracle/ref.py passes it (from DML_REFERENCE_ROOT).
ifndef REF
$(error REF must name the reference source tree)
endif
OUT := _ref
CXX ?= g++
CXXFLAGS := -O1 -std=c++14 -fPIC -ffp-contract=off -w
REFINC := -I$(REF) -I$(REF)/source_shared -I$(REF)/source_shared/include \
  -I$(REF)/lib_core/include -I$(REF)/lib_core/source \
  -I$(REF)/lib_data/include -I$(REF)/lib_data/source \
  -I$(REF)/lib_models/include -I$(REF)/lib_parsing/include \
  -I$(REF)/lib_parsing/source -I$(REF)/lib_algorithms/include
HOSTSRC := lib_core/source/core_interface.cc lib_core/source/barrier_impl.cc \
  lib_data/source/data_interface.cc lib_data/source/ml_dataframe_impl.cc \
  lib_data/source/ml_resultdata_impl.cc lib_parsing/source/csv_parser.cc \
  lib_parsing/source/parsing_interface.cc lib_parsing/source/ml_parser.cc
HOSTOBJ := $(addprefix $(OUT)/,$(notdir $(HOSTSRC:.cc=.o)))

all: $(OUT)/libref.so

$(OUT)/%.o:
	mkdir -p $(OUT)
	$(CXX) $(CXXFLAGS) -DUnixBuild -include $(REF)/source_shared/precomp.h $(REFINC) -c $(REF)/$(filter %/$*.cc,$(HOSTSRC)) -o $@

$(OUT)/ref_harness.o: ref_harness.cc ref_shim/host_emulation.h
	mkdir -p $(OUT)
	$(CXX) $(CXXFLAGS) -Iref_shim $(REFINC) -c ref_harness.cc -o $@

$(OUT)/libref.so: $(HOSTOBJ) $(OUT)/ref_harness.o
	$(CXX) -shared -o $@ $^ -lpthread

clean:
	rm -rf $(OUT)

.PHONY: all clean
