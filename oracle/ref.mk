# Builds the reference's AD-only executable from its own sources, where they
# lie, into oracle/_ref/ (nvcc, sm_103a).  PPESolver.cu is left out: it does
# not compile, and main() does not call it.  The executable reads
# ../inputs/inputs.txt and ../inputs/xgrid.dat2 / ygrid.dat2 and writes
# ../results/*.dat relative to where it runs.
#   make -f oracle/ref.mk REF=<reference checkout>
REF ?= /root/reference
NVCC ?= /usr/local/cuda/bin/nvcc
OUT := $(dir $(lastword $(MAKEFILE_LIST)))_ref
SRC := $(REF)/src/include/globalVariables.cu $(REF)/src/include/preSim.cu $(REF)/src/include/ADSolver.cu \
       $(REF)/src/include/AD_PPE_Correction.cu $(REF)/src/include/postSim.cu $(REF)/src/main.cu
OBJ := $(patsubst $(REF)/src/%.cu,$(OUT)/obj/%.o,$(SRC))

ifeq ($(wildcard $(REF)/src/main.cu),)
all:
	@echo "reference sources absent: nothing to build"
else
all: $(OUT)/immerseflow_ref
endif

$(OUT)/immerseflow_ref: $(OBJ)
	$(NVCC) -gencode arch=compute_103a,code=sm_103a -o $@ $(OBJ)

$(OUT)/obj/%.o: $(REF)/src/%.cu
	@mkdir -p $(dir $@)
	$(NVCC) -gencode arch=compute_103a,code=sm_103a -O2 -w -c $< -o $@

.PHONY: all clean
clean:
	rm -rf $(OUT)
