# The reference's own AD-only CUDA executable (test and baseline side only).
#
#   make -f oracle/ref.mk stage REF=<reference checkout>
#       copies the sources the executable needs (src/main.cu, src/header/,
#       src/include/{globalVariables,preSim,ADSolver,AD_PPE_Correction,postSim}.cu)
#       unmodified into oracle/_ref/src/, with a NOTICE naming their origin and
#       licence (MIT, the reference's README.md:3).  oracle/_ref/ is git-ignored:
#       the copy is never committed, it only travels with the working tree to
#       the machine that builds and runs it.
#   make -f oracle/ref.mk
#       builds oracle/_ref/immerseflow_ref from the staged copy (nvcc, sm_103a,
#       otherwise the flags of the reference's own src/Makefile), with
#       oracle/ref_guard.h force-included: it pads every cudaMalloc so that the
#       initial-condition kernel's writes past the face arrays stay in owned
#       memory.  PPESolver.cu is left out: it does not compile, and main()
#       does not call it.
#
# The executable reads ../inputs/inputs.txt and ../inputs/xgrid.dat2 /
# ygrid.dat2 and writes ../results/*.dat relative to its working directory
# (oracle/ref_run.py sets that up).
NVCC ?= /usr/local/cuda/bin/nvcc
OUT := $(dir $(lastword $(MAKEFILE_LIST)))_ref
SRCDIR := $(OUT)/src
UNITS := include/globalVariables include/preSim include/ADSolver include/AD_PPE_Correction include/postSim main
OBJ := $(patsubst %,$(OUT)/obj/%.o,$(UNITS))
GUARD := $(abspath $(dir $(lastword $(MAKEFILE_LIST)))ref_guard.h)

ifeq ($(wildcard $(SRCDIR)/main.cu),)
all:
	@echo "reference sources not staged in $(SRCDIR): nothing to build"
else
all: $(OUT)/immerseflow_ref
endif

stage:
ifeq ($(REF),)
	$(error stage needs REF=<reference checkout>)
endif
	@test -f $(REF)/src/main.cu || { echo "no reference sources under $(REF)"; exit 1; }
	@mkdir -p $(SRCDIR)/include $(SRCDIR)/header
	@cp $(REF)/src/main.cu $(SRCDIR)/main.cu
	@cp $(REF)/src/header/*.cuh $(REF)/src/header/*.h $(SRCDIR)/header/
	@for u in globalVariables preSim ADSolver AD_PPE_Correction postSim; do \
	    cp $(REF)/src/include/$$u.cu $(SRCDIR)/include/$$u.cu; done
	@{ echo "Unmodified sources of sushrutkr/ImmerseFlow (ImmerseFlow++), MIT licence"; \
	   echo "(the reference's README.md:3), staged for a build-and-compare baseline."; \
	   echo "Not part of this repository's product or history."; } > $(SRCDIR)/NOTICE

$(OUT)/immerseflow_ref: $(OBJ)
	$(NVCC) -gencode arch=compute_103a,code=sm_103a -o $@ $(OBJ)

$(OUT)/obj/%.o: $(SRCDIR)/%.cu $(GUARD)
	@mkdir -p $(dir $@)
	$(NVCC) -gencode arch=compute_103a,code=sm_103a -w -include $(GUARD) -c $< -o $@

.PHONY: all stage clean
clean:
	rm -rf $(OUT)/obj $(OUT)/immerseflow_ref
