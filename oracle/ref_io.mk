# Builds, from the reference's sources where they lie (src/Particle.cu, and
# src/main.cu for its globals and itoa with the reference's main renamed):
#   oracle/_ref/ref_io     GPUCell's own input loaders and output writers,
#                          driven by oracle/ref_io.cu; the boundary entry
#                          points Particle.cu also calls come from this
#                          library and are never called
#   oracle/_ref/ref_calls  its step driver against the recording entry points
#                          of oracle/ref_calls_stubs.cu, driven by
#                          oracle/ref_calls.cu
# Test infrastructure only: run from the repository root,
#   make -f oracle/ref_io.mk REF=<reference>/src
# (gpucell_gb300/build.py passes $GPUCELL_REFERENCE/src).  Without the
# reference's sources it builds nothing.
REF ?= $(GPUCELL_REFERENCE)/src
NVCC ?= nvcc
OUT := oracle/_ref
LIB := gpucell_gb300/lib

ifneq ($(wildcard $(REF)/Particle.cu),)
all: $(OUT)/ref_io $(OUT)/ref_calls
else
all:
	@echo "ref_io: no reference sources at $(REF); nothing to build"
endif

$(OUT)/ref_io: oracle/ref_io.cu $(REF)/Particle.cu $(REF)/main.cu $(LIB)/libgpucell_gb300.so
	mkdir -p $(OUT)
	$(NVCC) -w -O1 -I$(REF) -c $(REF)/Particle.cu -o $(OUT)/Particle.o
	$(NVCC) -w -O1 -I$(REF) -Dmain=gpucell_reference_main -c $(REF)/main.cu -o $(OUT)/main.o
	$(NVCC) -O1 -I$(REF) -c oracle/ref_io.cu -o $(OUT)/ref_io.o
	$(NVCC) $(OUT)/ref_io.o $(OUT)/Particle.o $(OUT)/main.o -o $@ -L$(LIB) -lgpucell_gb300 \
		-Xlinker -rpath=$(abspath $(LIB))

# GPUCell's step driver against recording entry points (no library)
$(OUT)/ref_calls: oracle/ref_calls.cu oracle/ref_calls_stubs.cu $(OUT)/ref_io
	$(NVCC) -O1 -I$(REF) -c oracle/ref_calls.cu -o $(OUT)/ref_calls.o
	$(NVCC) -O1 -Iinclude -c oracle/ref_calls_stubs.cu -o $(OUT)/ref_calls_stubs.o
	$(NVCC) $(OUT)/ref_calls.o $(OUT)/ref_calls_stubs.o $(OUT)/Particle.o $(OUT)/main.o -o $@
