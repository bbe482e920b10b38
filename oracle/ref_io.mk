# Builds oracle/_ref/ref_io: GPUCell's own input loaders and output writers
# (src/Particle.cu, with src/main.cu for its globals and itoa; the
# reference's main renamed) linked with oracle/ref_io.cu, from the
# reference's sources where they lie.  The boundary entry points that
# Particle.cu also calls come from this library (they are never called by
# ref_io).  Test infrastructure only: run from the repository root,
#   make -f oracle/ref_io.mk [REF=<reference>/src]
# Without the reference's sources it builds nothing.
REF ?= /root/reference/src
NVCC ?= nvcc
OUT := oracle/_ref
LIB := gpucell_gb300/lib

ifneq ($(wildcard $(REF)/Particle.cu),)
all: $(OUT)/ref_io
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
