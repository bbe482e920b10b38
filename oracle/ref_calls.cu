// ref_calls.cu -- GPUCell's own step driver (Particle::DrivePar and
// Particle::UpdatePar, src/Particle.cu:1302-1329) run on the host against
// recording entry points (oracle/ref_calls_stubs.cu): the trace is the
// sequence of boundary calls one step of the reference makes, with the counts
// it passes, which the engine behind the entry points and the host-frame
// mirror (gpucell_gb300/host.py) rely on.  Test infrastructure, built by
// oracle/ref_io.mk into oracle/_ref/ref_calls only where the reference's
// sources are present.
//
//   ref_calls <dir> <steps> <trace>   loads the input files in <dir> with the
//                                     reference's loaders, then runs <steps>
//                                     steps of its driver; one line per call
//
// Of the set-up (Particle::SetPar, src/Particle.cu:471-483) the parts that
// touch no device memory run, under a line "setup": SetParticle, then
// ConstantDataUp and ConCubeList as ConfigDomain ends (src/Particle.cu:
// 569-570); AllocGpuMemory and ParticlesDataUp do not, nor the CalGeoPara and
// SetMechPara calls that SetPar makes itself.  The steps start at StepCount
// 0, where SetPar leaves it (src/Particle.cu:482); a line "step" marks each.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <cuda_runtime.h>

// in the order the reference's own sources include them
#include "main.cuh"
#include "TypesDef.cuh"
#include "Particle.cuh"

extern "C" FILE* gc_ref_trace;

int main(int argc, char** argv) {
    if (argc != 4) {
        fprintf(stderr, "usage: ref_calls <dir> <steps> <trace>\n");
        return 1;
    }
    char trace[4096];
    if (argv[3][0] == '/') {
        snprintf(trace, sizeof(trace), "%s", argv[3]);
    } else {
        char cwd[2048];
        if (!getcwd(cwd, sizeof(cwd))) return 2;
        snprintf(trace, sizeof(trace), "%s/%s", cwd, argv[3]);
    }
    if (chdir(argv[1]) != 0) {   // the reference opens its files relative to the working directory
        fprintf(stderr, "ref_calls: cannot enter %s\n", argv[1]);
        return 2;
    }
    const int steps = atoi(argv[2]);
    Particle p;
    p.LoadParInfo();
    gc_ref_trace = fopen(trace, "w");
    if (!gc_ref_trace) return 2;
    fprintf(gc_ref_trace, "setup\n");
    p.SetParticle();
    p.ConstantDataUp();
    p.ConCubeList();
    StepCount = 0;
    for (int k = 0; k < steps; ++k) {   // the loop body of src/main.cu:39-47 without the output
        fprintf(gc_ref_trace, "step\n");
        p.DrivePar();
        p.UpdatePar();
        StepCount++;
    }
    return fclose(gc_ref_trace) == 0 ? 0 : 2;
}
