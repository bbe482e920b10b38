// ref_calls_stubs.cu -- the 20 boundary entry points as recorders: each
// writes its name and its count arguments to gc_ref_trace and touches no
// memory.  Linked in place of the library under GPUCell's own Particle.cu
// (oracle/ref_calls.cu runs its step driver), so that the trace is the call
// sequence of the reference's UpdatePar (src/Particle.cu:1310-1329) with the
// counts it passes.  Test infrastructure, built by oracle/ref_io.mk only
// where the reference's sources are present.
#include <stdio.h>

#include "gpucell/cupar.h"

extern "C" {
FILE* gc_ref_trace = nullptr;
}

namespace {
void rec(const char* name, long long a = -1, long long b = -1, long long c = -1, long long d = -1,
         long long e = -1) {
    if (!gc_ref_trace) return;
    fprintf(gc_ref_trace, "%s", name);
    for (long long v : {a, b, c, d, e})
        if (v != -1) fprintf(gc_ref_trace, " %lld", v);
    fprintf(gc_ref_trace, "\n");
}
}  // namespace

namespace cupar {
void ConstsDataUp(const Structconst*) { rec("ConstsDataUp"); }
void UpdateFluidCoor(int n, int*, float3*, float3*, float4*) { rec("UpdateFluidCoor", n); }
void AppFluidPeriodicBC(int n, int*, float3*, int3*, float*) { rec("AppFluidPeriodicBC", n); }
void CalFluidDen(int n, float3*, float4*, int3*, int*, float*, int*, int2*) { rec("CalFluidDen", n); }
void PredictFluidVel(int n, int*, float4*, float3*, float3*) { rec("PredictFluidVel", n); }
void CalBound2Vel(int n, float3*, float4*, int3*, int*, float*, int*, int2*) { rec("CalBound2Vel", n); }
void EOS(int n, int*, float4*, float*) { rec("EOS", n); }
void CalFluidSDPDForce(int n, tfloat3*, float3*, float4*, int3*, int*, int*, float*, int2*, float3*, float*) {
    rec("CalFluidSDPDForce", n);
}
void CalFluidRepForce(int n, float3*, int3*, int*, int*, float*, int2*, float3*) { rec("CalFluidRepForce", n); }
void SetFluidExtForce(int DriveOn, int n, int*, float3*) { rec("SetFluidExtForce", DriveOn, n); }
void CorrectFliudVel(int n, int*, float3*, float3*, float4*, float3*, int3*, int*, float*, int2*) {
    rec("CorrectFliudVel", n);
}
void CalGeoPara(long stepcount, int ntri, int ncell, float*, int*, int3*, int2*, int3*, float3*, float3*, float*,
                float*, float3*, float*, float*, float*, float*, float*, float*, float*) {
    rec("CalGeoPara", stepcount, ntri, ncell);
}
void SetMechPara(int ncell, int nedge, int6*, int*, float*, float*, float*, float*, float*, float*, float*, float*,
                 float*, float3*, float3*, float3*) {
    rec("SetMechPara", ncell, nedge);
}
void CalCellDefForce(int ncell, unsigned nedge, unsigned ntri, unsigned ntotalpar, unsigned ncellpar, float*, int6*,
                     int3*, float3*, tfloat3*, float3*, int3*, float*, float*, float*, float*, float3*, float3*, float*,
                     float*, float*, float*, float*, float*, float*, float*, float*, float*, float*, float3*, int*,
                     int*) {
    rec("CalCellDefForce", ncell, nedge, ntri, ntotalpar, ncellpar);
}
void CalCellAggForce(unsigned ncell, unsigned n, unsigned ncellpar, float3*, float3*, int3*, int*, int*, int*, float*,
                     int2*, float3*, float*) {
    rec("CalCellAggForce", ncell, n, ncellpar);
}
}  // namespace cupar

namespace cudiv {
void PreConList(int n, int cutradius, float3*, float*, float*, int*, int3*, int*, int*, int*) {
    rec("PreConList", n, cutradius);
}
void Sort(int n, int*, int*) { rec("Sort", n); }
// SizeCube is not recorded: ConfigDomain, which sets it, allocates device
// memory and does not run under the recorder
void CalBeginEndCube(int n, int, int*, int2*) { rec("CalBeginEndCube", n); }
void SortBasicArrays(int n, int*, int*, float3*, int3*, float4*, float3*, float3*, float*) {
    rec("SortBasicArrays", n);
}
void SortArraysWithCells(int n, int*, int*, int*, float3*, int3*, float4*, float3*, float3*, float*, int3*) {
    rec("SortArraysWithCells", n);
}
void Printf(int n, int*, int*, float3*) { rec("Printf", n); }
}  // namespace cudiv
