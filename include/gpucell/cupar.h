/*
 * cupar.h -- GPUCell's GPU boundary, as C++ declarations.
 *
 * GPUCell's host frame (src/Particle.cu) calls exactly these 20 functions;
 * their bodies (ParticleGPU.cu, ConfigDomain.cu) are not part of the
 * reference, so libgpucell_gb300.so supplies them.  Linking the unchanged
 * src/main.cu + src/Particle.cu against the library gives a working
 * program: the declarations below reproduce src/ParticleGPU.cuh:10-35 and
 * src/ConfigDomain.cuh:11-17 argument for argument, because the mangled
 * names (and so the link) depend on every parameter type.
 *
 * Contract of every function (kept from the reference call sites):
 *   - all pointers named d_* are device pointers owned by the caller;
 *   - work is enqueued on the legacy default stream (stream 0), so the
 *     caller's next synchronous cudaMemcpy sees it (src/Particle.cu:695);
 *   - on failure the function prints a CUDA-error report in the style of
 *     src/erro.cuh:6-20 and calls exit(1).
 * Each body forwards to the extern "C" gc_cupar_* / gc_cudiv_* function of
 * the same name (include/gpucell_gb300.h), which returns a status instead.
 */
#ifndef GPUCELL_CUPAR_H
#define GPUCELL_CUPAR_H

#include <vector_types.h>
#include "TypesDef.h"

#define SDPDSIZE 128   /* block size named by src/ParticleGPU.cuh:6 */
#define DIVSIZE 128    /* block size named by src/ConfigDomain.cuh:7 */

namespace cupar
{
/* src/ParticleGPU.cuh:10 -- K1: upload the physical constants */
void ConstsDataUp(const Structconst *consts);
/* src/ParticleGPU.cuh:11 -- K2: position update of fluid + membrane */
void UpdateFluidCoor(int n, int* d_sortpart, float3* d_Totalforce, float3* d_totalcoor, float4* d_velrhop);
/* src/ParticleGPU.cuh:12 -- K3: periodic wrap, crossing counts */
void AppFluidPeriodicBC(int n, int* d_sortpart, float3* d_totalcoor, int3* d_nthrobound, float* d_bboxsdpd);
/* src/ParticleGPU.cuh:13 -- K8: kernel-sum density */
void CalFluidDen(int n, float3* d_totalcoor, float4* d_velrhop, int3* d_cc, int* d_ncube, float* d_outerregion, int* d_sortpart, int2* d_beginendcube);
/* src/ParticleGPU.cuh:14 -- K9: velocity-Verlet predictor */
void PredictFluidVel(int n, int* d_sortpart, float4* d_velrhop, float3* d_velhalf, float3* d_Totalforce);
/* src/ParticleGPU.cuh:15 -- K10: no-slip velocity of Bound2 walls */
void CalBound2Vel(int n, float3* d_totalcoor, float4* d_velrhop, int3* d_cc, int* d_ncube, float* d_outerregion, int* d_sortpart, int2* d_beginendcube);
/* src/ParticleGPU.cuh:16 -- K11: equation of state */
void EOS(int n, int* d_sortpart, float4* d_velrhop, float* d_press);
/* src/ParticleGPU.cuh:17 -- K12: SDPD pair force (first writer of the force) */
void CalFluidSDPDForce(int n, tfloat3* d_sdpdforce, float3* d_totalcoor, float4* d_velrhop, int3* d_cc, int* d_ncube, int* d_sortpart, float* d_outerreigon, int2* d_beginendcube, float3* d_totalforce, float* d_press);
/* src/ParticleGPU.cuh:18 -- K13: Bound1 wall repulsion */
void CalFluidRepForce(int n, float3* d_totalcoor, int3* d_cc, int* d_ncube, int* d_sortpart, float* d_outerreigon, int2* d_beginendcube, float3* d_totalforce);
/* src/ParticleGPU.cuh:19 -- K14: body force */
void SetFluidExtForce(int DriveOn, int n, int* d_sortpart, float3* d_totalforce);
/* src/ParticleGPU.cuh:21 -- K19: velocity-Verlet corrector */
void CorrectFliudVel(int n, int* d_sortpart, float3* d_totalforce, float3* d_velhalf, float4* d_velrhop, float3* d_totalcoor, int3*d_cc, int* d_ncube, float* d_outerreigon, int2* d_beginendcube);
/* src/ParticleGPU.cuh:25-26 -- K15: membrane geometry, per-cell area/volume */
void CalGeoPara(long stepcount, int ntri, int ncell, float* d_bbox, int* d_curpos, int3* d_tri, int2* d_beginendtri, int3* d_nthrobound, float3* d_totalcoor, float3* d_trinordir, float* d_triarea,
    float* d_reftriarea, float3* d_tricenter, float* d_refarea_para, float* d_refvol_para, float* d_area_para, float* d_vol_para, float* d_area, float* d_vol, float* d_pararea);
/* src/ParticleGPU.cuh:28-29 -- K16: per-edge membrane parameters (set-up) */
void SetMechPara(int ncell, int nedge, int6* d_edge, int* d_curpos, float* d_refedgelen, float* d_maxrefedgelen, float* d_bendmodpara, float* d_shearmodpara, float* d_hbending,
    float* d_powerindex, float* d_perlenWLC, float* d_hpow, float* d_reftriangle, float3* d_trinordir, float3* d_tricente, float3* d_coor);
/* src/ParticleGPU.cuh:30-33 -- K17: membrane deformation force */
void CalCellDefForce(int ncell, unsigned nedge, unsigned ntri, unsigned ntotalpar, unsigned ncellpar, float* d_bbox, int6* d_edge, int3* d_tri, float3* d_coor, tfloat3* defforce, float3* d_defforce, int3* d_nthrobound,
    float* d_maxrefedgelen, float* d_powerindex, float* d_perlenWLC, float* d_hpow, float3* d_trinordir, float3* d_tricenter,
    float* d_reftriangle, float* d_hbending, float* d_triarea, float* d_reftriarea, float* d_hlarea_para, float* d_hgarea_para, float* d_area_para,
    float* d_refarea_para, float* d_hvol_para, float* d_vol_para, float* d_refvol_para, float3* d_totalforce, int* d_sortpart, int* d_curpos);
/* src/ParticleGPU.cuh:34-35 -- K18: Morse aggregation between cells */
void CalCellAggForce(unsigned ncell, unsigned n, unsigned ncellpar, float3* d_totalcoor, float3* d_aggforce, int3* d_cc, int* d_ncube, int* d_sortpart,
    int* d_celltab, float* d_outerreigon, int2* d_beginendcube, float3* d_totalforce, float* d_pararea);
}

namespace cudiv
{
/* src/ConfigDomain.cuh:11 -- K4: cube of every particle, sort keys */
void PreConList(int n, int cutradius, float3* d_totalcoor, float* d_bboxsph, float* d_invwid, int* d_ncube, int3* d_cc, int* d_cubepart, int* d_sortpart, int* d_oldpos);
/* src/ConfigDomain.cuh:12 -- K5: stable key/value sort */
void Sort(int n, int *keys, int *values);
/* src/ConfigDomain.cuh:13 -- K6: [begin, end) slot range of every cube */
void CalBeginEndCube(int n, int SizeCube, int* d_cubepart, int2* d_beginendcube);
/* src/ConfigDomain.cuh:14 -- K7: permute the particle arrays (no cells) */
void SortBasicArrays(int n, int* d_sortpart, int* d_oldpos, float3* d_totalcoor, int3* d_cc, float4* d_velrhop, float3* d_velhalf, float3* d_totalforce, float* d_press);
/* src/ConfigDomain.cuh:15 -- K7: permute the particle arrays (with cells) */
void SortArraysWithCells(int n, int* d_sortpart, int* d_oldpos, int* d_curpos, float3* d_totalcoor, int3* d_cc, float4* d_velrhop, float3* d_velhalf, float3* d_totalforce, float* d_press, int3* d_nthrobound);
/* src/ConfigDomain.cuh:17 -- debug print, never called by the reference */
void Printf(int n, int * d_curtpart, int *d_sortpart, float3* d_TotalCoor);
}

#endif /* GPUCELL_CUPAR_H */
