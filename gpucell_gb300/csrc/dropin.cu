// dropin.cu -- the C++ symbols of GPUCell's GPU boundary (cupar::, cudiv::).
//
// GPUCell's host frame (src/Particle.cu) calls these by their C++ names; the
// signatures come from include/gpucell/cupar.h, which reproduces
// src/ParticleGPU.cuh:10-35 and src/ConfigDomain.cuh:11-17.  Each body
// forwards to the extern "C" function of the same name and, on failure,
// reports in the layout of the reference's CHECK macro (src/erro.cuh:6-20)
// and exits with status 1, which is what the reference does on any CUDA
// error.  Work goes to the legacy default stream unless gc_set_stream chose
// another, so the host's synchronous cudaMemcpy (src/Particle.cu:695-708)
// sees it.
#include <stdio.h>
#include <stdlib.h>

#include "gpucell/cupar.h"
#include "gpucell_gb300.h"

namespace {
void check(int rc, const char* fn) {
    if (rc == GC_OK) return;
    printf("CUDA Error:\n");
    printf("    File:       %s\n", __FILE__);
    printf("    Function:   %s\n", fn);
    printf("    Error code: %d\n", rc);
    printf("    Error text: %s\n", gc_last_error());
    fflush(stdout);
    exit(1);
}
}  // namespace

#define FWD(name, ...) check(gc_cupar_##name(__VA_ARGS__), "cupar::" #name)
#define FWD_DIV(name, ...) check(gc_cudiv_##name(__VA_ARGS__), "cudiv::" #name)

namespace cupar
{
void ConstsDataUp(const Structconst* consts) { FWD(ConstsDataUp, consts); }

void UpdateFluidCoor(int n, int* d_sortpart, float3* d_Totalforce, float3* d_totalcoor, float4* d_velrhop) {
    FWD(UpdateFluidCoor, n, d_sortpart, (float*)d_Totalforce, (float*)d_totalcoor, (float*)d_velrhop);
}

void AppFluidPeriodicBC(int n, int* d_sortpart, float3* d_totalcoor, int3* d_nthrobound, float* d_bboxsdpd) {
    FWD(AppFluidPeriodicBC, n, d_sortpart, (float*)d_totalcoor, (int*)d_nthrobound, d_bboxsdpd);
}

void CalFluidDen(int n, float3* d_totalcoor, float4* d_velrhop, int3* d_cc, int* d_ncube, float* d_outerregion,
                 int* d_sortpart, int2* d_beginendcube) {
    FWD(CalFluidDen, n, (float*)d_totalcoor, (float*)d_velrhop, (int*)d_cc, d_ncube, d_outerregion, d_sortpart,
        (int*)d_beginendcube);
}

void PredictFluidVel(int n, int* d_sortpart, float4* d_velrhop, float3* d_velhalf, float3* d_Totalforce) {
    FWD(PredictFluidVel, n, d_sortpart, (float*)d_velrhop, (float*)d_velhalf, (float*)d_Totalforce);
}

void CalBound2Vel(int n, float3* d_totalcoor, float4* d_velrhop, int3* d_cc, int* d_ncube, float* d_outerregion,
                  int* d_sortpart, int2* d_beginendcube) {
    FWD(CalBound2Vel, n, (float*)d_totalcoor, (float*)d_velrhop, (int*)d_cc, d_ncube, d_outerregion, d_sortpart,
        (int*)d_beginendcube);
}

void EOS(int n, int* d_sortpart, float4* d_velrhop, float* d_press) {
    FWD(EOS, n, d_sortpart, (float*)d_velrhop, d_press);
}

void CalFluidSDPDForce(int n, tfloat3* d_sdpdforce, float3* d_totalcoor, float4* d_velrhop, int3* d_cc, int* d_ncube,
                       int* d_sortpart, float* d_outerreigon, int2* d_beginendcube, float3* d_totalforce,
                       float* d_press) {
    FWD(CalFluidSDPDForce, n, (float*)d_sdpdforce, (float*)d_totalcoor, (float*)d_velrhop, (int*)d_cc, d_ncube,
        d_sortpart, d_outerreigon, (int*)d_beginendcube, (float*)d_totalforce, d_press);
}

void CalFluidRepForce(int n, float3* d_totalcoor, int3* d_cc, int* d_ncube, int* d_sortpart, float* d_outerreigon,
                      int2* d_beginendcube, float3* d_totalforce) {
    FWD(CalFluidRepForce, n, (float*)d_totalcoor, (int*)d_cc, d_ncube, d_sortpart, d_outerreigon,
        (int*)d_beginendcube, (float*)d_totalforce);
}

void SetFluidExtForce(int DriveOn, int n, int* d_sortpart, float3* d_totalforce) {
    FWD(SetFluidExtForce, DriveOn, n, d_sortpart, (float*)d_totalforce);
}

void CorrectFliudVel(int n, int* d_sortpart, float3* d_totalforce, float3* d_velhalf, float4* d_velrhop,
                     float3* d_totalcoor, int3* d_cc, int* d_ncube, float* d_outerreigon, int2* d_beginendcube) {
    FWD(CorrectFliudVel, n, d_sortpart, (float*)d_totalforce, (float*)d_velhalf, (float*)d_velrhop,
        (float*)d_totalcoor, (int*)d_cc, d_ncube, d_outerreigon, (int*)d_beginendcube);
}

void CalGeoPara(long stepcount, int ntri, int ncell, float* d_bbox, int* d_curpos, int3* d_tri, int2* d_beginendtri,
                int3* d_nthrobound, float3* d_totalcoor, float3* d_trinordir, float* d_triarea, float* d_reftriarea,
                float3* d_tricenter, float* d_refarea_para, float* d_refvol_para, float* d_area_para,
                float* d_vol_para, float* d_area, float* d_vol, float* d_pararea) {
    FWD(CalGeoPara, stepcount, ntri, ncell, d_bbox, d_curpos, (int*)d_tri, (int*)d_beginendtri, (int*)d_nthrobound,
        (float*)d_totalcoor, (float*)d_trinordir, d_triarea, d_reftriarea, (float*)d_tricenter, d_refarea_para,
        d_refvol_para, d_area_para, d_vol_para, d_area, d_vol, d_pararea);
}

void SetMechPara(int ncell, int nedge, int6* d_edge, int* d_curpos, float* d_refedgelen, float* d_maxrefedgelen,
                 float* d_bendmodpara, float* d_shearmodpara, float* d_hbending, float* d_powerindex,
                 float* d_perlenWLC, float* d_hpow, float* d_reftriangle, float3* d_trinordir, float3* d_tricente,
                 float3* d_coor) {
    FWD(SetMechPara, ncell, nedge, (int*)d_edge, d_curpos, d_refedgelen, d_maxrefedgelen, d_bendmodpara,
        d_shearmodpara, d_hbending, d_powerindex, d_perlenWLC, d_hpow, d_reftriangle, (float*)d_trinordir,
        (float*)d_tricente, (float*)d_coor);
}

void CalCellDefForce(int ncell, unsigned nedge, unsigned ntri, unsigned ntotalpar, unsigned ncellpar, float* d_bbox,
                     int6* d_edge, int3* d_tri, float3* d_coor, tfloat3* defforce, float3* d_defforce,
                     int3* d_nthrobound, float* d_maxrefedgelen, float* d_powerindex, float* d_perlenWLC,
                     float* d_hpow, float3* d_trinordir, float3* d_tricenter, float* d_reftriangle, float* d_hbending,
                     float* d_triarea, float* d_reftriarea, float* d_hlarea_para, float* d_hgarea_para,
                     float* d_area_para, float* d_refarea_para, float* d_hvol_para, float* d_vol_para,
                     float* d_refvol_para, float3* d_totalforce, int* d_sortpart, int* d_curpos) {
    FWD(CalCellDefForce, ncell, nedge, ntri, ntotalpar, ncellpar, d_bbox, (int*)d_edge, (int*)d_tri, (float*)d_coor,
        (float*)defforce, (float*)d_defforce, (int*)d_nthrobound, d_maxrefedgelen, d_powerindex, d_perlenWLC, d_hpow,
        (float*)d_trinordir, (float*)d_tricenter, d_reftriangle, d_hbending, d_triarea, d_reftriarea, d_hlarea_para,
        d_hgarea_para, d_area_para, d_refarea_para, d_hvol_para, d_vol_para, d_refvol_para, (float*)d_totalforce,
        d_sortpart, d_curpos);
}

void CalCellAggForce(unsigned ncell, unsigned n, unsigned ncellpar, float3* d_totalcoor, float3* d_aggforce,
                     int3* d_cc, int* d_ncube, int* d_sortpart, int* d_celltab, float* d_outerreigon,
                     int2* d_beginendcube, float3* d_totalforce, float* d_pararea) {
    FWD(CalCellAggForce, ncell, n, ncellpar, (float*)d_totalcoor, (float*)d_aggforce, (int*)d_cc, d_ncube, d_sortpart,
        d_celltab, d_outerreigon, (int*)d_beginendcube, (float*)d_totalforce, d_pararea);
}
}  // namespace cupar

namespace cudiv
{
void PreConList(int n, int cutradius, float3* d_totalcoor, float* d_bboxsph, float* d_invwid, int* d_ncube,
                int3* d_cc, int* d_cubepart, int* d_sortpart, int* d_oldpos) {
    FWD_DIV(PreConList, n, cutradius, (float*)d_totalcoor, d_bboxsph, d_invwid, d_ncube, (int*)d_cc, d_cubepart,
            d_sortpart, d_oldpos);
}

void Sort(int n, int* keys, int* values) { FWD_DIV(Sort, n, keys, values); }

void CalBeginEndCube(int n, int SizeCube, int* d_cubepart, int2* d_beginendcube) {
    FWD_DIV(CalBeginEndCube, n, SizeCube, d_cubepart, (int*)d_beginendcube);
}

void SortBasicArrays(int n, int* d_sortpart, int* d_oldpos, float3* d_totalcoor, int3* d_cc, float4* d_velrhop,
                     float3* d_velhalf, float3* d_totalforce, float* d_press) {
    FWD_DIV(SortBasicArrays, n, d_sortpart, d_oldpos, (float*)d_totalcoor, (int*)d_cc, (float*)d_velrhop,
            (float*)d_velhalf, (float*)d_totalforce, d_press);
}

void SortArraysWithCells(int n, int* d_sortpart, int* d_oldpos, int* d_curpos, float3* d_totalcoor, int3* d_cc,
                         float4* d_velrhop, float3* d_velhalf, float3* d_totalforce, float* d_press,
                         int3* d_nthrobound) {
    FWD_DIV(SortArraysWithCells, n, d_sortpart, d_oldpos, d_curpos, (float*)d_totalcoor, (int*)d_cc,
            (float*)d_velrhop, (float*)d_velhalf, (float*)d_totalforce, d_press, (int*)d_nthrobound);
}

void Printf(int n, int* d_curtpart, int* d_sortpart, float3* d_TotalCoor) {
    FWD_DIV(Printf, n, d_curtpart, d_sortpart, (float*)d_TotalCoor);
}
}  // namespace cudiv
