// fused_engine.cu -- the fused step behind the boundary entry points (GPUCELL_ENGINE=fused).
#include "fused_internal.cuh"

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

using namespace gcf;

// ---------------------------------------------------------------------------
// The fused engine behind the boundary entry points (GPUCELL_ENGINE=fused).
//
// GPUCell's host frame owns the state in its own buffers and layout and
// reads them between steps (src/Particle.cu:693-710).  The engine adopts the
// state once -- positions, velocities, VelHalf, forces and crossing counts in
// the caller's slot order, the membrane topology and the reference geometry
// its set-up calls computed -- then runs each step fused on its own arrays
// and writes back, at the end of every step, everything the host reads: the
// particle arrays in the engine's slot order with SortPart and CurPos to
// match, and the per-cell, per-triangle and per-vertex membrane outputs.
// ---------------------------------------------------------------------------
namespace {

__global__ void fk_import_ref(int n, unsigned nC, const int* __restrict__ sortpart, const float* __restrict__ coor,
                              const float* __restrict__ velrhop, const float* __restrict__ velhalf,
                              const float* __restrict__ force, const int* __restrict__ nthro, SlotArrays a,
                              int* __restrict__ slot_of, float4* __restrict__ mpos, float4* __restrict__ mplo,
                              int4* __restrict__ mnthro,
                              unsigned* flags) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    int id = sortpart[q];
    if (id < 0 || id >= n) {
        raise_flag(flags, GC_FLAG_BAD_INDEX);
        return;
    }
    float4 x = make_float4(coor[3 * q], coor[3 * q + 1], coor[3 * q + 2], __uint_as_float((unsigned)id));
    a.pos[q] = x;
    a.plo[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 v = make_float4(velrhop[4 * q], velrhop[4 * q + 1], velrhop[4 * q + 2], 0.f);
    a.vel[q] = v;
    a.vpred[q] = v;
    a.vh[q] = make_float4(velhalf[3 * q], velhalf[3 * q + 1], velhalf[3 * q + 2], 0.f);
    a.force[q] = make_float4(force[3 * q], force[3 * q + 1], force[3 * q + 2], 0.f);
    int4 t = nthro ? make_int4(nthro[3 * q], nthro[3 * q + 1], nthro[3 * q + 2], 0) : make_int4(0, 0, 0, 0);
    a.nthro[q] = t;
    slot_of[id] = q;
    if ((unsigned)id >= nC && mpos) {
        mpos[id - nC] = x;
        mplo[id - nC] = make_float4(0.f, 0.f, 0.f, 0.f);
        mnthro[id - nC] = t;
    }
}

__global__ void fk_export_ref(int n, GcParams p, SlotArrays a, const float2* __restrict__ dp, int* __restrict__ sortpart,
                              int* __restrict__ curpos, float* __restrict__ coor, float* __restrict__ velrhop,
                              float* __restrict__ velhalf, float* __restrict__ force, float* __restrict__ press,
                              int* __restrict__ nthro) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    float4 x = a.pos[q];
    unsigned id = fid(x);
    sortpart[q] = (int)id;
    if (curpos) curpos[id] = q;
    coor[3 * q] = x.x; coor[3 * q + 1] = x.y; coor[3 * q + 2] = x.z;
    float4 v = a.vel[q];
    float2 d = dp[q];
    velrhop[4 * q] = v.x; velrhop[4 * q + 1] = v.y; velrhop[4 * q + 2] = v.z; velrhop[4 * q + 3] = p.mass / d.x;
    float4 h = a.vh[q];
    velhalf[3 * q] = h.x; velhalf[3 * q + 1] = h.y; velhalf[3 * q + 2] = h.z;
    float4 f = a.force[q];
    force[3 * q] = f.x; force[3 * q + 1] = f.y; force[3 * q + 2] = f.z;
    if (press) press[q] = d.y / (d.x * d.x);
    if (nthro) {
        int4 t = a.nthro[q];
        nthro[3 * q] = t.x; nthro[3 * q + 1] = t.y; nthro[3 * q + 2] = t.z;
    }
}

// one block per cell: cell values and their per-triangle copies
__global__ void fk_export_cells_ref(int ncell, int ntri, const int2* __restrict__ betri, const double* __restrict__ carea,
                                    const double* __restrict__ cvol, const float* __restrict__ tarea,
                                    const float4* __restrict__ tnorm, const float4* __restrict__ tcen,
                                    float* __restrict__ area, float* __restrict__ vol, float* __restrict__ area_para,
                                    float* __restrict__ vol_para, float* __restrict__ triarea,
                                    float* __restrict__ trinordir, float* __restrict__ tricenter) {
    int c = blockIdx.x;
    int2 be = betri[c];
    if (be.x < 0 || be.y >= ntri || be.y < be.x) return;
    float A = (float)carea[c], V = (float)cvol[c];
    if (threadIdx.x == 0) {
        if (area) area[c] = A;
        if (vol) vol[c] = V;
    }
    for (int t = be.x + threadIdx.x; t <= be.y; t += blockDim.x) {
        if (area_para) area_para[t] = A;
        if (vol_para) vol_para[t] = V;
        if (triarea) triarea[t] = tarea[t];
        float4 nrm = tnorm[t], cen = tcen[t];
        if (trinordir) { trinordir[3 * t] = nrm.x; trinordir[3 * t + 1] = nrm.y; trinordir[3 * t + 2] = nrm.z; }
        if (tricenter) { tricenter[3 * t] = cen.x; tricenter[3 * t + 1] = cen.y; tricenter[3 * t + 2] = cen.z; }
    }
}

__global__ void fk_import_cellrefs(int ncell, int ntri, const int2* __restrict__ betri,
                                   const float* __restrict__ refarea_para, const float* __restrict__ refvol_para,
                                   double* __restrict__ crefarea, double* __restrict__ crefvol) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    int t = betri[c].x;
    if (t < 0 || t >= ntri) return;
    crefarea[c] = (double)refarea_para[t];
    crefvol[c] = (double)refvol_para[t];
}

// Adopts the membrane topology, moduli and set-up geometry from the caller's
// device buffers.
int engine_cells(GcFused* f, const GcRefPtrs& r) {
    int ncell = r.ncell, ntri = r.ntri, nedge = r.nedge, ncp = (int)f->p.nCP;
    if (ncell <= 0) return GC_OK;
    if (!r.tri || !r.betri || !r.edge || !r.celltab || !r.hlarea || !r.hgarea || !r.hvol || !r.refedgelen ||
        !r.maxrefedgelen || !r.perlen || !r.hpow || !r.hbending || !r.reftriangle || !r.reftriarea ||
        !r.refarea_para || !r.refvol_para)
        return gc_fail(GC_ESTATE, "fused engine: a membrane buffer of the set-up calls was not seen");
    GC_TRY(alloc_cells(f, ncell, ntri, nedge, ncp));
    f->cells_adopted = true;
    cudaStream_t st = f->st;
    auto d2d = [&](void* dst, const void* src, size_t bytes) -> int {
        if (!src) return GC_OK;
        GC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st), "fused engine: adopt cells");
        return GC_OK;
    };
    GC_TRY(d2d(f->tri, r.tri, (size_t)ntri * 12));
    GC_TRY(d2d(f->edge, r.edge, (size_t)nedge * 24));
    GC_TRY(d2d(f->betri, r.betri, (size_t)ncell * 8));
    GC_TRY(d2d(f->celltab, r.celltab, (size_t)ncp * 4));
    GC_TRY(d2d(f->shear, r.shearmod, (size_t)nedge * 4));
    GC_TRY(d2d(f->bend, r.bendmod, (size_t)nedge * 4));
    GC_TRY(d2d(f->hl, r.hlarea, (size_t)ntri * 4));
    GC_TRY(d2d(f->hg, r.hgarea, (size_t)ntri * 4));
    GC_TRY(d2d(f->hv, r.hvol, (size_t)ntri * 4));
    GC_TRY(d2d(f->l0, r.refedgelen, (size_t)nedge * 4));
    GC_TRY(d2d(f->lmax, r.maxrefedgelen, (size_t)nedge * 4));
    GC_TRY(d2d(f->perlen, r.perlen, (size_t)nedge * 4));
    GC_TRY(d2d(f->hpow, r.hpow, (size_t)nedge * 4));
    GC_TRY(d2d(f->hbend, r.hbending, (size_t)nedge * 4));
    GC_TRY(d2d(f->refang, r.reftriangle, (size_t)nedge * 4));
    GC_TRY(d2d(f->reftarea, r.reftriarea, (size_t)ntri * 4));
    fk_import_cellrefs<<<gc_blocks(ncell, 128), 128, 0, st>>>(ncell, ntri, f->betri, r.refarea_para, r.refvol_para,
                                                            f->crefarea, f->crefvol);
    GC_CHECK_LAUNCH("fused engine: reference areas and volumes");
    std::vector<int> htri(3 * (size_t)ntri), hedge(6 * (size_t)nedge);
    GC_CUDA(cudaMemcpyAsync(htri.data(), f->tri, htri.size() * 4, cudaMemcpyDeviceToHost, st), "fused engine: topology");
    GC_CUDA(cudaMemcpyAsync(hedge.data(), f->edge, hedge.size() * 4, cudaMemcpyDeviceToHost, st), "fused engine: topology");
    GC_CUDA(cudaStreamSynchronize(st), "fused engine: topology");
    GC_TRY(build_incidence(f, htri.data(), hedge.data()));
    return build_grids(f);   // aggregation grid
}

int engine_start(GcState& s) {
    const GcRefPtrs& r = s.ref;
    if (!r.sortpart || !r.coor || !r.velrhop || !r.velhalf || !r.force || !r.bbox)
        return gc_fail(GC_ESTATE, "fused engine: the first step did not show every particle buffer");
    float bb[6];
    GC_CUDA(cudaMemcpyAsync(bb, r.bbox, sizeof(bb), cudaMemcpyDeviceToHost, s.stream), "fused engine: bbox");
    GC_CUDA(cudaStreamSynchronize(s.stream), "fused engine: bbox");
    GcFused* f = nullptr;
    GcFusedOptions opt;
    memset(&opt, 0, sizeof(opt));
    opt.compact = 1;
    GC_TRY(gc_fused_create(&s.c, bb, s.periodic_mask, s.noise_on, &opt, &f));
    int rc = engine_cells(f, r);
    if (rc == GC_OK) {
        fk_import_ref<<<gc_blocks(f->n, f->block), f->block, 0, f->st>>>(
            f->n, f->p.nC, r.sortpart, r.coor, r.velrhop, r.velhalf, r.force, r.nthro, f->a, f->slot_of,
            f->ncell > 0 ? f->mpos : nullptr, f->mplo, f->mnthro, f->flags);
        cudaError_t e = cudaGetLastError();
        gc_count_launch();
        if (e != cudaSuccess) rc = gc_cuda_fail(e, "fused engine: adopt state");
    }
    if (rc == GC_OK) rc = rebuild_lists(f);
    if (rc != GC_OK) {
        gc_fused_destroy(f);
        return rc;
    }
    for (int k = 0; k < f->nsys; ++k) f->sys_loaded[k] = 1;
    f->setup_done = true;
    s.engine = f;
    return GC_OK;
}

int engine_export(GcFused* f, const GcRefPtrs& r) {
    cudaStream_t st = f->st;
    fk_export_ref<<<gc_blocks(f->n, f->block), f->block, 0, st>>>(f->n, f->p, f->a, f->dp, r.sortpart, r.curpos,
                                                                 r.coor, r.velrhop, r.velhalf, r.force, r.press,
                                                                 r.nthro);
    GC_CHECK_LAUNCH("fused engine: write back particles");
    if (f->ncell > 0) {
        fk_export_cells_ref<<<f->ncell, 256, 0, st>>>(f->ncell, f->ntri, f->betri, f->carea, f->cvol, f->tarea,
                                                     f->tnorm, f->tcen, r.area, r.vol, r.area_para, r.vol_para,
                                                     r.triarea, r.trinordir, r.tricenter);
        GC_CHECK_LAUNCH("fused engine: write back cells");
        int m = f->ncp;
        fk_store_cells<<<gc_blocks(m, 128), 128, 0, st>>>(m, 0, 0, 0, f->mforce, f->magg, f->parea, f->tnorm, f->tcen,
                                                         r.defforce, r.aggforce, r.pararea, nullptr, nullptr,
                                                         f->have_agg ? 1 : 0);
        GC_CHECK_LAUNCH("fused engine: write back membrane forces");
    }
    return GC_OK;
}

}  // namespace

int gc_engine_step(int drive_on) {
    GcState& s = gc_state();
    if (!s.engine) GC_TRY(engine_start(s));
    GcFused* f = s.engine;
    f->step = s.step - 1;   // one_step advances it to the step index of this UpdatePar
    GC_TRY(one_step(f, drive_on));
    return engine_export(f, s.ref);
}

void gc_engine_reset() {
    GcState& s = gc_state();
    if (s.engine) gc_fused_destroy(s.engine);
    s.engine = nullptr;
}
