// fused_report.cu -- per-cell statistics, diagnostics and output files of a fused handle.
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

namespace {

// Per-cell statistics for GPUCell's per-cell time series: mean deformation
// and aggregation force and mean velocity over the cell's vertices, the
// magnitude of the mean velocity, area and volume; FP64 sums, one block per
// cell.
__global__ void fk_cell_stats(int c0, const int2* __restrict__ cell_verts, const SysInfo* __restrict__ sys,
                              const int* __restrict__ cellsys, const int* __restrict__ slot_of,
                              const float4* __restrict__ vel, const float4* __restrict__ mforce,
                              const float4* __restrict__ magg, int have_agg, const double* __restrict__ carea,
                              const double* __restrict__ cvol, double* __restrict__ out) {
    __shared__ double sh[32];
    const int c = c0 + blockIdx.x;
    const int2 vr = cell_verts[c];
    const SysInfo& S = sys[cellsys ? cellsys[c] : 0];
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int v = vr.x + threadIdx.x; v <= vr.y; v += blockDim.x) {
        float4 m = mforce[v];
        float4 a = have_agg ? magg[v] : make_float4(0.f, 0.f, 0.f, 0.f);
        float4 u = vel[slot_of[S.cs + (unsigned)(v - (int)S.m0)]];
        acc[0] += (double)(m.x - a.x); acc[1] += (double)(m.y - a.y); acc[2] += (double)(m.z - a.z);
        acc[3] += a.x; acc[4] += a.y; acc[5] += a.z;
        acc[6] += u.x; acc[7] += u.y; acc[8] += u.z;
    }
    const double inv = 1.0 / (double)(vr.y - vr.x + 1);
    double r[9];
    for (int k = 0; k < 9; ++k) r[k] = block_sum_d(acc[k], sh) * inv;
    if (threadIdx.x == 0) {
        double* o = out + 12 * (size_t)blockIdx.x;
        for (int k = 0; k < 9; ++k) o[k] = r[k];
        o[9] = sqrt(r[6] * r[6] + r[7] * r[7] + r[8] * r[8]);
        o[10] = carea[c];
        o[11] = cvol[c];
    }
}

// Diagnostics of the ids [id0, id0 + count): per block, FP64 partial sums of
// the momentum and kinetic energy of the moving particles (fluid and
// membrane), their count, the largest speed, and the density sum and count
// of the fluid particles; fk_diag_final adds the blocks in order.
constexpr int kDiagBS = 256;

// Largest value over the block (non-negative inputs), on every thread.
__device__ __forceinline__ double block_max_d(double v, double* sh) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o; o >>= 1) t = fmax(t, __shfl_xor_sync(0xffffffffu, t, o));
        if (threadIdx.x == 0) sh[0] = t;
    }
    __syncthreads();
    double t = sh[0];
    __syncthreads();
    return t;
}
constexpr int kDiagVals = 9;   // px py pz  2 E_kin  n_mobile  max|v|  sum rho  n_fluid  (unused)

__global__ void __launch_bounds__(kDiagBS) fk_diag_partial(int count, unsigned id0, unsigned fl, unsigned cs,
                                                          float mass, const int* __restrict__ slot_of,
                                                          const float4* __restrict__ vel,
                                                          const float2* __restrict__ dp,
                                                          double* __restrict__ partial) {
    __shared__ double sh[32];
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    double v[kDiagVals] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (k < count) {
        unsigned id = id0 + k;
        int i = slot_of[id];
        if (id >= fl) {
            float4 u = vel[i];
            v[0] = (double)mass * u.x;
            v[1] = (double)mass * u.y;
            v[2] = (double)mass * u.z;
            v[3] = (double)mass * ((double)u.x * u.x + (double)u.y * u.y + (double)u.z * u.z);
            v[4] = 1.0;
            v[5] = sqrt((double)u.x * u.x + (double)u.y * u.y + (double)u.z * u.z);
        }
        if (id >= fl && id < cs) {
            v[6] = (double)mass / (double)dp[i].x;
            v[7] = 1.0;
        }
    }
    for (int q = 0; q < kDiagVals; ++q) {
        double t = q == 5 ? block_max_d(v[q], sh) : block_sum_d(v[q], sh);
        if (threadIdx.x == 0) partial[(size_t)blockIdx.x * kDiagVals + q] = t;
    }
}

// One block adds the blocks' partials: thread t takes the partials t,
// t + kDiagBS, ... in order, then a fixed tree joins the threads, so the
// result does not depend on timing.
__global__ void __launch_bounds__(kDiagBS) fk_diag_final(int nblocks, const double* __restrict__ partial,
                                                        double* __restrict__ out) {
    __shared__ double sh[32];
    double acc[kDiagVals] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
        for (int q = 0; q < kDiagVals; ++q) {
            double x = partial[(size_t)b * kDiagVals + q];
            acc[q] = q == 5 ? fmax(acc[q], x) : acc[q] + x;
        }
    for (int q = 0; q < kDiagVals; ++q) {
        double t = q == 5 ? block_max_d(acc[q], sh) : block_sum_d(acc[q], sh);
        if (threadIdx.x == 0) out[q] = t;
    }
}


// Rouleaux, step 1: centre and bounding radius of each cell of a system, one
// block per cell.  The centre is the mean of the vertices taken as minimum
// images about the first vertex (FP64 sums), the radius the largest distance
// of a vertex from it.
__global__ void fk_cell_bounds(int c0, const int2* __restrict__ cell_verts, const SysInfo* __restrict__ sys,
                               const int* __restrict__ cellsys, const float4* __restrict__ mpos,
                               float4* __restrict__ out) {
    __shared__ double sh[32];
    __shared__ unsigned rmax;
    const int c = c0 + blockIdx.x;
    const int2 vr = cell_verts[c];
    if (vr.y < vr.x) {   // a cell without vertices (uniform across the block): no sphere
        if (threadIdx.x == 0) out[blockIdx.x] = make_float4(0.f, 0.f, 0.f, -1.f);
        return;
    }
    const GcGrid& g = sys[cellsys ? cellsys[c] : 0].g;
    const float3 x0 = xyz(mpos[vr.x]);
    double acc[3] = {0, 0, 0};
    for (int v = vr.x + threadIdx.x; v <= vr.y; v += blockDim.x) {
        float3 d = min_image(xyz(mpos[v]), x0, g);
        acc[0] += d.x; acc[1] += d.y; acc[2] += d.z;
    }
    const double inv = 1.0 / (double)(vr.y - vr.x + 1);
    double m[3];
    for (int k = 0; k < 3; ++k) m[k] = block_sum_d(acc[k], sh) * inv;
    const float3 cen = f3((float)(x0.x + m[0]), (float)(x0.y + m[1]), (float)(x0.z + m[2]));
    if (threadIdx.x == 0) rmax = 0u;
    __syncthreads();
    float r2 = 0.f;
    for (int v = vr.x + threadIdx.x; v <= vr.y; v += blockDim.x) r2 = fmaxf(r2, norm2_rn(min_image(xyz(mpos[v]), cen, g)));
#pragma unroll
    for (int o = 16; o; o >>= 1) r2 = fmaxf(r2, __shfl_xor_sync(0xffffffffu, r2, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&rmax, __float_as_uint(r2));   // non-negative floats order as their bits
    __syncthreads();
    if (threadIdx.x == 0) out[blockIdx.x] = make_float4(cen.x, cen.y, cen.z, sqrtf(__uint_as_float(rmax)));
}

// Rouleaux, step 2: one block per candidate pair of cells (a, b), which are
// in contact when some vertex of a and some vertex of b are closer than the
// contact distance (squared distance of their minimum image, FP32, < contact2).
// The vertices of b that can reach a (within a's radius + reach of its
// centre) are gathered into shared memory, 1024 at a time, and every vertex
// of a that can reach b is tested against them; the block stops at the first
// contact.
constexpr int kContactTile = 1024;

__global__ void __launch_bounds__(256) fk_cell_contact(int c0, const int2* __restrict__ pairs,
                                                       const int2* __restrict__ cell_verts, GcGrid g,
                                                       const float4* __restrict__ bounds,
                                                       const float4* __restrict__ mpos, float contact2, float reach,
                                                       int* __restrict__ hit) {
    __shared__ float4 tile[kContactTile];
    __shared__ int ntile, found;
    const int2 pr = pairs[blockIdx.x];
    const int2 va = cell_verts[c0 + pr.x], vb = cell_verts[c0 + pr.y];
    const float4 ba = bounds[pr.x], bb = bounds[pr.y];
    const float3 ca = f3(ba.x, ba.y, ba.z), cb = f3(bb.x, bb.y, bb.z);
    const float reach_a = ba.w + reach, reach_b = bb.w + reach;
    if (threadIdx.x == 0) found = 0;
    for (int b0 = vb.x; b0 <= vb.y; b0 += kContactTile) {
        const int b1 = min(vb.y + 1, b0 + kContactTile);
        if (threadIdx.x == 0) ntile = 0;
        __syncthreads();
        for (int v = b0 + threadIdx.x; v < b1; v += blockDim.x) {
            float4 x = mpos[v];
            if (norm2_rn(min_image(xyz(x), ca, g)) <= reach_a * reach_a) tile[atomicAdd(&ntile, 1)] = x;
        }
        __syncthreads();
        const int nt = ntile;
        for (int v = va.x + threadIdx.x; nt > 0 && v <= va.y; v += blockDim.x) {
            if (*(volatile int*)&found) break;
            const float3 x = xyz(mpos[v]);
            if (norm2_rn(min_image(x, cb, g)) > reach_b * reach_b) continue;
            for (int k = 0; k < nt; ++k) {
                if (norm2_rn(min_image(x, xyz(tile[k]), g)) < contact2) {
                    found = 1;
                    break;
                }
            }
        }
        __syncthreads();
        if (found) break;
    }
    if (threadIdx.x == 0) hit[blockIdx.x] = found;
}

}  // namespace

extern "C" {

int gc_ensemble_cell_stats(GcFused* f, int sys, double* out) {
    GC_TRY(check_sys(f, sys, "cell_stats"));
    if (!out) return gc_fail(GC_EINVAL, "cell_stats: NULL output");
    if (!f->setup_done) return gc_fail(GC_ESTATE, "cell_stats: call gc_fused_setup first");
    const HostCells& h = f->hcells[sys];
    if (!h.set || h.ncell <= 0) return GC_OK;
    fk_cell_stats<<<h.ncell, 256, 0, f->st>>>(f->c0[sys], f->cell_verts, f->dsys, f->cellsys, f->slot_of, f->a.vel,
                                             f->mforce, f->magg, f->have_agg ? 1 : 0, f->carea, f->cvol,
                                             f->cell_stats);
    GC_CHECK_LAUNCH("fused: cell statistics");
    GC_CUDA(cudaMemcpyAsync(out, f->cell_stats, 12 * sizeof(double) * h.ncell, cudaMemcpyDeviceToHost, f->st),
            "cell_stats");
    GC_CUDA(cudaStreamSynchronize(f->st), "cell_stats");
    return GC_OK;
}

int gc_ensemble_diagnostics(GcFused* f, int sys, double* out) {
    GC_TRY(check_sys(f, sys, "diagnostics"));
    if (!out) return gc_fail(GC_EINVAL, "diagnostics: NULL output");
    if (!f->setup_done) return gc_fail(GC_ESTATE, "diagnostics: call gc_fused_setup first");
    const SysInfo& S = f->hsys[sys];
    const int count = (int)(S.end - S.id0);
    const int nb = gc_blocks(count, kDiagBS);
    if (!f->diag) {
        int most = 0;
        for (const SysInfo& T : f->hsys) most = std::max(most, gc_blocks((int)(T.end - T.id0), kDiagBS));
        GC_TRY(falloc(f, &f->diag, (size_t)(most + 1) * kDiagVals));
    }
    fk_diag_partial<<<nb, kDiagBS, 0, f->st>>>(count, S.id0, S.fl, S.cs, f->p.mass, f->slot_of, f->a.vel, f->dp,
                                              f->diag);
    GC_CHECK_LAUNCH("fused: diagnostics");
    double* res = f->diag + (size_t)nb * kDiagVals;
    fk_diag_final<<<1, kDiagBS, 0, f->st>>>(nb, f->diag, res);
    GC_CHECK_LAUNCH("fused: diagnostics");
    double r[kDiagVals];
    GC_CUDA(cudaMemcpyAsync(r, res, sizeof(r), cudaMemcpyDeviceToHost, f->st), "diagnostics");
    GC_CUDA(cudaStreamSynchronize(f->st), "diagnostics");
    const double nm = r[4] > 0 ? r[4] : 1.0;
    out[0] = r[0];
    out[1] = r[1];
    out[2] = r[2];
    out[3] = 0.5 * r[3];                                        // kinetic energy
    // temperature from the peculiar velocities: (2 E_kin - |P|^2 / M) / (3 N)
    out[4] = (r[3] - (r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) / (f->p.mass * nm)) / (3.0 * nm);
    out[5] = r[5];                                              // largest speed
    out[6] = r[7] > 0 ? r[6] / r[7] : 0.0;                      // mean fluid density
    out[7] = r[4];                                              // moving particles
    return GC_OK;
}

int gc_ensemble_write_output(GcFused* f, int sys, const char* dir, long long step_data, double time, int first,
                             int threads) {
    GC_TRY(check_sys(f, sys, "write_output"));
    if (!dir) return gc_fail(GC_EINVAL, "write_output: NULL directory");
    if (!f->setup_done) return gc_fail(GC_ESTATE, "write_output: call gc_fused_setup first");
    const SysInfo& S = f->hsys[sys];
    const HostCells& h = f->hcells[sys];
    const int n = (int)(S.end - S.id0), ncp = (int)(S.end - S.cs);
    std::vector<float> pos(3 * (size_t)n), vel(3 * (size_t)n), rho(n), press(n);
    GC_TRY(store_range(f, S.id0, n, pos.data(), vel.data(), rho.data(), press.data(), nullptr, nullptr, nullptr, 0));
    GcOutputFrame fr;
    memset(&fr, 0, sizeof(fr));
    fr.n = n;
    fr.n_b1 = S.b2 - S.id0;
    fr.n_b2 = S.fl - S.b2;
    fr.n_cell_start = S.cs - S.id0;
    fr.pos = pos.data();
    fr.vel = vel.data();
    fr.rho = rho.data();
    fr.press = press.data();
    fr.threads = threads;
    std::vector<float> def, agg, cen, nor;
    std::vector<double> stats;
    if (h.set && h.ncell > 0) {
        def.resize(3 * (size_t)ncp);
        agg.resize(3 * (size_t)ncp);
        cen.resize(3 * (size_t)h.ntri);
        nor.resize(3 * (size_t)h.ntri);
        stats.resize(12 * (size_t)h.ncell);
        GC_TRY(gc_ensemble_store_cells(f, sys, nullptr, nullptr, def.data(), agg.data(), nor.data(), cen.data(),
                                       nullptr, 0));
        GC_TRY(gc_ensemble_cell_stats(f, sys, stats.data()));
        fr.ncell = h.ncell;
        fr.ntri = h.ntri;
        fr.cell_verts = h.verts.data();
        fr.tri = h.tri.data();
        fr.betri = h.betri.data();
        fr.defforce = def.data();
        fr.aggforce = agg.data();
        fr.tricenter = cen.data();
        fr.trinordir = nor.data();
        fr.cell_stats = stats.data();
    }
    return gc_output_write(&fr, dir, step_data, time, first);
}

int gc_fused_write_output(GcFused* f, const char* dir, long long step_data, double time, int first, int threads) {
    if (!f) return gc_fail(GC_EINVAL, "write_output: NULL handle");
    if (f->nsys != 1) return gc_fail(GC_EINVAL, "write_output: an ensemble writes one system at a time");
    return gc_ensemble_write_output(f, 0, dir, step_data, time, first, threads);
}



int gc_rouleaux_from_pairs(int ncell, int npairs, const int* pairs, int* label, int* size, int* nrouleaux) {
    if (ncell < 0 || npairs < 0 || !nrouleaux || (npairs > 0 && !pairs))
        return gc_fail(GC_EINVAL, "rouleaux: bad arguments (ncell %d, npairs %d)", ncell, npairs);
    std::vector<int> up(ncell);
    for (int c = 0; c < ncell; ++c) up[c] = c;
    auto root = [&](int c) {
        while (up[c] != c) c = up[c] = up[up[c]];   // path halving
        return c;
    };
    for (int k = 0; k < npairs; ++k) {
        int a = pairs[2 * k], b = pairs[2 * k + 1];
        if (a < 0 || a >= ncell || b < 0 || b >= ncell)
            return gc_fail(GC_EINVAL, "rouleaux: pair %d (%d, %d) outside 0..%d", k, a, b, ncell - 1);
        a = root(a);
        b = root(b);
        if (a != b) up[std::max(a, b)] = std::min(a, b);   // the lower cell stays the root
    }
    std::vector<int> lab(ncell, -1);
    int n = 0;
    if (size)
        for (int c = 0; c < ncell; ++c) size[c] = 0;
    for (int c = 0; c < ncell; ++c) {
        int r = root(c);
        if (lab[r] < 0) lab[r] = n++;
        if (label) label[c] = lab[r];
        if (size) ++size[lab[r]];
    }
    *nrouleaux = n;
    return GC_OK;
}

int gc_ensemble_rouleaux(GcFused* f, int sys, float contact, int* label, int* size, int* nrouleaux) {
    GC_TRY(check_sys(f, sys, "rouleaux"));
    if (!nrouleaux) return gc_fail(GC_EINVAL, "rouleaux: NULL count");
    if (!(contact > 0.f) || !isfinite(contact)) return gc_fail(GC_EINVAL, "rouleaux: contact distance %g", contact);
    if (!f->setup_done) return gc_fail(GC_ESTATE, "rouleaux: call gc_fused_setup first");
    const HostCells& h = f->hcells[sys];
    const int nc = h.set ? h.ncell : 0;
    if (nc == 0) {
        *nrouleaux = 0;
        return GC_OK;
    }
    const GcGrid& g = f->hsys[sys].g;
    const int c0 = f->c0[sys];
    // centres and radii
    GC_TRY(stage_bytes(f, (size_t)nc * 16));
    float4* dbounds = (float4*)f->stage;
    fk_cell_bounds<<<nc, 256, 0, f->st>>>(c0, f->cell_verts, f->dsys, f->cellsys, f->mpos, dbounds);
    GC_CHECK_LAUNCH("fused: cell bounds");
    std::vector<float4> bounds(nc);
    GC_CUDA(cudaMemcpyAsync(bounds.data(), dbounds, (size_t)nc * 16, cudaMemcpyDeviceToHost, f->st), "rouleaux");
    GC_CUDA(cudaStreamSynchronize(f->st), "rouleaux");
    // candidate pairs: bounding spheres within the contact distance (plus a
    // margin far above FP32 rounding of the centres and radii)
    const float reach = contact + 1e-3f;
    std::vector<int> cand;
    for (int a = 0; a < nc; ++a)
        for (int b = a + 1; b < nc; ++b) {
            if (bounds[a].w < 0.f || bounds[b].w < 0.f) continue;
            double d2 = 0;
            const float* pa = &bounds[a].x;
            const float* pb = &bounds[b].x;
            for (int k = 0; k < 3; ++k) {
                double d = (double)pa[k] - pb[k];
                if (g.pmask & (1 << k)) d -= g.L[k] * rint(d / g.L[k]);
                d2 += d * d;
            }
            double r = (double)bounds[a].w + bounds[b].w + reach;
            if (d2 <= r * r) {
                cand.push_back(a);
                cand.push_back(b);
            }
        }
    const int np = (int)cand.size() / 2;
    std::vector<int> contacts;
    if (np > 0) {
        // (a larger staging buffer is a new one: the bounds go up again)
        GC_TRY(stage_bytes(f, (size_t)nc * 16 + (size_t)np * 12));
        dbounds = (float4*)f->stage;
        int2* dpairs = (int2*)((char*)f->stage + (size_t)nc * 16);
        int* dhit = (int*)(dpairs + np);
        GC_CUDA(cudaMemcpyAsync(dbounds, bounds.data(), (size_t)nc * 16, cudaMemcpyHostToDevice, f->st), "rouleaux");
        GC_CUDA(cudaMemcpyAsync(dpairs, cand.data(), (size_t)np * 8, cudaMemcpyHostToDevice, f->st), "rouleaux");
        fk_cell_contact<<<np, 256, 0, f->st>>>(c0, dpairs, f->cell_verts, g, dbounds, f->mpos, contact * contact,
                                               reach, dhit);
        GC_CHECK_LAUNCH("fused: cell contacts");
        std::vector<int> hit(np);
        GC_CUDA(cudaMemcpyAsync(hit.data(), dhit, (size_t)np * 4, cudaMemcpyDeviceToHost, f->st), "rouleaux");
        GC_CUDA(cudaStreamSynchronize(f->st), "rouleaux");
        for (int k = 0; k < np; ++k)
            if (hit[k]) {
                contacts.push_back(cand[2 * k]);
                contacts.push_back(cand[2 * k + 1]);
            }
    }
    return gc_rouleaux_from_pairs(nc, (int)contacts.size() / 2, contacts.data(), label, size, nrouleaux);
}

}  // extern "C"
