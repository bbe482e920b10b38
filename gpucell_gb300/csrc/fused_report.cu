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
        double x = v[q];
        if (q == 5) {   // maximum
#pragma unroll
            for (int o = 16; o; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
            if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = x;
            __syncthreads();
            if (threadIdx.x == 0) {
                double m = 0.0;
                for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, sh[w]);
                partial[(size_t)blockIdx.x * kDiagVals + q] = m;
            }
            __syncthreads();
        } else {
            double t = block_sum_d(x, sh);
            if (threadIdx.x == 0) partial[(size_t)blockIdx.x * kDiagVals + q] = t;
        }
    }
}

__global__ void fk_diag_final(int nblocks, const double* __restrict__ partial, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double acc[kDiagVals] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int b = 0; b < nblocks; ++b)
        for (int q = 0; q < kDiagVals; ++q) {
            double x = partial[(size_t)b * kDiagVals + q];
            acc[q] = q == 5 ? fmax(acc[q], x) : acc[q] + x;
        }
    for (int q = 0; q < kDiagVals; ++q) out[q] = acc[q];
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
    fk_diag_final<<<1, 32, 0, f->st>>>(nb, f->diag, res);
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


}  // extern "C"
