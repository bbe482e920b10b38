// fused.cu -- the fused SDPD + membrane timestep on library-owned state, for
// one simulation or for an ensemble of independent ones in the same launches.
//
// Same method and the same step order as the boundary entry points
// (Particle::UpdatePar, src/Particle.cu:1310-1329), restructured for the GPU:
//
//   * State lives in the library, in slot order (sorted by cube), as float4
//     records: position + global id, velocity, predicted velocity, VelHalf,
//     force, and (1/d, P/d^2) per particle.  Membrane vertices additionally
//     have a membrane-ordered copy of their position and crossing counts, so
//     the membrane kernels index topology directly.
//   * An ensemble of independent simulations ("systems") shares the arrays.
//     System s owns the global ids [id0_s, end_s), in the same type order as
//     one simulation (Bound1, Bound2, fluid, membrane), its own box, cube
//     grid, body force and noise seed, and a contiguous range of the global
//     cube numbering; so the sort and every pass run once over all systems
//     and no pair ever spans two systems.  Each slot carries its system
//     index.  One simulation is an ensemble of one whose kernels take the
//     system from their parameters instead of the table.
//   * Neighbours come from Verlet lists with a skin: built from a scan of
//     the cubes around each particle at cut-off rc + skin (5 x 5 x 5 cubes
//     half that wide, rows and cells beyond the cut-off skipped; 27 cubes of
//     full width where a periodic axis has fewer than five), stored 32 slots
//     interleaved (entry k of slot i at ((i/32)*cap + k)*32 + i%32, so a
//     warp reads 128 contiguous bytes per k), and rebuilt (with a re-sort)
//     only when some particle has moved more than skin/2 since the last
//     build.  The Morse aggregation's pairs (vertices of different cells)
//     have lists of their own, built with these.  Every step still tests
//     r^2 < rc^2 in FP32 on the listed pairs, with r^2 formed by fused
//     multiply-adds (the boundary kernels and the oracle round each square:
//     a pair within one rounding of the cut-off, where the kernel and its
//     derivative are below 1e-21 of their peaks, may count in one and not
//     in the other).
//   * Passes are fused: integrate + periodic wrap + predictor (K2, K3, K9);
//     density + equation of state + wall velocity (K8, K11, K10); SDPD +
//     wall repulsion + body force + membrane forces + corrector (K12, K13,
//     K14, K17/K18 add, K19); wall velocity again (K10).
//   * Per-cell membrane area and volume are summed in FP64.
//   * Optionally each step is one captured CUDA graph: the rebuild decision
//     is taken on the device (a conditional node runs the re-sort and list
//     build only when some particle moved more than skin/2), the noise key of
//     the step is derived on the device from a step counter, and the host
//     synchronises once per gc_fused_step call instead of once per step.
#include "fused_internal.cuh"

#include <cuda_fp16.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

namespace gcf {





// Pair difference without the image shift: exact for a particle farther
// than rc + 2 skin from every periodic face (its listed partners, which have
// moved at most skin/2 each since the lists were built, are then less than
// L/2 away along every axis, where rint(d/L) = 0 and pair_image returns the
// plain difference).
template <bool WRAP>
__device__ __forceinline__ float3 pair_diff(float3 a, float3 b, const Box& B) {
    if constexpr (WRAP) return pair_image(a, b, B);
    else return f3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}

// Whether a particle at x is within `margin` of a periodic face of its box.
__device__ __forceinline__ bool near_face(float3 x, const GcGrid& g, float margin) {
    bool w = false;
    if (g.pmask & 1) w |= (x.x - g.lo[0] < margin) || (g.hi[0] - x.x <= margin);
    if (g.pmask & 2) w |= (x.y - g.lo[1] < margin) || (g.hi[1] - x.y <= margin);
    if (g.pmask & 4) w |= (x.z - g.lo[2] < margin) || (g.hi[2] - x.z <= margin);
    return w;
}

// ---------------------------------------------------------------------------
// Step prologue on the device: advance the step counter, derive every
// system's noise key for the new step, clear the rebuild flag.
// ---------------------------------------------------------------------------
__global__ void fk_step_begin(int nsys, const SysInfo* __restrict__ sys, long long* __restrict__ dstep,
                              unsigned* __restrict__ nkey, int* __restrict__ rebuild) {
    long long s = *dstep + 1;
    for (int k = threadIdx.x; k < nsys; k += blockDim.x) nkey[k] = noise_key(sys[k].seed, (uint64_t)s);
    __syncthreads();
    if (threadIdx.x == 0) {
        *dstep = s;
        *rebuild = 0;
    }
}

// Sets the condition of the rebuild node of a captured step and counts the
// rebuilds.  Launched only inside a captured graph.
__global__ void fk_set_cond(cudaGraphConditionalHandle h, const int* __restrict__ rebuild,
                            unsigned long long* __restrict__ count) {
    unsigned v = *rebuild != 0;
    cudaGraphSetConditional(h, v);
    if (v) *count += 1;
}

// ---------------------------------------------------------------------------
// K2 + K3 + K9 for fluid and membrane slots
// ---------------------------------------------------------------------------
template <bool ENS>
__global__ void fk_integrate(int n, GcParams p, SysInfo s0, const SysInfo* __restrict__ sys,
                             const int* __restrict__ sysid, float4* __restrict__ pos, const float4* __restrict__ vel,
                             float4* __restrict__ vh, float4* __restrict__ vpred, const float4* __restrict__ force,
                             float4* __restrict__ plo, const float4* __restrict__ refpos, int4* __restrict__ nthro,
                             float half_skin2, int* __restrict__ rebuild, float4* __restrict__ mpos,
                             float4* __restrict__ mplo, int4* __restrict__ mnthro, unsigned* flags, int ddpos) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool far = false;
    if (i < n) {
        float4 x = pos[i];
        unsigned id = fid(x);
        GC_SYS_OF(S, i);
        if (id >= S.fl) {
            float4 v = vel[i], f = force[i];
            float h = 0.5f * p.dt * p.dt * p.inv_mass;
            // the displacement in FP32, added to the double-float position
            float4 lo = plo[i];
            pos_add(x.x, lo.x, p.dt * v.x + h * f.x, ddpos);
            pos_add(x.y, lo.y, p.dt * v.y + h * f.y, ddpos);
            pos_add(x.z, lo.z, p.dt * v.z + h * f.z, ddpos);
            if (!(isfinite(x.x) && isfinite(x.y) && isfinite(x.z))) raise_flag(flags, GC_FLAG_NONFINITE);
            // periodic crossings; the crossing counts are read only where
            // they change or are mirrored (membrane vertices)
            int cr[3] = {0, 0, 0};
            float* xs[3] = {&x.x, &x.y, &x.z};
            float* ls[3] = {&lo.x, &lo.y, &lo.z};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (!(S.g.pmask & (1 << a))) continue;
                float c = *xs[a];
                if (c >= S.g.hi[a]) { pos_add(*xs[a], *ls[a], -S.g.L[a], ddpos); cr[a] = 1; }
                else if (c < S.g.lo[a]) { pos_add(*xs[a], *ls[a], S.g.L[a], ddpos); cr[a] = -1; }
            }
            const bool crossed = (cr[0] | cr[1] | cr[2]) != 0, memb = id >= S.cs;
            int4 t = make_int4(0, 0, 0, 0);
            if (crossed || memb) {
                t = nthro[i];
                t.x += cr[0];
                t.y += cr[1];
                t.z += cr[2];
                if (crossed) nthro[i] = t;
            }
            pos[i] = x;
            plo[i] = lo;
            // VelHalf's fourth word is always zero
            float hs = 0.5f * p.dt * p.inv_mass, l = p.lambda * p.dt * p.inv_mass;
            vh[i] = make_float4(v.x + hs * f.x, v.y + hs * f.y, v.z + hs * f.z, 0.f);
            vpred[i] = make_float4(v.x + l * f.x, v.y + l * f.y, v.z + l * f.z, 0.f);
            float3 d = min_image(xyz(x), xyz(refpos[i]), S.g);
            far = norm2_rn(d) > half_skin2;
            if (memb) {
                unsigned m = S.m0 + (id - S.cs);
                mpos[m] = x;
                mplo[m] = lo;
                mnthro[m] = t;
            }
        }
    }
    if (__any_sync(0xffffffffu, far) && (threadIdx.x & 31) == 0) atomicOr(rebuild, 1);
}

// ---------------------------------------------------------------------------
// Rebuild: cube keys, permutation, neighbour lists
// ---------------------------------------------------------------------------
__global__ void fk_cellkey(int n, const SysInfo* __restrict__ sys, const int* __restrict__ sysid,
                           const float4* __restrict__ pos, int* __restrict__ keys, int* __restrict__ vals) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SysInfo& S = sys[sysid ? sysid[i] : 0];
    float4 x = pos[i];
    keys[i] = S.cube0 + cube_key(cube_coord(x.x, 0, S.g), cube_coord(x.y, 1, S.g), cube_coord(x.z, 2, S.g), S.g);
    vals[i] = i;
}


// Gathers the slot arrays into the new order and wraps every position into
// its box on periodic axes (counting the crossings), so that the list build
// can use one image shift per row of cubes.
__global__ void fk_permute(int n, const SysInfo* __restrict__ sys, const int* __restrict__ perm, SlotArrays src,
                           SlotArrays dst, float4* __restrict__ refpos, int* __restrict__ slot_of, int ddpos) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    int o = perm[q];
    int s = src.sys ? src.sys[o] : 0;
    const GcGrid& g = sys[s].g;
    float4 x = src.pos[o], lo = src.plo[o];
    int4 t = src.nthro[o];
    float* xs[3] = {&x.x, &x.y, &x.z};
    float* ls[3] = {&lo.x, &lo.y, &lo.z};
    int* ts[3] = {&t.x, &t.y, &t.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (!(g.pmask & (1 << a))) continue;
        float c = *xs[a];
        if (!isfinite(c)) continue;
        int w = (int)floorf((c - g.lo[a]) / g.L[a]);
        if (w != 0) {
            pos_add(*xs[a], *ls[a], -(float)w * g.L[a], ddpos);
            if (*xs[a] >= g.hi[a]) { pos_add(*xs[a], *ls[a], -g.L[a], ddpos); ++w; }
            else if (*xs[a] < g.lo[a]) { pos_add(*xs[a], *ls[a], g.L[a], ddpos); --w; }
            *ts[a] += w;
        }
    }
    dst.pos[q] = x;
    dst.plo[q] = lo;
    dst.vel[q] = src.vel[o];
    dst.vpred[q] = src.vpred[o];
    dst.vh[q] = src.vh[o];
    dst.force[q] = src.force[o];
    dst.nthro[q] = t;
    if (dst.sys) dst.sys[q] = s;
    refpos[q] = x;
    slot_of[fid(x)] = q;
}

// Copies the permuted slot arrays back (captured steps, whose launches are
// bound to fixed buffers, cannot swap them).
__global__ void fk_copy_slots(int n, SlotArrays src, SlotArrays dst) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    dst.pos[q] = src.pos[q];
    dst.plo[q] = src.plo[q];
    dst.vel[q] = src.vel[q];
    dst.vpred[q] = src.vpred[q];
    dst.vh[q] = src.vh[q];
    dst.force[q] = src.force[q];
    dst.nthro[q] = src.nthro[q];
    if (dst.sys) dst.sys[q] = src.sys[q];
}

// Candidates [b, e) of one row of cubes against xs, the image of slot i's
// position that the row needs; appends the ones within the cut-off to the
// list of slot i (entry k at lst[32 k]).
__device__ __forceinline__ void scan_range(const float4* __restrict__ pos, unsigned b, unsigned e, float3 xs, int i,
                                           float cut2, bool mobile_only, unsigned fl, int cap,
                                           int* __restrict__ lst, int& k) {
    // one predicate per candidate and a predicated store, no branches: the
    // lanes of a warp stay together through the scan (12 % faster than
    // skipping a rejected candidate with a branch)
#pragma unroll 4
    for (unsigned j = b; j < e; ++j) {
        float4 xj = pos[j];
        float dx = xs.x - xj.x, dy = xs.y - xj.y, dz = xs.z - xj.z;
        float r2 = dx * dx + dy * dy + dz * dz;
        const bool take = r2 < cut2 && (int)j != i && !(mobile_only && fid(xj) < fl);
        if (take && k < cap) lst[(size_t)k * 32] = (int)j;
        k += take;
    }
}

// Gap between a coordinate and the slab of cell c along an axis (0 inside
// it); the first and last cells of a wall axis extend to infinity.
__device__ __forceinline__ float slab_gap(float x, int c, int axis, const GcGrid& g) {
    const bool per = g.pmask & (1 << axis);
    const float w = 1.f / g.invw[axis];
    const float lo = g.origin[axis] + (float)c * w, hi = lo + w;
    float gap = 0.f;
    if (x < lo && (per || c > 0)) gap = lo - x;
    else if (x > hi && (per || c < g.n[axis] - 1)) gap = x - hi;
    return gap;
}

// One thread per slot scans the cells of its system's list grid within the
// stencil radius R around its own (R = 2 for cells at least (rc + skin)/2
// wide, R = 1 for cubes at least rc + skin wide; either way every pair
// within rc + skin is found).  Fluid and membrane slots list every particle
// within rc + skin; Bound2 slots list the moving particles (for their wall
// velocity); Bound1 slots list nothing.  Positions are inside the box on
// periodic axes (the permutation wraps them), so each neighbouring row of
// cells has one image shift, and the 2R + 1 cells of a row that do not wrap
// are one contiguous range of slots.
__global__ void __launch_bounds__(kMaxBS, GC_BUILD_MIN_BLOCKS) fk_build_list(int n, const SysInfo* __restrict__ sys,
                                                     const int* __restrict__ sysid, const float4* __restrict__ pos,
                                                     const unsigned* __restrict__ start, int* __restrict__ nbr,
                                                     int* __restrict__ cnt, int cap, float cut2, unsigned* flags,
                                                     int* __restrict__ need, int walls_only) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 xi4 = pos[i];
    float3 xi = xyz(xi4);
    unsigned id = fid(xi4);
    const SysInfo& S = sys[sysid ? sysid[i] : 0];
    int t = stype(id, S);
    if (walls_only && t != PT_B2) {   // the pair tiles cover the other slots
        cnt[i] = 0;
        return;
    }
    int k = 0;
    const GcGrid& g = S.g;
    const unsigned fl = S.fl;
    int* lst = nbr + sell(i, 0, cap);
    const bool mobile_only = t == PT_B2;
    if (t != PT_B1) {
        const int R = S.lr;
        int cx = cube_coord(xi.x, 0, g), cy = cube_coord(xi.y, 1, g), cz = cube_coord(xi.z, 2, g);
        // Rows and cells that lie wholly beyond the cut-off are not scanned:
        // the distance from the (image of the) position to a row's y/z slab
        // leaves a reach along x, and only the cells within it are read.
        // The slabs are taken with a margin far above the rounding of the
        // cell assignment, and the edge cells of a wall axis reach to
        // infinity (particles beyond the grid are clamped into them), so no
        // candidate within the cut-off is skipped and the lists are the same
        // entries in the same order as a scan of all (2R+1)^3 cells.
        const float cut = sqrtf(cut2), eps = 2e-3f;
        const float lim2 = (cut + eps) * (cut + eps);
        for (int dz = -R; dz <= R; ++dz) {
            int z = cz + dz;
            float sz = 0.f;
            if (z < 0) { if (!(g.pmask & 4)) continue; z += g.n[2]; sz = g.L[2]; }
            else if (z >= g.n[2]) { if (!(g.pmask & 4)) continue; z -= g.n[2]; sz = -g.L[2]; }
            const float dzv = slab_gap(xi.z + sz, z, 2, g);
            if (dzv * dzv > lim2) continue;
            for (int dy = -R; dy <= R; ++dy) {
                int y = cy + dy;
                float sy = 0.f;
                if (y < 0) { if (!(g.pmask & 2)) continue; y += g.n[1]; sy = g.L[1]; }
                else if (y >= g.n[1]) { if (!(g.pmask & 2)) continue; y -= g.n[1]; sy = -g.L[1]; }
                const float dyv = slab_gap(xi.y + sy, y, 1, g);
                const float d2 = dyv * dyv + dzv * dzv;
                if (d2 > lim2) continue;
                // cells along x within the reach left by this row
                const float reach = sqrtf(fmaxf(cut2 - d2, 0.f)) + eps;
                const int xlo = max(cx - R, (int)floorf((xi.x - reach - g.origin[0]) * g.invw[0]));
                const int xhi = min(cx + R, (int)floorf((xi.x + reach - g.origin[0]) * g.invw[0]));
                int row = S.cube0 + g.n[0] * (y + g.n[1] * z);
                if (xlo >= 0 && xhi < g.n[0]) {
                    if (xlo <= xhi)
                        scan_range(pos, start[row + xlo], start[row + xhi + 1], f3(xi.x, xi.y + sy, xi.z + sz), i,
                                   cut2, mobile_only, fl, cap, lst, k);
                } else {
                    // near a face of the x axis: cell by cell (the edge cells
                    // of a wall axis hold clamped particles: always scanned)
                    const int a = (g.pmask & 1) ? xlo : cx - R, b = (g.pmask & 1) ? xhi : cx + R;
                    for (int x0 = a; x0 <= b; ++x0) {
                        int x = x0;
                        float sx = 0.f;
                        if (x < 0) { if (!(g.pmask & 1)) continue; x += g.n[0]; sx = g.L[0]; }
                        else if (x >= g.n[0]) { if (!(g.pmask & 1)) continue; x -= g.n[0]; sx = -g.L[0]; }
                        scan_range(pos, start[row + x], start[row + x + 1], f3(xi.x + sx, xi.y + sy, xi.z + sz), i,
                                   cut2, mobile_only, fl, cap, lst, k);
                    }
                }
            }
        }
    }
    if (k > cap) {   // the list holds cap entries; the host grows it to the longest wanted
        raise_flag(flags, GC_FLAG_CELL_OVERFLOW);
        atomicMax(need, k);
        k = cap;
    }
    cnt[i] = k;
    // pad to a multiple of four with the sentinel slot n (its position is
    // NaN, so it never passes a cut-off test); the capacity is a multiple of 8
    for (int q = k; q < ((k + 3) & ~3); ++q) nbr[sell(i, q, cap)] = n;
}

// ---------------------------------------------------------------------------
// K8 + K11 (+ K10 for Bound2 slots)
// ---------------------------------------------------------------------------

// With `cmask` set, fluid and membrane slots also record which of their list
// entries act this step (SDPD partners within rc, Bound1 walls within the
// repulsion range): one bit per entry, 32 entries per word, words of 32 slots
// interleaved like the lists (word w of slot i at ((i/32)*mw + w)*32 + i%32),
// and the number of set bits in ccnt.  The force pass then iterates only the
// set bits, so no lane idles on an entry that does not act.

#ifndef GC_DENS_MIN_BLOCKS
#define GC_DENS_MIN_BLOCKS 5
#endif

template <bool ENS, bool B1>
__global__ void __launch_bounds__(kMaxBS, GC_DENS_MIN_BLOCKS) fk_density(int n, GcParams p, SysInfo s0, const SysInfo* __restrict__ sys,
                                                  const int* __restrict__ sysid, const float4* __restrict__ pos,
                                                  float4* __restrict__ vpred, const float4* __restrict__ vh,
                                                  float2* __restrict__ dp, const int* __restrict__ nbr,
                                                  const int* __restrict__ cnt, int cap, unsigned* __restrict__ cmask,
                                                  int mw, int* __restrict__ ccnt, float wrap_margin) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 xi4 = pos[i];
    float3 xi = xyz(xi4);
    unsigned id = fid(xi4);
    GC_SYS_OF(S, i);
    const Box B = box_of(S);
    const unsigned b2 = S.b2;
    int t = stype(id, S);
    int c = cnt[i];
    const int* lp = nbr + sell(i, 0, cap);
    if (t == PT_FLUID || t == PT_MEMB) {
        // the sum of W / wnorm, the particle's own share (W(0) / wnorm = 1)
        // first; wnorm multiplies it once at the end
        float acc = 1.f;
        const float inv_rc4 = 4.f * p.inv_rc;
        int kc = 0;
        // The list is padded to a multiple of four entries with the sentinel
        // slot.  Entries go in groups of four: the indices of the next group
        // are loaded while the current group is evaluated, so that a thread
        // keeps four index loads and four position loads in flight; the
        // acting-entry bits of each 32-entry word are stored once.  The
        // lanes of a warp read each line of the list together, once: the
        // index loads stream (evict first), so that the list does not push
        // the particle data the gathers need out of the caches.
        const int c4 = (c + 3) & ~3;
        auto run = [&](auto wrap) {
            constexpr bool W = decltype(wrap)::value;
            int jq[4];
            if (c4 > 0) {
#pragma unroll
                for (int u = 0; u < 4; ++u) jq[u] = __ldcs(lp + (size_t)u * 32);
            }
            for (int w0 = 0; w0 < c4; w0 += 32) {
                unsigned m = 0;
                const int wend = min(w0 + 32, c4);
                for (int k0 = w0; k0 < wend; k0 += 4) {
                    float4 xj[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) xj[u] = pos[jq[u]];
                    if (k0 + 4 < c4) {
#pragma unroll
                        for (int u = 0; u < 4; ++u) jq[u] = __ldcs(lp + (size_t)(k0 + 4 + u) * 32);
                    }
                    // without branches: W is formed for every entry and added
                    // (as +0 when the entry does not count, which leaves the sum
                    // as it is), so that no lane waits on another's branch
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const float3 dd = pair_diff<W>(xi, xyz(xj[u]), B);
                        const float r2 = norm2_fma(dd);
                        // without Bound1 walls in any system (B1 false) every partner is SDPD
                        const bool in = r2 < p.rc2, apart = r2 > 0.f, sdpd = !B1 || fid(xj[u]) >= b2;
                        const float r = apart ? r2 * rsqrt_ftz(r2) : 0.f;
                        // (1 - s)^4 (1 + 4 s), s = r / rc
                        const float tt = fmaf(-r, p.inv_rc, 1.f), t2 = tt * tt;
                        acc += in && sdpd ? t2 * t2 * fmaf(r, inv_rc4, 1.f) : 0.f;
                        // acting: an SDPD partner within rc, or a Bound1 wall within the repulsion range
                        const bool act = in && apart && (sdpd || (B1 && r2 < p.rep_r0sq));
                        m |= (unsigned)act << (k0 - w0 + u);
                    }
                }
                if (cmask) {
                    cmask[mrow(i, w0 >> 5, mw)] = m;
                    kc += __popc(m);
                }
            }
        };
        // one form per warp (the image where any of its particles is near a
        // periodic face), so that a warp does not run both
        if (__any_sync(__activemask(), near_face(xi, S.g, wrap_margin))) run(std::true_type{});
        else run(std::false_type{});
        if (ccnt) ccnt[i] = kc;
        const float sum = p.wnorm * acc;
        float rho = p.mass * sum;
        float c2 = (t == PT_MEMB) ? p.c2sq : p.c1sq;
        float inv_d = __frcp_rn(sum);
        dp[i] = make_float2(inv_d, c2 * (rho - p.rho0) * inv_d * inv_d);
        return;
    }
    dp[i] = make_float2(p.mass / p.rho0, 0.f);
    if (t != PT_B2) return;
    float3 num = f3(0.f, 0.f, 0.f);
    float den = 0.f;
    for (int k = 0; k < c; ++k) {
        int j = __ldg(lp + (size_t)k * 32);
        float r2 = norm2_rn(pair_image(xi, xyz(pos[j]), B));
        if (r2 >= p.rc2) continue;
        float r = r2 > 0.f ? r2 * rsqrtf(r2) : 0.f;
        float w = wendland_w(r, p);
        float4 vj = vpred[j];
        num += w * f3(vj.x, vj.y, vj.z);
        den += w;
    }
    float4 w4 = vh[i];
    float3 v = den > 0.f ? f3(2.f * w4.x - num.x / den, 2.f * w4.y - num.y / den, 2.f * w4.z - num.z / den)
                         : f3(w4.x, w4.y, w4.z);
    vpred[i] = make_float4(v.x, v.y, v.z, 0.f);
}

// ---------------------------------------------------------------------------
// K12 + K13 + K14 + membrane forces + K19
// ---------------------------------------------------------------------------
// COMPACT: iterate only the entries fk_density marked as acting this step,
// so the cut-off test is already done.  The pair noise is keyed by the ids
// local to the system, so a system draws the same noise in an ensemble as
// alone.
// Acting entries are taken in groups of kForceGroup: the list indices of the
// next group are loaded while the current group is evaluated, and a group's
// position, density and velocity loads are issued together, so that each
// thread has several independent gathers in flight.
#ifndef GC_FORCE_GROUP
#define GC_FORCE_GROUP 1
#endif
#ifndef GC_FORCE_AHEAD
#define GC_FORCE_AHEAD 1
#endif
constexpr int kForceGroup = GC_FORCE_GROUP;
constexpr int kForceAhead = GC_FORCE_AHEAD;   // groups of list indices loaded ahead

#ifndef GC_FORCE_MIN_BLOCKS
#define GC_FORCE_MIN_BLOCKS (kForceGroup == 1 ? 6 : (kForceGroup == 2 ? 4 : 3))
#endif
constexpr int force_min_blocks(bool ens) { return GC_FORCE_MIN_BLOCKS - (ens ? 1 : 0); }

// The predicted velocity of a neighbour packed to FP16 (x, y | z, 0): 8 bytes
// per gather instead of 16 (GcFusedOptions.half_velocity, an experiment).
__device__ __forceinline__ float4 unpack_vel(uint2 u) {
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
    return make_float4(a.x, a.y, b.x, 0.f);
}

__global__ void fk_pack_vel(int n, const float4* __restrict__ v, uint2* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 x = v[i];
    const __half2 a = __floats2half2_rn(x.x, x.y), b = __floats2half2_rn(x.z, 0.f);
    out[i] = make_uint2(*reinterpret_cast<const unsigned*>(&a), *reinterpret_cast<const unsigned*>(&b));
}

template <bool COMPACT, bool ENS, bool HALFV, bool NOISE, bool B1>
__global__ void __launch_bounds__(kMaxBS, force_min_blocks(ENS))
    fk_force(int n, GcParams p, SysInfo s0, const SysInfo* __restrict__ sys, const int* __restrict__ sysid,
             const unsigned* __restrict__ nkey, const float4* __restrict__ pos, const float4* __restrict__ vpred,
             const float4* __restrict__ vh, const float2* __restrict__ dp, float4* __restrict__ force,
             float4* __restrict__ vel, const int* __restrict__ nbr, const int* __restrict__ cnt, int cap,
             const unsigned* __restrict__ cmask, int mw, const float4* __restrict__ mforce, int drive,
             const uint2* __restrict__ vph, float wrap_margin) {
    constexpr int G = kForceGroup;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 xi4 = pos[i];
    float3 xi = xyz(xi4);
    unsigned id = fid(xi4);
    const int s = ENS ? (sysid ? sysid[i] : 0) : 0;
    GC_SYS_OF(S, i);
    if (id < S.fl) {
        force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const Box B = box_of(S);
    const unsigned b2 = S.b2;
    const unsigned id0 = S.id0;
    // one system: the key of the step from the parameters, or, in a captured
    // step, from the device (fk_step_begin derives it at each replay)
    const uint32_t key = ENS ? nkey[s] : (nkey ? nkey[0] : p.noise_key);
    float4 vi = vpred[i];
    float2 dpi = dp[i];
    float3 f = f3(0.f, 0.f, 0.f);
    int c = cnt[i];
    const int* lp = nbr + sell(i, 0, cap);
    const unsigned* mp = COMPACT ? cmask + mrow(i, 0, mw) : nullptr;
    unsigned m = 0;
    int base = -32;
    // index of the next acting entry (COMPACT) or of the next entry; called
    // once per entry, in order.  The scan for a non-empty mask word ends: it
    // runs only while k < c, and c = ccnt[i] is the number of bits set in the
    // row's mask words, which fk_density writes together with it, word by
    // word, in the same thread.  Every launch of this kernel with COMPACT
    // follows a fk_density launch with the mask on in the same step (host-
    // driven steps, captured steps, refresh after a rebuild, a restore or a
    // change of options); set-up's density pass without the mask is always
    // followed by such a step before any force pass.  A list that overflowed
    // keeps cap entries, and both passes read the same c <= cap of them.  (A
    // bound on the row's words cost 6 % of this kernel.)
    auto next_k = [&](int k) -> int {
        if constexpr (COMPACT) {
            while (m == 0) {
                base += 32;
                m = __ldg(mp + (size_t)(base >> 5) * 32);
            }
            int b = __ffs(m) - 1;
            m &= m - 1;
            return base + b;
        } else {
            return k;
        }
    };
    constexpr int A = kForceAhead;
    // The pair terms are gathered into three vectors: one coefficient along
    // d = x_i - x_j (pressure, the e e^T parts of the viscous and random
    // forces, with e = d / r folded into the coefficients as 1/r^2), one
    // along v_ij (viscous) and one along xi_ij (random).  F (d_i^-1 d_j^-1)
    // is formed as F times the product of the two inverse number densities,
    // the same product from either side of the pair.
    const float cAB = p.sqrtAB - p.sqrtA;
    // one pair: neighbour position (with its id), (1/d, P/d^2) and velocity
    auto pair = [&](auto wrapc, float4 xj4, float2 dpj, float4 vj) {
        constexpr bool W = decltype(wrapc)::value;
        float3 d = pair_diff<W>(xi, xyz(xj4), B);
        float r2 = norm2_fma(d);   // as in fk_density
        if (!COMPACT && (r2 >= p.rc2 || r2 <= 0.f)) return;   // coincident pairs exert no force
        unsigned idj = fid(xj4);
        float inv_r = rsqrt_ftz(r2);
        if (B1 && idj < b2) {   // Bound1: repulsion only (B1: some system has such walls)
            if (r2 < p.rep_r0sq) {
                float ir2 = inv_r * inv_r;
                float q2 = p.rep_r0sq * ir2, q4 = q2 * q2, q12 = q4 * q4 * q4;
                f += (p.rep_D * (q12 - q4) * ir2) * d;
            }
            return;
        }
        float F = wendland_f(r2 * inv_r, p);
        float ir2 = inv_r * inv_r;
        float3 vij = f3(vi.x - vj.x, vi.y - vj.y, vi.z - vj.z);
        float fdd = F * (dpi.x * dpj.x);
        float cd = (dpi.y + dpj.y) * F - (fdd * p.visB) * dot3(d, vij) * ir2;
        f += (-fdd * p.visA) * vij;
        if constexpr (NOISE) {
            float qq = p.noise_pref * fdd;
            float q = qq > 0.f ? qq * rsqrt_ftz(qq) : 0.f;
            q = id < idj ? q : -q;   // the pair sign of xi_ij
            float3 xi_ = pair_noise_unsigned_k(id - id0, idj - id0, key);
            cd += (q * cAB) * dot3(d, xi_) * ir2;
            f += (q * p.sqrtA) * xi_;
        }
        f += cd * d;
    };
    auto gather_v = [&](int j) -> float4 { return HALFV ? unpack_vel(vph[j]) : vpred[j]; };
    auto run = [&](auto wrapc) {
        {
            int jq[A][G];
#pragma unroll
            for (int a = 0; a < A; ++a)
#pragma unroll
                for (int u = 0; u < G; ++u) {
                    int k = a * G + u;
                    jq[a][u] = k < c ? __ldg(lp + (size_t)next_k(k) * 32) : i;
                }
            for (int k0 = 0; k0 < c; k0 += G) {
                float4 xg[G], vg[G];
                float2 dg[G];
#pragma unroll
                for (int u = 0; u < G; ++u) {
                    xg[u] = pos[jq[0][u]];
                    dg[u] = dp[jq[0][u]];
                    vg[u] = gather_v(jq[0][u]);
                }
#pragma unroll
                for (int a = 0; a + 1 < A; ++a)
#pragma unroll
                    for (int u = 0; u < G; ++u) jq[a][u] = jq[a + 1][u];
#pragma unroll
                for (int u = 0; u < G; ++u) {
                    int k = k0 + A * G + u;
                    jq[A - 1][u] = k < c ? __ldg(lp + (size_t)next_k(k) * 32) : i;
                }
#pragma unroll
                for (int u = 0; u < G; ++u) {
                    if (k0 + u >= c) break;
                    pair(wrapc, xg[u], dg[u], vg[u]);
                }
            }
        }
    };
    // A warp whose particles all lie farther than wrap_margin from every
    // periodic face forms plain differences (equal to the minimum image for
    // every listed pair there); any other warp forms the image.
    if (__any_sync(__activemask(), near_face(xi, S.g, wrap_margin))) run(std::true_type{});
    else run(std::false_type{});
    if (drive) f.x += S.gx;
    if (id >= S.cs && mforce) {
        float4 mf = mforce[S.m0 + (id - S.cs)];
        f += f3(mf.x, mf.y, mf.z);
    }
    // a non-finite force shows up as a non-finite position in the next
    // fk_integrate, which raises GC_FLAG_NONFINITE
    force[i] = make_float4(f.x, f.y, f.z, 0.f);
    float4 h = vh[i];
    float sc = 0.5f * p.dt * p.inv_mass;
    vel[i] = make_float4(h.x + sc * f.x, h.y + sc * f.y, h.z + sc * f.z, 0.f);
}

// second K10: wall velocity from the corrected velocities
template <bool ENS>
__global__ void fk_wallvel(int n, GcParams p, SysInfo s0, const SysInfo* __restrict__ sys,
                           const int* __restrict__ sysid, const float4* __restrict__ pos, float4* __restrict__ vel,
                           const float4* __restrict__ vh, const int* __restrict__ nbr, const int* __restrict__ cnt,
                           int cap) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 xi4 = pos[i];
    GC_SYS_OF(S, i);
    if (stype(fid(xi4), S) != PT_B2) return;
    const Box B = box_of(S);
    float3 xi = xyz(xi4);
    float3 num = f3(0.f, 0.f, 0.f);
    float den = 0.f;
    int c = cnt[i];
    for (int k = 0; k < c; ++k) {
        int j = __ldg(nbr + sell(i, k, cap));
        float r2 = norm2_rn(pair_image(xi, xyz(pos[j]), B));
        if (r2 >= p.rc2) continue;
        float w = wendland_w(r2 > 0.f ? r2 * rsqrtf(r2) : 0.f, p);
        float4 vj = vel[j];
        num += w * f3(vj.x, vj.y, vj.z);
        den += w;
    }
    float4 w4 = vh[i];
    float3 v = den > 0.f ? f3(2.f * w4.x - num.x / den, 2.f * w4.y - num.y / den, 2.f * w4.z - num.z / den)
                         : f3(w4.x, w4.y, w4.z);
    vel[i] = make_float4(v.x, v.y, v.z, 0.f);
}

// ---------------------------------------------------------------------------
// Membranes (membrane order; positions unwrapped with crossing counts).
// Vertex, triangle and cell indices are global over the ensemble; msys and
// cellsys give the system of a vertex and of a cell (nullptr: system 0).
// ---------------------------------------------------------------------------
// (a + la) - (b + lb) + k L along one axis for double-float positions
// (value a, low part la) and crossing counts differing by k: the rounding
// errors of a - b, of k L and of adding it are kept by TwoSum / FMA and
// added with the low parts at the end, so the result is the difference of
// the exact positions rounded once.  A cell's geometry is then the same
// whether its vertices are wrapped into the box or not.
__device__ __forceinline__ float dd_sub1(float a, float la, float b, float lb, int k, float L) {
    const float nb = -b;
    const float s = __fadd_rn(a, nb), s1 = __fsub_rn(s, a);
    const float e1 = __fadd_rn(__fsub_rn(a, __fsub_rn(s, s1)), __fsub_rn(nb, s1));
    const float sh = __fmul_rn((float)k, L), esh = fmaf((float)k, L, -sh);
    const float t = __fadd_rn(s, sh), t1 = __fsub_rn(t, s);
    const float e2 = __fadd_rn(__fsub_rn(s, __fsub_rn(t, t1)), __fsub_rn(sh, t1));
    return __fadd_rn(t, __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(esh, __fsub_rn(la, lb))));
}

__device__ __forceinline__ float3 mdiff(const float4* mpos, const float4* mplo, const int4* mnt, int a, int b,
                                        const GcGrid& g) {
    const float4 xa = mpos[a], xb = mpos[b], la = mplo[a], lb = mplo[b];
    const int4 ta = mnt[a], tb = mnt[b];
    return f3(dd_sub1(xa.x, la.x, xb.x, lb.x, (g.pmask & 1) ? ta.x - tb.x : 0, g.L[0]),
              dd_sub1(xa.y, la.y, xb.y, lb.y, (g.pmask & 2) ? ta.y - tb.y : 0, g.L[1]),
              dd_sub1(xa.z, la.z, xb.z, lb.z, (g.pmask & 4) ? ta.z - tb.z : 0, g.L[2]));
}


// Triangle geometry and per-cell area/volume (FP64 sums), one block per cell.
__global__ void fk_mgeo(GcParams p, const SysInfo* __restrict__ sys, const int* __restrict__ cellsys, int ncell,
                        int ntri, const int3* __restrict__ tri, const int2* __restrict__ betri,
                        const float4* __restrict__ mpos, const float4* __restrict__ mplo,
                        const int4* __restrict__ mnt, float* __restrict__ tarea,
                        float4* __restrict__ tnorm, float4* __restrict__ tcen, float* __restrict__ reftarea,
                        double* __restrict__ carea, double* __restrict__ cvol, double* __restrict__ crefarea,
                        double* __restrict__ crefvol, int setup, unsigned* flags) {
    __shared__ double sh[32];
    int c = blockIdx.x;
    int2 be = betri[c];
    if (be.x < 0 || be.y >= ntri || be.y < be.x) {
        if (threadIdx.x == 0) raise_flag(flags, GC_FLAG_BAD_INDEX);
        return;
    }
    const GcGrid& g = sys[cellsys ? cellsys[c] : 0].g;
    int ncp = (int)p.nCP;
    int r = tri[be.x].x - 1;
    if (r < 0 || r >= ncp) {
        if (threadIdx.x == 0) raise_flag(flags, GC_FLAG_BAD_INDEX);
        return;
    }
    float4 xr = mpos[r];
    int4 tr = mnt[r];
    float3 xru = f3(xr.x, xr.y, xr.z);
    if (g.pmask & 1) xru.x += (float)tr.x * g.L[0];
    if (g.pmask & 2) xru.y += (float)tr.y * g.L[1];
    if (g.pmask & 4) xru.z += (float)tr.z * g.L[2];
    double accA = 0.0, accV = 0.0;
    for (int t = be.x + threadIdx.x; t <= be.y; t += blockDim.x) {
        int3 v = tri[t];
        int a = v.x - 1, b = v.y - 1, cc = v.z - 1;
        if (a < 0 || b < 0 || cc < 0 || a >= ncp || b >= ncp || cc >= ncp) {
            raise_flag(flags, GC_FLAG_BAD_INDEX);
            tarea[t] = 0.f;
            continue;
        }
        float3 u1 = mdiff(mpos, mplo, mnt, a, r, g);
        float3 e1 = mdiff(mpos, mplo, mnt, b, a, g), e2 = mdiff(mpos, mplo, mnt, cc, a, g);
        float3 xi = cross3(e1, e2);
        float len = sqrtf(dot3(xi, xi));
        float A = 0.5f * len;
        float3 nrm = len > 0.f ? (1.f / len) * xi : f3(0.f, 0.f, 0.f);
        float3 u2 = u1 + e1, u3 = u1 + e2;
        tarea[t] = A;
        tnorm[t] = make_float4(nrm.x, nrm.y, nrm.z, 0.f);
        float3 cen = xru + (1.f / 3.f) * (u1 + u2 + u3);
        tcen[t] = make_float4(cen.x, cen.y, cen.z, 0.f);
        if (setup) reftarea[t] = A;
        accA += (double)A;
        // volume relative to the cell's first vertex, in FP64
        double v1x = u1.x, v1y = u1.y, v1z = u1.z, v2x = u2.x, v2y = u2.y, v2z = u2.z, v3x = u3.x, v3y = u3.y,
               v3z = u3.z;
        accV += (v1x * (v2y * v3z - v2z * v3y) + v1y * (v2z * v3x - v2x * v3z) + v1z * (v2x * v3y - v2y * v3x)) / 6.0;
    }
    double Ac = block_sum_d(accA, sh);
    double Vc = block_sum_d(accV, sh);
    if (threadIdx.x == 0) {
        carea[c] = Ac;
        cvol[c] = Vc;
        if (setup) {
            crefarea[c] = Ac;
            crefvol[c] = Vc;
        }
    }
}

// Dihedral angle of (i, j, k, l) (GROMACS-manual convention) and gradient.
struct Dih {
    float c, s;
    float3 gi, gj, gk, gl;
};

__device__ __forceinline__ Dih dihedral_f(float3 xi, float3 xj, float3 xk, float3 xl) {
    Dih D;
    float3 rij = xi - xj, rkj = xk - xj, rkl = xk - xl;
    float3 m = cross3(rij, rkj), nn = cross3(rkj, rkl);
    float m2 = dot3(m, m), n2 = dot3(nn, nn), kj2 = dot3(rkj, rkj);
    float kj = sqrtf(kj2);
    float mn = sqrtf(m2 * n2);
    float inv = mn > 0.f ? 1.f / mn : 0.f;
    D.c = dot3(m, nn) * inv;
    D.s = dot3(m, rkl) * kj * inv;
    float im2 = m2 > 0.f ? 1.f / m2 : 0.f, in2 = n2 > 0.f ? 1.f / n2 : 0.f;
    D.gi = (kj * im2) * m;
    D.gl = -(kj * in2) * nn;
    float ikj2 = kj2 > 0.f ? 1.f / kj2 : 0.f;
    float a = dot3(rij, rkj) * ikj2, b = dot3(rkl, rkj) * ikj2;
    D.gj = (a - 1.f) * D.gi - b * D.gl;
    D.gk = (b - 1.f) * D.gl - a * D.gi;
    return D;
}

__device__ __forceinline__ bool edge_ok(int6 E, int ncp, int* a, int* b, int* c, int* d) {
    *a = E.x - 1; *b = E.y - 1; *c = E.z - 1; *d = E.k - 1;
    return *a >= 0 && *b >= 0 && *c >= 0 && *d >= 0 && *a < ncp && *b < ncp && *c < ncp && *d < ncp;
}

__global__ void fk_mech_setup(GcParams p, const SysInfo* __restrict__ sys, const int* __restrict__ msys, int nedge,
                              const int6* __restrict__ edge, const float4* __restrict__ mpos,
                              const float4* __restrict__ mplo, const int4* __restrict__ mnt,
                              const float* __restrict__ shear,
                              const float* __restrict__ bend, float* __restrict__ l0a, float* __restrict__ lmax,
                              float* __restrict__ perlen, float* __restrict__ hpow, float* __restrict__ hbend,
                              float* __restrict__ refang, unsigned* flags) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nedge) return;
    int a, b, c, d;
    if (!edge_ok(edge[e], (int)p.nCP, &a, &b, &c, &d)) {
        raise_flag(flags, GC_FLAG_BAD_INDEX);
        return;
    }
    const GcGrid& g = sys[msys ? msys[a] : 0].g;
    float3 xb = mdiff(mpos, mplo, mnt, b, a, g), xc = mdiff(mpos, mplo, mnt, c, a, g), xd = mdiff(mpos, mplo, mnt, d, a, g);
    float l0 = sqrtf(dot3(xb, xb));
    const float x0 = 1.f / 2.2f, m = 2.f;
    float u = 1.f - x0;
    float kwlc = 1.f / (4.f * u * u) - 0.25f + x0;
    float kmod = x0 / (2.f * u * u * u) - 1.f / (4.f * u * u) + 0.25f;
    float C = 1.7320508075688772f / (4.f * l0) * (kmod + (m + 1.f) * kwlc);
    float mu0 = shear[e];
    float pl = (mu0 > 0.f && p.kT > 0.f) ? p.kT * C / mu0 : 0.f;
    l0a[e] = l0;
    lmax[e] = l0 / x0;
    perlen[e] = pl;
    hpow[e] = pl > 0.f ? (p.kT / pl) * l0 * l0 * kwlc : 0.f;
    hbend[e] = 2.f * bend[e] / 1.7320508075688772f;
    Dih D = dihedral_f(xc, f3(0.f, 0.f, 0.f), xb, xd);
    refang[e] = atan2f(D.s, D.c);
}

// The edge and triangle kernels write the force on each of their vertices
// into a slot of their own (edge e, vertex r of p1..p4: part 4e + r;
// triangle t, vertex r: part 4 nedge + 3t + r); fk_mgather then sums each
// vertex's parts in a fixed order.  No float atomics, so the membrane forces
// -- and with them the whole step -- are the same from run to run.
__device__ __forceinline__ float4 part(float3 f) { return make_float4(f.x, f.y, f.z, 0.f); }

__global__ void fk_medge(GcParams p, const SysInfo* __restrict__ sys, const int* __restrict__ msys, int nedge,
                         const int6* __restrict__ edge, const float4* __restrict__ mpos,
                         const float4* __restrict__ mplo, const int4* __restrict__ mnt, const float* __restrict__ l0a, const float* __restrict__ lmax, const float* __restrict__ perlen,
                         const float* __restrict__ hpow, const float* __restrict__ refang,
                         const float* __restrict__ hbend, float4* __restrict__ parts, unsigned* flags) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nedge) return;
    int a, b, c, d;
    float4* out = parts + 4 * (size_t)e;
    if (!edge_ok(edge[e], (int)p.nCP, &a, &b, &c, &d)) {
        raise_flag(flags, GC_FLAG_BAD_INDEX);
        out[0] = out[1] = out[2] = out[3] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const GcGrid& g = sys[msys ? msys[a] : 0].g;
    float3 z = f3(0.f, 0.f, 0.f);
    float3 xb = mdiff(mpos, mplo, mnt, b, a, g), xc = mdiff(mpos, mplo, mnt, c, a, g), xd = mdiff(mpos, mplo, mnt, d, a, g);
    float3 f1 = z, f2 = z, f3v = z, f4 = z;
    float pl = perlen[e];
    float r = sqrtf(dot3(xb, xb));
    if (pl > 0.f && r > 0.f) {
        const float lm = lmax[e];
        float x = r / lm;
        float fm;
        if (x >= 0.99f) {
            raise_flag(flags, GC_FLAG_STRETCH);
            x = 0.99f;
            float u = 1.f - x;
            fm = -(p.kT / pl) * (1.f / (4.f * u * u) - 0.25f + x) + hpow[e] / (r * r);   // power index 2
        } else {
            // The WLC and POW terms are large and cancel at the rest length
            // l0 (hpow is set so); the same force with the factor r - l0
            // taken out has no cancellation, and is exactly zero at rest:
            // fm = (kT/p)(r - l0) [-(1/lmax)((2 - x - x0) / (4 u^2 u0^2) + 1)
            //                      - kwlc (l0 + r) / r^2],  x0 = l0/lmax,
            // kwlc = 1/(4 u0^2) - 1/4 + x0, u = 1 - x, u0 = 1 - x0.
            const float l0 = l0a[e], x0 = l0 / lm;
            const float u = 1.f - x, u0 = 1.f - x0;
            const float kwlc = 1.f / (4.f * u0 * u0) - 0.25f + x0;
            const float dwlc = (2.f - x - x0) / (4.f * u * u * u0 * u0) + 1.f;
            fm = (p.kT / pl) * (r - l0) * (-dwlc / lm - kwlc * (l0 + r) / (r * r));
        }
        float3 eh = (-1.f / r) * xb;
        f1 += fm * eh;
        f2 -= fm * eh;
    }
    float kb = hbend[e];
    if (kb != 0.f) {
        Dih D = dihedral_f(xc, z, xb, xd);
        float s0, c0;
        sincosf(refang[e], &s0, &c0);
        float dE = kb * (D.s * c0 - D.c * s0);
        f3v -= dE * D.gi;
        f1 -= dE * D.gj;
        f2 -= dE * D.gk;
        f4 -= dE * D.gl;
    }
    out[0] = part(f1);
    out[1] = part(f2);
    out[2] = part(f3v);
    out[3] = part(f4);
}

__global__ void fk_mtri(GcParams p, const SysInfo* __restrict__ sys, const int* __restrict__ cellsys, int ncell,
                        const int2* __restrict__ betri, const int3* __restrict__ tri, const float4* __restrict__ mpos,
                        const float4* __restrict__ mplo, const int4* __restrict__ mnt,
                        const float* __restrict__ reftarea,
                        const float* __restrict__ hl, const float* __restrict__ hg, const float* __restrict__ hv,
                        const double* __restrict__ carea, const double* __restrict__ cvol,
                        const double* __restrict__ crefarea, const double* __restrict__ crefvol,
                        float4* __restrict__ parts, int ntri) {
    // one block per cell: the cell's coefficients are read once
    int c = blockIdx.x;
    int2 be = betri[c];
    if (be.x < 0 || be.y >= ntri || be.y < be.x) return;
    const GcGrid& g = sys[cellsys ? cellsys[c] : 0].g;
    float dA = (float)((carea[c] - crefarea[c]) / crefarea[c]);
    float dV = (float)((cvol[c] - crefvol[c]) / crefvol[c]);
    int ncp = (int)p.nCP;
    for (int t = be.x + threadIdx.x; t <= be.y; t += blockDim.x) {
        int3 v = tri[t];
        int a = v.x - 1, b = v.y - 1, cc = v.z - 1;
        float4* out = parts + 3 * (size_t)t;
        out[0] = out[1] = out[2] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (a < 0 || b < 0 || cc < 0 || a >= ncp || b >= ncp || cc >= ncp) continue;
        float3 x2 = mdiff(mpos, mplo, mnt, b, a, g), x3 = mdiff(mpos, mplo, mnt, cc, a, g);
        float3 xi = cross3(x2, x3);
        float len = sqrtf(dot3(xi, xi));
        if (!(len > 0.f)) continue;
        float At = 0.5f * len;
        float3 nh = (1.f / len) * xi;
        float A0t = reftarea[t];
        float cA = hg[t] * dA + hl[t] * (At - A0t) / A0t;
        float cV = hv[t] * dV * (1.f / 6.f);
        float3 g1 = 0.5f * cross3(nh, x3 - x2), g2 = 0.5f * cross3(nh, -x3), g3 = 0.5f * cross3(nh, x2);
        float3 fv = -cV * xi;
        out[0] = part(fv - cA * g1);
        out[1] = part(fv - cA * g2);
        out[2] = part(fv - cA * g3);
    }
}

// Per vertex: the sum of its edge and triangle parts (in the fixed order of
// the incidence list: its edges, then its triangles, each by index) and its
// area, a third of each incident triangle.
__global__ void fk_mgather(int ncp, int nedge, const int* __restrict__ inc_ptr, const int* __restrict__ inc,
                           const float4* __restrict__ parts, const float* __restrict__ tarea,
                           float4* __restrict__ mforce, float* __restrict__ parea) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= ncp) return;
    float3 f = f3(0.f, 0.f, 0.f);
    float a = 0.f;
    const int tri0 = 4 * nedge;
    for (int q = inc_ptr[v]; q < inc_ptr[v + 1]; ++q) {
        int k = inc[q];
        float4 x = parts[k];
        f += f3(x.x, x.y, x.z);
        if (k >= tri0) a += tarea[(k - tri0) / 3] * (1.f / 3.f);
    }
    mforce[v] = make_float4(f.x, f.y, f.z, 0.f);
    parea[v] = a;
}

// Morse aggregation on membrane-only grids (cubes at least MaxCut wide).
__global__ void fk_mkey(int ncp, const SysInfo* __restrict__ sys, const int* __restrict__ msys,
                        const float4* __restrict__ mpos, int* __restrict__ keys, int* __restrict__ vals) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= ncp) return;
    const SysInfo& S = sys[msys ? msys[v] : 0];
    float4 x = mpos[v];
    keys[v] = S.mcube0 + cube_key(cube_coord(x.x, 0, S.mg), cube_coord(x.y, 1, S.mg), cube_coord(x.z, 2, S.mg), S.mg);
    vals[v] = v;
}

// Membrane positions and vertex areas in aggregation-grid order, so that the
// candidates of a cube are contiguous runs of loads (the id bits in .w say
// which vertex each is).
__global__ void fk_msort(int ncp, const int* __restrict__ order, const float4* __restrict__ mpos,
                         const float* __restrict__ parea, float4* __restrict__ mspos, float* __restrict__ msarea) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ncp) return;
    int v = order[q];
    mspos[q] = mpos[v];
    msarea[q] = parea[v];
}

// Morse force on a vertex at xi (area ai) from a vertex at y (area *aj).
// One Morse pair.  WRAP false: the vertex lies farther than the stencil's
// reach from every periodic face, where the plain difference is the minimum
// image.  De beta (e^2 - e) (a_i + a_j) is 2 De beta (e^2 - e) (a_i + a_j) / 2
// exactly (the factors of two are exact).
template <bool WRAP>
__device__ __forceinline__ void morse_pair(const GcParams& p, const GcGrid& g, float3 xi, float ai, float4 y,
                                           const float* __restrict__ aj, float3& f) {
    const float3 d = WRAP ? min_image(xi, xyz(y), g) : f3(__fsub_rn(xi.x, y.x), __fsub_rn(xi.y, y.y), __fsub_rn(xi.z, y.z));
    float r2 = norm2_rn(d);
    if (r2 >= p.maxcut2 || r2 <= 0.f) return;
    const float inv_r = rsqrt_ftz(r2);
    const float r = r2 * inv_r;
    float ex = __expf(p.beta * (p.r0m - r));
    float fm = p.De * p.beta * (ex * ex - ex) * (ai + *aj);
    f += (fm * inv_r) * d;
}

// Candidates [a, b) of the cube-ordered arrays, four loads in flight.
template <bool WRAP>
__device__ __forceinline__ void morse_run(const GcParams& p, const GcGrid& g, float3 xi, float ai, unsigned a,
                                          unsigned b, const float4* __restrict__ mspos,
                                          const float* __restrict__ msarea, float3& f) {
    unsigned s = a;
    for (; s + 4 <= b; s += 4) {
        float4 y0 = mspos[s], y1 = mspos[s + 1], y2 = mspos[s + 2], y3 = mspos[s + 3];
        morse_pair<WRAP>(p, g, xi, ai, y0, msarea + s, f);
        morse_pair<WRAP>(p, g, xi, ai, y1, msarea + s + 1, f);
        morse_pair<WRAP>(p, g, xi, ai, y2, msarea + s + 2, f);
        morse_pair<WRAP>(p, g, xi, ai, y3, msarea + s + 3, f);
    }
    for (; s < b; ++s) morse_pair<WRAP>(p, g, xi, ai, mspos[s], msarea + s, f);
}

// Morse aggregation by Verlet lists of its own.  When the neighbour lists
// are rebuilt, each membrane vertex lists the vertices of other cells within
// MaxCut + skin (no particle moves more than skin/2 before the next rebuild,
// so every pair within MaxCut until then is listed); each step evaluates
// only the listed pairs.
//
// The list build (fk_mlist) runs eight lanes per vertex in aggregation-grid
// order over the (2R+1)^3 aggregation cubes around it (R = 2 for cubes at
// least MaxCut/2 wide, 1 for cubes at least MaxCut wide): lane k scans the
// rows (dy, dz) k, k + 8, ... of the stencil, skipping rows and cubes
// farther than the cut-off; a first pass counts each lane's candidates, a
// scan places them, and a second pass writes them, so a vertex's list is
// lane 0's candidates, then lane 1's, ... in scan order.  The sort is stable
// and membrane vertices are in id order, so within a cube the candidates
// ascend by id.  RUNS (every cell is one contiguous id range that carries
// its CellTab index, checked at set-up): a cube of the own cell alone is
// skipped from its first and last ids, and otherwise the own cell is one run
// bounded by two binary searches; without RUNS every candidate's CellTab is
// compared.  Both find the same candidates in the same order.
//
// The pass (fk_maggl) runs eight lanes per vertex in membrane order, lane k
// taking the entries k, k + 8, ... of the vertex's list; the group adds its
// eight partial forces by a fixed xor tree.
#ifndef GC_AGG_BS
#define GC_AGG_BS 128
#endif
constexpr int kAggBS = GC_AGG_BS;
constexpr int kAggLanes = 8;   // lanes per vertex (a power of two dividing 32)
// Overflow of the Morse lists inside a captured step (a word of the handle's
// internal overflow flags, never reported as a device status)
constexpr unsigned kMorseFull = 1u << 24;

template <bool RUNS, bool FILL>
__global__ void __launch_bounds__(kAggBS) fk_mlist(int ncp, GcParams p, float cutl, const SysInfo* __restrict__ sys,
                                                   const int* __restrict__ msys, const int* __restrict__ order,
                                                   const unsigned* __restrict__ start,
                                                   const float4* __restrict__ mspos, const int* __restrict__ celltab,
                                                   const int2* __restrict__ cell_verts, unsigned* __restrict__ moff,
                                                   unsigned* __restrict__ mcnt, int* __restrict__ mlist,
                                                   unsigned mcap, unsigned* __restrict__ oflag) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = (int)(t / kAggLanes), k = (int)(t % kAggLanes);
    if (q >= ncp) return;   // whole groups: kAggLanes divides the block
    const int v = order[q];
    const SysInfo& S = sys[msys ? msys[v] : 0];
    const GcGrid& g = S.mg;
    const float3 xi = xyz(mspos[q]);
    const int ci = celltab[v];
    unsigned own_lo = 0, own_hi = 0;   // ids of the vertex's own cell
    if (RUNS) {
        int2 cv = cell_verts[ci];
        own_lo = S.cs + (unsigned)(cv.x - (int)S.m0);
        own_hi = S.cs + (unsigned)(cv.y - (int)S.m0);
    }
    const size_t slot = (size_t)v * kAggLanes + k;
    unsigned w = 0, wend = 0;   // this lane's entries (FILL): after the vertex's offset, the lower lanes' counts
    bool write = true;
    if (FILL) {
        w = moff[v];
        for (int l = 0; l < k; ++l) w += mcnt[(size_t)v * kAggLanes + l];
        wend = w + mcnt[slot];
        if (moff[ncp] > mcap) {   // the lists do not fit: the host grows them
            write = false;
            if (k == 0 && q == 0) atomicOr(oflag, kMorseFull);
        }
    }
    const float cut2 = cutl * cutl;
    unsigned cnt = 0;
    auto take = [&](unsigned s, float3 d) {
        const float r2 = norm2_rn(d);
        if (r2 < cut2) {
            if (FILL) {
                if (write && w < wend) mlist[w] = order[s];
                ++w;
            } else {
                ++cnt;
            }
        }
    };
    const int cx = cube_coord(xi.x, 0, g), cy = cube_coord(xi.y, 1, g), cz = cube_coord(xi.z, 2, g);
    const int R = S.mlr, side = 2 * R + 1;
    // distance from the vertex to the cube dc steps away along an axis (its
    // offset f inside its own cube, cube width w): rows and cubes farther
    // than the cut-off (with a margin far above the rounding) hold no
    // candidate and are not read
    const float wx = 1.f / g.invw[0], wy = 1.f / g.invw[1], wz = 1.f / g.invw[2];
    const float fx = xi.x - (g.origin[0] + (float)cx * wx), fy = xi.y - (g.origin[1] + (float)cy * wy),
                fz = xi.z - (g.origin[2] + (float)cz * wz);
    auto gap = [](int dc, float f, float w) {
        return fmaxf(0.f, dc > 0 ? (float)dc * w - f : (dc < 0 ? f - (float)(dc + 1) * w : 0.f));
    };
    const float cutm = cutl + 1e-3f, cutm2 = cutm * cutm;
    for (int row = k; row < side * side; row += kAggLanes) {
        const int dz = row / side - R, dy = row % side - R;
        const float gz = gap(dz, fz, wz), gy = gap(dy, fy, wy), dyz = gy * gy + gz * gz;
        if (dyz > cutm2) continue;
        const int z = cube_step(cz, dz, 2, g);
        const int y = cube_step(cy, dy, 1, g);
        if (z < 0 || y < 0) continue;
        for (int dx = -R; dx <= R; ++dx) {
            const float gx = gap(dx, fx, wx);
            if (dyz + gx * gx > cutm2) continue;
            int x = cube_step(cx, dx, 0, g);
            if (x < 0) continue;
            int c = S.mcube0 + cube_key(x, y, z, g);
            const unsigned s0 = start[c], s1 = start[c + 1];
            if (s0 == s1) continue;
            auto run = [&](unsigned a, unsigned b) {
                for (unsigned s = a; s < b; ++s) take(s, min_image(xi, xyz(mspos[s]), g));
            };
            if (RUNS) {
                const unsigned id_first = fid(mspos[s0]), id_last = fid(mspos[s1 - 1]);
                if (own_hi < id_first || own_lo > id_last) {
                    run(s0, s1);
                    continue;
                }
                // ids ascend within a cube: a cube of the own cell alone has no candidate
                if (own_lo <= id_first && id_last <= own_hi) continue;
                unsigned lo = s0, hi = s1;
                while (lo < hi) {   // first candidate of the own cell
                    unsigned mid = (lo + hi) >> 1;
                    if (fid(mspos[mid]) < own_lo) lo = mid + 1;
                    else hi = mid;
                }
                const unsigned a = lo;
                hi = s1;
                while (lo < hi) {   // first candidate past it
                    unsigned mid = (lo + hi) >> 1;
                    if (fid(mspos[mid]) <= own_hi) lo = mid + 1;
                    else hi = mid;
                }
                run(s0, a);
                run(lo, s1);
            } else {
                for (unsigned s = s0; s < s1; ++s)
                    if (celltab[order[s]] != ci) take(s, min_image(xi, xyz(mspos[s]), g));
            }
        }
    }
    if (!FILL) {
        // this lane's count, and the vertex's total (the group's eight lanes)
        mcnt[slot] = cnt;
        const unsigned gm = 0xFFu << (threadIdx.x & 24);
#pragma unroll
        for (int o = kAggLanes / 2; o; o >>= 1) cnt += __shfl_xor_sync(gm, cnt, o, kAggLanes);
        if (k == 0) moff[v] = cnt;
    }
}

__global__ void __launch_bounds__(kAggBS) fk_maggl(int ncp, GcParams p, const SysInfo* __restrict__ sys,
                                                   const int* __restrict__ msys, const float4* __restrict__ mpos,
                                                   const float* __restrict__ parea, const unsigned* __restrict__ moff,
                                                   const int* __restrict__ mlist, unsigned mcap,
                                                   float4* __restrict__ magg, float4* __restrict__ mforce) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int v = (int)(t / kAggLanes), k = (int)(t % kAggLanes);
    // whole groups: kAggLanes divides the block.  Lists that did not fit
    // (raised as kMorseFull; the host runs the steps again with room) are
    // not read.
    const bool live = v < ncp && moff[ncp] <= mcap;
    float3 f = f3(0.f, 0.f, 0.f);
    if (live) {
        const GcGrid& g = sys[msys ? msys[v] : 0].mg;
        const float3 xi = xyz(mpos[v]);
        const float ai = parea[v];
        const unsigned b = moff[v], e = moff[v + 1];
        for (unsigned u = b + k; u < e; u += kAggLanes) {
            const int j = mlist[u];
            morse_pair<true>(p, g, xi, ai, mpos[j], parea + j, f);
        }
    }
    // the group's partial forces, added by a fixed tree
#pragma unroll
    for (int o = kAggLanes / 2; o; o >>= 1) {
        f.x += __shfl_xor_sync(0xffffffffu, f.x, o, kAggLanes);
        f.y += __shfl_xor_sync(0xffffffffu, f.y, o, kAggLanes);
        f.z += __shfl_xor_sync(0xffffffffu, f.z, o, kAggLanes);
    }
    if (!live || k != 0) return;
    magg[v] = make_float4(f.x, f.y, f.z, 0.f);
    float4* o = &mforce[v];
    o->x += f.x;   // one thread per vertex, after the deformation kernels
    o->y += f.y;
    o->z += f.z;
}

// Membrane positions at the latest rebuild (the reference positions of the
// displacement check), in membrane order: a restored handle rebuilds its
// Morse lists from them, as the run it continues built them.
__global__ void fk_gather_mref(int ncp, const SysInfo* __restrict__ sys, const int* __restrict__ msys,
                               const int* __restrict__ slot_of, const float4* __restrict__ refpos,
                               float4* __restrict__ mref) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= ncp) return;
    const SysInfo& S = sys[msys ? msys[m] : 0];
    mref[m] = refpos[slot_of[S.cs + (unsigned)(m - (int)S.m0)]];
}

// ---------------------------------------------------------------------------
// Import / export in original (global id) order, for the ids
// [id_base, id_base + count).  Host-side arrays are indexed from id_base.
// ---------------------------------------------------------------------------
// Before set-up the slots are in id order (slot = id); afterwards a load
// replaces the state in the current slot order (the displacement check of
// the next step decides whether the lists need a rebuild).
__global__ void fk_load(int count, unsigned id_base, const SysInfo* __restrict__ sys, int nsys, int keep,
                        const float* __restrict__ x, const float* __restrict__ v, const float* __restrict__ vhalf,
                        const float* __restrict__ f, const int* __restrict__ nt, int* __restrict__ slot_of,
                        float4* __restrict__ pos, float4* __restrict__ plo, float4* __restrict__ vel,
                        float4* __restrict__ vh, float4* __restrict__ force, int4* __restrict__ nthro,
                        float4* __restrict__ mpos, float4* __restrict__ mplo, int4* __restrict__ mnthro) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    unsigned id = id_base + k;
    int i;
    if (keep) {
        i = slot_of[id];
    } else {
        i = (int)id;
        slot_of[id] = i;
    }
    float4 a = make_float4(x[3 * k], x[3 * k + 1], x[3 * k + 2], __uint_as_float(id));
    pos[i] = a;
    float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    plo[i] = z;   // an FP32 position is exact: no low part
    if (v) vel[i] = make_float4(v[3 * k], v[3 * k + 1], v[3 * k + 2], 0.f);
    else if (!keep) vel[i] = z;
    if (vhalf) vh[i] = make_float4(vhalf[3 * k], vhalf[3 * k + 1], vhalf[3 * k + 2], 0.f);
    else if (!keep) vh[i] = z;
    if (f) force[i] = make_float4(f[3 * k], f[3 * k + 1], f[3 * k + 2], 0.f);
    else if (!keep) force[i] = z;
    int4 t = nt ? make_int4(nt[3 * k], nt[3 * k + 1], nt[3 * k + 2], 0) : (keep ? nthro[i] : make_int4(0, 0, 0, 0));
    if (nt || !keep) nthro[i] = t;
    if (mpos) {
        const SysInfo& S = sys[find_sys(sys, nsys, id)];
        if (id >= S.cs) {
            mpos[S.m0 + id - S.cs] = a;
            mplo[S.m0 + id - S.cs] = z;
            mnthro[S.m0 + id - S.cs] = t;
        }
    }
}

// Membrane-ordered positions from the slots (set-up).
__global__ void fk_gather_mpos(int ncp, const SysInfo* __restrict__ sys, const int* __restrict__ msys,
                               const int* __restrict__ slot_of, const float4* __restrict__ pos,
                               const int4* __restrict__ nthro, const float4* __restrict__ plo,
                               float4* __restrict__ mpos, float4* __restrict__ mplo, int4* __restrict__ mnthro) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= ncp) return;
    const SysInfo& S = sys[msys ? msys[m] : 0];
    int i = slot_of[S.cs + (unsigned)(m - (int)S.m0)];
    mpos[m] = pos[i];
    mplo[m] = plo[i];
    mnthro[m] = nthro[i];
}

__global__ void fk_store(int count, unsigned id_base, GcParams p, const int* __restrict__ slot_of,
                         const float4* __restrict__ pos, const float4* __restrict__ vel,
                         const float4* __restrict__ vh, const float4* __restrict__ force,
                         const float2* __restrict__ dp, const int4* __restrict__ nthro, float* __restrict__ x,
                         float* __restrict__ v, float* __restrict__ rho, float* __restrict__ press,
                         float* __restrict__ f, float* __restrict__ vhalf, int* __restrict__ nt) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    int i = slot_of[id_base + k];
    if (x) { float4 a = pos[i]; x[3 * k] = a.x; x[3 * k + 1] = a.y; x[3 * k + 2] = a.z; }
    if (v) { float4 b = vel[i]; v[3 * k] = b.x; v[3 * k + 1] = b.y; v[3 * k + 2] = b.z; }
    if (vhalf) { float4 b = vh[i]; vhalf[3 * k] = b.x; vhalf[3 * k + 1] = b.y; vhalf[3 * k + 2] = b.z; }
    if (f) { float4 b = force[i]; f[3 * k] = b.x; f[3 * k + 1] = b.y; f[3 * k + 2] = b.z; }
    if (nt) { int4 b = nthro[i]; nt[3 * k] = b.x; nt[3 * k + 1] = b.y; nt[3 * k + 2] = b.z; }
    if (rho || press) {
        float2 q = dp[i];
        if (rho) rho[k] = p.mass / q.x;
        if (press) press[k] = q.y / (q.x * q.x);
    }
}

// membrane outputs: vertices [m0, m0 + ncp), triangles [t0, t0 + ntri)
__global__ void fk_store_cells(int ncp, int m0, int ntri, int t0, const float4* __restrict__ mforce,
                               const float4* __restrict__ magg, const float* __restrict__ parea,
                               const float4* __restrict__ tnorm, const float4* __restrict__ tcen,
                               float* __restrict__ defforce, float* __restrict__ aggforce, float* __restrict__ pararea,
                               float* __restrict__ trinor, float* __restrict__ tricen, int have_agg) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ncp) {
        float4 a = have_agg ? magg[m0 + i] : make_float4(0.f, 0.f, 0.f, 0.f);
        float4 m = mforce[m0 + i];
        if (defforce) { defforce[3 * i] = m.x - a.x; defforce[3 * i + 1] = m.y - a.y; defforce[3 * i + 2] = m.z - a.z; }
        if (aggforce) { aggforce[3 * i] = a.x; aggforce[3 * i + 1] = a.y; aggforce[3 * i + 2] = a.z; }
        if (pararea) pararea[i] = parea[m0 + i];
    }
    if (i < ntri) {
        float4 b = tnorm[t0 + i], c = tcen[t0 + i];
        if (trinor) { trinor[3 * i] = b.x; trinor[3 * i + 1] = b.y; trinor[3 * i + 2] = b.z; }
        if (tricen) { tricen[3 * i] = c.x; tricen[3 * i + 1] = c.y; tricen[3 * i + 2] = c.z; }
    }
}

__global__ void fk_cast_cells(int ncell, int c0, const double* __restrict__ a, const double* __restrict__ v,
                              float* __restrict__ area, float* __restrict__ vol) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    if (area) area[c] = (float)a[c0 + c];
    if (vol) vol[c] = (float)v[c0 + c];
}

__global__ void fk_count_stats(int n, const int* __restrict__ cnt, unsigned long long* __restrict__ sum,
                               int* __restrict__ mx) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int c = i < n ? cnt[i] : 0;
    int m = c;
    unsigned long long s = (unsigned long long)c;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(sum, s);
        atomicMax(mx, m);
    }
}




// system index of the slots (set-up, slot = id)
__global__ void fk_fill_sys(int n, const SysInfo* __restrict__ sys, int nsys, int* __restrict__ sysid) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) sysid[i] = find_sys(sys, nsys, (unsigned)i);
}

}  // namespace gcf



namespace gcf {


int stage_bytes(GcFused* f, size_t bytes) {
    if (f->stage_bytes >= bytes) return GC_OK;
    if (f->stage) cudaFree(f->stage);
    f->stage = nullptr;
    f->stage_bytes = 0;
    GC_CUDA(cudaMalloc(&f->stage, bytes), "fused: staging buffer");
    f->stage_bytes = bytes;
    return GC_OK;
}

void drop_graphs(GcFused* f) {
    for (int d = 0; d < 2; ++d) {
        if (f->gexec[d]) cudaGraphExecDestroy(f->gexec[d]);
        if (f->cg[d]) cudaGraphDestroy(f->cg[d]);
        f->gexec[d] = nullptr;
        f->cg[d] = nullptr;
    }
    f->graph_dirty = true;
}

int alloc_list(GcFused* f, int cap) {
    size_t rows = (size_t)((f->n + 31) / 32) * 32;
    size_t need = rows * (size_t)cap;
    if (!f->nbr || need > f->nbr_elems) {
        if (f->nbr) cudaFree(f->nbr);
        f->nbr = nullptr;
        f->nbr_elems = 0;
        GC_CUDA(cudaMalloc(&f->nbr, need * sizeof(int)), "fused: neighbour lists");
        f->nbr_elems = need;
        drop_graphs(f);
    }
    f->mw = (cap + 31) / 32;
    if (f->compact) {
        size_t mneed = rows * (size_t)f->mw;
        if (!f->cmask || mneed > f->cmask_elems) {
            if (f->cmask) cudaFree(f->cmask);
            f->cmask = nullptr;
            f->cmask_elems = 0;
            GC_CUDA(cudaMalloc(&f->cmask, mneed * sizeof(unsigned)), "fused: masks");
            f->cmask_elems = mneed;
            drop_graphs(f);
        }
    }
    if (f->cap != cap) drop_graphs(f);
    f->cap = cap;
    return GC_OK;
}

int ensure_sort_bufs(GcFused* f) {
    int nn = f->n > f->ncp ? f->n : f->ncp;
    int KK = f->K > f->Kagg ? f->K : f->Kagg;
    if (f->sortmem && nn <= f->sort_n && KK <= f->sort_K) return GC_OK;
    if (f->sortmem) cudaFree(f->sortmem);
    f->sortmem = nullptr;
    size_t bytes = gc_sort_bufs_bytes(nn, KK);
    GC_CUDA(cudaMalloc(&f->sortmem, bytes), "fused: sort temporaries");
    f->sortmem_bytes = bytes;
    f->sort_n = nn;
    f->sort_K = KK;
    gc_sort_bufs_carve(f->sortmem, nn, KK, &f->sb);
    drop_graphs(f);
    return GC_OK;
}

int ensure_agg_sort_bufs(GcFused* f) {
    if (!f->have_agg || f->ncp <= 0) return GC_OK;
    if (f->sortmem_agg && f->ncp <= f->sort_agg_n && f->Kagg <= f->sort_agg_K) return GC_OK;
    if (f->sortmem_agg) cudaFree(f->sortmem_agg);
    f->sortmem_agg = nullptr;
    GC_CUDA(cudaMalloc(&f->sortmem_agg, gc_sort_bufs_bytes(f->ncp, f->Kagg)), "fused: aggregation sort");
    f->sort_agg_n = f->ncp;
    f->sort_agg_K = f->Kagg;
    gc_sort_bufs_carve(f->sortmem_agg, f->ncp, f->Kagg, &f->sb_agg);
    drop_graphs(f);
    return GC_OK;
}

// The Morse lists of the current membrane positions `mp` (membrane order):
// sort the vertices into the aggregation cubes, count each lane's
// candidates within MaxCut + skin, scan, write.  From the host (`host`) the
// entries grow to fit, with room for the rebuilds of captured steps; inside
// a captured step a list that does not fit raises kMorseFull in the
// overflow flags and the host runs the steps again with room.
int build_morse_lists(GcFused* f, cudaStream_t st, const float4* mp, bool host) {
    if (!f->have_agg || f->ncp <= 0 || f->ncell <= 0) return GC_OK;
    const int ncp = f->ncp;
    const size_t nl = (size_t)ncp + 1;   // per vertex, scanned into offsets
    if (host && !f->moff) {
        GC_CUDA(cudaMalloc(&f->moff, nl * sizeof(unsigned)), "fused: Morse lists");
        GC_CUDA(cudaMalloc(&f->mcnt, (size_t)ncp * kAggLanes * sizeof(unsigned)), "fused: Morse lists");
        GC_CUDA(cudaMalloc(&f->mscan, gc_scan_blocks((int)nl) * sizeof(unsigned)), "fused: Morse lists");
        drop_graphs(f);
    }
    if (!f->moff) return gc_fail(GC_ESTATE, "fused: Morse lists not allocated");
    fk_mkey<<<gc_blocks(ncp, f->block), f->block, 0, st>>>(ncp, f->dsys, f->msys, mp, f->mkeys, f->mvals);
    GC_CHECK_LAUNCH("fused: aggregation keys");
    GC_TRY(gc_counting_sort_bufs(ncp, f->Kagg, f->mkeys, f->mvals, f->sb_agg, f->flags, st));
    fk_msort<<<gc_blocks(ncp, f->block), f->block, 0, st>>>(ncp, f->mvals, mp, f->parea, f->mspos, f->msarea);
    GC_CHECK_LAUNCH("fused: aggregation order");
    const float cutl = f->p.maxcut + f->skin;
    const int nba = gc_blocks((int)((long long)ncp * kAggLanes), kAggBS);
    GC_CUDA(cudaMemsetAsync(f->moff + (nl - 1), 0, sizeof(unsigned), st), "fused: Morse lists");
    auto pass = [&](auto fill) -> int {
        constexpr bool F = decltype(fill)::value;
        if (f->agg_runs)
            fk_mlist<true, F><<<nba, kAggBS, 0, st>>>(ncp, f->p, cutl, f->dsys, f->msys, f->mvals, f->sb_agg.cnt,
                                                      f->mspos, f->celltab, f->cell_verts, f->moff, f->mcnt,
                                                      f->mlist, (unsigned)f->mcap, f->oflag);
        else
            fk_mlist<false, F><<<nba, kAggBS, 0, st>>>(ncp, f->p, cutl, f->dsys, f->msys, f->mvals, f->sb_agg.cnt,
                                                       f->mspos, f->celltab, f->cell_verts, f->moff, f->mcnt,
                                                       f->mlist, (unsigned)f->mcap, f->oflag);
        GC_CHECK_LAUNCH("fused: Morse lists");
        return GC_OK;
    };
    GC_TRY(pass(std::false_type{}));
    GC_TRY(gc_scan_exclusive(f->moff, (int)nl, f->mscan, st));
    if (host) {
        unsigned total = 0;
        GC_CUDA(cudaMemcpyAsync(&total, f->moff + (nl - 1), sizeof(unsigned), cudaMemcpyDeviceToHost, st),
                "fused: Morse lists");
        GC_CUDA(cudaStreamSynchronize(st), "fused: Morse lists");
        if ((size_t)(f->mroom * total) + f->mextra > f->mcap || !f->mlist) {
            // room for the lists to grow in the rebuilds of captured steps
            const size_t want = (size_t)((f->mroom + f->mslack) * total) + f->mextra;
            if (f->mlist) cudaFree(f->mlist);
            f->mlist = nullptr;
            f->mcap = 0;
            GC_CUDA(cudaMalloc(&f->mlist, want * sizeof(int)), "fused: Morse lists");
            f->mcap = want;
            drop_graphs(f);
        }
    }
    return pass(std::true_type{});
}

// The Morse lists as the latest rebuild built them: from the reference
// positions of the displacement check (a restore).
int build_morse_lists_from_ref(GcFused* f, cudaStream_t st) {
    if (!f->have_agg || f->ncp <= 0 || f->ncell <= 0) return GC_OK;
    if (!f->mref) GC_CUDA(cudaMalloc(&f->mref, (size_t)f->ncp * sizeof(float4)), "fused: Morse lists");
    fk_gather_mref<<<gc_blocks(f->ncp, 256), 256, 0, st>>>(f->ncp, f->dsys, f->msys, f->slot_of, f->refpos, f->mref);
    GC_CHECK_LAUNCH("fused: reference membrane positions");
    return build_morse_lists(f, st, f->mref, true);
}

// Per-system list grids (cubes at least rc + skin wide) and aggregation
// grids, their global cube offsets, and the device copy of the table.
int build_grids(GcFused* f) {
    if (!f->lists) {
        // the pair tiles need at least three cubes of rc + skin along every
        // periodic axis; a smaller box takes per-particle lists over
        // half-width cells instead
        for (int s = 0; s < f->nsys; ++s) {
            const GcSystemDesc& d = f->desc[s];
            const float cut = d.consts.CutRadius + f->skin;
            for (int a = 0; a < 3; ++a)
                if ((d.periodic_mask >> a) & 1) {
                    const double L = (double)d.bbox[2 * a + 1] - (double)d.bbox[2 * a];
                    if (floor(L / ((double)cut * (1.0 + 1e-4))) < 3.0) f->lists = true;
                }
        }
        if (f->lists) drop_graphs(f);
    }
    int K = 0, Kagg = 0;
    for (int s = 0; s < f->nsys; ++s) {
        SysInfo& S = f->hsys[s];
        const GcSystemDesc& d = f->desc[s];
        // half-width cells (a 5x5x5 stencil scans ~40 % fewer candidates than
        // 3x3x3 cubes) wherever every periodic axis has at least 5 of them
        const float cut = d.consts.CutRadius + f->skin;
        S.lr = 2;
        if (!f->lists || gc_build_grid(d.bbox, 0.5f * cut, d.periodic_mask, &S.g) != GC_OK ||
            ((d.periodic_mask & 1) && S.g.n[0] < 5) || ((d.periodic_mask & 2) && S.g.n[1] < 5) ||
            ((d.periodic_mask & 4) && S.g.n[2] < 5)) {
            S.lr = 1;
            GC_TRY(gc_build_grid(d.bbox, cut, d.periodic_mask, &S.g));
        }
        for (int a = 0; a < 3; ++a) S.invL[a] = 1.f / S.g.L[a];
        S.cube0 = K;
        K += S.g.ncells;
        if (f->have_agg) {
            // the same for the aggregation grid: half-width cubes cut the
            // candidates of the Morse pass by ~40 %
            S.mlr = 2;
            if (gc_build_grid(d.bbox, 0.5f * f->p.maxcut, d.periodic_mask, &S.mg) != GC_OK ||
                ((d.periodic_mask & 1) && S.mg.n[0] < 5) || ((d.periodic_mask & 2) && S.mg.n[1] < 5) ||
                ((d.periodic_mask & 4) && S.mg.n[2] < 5)) {
                S.mlr = 1;
                GC_TRY(gc_build_grid(d.bbox, f->p.maxcut, d.periodic_mask, &S.mg));
            }
            S.mcube0 = Kagg;
            Kagg += S.mg.ncells;
        } else {
            S.mg = S.g;
            S.mlr = S.lr;
            S.mcube0 = 0;
        }
    }
    f->K = K;
    f->Kagg = Kagg;
    if (f->dsys)
        GC_CUDA(cudaMemcpyAsync(f->dsys, f->hsys.data(), sizeof(SysInfo) * f->nsys, cudaMemcpyHostToDevice, f->st),
                "fused: system table");
    GC_TRY(ensure_sort_bufs(f));
    GC_TRY(ensure_agg_sort_bufs(f));
    GC_TRY(tiles_grid(f));
    drop_graphs(f);
    return GC_OK;
}

int sync_dstep(GcFused* f) {
    long long v = f->step;
    GC_CUDA(cudaMemcpyAsync(f->dstep, &v, sizeof(v), cudaMemcpyHostToDevice, f->st), "fused: step counter");
    GC_CUDA(cudaStreamSynchronize(f->st), "fused: step counter");
    return GC_OK;
}

const SysInfo& s0(GcFused* f) { return f->hsys[0]; }

// Distance from a periodic face beyond which a particle's listed pairs need
// no image shift: rc + 2 skin (each particle moves less than skin/2 between
// rebuilds), with 1 % of rc to spare.
float wrap_margin(const GcFused* f) { return 1.01f * f->p.rc + 2.f * f->skin; }

// Re-sort and list build on the host-driven path (swaps the slot arrays;
// grows the lists and rebuilds when a particle had more neighbours than the
// lists hold).
// List capacity after an overflow: the longest list the build wanted
// (f->h->need, read back with the overflow flag) with a quarter and 16 to
// spare, and at least at_least; a multiple of 8.
int grown_capacity(const GcFused* f, int at_least) {
    const int want = (int)(1.25 * f->h->need) + 16;
    return ((want > at_least ? want : at_least) + 7) & ~7;
}

// Turns a handle from pair tiles to per-particle lists (a cube holds more
// particles than the tiles take): half-width cells where they fit, lists
// for every slot.
int switch_to_lists(GcFused* f) {
    f->lists = true;
    GC_TRY(build_grids(f));
    GC_TRY(alloc_list(f, f->cap));
    drop_graphs(f);
    return GC_OK;
}

int rebuild_lists(GcFused* f) {
    const int n = f->n;
    const int nb = gc_blocks(n, f->block);
    cudaStream_t st = f->st;
    fk_cellkey<<<nb, f->block, 0, st>>>(n, f->dsys, f->a.sys, f->a.pos, f->keys, f->vals);
    GC_CHECK_LAUNCH("fused: cube keys");
    GC_TRY(gc_counting_sort_bufs(n, f->K, f->keys, f->vals, f->sb, f->flags, st));
    fk_permute<<<nb, f->block, 0, st>>>(n, f->dsys, f->vals, f->a, f->b, f->refpos, f->slot_of, f->ddpos);
    GC_CHECK_LAUNCH("fused: permute");
    std::swap(f->a, f->b);
    drop_graphs(f);   // captured steps are bound to the old slot arrays
    if (!f->lists) {
        GC_TRY(wall_lists(f, st, f->a.pos, true));
        GC_CUDA(cudaMemsetAsync(f->oflag, 0, sizeof(unsigned), st), "fused: flags");
        GC_TRY(tiles_build(f, st, f->a.pos, true));
        if (f->h->oflag & GC_FLAG_TILE_FULL) {
            // a cube holds more particles than the tiles take: per-particle
            // lists from now on (another grid, so sort again)
            GC_TRY(switch_to_lists(f));
            return rebuild_lists(f);
        }
        GC_TRY(build_morse_lists(f, st, f->mpos, true));
        f->rebuilds++;
        return GC_OK;
    }
    float cut = f->p.rc + f->skin;
    float cut2 = cut * cut;
    for (int attempt = 0; attempt < 4; ++attempt) {
        GC_CUDA(cudaMemsetAsync(f->oflag, 0, sizeof(unsigned), st), "fused: flags");
        GC_CUDA(cudaMemsetAsync(f->need, 0, sizeof(int), st), "fused: flags");
        fk_build_list<<<nb, f->block, 0, st>>>(n, f->dsys, f->a.sys, f->a.pos, f->sb.cnt, f->nbr, f->cnt, f->cap,
                                              cut2, f->oflag, f->need, 0);
        GC_CHECK_LAUNCH("fused: build lists");
        GC_CUDA(cudaMemcpyAsync(&f->h->oflag, f->oflag, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "fused: flags");
        GC_CUDA(cudaMemcpyAsync(&f->h->need, f->need, sizeof(int), cudaMemcpyDeviceToHost, st), "fused: flags");
        GC_CUDA(cudaStreamSynchronize(st), "fused: flags");
        if (!(f->h->oflag & GC_FLAG_CELL_OVERFLOW)) break;
        if (attempt == 3) return gc_fail(GC_EDEVICE, "fused: neighbour lists overflow %d entries", f->cap);
        // a particle had more neighbours than the list holds: grow to the
        // longest list wanted (with room) and rebuild
        GC_TRY(alloc_list(f, grown_capacity(f, 2 * f->cap)));
    }
    GC_TRY(build_morse_lists(f, st, f->mpos, true));
    f->rebuilds++;
    return GC_OK;
}

cudaEvent_t prof_event(GcFused* f) {
    if (f->ev_used == f->ev.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        f->ev.push_back(e);
    }
    return f->ev[f->ev_used++];
}

void prof_mark(GcFused* f, cudaStream_t st) {
    if (!f->profile) return;
    cudaEvent_t e = prof_event(f);
    if (e) cudaEventRecord(e, st);
}

// ---- launches shared by the host-driven and the captured step --------------

int launch_integrate(GcFused* f, cudaStream_t st, const GcParams& p) {
    const int n = f->n, nb = gc_blocks(n, f->block);
    float hs = 0.5f * f->skin * 0.99f;
    if (f->ens)
        fk_integrate<true><<<nb, f->block, 0, st>>>(n, p, s0(f), f->dsys, f->a.sys, f->a.pos, f->a.vel, f->a.vh,
                                                     f->a.vpred, f->a.force, f->a.plo, f->refpos, f->a.nthro,
                                                     hs * hs, f->rebuild, f->mpos, f->mplo, f->mnthro, f->flags,
                                                     f->ddpos);
    else
        fk_integrate<false><<<nb, f->block, 0, st>>>(n, p, s0(f), f->dsys, f->a.sys, f->a.pos, f->a.vel, f->a.vh,
                                                      f->a.vpred, f->a.force, f->a.plo, f->refpos, f->a.nthro,
                                                      hs * hs, f->rebuild, f->mpos, f->mplo, f->mnthro, f->flags,
                                                     f->ddpos);
    GC_CHECK_LAUNCH("fused: integrate");
    return GC_OK;
}

int launch_density(GcFused* f, cudaStream_t st, const GcParams& p, bool mark) {
    if (!f->lists) return launch_tile_density(f, st, p, false);
    const int n = f->n, nb = gc_blocks(n, f->block);
    unsigned* cm = mark && f->compact ? f->cmask : nullptr;
    int* cc = mark && f->compact ? f->ccnt : nullptr;
    if (f->ens) {
        if (f->has_b1)
            fk_density<true, true><<<nb, f->block, 0, st>>>(n, p, s0(f), f->dsys, f->a.sys, f->a.pos, f->a.vpred,
                                                            f->a.vh, f->dp, f->nbr, f->cnt, f->cap, cm, f->mw, cc,
                                                            wrap_margin(f));
        else
            fk_density<true, false><<<nb, f->block, 0, st>>>(n, p, s0(f), f->dsys, f->a.sys, f->a.pos, f->a.vpred,
                                                             f->a.vh, f->dp, f->nbr, f->cnt, f->cap, cm, f->mw, cc,
                                                             wrap_margin(f));
    } else {
        if (f->has_b1)
            fk_density<false, true><<<nb, f->block, 0, st>>>(n, p, s0(f), f->dsys, f->a.sys, f->a.pos, f->a.vpred,
                                                             f->a.vh, f->dp, f->nbr, f->cnt, f->cap, cm, f->mw, cc,
                                                             wrap_margin(f));
        else
            fk_density<false, false><<<nb, f->block, 0, st>>>(n, p, s0(f), f->dsys, f->a.sys, f->a.pos, f->a.vpred,
                                                              f->a.vh, f->dp, f->nbr, f->cnt, f->cap, cm, f->mw, cc,
                                                              wrap_margin(f));
    }
    GC_CHECK_LAUNCH("fused: density");
    return GC_OK;
}

int launch_membranes(GcFused* f, cudaStream_t st, const GcParams& p) {
    if (f->ncell <= 0) return GC_OK;
    fk_mgeo<<<f->ncell, 256, 0, st>>>(p, f->dsys, f->cellsys, f->ncell, f->ntri, f->tri, f->betri, f->mpos, f->mplo,
                                      f->mnthro,
                                     f->tarea, f->tnorm, f->tcen, f->reftarea, f->carea, f->cvol, f->crefarea,
                                     f->crefvol, 0, f->flags);
    GC_CHECK_LAUNCH("fused: membrane geometry");
    fk_medge<<<gc_blocks(f->nedge, f->block), f->block, 0, st>>>(p, f->dsys, f->msys, f->nedge, f->edge, f->mpos,
                                                                 f->mplo, f->mnthro, f->l0, f->lmax, f->perlen, f->hpow, f->refang,
                                                                 f->hbend, f->mparts, f->flags);
    GC_CHECK_LAUNCH("fused: membrane edges");
    fk_mtri<<<f->ncell, 256, 0, st>>>(p, f->dsys, f->cellsys, f->ncell, f->betri, f->tri, f->mpos, f->mplo,
                                      f->mnthro,
                                     f->reftarea, f->hl, f->hg, f->hv, f->carea, f->cvol, f->crefarea, f->crefvol,
                                     f->mparts + 4 * (size_t)f->nedge, f->ntri);
    GC_CHECK_LAUNCH("fused: membrane triangles");
    fk_mgather<<<gc_blocks(f->ncp, f->block), f->block, 0, st>>>(f->ncp, f->nedge, f->inc_ptr, f->inc, f->mparts,
                                                                 f->tarea, f->mforce, f->parea);
    GC_CHECK_LAUNCH("fused: membrane forces per vertex");
    if (f->have_agg) {
        // the listed pairs (the lists are built with the neighbour lists)
        const int nba = gc_blocks((int)((long long)f->ncp * kAggLanes), kAggBS);
        fk_maggl<<<nba, kAggBS, 0, st>>>(f->ncp, p, f->dsys, f->msys, f->mpos, f->parea, f->moff, f->mlist,
                                         (unsigned)f->mcap, f->magg, f->mforce);
        GC_CHECK_LAUNCH("fused: aggregation");
    }
    return GC_OK;
}

template <bool COMPACT, bool HALFV, bool NOISE, bool B1>
void force_launch_n(GcFused* f, cudaStream_t st, const GcParams& p, int drive) {
    const int n = f->n, nb = gc_blocks(n, f->block);
    const float4* mf = f->ncell > 0 ? f->mforce : nullptr;
    const int* c = COMPACT ? f->ccnt : f->cnt;
    const unsigned* cm = COMPACT ? f->cmask : nullptr;
    const unsigned* nk = f->ens || f->capturing ? f->nkey : nullptr;
    if (f->ens)
        fk_force<COMPACT, true, HALFV, NOISE, B1><<<nb, f->block, 0, st>>>(
            n, p, s0(f), f->dsys, f->a.sys, nk, f->a.pos, f->a.vpred, f->a.vh, f->dp, f->a.force, f->a.vel,
            f->nbr, c, f->cap, cm, f->mw, mf, drive, f->vph, wrap_margin(f));
    else
        fk_force<COMPACT, false, HALFV, NOISE, B1><<<nb, f->block, 0, st>>>(
            n, p, s0(f), f->dsys, f->a.sys, nk, f->a.pos, f->a.vpred, f->a.vh, f->dp, f->a.force, f->a.vel,
            f->nbr, c, f->cap, cm, f->mw, mf, drive, f->vph, wrap_margin(f));
}

template <bool COMPACT, bool HALFV>
void force_launch(GcFused* f, cudaStream_t st, const GcParams& p, int drive) {
    const bool noise = p.noise_pref > 0.f;
    if (f->has_b1) {
        if (noise) force_launch_n<COMPACT, HALFV, true, true>(f, st, p, drive);
        else force_launch_n<COMPACT, HALFV, false, true>(f, st, p, drive);
    } else {
        if (noise) force_launch_n<COMPACT, HALFV, true, false>(f, st, p, drive);
        else force_launch_n<COMPACT, HALFV, false, false>(f, st, p, drive);
    }
}

int launch_force(GcFused* f, cudaStream_t st, const GcParams& p, int drive) {
    if (!f->lists) return launch_tile_force(f, st, p, drive, false);
    if (f->halfv) {
        fk_pack_vel<<<gc_blocks(f->n, 256), 256, 0, st>>>(f->n, f->a.vpred, f->vph);
        GC_CHECK_LAUNCH("fused: pack velocities");
        if (f->compact) force_launch<true, true>(f, st, p, drive);
        else force_launch<false, true>(f, st, p, drive);
    } else {
        if (f->compact) force_launch<true, false>(f, st, p, drive);
        else force_launch<false, false>(f, st, p, drive);
    }
    GC_CHECK_LAUNCH("fused: force");
    return GC_OK;
}

bool any_bound2(const GcFused* f) {
    for (const SysInfo& S : f->hsys)
        if (S.fl > S.b2) return true;
    return false;
}

int launch_wallvel(GcFused* f, cudaStream_t st, const GcParams& p) {
    if (!any_bound2(f)) return GC_OK;
    const int n = f->n, nb = gc_blocks(n, f->block);
    if (f->ens)
        fk_wallvel<true><<<nb, f->block, 0, st>>>(n, p, s0(f), f->dsys, f->a.sys, f->a.pos, f->a.vel, f->a.vh, f->nbr,
                                                   f->cnt, f->cap);
    else
        fk_wallvel<false><<<nb, f->block, 0, st>>>(n, p, s0(f), f->dsys, f->a.sys, f->a.pos, f->a.vel, f->a.vh,
                                                    f->nbr, f->cnt, f->cap);
    GC_CHECK_LAUNCH("fused: wall velocity");
    return GC_OK;
}

int launch_step_begin(GcFused* f, cudaStream_t st) {
    fk_step_begin<<<1, 256, 0, st>>>(f->nsys, f->dsys, f->dstep, f->nkey, f->rebuild);
    GC_CHECK_LAUNCH("fused: step prologue");
    return GC_OK;
}

// The membrane kernels of a step on stream `ms`, after the integration that
// `st` has queued; join_membranes makes `st` wait for them.
int fork_membranes(GcFused* f, cudaStream_t st, cudaStream_t ms, const GcParams& p) {
    if (f->ncell <= 0) return GC_OK;
    GC_CUDA(cudaEventRecord(f->ev_fork, st), "fused: fork");
    GC_CUDA(cudaStreamWaitEvent(ms, f->ev_fork, 0), "fused: fork");
    GC_TRY(launch_membranes(f, ms, p));
    GC_CUDA(cudaEventRecord(f->ev_join, ms), "fused: join");
    return GC_OK;
}

int join_membranes(GcFused* f, cudaStream_t st) {
    if (f->ncell <= 0) return GC_OK;
    GC_CUDA(cudaStreamWaitEvent(st, f->ev_join, 0), "fused: join");
    return GC_OK;
}

int early_store(GcFused* f, cudaStream_t st, int phase);

// One step on the host-driven path: the host reads the rebuild flag.
int one_step(GcFused* f, int drive) {
    cudaStream_t st = f->st;
    f->step += 1;
    GcParams p = f->p;
    p.noise_key = noise_key(p.seed, (uint64_t)f->step);
    if (f->ens) GC_TRY(launch_step_begin(f, st));
    else GC_CUDA(cudaMemsetAsync(f->rebuild, 0, sizeof(int), st), "fused: flag");
    GC_TRY(launch_integrate(f, st, p));
    GC_CUDA(cudaMemcpyAsync(&f->h->rebuild, f->rebuild, sizeof(int), cudaMemcpyDeviceToHost, st), "fused: flag");
    GC_CUDA(cudaStreamSynchronize(st), "fused: flag");
    if (f->h->rebuild) GC_TRY(rebuild_lists(f));
    // the membrane passes beside the density pass (after a rebuild, which
    // writes the Morse lists they read)
    GC_TRY(fork_membranes(f, st, f->mst, p));
    if (f->early) GC_TRY(f->early(f, st, 0));
    prof_mark(f, st);
    GC_TRY(launch_density(f, st, p, true));
    if (f->early) GC_TRY(f->early(f, st, 1));
    prof_mark(f, st);
    GC_TRY(join_membranes(f, st));
    if (f->early) GC_TRY(f->early(f, st, 2));
    prof_mark(f, st);
    GC_TRY(launch_force(f, st, p, drive));
    prof_mark(f, st);
    GC_TRY(launch_wallvel(f, st, p));
    if (f->early) GC_TRY(f->early(f, st, 3));
    f->steps++;
    return GC_OK;
}

// ---- captured steps -------------------------------------------------------

// The rebuild of a captured step: the same sort and list build as
// rebuild_lists, permuting into the spare arrays and copying back, with the
// list capacity fixed (an overflow raises oflag, which the host checks after
// the call's steps and recovers from).
int launch_rebuild_body(GcFused* f, cudaStream_t st) {
    const int n = f->n, nb = gc_blocks(n, f->block);
    fk_cellkey<<<nb, f->block, 0, st>>>(n, f->dsys, f->a.sys, f->a.pos, f->keys, f->vals);
    GC_CHECK_LAUNCH("fused: cube keys");
    GC_TRY(gc_counting_sort_bufs(n, f->K, f->keys, f->vals, f->sb, f->flags, st));
    fk_permute<<<nb, f->block, 0, st>>>(n, f->dsys, f->vals, f->a, f->b, f->refpos, f->slot_of, f->ddpos);
    GC_CHECK_LAUNCH("fused: permute");
    fk_copy_slots<<<nb, f->block, 0, st>>>(n, f->b, f->a);
    GC_CHECK_LAUNCH("fused: copy slots");
    if (!f->lists) {
        GC_TRY(wall_lists(f, st, f->a.pos, false));
        GC_TRY(tiles_build(f, st, f->a.pos, false));
        return build_morse_lists(f, st, f->mpos, false);
    }
    float cut = f->p.rc + f->skin;
    fk_build_list<<<nb, f->block, 0, st>>>(n, f->dsys, f->a.sys, f->a.pos, f->sb.cnt, f->nbr, f->cnt, f->cap,
                                          cut * cut, f->oflag, f->need, 0);
    GC_CHECK_LAUNCH("fused: build lists");
    return build_morse_lists(f, st, f->mpos, false);
}

int capture_step(GcFused* f, int drive) {
    if (!f->gst) GC_CUDA(cudaStreamCreateWithFlags(&f->gst, cudaStreamNonBlocking), "fused: capture stream");
    if (!f->gst2) GC_CUDA(cudaStreamCreateWithFlags(&f->gst2, cudaStreamNonBlocking), "fused: capture stream");
    if (!f->gst3) GC_CUDA(cudaStreamCreateWithFlags(&f->gst3, cudaStreamNonBlocking), "fused: capture stream");
    cudaStream_t st = f->gst;
    GcParams p = f->p;
    unsigned long long l0 = gc_launch_count();
    GC_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "fused: begin capture");
    f->capturing = true;
    int rc = GC_OK;
    cudaGraph_t g = nullptr;
    cudaGraphConditionalHandle hcond = 0;
    long long main_kernels = 0, body_kernels = 0;
    do {
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps);
        if (e != cudaSuccess) { rc = gc_cuda_fail(e, "fused: capture info"); break; }
        e = cudaGraphConditionalHandleCreate(&hcond, g, 0, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) { rc = gc_cuda_fail(e, "fused: conditional handle"); break; }
        if ((rc = launch_step_begin(f, st)) != GC_OK) break;
        if ((rc = launch_integrate(f, st, p)) != GC_OK) break;
        fk_set_cond<<<1, 1, 0, st>>>(hcond, f->rebuild, f->drebuilds);
        gc_count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) { rc = gc_cuda_fail(e, "fused: set condition"); break; }
        e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps);
        if (e != cudaSuccess) { rc = gc_cuda_fail(e, "fused: capture info"); break; }
        cudaGraphNodeParams np = {};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = hcond;
        np.conditional.type = cudaGraphCondTypeIf;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        e = cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &np);
        if (e != cudaSuccess) { rc = gc_cuda_fail(e, "fused: conditional node"); break; }
        cudaGraph_t body = np.conditional.phGraph_out[0];
        e = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
        if (e != cudaSuccess) { rc = gc_cuda_fail(e, "fused: capture dependencies"); break; }
        unsigned long long lb = gc_launch_count();
        e = cudaStreamBeginCaptureToGraph(f->gst2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) { rc = gc_cuda_fail(e, "fused: capture rebuild"); break; }
        rc = launch_rebuild_body(f, f->gst2);
        cudaGraph_t body_out = nullptr;
        e = cudaStreamEndCapture(f->gst2, &body_out);
        if (rc != GC_OK) break;
        if (e != cudaSuccess) { rc = gc_cuda_fail(e, "fused: end rebuild capture"); break; }
        body_kernels = (long long)(gc_launch_count() - lb);
        // the membrane passes after the conditional rebuild (which writes the
        // Morse lists they read), beside the density pass
        if ((rc = fork_membranes(f, st, f->gst3, p)) != GC_OK) break;
        if ((rc = launch_density(f, st, p, true)) != GC_OK) break;
        if ((rc = join_membranes(f, st)) != GC_OK) break;
        if ((rc = launch_force(f, st, p, drive)) != GC_OK) break;
        if ((rc = launch_wallvel(f, st, p)) != GC_OK) break;
    } while (0);
    f->capturing = false;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    unsigned long long l1 = gc_launch_count();
    gc_add_launches(-(long long)(l1 - l0));   // capturing launches nothing
    if (rc != GC_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return gc_cuda_fail(e, "fused: end capture");
    main_kernels = (long long)(l1 - l0) - body_kernels;
    cudaGraphExec_t ex = nullptr;
    e = cudaGraphInstantiate(&ex, graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        return gc_cuda_fail(e, "fused: instantiate step graph");
    }
    f->cg[drive] = graph;
    f->gexec[drive] = ex;
    f->kernels_step = main_kernels;
    f->kernels_rebuild = body_kernels;
    return GC_OK;
}

int alloc_copy(GcFused* f, StateCopy* c) {
    if (c->have) return GC_OK;
    size_t n = f->n;
    GC_TRY(falloc(f, &c->s.pos, n));
    GC_TRY(falloc(f, &c->s.plo, n));
    GC_TRY(falloc(f, &c->s.vel, n));
    GC_TRY(falloc(f, &c->s.vpred, n));
    GC_TRY(falloc(f, &c->s.vh, n));
    GC_TRY(falloc(f, &c->s.force, n));
    GC_TRY(falloc(f, &c->s.nthro, n));
    if (f->a.sys) GC_TRY(falloc(f, &c->s.sys, n));
    if (f->ncp > 0) {
        GC_TRY(falloc(f, &c->mpos, f->ncp));
        GC_TRY(falloc(f, &c->mplo, f->ncp));
        GC_TRY(falloc(f, &c->mnthro, f->ncp));
    }
    GC_TRY(falloc(f, &c->dstep, 1));
    c->have = true;
    return GC_OK;
}

int copy_state(GcFused* f, const SlotArrays& src, const float4* mpos, const float4* mplo, const int4* mnt,
               const long long* dstep, SlotArrays& dst, float4* dmpos, float4* dmplo, int4* dmnt,
               long long* ddstep) {
    cudaStream_t st = f->st;
    size_t n = f->n;
    auto cp = [&](void* d, const void* s, size_t bytes) -> int {
        if (!d || !s || !bytes) return GC_OK;
        GC_CUDA(cudaMemcpyAsync(d, s, bytes, cudaMemcpyDeviceToDevice, st), "fused: state copy");
        return GC_OK;
    };
    GC_TRY(cp(dst.pos, src.pos, n * 16));
    GC_TRY(cp(dst.plo, src.plo, n * 16));
    GC_TRY(cp(dst.vel, src.vel, n * 16));
    GC_TRY(cp(dst.vpred, src.vpred, n * 16));
    GC_TRY(cp(dst.vh, src.vh, n * 16));
    GC_TRY(cp(dst.force, src.force, n * 16));
    GC_TRY(cp(dst.nthro, src.nthro, n * 16));
    GC_TRY(cp(dst.sys, src.sys, n * 4));
    GC_TRY(cp(dmpos, mpos, (size_t)f->ncp * 16));
    GC_TRY(cp(dmplo, mplo, (size_t)f->ncp * 16));
    GC_TRY(cp(dmnt, mnt, (size_t)f->ncp * 16));
    GC_TRY(cp(ddstep, dstep, 8));
    return GC_OK;
}

int save_state(GcFused* f, StateCopy* c) {
    GC_TRY(alloc_copy(f, c));
    return copy_state(f, f->a, f->mpos, f->mplo, f->mnthro, f->dstep, c->s, c->mpos, c->mplo, c->mnthro, c->dstep);
}

int restore_state(GcFused* f, StateCopy* c) {
    return copy_state(f, c->s, c->mpos, c->mplo, c->mnthro, c->dstep, f->a, f->mpos, f->mplo, f->mnthro, f->dstep);
}

// Re-sort and rebuild outside a step, then recompute what the outputs show
// (density and pressure in the new slot order, membrane forces).
int refresh(GcFused* f) {
    GC_TRY(rebuild_lists(f));
    GcParams p = f->p;
    p.noise_key = noise_key(p.seed, (uint64_t)(f->step < 0 ? 0 : f->step));
    GC_TRY(launch_density(f, f->st, p, true));
    GC_TRY(launch_membranes(f, f->st, p));
    return GC_OK;
}

// Fresh lists with room for growth, then capture.
int prepare_graph(GcFused* f, int drive) {
    if (f->graph_dirty) {
        GC_TRY(rebuild_lists(f));
        if (!f->lists) {
            // room in the pair lists for the rebuilds inside captured steps
            const size_t want = (size_t)(1.25 * f->h->tchunks) + 256;
            if (want > f->tent_chunks) {
                GC_TRY(tiles_alloc_entries(f, want));
                GC_TRY(rebuild_lists(f));
            }
        }
        // capacity for captured steps: the longest list now plus a margin
        GC_CUDA(cudaMemsetAsync(f->stat_max, 0, sizeof(int), f->st), "fused: stats");
        GC_CUDA(cudaMemsetAsync(f->stat_sum, 0, sizeof(unsigned long long), f->st), "fused: stats");
        fk_count_stats<<<gc_blocks(f->n, 256), 256, 0, f->st>>>(f->n, f->cnt, f->stat_sum, f->stat_max);
        GC_CHECK_LAUNCH("fused: stats");
        int mx = 0;
        GC_CUDA(cudaMemcpyAsync(&mx, f->stat_max, 4, cudaMemcpyDeviceToHost, f->st), "fused: stats");
        GC_CUDA(cudaStreamSynchronize(f->st), "fused: stats");
        int want = ((int)(1.25 * mx) + 16 + 7) & ~7;
        if (want > f->cap) {
            GC_TRY(alloc_list(f, want));
            GC_TRY(rebuild_lists(f));
        }
        GC_TRY(sync_dstep(f));
        drop_graphs(f);
        f->graph_dirty = false;
    }
    if (!f->gexec[drive]) GC_TRY(capture_step(f, drive));
    return GC_OK;
}

// Captured steps run in segments of at most kGraphSegment steps, each from a
// snapshot of the state: a list overflow (checked after each segment) sends
// only that segment back to its snapshot, to run again with longer lists.
constexpr int kGraphSegment = 128;

int graph_segment(GcFused* f, int nsteps, int drive);

int graph_steps(GcFused* f, int nsteps, int drive) {
    for (int done = 0; done < nsteps; done += kGraphSegment)
        GC_TRY(graph_segment(f, std::min(kGraphSegment, nsteps - done), drive));
    return GC_OK;
}

int graph_segment(GcFused* f, int nsteps, int drive) {
    if (nsteps <= 0) return GC_OK;
    long long step0 = f->step;
    for (int attempt = 0; attempt < 4; ++attempt) {
        GC_TRY(prepare_graph(f, drive));
        GC_TRY(save_state(f, &f->snap));
        GC_CUDA(cudaMemsetAsync(f->oflag, 0, sizeof(unsigned), f->st), "fused: flags");
        GC_CUDA(cudaMemsetAsync(f->need, 0, sizeof(int), f->st), "fused: flags");
        for (int k = 0; k < nsteps; ++k)
            GC_CUDA(cudaGraphLaunch(f->gexec[drive], f->st), "fused: launch step graph");
        GC_CUDA(cudaMemcpyAsync(&f->h->oflag, f->oflag, sizeof(unsigned), cudaMemcpyDeviceToHost, f->st), "fused: flags");
        GC_CUDA(cudaMemcpyAsync(&f->h->drebuilds, f->drebuilds, 8, cudaMemcpyDeviceToHost, f->st), "fused: flags");
        GC_CUDA(cudaMemcpyAsync(&f->h->need, f->need, sizeof(int), cudaMemcpyDeviceToHost, f->st), "fused: flags");
        GC_CUDA(cudaStreamSynchronize(f->st), "fused: step graphs");
        long long nreb = (long long)(f->h->drebuilds - f->drebuilds_seen);
        f->drebuilds_seen = f->h->drebuilds;
        gc_add_launches(f->kernels_step * nsteps + f->kernels_rebuild * nreb);
        if (!(f->h->oflag & (GC_FLAG_CELL_OVERFLOW | GC_FLAG_TILE_FULL | kMorseFull))) {
            f->step = step0 + nsteps;
            f->steps += nsteps;
            f->rebuilds += nreb;
            return GC_OK;
        }
        // a list overflowed: go back to the state before these steps, grow
        // the lists (or, with a cube too full for the pair tiles, turn to
        // per-particle lists) and run them again
        GC_TRY(restore_state(f, &f->snap));
        f->step = step0;
        if (f->h->oflag & kMorseFull) {
            // the Morse lists: room for what the failed rebuild wanted
            unsigned need = 0;
            GC_CUDA(cudaMemcpy(&need, f->moff + f->ncp, sizeof(unsigned), cudaMemcpyDeviceToHost),
                    "fused: Morse lists");
            const size_t want = (size_t)(1.5 * (need > f->mcap ? need : f->mcap)) + 4096;
            if (f->mlist) cudaFree(f->mlist);
            f->mlist = nullptr;
            f->mcap = 0;
            GC_CUDA(cudaMalloc(&f->mlist, want * sizeof(int)), "fused: Morse lists");
            f->mcap = want;
        }
        if (!(f->h->oflag & (GC_FLAG_CELL_OVERFLOW | GC_FLAG_TILE_FULL))) {
            // only the Morse lists overflowed
        } else if (f->h->oflag & GC_FLAG_TILE_FULL) {
            GC_TRY(switch_to_lists(f));
        } else if (!f->lists) {
            unsigned need = 0;
            GC_CUDA(cudaMemcpy(&need, f->toff + (size_t)f->K * kTilePairs, sizeof(unsigned), cudaMemcpyDeviceToHost),
                    "fused: tiles");
            GC_TRY(tiles_alloc_entries(f, (size_t)(1.25 * (need > f->tent_chunks ? need : f->tent_chunks)) + 256));
            if (f->h->need > 0) GC_TRY(alloc_list(f, grown_capacity(f, f->cap + f->cap / 2 + 8)));
        } else {
            GC_TRY(alloc_list(f, grown_capacity(f, f->cap + f->cap / 2 + 8)));
        }
        f->graph_dirty = true;
    }
    return gc_fail(GC_EDEVICE, "fused: neighbour lists keep overflowing in captured steps (capacity %d)", f->cap);
}

// ---- membranes: device arrays ---------------------------------------------

int alloc_cells(GcFused* f, int ncell, int ntri, int nedge, int ncp) {
    f->ncell = ncell;
    f->ntri = ntri;
    f->nedge = nedge;
    f->ncp = ncp;
    GC_TRY(falloc(f, &f->tri, ntri));
    GC_TRY(falloc(f, &f->edge, nedge));
    GC_TRY(falloc(f, &f->betri, ncell));
    GC_TRY(falloc(f, &f->celltab, ncp));
    float** e1[] = {&f->shear, &f->bend, &f->l0, &f->lmax, &f->perlen, &f->hpow, &f->hbend, &f->refang};
    for (float** q : e1) GC_TRY(falloc(f, q, nedge));
    float** t1[] = {&f->hl, &f->hg, &f->hv, &f->tarea, &f->reftarea};
    for (float** q : t1) GC_TRY(falloc(f, q, ntri));
    GC_TRY(falloc(f, &f->tnorm, ntri));
    GC_TRY(falloc(f, &f->tcen, ntri));
    double** c1[] = {&f->carea, &f->cvol, &f->crefarea, &f->crefvol};
    for (double** q : c1) GC_TRY(falloc(f, q, ncell));
    GC_TRY(falloc(f, &f->mforce, ncp));
    GC_TRY(falloc(f, &f->magg, ncp));
    GC_TRY(falloc(f, &f->parea, ncp));
    GC_TRY(falloc(f, &f->mkeys, ncp));
    GC_TRY(falloc(f, &f->mspos, ncp));
    GC_TRY(falloc(f, &f->msarea, ncp));
    GC_TRY(falloc(f, &f->mvals, ncp));
    GC_TRY(falloc(f, &f->mparts, 4 * (size_t)nedge + 3 * (size_t)ntri));
    GC_TRY(falloc(f, &f->inc_ptr, (size_t)ncp + 1));
    GC_TRY(falloc(f, &f->inc, 4 * (size_t)nedge + 3 * (size_t)ntri));
    GC_CUDA(cudaMemsetAsync(f->magg, 0, (size_t)ncp * sizeof(float4), f->st), "fused: magg");
    f->have_agg = f->p.De != 0.f && f->p.maxcut > 0.f;
    // GPUCELL_MORSE_ROOM (tests): the Morse lists' room beyond the latest
    // build as a factor, with no extra entries (1 fills them exactly)
    if (const char* e = getenv("GPUCELL_MORSE_ROOM")) {
        const double r = atof(e);
        if (r >= 1.0) {
            f->mroom = r;
            f->mslack = 0.0;
            f->mextra = 0;
        }
    }
    return GC_OK;
}

// Vertex -> part incidence (CSR) from the global 1-based topology (host
// arrays): for every vertex its edge parts in edge order, then its triangle
// parts in triangle order.  Out-of-range indices contribute nothing.
int build_incidence(GcFused* f, const int* tri, const int* edge) {
    const int ncp = f->ncp, ne = f->nedge, nt = f->ntri;
    std::vector<int> cnt((size_t)ncp + 1, 0);
    auto ok = [&](int v) { return v >= 1 && v <= ncp; };
    for (int e = 0; e < ne; ++e)
        for (int r = 0; r < 4; ++r)
            if (ok(edge[6 * (size_t)e + r])) ++cnt[edge[6 * (size_t)e + r]];
    for (int t = 0; t < nt; ++t)
        for (int r = 0; r < 3; ++r)
            if (ok(tri[3 * (size_t)t + r])) ++cnt[tri[3 * (size_t)t + r]];
    std::vector<int> ptr((size_t)ncp + 1, 0);
    for (int v = 0; v < ncp; ++v) ptr[v + 1] = ptr[v] + cnt[v + 1];
    std::vector<int> fill(ptr.begin(), ptr.end() - 1), inc((size_t)ptr[ncp]);
    for (int e = 0; e < ne; ++e)
        for (int r = 0; r < 4; ++r) {
            int v = edge[6 * (size_t)e + r];
            if (ok(v)) inc[fill[v - 1]++] = 4 * e + r;
        }
    for (int t = 0; t < nt; ++t)
        for (int r = 0; r < 3; ++r) {
            int v = tri[3 * (size_t)t + r];
            if (ok(v)) inc[fill[v - 1]++] = 4 * ne + 3 * t + r;
        }
    GC_CUDA(cudaMemcpyAsync(f->inc_ptr, ptr.data(), ptr.size() * 4, cudaMemcpyHostToDevice, f->st), "fused: incidence");
    GC_CUDA(cudaMemcpyAsync(f->inc, inc.data(), inc.size() * 4, cudaMemcpyHostToDevice, f->st), "fused: incidence");
    GC_CUDA(cudaStreamSynchronize(f->st), "fused: incidence");
    return GC_OK;
}

// Concatenates the systems' topologies with global vertex, triangle and cell
// offsets and uploads them.
int finalize_cells(GcFused* f) {
    int ncell = 0, ntri = 0, nedge = 0;
    f->c0.assign(f->nsys, 0);
    f->t0.assign(f->nsys, 0);
    for (int s = 0; s < f->nsys; ++s) {
        f->c0[s] = ncell;
        f->t0[s] = ntri;
        const HostCells& h = f->hcells[s];
        if (!h.set) continue;
        ncell += h.ncell;
        ntri += h.ntri;
        nedge += h.nedge;
    }
    if (ncell == 0) return GC_OK;
    std::vector<int> tri(3 * (size_t)ntri), edge(6 * (size_t)nedge), betri(2 * (size_t)ncell), celltab(f->ncp, -1);
    std::vector<float> shear(nedge), bend(nedge), hl(ntri), hg(ntri), hv(ntri);
    std::vector<int> msys(f->ncp, 0), cellsys(ncell, 0);
    size_t ot = 0, oe = 0, oc = 0;
    for (int s = 0; s < f->nsys; ++s) {
        const HostCells& h = f->hcells[s];
        const SysInfo& S = f->hsys[s];
        int m0 = (int)S.m0, ncps = (int)(S.end - S.cs);
        for (int v = 0; v < ncps; ++v) msys[m0 + v] = s;
        if (!h.set) continue;
        int t0 = f->t0[s], c0 = f->c0[s];
        for (int k = 0; k < 3 * h.ntri; ++k) tri[3 * ot + k] = h.tri[k] + m0;
        for (int k = 0; k < h.nedge; ++k) {
            for (int q = 0; q < 4; ++q) edge[6 * (oe + k) + q] = h.edge[6 * k + q] + m0;
            for (int q = 4; q < 6; ++q) edge[6 * (oe + k) + q] = h.edge[6 * k + q] + t0;
        }
        for (int k = 0; k < h.ncell; ++k) {
            betri[2 * (oc + k)] = h.betri[2 * k] + t0;
            betri[2 * (oc + k) + 1] = h.betri[2 * k + 1] + t0;
            cellsys[oc + k] = s;
        }
        for (int v = 0; v < ncps; ++v) celltab[m0 + v] = h.celltab[v] + c0;
        std::copy(h.shear.begin(), h.shear.end(), shear.begin() + oe);
        std::copy(h.bend.begin(), h.bend.end(), bend.begin() + oe);
        std::copy(h.hl.begin(), h.hl.end(), hl.begin() + ot);
        std::copy(h.hg.begin(), h.hg.end(), hg.begin() + ot);
        std::copy(h.hv.begin(), h.hv.end(), hv.begin() + ot);
        ot += h.ntri;
        oe += h.nedge;
        oc += h.ncell;
    }
    GC_TRY(alloc_cells(f, ncell, ntri, nedge, f->ncp));
    cudaStream_t st = f->st;
    auto up = [&](void* d, const void* s, size_t bytes) -> int {
        GC_CUDA(cudaMemcpyAsync(d, s, bytes, cudaMemcpyHostToDevice, st), "fused: upload cells");
        return GC_OK;
    };
    GC_TRY(up(f->tri, tri.data(), tri.size() * 4));
    GC_TRY(up(f->edge, edge.data(), edge.size() * 4));
    GC_TRY(up(f->betri, betri.data(), betri.size() * 4));
    GC_TRY(up(f->celltab, celltab.data(), celltab.size() * 4));
    GC_TRY(up(f->shear, shear.data(), shear.size() * 4));
    GC_TRY(up(f->bend, bend.data(), bend.size() * 4));
    GC_TRY(up(f->hl, hl.data(), hl.size() * 4));
    GC_TRY(up(f->hg, hg.data(), hg.size() * 4));
    GC_TRY(up(f->hv, hv.data(), hv.size() * 4));
    GC_TRY(build_incidence(f, tri.data(), edge.data()));
    {
        std::vector<int> cv(2 * (size_t)ncell);
        size_t oc2 = 0;
        for (int s = 0; s < f->nsys; ++s) {
            const HostCells& h = f->hcells[s];
            if (!h.set) continue;
            for (int k = 0; k < 2 * h.ncell; ++k) cv[2 * oc2 + k] = h.verts[k] + (int)f->hsys[s].m0;
            oc2 += h.ncell;
        }
        GC_TRY(falloc(f, &f->cell_verts, ncell));
        GC_TRY(falloc(f, &f->cell_stats, 12 * (size_t)ncell));
        GC_TRY(up(f->cell_verts, cv.data(), cv.size() * 4));
        // the aggregation pass may skip a vertex's own cell as one run of
        // ids when each cell's vertex range is exactly the vertices whose
        // CellTab names it (GPUCell labels the vertices of each cell in
        // file order, src/Particle.cu:240)
        bool runs = true;
        for (int c = 0; c < ncell && runs; ++c) {
            if (cv[2 * c] < 0 || cv[2 * c + 1] >= f->ncp || cv[2 * c + 1] < cv[2 * c]) runs = false;
            for (int v = cv[2 * c]; runs && v <= cv[2 * c + 1]; ++v) runs = celltab[v] == c;
        }
        for (int v = 0; v < f->ncp && runs; ++v) {
            int c = celltab[v];
            runs = c >= 0 && c < ncell && v >= cv[2 * c] && v <= cv[2 * c + 1];
        }
        f->agg_runs = runs;
    }
    if (f->nsys > 1) {
        GC_TRY(falloc(f, &f->msys, f->ncp));
        GC_TRY(falloc(f, &f->cellsys, ncell));
        GC_TRY(up(f->msys, msys.data(), msys.size() * 4));
        GC_TRY(up(f->cellsys, cellsys.data(), cellsys.size() * 4));
    }
    GC_CUDA(cudaStreamSynchronize(st), "fused: upload cells");   // the host vectors go out of scope
    return GC_OK;
}

bool same_physics(const Structconst& a, const Structconst& b) {
    return a.CutRadius == b.CutRadius && a.Mass == b.Mass && a.SoundSpeed1 == b.SoundSpeed1 &&
           a.SoundSpeed2 == b.SoundSpeed2 && a.DenInit == b.DenInit && a.VVsigma == b.VVsigma &&
           a.ShearVis == b.ShearVis && a.BulkVis == b.BulkVis && a.TimeStep == b.TimeStep &&
           a.surEnergy == b.surEnergy && a.MaxCut == b.MaxCut && a.zeroLen == b.zeroLen && a.scaFac == b.scaFac &&
           a.Temp == b.Temp;
}

int check_sys(GcFused* f, int sys, const char* what) {
    if (!f) return gc_fail(GC_EINVAL, "%s: NULL handle", what);
    if (sys < 0 || sys >= f->nsys) return gc_fail(GC_EINVAL, "%s: system %d outside 0..%d", what, sys, f->nsys - 1);
    return GC_OK;
}

int apply_options(GcFused* f, const GcFusedOptions* opt) {
    if (!opt) return GC_OK;
    if (opt->block != 0 && opt->block != 64 && opt->block != 128 && opt->block != kMaxBS)
        return gc_fail(GC_EINVAL, "fused: block %d is not 64, 128 or 256", opt->block);
    if (opt->skin < 0.f || opt->skin > 1.f) return gc_fail(GC_EINVAL, "fused: skin %g outside [0, 1] rc", opt->skin);
    if (opt->skin > 0.f) f->skin_rel = opt->skin;
    if (opt->block) f->block = opt->block;
    f->compact = opt->compact != 0;
    f->graph = opt->graph != 0;
    f->lists = opt->tiles == 0;
    f->ddpos = opt->fp32_positions ? 0 : 1;
    f->halfv = opt->half_velocity != 0;
    return GC_OK;
}

}  // namespace gcf

namespace gcf {

// Loads the ids [id_base, id_base + count) from host or device arrays.
// Host transfers of at least kXferSplit particles go in kXferChunks pieces:
// the copies of piece c on the library's stream overlap the conversion
// kernel of piece c - 1 (load) or c + 1 (store) on the side stream, so the
// copy engines are not left idle while the kernels run.
constexpr int kXferChunks = 4;
constexpr int kXferSplit = 1 << 20;

static void load_piece(GcFused* f, cudaStream_t ks, unsigned id_base, int k0, int k1, const float* dx,
                       const float* dv, const float* dh, const float* df, const int* dn) {
    const int keep = f->setup_done ? 1 : 0;
    auto at = [&](const auto* a) { return a ? a + 3 * (size_t)k0 : a; };
    fk_load<<<gc_blocks(k1 - k0, f->block), f->block, 0, ks>>>(
        k1 - k0, id_base + (unsigned)k0, f->dsys, f->nsys, keep, at(dx), at(dv), at(dh), at(df), at(dn), f->slot_of,
        f->a.pos, f->a.plo, f->a.vel, f->a.vh, f->a.force, f->a.nthro, keep && f->ncell > 0 ? f->mpos : nullptr,
        f->mplo, f->mnthro);
}

int load_range(GcFused* f, unsigned id_base, int count, const float* pos, const float* vel,
                      const float* velhalf, const float* force, const int* nthro, int from_device) {
    if (count <= 0) return GC_OK;
    cudaStream_t st = f->st;
    if (from_device) {
        load_piece(f, st, id_base, 0, count, pos, vel, velhalf, force, nthro);
        GC_CHECK_LAUNCH("fused: load");
        return GC_OK;
    }
    const size_t b3 = (size_t)count * 12;
    GC_TRY(stage_bytes(f, 5 * b3));
    char* s = (char*)f->stage;
    const void* src[5] = {pos, vel, velhalf, force, nthro};
    const int nch = count >= kXferSplit ? kXferChunks : 1;
    for (int c = 0; c < nch; ++c) {
        const int k0 = (int)((long long)count * c / nch), k1 = (int)((long long)count * (c + 1) / nch);
        for (int a = 0; a < 5; ++a)
            if (src[a])
                GC_CUDA(cudaMemcpyAsync(s + a * b3 + (size_t)k0 * 12, (const char*)src[a] + (size_t)k0 * 12,
                                        (size_t)(k1 - k0) * 12, cudaMemcpyHostToDevice, st),
                        "fused_load: upload");
        cudaStream_t ks = st;
        if (nch > 1) {   // piece c converts on the side stream once its copies are in
            GC_CUDA(cudaEventRecord(f->xev[c], st), "fused_load");
            GC_CUDA(cudaStreamWaitEvent(f->mst, f->xev[c], 0), "fused_load");
            ks = f->mst;
        }
        auto st_of = [&](int a) { return src[a] ? (const float*)(s + a * b3) : nullptr; };
        load_piece(f, ks, id_base, k0, k1, st_of(0), st_of(1), st_of(2), st_of(3), (const int*)st_of(4));
        GC_CHECK_LAUNCH("fused: load");
    }
    if (nch > 1) {
        GC_CUDA(cudaEventRecord(f->ev_join, f->mst), "fused_load");
        GC_CUDA(cudaStreamWaitEvent(st, f->ev_join, 0), "fused_load");
    }
    GC_CUDA(cudaStreamSynchronize(st), "fused_load");   // the staging buffer is reused
    return GC_OK;
}

int store_range(GcFused* f, unsigned id_base, int count, float* pos, float* vel, float* rho, float* press,
                       float* force, float* velhalf, int* nthro, int to_device) {
    if (count <= 0) return GC_OK;
    cudaStream_t st = f->st;
    auto piece = [&](cudaStream_t ks, int k0, int k1, float* x, float* v, float* r, float* pr, float* fo, float* vh,
                     int* nt) {
        auto at3 = [&](auto* a) { return a ? a + 3 * (size_t)k0 : a; };
        auto at1 = [&](float* a) { return a ? a + k0 : a; };
        fk_store<<<gc_blocks(k1 - k0, f->block), f->block, 0, ks>>>(
            k1 - k0, id_base + (unsigned)k0, f->p, f->slot_of, f->a.pos, f->a.vel, f->a.vh, f->a.force, f->dp,
            f->a.nthro, at3(x), at3(v), at1(r), at1(pr), at3(fo), at3(vh), at3(nt));
    };
    if (to_device) {
        piece(st, 0, count, pos, vel, rho, press, force, velhalf, nthro);
        GC_CHECK_LAUNCH("fused: store");
        return GC_OK;
    }
    const size_t b3 = (size_t)count * 12, b1 = (size_t)count * 4;
    GC_TRY(stage_bytes(f, 5 * b3 + 2 * b1));
    char* s = (char*)f->stage;
    float* x = pos ? (float*)(s) : nullptr;
    float* v = vel ? (float*)(s + b3) : nullptr;
    float* fo = force ? (float*)(s + 2 * b3) : nullptr;
    float* vh = velhalf ? (float*)(s + 3 * b3) : nullptr;
    int* nt = nthro ? (int*)(s + 4 * b3) : nullptr;
    float* r = rho ? (float*)(s + 5 * b3) : nullptr;
    float* pr = press ? (float*)(s + 5 * b3 + b1) : nullptr;
    const int nch = count >= kXferSplit ? kXferChunks : 1;
    if (nch > 1) {   // the side stream starts after the work before the store
        GC_CUDA(cudaEventRecord(f->ev_fork, st), "fused_store");
        GC_CUDA(cudaStreamWaitEvent(f->mst, f->ev_fork, 0), "fused_store");
    }
    for (int c = 0; c < nch; ++c) {
        const int k0 = (int)((long long)count * c / nch), k1 = (int)((long long)count * (c + 1) / nch);
        const size_t o3 = (size_t)k0 * 12, n3 = (size_t)(k1 - k0) * 12, o1 = (size_t)k0 * 4, n1 = (size_t)(k1 - k0) * 4;
        if (nch > 1) {   // piece c gathers on the side stream, its copies wait for it
            piece(f->mst, k0, k1, x, v, r, pr, fo, vh, nt);
            GC_CHECK_LAUNCH("fused: store");
            GC_CUDA(cudaEventRecord(f->xev[c], f->mst), "fused_store");
            GC_CUDA(cudaStreamWaitEvent(st, f->xev[c], 0), "fused_store");
        } else {
            piece(st, k0, k1, x, v, r, pr, fo, vh, nt);
            GC_CHECK_LAUNCH("fused: store");
        }
        auto down = [&](void* dst, const void* src, size_t off, size_t bytes) -> int {
            if (!dst) return GC_OK;
            GC_CUDA(cudaMemcpyAsync((char*)dst + off, (const char*)src + off, bytes, cudaMemcpyDeviceToHost, st),
                    "fused_store");
            return GC_OK;
        };
        GC_TRY(down(pos, x, o3, n3));
        GC_TRY(down(vel, v, o3, n3));
        GC_TRY(down(force, fo, o3, n3));
        GC_TRY(down(velhalf, vh, o3, n3));
        GC_TRY(down(nthro, nt, o3, n3));
        GC_TRY(down(rho, r, o1, n1));
        GC_TRY(down(press, pr, o1, n1));
    }
    GC_CUDA(cudaStreamSynchronize(st), "fused_store");
    return GC_OK;
}

// Membrane outputs of cells [c0, c0 + nc), vertices [m0, m0 + nv),
// triangles [t0, t0 + nt).
size_t cells_stage_bytes(size_t snc, size_t snv, size_t snt) {
    return 4 * (2 * snc + 3 * snv + 3 * snv + 3 * snt + 3 * snt + snv) + 64;
}

// The membrane outputs through the staging area `stage` on stream `st`;
// `sync`: wait for the copies.
int store_cells_on(GcFused* f, cudaStream_t st, char* stage, bool sync, int c0, int nc, int m0, int nv, int t0,
                   int nt, float* area, float* vol, float* defforce, float* aggforce, float* trinordir,
                   float* tricenter, float* pararea, int to_device) {
    if (f->ncell <= 0 || nc <= 0) return GC_OK;
    float *a = area, *vo = vol, *df = defforce, *ag = aggforce, *tn = trinordir, *tc = tricenter, *pa = pararea;
    size_t snc = nc, snv = nv, snt = nt;
    if (!to_device) {
        char* s = stage;
        size_t off = 0;
        auto take = [&](size_t cnt) { float* q = (float*)(s + off); off += 4 * cnt; return q; };
        a = take(snc); vo = take(snc); df = take(3 * snv); ag = take(3 * snv); tn = take(3 * snt); tc = take(3 * snt);
        pa = take(snv);
    }
    fk_cast_cells<<<gc_blocks(nc, 128), 128, 0, st>>>(nc, c0, f->carea, f->cvol, a, vo);
    GC_CHECK_LAUNCH("fused: store cells");
    int m = nv > nt ? nv : nt;
    fk_store_cells<<<gc_blocks(m, 128), 128, 0, st>>>(nv, m0, nt, t0, f->mforce, f->magg, f->parea, f->tnorm, f->tcen,
                                                     df, ag, pa, tn, tc, f->have_agg ? 1 : 0);
    GC_CHECK_LAUNCH("fused: store cells");
    if (!to_device) {
        if (area) GC_CUDA(cudaMemcpyAsync(area, a, 4 * snc, cudaMemcpyDeviceToHost, st), "store cells");
        if (vol) GC_CUDA(cudaMemcpyAsync(vol, vo, 4 * snc, cudaMemcpyDeviceToHost, st), "store cells");
        if (defforce) GC_CUDA(cudaMemcpyAsync(defforce, df, 12 * snv, cudaMemcpyDeviceToHost, st), "store cells");
        if (aggforce) GC_CUDA(cudaMemcpyAsync(aggforce, ag, 12 * snv, cudaMemcpyDeviceToHost, st), "store cells");
        if (trinordir) GC_CUDA(cudaMemcpyAsync(trinordir, tn, 12 * snt, cudaMemcpyDeviceToHost, st), "store cells");
        if (tricenter) GC_CUDA(cudaMemcpyAsync(tricenter, tc, 12 * snt, cudaMemcpyDeviceToHost, st), "store cells");
        if (pararea) GC_CUDA(cudaMemcpyAsync(pararea, pa, 4 * snv, cudaMemcpyDeviceToHost, st), "store cells");
        if (sync) GC_CUDA(cudaStreamSynchronize(st), "store cells");
    }
    return GC_OK;
}

int store_cells_range(GcFused* f, int c0, int nc, int m0, int nv, int t0, int nt, float* area, float* vol,
                             float* defforce, float* aggforce, float* trinordir, float* tricenter, float* pararea,
                             int to_device) {
    if (f->ncell <= 0 || nc <= 0) return GC_OK;
    if (!to_device) GC_TRY(stage_bytes(f, cells_stage_bytes(nc, nv, nt)));
    return store_cells_on(f, f->st, (char*)f->stage, true, c0, nc, m0, nv, t0, nt, area, vol, defforce, aggforce,
                          trinordir, tricenter, pararea, to_device);
}

// The particle outputs of every slot gathered into the staging area `s`
// (one region per array, as store_range lays them out) and copied to host
// memory on stream `ks`, without waiting (NULL outputs are skipped).
size_t particle_stage_bytes(size_t n) { return 5 * n * 12 + 2 * n * 4; }

int store_particles_on(GcFused* f, cudaStream_t ks, char* s, float* pos, float* vel, float* rho, float* press,
                       float* force, float* velhalf, int* nthro) {
    if (!(pos || vel || rho || press || force || velhalf || nthro)) return GC_OK;
    const size_t n = f->n, b3 = n * 12, b1 = n * 4;
    float* x = pos ? (float*)(s) : nullptr;
    float* v = vel ? (float*)(s + b3) : nullptr;
    float* fo = force ? (float*)(s + 2 * b3) : nullptr;
    float* vh = velhalf ? (float*)(s + 3 * b3) : nullptr;
    int* nt = nthro ? (int*)(s + 4 * b3) : nullptr;
    float* r = rho ? (float*)(s + 5 * b3) : nullptr;
    float* pr = press ? (float*)(s + 5 * b3 + b1) : nullptr;
    fk_store<<<gc_blocks(f->n, f->block), f->block, 0, ks>>>(f->n, 0u, f->p, f->slot_of, f->a.pos, f->a.vel, f->a.vh,
                                                             f->a.force, f->dp, f->a.nthro, x, v, r, pr, fo, vh, nt);
    GC_CHECK_LAUNCH("fused: store");
    auto down = [&](void* dst, const void* src, size_t bytes) -> int {
        if (!dst) return GC_OK;
        GC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ks), "fused_step_store");
        return GC_OK;
    };
    GC_TRY(down(pos, x, b3));
    GC_TRY(down(vel, v, b3));
    GC_TRY(down(force, fo, b3));
    GC_TRY(down(velhalf, vh, b3));
    GC_TRY(down(nthro, nt, b3));
    GC_TRY(down(rho, r, b1));
    GC_TRY(down(press, pr, b1));
    return GC_OK;
}

// gc_fused_step_store's copies at the points of the step where their data
// are final: 0 after the integration and any rebuild (positions, VelHalf,
// crossing counts), 1 after the density pass (density, pressure), 2 after
// the membrane passes (membrane outputs) -- these on the copy stream,
// beside the rest of the step -- and 3 at the end (velocities, forces),
// after which the step's stream waits for the copy stream.
int ensure_early_stream(GcFused* f) {
    if (!f->xst) GC_CUDA(cudaStreamCreateWithFlags(&f->xst, cudaStreamNonBlocking), "fused: write stream");
    for (int k = 0; k < 4; ++k)
        if (!f->xe[k]) GC_CUDA(cudaEventCreateWithFlags(&f->xe[k], cudaEventDisableTiming), "fused: write events");
    return GC_OK;
}

int early_store(GcFused* f, cudaStream_t st, int phase) {
    const EarlyStore& e = *f->es;
    char* s = (char*)f->stage;
    if (phase < 3) {
        GC_CUDA(cudaEventRecord(f->xe[phase], st), "fused_step_store");
        GC_CUDA(cudaStreamWaitEvent(f->xst, f->xe[phase], 0), "fused_step_store");
    }
    switch (phase) {
    case 0: return store_particles_on(f, f->xst, s, e.pos, nullptr, nullptr, nullptr, nullptr, e.velhalf, e.nthro);
    case 1: return store_particles_on(f, f->xst, s, nullptr, nullptr, e.rho, e.press, nullptr, nullptr, nullptr);
    case 2:
        return store_cells_on(f, f->xst, s + particle_stage_bytes(f->n), false, 0, f->ncell, 0, f->ncp, 0, f->ntri,
                              e.area, e.vol, e.defforce, e.aggforce, e.trinordir, e.tricenter, e.pararea, 0);
    default:
        GC_TRY(store_particles_on(f, st, s, nullptr, e.vel, nullptr, nullptr, e.force, nullptr, nullptr));
        GC_CUDA(cudaEventRecord(f->xe[3], f->xst), "fused_step_store");
        GC_CUDA(cudaStreamWaitEvent(st, f->xe[3], 0), "fused_step_store");
        return GC_OK;
    }
}

int cell_sums_range(GcFused* f, int c0, int nc, double* area, double* vol) {
    if (f->ncell <= 0 || nc <= 0) return GC_OK;
    if (area) GC_CUDA(cudaMemcpyAsync(area, f->carea + c0, 8 * (size_t)nc, cudaMemcpyDeviceToHost, f->st), "cell sums");
    if (vol) GC_CUDA(cudaMemcpyAsync(vol, f->cvol + c0, 8 * (size_t)nc, cudaMemcpyDeviceToHost, f->st), "cell sums");
    GC_CUDA(cudaStreamSynchronize(f->st), "cell sums");
    return GC_OK;
}

}  // namespace gcf

using namespace gcf;

extern "C" {

int gc_ensemble_create(int nsys, const GcSystemDesc* d, int noise_on, const GcFusedOptions* opt, GcFused** out) {
    if (!d || !out) return gc_fail(GC_EINVAL, "ensemble_create: NULL argument");
    if (nsys < 1) return gc_fail(GC_EINVAL, "ensemble_create: %d systems", nsys);
    unsigned long long ntot = 0, ncp = 0;
    for (int s = 0; s < nsys; ++s) {
        const Structconst& c = d[s].consts;
        if (d[s].periodic_mask < 0 || d[s].periodic_mask > 7)
            return gc_fail(GC_EINVAL, "ensemble_create: system %d: bad periodic mask", s);
        if (!(c.nBound2Start <= c.nFluidStart && c.nFluidStart <= c.nCellStart &&
              c.nCellStart + c.nCellPar == c.nTotalPar))
            return gc_fail(GC_EINVAL, "ensemble_create: system %d: inconsistent type boundaries", s);
        if (!same_physics(c, d[0].consts))
            return gc_fail(GC_EINVAL, "ensemble_create: system %d has other physics than system 0 (only counts, "
                                      "iSeed and ConstExtForce may differ)", s);
        ntot += c.nTotalPar;
        ncp += c.nCellPar;
    }
    if (ntot == 0) return gc_fail(GC_EINVAL, "ensemble_create: no particles");
    if (ntot >= (1ull << 30)) return gc_fail(GC_EINVAL, "ensemble_create: too many particles");
    GcFused* f = new GcFused();
    f->st = gc_state().stream;
    int rc = gc_params_from(d[0].consts, noise_on, &f->p);   // the same builder as the boundary entry points
    if (rc == GC_OK) rc = apply_options(f, opt);
    if (rc != GC_OK) {
        delete f;
        return rc;
    }
    f->nsys = nsys;
    f->desc.assign(d, d + nsys);
    f->hcells.resize(nsys);
    f->sys_loaded.assign(nsys, 0);
    f->noise_on = noise_on ? 1 : 0;
    f->n = (int)ntot;
    f->ncp = (int)ncp;
    f->p.nT = (unsigned)ntot;
    f->p.nCP = (unsigned)ncp;
    f->skin = f->skin_rel * f->p.rc;
    f->ens = nsys > 1;
    f->hsys.resize(nsys);
    unsigned id0 = 0, m0 = 0;
    for (int s = 0; s < nsys; ++s) {
        const Structconst& c = d[s].consts;
        SysInfo& S = f->hsys[s];
        memset(&S, 0, sizeof(S));
        S.seed = (uint64_t)c.iSeed;
        S.id0 = id0;
        S.b2 = id0 + c.nBound2Start;
        S.fl = id0 + c.nFluidStart;
        S.cs = id0 + c.nCellStart;
        S.end = id0 + c.nTotalPar;
        S.m0 = m0;
        S.gx = c.ConstExtForce;
        id0 += c.nTotalPar;
        m0 += c.nCellPar;
    }
    f->has_b1 = false;
    for (const SysInfo& S : f->hsys) f->has_b1 = f->has_b1 || S.b2 > S.id0;
    const int n = f->n;
    int ok = GC_OK;
    SlotArrays* sa[2] = {&f->a, &f->b};
    for (SlotArrays* s : sa) {
        if (ok == GC_OK) ok = falloc(f, &s->pos, (size_t)n + 1);   // slot n: the list padding sentinel
        if (ok == GC_OK) ok = falloc(f, &s->plo, n);
        if (ok == GC_OK) ok = falloc(f, &s->vel, n);
        if (ok == GC_OK) ok = falloc(f, &s->vpred, n);
        if (ok == GC_OK) ok = falloc(f, &s->vh, n);
        if (ok == GC_OK) ok = falloc(f, &s->force, n);
        if (ok == GC_OK) ok = falloc(f, &s->nthro, n);
        if (ok == GC_OK && nsys > 1) ok = falloc(f, &s->sys, n);
    }
    if (ok == GC_OK) ok = falloc(f, &f->refpos, n);
    if (ok == GC_OK) ok = falloc(f, &f->dp, n);
    if (ok == GC_OK) ok = falloc(f, &f->vph, (size_t)n + 1);
    if (ok == GC_OK) ok = falloc(f, &f->slot_of, n);
    if (ok == GC_OK) ok = falloc(f, &f->keys, n > f->ncp ? n : f->ncp);
    if (ok == GC_OK) ok = falloc(f, &f->vals, n > f->ncp ? n : f->ncp);
    if (ok == GC_OK) ok = falloc(f, &f->cnt, n);
    if (ok == GC_OK) ok = falloc(f, &f->ccnt, n);
    if (ok == GC_OK) ok = falloc(f, &f->rebuild, 1);
    if (ok == GC_OK) ok = falloc(f, &f->flags, 1);
    if (ok == GC_OK) ok = falloc(f, &f->oflag, 1);
    if (ok == GC_OK) ok = falloc(f, &f->need, 1);
    if (ok == GC_OK) ok = falloc(f, &f->stat_sum, 1);
    if (ok == GC_OK) ok = falloc(f, &f->stat_max, 1);
    if (ok == GC_OK) ok = falloc(f, &f->dstep, 1);
    if (ok == GC_OK) ok = falloc(f, &f->nkey, nsys);
    if (ok == GC_OK) ok = falloc(f, &f->drebuilds, 1);
    if (ok == GC_OK) ok = falloc(f, &f->dsys, nsys);
    if (ok == GC_OK && f->ncp > 0) ok = falloc(f, &f->mpos, f->ncp);
    if (ok == GC_OK && f->ncp > 0) ok = falloc(f, &f->mplo, f->ncp);
    if (ok == GC_OK && f->ncp > 0) ok = falloc(f, &f->mnthro, f->ncp);
    if (ok == GC_OK && cudaMallocHost(&f->h, sizeof(GcFused::Pinned)) != cudaSuccess)
        ok = gc_fail(GC_ENOMEM, "fused: pinned words");
    if (ok == GC_OK && (cudaStreamCreateWithFlags(&f->mst, cudaStreamNonBlocking) != cudaSuccess ||
                        cudaEventCreateWithFlags(&f->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
                        cudaEventCreateWithFlags(&f->ev_join, cudaEventDisableTiming) != cudaSuccess))
        ok = gc_fail(GC_ECUDA, "fused: membrane stream");
    for (int c = 0; c < 4 && ok == GC_OK; ++c)
        if (cudaEventCreateWithFlags(&f->xev[c], cudaEventDisableTiming) != cudaSuccess)
            ok = gc_fail(GC_ECUDA, "fused: transfer events");
    if (ok == GC_OK) ok = build_grids(f);
    if (ok == GC_OK) {
        // list capacity: expected neighbours within rc + skin at the largest
        // mean density of a system, with room for membranes and fluctuations
        double dens = 0.0;
        for (int s = 0; s < nsys; ++s) {
            const GcGrid& g = f->hsys[s].g;
            double vol = (double)g.L[0] * g.L[1] * g.L[2];
            double ds = d[s].consts.nTotalPar / vol;
            if (ds > dens) dens = ds;
        }
        double cutr = f->p.rc + f->skin;
        int capn = (int)(2.0 * 4.18879 * cutr * cutr * cutr * dens) + 32;
        if (!f->lists && !any_bound2(f)) capn = 8;   // the pair tiles need lists only for Bound2 walls
        if (opt && opt->list_capacity > 0) capn = opt->list_capacity;
        capn = (capn + 7) & ~7;
        ok = alloc_list(f, capn);
    }
    if (ok == GC_OK) {
        // the sentinel slot that pads the lists: NaN position, fails every cut-off test
        const uint32_t bits[4] = {0x7fc00000u, 0x7fc00000u, 0x7fc00000u, 0xffffffffu};
        float4 sentinel;
        memcpy(&sentinel, bits, sizeof(sentinel));
        if (cudaMemcpy(f->a.pos + n, &sentinel, sizeof(sentinel), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(f->b.pos + n, &sentinel, sizeof(sentinel), cudaMemcpyHostToDevice) != cudaSuccess)
            ok = gc_fail(GC_ECUDA, "fused: sentinel slot");
    }
    if (ok == GC_OK) {
        f->h->drebuilds = 0;
        f->h->need = 0;
        if (cudaMemsetAsync(f->flags, 0, sizeof(unsigned), f->st) != cudaSuccess ||
            cudaMemsetAsync(f->cnt, 0, (size_t)n * sizeof(int), f->st) != cudaSuccess ||   // lists of no slot yet
            cudaMemsetAsync(f->vph, 0, ((size_t)n + 1) * sizeof(uint2), f->st) != cudaSuccess ||
            cudaMemsetAsync(f->drebuilds, 0, 8, f->st) != cudaSuccess ||
            cudaMemsetAsync(f->dstep, 0xff, 8, f->st) != cudaSuccess)   // -1
            ok = gc_fail(GC_ECUDA, "fused: clear counters");
    }
    if (ok != GC_OK) {
        gc_fused_destroy(f);
        return ok;
    }
    *out = f;
    return GC_OK;
}

int gc_fused_create(const Structconst* consts, const float* bbox6, int periodic_mask, int noise_on,
                    const GcFusedOptions* opt, GcFused** out) {
    if (!consts || !bbox6 || !out) return gc_fail(GC_EINVAL, "fused_create: NULL argument");
    if (periodic_mask < 0 || periodic_mask > 7) return gc_fail(GC_EINVAL, "fused_create: bad periodic mask");
    GcSystemDesc d;
    memset(&d, 0, sizeof(d));
    d.consts = *consts;
    memcpy(d.bbox, bbox6, sizeof(d.bbox));
    d.periodic_mask = periodic_mask;
    return gc_ensemble_create(1, &d, noise_on, opt, out);
}

int gc_ensemble_size(GcFused* f, int* nsys, long long* nparticles) {
    if (!f) return gc_fail(GC_EINVAL, "ensemble_size: NULL handle");
    if (nsys) *nsys = f->nsys;
    if (nparticles) *nparticles = f->n;
    return GC_OK;
}

int gc_ensemble_set_cells(GcFused* f, int sys, int ncell, int ntri, int nedge, const int* tri, const int* edge,
                          const int* betri, const int* celltab, const float* shearmod, const float* bendmod,
                          const float* hlarea, const float* hgarea, const float* hvol) {
    GC_TRY(check_sys(f, sys, "set_cells"));
    if (f->setup_done || f->cells_adopted) return gc_fail(GC_ESTATE, "set_cells: call before gc_fused_setup");
    if (ncell <= 0) return GC_OK;
    int ncp = (int)f->desc[sys].consts.nCellPar;
    if (ncp <= 0 || ntri <= 0 || nedge <= 0) return gc_fail(GC_EINVAL, "set_cells: empty topology");
    if (!tri || !edge || !betri || !celltab || !shearmod || !bendmod || !hlarea || !hgarea || !hvol)
        return gc_fail(GC_EINVAL, "set_cells: NULL array");
    for (int k = 0; k < 3 * ntri; ++k)
        if (tri[k] < 1 || tri[k] > ncp) return gc_fail(GC_EINVAL, "set_cells: triangle index out of range");
    for (int k = 0; k < nedge; ++k) {
        for (int q = 0; q < 4; ++q)
            if (edge[6 * k + q] < 1 || edge[6 * k + q] > ncp)
                return gc_fail(GC_EINVAL, "set_cells: edge index out of range");
        for (int q = 4; q < 6; ++q)
            if (edge[6 * k + q] < 1 || edge[6 * k + q] > ntri)
                return gc_fail(GC_EINVAL, "set_cells: edge triangle index out of range");
    }
    for (int k = 0; k < ncell; ++k)
        if (betri[2 * k] < 0 || betri[2 * k + 1] >= ntri || betri[2 * k + 1] < betri[2 * k])
            return gc_fail(GC_EINVAL, "set_cells: bad triangle range of cell %d", k);
    HostCells& h = f->hcells[sys];
    h.set = true;
    h.ncell = ncell;
    h.ntri = ntri;
    h.nedge = nedge;
    h.tri.assign(tri, tri + 3 * (size_t)ntri);
    h.edge.assign(edge, edge + 6 * (size_t)nedge);
    h.betri.assign(betri, betri + 2 * (size_t)ncell);
    h.celltab.assign(celltab, celltab + ncp);
    h.shear.assign(shearmod, shearmod + nedge);
    h.bend.assign(bendmod, bendmod + nedge);
    h.hl.assign(hlarea, hlarea + ntri);
    h.hg.assign(hgarea, hgarea + ntri);
    h.hv.assign(hvol, hvol + ntri);
    h.verts.assign(2 * (size_t)ncell, 0);
    for (int k = 0; k < ncell; ++k) {
        int lo = ncp, hi = -1;
        for (int t = betri[2 * k]; t <= betri[2 * k + 1]; ++t)
            for (int q = 0; q < 3; ++q) {
                lo = std::min(lo, tri[3 * t + q] - 1);
                hi = std::max(hi, tri[3 * t + q] - 1);
            }
        h.verts[2 * k] = lo;
        h.verts[2 * k + 1] = hi;
    }
    return GC_OK;
}

int gc_fused_set_cells(GcFused* f, int ncell, int ntri, int nedge, const int* tri, const int* edge, const int* betri,
                       const int* celltab, const float* shearmod, const float* bendmod, const float* hlarea,
                       const float* hgarea, const float* hvol) {
    if (!f) return gc_fail(GC_EINVAL, "fused_set_cells: NULL handle");
    if (f->nsys != 1) return gc_fail(GC_EINVAL, "fused_set_cells: an ensemble takes gc_ensemble_set_cells");
    return gc_ensemble_set_cells(f, 0, ncell, ntri, nedge, tri, edge, betri, celltab, shearmod, bendmod, hlarea,
                                 hgarea, hvol);
}


int gc_ensemble_load(GcFused* f, int sys, const float* pos, const float* vel, const float* velhalf, const float* force,
                     const int* nthro, int from_device) {
    GC_TRY(check_sys(f, sys, "load"));
    if (!pos) return gc_fail(GC_EINVAL, "load: NULL positions");
    const SysInfo& S = f->hsys[sys];
    GC_TRY(load_range(f, S.id0, (int)(S.end - S.id0), pos, vel, velhalf, force, nthro, from_device));
    f->sys_loaded[sys] = 1;
    return GC_OK;
}

int gc_fused_load(GcFused* f, const float* pos, const float* vel, const float* velhalf, const float* force,
                  const int* nthro, int from_device) {
    if (!f || !pos) return gc_fail(GC_EINVAL, "fused_load: NULL argument");
    GC_TRY(load_range(f, 0, f->n, pos, vel, velhalf, force, nthro, from_device));
    for (int s = 0; s < f->nsys; ++s) f->sys_loaded[s] = 1;
    return GC_OK;
}

int gc_fused_setup(GcFused* f) {
    if (!f) return gc_fail(GC_EINVAL, "fused_setup: NULL handle");
    for (int s = 0; s < f->nsys; ++s)
        if (!f->sys_loaded[s]) return gc_fail(GC_ESTATE, "fused_setup: load the state of system %d first", s);
    if (f->setup_done) return gc_fail(GC_ESTATE, "fused_setup: already set up");
    cudaStream_t st = f->st;
    GC_TRY(finalize_cells(f));
    GC_TRY(build_grids(f));   // the aggregation grids exist once the cells are known
    const int n = f->n;
    GC_CUDA(cudaMemcpyAsync(f->a.vpred, f->a.vel, (size_t)n * sizeof(float4), cudaMemcpyDeviceToDevice, st),
            "fused: predicted velocity");
    if (f->a.sys) {
        fk_fill_sys<<<gc_blocks(n, 256), 256, 0, st>>>(n, f->dsys, f->nsys, f->a.sys);
        GC_CHECK_LAUNCH("fused: system of each slot");
    }
    GcParams p = f->p;
    if (f->ncell > 0) {
        fk_gather_mpos<<<gc_blocks(f->ncp, 256), 256, 0, st>>>(f->ncp, f->dsys, f->msys, f->slot_of, f->a.pos,
                                                              f->a.nthro, f->a.plo, f->mpos, f->mplo, f->mnthro);
        GC_CHECK_LAUNCH("fused: membrane positions");
        fk_mgeo<<<f->ncell, 256, 0, st>>>(p, f->dsys, f->cellsys, f->ncell, f->ntri, f->tri, f->betri, f->mpos,
                                         f->mplo, f->mnthro, f->tarea, f->tnorm, f->tcen, f->reftarea, f->carea, f->cvol,
                                         f->crefarea, f->crefvol, 1, f->flags);
        GC_CHECK_LAUNCH("fused: set-up geometry");
        fk_mech_setup<<<gc_blocks(f->nedge, f->block), f->block, 0, st>>>(
            p, f->dsys, f->msys, f->nedge, f->edge, f->mpos, f->mplo, f->mnthro, f->shear, f->bend, f->l0, f->lmax, f->perlen,
            f->hpow, f->hbend, f->refang, f->flags);
        GC_CHECK_LAUNCH("fused: set-up mechanics");
        GC_TRY(build_morse_lists(f, st, f->mpos, true));
        GC_TRY(launch_membranes(f, st, p));   // membrane outputs of the loaded state
    }
    f->step = -1;
    GC_TRY(sync_dstep(f));
    GC_TRY(rebuild_lists(f));
    // density and pressure of the loaded state (the reference has them from
    // DenInit until the first step recomputes them)
    GC_TRY(launch_density(f, st, p, false));
    f->setup_done = true;
    return GC_OK;
}

int gc_fused_step(GcFused* f, int nsteps, int drive_on) {
    if (!f || !f->setup_done) return gc_fail(GC_ESTATE, "fused_step: call gc_fused_setup first");
    if (nsteps < 0) return gc_fail(GC_EINVAL, "fused_step: nsteps < 0");
    int drive = drive_on ? 1 : 0;
    if (f->graph && !f->profile) return graph_steps(f, nsteps, drive);
    for (int k = 0; k < nsteps; ++k) GC_TRY(one_step(f, drive));
    return GC_OK;
}


int gc_fused_store(GcFused* f, float* pos, float* vel, float* rho, float* press, float* force, float* velhalf,
                   int* nthro, int to_device) {
    if (!f) return gc_fail(GC_EINVAL, "fused_store: NULL handle");
    return store_range(f, 0, f->n, pos, vel, rho, press, force, velhalf, nthro, to_device);
}

int gc_ensemble_store(GcFused* f, int sys, float* pos, float* vel, float* rho, float* press, float* force,
                      float* velhalf, int* nthro, int to_device) {
    GC_TRY(check_sys(f, sys, "store"));
    const SysInfo& S = f->hsys[sys];
    return store_range(f, S.id0, (int)(S.end - S.id0), pos, vel, rho, press, force, velhalf, nthro, to_device);
}


int gc_fused_store_cells(GcFused* f, float* area, float* vol, float* defforce, float* aggforce, float* trinordir,
                         float* tricenter, float* pararea, int to_device) {
    if (!f) return gc_fail(GC_EINVAL, "fused_store_cells: NULL handle");
    return store_cells_range(f, 0, f->ncell, 0, f->ncp, 0, f->ntri, area, vol, defforce, aggforce, trinordir,
                             tricenter, pararea, to_device);
}

int gc_fused_step_store(GcFused* f, int drive_on, float* pos, float* vel, float* rho, float* press, float* force,
                        float* velhalf, int* nthro, float* area, float* vol, float* defforce, float* aggforce,
                        float* trinordir, float* tricenter, float* pararea) {
    if (!f || !f->setup_done) return gc_fail(GC_ESTATE, "fused_step_store: call gc_fused_setup first");
    if (f->graph && !f->profile) {   // captured steps: the step, then the stores
        GC_TRY(gc_fused_step(f, 1, drive_on));
        GC_TRY(store_range(f, 0, f->n, pos, vel, rho, press, force, velhalf, nthro, 0));
        return store_cells_range(f, 0, f->ncell, 0, f->ncp, 0, f->ntri, area, vol, defforce, aggforce, trinordir,
                                 tricenter, pararea, 0);
    }
    GC_TRY(stage_bytes(f, particle_stage_bytes(f->n) + cells_stage_bytes(f->ncell, f->ncp, f->ntri)));
    GC_TRY(ensure_early_stream(f));
    EarlyStore e{pos, vel, rho, press, force, velhalf, nthro, area, vol, defforce, aggforce, trinordir, tricenter,
                 pararea};
    f->es = &e;
    f->early = early_store;
    const int rc = one_step(f, drive_on ? 1 : 0);
    f->early = nullptr;
    f->es = nullptr;
    cudaStreamSynchronize(f->xst);
    GC_TRY(rc);
    GC_CUDA(cudaStreamSynchronize(f->st), "fused_step_store");
    return GC_OK;
}

int gc_ensemble_store_cells(GcFused* f, int sys, float* area, float* vol, float* defforce, float* aggforce,
                            float* trinordir, float* tricenter, float* pararea, int to_device) {
    GC_TRY(check_sys(f, sys, "store_cells"));
    if (!f->setup_done) return gc_fail(GC_ESTATE, "store_cells: call gc_fused_setup first");
    const HostCells& h = f->hcells[sys];
    if (!h.set) return GC_OK;
    const SysInfo& S = f->hsys[sys];
    return store_cells_range(f, f->c0[sys], h.ncell, (int)S.m0, (int)(S.end - S.cs), f->t0[sys], h.ntri, area, vol,
                             defforce, aggforce, trinordir, tricenter, pararea, to_device);
}


int gc_fused_cell_sums(GcFused* f, double* area, double* vol) {
    if (!f) return gc_fail(GC_EINVAL, "fused_cell_sums: NULL handle");
    return cell_sums_range(f, 0, f->ncell, area, vol);
}

int gc_ensemble_cell_sums(GcFused* f, int sys, double* area, double* vol) {
    GC_TRY(check_sys(f, sys, "cell_sums"));
    if (!f->setup_done || !f->hcells[sys].set) return GC_OK;
    return cell_sums_range(f, f->c0[sys], f->hcells[sys].ncell, area, vol);
}

int gc_fused_stats(GcFused* f, long long* rebuilds, long long* steps, int* list_capacity, double* mean_neighbors,
                   int* max_neighbors) {
    if (!f) return gc_fail(GC_EINVAL, "fused_stats: NULL handle");
    if (rebuilds) *rebuilds = f->rebuilds;
    if (steps) *steps = f->steps;
    if (list_capacity) *list_capacity = f->cap;
    if (!f->lists && mean_neighbors) {
        // pair tiles: each candidate pair counts for both of its particles
        unsigned long long pairs = 0;
        GC_CUDA(cudaMemcpyAsync(&pairs, f->tpairs, 8, cudaMemcpyDeviceToHost, f->st), "stats");
        GC_CUDA(cudaStreamSynchronize(f->st), "stats");
        *mean_neighbors = 2.0 * (double)pairs / (f->n > 0 ? f->n : 1);
        mean_neighbors = nullptr;
    }
    if (mean_neighbors || max_neighbors) {
        GC_CUDA(cudaMemsetAsync(f->stat_sum, 0, sizeof(unsigned long long), f->st), "stats");
        GC_CUDA(cudaMemsetAsync(f->stat_max, 0, sizeof(int), f->st), "stats");
        fk_count_stats<<<gc_blocks(f->n, 256), 256, 0, f->st>>>(f->n, f->cnt, f->stat_sum, f->stat_max);
        GC_CHECK_LAUNCH("fused: stats");
        unsigned long long s = 0;
        int m = 0;
        GC_CUDA(cudaMemcpyAsync(&s, f->stat_sum, 8, cudaMemcpyDeviceToHost, f->st), "stats");
        GC_CUDA(cudaMemcpyAsync(&m, f->stat_max, 4, cudaMemcpyDeviceToHost, f->st), "stats");
        GC_CUDA(cudaStreamSynchronize(f->st), "stats");
        if (mean_neighbors) *mean_neighbors = (double)s / (f->n > 0 ? f->n : 1);
        if (max_neighbors) *max_neighbors = m;   // with pair tiles: the walls' lists
    }
    return GC_OK;
}

int gc_fused_flags(GcFused* f, unsigned* flags) {
    if (!f || !flags) return gc_fail(GC_EINVAL, "fused_flags: NULL argument");
    GC_CUDA(cudaMemcpyAsync(flags, f->flags, sizeof(unsigned), cudaMemcpyDeviceToHost, f->st), "flags");
    GC_CUDA(cudaMemsetAsync(f->flags, 0, sizeof(unsigned), f->st), "flags");
    GC_CUDA(cudaStreamSynchronize(f->st), "flags");
    return GC_OK;
}

int gc_fused_profile(GcFused* f, int enable) {
    if (!f) return gc_fail(GC_EINVAL, "fused_profile: NULL handle");
    f->profile = enable != 0;
    f->ev_used = 0;
    return GC_OK;
}

int gc_fused_profile_read(GcFused* f, double* density_ms, double* force_ms, long long* launches) {
    if (!f) return gc_fail(GC_EINVAL, "fused_profile_read: NULL handle");
    GC_CUDA(cudaStreamSynchronize(f->st), "fused_profile_read");
    double d = 0.0, fo = 0.0;
    size_t k = 0;
    for (; k + 4 <= f->ev_used; k += 4) {
        float a = 0.f, b = 0.f;
        GC_CUDA(cudaEventElapsedTime(&a, f->ev[k], f->ev[k + 1]), "fused_profile_read");
        GC_CUDA(cudaEventElapsedTime(&b, f->ev[k + 2], f->ev[k + 3]), "fused_profile_read");
        d += a;
        fo += b;
    }
    if (density_ms) *density_ms = d;
    if (force_ms) *force_ms = fo;
    if (launches) *launches = (long long)(k / 4);
    f->ev_used = 0;
    return GC_OK;
}

int gc_fused_get_options(GcFused* f, GcFusedOptions* opt) {
    if (!f || !opt) return gc_fail(GC_EINVAL, "fused_get_options: NULL argument");
    memset(opt, 0, sizeof(*opt));
    opt->skin = f->skin_rel;
    opt->block = f->block;
    opt->list_capacity = f->cap;
    opt->compact = f->compact ? 1 : 0;
    opt->graph = f->graph ? 1 : 0;
    opt->tiles = f->lists ? 0 : 1;
    opt->fp32_positions = f->ddpos ? 0 : 1;
    opt->half_velocity = f->halfv ? 1 : 0;
    return GC_OK;
}

int gc_fused_set_options(GcFused* f, const GcFusedOptions* opt) {
    if (!f || !opt) return gc_fail(GC_EINVAL, "fused_set_options: NULL argument");
    float old_skin = f->skin_rel;
    bool old_compact = f->compact;
    bool old_lists = f->lists;
    int old_block = f->block;
    GC_TRY(apply_options(f, opt));
    f->skin = f->skin_rel * f->p.rc;
    f->ens = f->nsys > 1;
    bool regrid = f->skin_rel != old_skin || f->lists != old_lists;
    if (regrid) GC_TRY(build_grids(f));
    int cap = f->cap;
    if (opt->list_capacity > cap) cap = (opt->list_capacity + 7) & ~7;
    if (regrid) {
        double grow = pow((f->p.rc + f->skin) / (f->p.rc + old_skin * f->p.rc), 3.0);
        if (grow > 1.0) cap = ((int)(cap * grow) + 8) & ~7;
    }
    GC_TRY(alloc_list(f, cap));
    if (f->compact != old_compact || f->block != old_block) drop_graphs(f);
    if (f->lists && !old_lists && cap < 16) cap = 64;   // every slot lists again (grown on overflow)
    if (f->lists != old_lists) GC_TRY(alloc_list(f, cap));
    if (f->setup_done) {
        GC_TRY(sync_dstep(f));
        if (regrid || f->compact != old_compact || opt->list_capacity > 0) GC_TRY(refresh(f));
    }
    return GC_OK;
}

int gc_fused_destroy(GcFused* f) {
    if (!f) return GC_OK;
    cudaStreamSynchronize(f->st);
    for (int d = 0; d < 2; ++d) {
        if (f->gexec[d]) cudaGraphExecDestroy(f->gexec[d]);
        if (f->cg[d]) cudaGraphDestroy(f->cg[d]);
    }
    if (f->mst) cudaStreamSynchronize(f->mst);
    if (f->gst) cudaStreamDestroy(f->gst);
    if (f->gst2) cudaStreamDestroy(f->gst2);
    if (f->gst3) cudaStreamDestroy(f->gst3);
    if (f->mst) cudaStreamDestroy(f->mst);
    if (f->ev_fork) cudaEventDestroy(f->ev_fork);
    if (f->ev_join) cudaEventDestroy(f->ev_join);
    for (int c = 0; c < 4; ++c)
        if (f->xev[c]) cudaEventDestroy(f->xev[c]);
    if (f->sortmem_agg) cudaFree(f->sortmem_agg);
    for (void* q : {(void*)f->moff, (void*)f->mcnt, (void*)f->mscan, (void*)f->mlist, (void*)f->mref})
        if (q) cudaFree(q);
    if (f->xst) cudaStreamSynchronize(f->xst);
    for (int k = 0; k < 4; ++k)
        if (f->xe[k]) cudaEventDestroy(f->xe[k]);
    if (f->xst) cudaStreamDestroy(f->xst);
    for (cudaEvent_t e : f->ev) cudaEventDestroy(e);
    for (void* q : f->allocs) cudaFree(q);
    if (f->nbr) cudaFree(f->nbr);
    if (f->cmask) cudaFree(f->cmask);
    for (void* q : {(void*)f->cube_sys, (void*)f->bmask, (void*)f->tnb, (void*)f->toff, (void*)f->tscan,
                    (void*)f->tent, (void*)f->pd, (void*)f->pf, (void*)f->tpairs})
        if (q) cudaFree(q);
    if (f->sortmem) cudaFree(f->sortmem);
    if (f->stage) cudaFree(f->stage);
    if (f->h) cudaFreeHost(f->h);
    delete f;
    return GC_OK;
}

}  // extern "C"


