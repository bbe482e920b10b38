// fused.cu -- the fused SDPD + membrane timestep on library-owned state.
//
// Same method and the same step order as the boundary entry points
// (Particle::UpdatePar, src/Particle.cu:1310-1329), restructured for the GPU:
//
//   * State lives in the library, in slot order (sorted by cube), as float4
//     records: position + id, velocity, predicted velocity, VelHalf, force,
//     and (1/d, P/d^2) per particle.  Membrane vertices additionally have a
//     membrane-ordered copy of their position and crossing counts, so the
//     membrane kernels index topology directly.
//   * Neighbours come from Verlet lists with a skin: built from a 27-cube
//     scan at cut-off rc + skin, stored 32 slots interleaved (entry k of slot
//     i at ((i/32)*cap + k)*32 + i%32, so a warp reads 128 contiguous bytes
//     per k), and rebuilt (with a re-sort) only when some particle has moved
//     more than skin/2 since the last build.  Every step still tests
//     r^2 < rc^2 with the same FP32 expression as the boundary kernels, so
//     the pairs that interact are exactly the same.
//   * Passes are fused: integrate + periodic wrap + predictor (K2, K3, K9);
//     density + equation of state + wall velocity (K8, K11, K10); SDPD +
//     wall repulsion + body force + membrane forces + corrector (K12, K13,
//     K14, K17/K18 add, K19); wall velocity again (K10).
//   * Per-cell membrane area and volume are summed in FP64.
#include "gc_internal.cuh"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <utility>
#include <vector>

namespace {

constexpr int kBS = 128;      // default threads per block
constexpr int kMaxBS = 256;   // largest block the particle kernels accept

__device__ __forceinline__ unsigned fid(float4 x) { return __float_as_uint(x.w); }
__device__ __forceinline__ float3 xyz(float4 a) { return f3(a.x, a.y, a.z); }

__device__ __forceinline__ size_t sell(int i, int k, int cap) {
    return ((size_t)(i >> 5) * cap + k) * 32 + (i & 31);
}

// Box constants of the per-step kernels.
struct Box {
    float L[3], invL[3];
    int pmask;
};

// Minimum image of a list pair.  A listed pair is either far closer than
// L/2 or close to L apart along a periodic axis, so d - L rint(d/L) makes
// the same shift as the conditional form of the boundary kernels and
// rounds the same way (one subtraction of L), i.e. the same FP32 value.
__device__ __forceinline__ float3 pair_image(float3 a, float3 b, const Box& B) {
    float3 d = f3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
    if (B.pmask & 1) d.x = fmaf(-B.L[0], rintf(d.x * B.invL[0]), d.x);
    if (B.pmask & 2) d.y = fmaf(-B.L[1], rintf(d.y * B.invL[1]), d.y);
    if (B.pmask & 4) d.z = fmaf(-B.L[2], rintf(d.z * B.invL[2]), d.z);
    return d;
}

// ---------------------------------------------------------------------------
// K2 + K3 + K9 for fluid and membrane slots
// ---------------------------------------------------------------------------
__global__ void fk_integrate(int n, GcParams p, float4* __restrict__ pos, const float4* __restrict__ vel,
                             float4* __restrict__ vh, float4* __restrict__ vpred, const float4* __restrict__ force,
                             const float4* __restrict__ refpos, int4* __restrict__ nthro, float half_skin2,
                             int* __restrict__ rebuild, float4* __restrict__ mpos, int4* __restrict__ mnthro,
                             unsigned* flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool far = false;
    if (i < n) {
        float4 x = pos[i];
        unsigned id = fid(x);
        if (is_mobile(id, p)) {
            float4 v = vel[i], f = force[i];
            float h = 0.5f * p.dt * p.dt * p.inv_mass;
            x.x += p.dt * v.x + h * f.x;
            x.y += p.dt * v.y + h * f.y;
            x.z += p.dt * v.z + h * f.z;
            if (!(isfinite(x.x) && isfinite(x.y) && isfinite(x.z))) raise_flag(flags, GC_FLAG_NONFINITE);
            int4 t = nthro[i];
            bool crossed = false;
            float* xs[3] = {&x.x, &x.y, &x.z};
            int* ts[3] = {&t.x, &t.y, &t.z};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (!(p.g.pmask & (1 << a))) continue;
                float c = *xs[a];
                if (c >= p.g.hi[a]) { c -= p.g.L[a]; *ts[a] += 1; crossed = true; }
                else if (c < p.g.lo[a]) { c += p.g.L[a]; *ts[a] -= 1; crossed = true; }
                *xs[a] = c;
            }
            if (crossed) nthro[i] = t;
            pos[i] = x;
            float hs = 0.5f * p.dt * p.inv_mass, l = p.lambda * p.dt * p.inv_mass;
            float4 w = vh[i];
            vh[i] = make_float4(v.x + hs * f.x, v.y + hs * f.y, v.z + hs * f.z, w.w);
            vpred[i] = make_float4(v.x + l * f.x, v.y + l * f.y, v.z + l * f.z, 0.f);
            float3 d = min_image(xyz(x), xyz(refpos[i]), p.g);
            far = norm2_rn(d) > half_skin2;
            if (id >= p.nC) {
                unsigned m = id - p.nC;
                mpos[m] = x;
                mnthro[m] = t;
            }
        }
    }
    if (__any_sync(0xffffffffu, far) && (threadIdx.x & 31) == 0) atomicOr(rebuild, 1);
}

// ---------------------------------------------------------------------------
// Rebuild: cube keys, permutation, neighbour lists
// ---------------------------------------------------------------------------
__global__ void fk_cellkey(int n, GcGrid g, const float4* __restrict__ pos, int* __restrict__ keys,
                           int* __restrict__ vals) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 x = pos[i];
    keys[i] = cube_key(cube_coord(x.x, 0, g), cube_coord(x.y, 1, g), cube_coord(x.z, 2, g), g);
    vals[i] = i;
}

struct SlotArrays {
    float4 *pos, *vel, *vpred, *vh, *force;
    int4* nthro;
};

// Gathers the slot arrays into the new order and wraps every position into
// the box on periodic axes (counting the crossings), so that the list build
// can use one image shift per row of cubes.
__global__ void fk_permute(int n, GcGrid g, const int* __restrict__ perm, SlotArrays src, SlotArrays dst,
                           float4* __restrict__ refpos, int* __restrict__ slot_of) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    int o = perm[q];
    float4 x = src.pos[o];
    int4 t = src.nthro[o];
    float* xs[3] = {&x.x, &x.y, &x.z};
    int* ts[3] = {&t.x, &t.y, &t.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (!(g.pmask & (1 << a))) continue;
        float c = *xs[a];
        if (!isfinite(c)) continue;
        int w = (int)floorf((c - g.lo[a]) / g.L[a]);
        if (w != 0) {
            c -= (float)w * g.L[a];
            if (c >= g.hi[a]) { c -= g.L[a]; ++w; }
            else if (c < g.lo[a]) { c += g.L[a]; --w; }
            *xs[a] = c;
            *ts[a] += w;
        }
    }
    dst.pos[q] = x;
    dst.vel[q] = src.vel[o];
    dst.vpred[q] = src.vpred[o];
    dst.vh[q] = src.vh[o];
    dst.force[q] = src.force[o];
    dst.nthro[q] = t;
    refpos[q] = x;
    slot_of[fid(x)] = q;
}

// One thread per slot scans the cubes of the list grid around its own.
// Fluid and membrane slots list every particle within rc + skin; Bound2
// slots list the moving particles (for their wall velocity); Bound1 slots
// list nothing.  Positions are inside the box on periodic axes (the
// permutation wraps them), so each neighbouring row of cubes has one image
// shift, and the three cubes of a row that do not wrap are one contiguous
// range of slots.
__global__ void __launch_bounds__(kMaxBS) fk_build_list(int n, GcParams p, const float4* __restrict__ pos,
                                                     const unsigned* __restrict__ start, int* __restrict__ nbr,
                                                     int* __restrict__ cnt, int cap, float cut2, unsigned* flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 xi4 = pos[i];
    float3 xi = xyz(xi4);
    unsigned id = fid(xi4);
    int t = ptype(id, p);
    int k = 0;
    const GcGrid& g = p.g;
    auto scan = [&](unsigned b, unsigned e, float sx, float sy, float sz) {
        for (unsigned j = b; j < e; ++j) {
            float4 xj = pos[j];
            float dx = (xi.x - xj.x) + sx, dy = (xi.y - xj.y) + sy, dz = (xi.z - xj.z) + sz;
            float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 >= cut2 || (int)j == i) continue;
            if (t == PT_B2 && !is_mobile(fid(xj), p)) continue;
            if (k < cap) nbr[sell(i, k, cap)] = (int)j;
            ++k;
        }
    };
    if (t != PT_B1) {
        int cx = cube_coord(xi.x, 0, g), cy = cube_coord(xi.y, 1, g), cz = cube_coord(xi.z, 2, g);
        for (int dz = -1; dz <= 1; ++dz) {
            int z = cz + dz;
            float sz = 0.f;
            if (z < 0) { if (!(g.pmask & 4)) continue; z += g.n[2]; sz = g.L[2]; }
            else if (z >= g.n[2]) { if (!(g.pmask & 4)) continue; z -= g.n[2]; sz = -g.L[2]; }
            for (int dy = -1; dy <= 1; ++dy) {
                int y = cy + dy;
                float sy = 0.f;
                if (y < 0) { if (!(g.pmask & 2)) continue; y += g.n[1]; sy = g.L[1]; }
                else if (y >= g.n[1]) { if (!(g.pmask & 2)) continue; y -= g.n[1]; sy = -g.L[1]; }
                int row = g.n[0] * (y + g.n[1] * z);
                if (cx >= 1 && cx + 1 < g.n[0]) {
                    scan(start[row + cx - 1], start[row + cx + 2], 0.f, sy, sz);
                } else {
                    for (int dx = -1; dx <= 1; ++dx) {
                        int x = cx + dx;
                        float sx = 0.f;
                        if (x < 0) { if (!(g.pmask & 1)) continue; x += g.n[0]; sx = g.L[0]; }
                        else if (x >= g.n[0]) { if (!(g.pmask & 1)) continue; x -= g.n[0]; sx = -g.L[0]; }
                        scan(start[row + x], start[row + x + 1], sx, sy, sz);
                    }
                }
            }
        }
    }
    if (k > cap) {
        raise_flag(flags, GC_FLAG_CELL_OVERFLOW);
        k = cap;
    }
    cnt[i] = k;
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
__device__ __forceinline__ size_t mrow(int i, int w, int mw) {
    return ((size_t)(i >> 5) * mw + w) * 32 + (i & 31);
}

__global__ void __launch_bounds__(kMaxBS) fk_density(int n, GcParams p, Box B, const float4* __restrict__ pos,
                                                  float4* __restrict__ vpred, const float4* __restrict__ vh,
                                                  float2* __restrict__ dp, const int* __restrict__ nbr,
                                                  const int* __restrict__ cnt, int cap, unsigned* __restrict__ cmask,
                                                  int mw, int* __restrict__ ccnt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 xi4 = pos[i];
    float3 xi = xyz(xi4);
    unsigned id = fid(xi4);
    int t = ptype(id, p);
    int c = cnt[i];
    const int* lp = nbr + sell(i, 0, cap);
    if (t == PT_FLUID || t == PT_MEMB) {
        float sum = p.w0;
        int kc = 0;
        unsigned m = 0;
        int jn = c > 0 ? __ldg(lp) : 0;
        float4 xn = pos[jn];
        for (int k = 0; k < c; ++k) {
            float4 xj = xn;
            if (k + 1 < c) {
                jn = __ldg(lp + (size_t)(k + 1) * 32);
                xn = pos[jn];
            }
            float r2 = norm2_rn(pair_image(xi, xyz(xj), B));
            if (r2 < p.rc2) {
                if (is_sdpd(fid(xj), p)) {
                    float r = r2 > 0.f ? r2 * rsqrtf(r2) : 0.f;
                    sum += wendland_w(r, p);
                    if (r2 > 0.f) m |= 1u << (k & 31);
                } else if (r2 < p.rep_r0sq && r2 > 0.f) {
                    m |= 1u << (k & 31);
                }
            }
            if (cmask && ((k & 31) == 31 || k + 1 == c)) {
                cmask[mrow(i, k >> 5, mw)] = m;
                kc += __popc(m);
                m = 0;
            }
        }
        if (ccnt) ccnt[i] = kc;
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
// so the cut-off test is already done.
template <bool COMPACT>
__global__ void __launch_bounds__(kMaxBS, 6) fk_force(int n, GcParams p, Box B, const float4* __restrict__ pos,
                                                const float4* __restrict__ vpred, const float4* __restrict__ vh,
                                                const float2* __restrict__ dp, float4* __restrict__ force,
                                                float4* __restrict__ vel, const int* __restrict__ nbr,
                                                const int* __restrict__ cnt, int cap,
                                                const unsigned* __restrict__ cmask, int mw,
                                                const float4* __restrict__ mforce, int drive) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 xi4 = pos[i];
    float3 xi = xyz(xi4);
    unsigned id = fid(xi4);
    if (!is_mobile(id, p)) {
        force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    float4 vi = vpred[i];
    float2 dpi = dp[i];
    bool noise = p.noise_pref > 0.f;
    float3 f = f3(0.f, 0.f, 0.f);
    int c = cnt[i];
    const int* lp = nbr + sell(i, 0, cap);
    const unsigned* mp = COMPACT ? cmask + mrow(i, 0, mw) : nullptr;
    unsigned m = 0;
    int base = -32;
    // index of the next acting entry (COMPACT) or of the next entry
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
    int jn = 0;
    float4 xn;
    if (c > 0) {
        jn = __ldg(lp + (size_t)next_k(0) * 32);
        xn = pos[jn];
    }
    for (int k = 0; k < c; ++k) {
        int j = jn;
        float4 xj4 = xn;
        if (k + 1 < c) {   // prefetch the next entry while this one is computed
            jn = __ldg(lp + (size_t)next_k(k + 1) * 32);
            xn = pos[jn];
        }
        float3 d = pair_image(xi, xyz(xj4), B);
        float r2 = norm2_rn(d);
        if (!COMPACT && (r2 >= p.rc2 || r2 <= 0.f)) continue;   // coincident pairs exert no force
        unsigned idj = fid(xj4);
        float inv_r = rsqrtf(r2);
        if (!is_sdpd(idj, p)) {   // Bound1: repulsion only
            if (r2 < p.rep_r0sq) {
                float ir2 = inv_r * inv_r;
                float q2 = p.rep_r0sq * ir2, q4 = q2 * q2, q12 = q4 * q4 * q4;
                f += (p.rep_D * (q12 - q4) * ir2) * d;
            }
            continue;
        }
        float2 dpj = dp[j];
        float4 vj = vpred[j];
        float r = r2 * inv_r;
        float F = wendland_f(r, p);
        f += ((dpi.y + dpj.y) * F) * d;
        float3 e = inv_r * d;
        float3 vij = f3(vi.x - vj.x, vi.y - vj.y, vi.z - vj.z);
        float ev = dot3(e, vij);
        float fdd = F * dpi.x * dpj.x;
        f -= fdd * (p.visA * vij + (p.visB * ev) * e);
        if (noise) {
            float qq = p.noise_pref * fdd;
            float q = qq > 0.f ? qq * rsqrtf(qq) : 0.f;
            q = id < idj ? q : -q;   // the pair sign of xi_ij
            float3 xi_ = pair_noise_unsigned(id, idj, p);
            float exi = dot3(e, xi_);
            f += q * (p.sqrtA * xi_ + ((p.sqrtAB - p.sqrtA) * exi) * e);
        }
    }
    if (drive) f.x += p.gx;
    if (id >= p.nC && mforce) {
        float4 mf = mforce[id - p.nC];
        f += f3(mf.x, mf.y, mf.z);
    }
    // a non-finite force shows up as a non-finite position in the next
    // fk_integrate, which raises GC_FLAG_NONFINITE
    force[i] = make_float4(f.x, f.y, f.z, 0.f);
    float4 h = vh[i];
    float s = 0.5f * p.dt * p.inv_mass;
    vel[i] = make_float4(h.x + s * f.x, h.y + s * f.y, h.z + s * f.z, 0.f);
}

// second K10: wall velocity from the corrected velocities
__global__ void fk_wallvel(int n, GcParams p, Box B, const float4* __restrict__ pos, float4* __restrict__ vel,
                           const float4* __restrict__ vh, const int* __restrict__ nbr, const int* __restrict__ cnt,
                           int cap) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 xi4 = pos[i];
    if (ptype(fid(xi4), p) != PT_B2) return;
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
// Membranes (membrane order; positions unwrapped with crossing counts)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float3 mdiff(const float4* mpos, const int4* mnt, int a, int b, const GcGrid& g) {
    float4 xa = mpos[a], xb = mpos[b];
    int4 ta = mnt[a], tb = mnt[b];
    float3 d = f3(xa.x - xb.x, xa.y - xb.y, xa.z - xb.z);
    if (g.pmask & 1) d.x += (float)(ta.x - tb.x) * g.L[0];
    if (g.pmask & 2) d.y += (float)(ta.y - tb.y) * g.L[1];
    if (g.pmask & 4) d.z += (float)(ta.z - tb.z) * g.L[2];
    return d;
}

__device__ double block_sum_d(double v, double* sh) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) sh[0] = t;
    }
    __syncthreads();
    double t = sh[0];
    __syncthreads();
    return t;
}

// Triangle geometry and per-cell area/volume (FP64 sums), one block per cell.
__global__ void fk_mgeo(GcParams p, int ncell, int ntri, const int3* __restrict__ tri, const int2* __restrict__ betri,
                        const float4* __restrict__ mpos, const int4* __restrict__ mnt, float* __restrict__ tarea,
                        float4* __restrict__ tnorm, float4* __restrict__ tcen, float* __restrict__ reftarea,
                        double* __restrict__ carea, double* __restrict__ cvol, double* __restrict__ crefarea,
                        double* __restrict__ crefvol, float* __restrict__ parea, int setup, unsigned* flags) {
    __shared__ double sh[32];
    int c = blockIdx.x;
    int2 be = betri[c];
    if (be.x < 0 || be.y >= ntri || be.y < be.x) {
        if (threadIdx.x == 0) raise_flag(flags, GC_FLAG_BAD_INDEX);
        return;
    }
    int r = tri[be.x].x - 1;
    float4 xr = mpos[r];
    int4 tr = mnt[r];
    float3 xru = f3(xr.x, xr.y, xr.z);
    if (p.g.pmask & 1) xru.x += (float)tr.x * p.g.L[0];
    if (p.g.pmask & 2) xru.y += (float)tr.y * p.g.L[1];
    if (p.g.pmask & 4) xru.z += (float)tr.z * p.g.L[2];
    double accA = 0.0, accV = 0.0;
    for (int t = be.x + threadIdx.x; t <= be.y; t += blockDim.x) {
        int3 v = tri[t];
        int a = v.x - 1, b = v.y - 1, cc = v.z - 1;
        if (a < 0 || b < 0 || cc < 0 || a >= (int)p.nCP || b >= (int)p.nCP || cc >= (int)p.nCP) {
            raise_flag(flags, GC_FLAG_BAD_INDEX);
            continue;
        }
        float3 u1 = mdiff(mpos, mnt, a, r, p.g);
        float3 e1 = mdiff(mpos, mnt, b, a, p.g), e2 = mdiff(mpos, mnt, cc, a, p.g);
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
        float a3 = A * (1.f / 3.f);
        atomicAdd(&parea[a], a3);
        atomicAdd(&parea[b], a3);
        atomicAdd(&parea[cc], a3);
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

__global__ void fk_mech_setup(GcParams p, int nedge, const int6* __restrict__ edge, const float4* __restrict__ mpos,
                              const int4* __restrict__ mnt, const float* __restrict__ shear,
                              const float* __restrict__ bend, float* __restrict__ l0a, float* __restrict__ lmax,
                              float* __restrict__ perlen, float* __restrict__ hpow, float* __restrict__ hbend,
                              float* __restrict__ refang, unsigned* flags) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nedge) return;
    int6 E = edge[e];
    int a = E.x - 1, b = E.y - 1, c = E.z - 1, d = E.k - 1;
    int ncp = (int)p.nCP;
    if (a < 0 || b < 0 || c < 0 || d < 0 || a >= ncp || b >= ncp || c >= ncp || d >= ncp) {
        raise_flag(flags, GC_FLAG_BAD_INDEX);
        return;
    }
    float3 xb = mdiff(mpos, mnt, b, a, p.g), xc = mdiff(mpos, mnt, c, a, p.g), xd = mdiff(mpos, mnt, d, a, p.g);
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

__device__ __forceinline__ void add4(float4* o, float3 f) {
    atomicAdd(&o->x, f.x);
    atomicAdd(&o->y, f.y);
    atomicAdd(&o->z, f.z);
}

__global__ void fk_medge(GcParams p, int nedge, const int6* __restrict__ edge, const float4* __restrict__ mpos,
                         const int4* __restrict__ mnt, const float* __restrict__ lmax,
                         const float* __restrict__ perlen, const float* __restrict__ hpow,
                         const float* __restrict__ refang, const float* __restrict__ hbend,
                         float4* __restrict__ mforce, unsigned* flags) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nedge) return;
    int6 E = edge[e];
    int a = E.x - 1, b = E.y - 1, c = E.z - 1, d = E.k - 1;
    int ncp = (int)p.nCP;
    if (a < 0 || b < 0 || c < 0 || d < 0 || a >= ncp || b >= ncp || c >= ncp || d >= ncp) {
        raise_flag(flags, GC_FLAG_BAD_INDEX);
        return;
    }
    float3 z = f3(0.f, 0.f, 0.f);
    float3 xb = mdiff(mpos, mnt, b, a, p.g), xc = mdiff(mpos, mnt, c, a, p.g), xd = mdiff(mpos, mnt, d, a, p.g);
    float3 f1 = z, f2 = z, f3v = z, f4 = z;
    float pl = perlen[e];
    float r = sqrtf(dot3(xb, xb));
    if (pl > 0.f && r > 0.f) {
        float x = r / lmax[e];
        if (x >= 0.99f) {
            raise_flag(flags, GC_FLAG_STRETCH);
            x = 0.99f;
        }
        float u = 1.f - x;
        float fm = -(p.kT / pl) * (1.f / (4.f * u * u) - 0.25f + x) + hpow[e] / (r * r);   // power index 2
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
    add4(&mforce[a], f1);
    add4(&mforce[b], f2);
    add4(&mforce[c], f3v);
    add4(&mforce[d], f4);
}

__global__ void fk_mtri(GcParams p, int ncell, const int2* __restrict__ betri, const int3* __restrict__ tri,
                        const float4* __restrict__ mpos, const int4* __restrict__ mnt,
                        const float* __restrict__ reftarea, const float* __restrict__ hl,
                        const float* __restrict__ hg, const float* __restrict__ hv, const double* __restrict__ carea,
                        const double* __restrict__ cvol, const double* __restrict__ crefarea,
                        const double* __restrict__ crefvol, float4* __restrict__ mforce, int ntri) {
    // one block per cell: the cell's coefficients are read once
    int c = blockIdx.x;
    int2 be = betri[c];
    if (be.x < 0 || be.y >= ntri || be.y < be.x) return;
    float dA = (float)((carea[c] - crefarea[c]) / crefarea[c]);
    float dV = (float)((cvol[c] - crefvol[c]) / crefvol[c]);
    int ncp = (int)p.nCP;
    for (int t = be.x + threadIdx.x; t <= be.y; t += blockDim.x) {
        int3 v = tri[t];
        int a = v.x - 1, b = v.y - 1, cc = v.z - 1;
        if (a < 0 || b < 0 || cc < 0 || a >= ncp || b >= ncp || cc >= ncp) continue;
        float3 x2 = mdiff(mpos, mnt, b, a, p.g), x3 = mdiff(mpos, mnt, cc, a, p.g);
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
        add4(&mforce[a], fv - cA * g1);
        add4(&mforce[b], fv - cA * g2);
        add4(&mforce[cc], fv - cA * g3);
    }
}

// Morse aggregation on a membrane-only grid (cubes at least MaxCut wide).
__global__ void fk_mkey(int ncp, GcGrid g, const float4* __restrict__ mpos, int* __restrict__ keys,
                        int* __restrict__ vals) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= ncp) return;
    float4 x = mpos[v];
    keys[v] = cube_key(cube_coord(x.x, 0, g), cube_coord(x.y, 1, g), cube_coord(x.z, 2, g), g);
    vals[v] = v;
}

__global__ void fk_magg(int ncp, GcParams p, GcGrid g, const int* __restrict__ order,
                        const unsigned* __restrict__ start, const float4* __restrict__ mpos,
                        const int* __restrict__ celltab, const float* __restrict__ parea, float4* __restrict__ magg,
                        float4* __restrict__ mforce) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ncp) return;
    int v = order[q];
    float4 x4 = mpos[v];
    float3 xi = xyz(x4);
    int ci = celltab[v];
    float ai = parea[v];
    int cx = cube_coord(xi.x, 0, g), cy = cube_coord(xi.y, 1, g), cz = cube_coord(xi.z, 2, g);
    float3 f = f3(0.f, 0.f, 0.f);
    for (int dz = -1; dz <= 1; ++dz) {
        int z = cube_step(cz, dz, 2, g);
        if (z < 0) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            int y = cube_step(cy, dy, 1, g);
            if (y < 0) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                int x = cube_step(cx, dx, 0, g);
                if (x < 0) continue;
                int c = cube_key(x, y, z, g);
                for (unsigned s = start[c]; s < start[c + 1]; ++s) {
                    int w = order[s];
                    if (celltab[w] == ci) continue;
                    float3 d = min_image(xi, xyz(mpos[w]), g);
                    float r2 = norm2_rn(d);
                    if (r2 >= p.maxcut2 || r2 <= 0.f) continue;
                    float r = sqrtf(r2);
                    float ex = __expf(p.beta * (p.r0m - r));
                    float fm = 2.f * p.De * p.beta * (ex * ex - ex) * 0.5f * (ai + parea[w]);
                    f += (fm / r) * d;
                }
            }
        }
    }
    magg[v] = make_float4(f.x, f.y, f.z, 0.f);
    float4* o = &mforce[v];
    o->x += f.x;   // one thread per vertex, after the deformation kernels
    o->y += f.y;
    o->z += f.z;
}

// ---------------------------------------------------------------------------
// Import / export in original order
// ---------------------------------------------------------------------------
__global__ void fk_load(int n, GcParams p, const float* __restrict__ x, const float* __restrict__ v,
                        const float* __restrict__ vhalf, const float* __restrict__ f, const int* __restrict__ nt,
                        float4* __restrict__ pos, float4* __restrict__ vel, float4* __restrict__ vh,
                        float4* __restrict__ force, int4* __restrict__ nthro) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pos[i] = make_float4(x[3 * i], x[3 * i + 1], x[3 * i + 2], __uint_as_float((unsigned)i));
    vel[i] = v ? make_float4(v[3 * i], v[3 * i + 1], v[3 * i + 2], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    vh[i] = vhalf ? make_float4(vhalf[3 * i], vhalf[3 * i + 1], vhalf[3 * i + 2], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    force[i] = f ? make_float4(f[3 * i], f[3 * i + 1], f[3 * i + 2], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    nthro[i] = nt ? make_int4(nt[3 * i], nt[3 * i + 1], nt[3 * i + 2], 0) : make_int4(0, 0, 0, 0);
}

// Load into the current slot order (a set-up handle keeps its lists; the
// displacement check decides whether they need a rebuild).
__global__ void fk_load_keep(int n, GcParams p, const int* __restrict__ slot_of, const float* __restrict__ x,
                             const float* __restrict__ v, const float* __restrict__ vhalf,
                             const float* __restrict__ f, const int* __restrict__ nt, float4* __restrict__ pos,
                             float4* __restrict__ vel, float4* __restrict__ vh, float4* __restrict__ force,
                             int4* __restrict__ nthro, float4* __restrict__ mpos, int4* __restrict__ mnthro) {
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    int i = slot_of[id];
    float4 a = make_float4(x[3 * id], x[3 * id + 1], x[3 * id + 2], __uint_as_float((unsigned)id));
    pos[i] = a;
    if (v) vel[i] = make_float4(v[3 * id], v[3 * id + 1], v[3 * id + 2], 0.f);
    if (vhalf) vh[i] = make_float4(vhalf[3 * id], vhalf[3 * id + 1], vhalf[3 * id + 2], 0.f);
    if (f) force[i] = make_float4(f[3 * id], f[3 * id + 1], f[3 * id + 2], 0.f);
    int4 t = nt ? make_int4(nt[3 * id], nt[3 * id + 1], nt[3 * id + 2], 0) : nthro[i];
    if (nt) nthro[i] = t;
    if (id >= (int)p.nC && mpos) {
        mpos[id - p.nC] = a;
        mnthro[id - p.nC] = t;
    }
}

__global__ void fk_store(int n, GcParams p, const float4* __restrict__ pos, const float4* __restrict__ vel,
                         const float4* __restrict__ vh, const float4* __restrict__ force,
                         const float2* __restrict__ dp, const int4* __restrict__ nthro, float* __restrict__ x,
                         float* __restrict__ v, float* __restrict__ rho, float* __restrict__ press,
                         float* __restrict__ f, float* __restrict__ vhalf, int* __restrict__ nt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = pos[i];
    unsigned id = fid(a);
    if (x) { x[3 * id] = a.x; x[3 * id + 1] = a.y; x[3 * id + 2] = a.z; }
    if (v) { float4 b = vel[i]; v[3 * id] = b.x; v[3 * id + 1] = b.y; v[3 * id + 2] = b.z; }
    if (vhalf) { float4 b = vh[i]; vhalf[3 * id] = b.x; vhalf[3 * id + 1] = b.y; vhalf[3 * id + 2] = b.z; }
    if (f) { float4 b = force[i]; f[3 * id] = b.x; f[3 * id + 1] = b.y; f[3 * id + 2] = b.z; }
    if (nt) { int4 b = nthro[i]; nt[3 * id] = b.x; nt[3 * id + 1] = b.y; nt[3 * id + 2] = b.z; }
    float2 q = dp[i];
    if (rho) rho[id] = p.mass / q.x;
    if (press) press[id] = q.y / (q.x * q.x);
}

__global__ void fk_store_cells(int ncp, int ntri, const float4* __restrict__ mforce, const float4* __restrict__ magg,
                               const float* __restrict__ parea, const float4* __restrict__ tnorm,
                               const float4* __restrict__ tcen, float* __restrict__ defforce,
                               float* __restrict__ aggforce, float* __restrict__ pararea, float* __restrict__ trinor,
                               float* __restrict__ tricen, int have_agg) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ncp) {
        float4 a = have_agg ? magg[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        float4 m = mforce[i];
        if (defforce) { defforce[3 * i] = m.x - a.x; defforce[3 * i + 1] = m.y - a.y; defforce[3 * i + 2] = m.z - a.z; }
        if (aggforce) { aggforce[3 * i] = a.x; aggforce[3 * i + 1] = a.y; aggforce[3 * i + 2] = a.z; }
        if (pararea) pararea[i] = parea[i];
    }
    if (i < ntri) {
        float4 b = tnorm[i], c = tcen[i];
        if (trinor) { trinor[3 * i] = b.x; trinor[3 * i + 1] = b.y; trinor[3 * i + 2] = b.z; }
        if (tricen) { tricen[3 * i] = c.x; tricen[3 * i + 1] = c.y; tricen[3 * i + 2] = c.z; }
    }
}

__global__ void fk_cast_cells(int ncell, const double* __restrict__ a, const double* __restrict__ v,
                              float* __restrict__ area, float* __restrict__ vol) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    if (area) area[c] = (float)a[c];
    if (vol) vol[c] = (float)v[c];
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

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

struct GcFused {
    GcParams p;
    GcGrid lgrid;                 // list/sort grid (cubes >= rc + skin)
    GcGrid mgrid;                 // membrane aggregation grid (cubes >= MaxCut)
    float skin = 0.1f;
    int n = 0, cap = 0, block = kBS;
    int noise_on = 1;
    long long step = -1;          // index keying the noise of the latest step
    long long rebuilds = 0, steps = 0;
    cudaStream_t st = 0;
    // slot arrays (current, and the permutation target)
    SlotArrays a{}, b{};
    float4* refpos = nullptr;
    float2* dp = nullptr;
    int* slot_of = nullptr;
    int *keys = nullptr, *vals = nullptr;
    int *nbr = nullptr, *cnt = nullptr;
    size_t nbr_elems = 0;
    bool compact = false;
    unsigned* cmask = nullptr;   // per-step bit mask of the acting list entries
    int* ccnt = nullptr;         // number of acting entries
    int mw = 0;                  // mask words per slot
    int* rebuild = nullptr;
    int* h_rebuild = nullptr;     // pinned
    unsigned* flags = nullptr;
    unsigned long long* stat_sum = nullptr;
    int* stat_max = nullptr;
    // membranes
    int ncell = 0, ntri = 0, nedge = 0, ncp = 0;
    int3* tri = nullptr;
    int6* edge = nullptr;
    int2* betri = nullptr;
    int* celltab = nullptr;
    float *shear = nullptr, *bend = nullptr, *hl = nullptr, *hg = nullptr, *hv = nullptr;
    float *l0 = nullptr, *lmax = nullptr, *perlen = nullptr, *hpow = nullptr, *hbend = nullptr, *refang = nullptr;
    float *tarea = nullptr, *reftarea = nullptr;
    float4 *tnorm = nullptr, *tcen = nullptr;
    double *carea = nullptr, *cvol = nullptr, *crefarea = nullptr, *crefvol = nullptr;
    float4 *mpos = nullptr, *mforce = nullptr, *magg = nullptr;
    int4* mnthro = nullptr;
    float* parea = nullptr;
    int *mkeys = nullptr, *mvals = nullptr;
    bool have_agg = false;
    bool setup_done = false;
    bool loaded = false;
    // optional CUDA-event timing of the dominant kernels (fk_density, fk_force)
    bool profile = false;
    std::vector<cudaEvent_t> ev;   // pairs: density start/stop, force start/stop
    size_t ev_used = 0;
    // staging for host pointers
    void* stage = nullptr;
    size_t stage_bytes = 0;
    std::vector<void*> allocs;
};

namespace {

template <class T>
int falloc(GcFused* f, T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, (count ? count : 1) * sizeof(T));
    if (e != cudaSuccess) return gc_fail(GC_ENOMEM, "fused: cudaMalloc(%zu) failed: %s", count * sizeof(T),
                                         cudaGetErrorString(e));
    f->allocs.push_back(q);
    *p = (T*)q;
    return GC_OK;
}

int stage_bytes(GcFused* f, size_t bytes) {
    if (f->stage_bytes >= bytes) return GC_OK;
    if (f->stage) cudaFree(f->stage);
    f->stage = nullptr;
    f->stage_bytes = 0;
    GC_CUDA(cudaMalloc(&f->stage, bytes), "fused: staging buffer");
    f->stage_bytes = bytes;
    return GC_OK;
}

int alloc_list(GcFused* f, int cap) {
    size_t need = (size_t)((f->n + 31) / 32) * 32 * (size_t)cap;
    if (f->nbr && need <= f->nbr_elems) {
        f->cap = cap;
        return GC_OK;
    }
    if (f->nbr) cudaFree(f->nbr);
    if (f->cmask) cudaFree(f->cmask);
    f->nbr = nullptr;
    f->cmask = nullptr;
    GC_CUDA(cudaMalloc(&f->nbr, need * sizeof(int)), "fused: neighbour lists");
    f->mw = (cap + 31) / 32;
    if (f->compact)
        GC_CUDA(cudaMalloc(&f->cmask, (size_t)((f->n + 31) / 32) * 32 * f->mw * sizeof(unsigned)), "fused: masks");
    f->nbr_elems = need;
    f->cap = cap;
    return GC_OK;
}

int rebuild_lists(GcFused* f) {
    const int n = f->n;
    const int nb = gc_blocks(n, f->block);
    cudaStream_t st = f->st;
    fk_cellkey<<<nb, f->block, 0, st>>>(n, f->lgrid, f->a.pos, f->keys, f->vals);
    GC_CHECK_LAUNCH("fused: cube keys");
    GC_TRY(gc_counting_sort(n, f->lgrid.ncells, f->keys, f->vals, st));
    fk_permute<<<nb, f->block, 0, st>>>(n, f->lgrid, f->vals, f->a, f->b, f->refpos, f->slot_of);
    GC_CHECK_LAUNCH("fused: permute");
    std::swap(f->a, f->b);
    GcParams lp = f->p;
    lp.g = f->lgrid;
    float cut = f->p.rc + f->skin;
    float cut2 = cut * cut;
    for (int attempt = 0; attempt < 4; ++attempt) {
        GC_CUDA(cudaMemsetAsync(f->flags, 0, sizeof(unsigned), st), "fused: flags");
        fk_build_list<<<nb, f->block, 0, st>>>(n, lp, f->a.pos, gc_sort_starts(), f->nbr, f->cnt, f->cap, cut2,
                                              f->flags);
        GC_CHECK_LAUNCH("fused: build lists");
        unsigned h = 0;
        GC_CUDA(cudaMemcpyAsync(&h, f->flags, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "fused: flags");
        GC_CUDA(cudaStreamSynchronize(st), "fused: flags");
        if (!(h & GC_FLAG_CELL_OVERFLOW)) break;
        if (attempt == 3) return gc_fail(GC_EDEVICE, "fused: neighbour lists overflow %d entries", f->cap);
        // a particle had more neighbours than the list holds: grow and rebuild
        GC_TRY(alloc_list(f, f->cap * 2));
    }
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

void prof_mark(GcFused* f) {
    if (!f->profile) return;
    cudaEvent_t e = prof_event(f);
    if (e) cudaEventRecord(e, f->st);
}

Box make_box(const GcGrid& g) {
    Box b;
    for (int a = 0; a < 3; ++a) {
        b.L[a] = g.L[a];
        b.invL[a] = 1.f / g.L[a];
    }
    b.pmask = g.pmask;
    return b;
}

int one_step(GcFused* f, int drive) {
    const int n = f->n;
    const Box B = make_box(f->lgrid);
    const int nb = gc_blocks(n, f->block);
    cudaStream_t st = f->st;
    f->step += 1;
    f->p.noise_key = noise_key(f->p.seed, (uint64_t)f->step);
    GcParams p = f->p;
    p.g = f->lgrid;
    float hs = 0.5f * f->skin * 0.99f;
    GC_CUDA(cudaMemsetAsync(f->rebuild, 0, sizeof(int), st), "fused: flag");
    fk_integrate<<<nb, f->block, 0, st>>>(n, p, f->a.pos, f->a.vel, f->a.vh, f->a.vpred, f->a.force, f->refpos,
                                         f->a.nthro, hs * hs, f->rebuild, f->mpos, f->mnthro, f->flags);
    GC_CHECK_LAUNCH("fused: integrate");
    GC_CUDA(cudaMemcpyAsync(f->h_rebuild, f->rebuild, sizeof(int), cudaMemcpyDeviceToHost, st), "fused: flag");
    GC_CUDA(cudaStreamSynchronize(st), "fused: flag");
    if (*f->h_rebuild) GC_TRY(rebuild_lists(f));
    prof_mark(f);
    fk_density<<<nb, f->block, 0, st>>>(n, p, B, f->a.pos, f->a.vpred, f->a.vh, f->dp, f->nbr, f->cnt, f->cap,
                                       f->compact ? f->cmask : nullptr, f->mw, f->compact ? f->ccnt : nullptr);
    GC_CHECK_LAUNCH("fused: density");
    prof_mark(f);
    if (f->ncell > 0) {
        GC_CUDA(cudaMemsetAsync(f->mforce, 0, (size_t)f->ncp * sizeof(float4), st), "fused: clear mforce");
        GC_CUDA(cudaMemsetAsync(f->parea, 0, (size_t)f->ncp * sizeof(float), st), "fused: clear parea");
        fk_mgeo<<<f->ncell, 256, 0, st>>>(p, f->ncell, f->ntri, f->tri, f->betri, f->mpos, f->mnthro, f->tarea,
                                         f->tnorm, f->tcen, f->reftarea, f->carea, f->cvol, f->crefarea, f->crefvol,
                                         f->parea, 0, f->flags);
        GC_CHECK_LAUNCH("fused: membrane geometry");
        fk_medge<<<gc_blocks(f->nedge, f->block), f->block, 0, st>>>(p, f->nedge, f->edge, f->mpos, f->mnthro,
                                                                     f->lmax, f->perlen, f->hpow, f->refang,
                                                                     f->hbend, f->mforce, f->flags);
        GC_CHECK_LAUNCH("fused: membrane edges");
        fk_mtri<<<f->ncell, 256, 0, st>>>(p, f->ncell, f->betri, f->tri, f->mpos, f->mnthro, f->reftarea, f->hl,
                                         f->hg, f->hv, f->carea, f->cvol, f->crefarea, f->crefvol, f->mforce,
                                         f->ntri);
        GC_CHECK_LAUNCH("fused: membrane triangles");
        if (f->have_agg) {
            fk_mkey<<<gc_blocks(f->ncp, f->block), f->block, 0, st>>>(f->ncp, f->mgrid, f->mpos, f->mkeys, f->mvals);
            GC_CHECK_LAUNCH("fused: aggregation keys");
            GC_TRY(gc_counting_sort(f->ncp, f->mgrid.ncells, f->mkeys, f->mvals, st));
            fk_magg<<<gc_blocks(f->ncp, f->block), f->block, 0, st>>>(f->ncp, p, f->mgrid, f->mvals, gc_sort_starts(),
                                                                      f->mpos, f->celltab, f->parea, f->magg,
                                                                      f->mforce);
            GC_CHECK_LAUNCH("fused: aggregation");
        }
    }
    prof_mark(f);
    if (f->compact)
        fk_force<true><<<nb, f->block, 0, st>>>(n, p, B, f->a.pos, f->a.vpred, f->a.vh, f->dp, f->a.force, f->a.vel,
                                               f->nbr, f->ccnt, f->cap, f->cmask, f->mw,
                                               f->ncell > 0 ? f->mforce : nullptr, drive);
    else
        fk_force<false><<<nb, f->block, 0, st>>>(n, p, B, f->a.pos, f->a.vpred, f->a.vh, f->dp, f->a.force, f->a.vel,
                                                f->nbr, f->cnt, f->cap, nullptr, 0,
                                                f->ncell > 0 ? f->mforce : nullptr, drive);
    GC_CHECK_LAUNCH("fused: force");
    prof_mark(f);
    if (p.nF > p.nB2) {
        fk_wallvel<<<nb, f->block, 0, st>>>(n, p, B, f->a.pos, f->a.vel, f->a.vh, f->nbr, f->cnt, f->cap);
        GC_CHECK_LAUNCH("fused: wall velocity");
    }
    f->steps++;
    return GC_OK;
}

}  // namespace

extern "C" {

int gc_fused_create(const Structconst* consts, const float* bbox6, int periodic_mask, int noise_on,
                    const GcFusedOptions* opt, GcFused** out) {
    if (!consts || !bbox6 || !out) return gc_fail(GC_EINVAL, "fused_create: NULL argument");
    if (periodic_mask < 0 || periodic_mask > 7) return gc_fail(GC_EINVAL, "fused_create: bad periodic mask");
    const Structconst& c = *consts;
    if (!(c.nBound2Start <= c.nFluidStart && c.nFluidStart <= c.nCellStart && c.nCellStart + c.nCellPar == c.nTotalPar))
        return gc_fail(GC_EINVAL, "fused_create: inconsistent type boundaries");
    if (c.nTotalPar >= (1u << 30)) return gc_fail(GC_EINVAL, "fused_create: too many particles");
    GcFused* f = new GcFused();
    f->st = gc_state().stream;
    int rc = gc_params_from(c, noise_on, &f->p);   // the same builder as the boundary entry points
    if (rc != GC_OK) {
        delete f;
        return rc;
    }
    f->noise_on = noise_on ? 1 : 0;
    if (opt) {
        f->compact = opt->compact != 0;
        if (opt->skin > 0.f) f->skin = opt->skin;
        if (opt->block == 64 || opt->block == 128 || opt->block == kMaxBS) f->block = opt->block;
    }
    int e = gc_build_grid(bbox6, c.CutRadius + f->skin, periodic_mask, &f->lgrid);
    GcGrid g0;
    if (e == GC_OK) e = gc_build_grid(bbox6, c.CutRadius, periodic_mask, &g0);
    if (e != GC_OK) {
        delete f;
        return e;
    }
    // the per-step predicate uses the box of the rc grid (same lo, hi, L)
    f->p.g = f->lgrid;
    f->n = (int)c.nTotalPar;
    int n = f->n;
    int ok = GC_OK;
    SlotArrays* sa[2] = {&f->a, &f->b};
    for (SlotArrays* s : sa) {
        if (ok == GC_OK) ok = falloc(f, &s->pos, n);
        if (ok == GC_OK) ok = falloc(f, &s->vel, n);
        if (ok == GC_OK) ok = falloc(f, &s->vpred, n);
        if (ok == GC_OK) ok = falloc(f, &s->vh, n);
        if (ok == GC_OK) ok = falloc(f, &s->force, n);
        if (ok == GC_OK) ok = falloc(f, &s->nthro, n);
    }
    if (ok == GC_OK) ok = falloc(f, &f->refpos, n);
    if (ok == GC_OK) ok = falloc(f, &f->dp, n);
    if (ok == GC_OK) ok = falloc(f, &f->slot_of, n);
    if (ok == GC_OK) ok = falloc(f, &f->keys, n);
    if (ok == GC_OK) ok = falloc(f, &f->vals, n);
    if (ok == GC_OK) ok = falloc(f, &f->cnt, n);
    if (ok == GC_OK) ok = falloc(f, &f->ccnt, n);
    if (ok == GC_OK) ok = falloc(f, &f->rebuild, 1);
    if (ok == GC_OK) ok = falloc(f, &f->flags, 1);
    if (ok == GC_OK) ok = falloc(f, &f->stat_sum, 1);
    if (ok == GC_OK) ok = falloc(f, &f->stat_max, 1);
    if (ok == GC_OK && cudaMallocHost(&f->h_rebuild, sizeof(int)) != cudaSuccess)
        ok = gc_fail(GC_ENOMEM, "fused: pinned flag");
    if (ok == GC_OK) {
        // list capacity: expected neighbours within rc + skin at the mean
        // density, with room for membranes and fluctuations
        double vol = (double)f->lgrid.L[0] * f->lgrid.L[1] * f->lgrid.L[2];
        double dens = n / vol;
        double cutr = c.CutRadius + f->skin;
        int capn = (int)(2.0 * 4.18879 * cutr * cutr * cutr * dens) + 32;
        if (opt && opt->list_capacity > 0) capn = opt->list_capacity;
        capn = (capn + 7) & ~7;
        ok = alloc_list(f, capn);
    }
    if (ok != GC_OK) {
        gc_fused_destroy(f);
        return ok;
    }
    GC_CUDA(cudaMemsetAsync(f->flags, 0, sizeof(unsigned), f->st), "fused: flags");
    *out = f;
    return GC_OK;
}

int gc_fused_set_cells(GcFused* f, int ncell, int ntri, int nedge, const int* tri, const int* edge, const int* betri,
                       const int* celltab, const float* shearmod, const float* bendmod, const float* hlarea,
                       const float* hgarea, const float* hvol) {
    if (!f) return gc_fail(GC_EINVAL, "fused_set_cells: NULL handle");
    if (ncell <= 0) return GC_OK;
    int ncp = (int)f->p.nCP;
    if (ncp <= 0 || ntri <= 0 || nedge <= 0) return gc_fail(GC_EINVAL, "fused_set_cells: empty topology");
    for (int k = 0; k < 3 * ntri; ++k)
        if (tri[k] < 1 || tri[k] > ncp) return gc_fail(GC_EINVAL, "fused_set_cells: triangle index out of range");
    for (int k = 0; k < nedge; ++k)
        for (int q = 0; q < 4; ++q)
            if (edge[6 * k + q] < 1 || edge[6 * k + q] > ncp)
                return gc_fail(GC_EINVAL, "fused_set_cells: edge index out of range");
    for (int k = 0; k < ncell; ++k)
        if (betri[2 * k] < 0 || betri[2 * k + 1] >= ntri || betri[2 * k + 1] < betri[2 * k])
            return gc_fail(GC_EINVAL, "fused_set_cells: bad triangle range of cell %d", k);
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
    GC_TRY(falloc(f, &f->mpos, ncp));
    GC_TRY(falloc(f, &f->mforce, ncp));
    GC_TRY(falloc(f, &f->magg, ncp));
    GC_TRY(falloc(f, &f->mnthro, ncp));
    GC_TRY(falloc(f, &f->parea, ncp));
    GC_TRY(falloc(f, &f->mkeys, ncp));
    GC_TRY(falloc(f, &f->mvals, ncp));
    cudaStream_t st = f->st;
    GC_CUDA(cudaMemcpyAsync(f->tri, tri, (size_t)ntri * 12, cudaMemcpyHostToDevice, st), "fused: tri");
    GC_CUDA(cudaMemcpyAsync(f->edge, edge, (size_t)nedge * 24, cudaMemcpyHostToDevice, st), "fused: edge");
    GC_CUDA(cudaMemcpyAsync(f->betri, betri, (size_t)ncell * 8, cudaMemcpyHostToDevice, st), "fused: betri");
    GC_CUDA(cudaMemcpyAsync(f->celltab, celltab, (size_t)ncp * 4, cudaMemcpyHostToDevice, st), "fused: celltab");
    GC_CUDA(cudaMemcpyAsync(f->shear, shearmod, (size_t)nedge * 4, cudaMemcpyHostToDevice, st), "fused: shear");
    GC_CUDA(cudaMemcpyAsync(f->bend, bendmod, (size_t)nedge * 4, cudaMemcpyHostToDevice, st), "fused: bend");
    GC_CUDA(cudaMemcpyAsync(f->hl, hlarea, (size_t)ntri * 4, cudaMemcpyHostToDevice, st), "fused: hl");
    GC_CUDA(cudaMemcpyAsync(f->hg, hgarea, (size_t)ntri * 4, cudaMemcpyHostToDevice, st), "fused: hg");
    GC_CUDA(cudaMemcpyAsync(f->hv, hvol, (size_t)ntri * 4, cudaMemcpyHostToDevice, st), "fused: hv");
    GC_CUDA(cudaMemsetAsync(f->magg, 0, (size_t)ncp * sizeof(float4), st), "fused: magg");
    if (f->p.De != 0.f && f->p.maxcut > 0.f) {
        float bb[6] = {f->lgrid.lo[0], f->lgrid.hi[0], f->lgrid.lo[1], f->lgrid.hi[1], f->lgrid.lo[2], f->lgrid.hi[2]};
        GC_TRY(gc_build_grid(bb, f->p.maxcut, f->lgrid.pmask, &f->mgrid));
        f->have_agg = true;
    }
    GC_CUDA(cudaStreamSynchronize(st), "fused: set cells");
    return GC_OK;
}

int gc_fused_load(GcFused* f, const float* pos, const float* vel, const float* velhalf, const float* force,
                  const int* nthro, int from_device) {
    if (!f || !pos) return gc_fail(GC_EINVAL, "fused_load: NULL argument");
    const int n = f->n;
    cudaStream_t st = f->st;
    const float *dx = pos, *dv = vel, *dh = velhalf, *df = force;
    const int* dn = nthro;
    if (!from_device) {
        size_t b3 = (size_t)n * 12;
        GC_TRY(stage_bytes(f, 5 * b3));
        char* s = (char*)f->stage;
        cudaError_t ce = cudaSuccess;
        auto up = [&](const void* src, size_t off) -> const void* {
            if (!src) return nullptr;
            cudaError_t e = cudaMemcpyAsync(s + off, src, b3, cudaMemcpyHostToDevice, st);
            if (e != cudaSuccess) ce = e;
            return s + off;
        };
        dx = (const float*)up(pos, 0);
        dv = (const float*)up(vel, b3);
        dh = (const float*)up(velhalf, 2 * b3);
        df = (const float*)up(force, 3 * b3);
        dn = (const int*)up(nthro, 4 * b3);
        GC_CUDA(ce, "fused_load: upload");
    }
    if (f->setup_done) {
        fk_load_keep<<<gc_blocks(n, f->block), f->block, 0, st>>>(n, f->p, f->slot_of, dx, dv, dh, df, dn, f->a.pos,
                                                                  f->a.vel, f->a.vh, f->a.force, f->a.nthro,
                                                                  f->ncell > 0 ? f->mpos : nullptr, f->mnthro);
        GC_CHECK_LAUNCH("fused: load in slot order");
        return GC_OK;
    }
    fk_load<<<gc_blocks(n, f->block), f->block, 0, st>>>(n, f->p, dx, dv, dh, df, dn, f->a.pos, f->a.vel, f->a.vh,
                                                        f->a.force, f->a.nthro);
    GC_CHECK_LAUNCH("fused: load");
    GC_CUDA(cudaMemcpyAsync(f->a.vpred, f->a.vel, (size_t)n * sizeof(float4), cudaMemcpyDeviceToDevice, st),
            "fused: load");
    // membrane-ordered positions for the set-up geometry
    if (f->ncell > 0) {
        // gather through the identity order of a fresh load: slot = id
        GC_CUDA(cudaMemcpyAsync(f->mpos, f->a.pos + f->p.nC, (size_t)f->ncp * sizeof(float4),
                                cudaMemcpyDeviceToDevice, st), "fused: load");
        GC_CUDA(cudaMemcpyAsync(f->mnthro, f->a.nthro + f->p.nC, (size_t)f->ncp * sizeof(int4),
                                cudaMemcpyDeviceToDevice, st), "fused: load");
    }
    f->loaded = true;
    f->setup_done = false;
    return GC_OK;
}

int gc_fused_setup(GcFused* f) {
    if (!f || !f->loaded) return gc_fail(GC_ESTATE, "fused_setup: load state first");
    cudaStream_t st = f->st;
    GcParams p = f->p;
    p.g = f->lgrid;
    if (f->ncell > 0) {
        GC_CUDA(cudaMemsetAsync(f->parea, 0, (size_t)f->ncp * sizeof(float), st), "fused: parea");
        fk_mgeo<<<f->ncell, 256, 0, st>>>(p, f->ncell, f->ntri, f->tri, f->betri, f->mpos, f->mnthro, f->tarea,
                                         f->tnorm, f->tcen, f->reftarea, f->carea, f->cvol, f->crefarea, f->crefvol,
                                         f->parea, 1, f->flags);
        GC_CHECK_LAUNCH("fused: set-up geometry");
        fk_mech_setup<<<gc_blocks(f->nedge, f->block), f->block, 0, st>>>(
            p, f->nedge, f->edge, f->mpos, f->mnthro, f->shear, f->bend, f->l0, f->lmax, f->perlen, f->hpow,
            f->hbend, f->refang, f->flags);
        GC_CHECK_LAUNCH("fused: set-up mechanics");
    }
    GC_TRY(rebuild_lists(f));
    // density and pressure of the loaded state (the reference has them from
    // DenInit until the first step recomputes them)
    fk_density<<<gc_blocks(f->n, f->block), f->block, 0, st>>>(f->n, p, make_box(f->lgrid), f->a.pos, f->a.vpred,
                                                               f->a.vh, f->dp, f->nbr, f->cnt, f->cap, nullptr, 0,
                                                               nullptr);
    GC_CHECK_LAUNCH("fused: set-up density");
    f->setup_done = true;
    f->step = -1;
    return GC_OK;
}

int gc_fused_step(GcFused* f, int nsteps, int drive_on) {
    if (!f || !f->setup_done) return gc_fail(GC_ESTATE, "fused_step: call gc_fused_setup first");
    for (int k = 0; k < nsteps; ++k) GC_TRY(one_step(f, drive_on));
    return GC_OK;
}

int gc_fused_store(GcFused* f, float* pos, float* vel, float* rho, float* press, float* force, float* velhalf,
                   int* nthro, int to_device) {
    if (!f) return gc_fail(GC_EINVAL, "fused_store: NULL handle");
    const int n = f->n;
    cudaStream_t st = f->st;
    float *x = pos, *v = vel, *r = rho, *pr = press, *fo = force, *vh = velhalf;
    int* nt = nthro;
    size_t b3 = (size_t)n * 12, b1 = (size_t)n * 4;
    char* s = nullptr;
    if (!to_device) {
        GC_TRY(stage_bytes(f, 5 * b3 + 2 * b1));
        s = (char*)f->stage;
        x = pos ? (float*)(s) : nullptr;
        v = vel ? (float*)(s + b3) : nullptr;
        fo = force ? (float*)(s + 2 * b3) : nullptr;
        vh = velhalf ? (float*)(s + 3 * b3) : nullptr;
        nt = nthro ? (int*)(s + 4 * b3) : nullptr;
        r = rho ? (float*)(s + 5 * b3) : nullptr;
        pr = press ? (float*)(s + 5 * b3 + b1) : nullptr;
    }
    fk_store<<<gc_blocks(n, f->block), f->block, 0, st>>>(n, f->p, f->a.pos, f->a.vel, f->a.vh, f->a.force, f->dp,
                                                         f->a.nthro, x, v, r, pr, fo, vh, nt);
    GC_CHECK_LAUNCH("fused: store");
    if (!to_device) {
        if (pos) GC_CUDA(cudaMemcpyAsync(pos, x, b3, cudaMemcpyDeviceToHost, st), "fused_store");
        if (vel) GC_CUDA(cudaMemcpyAsync(vel, v, b3, cudaMemcpyDeviceToHost, st), "fused_store");
        if (force) GC_CUDA(cudaMemcpyAsync(force, fo, b3, cudaMemcpyDeviceToHost, st), "fused_store");
        if (velhalf) GC_CUDA(cudaMemcpyAsync(velhalf, vh, b3, cudaMemcpyDeviceToHost, st), "fused_store");
        if (nthro) GC_CUDA(cudaMemcpyAsync(nthro, nt, b3, cudaMemcpyDeviceToHost, st), "fused_store");
        if (rho) GC_CUDA(cudaMemcpyAsync(rho, r, b1, cudaMemcpyDeviceToHost, st), "fused_store");
        if (press) GC_CUDA(cudaMemcpyAsync(press, pr, b1, cudaMemcpyDeviceToHost, st), "fused_store");
        GC_CUDA(cudaStreamSynchronize(st), "fused_store");
    }
    return GC_OK;
}

int gc_fused_store_cells(GcFused* f, float* area, float* vol, float* defforce, float* aggforce, float* trinordir,
                         float* tricenter, float* pararea, int to_device) {
    if (!f) return gc_fail(GC_EINVAL, "fused_store_cells: NULL handle");
    if (f->ncell <= 0) return GC_OK;
    cudaStream_t st = f->st;
    size_t nc = f->ncell, ncp = f->ncp, nt = f->ntri;
    float *a = area, *vo = vol, *df = defforce, *ag = aggforce, *tn = trinordir, *tc = tricenter, *pa = pararea;
    if (!to_device) {
        GC_TRY(stage_bytes(f, 4 * (2 * nc + 3 * ncp + 3 * ncp + 3 * nt + 3 * nt + ncp) + 64));
        char* s = (char*)f->stage;
        size_t off = 0;
        auto take = [&](size_t cnt) { float* q = (float*)(s + off); off += 4 * cnt; return q; };
        a = take(nc); vo = take(nc); df = take(3 * ncp); ag = take(3 * ncp); tn = take(3 * nt); tc = take(3 * nt);
        pa = take(ncp);
    }
    fk_cast_cells<<<gc_blocks(nc, 128), 128, 0, st>>>((int)nc, f->carea, f->cvol, a, vo);
    GC_CHECK_LAUNCH("fused: store cells");
    size_t m = ncp > nt ? ncp : nt;
    fk_store_cells<<<gc_blocks(m, 128), 128, 0, st>>>((int)ncp, (int)nt, f->mforce, f->magg, f->parea, f->tnorm,
                                                     f->tcen, df, ag, pa, tn, tc, f->have_agg ? 1 : 0);
    GC_CHECK_LAUNCH("fused: store cells");
    if (!to_device) {
        if (area) GC_CUDA(cudaMemcpyAsync(area, a, 4 * nc, cudaMemcpyDeviceToHost, st), "store cells");
        if (vol) GC_CUDA(cudaMemcpyAsync(vol, vo, 4 * nc, cudaMemcpyDeviceToHost, st), "store cells");
        if (defforce) GC_CUDA(cudaMemcpyAsync(defforce, df, 12 * ncp, cudaMemcpyDeviceToHost, st), "store cells");
        if (aggforce) GC_CUDA(cudaMemcpyAsync(aggforce, ag, 12 * ncp, cudaMemcpyDeviceToHost, st), "store cells");
        if (trinordir) GC_CUDA(cudaMemcpyAsync(trinordir, tn, 12 * nt, cudaMemcpyDeviceToHost, st), "store cells");
        if (tricenter) GC_CUDA(cudaMemcpyAsync(tricenter, tc, 12 * nt, cudaMemcpyDeviceToHost, st), "store cells");
        if (pararea) GC_CUDA(cudaMemcpyAsync(pararea, pa, 4 * ncp, cudaMemcpyDeviceToHost, st), "store cells");
        GC_CUDA(cudaStreamSynchronize(st), "store cells");
    }
    return GC_OK;
}

int gc_fused_cell_sums(GcFused* f, double* area, double* vol) {
    if (!f) return gc_fail(GC_EINVAL, "fused_cell_sums: NULL handle");
    if (f->ncell <= 0) return GC_OK;
    GC_CUDA(cudaMemcpyAsync(area, f->carea, 8 * (size_t)f->ncell, cudaMemcpyDeviceToHost, f->st), "cell sums");
    GC_CUDA(cudaMemcpyAsync(vol, f->cvol, 8 * (size_t)f->ncell, cudaMemcpyDeviceToHost, f->st), "cell sums");
    GC_CUDA(cudaStreamSynchronize(f->st), "cell sums");
    return GC_OK;
}

int gc_fused_stats(GcFused* f, long long* rebuilds, long long* steps, int* list_capacity, double* mean_neighbors,
                   int* max_neighbors) {
    if (!f) return gc_fail(GC_EINVAL, "fused_stats: NULL handle");
    if (rebuilds) *rebuilds = f->rebuilds;
    if (steps) *steps = f->steps;
    if (list_capacity) *list_capacity = f->cap;
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
        if (max_neighbors) *max_neighbors = m;
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

int gc_fused_destroy(GcFused* f) {
    if (!f) return GC_OK;
    cudaStreamSynchronize(f->st);
    for (cudaEvent_t e : f->ev) cudaEventDestroy(e);
    for (void* q : f->allocs) cudaFree(q);
    if (f->nbr) cudaFree(f->nbr);
    if (f->cmask) cudaFree(f->cmask);
    if (f->stage) cudaFree(f->stage);
    if (f->h_rebuild) cudaFreeHost(f->h_rebuild);
    delete f;
    return GC_OK;
}

}  // extern "C"

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
                              int* __restrict__ slot_of, float4* __restrict__ mpos, int4* __restrict__ mnthro,
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
    GC_TRY(falloc(f, &f->mpos, ncp));
    GC_TRY(falloc(f, &f->mforce, ncp));
    GC_TRY(falloc(f, &f->magg, ncp));
    GC_TRY(falloc(f, &f->mnthro, ncp));
    GC_TRY(falloc(f, &f->parea, ncp));
    GC_TRY(falloc(f, &f->mkeys, ncp));
    GC_TRY(falloc(f, &f->mvals, ncp));
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
    GC_CUDA(cudaMemsetAsync(f->magg, 0, (size_t)ncp * sizeof(float4), st), "fused engine: magg");
    fk_import_cellrefs<<<gc_blocks(ncell, 128), 128, 0, st>>>(ncell, ntri, f->betri, r.refarea_para, r.refvol_para,
                                                            f->crefarea, f->crefvol);
    GC_CHECK_LAUNCH("fused engine: reference areas and volumes");
    if (f->p.De != 0.f && f->p.maxcut > 0.f) {
        float bb[6] = {f->lgrid.lo[0], f->lgrid.hi[0], f->lgrid.lo[1], f->lgrid.hi[1], f->lgrid.lo[2], f->lgrid.hi[2]};
        GC_TRY(gc_build_grid(bb, f->p.maxcut, f->lgrid.pmask, &f->mgrid));
        f->have_agg = true;
    }
    return GC_OK;
}

int engine_start(GcState& s) {
    const GcRefPtrs& r = s.ref;
    if (!r.sortpart || !r.coor || !r.velrhop || !r.velhalf || !r.force || !r.bbox)
        return gc_fail(GC_ESTATE, "fused engine: the first step did not show every particle buffer");
    float bb[6];
    GC_CUDA(cudaMemcpyAsync(bb, r.bbox, sizeof(bb), cudaMemcpyDeviceToHost, s.stream), "fused engine: bbox");
    GC_CUDA(cudaStreamSynchronize(s.stream), "fused engine: bbox");
    GcFused* f = nullptr;
    GC_TRY(gc_fused_create(&s.c, bb, s.periodic_mask, s.noise_on, nullptr, &f));
    int rc = engine_cells(f, r);
    if (rc == GC_OK) {
        fk_import_ref<<<gc_blocks(f->n, f->block), f->block, 0, f->st>>>(
            f->n, f->p.nC, r.sortpart, r.coor, r.velrhop, r.velhalf, r.force, r.nthro, f->a, f->slot_of,
            f->ncell > 0 ? f->mpos : nullptr, f->mnthro, f->flags);
        cudaError_t e = cudaGetLastError();
        gc_count_launch();
        if (e != cudaSuccess) rc = gc_cuda_fail(e, "fused engine: adopt state");
    }
    if (rc == GC_OK) rc = rebuild_lists(f);
    if (rc != GC_OK) {
        gc_fused_destroy(f);
        return rc;
    }
    f->loaded = true;
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
        fk_store_cells<<<gc_blocks(m, 128), 128, 0, st>>>(m, 0, f->mforce, f->magg, f->parea, f->tnorm, f->tcen,
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
