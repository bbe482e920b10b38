// fused_tiles.cu -- the half-stencil pair passes of the fused step ("pair
// tiles"): every interacting pair of particles is evaluated once, its
// thermal noise drawn once, and each side of the pair gets its share.
//
// Layout.  Slots are sorted by cubes at least rc + skin wide (the list grid
// with a 3 x 3 x 3 stencil).  A cube pairs with itself and with its 13
// forward neighbours (dz = 1; dz = 0, dy = 1; dz = dy = 0, dx = 1), so every
// pair of neighbouring cubes -- and so every pair of particles within
// rc + skin -- belongs to exactly one (home cube, direction) pair; periodic
// axes have at least three cubes, so no two directions reach the same cube.
// At each rebuild one warp per home cube finds, for each of its 14 cube
// pairs, the pairs (a, b) of local indices within rc + skin (within r0 + skin
// when one side is a Bound1 wall particle; at least one side mobile).  A
// count pass sizes the lists and a device-wide scan places them; the fill
// pass cuts each list into 32 equal runs of consecutive pairs, one per lane,
// and stores it transposed.
//
// Passes.  One warp per home cube walks its 14 lists, 32 entries (one per
// lane) per iteration, evaluates each pair that acts this step (r < rc) once
// -- its thermal noise included -- and gives both sides their share in
// shared memory: the home cube's sums are kept over all 14 pairs, the partner
// cube's over one pair.  A lane meets each a of its run in one stretch, so it
// sums a's share in a register and adds it once; the shares of b are added
// by the lanes that have them, and lanes of one iteration that add to the
// same particle go one after another in the order of a rank the build stored
// in the entry.  So every sum has a fixed order (repeat runs are
// bit-identical) without atomics, whose throughput on shared memory (4.9
// 64-bit additions per SM clock without conflicts, 0.45 with 13 lanes on one
// address, measured) would bound the pass.  After each cube pair the
// partner cube's sums are written as the partial sum of that direction (a
// plane of 14 per quantity); the home sums go to direction 0.  A finish
// kernel per slot adds the partials of the directions whose backward
// neighbour exists, in a fixed order, and applies the equation of state
// (density) or the body force, membrane force and corrector (force).
//
// Bound2 walls keep per-particle lists of their mobile neighbours (the list
// build of fused.cu restricted to them) for the wall velocity, which the
// density pass of the list path computes.
#include "fused_internal.cuh"

#include <math.h>
#include <stdio.h>

namespace gcf {

constexpr int kTileBS = 32 * kTileWarps;

// The 14 directions of a home cube: itself, then the forward half.
__constant__ signed char c_tdir[kTilePairs][3] = {
    {0, 0, 0},  {1, 0, 0},  {-1, 1, 0}, {0, 1, 0},  {1, 1, 0},  {-1, -1, 1}, {0, -1, 1},
    {1, -1, 1}, {-1, 0, 1}, {0, 0, 1},  {1, 0, 1},  {-1, 1, 1}, {0, 1, 1},   {1, 1, 1}};

// pairs of one segment of a list (staged in shared memory at the build)
constexpr int kTileStage = 2048;

__device__ __forceinline__ void cube_xyz(int local, const GcGrid& g, int* x, int* y, int* z) {
    *x = local % g.n[0];
    *y = (local / g.n[0]) % g.n[1];
    *z = local / (g.n[0] * g.n[1]);
}

// Neighbour of home cube C (global) in direction p, or -1 off a wall axis;
// *img: the pair touches a periodic face (its particles' positions may wrap
// between rebuilds, so pairs take the minimum image).  Particles of interior
// cubes are more than a cube width from every face and cannot wrap before
// the next rebuild: their differences need no image.
__device__ __forceinline__ int tile_neighbor(int C, int p, const SysInfo& S, bool* img) {
    const GcGrid& g = S.g;
    int cx, cy, cz;
    cube_xyz(C - S.cube0, g, &cx, &cy, &cz);
    const int x = cube_step(cx, c_tdir[p][0], 0, g), y = cube_step(cy, c_tdir[p][1], 1, g),
              z = cube_step(cz, c_tdir[p][2], 2, g);
    if (x < 0 || y < 0 || z < 0) return -1;
    bool im = false;
    const int c[3] = {cx, cy, cz}, d[3] = {x, y, z};
#pragma unroll
    for (int a = 0; a < 3; ++a)
        if (g.pmask & (1 << a))
            im |= c[a] == 0 || c[a] == g.n[a] - 1 || d[a] == 0 || d[a] == g.n[a] - 1;
    *img = im;
    return S.cube0 + x + g.n[0] * (y + g.n[1] * z);
}

// Per cube: its system, and the directions p >= 1 whose backward neighbour
// (the home cube that sends this cube a partial sum in direction p) exists.
__global__ void fk_tile_cubes(int K, const SysInfo* __restrict__ sys, int nsys, int* __restrict__ cube_sys,
                              unsigned short* __restrict__ bmask) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= K) return;
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sys[mid].cube0 <= c) lo = mid;
        else hi = mid - 1;
    }
    cube_sys[c] = lo;
    const GcGrid& g = sys[lo].g;
    int cx, cy, cz;
    cube_xyz(c - sys[lo].cube0, g, &cx, &cy, &cz);
    unsigned m = 1;
    for (int p = 1; p < kTilePairs; ++p)
        if (cube_step(cx, -c_tdir[p][0], 0, g) >= 0 && cube_step(cy, -c_tdir[p][1], 1, g) >= 0 &&
            cube_step(cz, -c_tdir[p][2], 2, g) >= 0)
            m |= 1u << p;
    bmask[c] = (unsigned short)m;
}

// Whether a pair found at build time belongs to a list: at least one side
// mobile; a Bound1 particle only with a mobile partner within r0 + skin;
// otherwise both in the SDPD set within rc + skin.
__device__ __forceinline__ bool tile_take(unsigned ida, unsigned idb, float r2, const SysInfo& S, float cut2,
                                          float rep2) {
    const bool ma = ida >= S.fl, mb = idb >= S.fl;
    if (!(ma || mb)) return false;
    if (ida < S.b2 || idb < S.b2) return r2 < rep2;
    return r2 < cut2;
}

// Entry of a pair list: a and b (7 bits each), rb (5 bits: the lane's rank
// among the lanes of its iteration that add to the same b), ra (5 bits: the
// rank among the lanes of its iteration that add a finished run to the same
// a), the end of the lane's run of entries with this a, and a valid bit.
__device__ __forceinline__ unsigned tent_a(unsigned e) { return e & 127u; }
__device__ __forceinline__ unsigned tent_b(unsigned e) { return (e >> 7) & 127u; }
__device__ __forceinline__ unsigned tent_rb(unsigned e) { return (e >> 14) & 31u; }
__device__ __forceinline__ unsigned tent_ra(unsigned e) { return (e >> 19) & 31u; }
__device__ __forceinline__ bool tent_flush(unsigned e) { return (e >> 24) & 1u; }
__device__ __forceinline__ bool tent_valid(unsigned e) { return (e >> 25) & 1u; }

// Count (FILL = false: chunks of 32 per cube pair into toff, candidate pairs
// into *tpairs) or write (FILL = true) the pair lists, one warp per home
// cube.  The pairs (a, b) of a cube pair are found a-major and staged in
// shared memory; the list of L pairs is then cut into 32 runs of
// S = ceil(L / 32) consecutive pairs, lane l taking pairs l S .. l S + S - 1,
// and stored transposed (iteration t of lane l at t * 32 + l) so that the
// passes read 32 consecutive entries per iteration.  Within a run a lane
// meets each a in one stretch (a-major order), so it sums a's share in a
// register and adds it once, at the stretch's end; the ranks rb and ra order
// the lanes of an iteration that add to the same b (or a), so that those
// additions go one after another in a fixed order, with no atomics.
// Chunks of 32 entries a list of L pairs takes: full segments of kTileStage
// pairs, then the rest.
__host__ __device__ __forceinline__ unsigned tile_chunks(unsigned L) {
    return (L / kTileStage) * (kTileStage / 32) + ((L % kTileStage) + 31) / 32;
}

// Writes the L <= kTileStage staged pairs stg[0..L) as one segment at out:
// lane l takes pairs l S .. l S + S - 1 (S = ceil(L / 32)), stored transposed.
__device__ __forceinline__ void tile_write_segment(const unsigned* stg, unsigned L, unsigned* __restrict__ out,
                                                   int lane) {
    const unsigned lt = (1u << lane) - 1u;
    const unsigned S = (L + 31) >> 5;
    for (unsigned t = 0; t < S; ++t) {
        const unsigned q = lane * S + t;
        const bool valid = q < L;
        const unsigned e = valid ? stg[q] : 0u;
        const unsigned a = e & 127u, b = (e >> 7) & 127u;
        const bool more = valid && t + 1 < S && q + 1 < L;
        const bool flush = valid && !(more && (stg[q + 1] & 127u) == a);
        const unsigned mb = __match_any_sync(0xffffffffu, valid ? (int)b : 1024 + lane);
        const unsigned ma = __match_any_sync(0xffffffffu, flush ? (int)a : 2048 + lane);
        const unsigned rb = __popc(mb & lt), ra = __popc(ma & lt);
        out[(size_t)t * 32 + lane] =
            valid ? (a | (b << 7) | (rb << 14) | (ra << 19) | ((unsigned)flush << 24) | (1u << 25)) : 0u;
    }
    __syncwarp();
}

// Count (FILL = false: chunks of 32 per cube pair into toff, candidate pairs
// into *tpairs) or write (FILL = true) the pair lists, one warp per home
// cube.  The pairs (a, b) of a cube pair are found a-major and staged in
// shared memory; each segment of up to kTileStage pairs is then cut into 32
// runs of S = ceil(L / 32) consecutive pairs, lane l taking pairs
// l S .. l S + S - 1, and stored transposed (iteration t of lane l at
// t * 32 + l) so that the passes read 32 consecutive entries per iteration.
// Within a run a lane meets each a in one stretch (a-major order), so it
// sums a's share in a register and adds it once, at the stretch's end; the
// ranks rb and ra order the lanes of an iteration that add to the same b (or
// a), so that those additions go one after another in a fixed order, with
// no atomics.
template <bool FILL>
__global__ void __launch_bounds__(kTileBS) fk_tile_build(int K, const SysInfo* __restrict__ sys,
                                                        const int* __restrict__ cube_sys,
                                                        const unsigned* __restrict__ start,
                                                        const float4* __restrict__ pos, float cut2, float rep2,
                                                        int* __restrict__ tnb, unsigned* __restrict__ toff,
                                                        unsigned* __restrict__ tent, size_t cap_chunks,
                                                        unsigned* oflag, unsigned long long* __restrict__ tpairs) {
    __shared__ unsigned stg[FILL ? kTileWarps : 1][FILL ? kTileStage + 32 : 1];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int C = blockIdx.x * kTileWarps + w;
    if (C >= K) return;   // whole warps
    const SysInfo& S = sys[cube_sys[C]];
    const Box B = box_of(S);
    const unsigned sa = start[C], na = start[C + 1] - sa;
    bool full = na > (unsigned)kTileMax;
    if (FILL && toff[(size_t)K * kTilePairs] > cap_chunks) {
        // the entries do not fit (captured steps): the host grows them and runs the steps again
        if (lane == 0) atomicOr(oflag, GC_FLAG_CELL_OVERFLOW);
        return;
    }
    const unsigned lt = (1u << lane) - 1u;
    unsigned long long npairs = 0;
    for (int p = 0; p < kTilePairs; ++p) {
        bool img = false;
        int Cn = tile_neighbor(C, p, S, &img);
        unsigned sb = 0, nb = 0;
        if (Cn >= 0) {
            sb = start[Cn];
            nb = start[Cn + 1] - sb;
            full |= nb > (unsigned)kTileMax;
        }
        if (full) Cn = -1;
        unsigned cnt = 0;      // pairs of this cube pair
        unsigned staged = 0;   // pairs in the stage (FILL)
        unsigned* out = FILL ? tent + (size_t)toff[(size_t)C * kTilePairs + p] * 32 : nullptr;
        if (Cn >= 0 && na > 0 && nb > 0) {
            const unsigned total = na * nb;
            const float inv_nb = 1.f / (float)nb;
            for (unsigned q0 = 0; q0 < total; q0 += 32) {
                const unsigned q = q0 + lane;
                // q = a nb + b; (q + 1/2) / nb lies at least 1/(2 nb) from an integer,
                // far beyond the rounding of the product, so a is exact
                const unsigned a = (unsigned)(((float)q + 0.5f) * inv_nb);
                const unsigned b = q - a * nb;
                bool take = q < total && (p != 0 || b > a);
                if (take) {
                    const float4 xa = pos[sa + a], xb = pos[sb + b];
                    const float3 d = img ? pair_image(xyz(xa), xyz(xb), B)
                                         : f3(__fsub_rn(xa.x, xb.x), __fsub_rn(xa.y, xb.y), __fsub_rn(xa.z, xb.z));
                    take = tile_take(fid(xa), fid(xb), norm2_rn(d), S, cut2, rep2);
                }
                const unsigned bal = __ballot_sync(0xffffffffu, take);
                if (FILL) {
                    if (take) stg[w][staged + __popc(bal & lt)] = a | (b << 7);
                    staged += __popc(bal);
                    __syncwarp();
                    if (staged >= (unsigned)kTileStage) {   // a full segment: write it, keep the rest
                        tile_write_segment(stg[w], kTileStage, out, lane);
                        out += kTileStage;
                        const unsigned rest = staged - kTileStage;
                        const unsigned keep = lane < rest ? stg[w][kTileStage + lane] : 0u;
                        __syncwarp();
                        if (lane < rest) stg[w][lane] = keep;
                        staged = rest;
                        __syncwarp();
                    }
                }
                cnt += __popc(bal);
            }
        }
        npairs += cnt;
        if (FILL) {
            if (staged > 0) tile_write_segment(stg[w], staged, out, lane);
            if (lane == 0) tnb[(size_t)C * kTilePairs + p] = Cn < 0 ? -1 : (Cn | (img ? (1 << 30) : 0));
        } else if (lane == 0) {
            toff[(size_t)C * kTilePairs + p] = tile_chunks(cnt);
        }
    }
    if (!FILL && lane == 0) {
        atomicAdd(tpairs, npairs);
        if (full) atomicOr(oflag, GC_FLAG_TILE_FULL);
    }
}

// Adds v[k] to acc[k][idx] (k < NC) on the lanes with `on`; lanes that share
// an idx add one after another in the order of their rank, so every sum has
// a fixed order, with no atomics.  Called by the whole warp.
template <int NC>
__device__ __forceinline__ void tile_add(float (*acc)[kTileMax], bool on, unsigned idx, unsigned rank,
                                         const float* v) {
    if (!__any_sync(0xffffffffu, on)) return;
    const unsigned rmax = __reduce_max_sync(0xffffffffu, on ? rank : 0u);
    for (unsigned r = 0; r <= rmax; ++r) {
        if (on && rank == r) {
#pragma unroll
            for (int k = 0; k < NC; ++k) acc[k][idx] += v[k];
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Density (K8): W of every pair within rc between members of the SDPD set,
// added to each mobile side.
// ---------------------------------------------------------------------------
template <bool ENS>
__global__ void __launch_bounds__(kTileBS) fk_tile_density(int K, GcParams p, SysInfo s0,
                                                          const SysInfo* __restrict__ sys,
                                                          const int* __restrict__ cube_sys,
                                                          const unsigned* __restrict__ start,
                                                          const int* __restrict__ tnb, const unsigned* __restrict__ toff,
                                                          const unsigned* __restrict__ tent, size_t cap_chunks,
                                                          const float4* __restrict__ pos, float* __restrict__ pd, int n) {
    __shared__ float acc[kTileWarps][2][1][kTileMax];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int C = blockIdx.x * kTileWarps + w;
    if (C >= K) return;
    // lists that did not fit (captured steps; those steps are run again) are not read
    if (toff[(size_t)K * kTilePairs] > cap_chunks) return;
    const SysInfo& S = ENS ? sys[cube_sys[C]] : s0;
    const Box B = box_of(S);
    const unsigned b2 = S.b2, fl = S.fl;
    const unsigned sa = start[C], na = start[C + 1] - sa;
    if (na > (unsigned)kTileMax) return;   // the build raised GC_FLAG_TILE_FULL
    float(*A)[kTileMax] = acc[w][0];
    float(*Bn)[kTileMax] = acc[w][1];
    for (unsigned i = lane; i < na; i += 32) A[0][i] = 0.f;
    __syncwarp();
    for (int q = 0; q < kTilePairs; ++q) {
        const int t = tnb[(size_t)C * kTilePairs + q];
        if (t < 0) continue;
        const int Cn = t & 0x3FFFFFFF;
        const bool img = (t >> 30) & 1;
        const unsigned sb = start[Cn], nb = start[Cn + 1] - sb;
        if (nb > (unsigned)kTileMax) continue;   // only with GC_FLAG_TILE_FULL raised
        float(*Ab)[kTileMax] = q == 0 ? A : Bn;
        if (q != 0)
            for (unsigned i = lane; i < nb; i += 32) Bn[0][i] = 0.f;
        __syncwarp();
        float run = 0.f;   // this lane's share of its current a
        const unsigned c1 = toff[(size_t)C * kTilePairs + q + 1];
        for (unsigned c = toff[(size_t)C * kTilePairs + q]; c < c1; ++c) {
            const unsigned ent = __ldg(tent + (size_t)c * 32 + lane);
            const unsigned a = tent_a(ent), b = tent_b(ent);
            float wv = 0.f;
            bool tob = false;
            if (tent_valid(ent)) {
                const float4 xa = pos[sa + a], xb = pos[sb + b];
                const float3 d = img ? pair_image(xyz(xa), xyz(xb), B)
                                     : f3(__fsub_rn(xa.x, xb.x), __fsub_rn(xa.y, xb.y), __fsub_rn(xa.z, xb.z));
                const float r2 = norm2_rn(d);
                const unsigned ida = fid(xa), idb = fid(xb);
                if (r2 < p.rc2 && ida >= b2 && idb >= b2) {
                    const float r = r2 > 0.f ? r2 * rsqrtf(r2) : 0.f;
                    wv = wendland_w(r, p);
                    if (ida >= fl) run += wv;
                    tob = idb >= fl;
                }
            }
            tile_add<1>(Ab, tob, b, tent_rb(ent), &wv);
            const bool fa = tent_flush(ent);
            tile_add<1>(A, fa, a, tent_ra(ent), &run);
            if (fa) run = 0.f;
        }
        __syncwarp();
        if (q != 0)
            for (unsigned i = lane; i < nb; i += 32) pd[(size_t)q * n + sb + i] = Bn[0][i];
        __syncwarp();
    }
    for (unsigned i = lane; i < na; i += 32) pd[sa + i] = A[0][i];
}

// Density of every slot from its partial sums (direction 0, then the
// directions whose backward neighbour exists, in order); EOS (K11).
template <bool ENS>
__global__ void fk_tile_dfinish(int n, GcParams p, SysInfo s0, const SysInfo* __restrict__ sys,
                                const int* __restrict__ sysid, const float4* __restrict__ pos,
                                const int* __restrict__ keys, const unsigned short* __restrict__ bmask,
                                const float* __restrict__ pd, float2* __restrict__ dp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    GC_SYS_OF(S, i);
    const int t = stype(fid(pos[i]), S);
    if (t == PT_FLUID || t == PT_MEMB) {
        const unsigned m = bmask[keys[i]];
        float sum = p.w0 + pd[i];
#pragma unroll
        for (int q = 1; q < kTilePairs; ++q)
            if ((m >> q) & 1u) sum += pd[(size_t)q * n + i];
        const float rho = p.mass * sum;
        const float c2 = (t == PT_MEMB) ? p.c2sq : p.c1sq;
        const float inv_d = __frcp_rn(sum);
        dp[i] = make_float2(inv_d, c2 * (rho - p.rho0) * inv_d * inv_d);
    } else {
        dp[i] = make_float2(p.mass / p.rho0, 0.f);
    }
}

// ---------------------------------------------------------------------------
// Forces: SDPD pair force with its noise (K12) between members of the SDPD
// set within rc, and the Bound1 repulsion (K13) within r0, added to each
// mobile side (the pair's force on a, and its negative on b).
// ---------------------------------------------------------------------------
#ifndef GC_TILE_FORCE_MIN_BLOCKS
#define GC_TILE_FORCE_MIN_BLOCKS 8
#endif

template <bool ENS>
__global__ void __launch_bounds__(kTileBS, GC_TILE_FORCE_MIN_BLOCKS)
    fk_tile_force(int K, GcParams p, SysInfo s0, const SysInfo* __restrict__ sys, const int* __restrict__ cube_sys,
                  const unsigned* __restrict__ nkey, const unsigned* __restrict__ start, const int* __restrict__ tnb,
                  const unsigned* __restrict__ toff, const unsigned* __restrict__ tent, size_t cap_chunks,
                  const float4* __restrict__ pos, const float4* __restrict__ vpred, const float2* __restrict__ dp,
                  float* __restrict__ pf, int n, unsigned* flags) {
    __shared__ float acc[kTileWarps][2][3][kTileMax];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int C = blockIdx.x * kTileWarps + w;
    if (C >= K) return;
    // lists that did not fit (captured steps; those steps are run again) are not read
    if (toff[(size_t)K * kTilePairs] > cap_chunks) return;
    const int s = ENS ? cube_sys[C] : 0;
    const SysInfo& S = ENS ? sys[s] : s0;
    const Box B = box_of(S);
    const unsigned b2 = S.b2, fl = S.fl, id0 = S.id0;
    const uint32_t key = ENS ? nkey[s] : (nkey ? nkey[0] : p.noise_key);   // as in fk_force
    const bool noise = p.noise_pref > 0.f;
    const unsigned sa = start[C], na = start[C + 1] - sa;
    if (na > (unsigned)kTileMax) return;   // the build raised GC_FLAG_TILE_FULL
    float(*A)[kTileMax] = acc[w][0];
    float(*Bn)[kTileMax] = acc[w][1];
    for (unsigned i = lane; i < na; i += 32) A[0][i] = A[1][i] = A[2][i] = 0.f;
    __syncwarp();
    for (int q = 0; q < kTilePairs; ++q) {
        const int t = tnb[(size_t)C * kTilePairs + q];
        if (t < 0) continue;
        const int Cn = t & 0x3FFFFFFF;
        const bool img = (t >> 30) & 1;
        const unsigned sb = start[Cn], nb = start[Cn + 1] - sb;
        if (nb > (unsigned)kTileMax) continue;   // only with GC_FLAG_TILE_FULL raised
        float(*Ab)[kTileMax] = q == 0 ? A : Bn;
        if (q != 0)
            for (unsigned i = lane; i < nb; i += 32) Bn[0][i] = Bn[1][i] = Bn[2][i] = 0.f;
        __syncwarp();
        float run[3] = {0.f, 0.f, 0.f};   // this lane's share of its current a
        const unsigned c1 = toff[(size_t)C * kTilePairs + q + 1];
        for (unsigned c = toff[(size_t)C * kTilePairs + q]; c < c1; ++c) {
            const unsigned ent = __ldg(tent + (size_t)c * 32 + lane);
            const unsigned a = tent_a(ent), b = tent_b(ent);
            float3 f = f3(0.f, 0.f, 0.f);
            bool act = false;
            unsigned ida = 0, idb = 0;
            if (tent_valid(ent)) {
                const float4 xa = pos[sa + a], xb = pos[sb + b];
                const float3 d = img ? pair_image(xyz(xa), xyz(xb), B)
                                     : f3(__fsub_rn(xa.x, xb.x), __fsub_rn(xa.y, xb.y), __fsub_rn(xa.z, xb.z));
                const float r2 = norm2_rn(d);
                ida = fid(xa);
                idb = fid(xb);
                if (ida < b2 || idb < b2) {   // a Bound1 wall particle and a mobile one: repulsion only
                    if (r2 < p.rep_r0sq && r2 > 0.f) {
                        const float inv_r = rsqrtf(r2);
                        const float ir2 = inv_r * inv_r;
                        const float q2 = p.rep_r0sq * ir2, q4 = q2 * q2, q12 = q4 * q4 * q4;
                        f = (p.rep_D * (q12 - q4) * ir2) * d;
                        act = true;
                    }
                } else if (r2 < p.rc2 && r2 > 0.f) {   // coincident pairs exert no force
                    const float2 da = dp[sa + a], db = dp[sb + b];
                    const float4 va = vpred[sa + a], vb = vpred[sb + b];
                    const float inv_r = rsqrtf(r2);
                    const float r = r2 * inv_r;
                    const float F = wendland_f(r, p);
                    f = ((da.y + db.y) * F) * d;
                    const float3 e3 = inv_r * d;
                    const float3 vab = f3(va.x - vb.x, va.y - vb.y, va.z - vb.z);
                    const float ev = dot3(e3, vab);
                    const float fdd = F * da.x * db.x;
                    f -= fdd * (p.visA * vab + (p.visB * ev) * e3);
                    if (noise) {
                        const float qq = p.noise_pref * fdd;
                        float qn = qq > 0.f ? qq * rsqrtf(qq) : 0.f;
                        qn = ida < idb ? qn : -qn;   // the pair sign of xi_ab
                        const float3 xi = pair_noise_unsigned_k(ida - id0, idb - id0, key);
                        const float exi = dot3(e3, xi);
                        f += qn * (p.sqrtA * xi + ((p.sqrtAB - p.sqrtA) * exi) * e3);
                    }
                    act = true;
                }
            }
            if (act && ida >= fl) {
                run[0] += f.x;
                run[1] += f.y;
                run[2] += f.z;
            }
            const float fb[3] = {-f.x, -f.y, -f.z};
            tile_add<3>(Ab, act && idb >= fl, b, tent_rb(ent), fb);
            const bool fa = tent_flush(ent);
            tile_add<3>(A, fa, a, tent_ra(ent), run);
            if (fa) run[0] = run[1] = run[2] = 0.f;
        }
        __syncwarp();
        if (q != 0) {
            float* o = pf + (size_t)q * 3 * n + sb;
            for (unsigned i = lane; i < nb; i += 32) {
                o[i] = Bn[0][i];
                o[n + i] = Bn[1][i];
                o[2 * (size_t)n + i] = Bn[2][i];
            }
        }
        __syncwarp();
    }
    float* o = pf + sa;
    for (unsigned i = lane; i < na; i += 32) {
        o[i] = A[0][i];
        o[n + i] = A[1][i];
        o[2 * (size_t)n + i] = A[2][i];
    }
    (void)flags;
}

// Force of every slot from its partial sums (direction 0, then the
// directions whose backward neighbour exists, in order), body force (K14),
// membrane force (K17/K18), corrector (K19).
template <bool ENS>
__global__ void fk_tile_ffinish(int n, GcParams p, SysInfo s0, const SysInfo* __restrict__ sys,
                                const int* __restrict__ sysid, const float4* __restrict__ pos,
                                const int* __restrict__ keys, const unsigned short* __restrict__ bmask,
                                const float* __restrict__ pf, const float4* __restrict__ vh,
                                const float4* __restrict__ mforce, float4* __restrict__ force,
                                float4* __restrict__ vel, int drive) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned id = fid(pos[i]);
    GC_SYS_OF(S, i);
    if (id < S.fl) {
        force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const unsigned m = bmask[keys[i]];
    float3 f = f3(pf[i], pf[(size_t)n + i], pf[2 * (size_t)n + i]);
#pragma unroll
    for (int q = 1; q < kTilePairs; ++q)
        if ((m >> q) & 1u) {
            const float* o = pf + (size_t)q * 3 * n + i;
            f += f3(o[0], o[n], o[2 * (size_t)n]);
        }
    if (drive) f.x += S.gx;
    if (id >= S.cs && mforce) {
        const float4 mf = mforce[S.m0 + (id - S.cs)];
        f += f3(mf.x, mf.y, mf.z);
    }
    // a non-finite force shows up as a non-finite position in the next
    // fk_integrate, which raises GC_FLAG_NONFINITE
    force[i] = make_float4(f.x, f.y, f.z, 0.f);
    const float4 h = vh[i];
    const float sc = 0.5f * p.dt * p.inv_mass;
    vel[i] = make_float4(h.x + sc * f.x, h.y + sc * f.y, h.z + sc * f.z, 0.f);
}

// Wall velocity of the Bound2 slots (K10) from their lists of mobile
// neighbours: v_w = 2 VelHalf - sum v W / sum W, reading and writing `v`.
template <bool ENS>
__global__ void fk_tile_wallvel(int n, GcParams p, SysInfo s0, const SysInfo* __restrict__ sys,
                                const int* __restrict__ sysid, const float4* __restrict__ pos, float4* __restrict__ v,
                                const float4* __restrict__ vh, const int* __restrict__ nbr,
                                const int* __restrict__ cnt, int cap);

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

// Per-cube arrays of the grids built by build_grids (system, backward
// directions, neighbours, list offsets) and the partial-sum planes.
int tiles_grid(GcFused* f) {
    if (f->lists) return GC_OK;
    const int K = f->K;
    if (K > f->tK) {
        if (f->cube_sys) cudaFree(f->cube_sys);
        if (f->bmask) cudaFree(f->bmask);
        if (f->tnb) cudaFree(f->tnb);
        if (f->toff) cudaFree(f->toff);
        if (f->tscan) cudaFree(f->tscan);
        f->cube_sys = nullptr;
        f->bmask = nullptr;
        f->tnb = nullptr;
        f->toff = nullptr;
        f->tscan = nullptr;
        f->tK = 0;
        const size_t kp = (size_t)K * kTilePairs;
        if (kp + 1 > (size_t)4096 * 4096) return gc_fail(GC_EINVAL, "fused: %d cubes are too many for the pair tiles", K);
        GC_CUDA(cudaMalloc(&f->cube_sys, (size_t)K * sizeof(int)), "fused: tiles");
        GC_CUDA(cudaMalloc(&f->bmask, (size_t)K * sizeof(unsigned short)), "fused: tiles");
        GC_CUDA(cudaMalloc(&f->tnb, kp * sizeof(int)), "fused: tiles");
        GC_CUDA(cudaMalloc(&f->toff, (kp + 1) * sizeof(unsigned)), "fused: tiles");
        GC_CUDA(cudaMalloc(&f->tscan, gc_scan_blocks((int)kp) * sizeof(unsigned)), "fused: tiles");
        f->tK = K;
        drop_graphs(f);
    }
    if (!f->pd) {
        GC_CUDA(cudaMalloc(&f->pd, (size_t)kTilePairs * f->n * sizeof(float)), "fused: density partials");
        GC_CUDA(cudaMalloc(&f->pf, (size_t)kTilePairs * 3 * f->n * sizeof(float)), "fused: force partials");
        GC_CUDA(cudaMalloc(&f->tpairs, sizeof(unsigned long long)), "fused: tiles");
    }
    fk_tile_cubes<<<gc_blocks(K, 256), 256, 0, f->st>>>(K, f->dsys, f->nsys, f->cube_sys, f->bmask);
    GC_CHECK_LAUNCH("fused: tile cubes");
    return GC_OK;
}

int tiles_alloc_entries(GcFused* f, size_t chunks) {
    if (chunks <= f->tent_chunks && f->tent) return GC_OK;
    if (f->tent) cudaFree(f->tent);
    f->tent = nullptr;
    f->tent_chunks = 0;
    GC_CUDA(cudaMalloc(&f->tent, (chunks ? chunks : 1) * 32 * sizeof(unsigned)), "fused: pair lists");
    f->tent_chunks = chunks;
    drop_graphs(f);
    return GC_OK;
}

// The pair lists from the positions bpos (the slots' positions at this
// rebuild) and the cube starts of the latest sort.  Host-driven (host =
// true): the count is read back, the entries grown to fit, and a cube too
// full for the tiles turns the handle to per-particle lists (the caller
// rebuilds).  Captured: the fill checks the capacity on the device and
// raises oflag instead.
int tiles_build(GcFused* f, cudaStream_t st, const float4* bpos, bool host) {
    const int K = f->K;
    const int nb = (K + kTileWarps - 1) / kTileWarps;
    const float cut = f->p.rc + f->skin, rep = f->p.rep_r0 + f->skin;
    const size_t kp = (size_t)K * kTilePairs;
    GC_CUDA(cudaMemsetAsync(f->tpairs, 0, sizeof(unsigned long long), st), "fused: tiles");
    fk_tile_build<false><<<nb, kTileBS, 0, st>>>(K, f->dsys, f->cube_sys, f->sb.cnt, bpos, cut * cut, rep * rep,
                                                 f->tnb, f->toff, f->tent, f->tent_chunks, f->oflag, f->tpairs);
    GC_CHECK_LAUNCH("fused: tile count");
    GC_TRY(gc_scan_exclusive(f->toff, (int)kp, f->tscan, st));
    if (host) {
        GC_CUDA(cudaMemcpyAsync(&f->h->tchunks, f->toff + kp, sizeof(unsigned), cudaMemcpyDeviceToHost, st),
                "fused: tiles");
        GC_CUDA(cudaMemcpyAsync(&f->h->oflag, f->oflag, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "fused: tiles");
        GC_CUDA(cudaStreamSynchronize(st), "fused: tiles");
        if (f->h->oflag & GC_FLAG_TILE_FULL) return GC_OK;   // the caller switches to lists
        if (f->h->tchunks > f->tent_chunks) GC_TRY(tiles_alloc_entries(f, (size_t)(f->h->tchunks * 1.125) + 64));
    }
    fk_tile_build<true><<<nb, kTileBS, 0, st>>>(K, f->dsys, f->cube_sys, f->sb.cnt, bpos, cut * cut, rep * rep,
                                                f->tnb, f->toff, f->tent, f->tent_chunks, f->oflag, f->tpairs);
    GC_CHECK_LAUNCH("fused: tile fill");
    return GC_OK;
}

// Per-particle lists of the Bound2 slots (their mobile neighbours within
// rc + skin), for the wall velocity.
int wall_lists(GcFused* f, cudaStream_t st, const float4* bpos, bool host) {
    if (!any_bound2(f)) return GC_OK;
    const int n = f->n, nb = gc_blocks(n, f->block);
    const float cut = f->p.rc + f->skin;
    for (int attempt = 0; attempt < 4; ++attempt) {
        if (host) {
            GC_CUDA(cudaMemsetAsync(f->oflag, 0, sizeof(unsigned), st), "fused: flags");
            GC_CUDA(cudaMemsetAsync(f->need, 0, sizeof(int), st), "fused: flags");
        }
        fk_build_list<<<nb, f->block, 0, st>>>(n, f->dsys, f->a.sys, bpos, f->sb.cnt, f->nbr, f->cnt, f->cap,
                                              cut * cut, f->oflag, f->need, 1);
        GC_CHECK_LAUNCH("fused: wall lists");
        if (!host) return GC_OK;
        GC_CUDA(cudaMemcpyAsync(&f->h->oflag, f->oflag, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "fused: flags");
        GC_CUDA(cudaMemcpyAsync(&f->h->need, f->need, sizeof(int), cudaMemcpyDeviceToHost, st), "fused: flags");
        GC_CUDA(cudaStreamSynchronize(st), "fused: flags");
        if (!(f->h->oflag & GC_FLAG_CELL_OVERFLOW)) return GC_OK;
        GC_TRY(alloc_list(f, grown_capacity(f, 2 * f->cap)));
    }
    return gc_fail(GC_EDEVICE, "fused: wall lists overflow %d entries", f->cap);
}

template <bool ENS>
int tile_density_launch(GcFused* f, cudaStream_t st, const GcParams& p) {
    const int K = f->K, n = f->n;
    fk_tile_density<ENS><<<(K + kTileWarps - 1) / kTileWarps, kTileBS, 0, st>>>(
        K, p, f->hsys[0], f->dsys, f->cube_sys, f->sb.cnt, f->tnb, f->toff, f->tent, f->tent_chunks, f->a.pos, f->pd,
        n);
    GC_CHECK_LAUNCH("fused: tile density");
    fk_tile_dfinish<ENS><<<gc_blocks(n, f->block), f->block, 0, st>>>(n, p, f->hsys[0], f->dsys, f->a.sys, f->a.pos,
                                                                      f->keys, f->bmask, f->pd, f->dp);
    GC_CHECK_LAUNCH("fused: tile density finish");
    if (any_bound2(f)) {
        fk_tile_wallvel<ENS><<<gc_blocks(n, f->block), f->block, 0, st>>>(n, p, f->hsys[0], f->dsys, f->a.sys,
                                                                          f->a.pos, f->a.vpred, f->a.vh, f->nbr,
                                                                          f->cnt, f->cap);
        GC_CHECK_LAUNCH("fused: tile wall velocity");
    }
    return GC_OK;
}

template <bool ENS>
int tile_force_launch(GcFused* f, cudaStream_t st, const GcParams& p, int drive) {
    const int K = f->K, n = f->n;
    fk_tile_force<ENS><<<(K + kTileWarps - 1) / kTileWarps, kTileBS, 0, st>>>(
        K, p, f->hsys[0], f->dsys, f->cube_sys, f->ens || f->capturing ? f->nkey : nullptr, f->sb.cnt, f->tnb, f->toff,
        f->tent, f->tent_chunks, f->a.pos,
        f->a.vpred, f->dp, f->pf, n, f->flags);
    GC_CHECK_LAUNCH("fused: tile force");
    const float4* mf = f->ncell > 0 ? f->mforce : nullptr;
    fk_tile_ffinish<ENS><<<gc_blocks(n, f->block), f->block, 0, st>>>(n, p, f->hsys[0], f->dsys, f->a.sys, f->a.pos,
                                                                      f->keys, f->bmask, f->pf, f->a.vh, mf,
                                                                      f->a.force, f->a.vel, drive);
    GC_CHECK_LAUNCH("fused: tile force finish");
    return GC_OK;
}

int launch_tile_density(GcFused* f, cudaStream_t st, const GcParams& p, bool mark) {
    if (mark) prof_mark(f, st);
    GC_TRY(f->ens ? tile_density_launch<true>(f, st, p) : tile_density_launch<false>(f, st, p));
    if (mark) prof_mark(f, st);
    return GC_OK;
}

int launch_tile_force(GcFused* f, cudaStream_t st, const GcParams& p, int drive, bool mark) {
    if (mark) prof_mark(f, st);
    GC_TRY(f->ens ? tile_force_launch<true>(f, st, p, drive) : tile_force_launch<false>(f, st, p, drive));
    if (mark) prof_mark(f, st);
    return GC_OK;
}

template <bool ENS>
__global__ void fk_tile_wallvel(int n, GcParams p, SysInfo s0, const SysInfo* __restrict__ sys,
                                const int* __restrict__ sysid, const float4* __restrict__ pos, float4* __restrict__ v,
                                const float4* __restrict__ vh, const int* __restrict__ nbr,
                                const int* __restrict__ cnt, int cap) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 xi4 = pos[i];
    GC_SYS_OF(S, i);
    if (stype(fid(xi4), S) != PT_B2) return;
    const Box B = box_of(S);
    const float3 xi = xyz(xi4);
    float3 num = f3(0.f, 0.f, 0.f);
    float den = 0.f;
    const int c = cnt[i];
    for (int k = 0; k < c; ++k) {
        const int j = __ldg(nbr + sell(i, k, cap));
        const float r2 = norm2_rn(pair_image(xi, xyz(pos[j]), B));
        if (r2 >= p.rc2) continue;
        const float w = wendland_w(r2 > 0.f ? r2 * rsqrtf(r2) : 0.f, p);
        const float4 vj = v[j];
        num += w * f3(vj.x, vj.y, vj.z);
        den += w;
    }
    const float4 w4 = vh[i];
    const float3 r = den > 0.f ? f3(2.f * w4.x - num.x / den, 2.f * w4.y - num.y / den, 2.f * w4.z - num.z / den)
                               : f3(w4.x, w4.y, w4.z);
    v[i] = make_float4(r.x, r.y, r.z, 0.f);
}

}  // namespace gcf
