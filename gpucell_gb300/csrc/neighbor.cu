// neighbor.cu -- the neighbour grid: GPUCell's cudiv:: entry points
// (src/ConfigDomain.cuh:11-15), called once per step by Particle::ConCubeList
// (src/Particle.cu:666-678) in the order PreConList -> Sort ->
// CalBeginEndCube -> SortArraysWithCells / SortBasicArrays.
//
// Slot bookkeeping (kept from the reference call sites): d_sortpart[slot] is
// the original id of the particle in that slot (the output writers rely on
// it, src/Particle.cu:734) and d_curpos[id] its slot.  PreConList saves the
// ids in d_oldpos and puts the slot number in d_sortpart, so that after the
// key/value sort d_sortpart[new slot] = old slot: the gather permutation.
// The array sort then restores d_sortpart to ids.
//
// The sort is a stable counting sort by cube: a warp-aggregated count, one
// device-wide exclusive scan of the cube counts, a scatter, and a per-cube
// rank fix that restores the input order inside each cube.  The result is
// exactly that of a stable radix sort, with one pass over the keys instead of
// one per digit.
#include "gc_internal.cuh"

#include <stdio.h>

#include <mutex>

namespace {

constexpr int kBS = 256;

// --------------------------------------------------------------------------
// K4: cube coordinates and keys
// --------------------------------------------------------------------------
__global__ void k_preconlist(int n, GcParams p, const float3* __restrict__ coor, int3* __restrict__ cc,
                             int* __restrict__ cubepart, int* __restrict__ sortpart, int* __restrict__ oldpos) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 x = coor[i];
    int cx = cube_coord(x.x, 0, p.g), cy = cube_coord(x.y, 1, p.g), cz = cube_coord(x.z, 2, p.g);
    cc[i] = make_int3(cx, cy, cz);
    cubepart[i] = cube_key(cx, cy, cz, p.g);
    oldpos[i] = sortpart[i];
    sortpart[i] = i;
}

// --------------------------------------------------------------------------
// K5: stable counting sort
// --------------------------------------------------------------------------

// Count keys per cube; rank[i] = position of element i among the elements of
// its cube in arrival order of the atomics (made stable later).
__global__ void k_sort_count(int n, int K, const int* __restrict__ keys, unsigned* __restrict__ cnt,
                             unsigned* __restrict__ rank, unsigned* flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool act = i < n;
    int k = act ? keys[i] : -1;
    if (act && (k < 0 || k >= K)) {
        raise_flag(flags, GC_FLAG_BAD_INDEX);
        k = k < 0 ? 0 : K - 1;
    }
    unsigned mask = __ballot_sync(0xffffffffu, act);
    if (!act) return;
    unsigned peers = __match_any_sync(mask, k);
    int lane = threadIdx.x & 31;
    int leader = __ffs(peers) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(&cnt[k], (unsigned)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    rank[i] = base + __popc(peers & ((1u << lane) - 1u));
}

__global__ void k_sort_scatter(int n, int K, const int* __restrict__ keys, const int* __restrict__ vals,
                               const unsigned* __restrict__ start, const unsigned* __restrict__ rank,
                               int* __restrict__ okey, int* __restrict__ oval, int* __restrict__ osrc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int k = keys[i];
    k = k < 0 ? 0 : (k >= K ? K - 1 : k);
    unsigned d = start[k] + rank[i];
    okey[d] = k;
    oval[d] = vals[i];
    osrc[d] = i;
}

// One warp per cube: the final position of each element inside its cube is
// the number of elements of that cube that came earlier in the input.
__global__ void k_sort_fix(int K, const unsigned* __restrict__ start, const int* __restrict__ tkey,
                           const int* __restrict__ tval, const int* __restrict__ tsrc, int* __restrict__ keys,
                           int* __restrict__ vals) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (warp >= K) return;
    unsigned b = start[warp], e = start[warp + 1];
    unsigned c = e - b;
    if (c == 0) return;
    if (c <= 32) {
        int src = lane < (int)c ? tsrc[b + lane] : 0x7fffffff;
        int r = 0;
        for (int t = 0; t < (int)c; ++t) {
            int o = __shfl_sync(0xffffffffu, src, t);
            r += (o < src);
        }
        if (lane < (int)c) {
            keys[b + r] = tkey[b + lane];
            vals[b + r] = tval[b + lane];
        }
    } else {
        for (unsigned q = lane; q < c; q += 32) {
            int src = tsrc[b + q];
            unsigned r = 0;
            for (unsigned t = 0; t < c; ++t) r += (tsrc[b + t] < src);
            keys[b + r] = tkey[b + q];
            vals[b + r] = tval[b + q];
        }
    }
}

// --------------------------------------------------------------------------
// Device-wide exclusive scan of uint32 (two levels: 4096 per block, block
// sums scanned by one block).  Writes out[0..n] with out[n] = total.
// --------------------------------------------------------------------------
constexpr int kScanBS = 1024, kScanIPT = 4, kScanTile = kScanBS * kScanIPT;

__device__ unsigned block_exclusive_scan(unsigned v, unsigned* sh, unsigned* total) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    if (wid == 0) {
        unsigned w = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        sh[lane] = w;
    }
    __syncthreads();
    unsigned warp_off = wid ? sh[wid - 1] : 0;
    *total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_off + x - v;
}

__global__ void k_scan_tiles(int n, const unsigned* in, unsigned* out,  // may alias (in-place scan)
                             unsigned* __restrict__ bsum) {
    __shared__ unsigned sh[32];
    long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanIPT;
    unsigned v[kScanIPT], s = 0;
#pragma unroll
    for (int k = 0; k < kScanIPT; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0u;
        s += v[k];
    }
    unsigned tot;
    unsigned off = block_exclusive_scan(s, sh, &tot);
#pragma unroll
    for (int k = 0; k < kScanIPT; ++k) {
        if (base + k < n) out[base + k] = off;
        off += v[k];
    }
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void k_scan_bsums(int nb, unsigned* __restrict__ bsum, unsigned* __restrict__ total_out) {
    __shared__ unsigned sh[32];
    unsigned v[kScanIPT], s = 0;
    int base = threadIdx.x * kScanIPT;
#pragma unroll
    for (int k = 0; k < kScanIPT; ++k) {
        v[k] = (base + k < nb) ? bsum[base + k] : 0u;
        s += v[k];
    }
    unsigned tot;
    unsigned off = block_exclusive_scan(s, sh, &tot);
#pragma unroll
    for (int k = 0; k < kScanIPT; ++k) {
        if (base + k < nb) bsum[base + k] = off;
        off += v[k];
    }
    if (threadIdx.x == 0) *total_out = tot;
}

__global__ void k_scan_add(int n, unsigned* __restrict__ out, const unsigned* __restrict__ bsum) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += bsum[i / kScanTile];
}

__global__ void k_maxkey(int n, const int* __restrict__ keys, int* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int k = i < n ? keys[i] : 0;
#pragma unroll
    for (int o = 16; o; o >>= 1) k = max(k, __shfl_xor_sync(0xffffffffu, k, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, k);
}

// --------------------------------------------------------------------------
// K6: [begin, end) of every cube from the sorted keys; empty cubes (0, 0).
// --------------------------------------------------------------------------
__global__ void k_begin_end(int n, int sizecube, const int* __restrict__ keys, int2* __restrict__ bec) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int k = keys[i];
    if (k < 0 || k >= sizecube) return;
    if (i == 0 || keys[i - 1] != k) bec[k].x = i;
    if (i == n - 1 || keys[i + 1] != k) bec[k].y = i + 1;
}

// --------------------------------------------------------------------------
// K7: gather the particle arrays into the new slot order.
// --------------------------------------------------------------------------
struct GatherBufs {
    float3* coor; int3* cc; float4* velrhop; float3* velhalf; float3* force; float* press; int3* nthro;
};

__global__ void k_gather(int n, int* __restrict__ sortpart, const int* __restrict__ oldpos, int* __restrict__ curpos,
                         const float3* __restrict__ coor, const int3* __restrict__ cc, const float4* __restrict__ velrhop,
                         const float3* __restrict__ velhalf, const float3* __restrict__ force,
                         const float* __restrict__ press, const int3* __restrict__ nthro, GatherBufs o,
                         unsigned* flags) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    int s = sortpart[q];
    if (s < 0 || s >= n) {   // not a permutation from Sort: refuse to read out of bounds
        raise_flag(flags, GC_FLAG_BAD_INDEX);
        return;
    }
    o.coor[q] = coor[s];
    o.cc[q] = cc[s];
    o.velrhop[q] = velrhop[s];
    o.velhalf[q] = velhalf[s];
    o.force[q] = force[s];
    o.press[q] = press[s];
    if (nthro) o.nthro[q] = nthro[s];
    int id = oldpos[s];
    sortpart[q] = id;
    if (curpos) {
        if (id >= 0 && id < n) curpos[id] = q;
        else raise_flag(flags, GC_FLAG_BAD_INDEX);
    }
}

// In-place exclusive scan of buf[0..n) with buf[n] = total; `bsum` holds
// (n / kScanTile + 1) block sums.
int scan_exclusive_with(unsigned* buf, int n, unsigned* bsum, cudaStream_t st) {
    int nb = (n + kScanTile - 1) / kScanTile;
    if (nb > kScanTile) return gc_fail(GC_EINVAL, "scan of %d elements exceeds the two-level limit", n);
    k_scan_tiles<<<nb, kScanBS, 0, st>>>(n, buf, buf, bsum);
    GC_CHECK_LAUNCH("scan: tiles");
    k_scan_bsums<<<1, kScanBS, 0, st>>>(nb, bsum, buf + n);
    GC_CHECK_LAUNCH("scan: block sums");
    k_scan_add<<<gc_blocks(n, kBS), kBS, 0, st>>>(n, buf, bsum);
    GC_CHECK_LAUNCH("scan: add");
    return GC_OK;
}

// The stable counting sort on caller-provided temporaries.
int sort_with(int n, int K, int* keys, int* vals, const GcSortBufs& b, unsigned* flags, cudaStream_t st) {
    if (n <= 0) return GC_OK;
    GC_CUDA(cudaMemsetAsync(b.cnt, 0, (size_t)(K + 1) * sizeof(unsigned), st), "sort: clear counts");
    k_sort_count<<<gc_blocks(n, kBS), kBS, 0, st>>>(n, K, keys, b.cnt, b.rank, flags);
    GC_CHECK_LAUNCH("sort: count");
    GC_TRY(scan_exclusive_with(b.cnt, K, b.bsum, st));
    k_sort_scatter<<<gc_blocks(n, kBS), kBS, 0, st>>>(n, K, keys, vals, b.cnt, b.rank, b.tkey, b.tval, b.tsrc);
    GC_CHECK_LAUNCH("sort: scatter");
    k_sort_fix<<<gc_blocks((long long)K * 32, kBS), kBS, 0, st>>>(K, b.cnt, b.tkey, b.tval, b.tsrc, keys, vals);
    GC_CHECK_LAUNCH("sort: fix");
    return GC_OK;
}

size_t round256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace

// Start of every key's range after the latest gc_counting_sort: K + 1
// entries, valid until the next sort.
const unsigned* gc_sort_starts() { return (const unsigned*)gc_state().scratch[SCR_SORT_COUNT]; }

// Stable sort of (keys, values) by key in [0, K); shared by K5 and the fused
// step.  `keys` and `vals` are sorted in place.
int gc_counting_sort(int n, int K, int* keys, int* vals, cudaStream_t st) {
    if (n <= 0) return GC_OK;
    GcSortBufs b;
    b.cnt = (unsigned*)gc_scratch(SCR_SORT_COUNT, (size_t)(K + 1) * sizeof(unsigned));
    b.rank = (unsigned*)gc_scratch(SCR_SORT_RANK, (size_t)n * sizeof(unsigned));
    b.tkey = (int*)gc_scratch(SCR_SORT_KEY, (size_t)n * sizeof(int));
    b.tval = (int*)gc_scratch(SCR_SORT_VAL, (size_t)n * sizeof(int));
    b.tsrc = (int*)gc_scratch(SCR_SORT_SRC, (size_t)n * sizeof(int));
    b.bsum = (unsigned*)gc_scratch(SCR_SCAN_BLOCKS, (size_t)(K / kScanTile + 2) * sizeof(unsigned));
    if (!b.cnt || !b.rank || !b.tkey || !b.tval || !b.tsrc || !b.bsum) return GC_ENOMEM;
    return sort_with(n, K, keys, vals, b, gc_flags_ptr(), st);
}

size_t gc_sort_bufs_bytes(int n, int K) {
    size_t nn = (size_t)(n > 0 ? n : 1), kk = (size_t)(K > 0 ? K : 1);
    return round256((kk + 1) * 4) + 4 * round256(nn * 4) + round256((kk / kScanTile + 2) * 4);
}

void gc_sort_bufs_carve(void* base, int n, int K, GcSortBufs* b) {
    size_t nn = (size_t)(n > 0 ? n : 1), kk = (size_t)(K > 0 ? K : 1);
    unsigned char* p = (unsigned char*)base;
    b->cnt = (unsigned*)p;
    p += round256((kk + 1) * 4);
    b->rank = (unsigned*)p;
    p += round256(nn * 4);
    b->tkey = (int*)p;
    p += round256(nn * 4);
    b->tval = (int*)p;
    p += round256(nn * 4);
    b->tsrc = (int*)p;
    p += round256(nn * 4);
    b->bsum = (unsigned*)p;
}

int gc_counting_sort_bufs(int n, int K, int* keys, int* vals, const GcSortBufs& b, unsigned* flags,
                          cudaStream_t st) {
    return sort_with(n, K, keys, vals, b, flags, st);
}

size_t gc_scan_blocks(int n) { return (size_t)(n / kScanTile + 2); }

int gc_scan_exclusive(unsigned* buf, int n, unsigned* bsum, cudaStream_t st) {
    if (n <= 0) return GC_OK;
    return scan_exclusive_with(buf, n, bsum, st);
}

extern "C" {

// K4 -- src/ConfigDomain.cuh:11, src/Particle.cu:668.  The cube geometry is
// the library's own (see GcGrid); d_invwid and d_ncube, which the host filled
// with the reference geometry, are not read.
int gc_cudiv_PreConList(int n, int cutradius, float* d_totalcoor, float* d_bboxsph, float* d_invwid, int* d_ncube,
                        int* d_cc, int* d_cubepart, int* d_sortpart, int* d_oldpos) {
    if (gc_state().in_fused_step) return GC_OK;
    (void)cutradius; (void)d_invwid; (void)d_ncube;
    GcState& s = gc_state();
    if (n < 0) return gc_fail(GC_EINVAL, "PreConList: n < 0");
    GC_TRY(gc_ensure_grid(d_bboxsph));
    GcParams p;
    GC_TRY(gc_make_params(&p, true));
    if (n == 0) return GC_OK;
    k_preconlist<<<gc_blocks(n, DIVSIZE), DIVSIZE, 0, s.stream>>>(n, p, (const float3*)d_totalcoor, (int3*)d_cc,
                                                                d_cubepart, d_sortpart, d_oldpos);
    GC_CHECK_LAUNCH("PreConList");
    return GC_OK;
}

// K5 -- src/ConfigDomain.cuh:12, src/Particle.cu:669.
int gc_cudiv_Sort(int n, int* keys, int* values) {
    if (gc_state().in_fused_step) return GC_OK;
    GcState& s = gc_state();
    if (n < 0) return gc_fail(GC_EINVAL, "Sort: n < 0");
    if (n == 0) return GC_OK;
    if (!keys || !values) return gc_fail(GC_EINVAL, "Sort: NULL array");
    int K;
    if (s.grid_set) {
        K = s.grid.ncells;
    } else {
        int* mk = (int*)gc_scratch(SCR_MAXKEY, sizeof(int));
        if (!mk) return GC_ENOMEM;
        GC_CUDA(cudaMemsetAsync(mk, 0, sizeof(int), s.stream), "Sort: max key");
        k_maxkey<<<gc_blocks(n, kBS), kBS, 0, s.stream>>>(n, keys, mk);
        GC_CHECK_LAUNCH("Sort: max key");
        int h = 0;
        GC_CUDA(cudaMemcpyAsync(&h, mk, sizeof(int), cudaMemcpyDeviceToHost, s.stream), "Sort: max key");
        GC_CUDA(cudaStreamSynchronize(s.stream), "Sort: max key");
        K = h + 1;
    }
    return gc_counting_sort(n, K, keys, values, s.stream);
}

// K6 -- src/ConfigDomain.cuh:13, src/Particle.cu:672.
int gc_cudiv_CalBeginEndCube(int n, int sizecube, int* d_cubepart, int* d_beginendcube) {
    if (gc_state().in_fused_step) return GC_OK;
    GcState& s = gc_state();
    if (n < 0 || sizecube <= 0) return gc_fail(GC_EINVAL, "CalBeginEndCube: bad sizes (%d, %d)", n, sizecube);
    if (s.grid_set && s.grid.ncells > sizecube)
        return gc_fail(GC_EINVAL, "CalBeginEndCube: grid has %d cubes but SizeCube is %d", s.grid.ncells, sizecube);
    GC_CUDA(cudaMemsetAsync(d_beginendcube, 0, (size_t)sizecube * sizeof(int2), s.stream), "CalBeginEndCube: clear");
    if (n == 0) return GC_OK;
    k_begin_end<<<gc_blocks(n, DIVSIZE), DIVSIZE, 0, s.stream>>>(n, sizecube, d_cubepart, (int2*)d_beginendcube);
    GC_CHECK_LAUNCH("CalBeginEndCube");
    return GC_OK;
}

static int sort_arrays(int n, int* d_sortpart, int* d_oldpos, int* d_curpos, float* d_totalcoor, int* d_cc,
                       float* d_velrhop, float* d_velhalf, float* d_totalforce, float* d_press, int* d_nthro) {
    GcState& s = gc_state();
    if (n < 0) return gc_fail(GC_EINVAL, "SortArrays: n < 0");
    if (n == 0) return GC_OK;
    const size_t per = 12 + 12 + 16 + 12 + 12 + 4 + (d_nthro ? 12 : 0);
    char* buf = (char*)gc_scratch(SCR_GATHER, per * (size_t)n + 256);
    if (!buf) return GC_ENOMEM;
    GatherBufs o;
    size_t off = 0;
    auto take = [&](size_t bytes) { char* p = buf + off; off += (bytes + 15) & ~(size_t)15; return p; };
    o.velrhop = (float4*)take(16 * (size_t)n);
    o.coor = (float3*)take(12 * (size_t)n);
    o.cc = (int3*)take(12 * (size_t)n);
    o.velhalf = (float3*)take(12 * (size_t)n);
    o.force = (float3*)take(12 * (size_t)n);
    o.press = (float*)take(4 * (size_t)n);
    o.nthro = d_nthro ? (int3*)take(12 * (size_t)n) : nullptr;
    k_gather<<<gc_blocks(n, DIVSIZE), DIVSIZE, 0, s.stream>>>(
        n, d_sortpart, d_oldpos, d_curpos, (const float3*)d_totalcoor, (const int3*)d_cc, (const float4*)d_velrhop,
        (const float3*)d_velhalf, (const float3*)d_totalforce, d_press, (const int3*)d_nthro, o, gc_flags_ptr());
    GC_CHECK_LAUNCH("SortArrays: gather");
    // The caller's pointers are fixed (src/Particle.cu:575-589), so the
    // gathered arrays are copied back.
    GC_CUDA(cudaMemcpyAsync(d_totalcoor, o.coor, 12 * (size_t)n, cudaMemcpyDeviceToDevice, s.stream), "copy back");
    GC_CUDA(cudaMemcpyAsync(d_cc, o.cc, 12 * (size_t)n, cudaMemcpyDeviceToDevice, s.stream), "copy back");
    GC_CUDA(cudaMemcpyAsync(d_velrhop, o.velrhop, 16 * (size_t)n, cudaMemcpyDeviceToDevice, s.stream), "copy back");
    GC_CUDA(cudaMemcpyAsync(d_velhalf, o.velhalf, 12 * (size_t)n, cudaMemcpyDeviceToDevice, s.stream), "copy back");
    GC_CUDA(cudaMemcpyAsync(d_totalforce, o.force, 12 * (size_t)n, cudaMemcpyDeviceToDevice, s.stream), "copy back");
    GC_CUDA(cudaMemcpyAsync(d_press, o.press, 4 * (size_t)n, cudaMemcpyDeviceToDevice, s.stream), "copy back");
    if (d_nthro)
        GC_CUDA(cudaMemcpyAsync(d_nthro, o.nthro, 12 * (size_t)n, cudaMemcpyDeviceToDevice, s.stream), "copy back");
    return GC_OK;
}

// K7 -- src/ConfigDomain.cuh:14, src/Particle.cu:677 (no membrane cells).
int gc_cudiv_SortBasicArrays(int n, int* d_sortpart, int* d_oldpos, float* d_totalcoor, int* d_cc, float* d_velrhop,
                             float* d_velhalf, float* d_totalforce, float* d_press) {
    if (gc_state().in_fused_step) return GC_OK;
    return sort_arrays(n, d_sortpart, d_oldpos, nullptr, d_totalcoor, d_cc, d_velrhop, d_velhalf, d_totalforce,
                       d_press, nullptr);
}

// K7 -- src/ConfigDomain.cuh:15, src/Particle.cu:675 (with cells: also the
// crossing counts and the id -> slot map).
int gc_cudiv_SortArraysWithCells(int n, int* d_sortpart, int* d_oldpos, int* d_curpos, float* d_totalcoor, int* d_cc,
                                 float* d_velrhop, float* d_velhalf, float* d_totalforce, float* d_press,
                                 int* d_nthrobound) {
    gc_state().ref.curpos = d_curpos;
    if (gc_state().in_fused_step) return GC_OK;
    if (!d_curpos) return gc_fail(GC_EINVAL, "SortArraysWithCells: curpos is NULL");
    return sort_arrays(n, d_sortpart, d_oldpos, d_curpos, d_totalcoor, d_cc, d_velrhop, d_velhalf, d_totalforce,
                       d_press, d_nthrobound);
}

// src/ConfigDomain.cuh:17 -- declared but never called by the reference.
int gc_cudiv_Printf(int n, int* d_curpos, int* d_sortpart, float* d_totalcoor) {
    GcState& s = gc_state();
    int m = n < 16 ? n : 16;
    if (m <= 0) return GC_OK;
    int sp[16], cp[16];
    float xyz[48];
    GC_CUDA(cudaStreamSynchronize(s.stream), "Printf");
    GC_CUDA(cudaMemcpy(sp, d_sortpart, m * sizeof(int), cudaMemcpyDeviceToHost), "Printf");
    GC_CUDA(cudaMemcpy(xyz, d_totalcoor, m * 12, cudaMemcpyDeviceToHost), "Printf");
    if (d_curpos) GC_CUDA(cudaMemcpy(cp, d_curpos, m * sizeof(int), cudaMemcpyDeviceToHost), "Printf");
    for (int i = 0; i < m; ++i)
        printf("slot %d id %d curpos %d pos %g %g %g\n", i, sp[i], d_curpos ? cp[i] : -1, xyz[3 * i], xyz[3 * i + 1],
               xyz[3 * i + 2]);
    return GC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// The stable sort of cudiv::Sort without any device allocation.
//
// gc_cudiv_Sort grows library scratch with cudaMalloc (and may cudaFree a
// smaller buffer first, which synchronises the device).  Some callers cannot
// allow that: a host program that reserves the device memory it will use up
// front and must not see a library take more, a process sharing a GPU under
// a fixed memory cap, or a loop that must not stall on the implicit device
// synchronisation of cudaFree.  gc_cudiv_Sort_noalloc runs the same kernels
// with their temporaries in the fixed array below instead.
//
// The array is a file-scope __device__ variable: every GPU that loads the
// library holds it (about 5.2 MB) until the process exits.  In host code its
// name is only a stand-in for the symbol, not a device address, so its
// device address is looked up once per device with cudaGetSymbolAddress and
// passed to the kernels.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNaAlign = 256;
constexpr size_t na_round(size_t b) { return (b + kNaAlign - 1) / kNaAlign * kNaAlign; }
constexpr size_t kNaCount = na_round(((size_t)GC_NOALLOC_SORT_MAX_KEYS + 1) * sizeof(unsigned));
constexpr size_t kNaArray = na_round((size_t)GC_NOALLOC_SORT_MAX_N * sizeof(int));
constexpr size_t kNaBlocks = na_round(((size_t)GC_NOALLOC_SORT_MAX_KEYS / kScanTile + 2) * sizeof(unsigned));
constexpr size_t kNaMaxKey = na_round(sizeof(int));
constexpr size_t kNaStatus = na_round(sizeof(unsigned));
// counts | rank | keys | values | input positions | scan block sums | max key | status
constexpr size_t kNaBytes = kNaCount + 4 * kNaArray + kNaBlocks + kNaMaxKey + kNaStatus;
constexpr size_t kNaStatusOffset = kNaBytes - kNaStatus;

static __device__ __align__(256) unsigned char g_noalloc_sort_scratch[kNaBytes];

constexpr int kNaMaxDevices = 64;
unsigned char* g_na_base[kNaMaxDevices] = {};
std::mutex g_na_mutex;

// Device address of the scratch array on the current device (looked up on
// the first call per device; with lookup = false, nullptr until then).
int noalloc_base(unsigned char** out, bool lookup = true) {
    int dev = 0;
    *out = nullptr;
    GC_CUDA(cudaGetDevice(&dev), "Sort_noalloc: current device");
    if (dev < 0 || dev >= kNaMaxDevices) return gc_fail(GC_EINVAL, "Sort_noalloc: device %d is out of range", dev);
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_base[dev] && lookup) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_sort_scratch);
        if (e != cudaSuccess) return gc_cuda_fail(e, "Sort_noalloc: scratch address");
        g_na_base[dev] = (unsigned char*)p;
    }
    *out = g_na_base[dev];
    return GC_OK;
}

}  // namespace

// The no-allocation sort's status word on the current device (a key outside
// [0, K) raises GC_FLAG_BAD_INDEX there): ORed into *flags and cleared, on
// stream st, without synchronising.  Nothing to do on a device where the sort
// has not run.
int gc_noalloc_status_take(unsigned* flags, cudaStream_t st) {
    unsigned char* base = nullptr;
    GC_TRY(noalloc_base(&base, false));
    if (!base) return GC_OK;
    unsigned* status = (unsigned*)(base + kNaStatusOffset);
    GC_CUDA(cudaMemcpyAsync(flags, status, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "Sort_noalloc: status");
    GC_CUDA(cudaMemsetAsync(status, 0, sizeof(unsigned), st), "Sort_noalloc: status");
    return GC_OK;
}

extern "C" int gc_cudiv_Sort_noalloc(int n, int* keys, int* values) {
    if (n < 0) return gc_fail(GC_EINVAL, "Sort_noalloc: n < 0");
    if (n == 0) return GC_OK;
    if (n > GC_NOALLOC_SORT_MAX_N)
        return gc_fail(GC_EINVAL, "Sort_noalloc: n = %d exceeds the fixed scratch (at most %d elements)", n,
                       GC_NOALLOC_SORT_MAX_N);
    if (!keys || !values) return gc_fail(GC_EINVAL, "Sort_noalloc: NULL array");
    GcState& s = gc_state();
    cudaStream_t st = s.stream;
    unsigned char* base = nullptr;
    GC_TRY(noalloc_base(&base));
    unsigned* cnt = (unsigned*)base;
    unsigned* rank = (unsigned*)(base + kNaCount);
    int* tkey = (int*)(base + kNaCount + kNaArray);
    int* tval = (int*)(base + kNaCount + 2 * kNaArray);
    int* tsrc = (int*)(base + kNaCount + 3 * kNaArray);
    unsigned* bsum = (unsigned*)(base + kNaCount + 4 * kNaArray);
    int* maxkey = (int*)(base + kNaCount + 4 * kNaArray + kNaBlocks);
    // a key outside [0, K) is clamped, as gc_cudiv_Sort does, and raises
    // GC_FLAG_BAD_INDEX in this word (read by gc_device_status); the array is
    // zero when the library loads and the word is cleared when it is read
    unsigned* status = (unsigned*)(base + kNaStatusOffset);
    int K;
    if (s.grid_set) {
        K = s.grid.ncells;
    } else {
        GC_CUDA(cudaMemsetAsync(maxkey, 0, sizeof(int), st), "Sort_noalloc: max key");
        k_maxkey<<<gc_blocks(n, kBS), kBS, 0, st>>>(n, keys, maxkey);
        GC_CHECK_LAUNCH("Sort_noalloc: max key");
        int h = 0;
        GC_CUDA(cudaMemcpyAsync(&h, maxkey, sizeof(int), cudaMemcpyDeviceToHost, st), "Sort_noalloc: max key");
        GC_CUDA(cudaStreamSynchronize(st), "Sort_noalloc: max key");
        K = h + 1;
    }
    if (K > GC_NOALLOC_SORT_MAX_KEYS)
        return gc_fail(GC_EINVAL, "Sort_noalloc: %d keys exceed the fixed scratch (at most %d)", K,
                       GC_NOALLOC_SORT_MAX_KEYS);
    GcSortBufs b;
    b.cnt = cnt;
    b.rank = rank;
    b.tkey = tkey;
    b.tval = tval;
    b.tsrc = tsrc;
    b.bsum = bsum;
    GC_TRY(sort_with(n, K, keys, values, b, status, st));
    return GC_OK;
}
