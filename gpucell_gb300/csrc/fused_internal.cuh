// fused_internal.cuh -- what the translation units of the fused step share:
// the per-system table, the slot arrays, the handle (GcFused), a few device
// helpers, and the host functions and kernels that more than one of
// fused.cu (state, passes, steps, API), fused_ckpt.cu (checkpoint and
// restart), fused_tune.cu (autotuner), fused_report.cu (per-cell statistics,
// diagnostics, output files) and fused_engine.cu (the engine behind the
// boundary entry points) use.
#pragma once

#include "gc_internal.cuh"

#include <cuda_runtime.h>

#include <vector>

namespace gcf {

constexpr int kBS = 128;      // default threads per block
constexpr int kMaxBS = 256;   // largest block the particle kernels accept

// Pair tiles (the half-stencil passes, fused_tiles.cu): particles are sorted
// by cubes at least rc + skin wide; each cube pairs with itself and its 13
// forward neighbours, and one warp takes a home cube and its 14 pairs.
constexpr int kTilePairs = 14;
constexpr int kTileMax = 96;       // particles per cube the tiles accept (local indices fit a byte)
constexpr int kTileWarps = 4;      // warps per block of the tile kernels
constexpr unsigned kTilePad = 0xFFFFFFFFu;   // padding entry of a pair list

__device__ __forceinline__ unsigned fid(float4 x) { return __float_as_uint(x.w); }
__device__ __forceinline__ float3 xyz(float4 a) { return f3(a.x, a.y, a.z); }

__device__ __forceinline__ size_t sell(int i, int k, int cap) {
    return ((size_t)(i >> 5) * cap + k) * 32 + (i & 31);
}

__device__ __forceinline__ size_t mrow(int i, int w, int mw) {
    return ((size_t)(i >> 5) * mw + w) * 32 + (i & 31);
}

// (hi, lo) += d for a double-float number: Knuth's TwoSum of hi + d, its
// rounding error folded into lo, renormalised by Dekker's Fast2Sum.  The
// _rn intrinsics keep the compiler from contracting or reordering them.
__device__ __forceinline__ void dd_add(float& hi, float& lo, float d) {
    float s = __fadd_rn(hi, d);
    float bb = __fsub_rn(s, hi);
    float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(d, bb));
    float t = __fadd_rn(lo, e);
    hi = __fadd_rn(s, t);
    lo = __fsub_rn(t, __fsub_rn(hi, s));
}

// x += d for a position: double-float (dd_add) or, with ddpos = 0 (the
// plain FP32 variant, GcFusedOptions.fp32_positions), one FP32 addition with
// the low part left as it is (zero).
__device__ __forceinline__ void pos_add(float& hi, float& lo, float d, int ddpos) {
    if (ddpos) dd_add(hi, lo, d);
    else hi = __fadd_rn(hi, d);
}

__device__ __forceinline__ double block_sum_d(double v, double* sh) {
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

// One system of an ensemble: global id ranges, grids, body force, seed.
struct SysInfo {
    uint64_t seed;                   // iSeed of the system (pair noise)
    unsigned id0, b2, fl, cs, end;   // first id; first Bound2, fluid and membrane id; one past the last
    unsigned m0;                     // first membrane index (membrane-ordered arrays)
    int cube0;                       // first global cube of the list grid
    int mcube0;                      // first global cube of the aggregation grid
    float gx;                        // body force in x (ConstExtForce)
    float invL[3];
    int lr;                          // list-grid stencil radius: 2 for cells >= (rc + skin)/2, 1 for cubes >= rc + skin
    int mlr;                         // aggregation-grid stencil radius: 2 for cubes >= MaxCut/2, 1 for cubes >= MaxCut
    GcGrid g;                        // list grid over the box
    GcGrid mg;                       // aggregation grid: cubes at least MaxCut wide
};

// Particle type, system lookup, box constants and the minimum image of a
// listed pair, shared by the list and the tile passes.
__device__ __forceinline__ int stype(unsigned id, const SysInfo& S) {
    return id < S.b2 ? PT_B1 : (id < S.fl ? PT_B2 : (id < S.cs ? PT_FLUID : PT_MEMB));
}

// System of the given global id (binary search over the id ranges).
__device__ __forceinline__ int find_sys(const SysInfo* sys, int nsys, unsigned id) {
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (sys[mid].id0 <= id) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Box constants of the per-step kernels.
struct Box {
    float L[3], invL[3];
    int pmask;
};

__device__ __forceinline__ Box box_of(const SysInfo& S) {
    Box b;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        b.L[a] = S.g.L[a];
        b.invL[a] = S.invL[a];
    }
    b.pmask = S.g.pmask;
    return b;
}

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

// The per-step kernels exist in two forms.  ENS = false: one system, given
// by value in the kernel parameters (constant bank, no per-thread loads).
// ENS = true: the system of each slot comes from the per-slot index and the
// device table (ensembles, and captured steps, whose noise keys are derived
// on the device).
#define GC_SYS_OF(S, i) const SysInfo& S = ENS ? sys[sysid ? sysid[i] : 0] : s0

// Positions are double-float: pos holds the FP32 position (what the pair,
// membrane and list kernels read) and plo the FP32 remainder x - pos, so that
// the position update accumulates with ~48-bit precision while the pair
// kernels keep FP32 arithmetic.
struct SlotArrays {
    float4 *pos, *vel, *vpred, *vh, *force;
    float4* plo;   // low parts of the positions (x, y, z; w unused)
    int4* nthro;
    int* sys;   // system of each slot (nullptr for one system)
};

// Membrane topology of one system as given (local, 1-based), until set-up.
struct HostCells {
    bool set = false;
    int ncell = 0, ntri = 0, nedge = 0;
    std::vector<int> tri, edge, betri, celltab;
    std::vector<int> verts;   // first and last vertex of each cell (0-based), from its triangles
    std::vector<float> shear, bend, hl, hg, hv;
};

// Device copy of the dynamic state (snapshots for captured steps and the
// autotuner).
struct StateCopy {
    SlotArrays s{};
    float4* mpos = nullptr;
    float4* mplo = nullptr;
    int4* mnthro = nullptr;
    long long* dstep = nullptr;
    bool have = false;
};


}  // namespace gcf

namespace gcf {
// Host outputs of gc_fused_step_store, copied while the step still runs.
struct EarlyStore {
    float *pos, *vel, *rho, *press, *force, *velhalf;
    int* nthro;
    float *area, *vol, *defforce, *aggforce, *trinordir, *tricenter, *pararea;
};
}  // namespace gcf

struct GcFused {
    GcParams p;
    int nsys = 1;
    std::vector<gcf::SysInfo> hsys;
    std::vector<GcSystemDesc> desc;
    std::vector<gcf::HostCells> hcells;
    std::vector<int> c0, t0;       // first cell and triangle of each system (after set-up)
    std::vector<char> sys_loaded;
    gcf::SysInfo* dsys = nullptr;
    int K = 0, Kagg = 0;           // cubes of all list grids, of all aggregation grids
    float skin_rel = 0.1f;         // skin in units of CutRadius
    float skin = 0.1f;             // skin length
    int n = 0, cap = 0, block = gcf::kBS;
    int noise_on = 1;
    bool compact = false;
    bool graph = false;            // steps run as captured graphs
    int ddpos = 1;                 // positions double-float (0: plain FP32, GcFusedOptions.fp32_positions)
    bool halfv = false;            // neighbour velocities packed to FP16 for the force pass
    uint2* vph = nullptr;          // those packed velocities (x, y, z, 0 as halves)
    bool ens = false;              // kernels read the system table (several systems)
    bool capturing = false;        // a step is being captured: the noise key comes from the device
    bool has_b1 = true;            // some system has Bound1 wall particles
    long long step = -1;           // index keying the noise of the latest step
    long long rebuilds = 0, steps = 0;
    cudaStream_t st = 0;
    // slot arrays (current, and the permutation target)
    gcf::SlotArrays a{}, b{};
    float4* refpos = nullptr;
    float2* dp = nullptr;
    int* slot_of = nullptr;
    int *keys = nullptr, *vals = nullptr;
    int *nbr = nullptr, *cnt = nullptr;
    size_t nbr_elems = 0;
    unsigned* cmask = nullptr;   // per-step bit mask of the acting list entries
    size_t cmask_elems = 0;
    int* ccnt = nullptr;         // number of acting entries
    int mw = 0;                  // mask words per slot
    int* rebuild = nullptr;
    // pair tiles (GcFusedOptions.tiles): lists per pair of neighbouring
    // cubes built at each rebuild, partial sums per pair direction, finish
    // passes; otherwise per-particle Verlet lists for every slot
    bool lists = true;
    int tK = 0;                     // cubes the per-cube tile arrays hold
    int* cube_sys = nullptr;        // system of each cube
    unsigned short* bmask = nullptr;   // per cube: pair directions whose backward neighbour exists
    int* tnb = nullptr;             // K x 14: neighbour cube of each pair (bit 30: minimum image), -1: none
    unsigned* toff = nullptr;       // K x 14 + 1: chunks of 32 entries per pair, then their exclusive scan
    unsigned* tscan = nullptr;      // block sums of that scan
    unsigned* tent = nullptr;       // pair entries (a | b << 8, kTilePad between lists)
    size_t tent_chunks = 0;         // capacity in chunks of 32 entries
    float* pd = nullptr;            // 14 x n density partial sums
    float* pf = nullptr;            // 14 x 3 x n force partial sums (x, y, z planes)
    unsigned long long* tpairs = nullptr;   // candidate pairs of the latest build
    unsigned* flags = nullptr;
    unsigned* oflag = nullptr;   // list overflow inside captured steps
    int* need = nullptr;         // the longest list an overflowing build wanted
    unsigned long long* stat_sum = nullptr;
    int* stat_max = nullptr;
    long long* dstep = nullptr;  // device step counter (ensembles, captured steps)
    unsigned* nkey = nullptr;    // per-system noise key of the current step
    unsigned long long* drebuilds = nullptr;   // rebuilds inside captured steps
    // pinned words read back after steps: rebuild flag, overflow flag, device rebuild count
    struct Pinned {
        int rebuild;
        unsigned oflag;
        int need;
        unsigned long long drebuilds;
        unsigned tchunks;            // chunks the latest tile build needs
        unsigned long long tpairs;
    }* h = nullptr;
    unsigned long long drebuilds_seen = 0;
    // counting-sort temporaries (owned, so a captured step can use them)
    void* sortmem = nullptr;
    size_t sortmem_bytes = 0;
    int sort_n = 0, sort_K = 0;
    GcSortBufs sb{};
    void* sortmem_agg = nullptr;   // the aggregation sort's own temporaries (the Morse list build)
    int sort_agg_n = 0, sort_agg_K = 0;
    // Morse Verlet lists: per vertex the offset of its entries (ncp + 1,
    // scanned from the counts), per vertex and lane of the build the count,
    // the scan's block sums, the entries (membrane indices) and their
    // capacity, and the membrane positions of a restore
    unsigned* moff = nullptr;
    unsigned* mcnt = nullptr;
    unsigned* mscan = nullptr;
    int* mlist = nullptr;
    size_t mcap = 0;
    double mroom = 1.25;           // Morse entries kept free beyond the latest build (factor)
    double mslack = 0.25;          // more when the entries are reallocated
    size_t mextra = 4096;          // and in addition
    float4* mref = nullptr;
    GcSortBufs sb_agg{};
    // The membrane kernels depend only on the integrated membrane positions:
    // they run on their own stream from the end of the integration to the
    // force pass, beside the rebuild check, the list rebuild and the density.
    cudaStream_t mst = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t xev[4] = {nullptr, nullptr, nullptr, nullptr};   // chunks of a host load / store
    // outputs written while a step runs (gc_fused_step_store, the engine's
    // write-back): called at four points of a host-driven step (0 after the
    // integration and any rebuild, 1 after the density pass, 2 after the
    // membrane passes, 3 at the end) with the step's stream
    int (*early)(GcFused*, cudaStream_t, int) = nullptr;
    const gcf::EarlyStore* es = nullptr;   // gc_fused_step_store's host buffers
    cudaStream_t xst = nullptr;            // the stream of those writes
    cudaEvent_t xe[4] = {nullptr, nullptr, nullptr, nullptr};
    // membranes (global indices over the ensemble)
    int ncell = 0, ntri = 0, nedge = 0, ncp = 0;
    int3* tri = nullptr;
    int6* edge = nullptr;
    int2* betri = nullptr;
    int* celltab = nullptr;
    int *msys = nullptr, *cellsys = nullptr;
    float *shear = nullptr, *bend = nullptr, *hl = nullptr, *hg = nullptr, *hv = nullptr;
    float *l0 = nullptr, *lmax = nullptr, *perlen = nullptr, *hpow = nullptr, *hbend = nullptr, *refang = nullptr;
    float *tarea = nullptr, *reftarea = nullptr;
    float4 *tnorm = nullptr, *tcen = nullptr;
    double *carea = nullptr, *cvol = nullptr, *crefarea = nullptr, *crefvol = nullptr;
    float4 *mpos = nullptr, *mforce = nullptr, *magg = nullptr;
    float4* mplo = nullptr;      // low parts of mpos (the double-float positions of the membrane vertices)
    int4* mnthro = nullptr;
    float* parea = nullptr;
    int *mkeys = nullptr, *mvals = nullptr;
    float4* mspos = nullptr;     // membrane positions in aggregation-grid order (after the aggregation sort)
    float* msarea = nullptr;     // vertex areas in the same order
    bool agg_runs = false;       // every cell's vertices are one contiguous range carrying its CellTab index
    float4* mparts = nullptr;    // per-edge and per-triangle vertex forces (4 per edge, then 3 per triangle)
    int *inc_ptr = nullptr, *inc = nullptr;   // vertex -> its parts (CSR)
    int2* cell_verts = nullptr;  // first and last membrane vertex of each cell (global, inclusive)
    double* cell_stats = nullptr;   // ncell x 12, see gc_ensemble_cell_stats
    double* diag = nullptr;         // diagnostics partial sums and result
    bool cells_adopted = false;   // membranes taken from the boundary entry points' buffers
    bool have_agg = false;
    bool setup_done = false;
    // captured steps
    cudaStream_t gst = nullptr, gst2 = nullptr, gst3 = nullptr;
    cudaGraph_t cg[2] = {};
    cudaGraphExec_t gexec[2] = {};
    bool graph_dirty = true;
    long long kernels_step = 0, kernels_rebuild = 0;   // kernels per captured step and per rebuild body
    gcf::StateCopy snap;    // state at the start of a captured gc_fused_step call
    gcf::StateCopy tsnap;   // state at the start of an autotune
    // optional CUDA-event timing of the dominant kernels (fk_density, fk_force)
    bool profile = false;
    std::vector<cudaEvent_t> ev;   // pairs: density start/stop, force start/stop
    size_t ev_used = 0;
    // staging for host pointers
    void* stage = nullptr;
    size_t stage_bytes = 0;
    std::vector<void*> allocs;
};

namespace gcf {

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

// pair tiles (fused_tiles.cu)
int tiles_grid(GcFused* f);
int tiles_build(GcFused* f, cudaStream_t st, const float4* bpos, bool host);
int tiles_alloc_entries(GcFused* f, size_t chunks);
int launch_tile_density(GcFused* f, cudaStream_t st, const GcParams& p, bool mark);
int launch_tile_force(GcFused* f, cudaStream_t st, const GcParams& p, int drive, bool mark);
int wall_lists(GcFused* f, cudaStream_t st, const float4* bpos, bool host);
bool any_bound2(const GcFused* f);
void prof_mark(GcFused* f, cudaStream_t st);
struct SysInfo;

int stage_bytes(GcFused* f, size_t bytes);
void drop_graphs(GcFused* f);
int alloc_list(GcFused* f, int cap);
int grown_capacity(const GcFused* f, int at_least);
int build_grids(GcFused* f);
int sync_dstep(GcFused* f);
int rebuild_lists(GcFused* f);
int launch_membranes(GcFused* f, cudaStream_t st, const GcParams& p);
int build_morse_lists(GcFused* f, cudaStream_t st, const float4* mp, bool host);
int ensure_early_stream(GcFused* f);
int build_morse_lists_from_ref(GcFused* f, cudaStream_t st);
int one_step(GcFused* f, int drive);
int prepare_graph(GcFused* f, int drive);
int save_state(GcFused* f, StateCopy* c);
int restore_state(GcFused* f, StateCopy* c);
int refresh(GcFused* f);
int alloc_cells(GcFused* f, int ncell, int ntri, int nedge, int ncp);
int build_incidence(GcFused* f, const int* tri, const int* edge);
int check_sys(GcFused* f, int sys, const char* what);
int store_range(GcFused* f, unsigned id_base, int count, float* pos, float* vel, float* rho, float* press,
                float* force, float* velhalf, int* nthro, int to_device);
int store_cells_range(GcFused* f, int c0, int nc, int m0, int nv, int t0, int nt, float* area, float* vol,
                      float* defforce, float* aggforce, float* trinordir, float* tricenter, float* pararea,
                      int to_device);

#ifndef GC_BUILD_MIN_BLOCKS
#define GC_BUILD_MIN_BLOCKS 4   // 64 registers: the build ran 0.554 ms against 0.578 ms unbounded (524k particles)
#endif
__global__ void __launch_bounds__(kMaxBS, GC_BUILD_MIN_BLOCKS) fk_build_list(int n, const SysInfo* __restrict__ sys,
                                                     const int* __restrict__ sysid, const float4* __restrict__ pos,
                                                     const unsigned* __restrict__ start, int* __restrict__ nbr,
                                                     int* __restrict__ cnt, int cap, float cut2, unsigned* flags,
                                                     int* __restrict__ need, int walls_only);

__global__ void fk_gather_mpos(int ncp, const SysInfo* __restrict__ sys, const int* __restrict__ msys,
                               const int* __restrict__ slot_of, const float4* __restrict__ pos,
                               const int4* __restrict__ nthro, const float4* __restrict__ plo,
                               float4* __restrict__ mpos, float4* __restrict__ mplo, int4* __restrict__ mnthro);

__global__ void fk_store_cells(int ncp, int m0, int ntri, int t0, const float4* __restrict__ mforce,
                               const float4* __restrict__ magg, const float* __restrict__ parea,
                               const float4* __restrict__ tnorm, const float4* __restrict__ tcen,
                               float* __restrict__ defforce, float* __restrict__ aggforce, float* __restrict__ pararea,
                               float* __restrict__ trinor, float* __restrict__ tricen, int have_agg);

}  // namespace gcf
