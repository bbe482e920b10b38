// gc_internal.cuh -- shared internals of libgpucell_gb300: the parameter block
// every kernel receives by value, device helpers (minimum image, cube
// coordinates, Wendland C2 kernel, Philox pair noise) and the host-side
// library state.
//
// The method these helpers implement is pinned in oracle/oracle.c (the FP64
// CPU restatement); both follow the same formulas, cited there against the
// literature, because GPUCell's own kernel bodies are not available.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include "gpucell_gb300.h"

// Block sizes named by src/ParticleGPU.cuh:6 and src/ConfigDomain.cuh:7.
#ifndef SDPDSIZE
#define SDPDSIZE 128
#endif
#ifndef DIVSIZE
#define DIVSIZE 128
#endif

// ---------------------------------------------------------------------------
// Grid and parameters
// ---------------------------------------------------------------------------

// Neighbour grid.  Per axis: a periodic axis is cut into floor(L/rc') cubes
// covering [lo, hi); a wall axis is padded by rc on each side and cut into
// floor((L + 2 rc)/rc') cubes, as GPUCell's host does for y and z
// (src/Particle.cu:551-559).  rc' = rc (1 + 1e-4) keeps every cube at least
// rc wide after FP32 rounding of the cube coordinate.  The cube count never
// exceeds the reference's SizeCube for the same box.
struct GcGrid {
    float lo[3], hi[3];     // bounding box
    float L[3], halfL[3];   // box lengths
    float origin[3];        // lower corner of cube 0
    float invw[3];          // cubes per unit length
    int   n[3];             // cubes per axis
    int   ncells;           // n[0]*n[1]*n[2]
    int   pmask;            // periodic axes (1 = x, 2 = y, 4 = z)
};

// Everything a kernel needs, passed by value (kernel parameters live in the
// constant bank, so this costs nothing per thread).
struct GcParams {
    // counts and type boundaries (Structconst, src/TypesDef.cuh:49-78)
    unsigned nB2, nF, nC, nT, nCP;   // nBound2Start, nFluidStart, nCellStart, nTotalPar, nCellPar
    float rc, inv_rc, rc2;
    float mass, inv_mass;
    float c1sq, c2sq;                // SoundSpeed1^2, SoundSpeed2^2
    float rho0;                      // DenInit
    float lambda;                    // VVsigma
    float dt;
    float gx;                        // ConstExtForce (already times Mass)
    float kT;
    // Wendland C2, support rc: W = wnorm (1-s)^4 (1+4s), F = -W'/r = fnorm (1-s)^3
    float wnorm, fnorm, w0;
    // SDPD dissipative/random coefficients (Espanol & Revenga 2003)
    float visA;                      // 5 eta/3 - zeta
    float visB;                      // 5 (zeta + eta/3)
    float sqrtA, sqrtAB;             // sqrt(visA), sqrt(visA + visB)
    float noise_pref;                // 2 kT / dt (0 when the noise is off)
    // Bound1 repulsion (Monaghan 1994, exponents 12 and 4)
    float rep_r0, rep_r0sq, rep_D;
    // Morse aggregation
    float De, beta, r0m, maxcut, maxcut2;
    // pair-noise key of the current step (noise_key(seed, step))
    uint64_t seed;
    uint32_t noise_key;
    GcGrid g;
};

// ---------------------------------------------------------------------------
// Small vector helpers
// ---------------------------------------------------------------------------

__host__ __device__ inline float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__host__ __device__ inline float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ inline float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ inline float3 operator*(float s, float3 a) { return f3(s * a.x, s * a.y, s * a.z); }
__host__ __device__ inline float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__host__ __device__ inline void operator+=(float3& a, float3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
__host__ __device__ inline void operator-=(float3& a, float3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; }
__host__ __device__ inline float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline float3 cross3(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Particle type from the original id (src/Particle.cu:432-435).
enum { PT_B1 = 0, PT_B2 = 1, PT_FLUID = 2, PT_MEMB = 3 };
__device__ __forceinline__ int ptype(unsigned id, const GcParams& p) {
    return id < p.nB2 ? PT_B1 : (id < p.nF ? PT_B2 : (id < p.nC ? PT_FLUID : PT_MEMB));
}
__device__ __forceinline__ bool is_mobile(unsigned id, const GcParams& p) { return id >= p.nF; }
// Members of the SDPD set (Bound2, fluid, membrane); Bound1 only repels.
__device__ __forceinline__ bool is_sdpd(unsigned id, const GcParams& p) { return id >= p.nB2; }

// ---------------------------------------------------------------------------
// Distances.  The neighbour predicate is r^2 < rc^2 with r^2 evaluated in
// FP32 exactly as written here (explicit round-to-nearest, no contraction);
// oracle/oracle.c evaluates the same expression with -ffp-contract=off, so
// both sides select bit-identical neighbour sets.
// ---------------------------------------------------------------------------

__device__ __forceinline__ float min_image_1(float d, int axis, const GcGrid& g) {
    if (g.pmask & (1 << axis)) {
        if (d > g.halfL[axis]) d = __fsub_rn(d, g.L[axis]);
        else if (d < -g.halfL[axis]) d = __fadd_rn(d, g.L[axis]);
    }
    return d;
}

__device__ __forceinline__ float3 min_image(float3 a, float3 b, const GcGrid& g) {
    return f3(min_image_1(__fsub_rn(a.x, b.x), 0, g),
              min_image_1(__fsub_rn(a.y, b.y), 1, g),
              min_image_1(__fsub_rn(a.z, b.z), 2, g));
}

// 1/sqrt(x) by the hardware approximation with subnormal inputs flushed to
// zero (PTX rsqrt.approx.ftz.f32): the pair loops call it only on normal
// numbers (r^2 of two distinct listed particles, positive noise
// amplitudes), where it matches rsqrtf without rsqrtf's subnormal path.
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// |d|^2 with fused multiply-adds: the form the fused step's pair passes use
// (one rounding fewer than norm2_rn; both passes of a step form it alike).
__device__ __forceinline__ float norm2_fma(float3 d) { return fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z)); }

__device__ __forceinline__ float norm2_rn(float3 d) {
    return __fadd_rn(__fadd_rn(__fmul_rn(d.x, d.x), __fmul_rn(d.y, d.y)), __fmul_rn(d.z, d.z));
}

// Cube coordinate along one axis: periodic axes wrap, wall axes clamp (a
// clamped particle is only ever farther from its true neighbours, so the
// 27-cube search stays complete).
__device__ __forceinline__ int cube_coord(float x, int axis, const GcGrid& g) {
    int c = (int)floorf(__fmul_rn(__fsub_rn(x, g.origin[axis]), g.invw[axis]));
    int n = g.n[axis];
    if (g.pmask & (1 << axis)) {
        c %= n;
        if (c < 0) c += n;
    } else {
        c = c < 0 ? 0 : (c >= n ? n - 1 : c);
    }
    return c;
}

__device__ __forceinline__ int cube_key(int cx, int cy, int cz, const GcGrid& g) {
    return cx + g.n[0] * (cy + g.n[1] * cz);
}

// Neighbouring cube index along an axis, or -1 when it falls off a wall axis.
__device__ __forceinline__ int cube_step(int c, int d, int axis, const GcGrid& g) {
    c += d;
    int n = g.n[axis];
    if (c < 0) return (g.pmask & (1 << axis)) ? c + n : -1;
    if (c >= n) return (g.pmask & (1 << axis)) ? c - n : -1;
    return c;
}

// ---------------------------------------------------------------------------
// Wendland C2 kernel in 3-D with support rc (h = rc/2):
//   W(r)     = 21/(2 pi rc^3) (1 - s)^4 (1 + 4 s),   s = r/rc
//   F(r)     = -W'(r)/r = 210/(pi rc^5) (1 - s)^3
// ---------------------------------------------------------------------------

__device__ __forceinline__ float wendland_w(float r, const GcParams& p) {
    float s = r * p.inv_rc;
    float t = 1.f - s;
    float t2 = t * t;
    return p.wnorm * t2 * t2 * (1.f + 4.f * s);
}

__device__ __forceinline__ float wendland_f(float r, const GcParams& p) {
    float t = 1.f - r * p.inv_rc;
    return p.fnorm * t * t * t;
}

// ---------------------------------------------------------------------------
// Pair noise: Philox2x32-10 (Salmon, Moraes, Dror & Shaw, SC'11).
// Counter = (min id, max id); key = a per-step word hashed from the 64-bit
// seed and the step index with the SplitMix64 finaliser (Steele, Lea &
// Flood 2014), computed once per step on the host (noise_key).  The same
// two words on both sides of a pair give an antisymmetric pair noise that
// does not depend on the particle order.
// ---------------------------------------------------------------------------

__host__ __device__ __forceinline__ uint64_t splitmix64_mix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Per-step key of the pair noise.
__host__ __device__ __forceinline__ uint32_t noise_key(uint64_t seed, uint64_t step) {
    return (uint32_t)(splitmix64_mix(seed * 0x9E3779B97F4A7C15ull + step) >> 32);
}

struct Philox2 {
    uint32_t w0, w1;
};

__host__ __device__ __forceinline__ Philox2 philox2x32_10(uint32_t c0, uint32_t c1, uint32_t k) {
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
    for (int r = 0; r < 10; ++r) {
        // one 32x32 -> 64-bit product gives both halves
        uint64_t pr = (uint64_t)0xD256D193u * c0;
        uint32_t hi = (uint32_t)(pr >> 32), lo = (uint32_t)pr;
        c0 = hi ^ k ^ c1;
        c1 = lo;
        k += 0x9E3779B9u;
    }
    return Philox2{c0, c1};
}

// Three uniform variates with zero mean and unit variance from the 63 low
// bits of the two words, 21 bits u each: sqrt(12) ((u + 1/2) / 2^21 - 1/2).
// Groot & Warren (1997) drive the same integrator with uniform noise; only
// the first two moments enter the fluctuation-dissipation balance.  On the
// device the 21 bits become the mantissa of a float in [1, 2), v = 1 + u/2^21,
// and the variate is sqrt(12) v - sqrt(12) (3/2 - 2^-22): no int-to-float
// conversion.
__device__ __forceinline__ float unit_uniform21(uint32_t u) {
    float v = __uint_as_float(0x3F800000u | (u << 2));
    return fmaf(v, 3.4641016151377544f, -3.4641016151377544f * (1.5f - 2.384185791015625e-7f));
}

// The noise components xi_ij for the pair (i, j) without the sign of the
// pair: xi_ij = pair_sign(i, j) * pair_noise_unsigned(i, j).
__device__ __forceinline__ float3 pair_noise_unsigned_k(unsigned id_i, unsigned id_j, uint32_t key) {
    unsigned a = id_i < id_j ? id_i : id_j;
    unsigned b = id_i < id_j ? id_j : id_i;
    Philox2 w = philox2x32_10(a, b, key);
    uint32_t u0 = w.w0 & 0x1FFFFFu;
    uint32_t u1 = (w.w0 >> 21) | ((w.w1 & 0x3FFu) << 11);
    uint32_t u2 = (w.w1 >> 10) & 0x1FFFFFu;
    return f3(unit_uniform21(u0), unit_uniform21(u1), unit_uniform21(u2));
}

__device__ __forceinline__ float3 pair_noise_unsigned(unsigned id_i, unsigned id_j, const GcParams& p) {
    return pair_noise_unsigned_k(id_i, id_j, p.noise_key);
}

__device__ __forceinline__ float pair_sign(unsigned id_i, unsigned id_j) { return id_i < id_j ? 1.f : -1.f; }

// The noise components xi_ij for the pair (i, j); xi_ji = -xi_ij.
__device__ __forceinline__ float3 pair_noise(unsigned id_i, unsigned id_j, const GcParams& p) {
    return pair_sign(id_i, id_j) * pair_noise_unsigned(id_i, id_j, p);
}

// ---------------------------------------------------------------------------
// Device status flags (GC_FLAG_*), one word per device.
// ---------------------------------------------------------------------------

__device__ __forceinline__ void raise_flag(unsigned* flags, unsigned f) {
    if (flags) atomicOr(flags, f);
}

// ---------------------------------------------------------------------------
// Host-side state
// ---------------------------------------------------------------------------

enum GcScratchSlot {
    SCR_FLAGS = 0,
    SCR_SORT_COUNT,      // cube counts / starts (uint32, ncells + 1)
    SCR_SORT_RANK,       // rank of each element within its cube
    SCR_SORT_KEY,        // scattered keys
    SCR_SORT_VAL,        // scattered values
    SCR_SORT_SRC,        // input position of each scattered element
    SCR_SCAN_BLOCKS,     // block sums of the device-wide scan
    SCR_MAXKEY,          // max key when the caller gave no grid
    SCR_GATHER,          // K7 gather buffer (80 bytes per particle)
    SCR_CELLSUM,         // per-cell area / volume sums
    SCR_COUNT_
};

// Caller buffers seen by the boundary entry points (device pointers), kept so
// that the fused engine can run GPUCell's step on them (GPUCELL_ENGINE=fused).
struct GcRefPtrs {
    int *sortpart = nullptr, *curpos = nullptr;
    float *coor = nullptr, *velrhop = nullptr, *velhalf = nullptr, *force = nullptr, *press = nullptr;
    int* nthro = nullptr;
    const float* bbox = nullptr;
    // membranes
    int ncell = 0, ntri = 0, nedge = 0;
    int *tri = nullptr, *betri = nullptr, *edge = nullptr, *celltab = nullptr;
    float *shearmod = nullptr, *bendmod = nullptr, *hlarea = nullptr, *hgarea = nullptr, *hvol = nullptr;
    float *refedgelen = nullptr, *maxrefedgelen = nullptr, *perlen = nullptr, *hpow = nullptr, *hbending = nullptr,
          *reftriangle = nullptr;
    float *trinordir = nullptr, *triarea = nullptr, *reftriarea = nullptr, *tricenter = nullptr;
    float *refarea_para = nullptr, *refvol_para = nullptr, *area_para = nullptr, *vol_para = nullptr;
    float *area = nullptr, *vol = nullptr, *pararea = nullptr, *defforce = nullptr, *aggforce = nullptr;
};

struct GcFused;

struct GcState {
    Structconst c;
    bool consts_set = false;
    int periodic_mask = 1;
    int noise_on = 1;
    long long step = -1;           // last step index seen by UpdateFluidCoor
    cudaStream_t stream = 0;
    float* velhalf_ptr = nullptr;  // caller's VelHalf, for the wall velocity
    // GPUCELL_ENGINE=fused: GPUCell's call sequence drives the fused step
    int engine_mode = 0;           // 0: one kernel per entry point; 1: fused step
    GcFused* engine = nullptr;
    long long plain_steps = 0;     // steps run on the entry-point kernels since ConstsDataUp
    bool in_fused_step = false;    // between UpdateFluidCoor and the end of a fused step
    GcRefPtrs ref;
    // grid cache
    bool grid_set = false;
    const float* grid_bbox_ptr = nullptr;
    int grid_mask = -1;
    float grid_rc = 0.f;
    GcGrid grid{};
    // scratch
    void* scratch[SCR_COUNT_] = {};
    size_t scratch_bytes[SCR_COUNT_] = {};
};

GcState& gc_state();
// Sets the thread's last-error text and returns `code`.
int gc_fail(int code, const char* fmt, ...);
// Maps a CUDA error to GC_ECUDA with a message naming `what`.
int gc_cuda_fail(cudaError_t e, const char* what);
// Grows scratch slot `slot` to at least `bytes`; returns nullptr on failure
// (with the error text set).
void* gc_scratch(int slot, size_t bytes);
unsigned* gc_flags_ptr();
// Reads and clears the no-allocation sort's status word of the current
// device into *flags (asynchronously, on st); nothing before its first call.
int gc_noalloc_status_take(unsigned* flags, cudaStream_t st);
// Fused engine behind the entry points (fused.cu).  gc_engine_step runs one
// fused step on the recorded caller buffers and writes the caller-visible
// state back; gc_engine_reset drops the engine.
int gc_engine_step(int drive_on);
void gc_engine_reset();
// Parameter block for the given constants (no grid, step 0).
int gc_params_from(const Structconst& c, int noise_on, GcParams* p);
// Parameter block for the current constants, grid and step.
int gc_make_params(GcParams* out, bool need_grid);
// Grid of cubes at least `cut` wide over the host bbox `bb` (6 floats).
int gc_build_grid(const float* bb, float cut, int mask, GcGrid* g);
// Stable sort of (keys, vals) by key in [0, K), in place (neighbor.cu).
int gc_counting_sort(int n, int K, int* keys, int* vals, cudaStream_t st);
// Temporaries of the counting sort.  After a sort, cnt[k] is the first
// position of key k and cnt[K] = n.
struct GcSortBufs {
    unsigned* cnt;    // K + 1
    unsigned* rank;   // n
    int *tkey, *tval, *tsrc;   // n each
    unsigned* bsum;   // K / 4096 + 2
};
// Bytes of one allocation that holds the temporaries for n elements and K keys.
size_t gc_sort_bufs_bytes(int n, int K);
// Splits such an allocation into the temporaries.
void gc_sort_bufs_carve(void* base, int n, int K, GcSortBufs* b);
// The same sort as gc_counting_sort on the given temporaries (no library
// scratch, so it can be captured into a CUDA graph).
int gc_counting_sort_bufs(int n, int K, int* keys, int* vals, const GcSortBufs& b, unsigned* flags,
                          cudaStream_t st);
// Device-wide exclusive scan of buf[0..n) in place, buf[n] = total; bsum
// holds gc_scan_blocks(n) block sums (n up to 4096^2).
size_t gc_scan_blocks(int n);
int gc_scan_exclusive(unsigned* buf, int n, unsigned* bsum, cudaStream_t st);
// Start of every key's range (K + 1 entries) after the latest counting sort.
const unsigned* gc_sort_starts();
// (Re)builds the grid from the caller's device bbox pointer.
int gc_ensure_grid(const float* d_bbox);
// Step index that keys the noise of the next force evaluation.
long long gc_noise_step();

// Counts one kernel launch of this library and returns GC_ECUDA if the
// launch failed.  Written after every <<<...>>> so that
// gc_launch_count() is exact.
void gc_count_launch();
// Adjusts the launch count by k.
void gc_add_launches(long long k);
#define GC_CHECK_LAUNCH(what)                                   \
    do {                                                        \
        gc_count_launch();                                      \
        cudaError_t e_ = cudaGetLastError();                    \
        if (e_ != cudaSuccess) return gc_cuda_fail(e_, what);   \
    } while (0)

#define GC_TRY(call)                                            \
    do {                                                        \
        int rc_ = (call);                                       \
        if (rc_ != GC_OK) return rc_;                           \
    } while (0)

#define GC_CUDA(call, what)                                     \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return gc_cuda_fail(e_, what);   \
    } while (0)

inline int gc_blocks(long long n, int bs) { return (int)((n + bs - 1) / bs); }
