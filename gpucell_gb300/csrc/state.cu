// state.cu -- library state, error reporting, scratch memory, the neighbour
// grid and the K1 entry point (ConstsDataUp, src/ParticleGPU.cuh:10).
//
// Ownership follows GPUCell's host frame: the caller cudaMallocs every
// particle and topology array (src/Particle.cu:573-625) and the boundary has
// no free hook, so the library allocates its own scratch lazily, grows it on
// demand and frees it in gc_shutdown() (also run at exit).
#include "gc_internal.cuh"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <mutex>

namespace {
GcState g_state;
unsigned long long g_launches = 0;
thread_local char g_err[512] = "";
std::once_flag g_once;

void gc_atexit() { gc_shutdown(); }

void init_from_env() {
    const char* pm = getenv("GPUCELL_PERIODIC");
    if (pm && *pm) {
        int m = 0;
        for (const char* s = pm; *s; ++s) {
            if (*s == 'x' || *s == 'X') m |= 1;
            if (*s == 'y' || *s == 'Y') m |= 2;
            if (*s == 'z' || *s == 'Z') m |= 4;
        }
        if (strcmp(pm, "none") == 0 || strcmp(pm, "0") == 0) m = 0;
        g_state.periodic_mask = m;
    }
    const char* nz = getenv("GPUCELL_NOISE");
    if (nz && (strcmp(nz, "0") == 0 || strcmp(nz, "off") == 0)) g_state.noise_on = 0;
    const char* en = getenv("GPUCELL_ENGINE");
    if (en && strcmp(en, "fused") == 0) g_state.engine_mode = 1;
    atexit(gc_atexit);
}
}  // namespace

void gc_count_launch() { ++g_launches; }

// Adjusts the count by k (captured launches that did not run, replays of
// captured graphs that did).
void gc_add_launches(long long k) { g_launches += (unsigned long long)k; }

GcState& gc_state() {
    std::call_once(g_once, init_from_env);
    return g_state;
}

int gc_fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int gc_cuda_fail(cudaError_t e, const char* what) {
    return gc_fail(GC_ECUDA, "%s: CUDA error %d (%s)", what, (int)e, cudaGetErrorString(e));
}

void* gc_scratch(int slot, size_t bytes) {
    GcState& s = gc_state();
    if (bytes == 0) bytes = 16;
    if (s.scratch_bytes[slot] >= bytes) return s.scratch[slot];
    if (s.scratch[slot]) {
        cudaFree(s.scratch[slot]);
        s.scratch[slot] = nullptr;
        s.scratch_bytes[slot] = 0;
    }
    size_t want = bytes + bytes / 8;   // headroom so slowly growing sizes do not reallocate every call
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
        gc_fail(GC_ENOMEM, "scratch slot %d: cudaMalloc(%zu) failed: %s", slot, want, cudaGetErrorString(e));
        return nullptr;
    }
    s.scratch[slot] = p;
    s.scratch_bytes[slot] = want;
    return p;
}

unsigned* gc_flags_ptr() {
    GcState& s = gc_state();
    bool fresh = s.scratch[SCR_FLAGS] == nullptr;
    unsigned* f = (unsigned*)gc_scratch(SCR_FLAGS, sizeof(unsigned));
    if (f && fresh) cudaMemsetAsync(f, 0, sizeof(unsigned), s.stream);
    return f;
}

long long gc_noise_step() {
    GcState& s = gc_state();
    return s.step < 0 ? 0 : s.step;
}

// Builds the grid for the bbox (lo_x, hi_x, lo_y, hi_y, lo_z, hi_z), cube
// size rc and periodic mask.  Layout of bbox follows BBox in src/main.cuh:12.
int gc_build_grid(const float* bb, float rc, int mask, GcGrid* g) {
    memset(g, 0, sizeof(*g));
    g->pmask = mask;
    long long total = 1;
    for (int a = 0; a < 3; ++a) {
        float lo = bb[2 * a], hi = bb[2 * a + 1];
        if (!(hi > lo) || !isfinite(lo) || !isfinite(hi))
            return gc_fail(GC_EINVAL, "bbox axis %d is empty or not finite (%g, %g)", a, lo, hi);
        g->lo[a] = lo;
        g->hi[a] = hi;
        g->L[a] = hi - lo;
        g->halfL[a] = 0.5f * g->L[a];
        bool per = (mask >> a) & 1;
        double span = per ? (double)g->L[a] : (double)g->L[a] + 2.0 * rc;
        int n = (int)floor(span / ((double)rc * (1.0 + 1e-4)));
        if (n < 1) n = 1;
        if (per && n < 3)
            return gc_fail(GC_EINVAL, "periodic axis %d is %g long: at least 3 cut-off radii are needed", a, g->L[a]);
        g->n[a] = n;
        g->origin[a] = per ? lo : lo - rc;
        g->invw[a] = (float)(n / span);
        total *= n;
    }
    if (total > (1LL << 30)) return gc_fail(GC_EINVAL, "grid of %lld cubes is too large", total);
    g->ncells = (int)total;
    return GC_OK;
}

int gc_ensure_grid(const float* d_bbox) {
    GcState& s = gc_state();
    if (!s.consts_set) return gc_fail(GC_ESTATE, "PreConList before ConstsDataUp");
    if (s.grid_set && s.grid_bbox_ptr == d_bbox && s.grid_mask == s.periodic_mask && s.grid_rc == s.c.CutRadius)
        return GC_OK;
    if (!d_bbox) return gc_fail(GC_EINVAL, "bbox pointer is NULL");
    float bb[6];
    GC_CUDA(cudaMemcpyAsync(bb, d_bbox, sizeof(bb), cudaMemcpyDeviceToHost, s.stream), "read bbox");
    GC_CUDA(cudaStreamSynchronize(s.stream), "read bbox");
    GC_TRY(gc_build_grid(bb, s.c.CutRadius, s.periodic_mask, &s.grid));
    s.grid_set = true;
    s.grid_bbox_ptr = d_bbox;
    s.grid_mask = s.periodic_mask;
    s.grid_rc = s.c.CutRadius;
    return GC_OK;
}

int gc_params_from(const Structconst& c, int noise_on, GcParams* p) {
    if (!(c.CutRadius > 0.f) || !(c.Mass > 0.f) || !(c.TimeStep > 0.f))
        return gc_fail(GC_EINVAL, "CutRadius, Mass and TimeStep must be positive");
    memset(p, 0, sizeof(*p));
    p->nB2 = c.nBound2Start;
    p->nF = c.nFluidStart;
    p->nC = c.nCellStart;
    p->nT = c.nTotalPar;
    p->nCP = c.nCellPar;
    p->rc = c.CutRadius;
    p->inv_rc = 1.f / c.CutRadius;
    p->rc2 = c.CutRadius * c.CutRadius;
    p->mass = c.Mass;
    p->inv_mass = 1.f / c.Mass;
    p->c1sq = c.SoundSpeed1 * c.SoundSpeed1;
    p->c2sq = c.SoundSpeed2 * c.SoundSpeed2;
    p->rho0 = c.DenInit;
    p->lambda = c.VVsigma;
    p->dt = c.TimeStep;
    p->gx = c.ConstExtForce;
    p->kT = c.Temp;
    double rc = c.CutRadius;
    p->wnorm = (float)(21.0 / (2.0 * M_PI * rc * rc * rc));
    p->fnorm = (float)(210.0 / (M_PI * rc * rc * rc * rc * rc));
    p->w0 = p->wnorm;
    double eta = c.ShearVis, zeta = c.BulkVis;
    double A = 5.0 * eta / 3.0 - zeta, B = 5.0 * (zeta + eta / 3.0);
    p->visA = (float)A;
    p->visB = (float)B;
    p->sqrtA = (float)sqrt(A > 0 ? A : 0.0);
    p->sqrtAB = (float)sqrt(A + B > 0 ? A + B : 0.0);
    p->noise_pref = (noise_on && c.Temp > 0.f) ? (float)(2.0 * c.Temp / c.TimeStep) : 0.f;
    p->rep_r0 = (float)(rc / 3.0);
    p->rep_r0sq = p->rep_r0 * p->rep_r0;
    p->rep_D = p->c1sq;
    p->De = c.surEnergy;
    p->beta = c.scaFac;
    p->r0m = c.zeroLen;
    p->maxcut = c.MaxCut;
    p->maxcut2 = c.MaxCut * c.MaxCut;
    p->seed = (uint64_t)c.iSeed;
    p->noise_key = noise_key(p->seed, 0);
    return GC_OK;
}

int gc_make_params(GcParams* p, bool need_grid) {
    GcState& s = gc_state();
    if (!s.consts_set) return gc_fail(GC_ESTATE, "called before ConstsDataUp");
    if (need_grid && !s.grid_set) return gc_fail(GC_ESTATE, "neighbour sweep before PreConList built the grid");
    GC_TRY(gc_params_from(s.c, s.noise_on, p));
    p->noise_key = noise_key(p->seed, (uint64_t)gc_noise_step());
    if (s.grid_set) p->g = s.grid;
    return GC_OK;
}

extern "C" {

const char* gc_last_error(void) { return g_err; }

unsigned long long gc_launch_count(void) { return g_launches; }

int gc_version(void) { return 10000 * 0 + 100 * 3 + 0; }

int gc_set_periodic(int mask) {
    if (mask < 0 || mask > 7) return gc_fail(GC_EINVAL, "periodic mask %d outside 0..7", mask);
    gc_state().periodic_mask = mask;
    return GC_OK;
}

int gc_get_periodic(void) { return gc_state().periodic_mask; }

int gc_set_engine(int mode) {
    if (mode != 0 && mode != 1) return gc_fail(GC_EINVAL, "engine %d is neither 0 (entry-point kernels) nor 1 (fused)", mode);
    GcState& s = gc_state();
    if (s.engine_mode != mode) {
        gc_engine_reset();
        s.in_fused_step = false;
    }
    s.engine_mode = mode;
    return GC_OK;
}

int gc_get_engine(void) { return gc_state().engine_mode; }

int gc_set_noise(int on) {
    gc_state().noise_on = on ? 1 : 0;
    return GC_OK;
}

int gc_set_step(long long step) {
    GcState& s = gc_state();
    s.step = step;
    return GC_OK;
}

long long gc_get_step(void) { return gc_state().step; }

int gc_set_stream(void* stream) {
    gc_state().stream = (cudaStream_t)stream;
    return GC_OK;
}

int gc_device_status(unsigned* flags) {
    GcState& s = gc_state();
    if (!flags) return gc_fail(GC_EINVAL, "flags is NULL");
    *flags = 0;
    unsigned main_word = 0, noalloc_word = 0;
    if (s.scratch[SCR_FLAGS]) {
        GC_CUDA(cudaMemcpyAsync(&main_word, s.scratch[SCR_FLAGS], sizeof(unsigned), cudaMemcpyDeviceToHost, s.stream),
                "read flags");
        GC_CUDA(cudaMemsetAsync(s.scratch[SCR_FLAGS], 0, sizeof(unsigned), s.stream), "clear flags");
    }
    GC_TRY(gc_noalloc_status_take(&noalloc_word, s.stream));
    GC_CUDA(cudaStreamSynchronize(s.stream), "read flags");
    *flags = main_word | noalloc_word;
    return GC_OK;
}

int gc_scratch_bytes(unsigned long long* bytes) {
    if (!bytes) return gc_fail(GC_EINVAL, "bytes is NULL");
    GcState& s = gc_state();
    unsigned long long t = 0;
    for (int i = 0; i < SCR_COUNT_; ++i) t += s.scratch[i] ? (unsigned long long)s.scratch_bytes[i] : 0ull;
    *bytes = t;
    return GC_OK;
}

int gc_shutdown(void) {
    GcState& s = gc_state();
    gc_engine_reset();
    s.in_fused_step = false;
    for (int i = 0; i < SCR_COUNT_; ++i) {
        if (s.scratch[i]) cudaFree(s.scratch[i]);
        s.scratch[i] = nullptr;
        s.scratch_bytes[i] = 0;
    }
    s.grid_set = false;
    s.grid_bbox_ptr = nullptr;
    return GC_OK;
}

// K1 -- src/ParticleGPU.cuh:10, called once at src/Particle.cu:662 before
// the first neighbour build.  Validates and keeps the constants host-side;
// every later launch receives them in its parameter block.
int gc_cupar_ConstsDataUp(const Structconst* consts) {
    if (!consts) return gc_fail(GC_EINVAL, "ConstsDataUp: consts is NULL");
    const Structconst& c = *consts;
    if (!(c.nBound2Start <= c.nFluidStart && c.nFluidStart <= c.nCellStart && c.nCellStart <= c.nTotalPar))
        return gc_fail(GC_EINVAL, "ConstsDataUp: type boundaries out of order (%u %u %u %u)", c.nBound2Start,
                       c.nFluidStart, c.nCellStart, c.nTotalPar);
    if (c.nCellStart + c.nCellPar != c.nTotalPar)
        return gc_fail(GC_EINVAL, "ConstsDataUp: nCellStart + nCellPar != nTotalPar");
    if (!(c.CutRadius > 0.f) || !(c.Mass > 0.f) || !(c.TimeStep > 0.f))
        return gc_fail(GC_EINVAL, "ConstsDataUp: CutRadius, Mass and TimeStep must be positive");
    GcState& s = gc_state();
    s.c = c;
    s.consts_set = true;
    s.step = -1;
    // a new simulation: its buffers may reuse the addresses of an old one's
    s.grid_set = false;
    s.grid_bbox_ptr = nullptr;
    s.velhalf_ptr = nullptr;
    gc_engine_reset();
    s.ref = GcRefPtrs();
    s.plain_steps = 0;
    s.in_fused_step = false;
    if (!gc_flags_ptr()) return GC_ENOMEM;
    return GC_OK;
}

}  // extern "C"
