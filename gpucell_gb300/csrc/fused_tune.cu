// fused_tune.cu -- the autotuner of the fused step.
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
// Autotuner: times short runs of candidate settings on the handle's own
// state and keeps the fastest.  Every trial starts from the same saved state
// and step index with freshly built lists, and the handle returns to that
// state afterwards, so tuning does not change the trajectory that follows
// (beyond the summation order the chosen settings imply).  The search is
// coordinate-wise: skin (the cube size rc + skin of the list grid and the
// list length), then threads per block, then per-step compaction of the
// acting entries (list passes only), then captured steps.  Choices are
// cached per size class (ensemble or single system, particle count,
// density, membranes present, noise, pair tiles or lists) for the life of
// the process.
// ---------------------------------------------------------------------------
namespace {

struct TuneKey {
    int nsys_class, n_class, dens_class, cells, noise, lists;
    bool operator<(const TuneKey& o) const {
        return std::tie(nsys_class, n_class, dens_class, cells, noise, lists) <
               std::tie(o.nsys_class, o.n_class, o.dens_class, o.cells, o.noise, o.lists);
    }
};

std::mutex g_tune_mutex;
std::map<TuneKey, GcFusedOptions> g_tune_cache;

TuneKey tune_key(GcFused* f) {
    double vol = 0.0;
    for (const SysInfo& S : f->hsys) vol += (double)S.g.L[0] * S.g.L[1] * S.g.L[2];
    double dens = f->n / (vol > 0 ? vol : 1.0);
    TuneKey k;
    k.nsys_class = f->nsys > 1 ? (int)lround(log2((double)f->nsys)) + 1 : 0;
    k.n_class = (int)lround(4.0 * log2((double)f->n));
    k.dens_class = (int)lround(8.0 * log2(dens * f->p.rc * f->p.rc * f->p.rc + 1e-30));
    k.cells = f->ncell > 0;
    k.noise = f->p.noise_pref > 0.f;
    k.lists = f->lists;
    return k;
}

// Milliseconds per step of `steps` steps with the given settings, from the
// saved state (HUGE_VAL if the settings do not run, e.g. out of memory).
double trial(GcFused* f, const GcFusedOptions& o, int steps, int drive, cudaEvent_t e0, cudaEvent_t e1) {
    long long step0 = f->step, steps0 = f->steps, reb0 = f->rebuilds;
    if (gc_fused_set_options(f, &o) != GC_OK) return HUGE_VAL;
    if (restore_state(f, &f->tsnap) != GC_OK) return HUGE_VAL;
    f->step = step0;
    if (refresh(f) != GC_OK) return HUGE_VAL;
    if (f->graph && (sync_dstep(f) != GC_OK || prepare_graph(f, drive) != GC_OK)) return HUGE_VAL;
    if (cudaEventRecord(e0, f->st) != cudaSuccess) return HUGE_VAL;
    int rc = gc_fused_step(f, steps, drive);
    cudaEventRecord(e1, f->st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    f->step = step0;
    f->steps = steps0;
    f->rebuilds = reb0;
    return rc == GC_OK ? ms / steps : HUGE_VAL;
}

}  // namespace

extern "C" int gc_fused_autotune(GcFused* f, int trial_steps, int drive_on, int flags, GcFusedOptions* chosen,
                                 double* ms_per_step) {
    if (!f || !f->setup_done) return gc_fail(GC_ESTATE, "fused_autotune: call gc_fused_setup first");
    if (trial_steps < 1) trial_steps = 30;
    int drive = drive_on ? 1 : 0;
    TuneKey key = tune_key(f);
    GcFusedOptions best;
    GC_TRY(gc_fused_get_options(f, &best));
    best.list_capacity = 0;
    if (flags & GC_TUNE_CACHE) {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            GcFusedOptions o = it->second;
            int rc = gc_fused_set_options(f, &o);
            if (rc == GC_OK && chosen) *chosen = o;
            if (ms_per_step) *ms_per_step = 0.0;
            return rc;
        }
    }
    bool prof = f->profile;
    f->profile = false;
    GC_TRY(save_state(f, &f->tsnap));
    cudaEvent_t e0, e1;
    GC_CUDA(cudaEventCreate(&e0), "autotune: events");
    GC_CUDA(cudaEventCreate(&e1), "autotune: events");
    double best_ms = trial(f, best, trial_steps, drive, e0, e1);
    const float skins[] = {0.05f, 0.075f, 0.1f, 0.15f};
    const int blocks[] = {64, 128, 256};
    for (float s : skins) {
        GcFusedOptions o = best;
        o.skin = s;
        if (o.skin == best.skin) continue;
        double ms = trial(f, o, trial_steps, drive, e0, e1);
        if (ms < best_ms) { best_ms = ms; best = o; }
    }
    for (int b : blocks) {
        GcFusedOptions o = best;
        o.block = b;
        if (o.block == best.block) continue;
        double ms = trial(f, o, trial_steps, drive, e0, e1);
        if (ms < best_ms) { best_ms = ms; best = o; }
    }
    for (int c = 0; c < 2 && f->lists; ++c) {   // compaction is a setting of the list passes
        GcFusedOptions o = best;
        o.compact = c;
        if (o.compact == best.compact) continue;
        double ms = trial(f, o, trial_steps, drive, e0, e1);
        if (ms < best_ms) { best_ms = ms; best = o; }
    }
    for (int g = 0; g < 2; ++g) {
        GcFusedOptions o = best;
        o.graph = g;
        if (o.graph == best.graph) continue;
        double ms = trial(f, o, trial_steps, drive, e0, e1);
        if (ms < best_ms) { best_ms = ms; best = o; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    long long step0 = f->step;
    GC_TRY(gc_fused_set_options(f, &best));
    GC_TRY(restore_state(f, &f->tsnap));
    f->step = step0;
    GC_TRY(sync_dstep(f));
    GC_TRY(refresh(f));
    f->profile = prof;
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tune_cache[key] = best;
    }
    if (chosen) *chosen = best;
    if (ms_per_step) *ms_per_step = best_ms;
    if (!(best_ms < HUGE_VAL)) return gc_fail(GC_EDEVICE, "fused_autotune: no setting ran");
    return GC_OK;
}

