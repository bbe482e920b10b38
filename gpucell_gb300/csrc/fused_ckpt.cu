// fused_ckpt.cu -- checkpoint and restart of a fused handle.
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
// Checkpoint and restart.
//
// The file holds what the next steps depend on: the slot-ordered state (with
// the slot order itself, through the ids in the positions), the positions
// and cube keys the current neighbour lists were built from, the density
// and pressure, the step index that keys the noise, and the membrane
// reference geometry recorded at set-up.  A restore rebuilds the lists from
// those positions and keys without re-sorting, which reproduces them entry
// for entry, so that a restored run continues bit for bit as the original
// would have (host-driven steps; captured steps rebuild their lists when
// they are captured).  Layout, little-endian: a 128-byte header, one
// 16-byte record per system (particles, membrane vertices, seed), then the
// arrays in the order of ckpt_arrays.
// ---------------------------------------------------------------------------
namespace {

// slot of every id from the ids carried in the positions (restore)
__global__ void fk_slot_of(int n, const float4* __restrict__ pos, int* __restrict__ slot_of, unsigned* flags) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    unsigned id = fid(pos[q]);
    if (id >= (unsigned)n) {
        raise_flag(flags, GC_FLAG_BAD_INDEX);
        return;
    }
    slot_of[id] = q;
}

__global__ void fk_iota(int n, int* __restrict__ v) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) v[q] = q;
}

struct CkptHeader {
    char magic[8];
    uint32_t version, nsys;
    uint64_t n, ncp, ncell, ntri, nedge;
    int64_t step;
    float skin_rel;
    int32_t K;
    uint32_t has_sys, has_cells;
    uint8_t reserved[128 - 8 - 8 - 40 - 8 - 4 - 4 - 8];
};
static_assert(sizeof(CkptHeader) == 128, "checkpoint header is 128 bytes");

struct CkptSys {
    uint32_t n, ncp;
    uint64_t seed;
};

struct CkptArray {
    void* dev;
    size_t bytes;
};

std::vector<CkptArray> ckpt_arrays(GcFused* f) {
    size_t n = f->n;
    std::vector<CkptArray> v = {
        {f->a.pos, n * 16}, {f->a.plo, n * 16}, {f->a.vel, n * 16}, {f->a.vpred, n * 16}, {f->a.vh, n * 16}, {f->a.force, n * 16},
        {f->a.nthro, n * 16}, {f->refpos, n * 16}, {f->keys, n * 4}, {f->dp, n * 8}};
    if (f->a.sys) v.push_back({f->a.sys, n * 4});
    if (f->ncell > 0) {
        size_t nt = f->ntri, nc = f->ncell, ne = f->nedge;
        v.push_back({f->reftarea, nt * 4});
        v.push_back({f->crefarea, nc * 8});
        v.push_back({f->crefvol, nc * 8});
        for (float* q : {f->l0, f->lmax, f->perlen, f->hpow, f->hbend, f->refang}) v.push_back({q, ne * 4});
    }
    return v;
}

void ckpt_header(GcFused* f, CkptHeader* h) {
    memset(h, 0, sizeof(*h));
    memcpy(h->magic, "GCFCKPT2", 8);
    h->version = 2;
    h->nsys = f->nsys;
    h->n = f->n;
    h->ncp = f->ncp;
    h->ncell = f->ncell;
    h->ntri = f->ntri;
    h->nedge = f->nedge;
    h->step = f->step;
    h->skin_rel = f->skin_rel;
    h->K = f->K;
    h->has_sys = f->a.sys ? 1 : 0;
    h->has_cells = f->ncell > 0 ? 1 : 0;
}

// The lists exactly as the last rebuild made them: the cube starts from the
// saved (sorted) keys and the scan over the saved build positions.
int rebuild_from_ref(GcFused* f) {
    const int n = f->n, nb = gc_blocks(n, f->block);
    cudaStream_t st = f->st;
    fk_iota<<<nb, f->block, 0, st>>>(n, f->vals);
    GC_CHECK_LAUNCH("restore: identity");
    GC_TRY(gc_counting_sort_bufs(n, f->K, f->keys, f->vals, f->sb, f->flags, st));
    if (!f->lists) {
        GC_TRY(wall_lists(f, st, f->refpos, true));
        GC_CUDA(cudaMemsetAsync(f->oflag, 0, sizeof(unsigned), st), "restore: flags");
        GC_TRY(tiles_build(f, st, f->refpos, true));
        if (f->h->oflag & GC_FLAG_TILE_FULL)
            return gc_fail(GC_EDEVICE, "restore: a cube holds more particles than the pair tiles take; restore into "
                                       "a handle with per-particle lists (GcFusedOptions.tiles = 0)");
        return build_morse_lists_from_ref(f, st);
    }
    float cut = f->p.rc + f->skin;
    for (int attempt = 0; attempt < 4; ++attempt) {
        GC_CUDA(cudaMemsetAsync(f->oflag, 0, sizeof(unsigned), st), "restore: flags");
        GC_CUDA(cudaMemsetAsync(f->need, 0, sizeof(int), st), "restore: flags");
        fk_build_list<<<nb, f->block, 0, st>>>(n, f->dsys, f->a.sys, f->refpos, f->sb.cnt, f->nbr, f->cnt, f->cap,
                                              cut * cut, f->oflag, f->need, 0);
        GC_CHECK_LAUNCH("restore: build lists");
        GC_CUDA(cudaMemcpyAsync(&f->h->oflag, f->oflag, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "restore");
        GC_CUDA(cudaMemcpyAsync(&f->h->need, f->need, sizeof(int), cudaMemcpyDeviceToHost, st), "restore");
        GC_CUDA(cudaStreamSynchronize(st), "restore");
        if (!(f->h->oflag & GC_FLAG_CELL_OVERFLOW)) return build_morse_lists_from_ref(f, st);
        GC_TRY(alloc_list(f, grown_capacity(f, 2 * f->cap)));
    }
    return gc_fail(GC_EDEVICE, "restore: neighbour lists overflow %d entries", f->cap);
}

}  // namespace

extern "C" int gc_fused_checkpoint(GcFused* f, const char* path) {
    if (!f || !path) return gc_fail(GC_EINVAL, "checkpoint: NULL argument");
    if (!f->setup_done) return gc_fail(GC_ESTATE, "checkpoint: call gc_fused_setup first");
    FILE* fp = fopen(path, "wb");
    if (!fp) return gc_fail(GC_EINVAL, "checkpoint: cannot open %s for writing", path);
    CkptHeader h;
    ckpt_header(f, &h);
    std::vector<CkptSys> sys(f->nsys);
    for (int s = 0; s < f->nsys; ++s) {
        sys[s].n = f->hsys[s].end - f->hsys[s].id0;
        sys[s].ncp = f->hsys[s].end - f->hsys[s].cs;
        sys[s].seed = f->hsys[s].seed;
    }
    bool ok = fwrite(&h, sizeof(h), 1, fp) == 1 && fwrite(sys.data(), sizeof(CkptSys), sys.size(), fp) == sys.size();
    std::vector<char> buf;
    int rc = GC_OK;
    for (const CkptArray& a : ckpt_arrays(f)) {
        if (!ok) break;
        buf.resize(a.bytes);
        cudaError_t e = cudaMemcpyAsync(buf.data(), a.dev, a.bytes, cudaMemcpyDeviceToHost, f->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(f->st);
        if (e != cudaSuccess) {
            rc = gc_cuda_fail(e, "checkpoint: read state");
            break;
        }
        ok = fwrite(buf.data(), 1, a.bytes, fp) == a.bytes;
    }
    if (fclose(fp) != 0) ok = false;
    if (rc != GC_OK) return rc;
    if (!ok) return gc_fail(GC_EINVAL, "checkpoint: write to %s failed", path);
    return GC_OK;
}

extern "C" int gc_fused_restore(GcFused* f, const char* path) {
    if (!f || !path) return gc_fail(GC_EINVAL, "restore: NULL argument");
    if (!f->setup_done) return gc_fail(GC_ESTATE, "restore: set the handle up as for the original run first");
    FILE* fp = fopen(path, "rb");
    if (!fp) return gc_fail(GC_EINVAL, "restore: cannot open %s", path);
    CkptHeader h;
    int rc = GC_OK;
    std::vector<CkptSys> sys;
    if (fread(&h, sizeof(h), 1, fp) != 1 || memcmp(h.magic, "GCFCKPT2", 8) != 0 || h.version != 2) {
        rc = gc_fail(GC_EINVAL, "restore: %s is not a checkpoint of this library", path);
    } else if (h.nsys != (uint32_t)f->nsys || h.n != (uint64_t)f->n || h.ncp != (uint64_t)f->ncp ||
               h.ncell != (uint64_t)f->ncell || h.ntri != (uint64_t)f->ntri || h.nedge != (uint64_t)f->nedge ||
               h.has_sys != (f->a.sys ? 1u : 0u)) {
        rc = gc_fail(GC_EINVAL, "restore: the checkpoint holds another configuration (%llu particles in %u systems, "
                                "%llu cells; this handle: %d in %d, %d)",
                     (unsigned long long)h.n, h.nsys, (unsigned long long)h.ncell, f->n, f->nsys, f->ncell);
    } else {
        sys.resize(h.nsys);
        if (fread(sys.data(), sizeof(CkptSys), sys.size(), fp) != sys.size()) {
            rc = gc_fail(GC_EINVAL, "restore: %s is truncated", path);
        } else {
            for (int s = 0; s < f->nsys && rc == GC_OK; ++s)
                if (sys[s].n != f->hsys[s].end - f->hsys[s].id0 || sys[s].ncp != f->hsys[s].end - f->hsys[s].cs ||
                    sys[s].seed != f->hsys[s].seed)
                    rc = gc_fail(GC_EINVAL, "restore: system %d differs from the checkpoint's", s);
        }
    }
    if (rc == GC_OK) {   // the file holds exactly the arrays of this configuration
        uint64_t want = sizeof(h) + sizeof(CkptSys) * (uint64_t)h.nsys;
        for (const CkptArray& a : ckpt_arrays(f)) want += a.bytes;
        const long here = ftell(fp);
        const bool sized = here >= 0 && fseek(fp, 0, SEEK_END) == 0;
        const long end = sized ? ftell(fp) : -1;
        if (!sized || end < 0 || fseek(fp, here, SEEK_SET) != 0)
            rc = gc_fail(GC_EINVAL, "restore: cannot read %s", path);
        else if ((uint64_t)end != want)
            rc = gc_fail(GC_EINVAL, "restore: %s holds %ld bytes, a checkpoint of this configuration %llu", path,
                         end, (unsigned long long)want);
    }
    if (rc == GC_OK && h.skin_rel != f->skin_rel) {   // the lists were built at the checkpoint's skin
        const float skin_rel = f->skin_rel;
        f->skin_rel = h.skin_rel;
        f->skin = f->skin_rel * f->p.rc;
        rc = build_grids(f);
        if (rc == GC_OK && h.K != f->K)
            rc = gc_fail(GC_EINVAL, "restore: the cube grids differ from the checkpoint's");
        if (rc != GC_OK) {   // refused: back to the handle's own skin and grids
            f->skin_rel = skin_rel;
            f->skin = f->skin_rel * f->p.rc;
            const int back = build_grids(f);
            if (back != GC_OK) rc = back;
        }
    } else if (rc == GC_OK && h.K != f->K) {
        rc = gc_fail(GC_EINVAL, "restore: the cube grids differ from the checkpoint's");
    }
    std::vector<char> buf;
    for (const CkptArray& a : ckpt_arrays(f)) {
        if (rc != GC_OK) break;
        buf.resize(a.bytes);
        if (fread(buf.data(), 1, a.bytes, fp) != a.bytes) {   // a read error: the length was checked
            rc = gc_fail(GC_EINVAL, "restore: reading %s failed; the handle's state is undefined", path);
            break;
        }
        cudaError_t e = cudaMemcpyAsync(a.dev, buf.data(), a.bytes, cudaMemcpyHostToDevice, f->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(f->st);   // the host buffer is reused
        if (e != cudaSuccess) rc = gc_cuda_fail(e, "restore: write state");
    }
    fclose(fp);
    if (rc != GC_OK) return rc;
    const int n = f->n;
    cudaStream_t st = f->st;
    fk_slot_of<<<gc_blocks(n, 256), 256, 0, st>>>(n, f->a.pos, f->slot_of, f->flags);
    GC_CHECK_LAUNCH("restore: slots");
    if (f->ncell > 0) {
        fk_gather_mpos<<<gc_blocks(f->ncp, 256), 256, 0, st>>>(f->ncp, f->dsys, f->msys, f->slot_of, f->a.pos,
                                                              f->a.nthro, f->a.plo, f->mpos, f->mplo, f->mnthro);
        GC_CHECK_LAUNCH("restore: membrane positions");
    }
    GC_TRY(rebuild_from_ref(f));
    f->step = h.step;
    GC_TRY(sync_dstep(f));
    drop_graphs(f);
    GcParams p = f->p;
    GC_TRY(launch_membranes(f, st, p));   // membrane outputs of the restored state
    GC_CUDA(cudaStreamSynchronize(st), "restore");
    return GC_OK;
}

