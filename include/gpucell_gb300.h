/*
 * gpucell_gb300.h -- C ABI of libgpucell_gb300.so.
 *
 * One extern "C" function per entry point of GPUCell's GPU boundary, with
 * the reference's argument order and meaning, plain pointers only:
 *   float3 / tfloat3 arrays  -> float*, 3 floats per element
 *   float4 arrays            -> float*, 4 floats per element
 *   int2 / int3 / int6       -> int*,   2 / 3 / 6 ints per element
 * Every function returns GC_OK (0) or a negative GC_E* status; the text of
 * the last error is available from gc_last_error().  Pointers named d_*
 * are device pointers owned by the caller; h_* are host pointers that the
 * reference passes but never reads back (accepted and ignored).  Work is
 * enqueued on the library's stream (gc_set_stream; the legacy default
 * stream unless changed), and no function synchronises the host except
 * where stated.
 *
 * The C++ symbols cupar::* / cudiv::* (include/gpucell/cupar.h) forward to
 * these and turn a failure into the reference's print-and-exit(1).
 *
 * Particle arrays are in "slot" order: the order of the latest neighbour
 * sort.  d_sortpart[slot] is the original id of the particle in that slot
 * and d_curpos[id] its slot (src/Particle.cu:734, :1322).  Original ids are
 * grouped by type as described in include/gpucell/TypesDef.h.
 */
#ifndef GPUCELL_GB300_H
#define GPUCELL_GB300_H

#include "gpucell/TypesDef.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GC_OK           0
#define GC_EINVAL      -1   /* bad argument (size, pointer, state) */
#define GC_ECUDA       -2   /* a CUDA runtime call or launch failed */
#define GC_ESTATE      -3   /* call out of order (e.g. before ConstsDataUp) */
#define GC_ENOMEM      -4   /* scratch allocation failed */
#define GC_EDEVICE     -5   /* a device-side check raised its flag */

/* device status flags reported by gc_device_status() */
#define GC_FLAG_NONFINITE     1u   /* a NaN/Inf position or force was seen */
#define GC_FLAG_BAD_INDEX     2u   /* a topology index pointed outside its array */
#define GC_FLAG_CELL_OVERFLOW 4u   /* a grid cell held more particles than a sweep stages */
#define GC_FLAG_STRETCH       8u   /* a membrane edge reached its maximum length */
#define GC_FLAG_TILE_FULL    16u   /* a cube held more particles than the pair tiles take (the handle
                                      turns to per-particle lists) */

/* ---- library controls (no counterpart in the reference) ---------------- */

/* Text of the most recent error of this thread ("" if none). */
const char* gc_last_error(void);
/* Library version as 10000*major + 100*minor + patch. */
int gc_version(void);
/* Periodic axes as a bit mask (1 = x, 2 = y, 4 = z).  The reference grid
 * pads y and z by one cube and leaves x unpadded (src/Particle.cu:551-556),
 * i.e. x periodic with walls in y and z: that is the default (mask 1).
 * The environment variable GPUCELL_PERIODIC (e.g. "xz") sets the initial
 * value.  Takes effect at the next gc_cudiv_PreConList. */
int gc_set_periodic(int mask);
int gc_get_periodic(void);
/* How the boundary entry points compute a step: 0 (default) runs one kernel
 * per entry point on the caller's buffers; 1 runs, from the second step
 * after ConstsDataUp on, the whole step as the fused step of gc_fused_*
 * inside SetFluidExtForce (which carries DriveOn), writes the state the host
 * reads back into the caller's buffers at the end of the step, and turns
 * the other calls of the step into no-ops.  The first step runs on the
 * entry-point kernels and records the caller's buffers.  The caller must not
 * change its buffers between steps (GPUCell's host frame only reads them).
 * GPUCELL_ENGINE=fused selects 1 at load time. */
int gc_set_engine(int mode);
int gc_get_engine(void);
/* Thermal pair noise on (1, default) or off (0). GPUCELL_NOISE=0 turns it
 * off at load time. */
int gc_set_noise(int on);
/* Step index that keys the pair noise.  The cupar:: path counts steps
 * itself (one per gc_cupar_UpdateFluidCoor, starting at 0); this sets the
 * counter to `step` for the next force evaluation. */
int gc_set_step(long long step);
long long gc_get_step(void);
/* Stream used by every gc_* launch (a cudaStream_t; NULL = legacy default). */
int gc_set_stream(void* stream);
/* Reads and clears the device-side status flags (GC_FLAG_*), including those
 * raised by gc_cudiv_Sort_noalloc on the current device.  Synchronises the
 * library's stream. */
int gc_device_status(unsigned* flags);
/* Bytes of device scratch the library holds now (what gc_shutdown frees;
 * the fixed array of gc_cudiv_Sort_noalloc is not counted). */
int gc_scratch_bytes(unsigned long long* bytes);
/* Number of kernels this library has launched since it was loaded. */
unsigned long long gc_launch_count(void);
/* Frees every scratch buffer the library allocated.  Safe to call twice;
 * also registered with atexit(). */
int gc_shutdown(void);

/* ---- cupar: particle physics (src/ParticleGPU.cuh:10-35) ---------------- */

/* src/ParticleGPU.cuh:10, called at src/Particle.cu:662 */
int gc_cupar_ConstsDataUp(const Structconst* consts);
/* src/ParticleGPU.cuh:11, src/Particle.cu:1333 */
int gc_cupar_UpdateFluidCoor(int n, int* d_sortpart, float* d_totalforce, float* d_totalcoor, float* d_velrhop);
/* src/ParticleGPU.cuh:12, src/Particle.cu:1338 */
int gc_cupar_AppFluidPeriodicBC(int n, int* d_sortpart, float* d_totalcoor, int* d_nthrobound, float* d_bboxsdpd);
/* src/ParticleGPU.cuh:13, src/Particle.cu:1343 */
int gc_cupar_CalFluidDen(int n, float* d_totalcoor, float* d_velrhop, int* d_cc, int* d_ncube, float* d_outerregion, int* d_sortpart, int* d_beginendcube);
/* src/ParticleGPU.cuh:14, src/Particle.cu:1348 */
int gc_cupar_PredictFluidVel(int n, int* d_sortpart, float* d_velrhop, float* d_velhalf, float* d_totalforce);
/* src/ParticleGPU.cuh:15, src/Particle.cu:1353 */
int gc_cupar_CalBound2Vel(int n, float* d_totalcoor, float* d_velrhop, int* d_cc, int* d_ncube, float* d_outerregion, int* d_sortpart, int* d_beginendcube);
/* src/ParticleGPU.cuh:16, src/Particle.cu:1358 */
int gc_cupar_EOS(int n, int* d_sortpart, float* d_velrhop, float* d_press);
/* src/ParticleGPU.cuh:17, src/Particle.cu:1363 */
int gc_cupar_CalFluidSDPDForce(int n, float* h_sdpdforce, float* d_totalcoor, float* d_velrhop, int* d_cc, int* d_ncube, int* d_sortpart, float* d_outerregion, int* d_beginendcube, float* d_totalforce, float* d_press);
/* src/ParticleGPU.cuh:18, src/Particle.cu:1368 */
int gc_cupar_CalFluidRepForce(int n, float* d_totalcoor, int* d_cc, int* d_ncube, int* d_sortpart, float* d_outerregion, int* d_beginendcube, float* d_totalforce);
/* src/ParticleGPU.cuh:19, src/Particle.cu:1373 */
int gc_cupar_SetFluidExtForce(int driveon, int n, int* d_sortpart, float* d_totalforce);
/* src/ParticleGPU.cuh:21, src/Particle.cu:1379 */
int gc_cupar_CorrectFliudVel(int n, int* d_sortpart, float* d_totalforce, float* d_velhalf, float* d_velrhop, float* d_totalcoor, int* d_cc, int* d_ncube, float* d_outerregion, int* d_beginendcube);
/* src/ParticleGPU.cuh:25-26, src/Particle.cu:476 (stepcount -1: records the
 * reference geometry) and :1322 (every step) */
int gc_cupar_CalGeoPara(long stepcount, int ntri, int ncell, float* d_bbox, int* d_curpos, int* d_tri, int* d_beginendtri, int* d_nthrobound, float* d_totalcoor, float* d_trinordir, float* d_triarea,
    float* d_reftriarea, float* d_tricenter, float* d_refarea_para, float* d_refvol_para, float* d_area_para, float* d_vol_para, float* d_area, float* d_vol, float* d_pararea);
/* src/ParticleGPU.cuh:28-29, src/Particle.cu:479 */
int gc_cupar_SetMechPara(int ncell, int nedge, int* d_edge, int* d_curpos, float* d_refedgelen, float* d_maxrefedgelen, float* d_bendmodpara, float* d_shearmodpara, float* d_hbending,
    float* d_powerindex, float* d_perlenWLC, float* d_hpow, float* d_reftriangle, float* d_trinordir, float* d_tricenter, float* d_coor);
/* src/ParticleGPU.cuh:30-33, src/Particle.cu:1385 */
int gc_cupar_CalCellDefForce(int ncell, unsigned nedge, unsigned ntri, unsigned ntotalpar, unsigned ncellpar, float* d_bbox, int* d_edge, int* d_tri, float* d_coor, float* h_defforce, float* d_defforce, int* d_nthrobound,
    float* d_maxrefedgelen, float* d_powerindex, float* d_perlenWLC, float* d_hpow, float* d_trinordir, float* d_tricenter,
    float* d_reftriangle, float* d_hbending, float* d_triarea, float* d_reftriarea, float* d_hlarea_para, float* d_hgarea_para, float* d_area_para,
    float* d_refarea_para, float* d_hvol_para, float* d_vol_para, float* d_refvol_para, float* d_totalforce, int* d_sortpart, int* d_curpos);
/* src/ParticleGPU.cuh:34-35, src/Particle.cu:1390 */
int gc_cupar_CalCellAggForce(unsigned ncell, unsigned n, unsigned ncellpar, float* d_totalcoor, float* d_aggforce, int* d_cc, int* d_ncube, int* d_sortpart,
    int* d_celltab, float* d_outerregion, int* d_beginendcube, float* d_totalforce, float* d_pararea);

/* ---- cudiv: neighbour grid (src/ConfigDomain.cuh:11-17) ----------------- */

/* src/ConfigDomain.cuh:11, src/Particle.cu:668.  Reads d_bboxsph to the
 * host (one synchronous 24-byte copy) the first time it sees that pointer. */
int gc_cudiv_PreConList(int n, int cutradius, float* d_totalcoor, float* d_bboxsph, float* d_invwid, int* d_ncube, int* d_cc, int* d_cubepart, int* d_sortpart, int* d_oldpos);
/* src/ConfigDomain.cuh:12, src/Particle.cu:669.  Stable sort of n (key,
 * value) pairs by key.  Keys must lie in [0, K) where K is the cube count of
 * the latest PreConList; without one, K is found on the device (one
 * synchronous 4-byte copy). */
int gc_cudiv_Sort(int n, int* keys, int* values);
/* No counterpart in the reference: the sort of gc_cudiv_Sort (same stable
 * order, same key rule) for callers that cannot let the library allocate
 * device memory -- a host program that reserves the device memory it will
 * use up front, a process sharing the GPU under a fixed memory cap, or a loop
 * that must not stall on the device synchronisation of cudaFree.  Its
 * temporaries live in one fixed array of about 5.2 MB; it calls no
 * cudaMalloc or cudaFree.  The array belongs to the library's code module,
 * which CUDA loads lazily by default: the array is committed on a device
 * when the first call there runs, and held until the process exits.  A
 * caller that budgets its memory should make one small call on each device
 * during set-up, before it reserves its own memory and before any stream
 * capture (that first call also looks up the array's device address).
 * Limits: n <= GC_NOALLOC_SORT_MAX_N elements and at most
 * GC_NOALLOC_SORT_MAX_KEYS keys (the grid's cube count, or the largest key
 * + 1 without a grid); larger inputs return GC_EINVAL.  A key outside
 * [0, K) is clamped into range, as gc_cudiv_Sort does, and raises
 * GC_FLAG_BAD_INDEX, which gc_device_status reports.  All calls share the
 * array: calls that may overlap on the GPU (different streams, or different
 * host threads) race and must be serialised by the caller. */
#define GC_NOALLOC_SORT_MAX_N    262144
#define GC_NOALLOC_SORT_MAX_KEYS 262144
int gc_cudiv_Sort_noalloc(int n, int* keys, int* values);
/* src/ConfigDomain.cuh:13, src/Particle.cu:672 */
int gc_cudiv_CalBeginEndCube(int n, int sizecube, int* d_cubepart, int* d_beginendcube);
/* src/ConfigDomain.cuh:14, src/Particle.cu:677 */
int gc_cudiv_SortBasicArrays(int n, int* d_sortpart, int* d_oldpos, float* d_totalcoor, int* d_cc, float* d_velrhop, float* d_velhalf, float* d_totalforce, float* d_press);
/* src/ConfigDomain.cuh:15, src/Particle.cu:675 */
int gc_cudiv_SortArraysWithCells(int n, int* d_sortpart, int* d_oldpos, int* d_curpos, float* d_totalcoor, int* d_cc, float* d_velrhop, float* d_velhalf, float* d_totalforce, float* d_press, int* d_nthrobound);
/* src/ConfigDomain.cuh:17 (never called by the reference): prints the
 * first min(n, 16) slots to stdout.  Synchronises. */
int gc_cudiv_Printf(int n, int* d_curpos, int* d_sortpart, float* d_totalcoor);

/* ---- fused timestep (no counterpart in the reference) -------------------
 *
 * The same method and step order as one Particle::UpdatePar sequence
 * (src/Particle.cu:1310-1329), on state the library owns: Verlet neighbour
 * lists with a skin (re-sorted and rebuilt only when a particle has moved
 * more than skin/2), fused passes, FP64 per-cell area/volume sums.  The
 * caller loads the state of GPUCell's host frame once (original particle
 * order, reference layouts), steps, and stores it back whenever it wants to
 * output; pointers are host pointers unless the *_device flag is set.
 * Noise steps are numbered from 0 after gc_fused_setup, as the boundary
 * entry points number them after ConstsDataUp. */
typedef struct GcFused GcFused;
typedef struct {
    float skin;           /* Verlet skin in units of CutRadius (0: 0.1) */
    int block;            /* threads per block of the particle kernels: 64, 128 or 256 (0: 128) */
    int list_capacity;    /* initial neighbour-list capacity per particle (0: from the density) */
    int compact;          /* 1: the density pass marks the list entries that act this step, and the force
                             pass iterates only those */
    int graph;            /* 1: each step runs as one captured CUDA graph; the list rebuild is a conditional
                             node decided on the device, and gc_fused_step synchronises once per call */
    int tiles;            /* 0 (default): per-particle Verlet lists, every pair evaluated from both ends;
                             1: pair tiles -- particles sorted by cubes at least rc + skin wide, one list
                             per pair of neighbouring cubes (each particle pair once), the density and force
                             passes evaluate every pair once and give each side its share.  A handle with
                             tiles turns to lists by itself when a cube holds more than 96 particles or a
                             periodic axis has fewer than three cubes */
    int fp32_positions;   /* 1: positions accumulate in plain FP32 (the double-float update off), for
                             comparing precisions */
    int half_velocity;    /* 1: the list force pass gathers neighbour velocities packed to FP16 (8 B instead
                             of 16), an experiment */
} GcFusedOptions;
/* bbox6 (host) as src/main.cuh:12; periodic_mask as gc_set_periodic. */
int gc_fused_create(const Structconst* consts, const float* bbox6, int periodic_mask, int noise_on,
                    const GcFusedOptions* opt, GcFused** out);
/* Membrane topology and per-edge / per-triangle moduli (host arrays, the
 * reference's 1-based conventions, src/Particle.cu:174-303, :405-425). */
int gc_fused_set_cells(GcFused* f, int ncell, int ntri, int nedge, const int* tri, const int* edge,
                       const int* betri, const int* celltab, const float* shearmod, const float* bendmod,
                       const float* hlarea, const float* hgarea, const float* hvol);
/* State in original order: positions, velocities, VelHalf (prescribed wall
 * velocity of Bound2 particles), forces, crossing counts (NULL = zero).
 * Before gc_fused_setup this is the initial state; afterwards it replaces
 * the state in place (NULL = keep) and the neighbour lists are kept unless
 * the displacement check of the next step asks for a rebuild. */
int gc_fused_load(GcFused* f, const float* pos, const float* vel, const float* velhalf, const float* force,
                  const int* nthro, int from_device);
/* Reference geometry and membrane mechanics (CalGeoPara with StepCount -1
 * and SetMechPara, src/Particle.cu:476-480) and the first neighbour lists. */
int gc_fused_setup(GcFused* f);
/* nsteps timesteps; drive_on as Particle::DrivePar (src/Particle.cu:1302). */
int gc_fused_step(GcFused* f, int nsteps, int drive_on);
/* State in original order (NULL pointers are skipped). */
int gc_fused_store(GcFused* f, float* pos, float* vel, float* rho, float* press, float* force, float* velhalf,
                   int* nthro, int to_device);
/* Membrane outputs of the latest step, in the reference's orders. */
int gc_fused_store_cells(GcFused* f, float* area, float* vol, float* defforce, float* aggforce, float* trinordir,
                         float* tricenter, float* pararea, int to_device);
/* One timestep with its outputs in host memory: the same results as
 * gc_fused_step(f, 1, drive_on) followed by gc_fused_store(..., 0) and
 * gc_fused_store_cells(..., 0) (NULL pointers are skipped).  What is final
 * early in the step is copied while the step still runs: positions, VelHalf
 * and crossing counts after the integration, density and pressure after the
 * density pass, the membrane outputs after the membrane passes; velocities
 * and forces at the end.  Host pointers (pinned memory lets the copies run
 * beside the kernels); returns when every copy is done.  In captured steps
 * (GcFusedOptions.graph) the step runs first and the stores after it. */
int gc_fused_step_store(GcFused* f, int drive_on, float* pos, float* vel, float* rho, float* press, float* force,
                        float* velhalf, int* nthro, float* area, float* vol, float* defforce, float* aggforce,
                        float* trinordir, float* tricenter, float* pararea);
/* Per-cell area and volume as summed (FP64), host pointers. */
int gc_fused_cell_sums(GcFused* f, double* area, double* vol);
/* List rebuilds, steps taken, list capacity, mean and max list length. */
int gc_fused_stats(GcFused* f, long long* rebuilds, long long* steps, int* list_capacity, double* mean_neighbors,
                   int* max_neighbors);
/* Reads and clears the handle's device status flags (GC_FLAG_*). */
int gc_fused_flags(GcFused* f, unsigned* flags);
/* Times the density and force kernels of every following step with CUDA
 * events on the library's stream (1) or stops doing so (0). */
int gc_fused_profile(GcFused* f, int enable);
/* Total milliseconds of the density and force kernels and the number of
 * steps timed since gc_fused_profile(f, 1) or the previous read.
 * Synchronises. */
int gc_fused_profile_read(GcFused* f, double* density_ms, double* force_ms, long long* steps);
/* Current settings (list_capacity = the current capacity). */
int gc_fused_get_options(GcFused* f, GcFusedOptions* opt);
/* Changes the settings of a handle, also after set-up (the lists are rebuilt
 * when the skin, compaction or capacity change; the state is kept). */
int gc_fused_set_options(GcFused* f, const GcFusedOptions* opt);
/* Autotuner: times trial_steps steps (0: 30) of candidate settings -- skin
 * 0.05/0.075/0.1/0.15 rc (the cube size of the list grid), 64/128/256
 * threads per block, compaction on/off, captured steps on/off, searched one
 * after the other -- each from the handle's current state, keeps the fastest
 * and returns the handle to that state.  With GC_TUNE_CACHE a choice cached
 * for the same size class (ensemble size, particle count and density to a
 * quarter octave, membranes, noise) is applied without trials.  Needs
 * gc_fused_setup; synchronises. */
#define GC_TUNE_CACHE 1
int gc_fused_autotune(GcFused* f, int trial_steps, int drive_on, int flags, GcFusedOptions* chosen,
                      double* ms_per_step);
/* Checkpoint and restart (no counterpart in the reference): writes the
 * complete dynamic state to a binary file -- slot-ordered state, the
 * positions and cube keys the neighbour lists were built from, density and
 * pressure, the step index that keys the noise, the membrane reference
 * geometry.  gc_fused_restore reads it into a handle created and set up as
 * for the original run (same systems, constants, boxes and membranes) and
 * rebuilds the lists exactly, so that host-driven steps continue bit for bit
 * as the original run would have.  A file that is not a checkpoint, holds
 * another configuration or has another length is refused (GC_EINVAL) before
 * the handle changes; a read or device error after that leaves the handle's
 * state undefined until the next successful restore or gc_fused_load.
 * Synchronise. */
int gc_fused_checkpoint(GcFused* f, const char* path);
int gc_fused_restore(GcFused* f, const char* path);
int gc_fused_destroy(GcFused* f);

/* ---- ensembles of independent simulations (no counterpart) --------------
 *
 * Many independent systems of uneven size stepped by the same launches: the
 * ids of system s follow those of systems 0..s-1, each system keeps its own
 * box, grid, body force (ConstExtForce) and noise seed (iSeed, keyed by the
 * system's own ids, so a system draws the same noise as when run alone);
 * every other Structconst field must be the same for all systems.  A handle
 * from gc_ensemble_create takes the gc_fused_* calls too: gc_fused_load,
 * _store, _store_cells and _cell_sums then cover all systems, concatenated in
 * system order; gc_ensemble_* cover one system, in that system's own ids. */
typedef struct {
    Structconst consts;   /* the system's counts and constants */
    float bbox[6];        /* as src/main.cuh:12 */
    int periodic_mask;    /* as gc_set_periodic */
    int reserved;
} GcSystemDesc;
int gc_ensemble_create(int nsys, const GcSystemDesc* systems, int noise_on, const GcFusedOptions* opt,
                       GcFused** out);
int gc_ensemble_size(GcFused* f, int* nsys, long long* nparticles);
int gc_ensemble_set_cells(GcFused* f, int sys, int ncell, int ntri, int nedge, const int* tri, const int* edge,
                          const int* betri, const int* celltab, const float* shearmod, const float* bendmod,
                          const float* hlarea, const float* hgarea, const float* hvol);
int gc_ensemble_load(GcFused* f, int sys, const float* pos, const float* vel, const float* velhalf,
                     const float* force, const int* nthro, int from_device);
int gc_ensemble_store(GcFused* f, int sys, float* pos, float* vel, float* rho, float* press, float* force,
                      float* velhalf, int* nthro, int to_device);
int gc_ensemble_store_cells(GcFused* f, int sys, float* area, float* vol, float* defforce, float* aggforce,
                            float* trinordir, float* tricenter, float* pararea, int to_device);
int gc_ensemble_cell_sums(GcFused* f, int sys, double* area, double* vol);

/* ---- output files (GPUCell's OutputPar, src/Particle.cu:681-1300) --------
 *
 * One output step in the reference's text formats: FluidCoor/<step>.plt,
 * FluidField/<step>.plt, CellCoor/<step>.plt, CellForce/<step>.plt,
 * CellNorDir/<step>.plt under `dir`, and one line per cell appended to
 * CellForce/TF_Cell<i>.plt and CellGeo/Geo_Cell<i>.plt (truncated first
 * when `first` is set, as the reference does at StepCount 0).  Particles are
 * written in original id order and each cell's vertices in membrane order
 * (the zone-local numbering of the triangles follows). */
typedef struct {
    long long n;              /* particles */
    long long n_b1, n_b2;     /* Bound1 ids [0, n_b1), Bound2 ids [n_b1, n_b1 + n_b2) */
    long long n_cell_start;   /* fluid ids up to here, membrane vertices from here to n */
    const float* pos;         /* n x 3, original order */
    const float* vel;         /* n x 3 */
    const float* rho;         /* n */
    const float* press;       /* n */
    int ncell, ntri;
    const int* cell_verts;    /* ncell x 2: first and last membrane vertex of each cell (0-based, inclusive) */
    const int* tri;           /* ntri x 3: 1-based membrane vertex indices */
    const int* betri;         /* ncell x 2: first and last triangle of each cell */
    const float* defforce;    /* ncp x 3 */
    const float* aggforce;    /* ncp x 3 */
    const float* tricenter;   /* ntri x 3 */
    const float* trinordir;   /* ntri x 3 */
    const double* cell_stats; /* ncell x 12: mean DefForce, mean AggForce, mean velocity (x, y, z each),
                                 |mean velocity|, area, volume */
    int threads;              /* formatting threads (0: all cores) */
    int reserved;
} GcOutputFrame;
int gc_output_write(const GcOutputFrame* frame, const char* dir, long long step_data, double time, int first);
/* Per-cell statistics of one system of a fused handle, reduced on the GPU in
 * FP64: ncell x 12 doubles as GcOutputFrame.cell_stats (host pointer). */
int gc_ensemble_cell_stats(GcFused* f, int sys, double* out);
/* Diagnostics of one system, reduced on the GPU in FP64 in a fixed order:
 * out[0..2] total momentum of the moving (fluid and membrane) particles,
 * out[3] their kinetic energy, out[4] k_B T from their peculiar velocities
 * ((2 E_kin - |P|^2/M) / 3N), out[5] the largest speed, out[6] the mean fluid
 * density, out[7] the number of moving particles.  Host pointer, 8 doubles. */
int gc_ensemble_diagnostics(GcFused* f, int sys, double* out);
/* Rouleaux (aggregates of red cells) of one system: two cells are in contact
 * when a vertex of one and a vertex of the other are closer than `contact`
 * (minimum image; FP32 squared distance < contact^2), and a rouleau is a
 * connected set of cells under contact.  label[c] (ncell ints, may be NULL)
 * receives the rouleau of cell c, numbered 0.. in the order of each
 * rouleau's lowest cell; size[k] (ncell ints, may be NULL) the number of
 * cells of rouleau k (0 past the last); *nrouleaux the number of rouleaux.
 * Contacts are found on the GPU: bounding spheres of the cells select the
 * candidate pairs, then one block per pair tests their vertices. */
int gc_ensemble_rouleaux(GcFused* f, int sys, float contact, int* label, int* size, int* nrouleaux);
/* The rouleau labelling of gc_ensemble_rouleaux from a list of contact pairs
 * (npairs x 2 cell indices in 0..ncell-1); host only. */
int gc_rouleaux_from_pairs(int ncell, int npairs, const int* pairs, int* label, int* size, int* nrouleaux);
/* Stores one system of a fused handle and writes its output files. */
int gc_ensemble_write_output(GcFused* f, int sys, const char* dir, long long step_data, double time, int first,
                             int threads);
int gc_fused_write_output(GcFused* f, const char* dir, long long step_data, double time, int first, int threads);

/* ---- input files (GPUCell's loaders, src/Particle.cu:45-380) -------------
 *
 * The four input files (SDPDParCoor.txt, SDPDPhyPara.txt, CELLParStruct.txt,
 * CELLPhyPara.txt) parsed with the reference's rules -- 20-character
 * columns, atof conversion, one header line before every block, the
 * per-cell vertex and triangle offsets added to the topology, the per-type
 * moduli spread over edges and triangles -- but without its fixed array
 * sizes (2,000,000 wall + fluid particles, 4,000,000 membrane vertices,
 * src/Particle.cu:31-32, 200-202).  The set owns its arrays (malloc);
 * gc_input_free releases them.  The binary form holds the same set for fast
 * reloading. */
typedef struct {
    long long n_b1, n_b2, n_fluid;   /* SDPDParCoor.txt */
    float* sdpd_coor;                /* (n_b1 + n_b2 + n_fluid) x 3: Bound1, Bound2, fluid */
    float sound1, sound2, shear_vis, bulk_vis, den_init, ext_force;   /* SDPDPhyPara.txt (force per mass) */
    int ncell, ntype;                /* CELLParStruct.txt, CELLPhyPara.txt */
    long long ncp, ntri, nedge;
    int* cell_type;                  /* ncell: 1-based type */
    int* npar;                       /* ncell: vertices per cell */
    int* ntri_cell;                  /* ncell: triangles per cell */
    float* cell_coor;                /* ncp x 3 */
    int* tri;                        /* ntri x 3: 1-based membrane vertex indices */
    int* edge;                       /* nedge x 6: p1..p4 1-based vertices, t1 t2 1-based triangles */
    int* betri;                      /* ncell x 2: first and last triangle of each cell */
    int* celltab;                    /* ncp: 0-based cell of each vertex */
    float *shear_mod, *bending_mod, *hgarea, *hlarea, *hvol;   /* ntype each */
    float max_cut, zero_len, sca_fac, sur_energy;
    float *shear_e, *bend_e;         /* nedge: moduli of each edge's cell type */
    float *hl_t, *hg_t, *hv_t;       /* ntri */
} GcInputSet;
int gc_input_read(const char* dir, GcInputSet* out);
int gc_input_write_binary(const char* path, const GcInputSet* set);
int gc_input_read_binary(const char* path, GcInputSet* out);
int gc_input_free(GcInputSet* set);

/* ---- test hooks (no counterpart in the reference) ----------------------- */

/* Runs the production neighbour traversal of CalFluidDen over the current
 * sort and, for every slot, writes the number of neighbours within
 * CutRadius (d_count) and an order-independent checksum of their original
 * ids (d_hash: the sum over neighbours of a 64-bit mix of the id).  Used to
 * prove the neighbour sets equal the oracle's. */
int gc_debug_neighbor_stats(int n, float* d_totalcoor, int* d_sortpart, int* d_beginendcube, int* d_count, unsigned long long* d_hash);

#ifdef __cplusplus
}
#endif

#endif /* GPUCELL_GB300_H */
