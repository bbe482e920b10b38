/*
 * TypesDef.h -- plain-data types shared with GPUCell's host frame.
 *
 * These layouts are an ABI contract, not a design choice: GPUCell's
 * Particle class (src/Particle.cuh:11-116) passes these structs and arrays
 * of them straight into the cupar:: / cudiv:: entry points, and the C++
 * symbol names of those entry points embed the type names below (a typedef
 * of an unnamed struct gives the struct that name for linkage).  So the
 * names, member order and member types follow src/TypesDef.cuh:6-78
 * exactly; everything else in this library is its own design.
 *
 * Structconst is 96 bytes on LP64 (x86-64 and aarch64): five unsigned
 * counts, 4 bytes of padding, the long seed at offset 24, then fifteen
 * floats from offset 32 (Temp at 88) and 4 bytes of tail padding.
 */
#ifndef GPUCELL_TYPESDEF_H
#define GPUCELL_TYPESDEF_H

/* src/TypesDef.cuh:6-10 */
typedef struct {
    int x, y;
} tint2;

/* src/TypesDef.cuh:12-16 */
typedef struct {
    int x, y, z;
} tint3;

/* src/TypesDef.cuh:18-22: membrane edge record (p1, p2, p3, p4, t1, t2) */
typedef struct {
    int x, y, z, k, v, w;
} tint6;

/* src/TypesDef.cuh:24-28: the device-side twin of tint6 */
typedef struct {
    int x, y, z, k, v, w;
} int6;

/* src/TypesDef.cuh:31-35 */
typedef struct {
    float x, y, z, w, v;
} tfloat5;

/* src/TypesDef.cuh:37-41 */
typedef struct {
    float x, y, z, w;
} tfloat4;

/* src/TypesDef.cuh:43-47 */
typedef struct {
    float x, y, z;
} tfloat3;

/*
 * src/TypesDef.cuh:49-78: physical constants of one simulation.
 * Particle ids are grouped by type (src/Particle.cu:432-435):
 *   [0, nBound2Start)           Bound1 walls (repulsion only)
 *   [nBound2Start, nFluidStart) Bound2 walls (SDPD no-slip walls)
 *   [nFluidStart, nCellStart)   fluid
 *   [nCellStart, nTotalPar)     membrane vertices (nCellPar of them)
 */
typedef struct {
    unsigned nFluidStart;
    unsigned nBound2Start;
    unsigned nCellStart;
    unsigned nTotalPar;
    unsigned nCellPar;

    long int iSeed;          /* seed of the pair noise */

    float CutRadius;         /* kernel support rc */
    float Mass;              /* particle mass */
    float SoundSpeed1;       /* sound speed of fluid (and Bound2) particles */
    float SoundSpeed2;       /* sound speed of membrane particles */
    float DenInit;           /* reference density rho0 */
    float VVsigma;           /* lambda of the modified velocity-Verlet */
    float ShearVis;          /* shear viscosity eta */
    float BulkVis;           /* bulk viscosity zeta */
    float ConstExtForce;     /* body force in x (already times Mass) */

    float TimeStep;

    float surEnergy;         /* Morse well depth (surface energy density) */
    float MaxCut;            /* Morse cut-off */
    float zeroLen;           /* Morse zero-force length r0 */
    float scaFac;            /* Morse scaling factor beta */
    float Temp;              /* k_B T */
} Structconst;

#ifdef __cplusplus
static_assert(sizeof(Structconst) == 96, "Structconst must be 96 bytes");
#else
_Static_assert(sizeof(Structconst) == 96, "Structconst must be 96 bytes");
#endif

#endif /* GPUCELL_TYPESDEF_H */
