/*
 * oracle.h -- FP64 CPU restatement of GPUCell's SDPD + membrane timestep.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is the checker for the CUDA library:
 * tests, the smoke check and the CPU-baseline leg of the benchmark call it;
 * the library never does.
 *
 * PARITY UNPINNED against GPUCell itself: the reference ships the headers of
 * its GPU code (src/ParticleGPU.cuh, src/ConfigDomain.cuh) but not the kernel
 * bodies, and it has no tests, golden vectors or run outputs.  The oracle
 * therefore restates the method from the literature the reference's
 * parameter names point to, and is pinned to analytic known answers
 * (tests/golden/) and to finite-difference gradients of its own energies.
 *
 * All arrays are in ORIGINAL particle order (no sorting).  Positions,
 * velocities and forces are double; topology arrays use the reference's
 * 1-based membrane indices (src/Particle.cu:252-284).
 */
#ifndef GPUCELL_ORACLE_H
#define GPUCELL_ORACLE_H

#include <stdint.h>
#include "gpucell/TypesDef.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    Structconst c;          /* constants, as passed to cupar::ConstsDataUp */
    double bbox[6];         /* lo_x, hi_x, lo_y, hi_y, lo_z, hi_z (src/main.cuh:12) */
    int pmask;              /* periodic axes: 1 = x, 2 = y, 4 = z */
    int noise_on;           /* thermal pair noise on/off */
    long long step;         /* step index keying the pair noise */
    int drive_on;           /* body force on/off (src/Particle.cu:1302-1308) */
    int nthreads;           /* OpenMP threads (0 = default) */

    /* particles, n = c.nTotalPar */
    double* pos;            /* 3n */
    double* vel;            /* 3n, velocity used by the forces (velrhop.xyz) */
    double* rho;            /* n  */
    double* press;          /* n  */
    double* force;          /* 3n */
    double* velhalf;        /* 3n */
    int* nthro;             /* 3n periodic crossing counts */

    /* membranes */
    int ncell, ntri, nedge;
    const int* tri;         /* 3 ntri, 1-based membrane indices */
    const int* edge;        /* 6 nedge: p1 p2 p3 p4 (1-based) t1 t2 */
    const int* betri;       /* 2 ncell: first, last triangle (inclusive) */
    const int* celltab;     /* nCellPar: cell of each membrane vertex */
    const double* shearmod; /* nedge */
    const double* bendmod;  /* nedge */
    const double* hlarea;   /* ntri */
    const double* hgarea;   /* ntri */
    const double* hvol;     /* ntri */
    /* set-up outputs (or_mech_setup / or_geo with setup = 1) */
    double* refedgelen;     /* nedge */
    double* maxrefedgelen;  /* nedge */
    double* perlen;         /* nedge */
    double* hpow;           /* nedge */
    double* hbending;       /* nedge */
    double* refangle;       /* nedge */
    double* reftriarea;     /* ntri */
    double* refarea;        /* ncell */
    double* refvol;         /* ncell */
    /* per-step outputs */
    double* triarea;        /* ntri */
    double* trinormal;      /* 3 ntri */
    double* tricenter;      /* 3 ntri */
    double* area;           /* ncell */
    double* vol;            /* ncell */
    double* pararea;        /* nCellPar */
    double* defforce;       /* 3 nCellPar */
    double* aggforce;       /* 3 nCellPar */
} or_state;

/* Neighbour statistics over all particle pairs with r^2 < rc^2 (FP32
 * predicate, see oracle.c): count and sum of mix64(id) per particle. */
int or_neighbor_stats(const or_state* s, int* count, uint64_t* hash);

int or_update_coor(or_state* s);     /* K2 */
int or_periodic(or_state* s);        /* K3 */
int or_density(or_state* s);         /* K8 */
int or_predict(or_state* s);         /* K9 */
int or_bound2_vel(or_state* s);      /* K10 */
int or_eos(or_state* s);             /* K11 */
int or_sdpd_force(or_state* s);      /* K12: writes force of every particle */
int or_rep_force(or_state* s);       /* K13: adds */
int or_ext_force(or_state* s);       /* K14: adds */
int or_geo(or_state* s, int setup);  /* K15 */
int or_mech_setup(or_state* s);      /* K16 */
int or_def_force(or_state* s);       /* K17: defforce, and adds into force */
int or_agg_force(or_state* s);       /* K18: aggforce, and adds into force */
int or_correct(or_state* s);         /* K19 */
/* One full step in the order of Particle::UpdatePar (src/Particle.cu:1310-1329),
 * without the neighbour sort (the oracle keeps original order). */
int or_step(or_state* s);

/* Per particle (n values): the sum of the magnitudes of the terms its force
 * adds up, on the state as it is (for the rounding scale of a per-particle
 * force comparison; see oracle.c), for the parts selected by `parts`. */
#define OR_SCALE_SDPD  1   /* SDPD pair terms: conservative, dissipative, random */
#define OR_SCALE_REP   2   /* Bound1 wall repulsion */
#define OR_SCALE_BODY  4   /* body force (with drive_on) */
#define OR_SCALE_MEMB  8   /* membrane springs, bending, area, volume */
#define OR_SCALE_MORSE 16  /* Morse aggregation */
#define OR_SCALE_EOS   32  /* the pressure term counted at the size of c^2 rho (the rounding of an FP32
                              density reaches P = c^2 (rho - rho0) at that size); without it at |P| */
#define OR_SCALE_ALL   63
int or_force_scale(const or_state* s, int parts, double* scale);

/* Energies for finite-difference checks of the conservative forces. */
double or_membrane_energy(const or_state* s);   /* springs + bending + area + volume */
double or_morse_energy(const or_state* s);      /* aggregation */

/* The pair noise xi_ij (3 components) for ids i, j at the state's step. */
void or_pair_noise(const or_state* s, unsigned id_i, unsigned id_j, double out[3]);

/* Philox4x32-10 and Philox2x32-10 on one counter (known-answer tests). */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void or_philox2x32_10(const uint32_t ctr[2], uint32_t key, uint32_t out[2]);
/* Key of the pair noise at `step` for `seed`. */
uint32_t or_noise_key(uint64_t seed, uint64_t step);

#ifdef __cplusplus
}
#endif

#endif /* GPUCELL_ORACLE_H */
