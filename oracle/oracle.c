/*
 * oracle.c -- FP64 CPU restatement of GPUCell's SDPD + membrane timestep.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library (tests, the
 * smoke check and the benchmark's CPU-baseline leg use it; the library never
 * calls it).  PARITY UNPINNED against GPUCell: the reference's kernel bodies
 * (ParticleGPU.cu, ConfigDomain.cu) are not in the reference, which keeps
 * only their headers and the host frame, so this file restates the method
 * from the literature its parameter names point to:
 *
 *   call order          Particle::UpdatePar, src/Particle.cu:1310-1329
 *   particle types      src/Particle.cu:432-435 (Bound1, Bound2, fluid, membrane)
 *   constants           src/TypesDef.cuh:49-78, src/Particle.cu:436-437, :654-660
 *   topology            src/Particle.cu:174-303 (1-based indices), :405-425
 *   kernel              Wendland C2, support rc
 *   SDPD                Espanol & Revenga, PRE 67, 026705 (2003)
 *   integrator          Groot & Warren, JCP 107, 4423 (1997), lambda = VVsigma
 *   walls               Adami, Hu & Adams, JCP 231, 7057 (2012) (no-slip),
 *                       Monaghan, JCP 110, 399 (1994) (repulsion, 12-4)
 *   membrane            Fedosov, Caswell & Karniadakis, Biophys. J. 98, 2215 (2010)
 *   aggregation         Morse potential, area-weighted
 *   pair noise          Philox2x32-10, Salmon et al., SC'11, keyed per step
 *                       by the SplitMix64 finaliser
 *
 * Everything is double precision except the neighbour predicate, which is
 * evaluated in FP32 from the FP32-rounded positions exactly as the GPU does
 * (min image by one conditional shift, then ((dx*dx + dy*dy) + dz*dz) with
 * round-to-nearest and no contraction; this file is compiled with
 * -ffp-contract=off), so both sides select the same neighbour sets.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_PI 3.14159265358979323846

/* ------------------------------------------------------------------------ */
/* basic helpers                                                             */
/* ------------------------------------------------------------------------ */

static inline int is_mobile(const or_state* s, unsigned id) { return id >= s->c.nFluidStart; }
static inline int is_sdpd(const or_state* s, unsigned id) { return id >= s->c.nBound2Start; }
static inline int is_b1(const or_state* s, unsigned id) { return id < s->c.nBound2Start; }
static inline int is_b2(const or_state* s, unsigned id) { return id >= s->c.nBound2Start && id < s->c.nFluidStart; }
static inline int is_memb(const or_state* s, unsigned id) { return id >= s->c.nCellStart; }

static inline double box_len(const or_state* s, int a) { return s->bbox[2 * a + 1] - s->bbox[2 * a]; }

typedef struct { double x, y, z; } v3;
static inline v3 mk(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 scl(double k, v3 a) { return mk(k * a.x, k * a.y, k * a.z); }
static inline double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 crs(v3 a, v3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline double nrm(v3 a) { return sqrt(dot(a, a)); }
static inline v3 ld3(const double* p, long i) { return mk(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
static inline void st3(double* p, long i, v3 v) { p[3 * i] = v.x; p[3 * i + 1] = v.y; p[3 * i + 2] = v.z; }
static inline void acc3(double* p, long i, v3 v) { p[3 * i] += v.x; p[3 * i + 1] += v.y; p[3 * i + 2] += v.z; }

/* Minimum-image displacement x_i - x_j in double. */
static inline v3 disp(const or_state* s, long i, long j) {
    double d[3];
    for (int a = 0; a < 3; ++a) {
        d[a] = s->pos[3 * i + a] - s->pos[3 * j + a];
        if (s->pmask & (1 << a)) {
            double L = box_len(s, a);
            if (d[a] > 0.5 * L) d[a] -= L;
            else if (d[a] < -0.5 * L) d[a] += L;
        }
    }
    return mk(d[0], d[1], d[2]);
}

/* The FP32 neighbour predicate value r^2 (see the file comment). */
static inline float r2_f32(const or_state* s, long i, long j) {
    float d[3];
    for (int a = 0; a < 3; ++a) {
        float xi = (float)s->pos[3 * i + a], xj = (float)s->pos[3 * j + a];
        float v = xi - xj;
        if (s->pmask & (1 << a)) {
            float L = (float)s->bbox[2 * a + 1] - (float)s->bbox[2 * a];
            float h = 0.5f * L;
            if (v > h) v = v - L;
            else if (v < -h) v = v + L;
        }
        d[a] = v;
    }
    float xx = d[0] * d[0], yy = d[1] * d[1], zz = d[2] * d[2];
    float t = xx + yy;
    return t + zz;
}

static inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 and the pair noise                                           */
/* ------------------------------------------------------------------------ */

void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Philox2x32-10: one 32x32 -> 64 multiply per round, Weyl key schedule. */
void or_philox2x32_10(const uint32_t ctr[2], uint32_t key, uint32_t out[2]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], k = key;
    for (int r = 0; r < 10; ++r) {
        uint64_t pr = (uint64_t)0xD256D193u * c0;
        uint32_t n0 = (uint32_t)(pr >> 32) ^ k ^ c1;
        c1 = (uint32_t)pr;
        c0 = n0;
        k += 0x9E3779B9u;
    }
    out[0] = c0;
    out[1] = c1;
}

/* Per-step key: SplitMix64 finaliser of seed * golden + step, high word. */
uint32_t or_noise_key(uint64_t seed, uint64_t step) {
    return (uint32_t)(mix64(seed * 0x9E3779B97F4A7C15ull + step) >> 32);
}

/* The pair noise: Philox2x32-10 on (min id, max id) with the step key; three
 * 21-bit fields of the 64 output bits, each mapped to a uniform variate of
 * zero mean and unit variance; antisymmetric in (i, j). */
void or_pair_noise(const or_state* s, unsigned id_i, unsigned id_j, double out[3]) {
    unsigned a = id_i < id_j ? id_i : id_j, b = id_i < id_j ? id_j : id_i;
    uint32_t ctr[2] = {a, b}, w[2];
    or_philox2x32_10(ctr, or_noise_key((uint64_t)s->c.iSeed, (uint64_t)s->step), w);
    uint32_t u[3] = {w[0] & 0x1FFFFFu, (w[0] >> 21) | ((w[1] & 0x3FFu) << 11), (w[1] >> 10) & 0x1FFFFFu};
    double sg = id_i < id_j ? 1.0 : -1.0;
    for (int k = 0; k < 3; ++k) out[k] = sg * (sqrt(12.0) * (((double)u[k] + 0.5) / 2097152.0) - sqrt(3.0));
}

/* ------------------------------------------------------------------------ */
/* Cell list (the oracle's own; any bins at least `cut` wide give the same  */
/* pair sets because the predicate decides)                                 */
/* ------------------------------------------------------------------------ */

typedef struct {
    int nb[3];
    double origin[3], invw[3];
    int pmask;
    int* start;   /* nbins + 1 */
    int* items;   /* member particle ids sorted by bin */
    int* binof;   /* bin of each particle (-1 = not a member) */
    long n;
} bins_t;

static int bin_coord(const bins_t* b, int a, double x) {
    int c = (int)floor((x - b->origin[a]) * b->invw[a]);
    int n = b->nb[a];
    if (b->pmask & (1 << a)) {
        c %= n;
        if (c < 0) c += n;
    } else {
        c = c < 0 ? 0 : (c >= n ? n - 1 : c);
    }
    return c;
}

/* member(i) decides which particles are binned (NULL = all). */
static int bins_build(bins_t* b, const or_state* s, double cut, int (*member)(const or_state*, unsigned)) {
    long n = s->c.nTotalPar;
    memset(b, 0, sizeof(*b));
    b->n = n;
    b->pmask = s->pmask;
    for (int a = 0; a < 3; ++a) {
        double lo, span;
        if (s->pmask & (1 << a)) {
            lo = s->bbox[2 * a];
            span = box_len(s, a);
        } else {
            double mn = s->bbox[2 * a], mx = s->bbox[2 * a + 1];
            for (long i = 0; i < n; ++i) {
                double x = s->pos[3 * i + a];
                if (x < mn) mn = x;
                if (x > mx) mx = x;
            }
            lo = mn - 1e-9;
            span = mx - mn + 2e-9;
        }
        int nb = (int)floor(span / (cut * (1.0 + 1e-3)));   /* margin covers FP32 rounding of the predicate */
        if (nb < 1) nb = 1;
        if (nb > 4096) nb = 4096;
        b->nb[a] = nb;
        b->origin[a] = lo;
        b->invw[a] = nb / span;
    }
    long nbins = (long)b->nb[0] * b->nb[1] * b->nb[2];
    b->start = (int*)calloc(nbins + 1, sizeof(int));
    b->items = (int*)malloc((n > 0 ? n : 1) * sizeof(int));
    b->binof = (int*)malloc((n > 0 ? n : 1) * sizeof(int));
    if (!b->start || !b->items || !b->binof) return -1;
    for (long i = 0; i < n; ++i) {
        if (member && !member(s, (unsigned)i)) {
            b->binof[i] = -1;
            continue;
        }
        int cx = bin_coord(b, 0, s->pos[3 * i]), cy = bin_coord(b, 1, s->pos[3 * i + 1]),
            cz = bin_coord(b, 2, s->pos[3 * i + 2]);
        int k = cx + b->nb[0] * (cy + b->nb[1] * cz);
        b->binof[i] = k;
        b->start[k + 1]++;
    }
    for (long k = 0; k < nbins; ++k) b->start[k + 1] += b->start[k];
    int* fill = (int*)malloc((nbins + 1) * sizeof(int));
    if (!fill) return -1;
    memcpy(fill, b->start, (nbins + 1) * sizeof(int));
    for (long i = 0; i < n; ++i)
        if (b->binof[i] >= 0) b->items[fill[b->binof[i]]++] = (int)i;
    free(fill);
    return 0;
}

static void bins_free(bins_t* b) {
    free(b->start);
    free(b->items);
    free(b->binof);
}

/* Unique candidate bins along axis a around coordinate c. */
static int cand_axis(const bins_t* b, int a, int c, int out[3]) {
    int n = b->nb[a], k = 0;
    if ((b->pmask & (1 << a)) && n <= 3) {
        for (int t = 0; t < n; ++t) out[k++] = t;
        return k;
    }
    for (int d = -1; d <= 1; ++d) {
        int t = c + d;
        if (b->pmask & (1 << a)) {
            if (t < 0) t += n;
            if (t >= n) t -= n;
        } else if (t < 0 || t >= n) {
            continue;
        }
        out[k++] = t;
    }
    return k;
}

/* Runs the trailing statement block with J bound to every binned particle in
 * the bins around particle i. */
#define FOR_CANDIDATES(b, s, i, J, ...)                                                 \
    do {                                                                                  \
        int cx_ = bin_coord(b, 0, (s)->pos[3 * (i)]), cy_ = bin_coord(b, 1, (s)->pos[3 * (i) + 1]), \
            cz_ = bin_coord(b, 2, (s)->pos[3 * (i) + 2]);                                 \
        int ax_[3], ay_[3], az_[3];                                                       \
        int nx_ = cand_axis(b, 0, cx_, ax_), ny_ = cand_axis(b, 1, cy_, ay_), nz_ = cand_axis(b, 2, cz_, az_); \
        for (int zz_ = 0; zz_ < nz_; ++zz_)                                               \
            for (int yy_ = 0; yy_ < ny_; ++yy_)                                           \
                for (int xx_ = 0; xx_ < nx_; ++xx_) {                                     \
                    int k_ = ax_[xx_] + (b)->nb[0] * (ay_[yy_] + (b)->nb[1] * az_[zz_]);  \
                    for (int q_ = (b)->start[k_]; q_ < (b)->start[k_ + 1]; ++q_) {        \
                        long J = (b)->items[q_];                                          \
                        __VA_ARGS__                                                       \
                    }                                                                     \
                }                                                                         \
    } while (0)

static void set_threads(const or_state* s) {
#ifdef _OPENMP
    if (s->nthreads > 0) omp_set_num_threads(s->nthreads);
#else
    (void)s;
#endif
}

/* ------------------------------------------------------------------------ */
/* Wendland C2                                                               */
/* ------------------------------------------------------------------------ */

static inline double wend_w(const or_state* s, double r) {
    double rc = s->c.CutRadius, q = r / rc, t = 1.0 - q;
    return 21.0 / (2.0 * OR_PI * rc * rc * rc) * t * t * t * t * (1.0 + 4.0 * q);
}

static inline double wend_f(const or_state* s, double r) {   /* -W'(r)/r */
    double rc = s->c.CutRadius, t = 1.0 - r / rc;
    return 210.0 / (OR_PI * rc * rc * rc * rc * rc) * t * t * t;
}

static inline float rc2_f(const or_state* s) { return s->c.CutRadius * s->c.CutRadius; }

/* ------------------------------------------------------------------------ */
/* Neighbour statistics                                                      */
/* ------------------------------------------------------------------------ */

int or_neighbor_stats(const or_state* s, int* count, uint64_t* hash) {
    bins_t b;
    if (bins_build(&b, s, s->c.CutRadius, NULL)) return -1;
    long n = s->c.nTotalPar;
    float rc2 = rc2_f(s);
    set_threads(s);
#pragma omp parallel for schedule(dynamic, 256)
    for (long i = 0; i < n; ++i) {
        int cnt = 0;
        uint64_t h = 0;
        FOR_CANDIDATES(&b, s, i, j, {
            if (j == i) continue;
            if (r2_f32(s, i, j) >= rc2) continue;
            ++cnt;
            h += mix64((uint64_t)j);
        });
        count[i] = cnt;
        hash[i] = h;
    }
    bins_free(&b);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Integrator stages (Groot & Warren 1997)                                   */
/* ------------------------------------------------------------------------ */

int or_update_coor(or_state* s) {   /* r += dt v + dt^2/2 F/m */
    long n = s->c.nTotalPar;
    double dt = s->c.TimeStep, im = 1.0 / s->c.Mass;
    for (long i = 0; i < n; ++i) {
        if (!is_mobile(s, (unsigned)i)) continue;
        for (int a = 0; a < 3; ++a)
            s->pos[3 * i + a] += dt * s->vel[3 * i + a] + 0.5 * dt * dt * im * s->force[3 * i + a];
    }
    return 0;
}

int or_periodic(or_state* s) {
    long n = s->c.nTotalPar;
    for (long i = 0; i < n; ++i) {
        if (!is_mobile(s, (unsigned)i)) continue;
        for (int a = 0; a < 3; ++a) {
            if (!(s->pmask & (1 << a))) continue;
            double lo = s->bbox[2 * a], hi = s->bbox[2 * a + 1], L = hi - lo;
            double x = s->pos[3 * i + a];
            if (x >= hi) { x -= L; s->nthro[3 * i + a] += 1; }
            else if (x < lo) { x += L; s->nthro[3 * i + a] -= 1; }
            s->pos[3 * i + a] = x;
        }
    }
    return 0;
}

int or_predict(or_state* s) {   /* VelHalf = v + dt/2 F/m; v += lambda dt F/m */
    long n = s->c.nTotalPar;
    double dt = s->c.TimeStep, im = 1.0 / s->c.Mass, lam = s->c.VVsigma;
    for (long i = 0; i < n; ++i) {
        if (!is_mobile(s, (unsigned)i)) continue;
        for (int a = 0; a < 3; ++a) {
            double f = s->force[3 * i + a];
            s->velhalf[3 * i + a] = s->vel[3 * i + a] + 0.5 * dt * im * f;
            s->vel[3 * i + a] += lam * dt * im * f;
        }
    }
    return 0;
}

int or_correct(or_state* s) {   /* v = VelHalf + dt/2 F/m */
    long n = s->c.nTotalPar;
    double dt = s->c.TimeStep, im = 1.0 / s->c.Mass;
    for (long i = 0; i < n; ++i) {
        if (!is_mobile(s, (unsigned)i)) continue;
        for (int a = 0; a < 3; ++a) s->vel[3 * i + a] = s->velhalf[3 * i + a] + 0.5 * dt * im * s->force[3 * i + a];
    }
    return 0;
}

int or_ext_force(or_state* s) {
    if (!s->drive_on) return 0;
    long n = s->c.nTotalPar;
    for (long i = 0; i < n; ++i)
        if (is_mobile(s, (unsigned)i)) s->force[3 * i] += s->c.ConstExtForce;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Density, EOS, wall velocity                                               */
/* ------------------------------------------------------------------------ */

int or_density(or_state* s) {
    bins_t b;
    if (bins_build(&b, s, s->c.CutRadius, NULL)) return -1;
    long n = s->c.nTotalPar;
    float rc2 = rc2_f(s);
    set_threads(s);
#pragma omp parallel for schedule(dynamic, 256)
    for (long i = 0; i < n; ++i) {
        if (!is_mobile(s, (unsigned)i)) continue;
        double sum = wend_w(s, 0.0);
        FOR_CANDIDATES(&b, s, i, j, {
            if (j == i || !is_sdpd(s, (unsigned)j)) continue;
            if (r2_f32(s, i, j) >= rc2) continue;
            sum += wend_w(s, nrm(disp(s, i, j)));
        });
        s->rho[i] = s->c.Mass * sum;
    }
    bins_free(&b);
    return 0;
}

int or_eos(or_state* s) {
    long n = s->c.nTotalPar;
    double c1 = s->c.SoundSpeed1, c2 = s->c.SoundSpeed2, r0 = s->c.DenInit;
    for (long i = 0; i < n; ++i) {
        unsigned id = (unsigned)i;
        if (is_b1(s, id)) s->press[i] = 0.0;
        else if (is_memb(s, id)) s->press[i] = c2 * c2 * (s->rho[i] - r0);
        else s->press[i] = c1 * c1 * (s->rho[i] - r0);
    }
    return 0;
}

int or_bound2_vel(or_state* s) {
    if (s->c.nFluidStart == s->c.nBound2Start) return 0;
    bins_t b;
    if (bins_build(&b, s, s->c.CutRadius, NULL)) return -1;
    float rc2 = rc2_f(s);
    long lo = s->c.nBound2Start, hi = s->c.nFluidStart;
    set_threads(s);
#pragma omp parallel for schedule(dynamic, 256)
    for (long i = lo; i < hi; ++i) {
        v3 num = mk(0, 0, 0);
        double den = 0.0;
        FOR_CANDIDATES(&b, s, i, j, {
            if (!is_mobile(s, (unsigned)j)) continue;
            if (r2_f32(s, i, j) >= rc2) continue;
            double w = wend_w(s, nrm(disp(s, i, j)));
            num = add(num, scl(w, ld3(s->vel, j)));
            den += w;
        });
        v3 vw = ld3(s->velhalf, i);
        if (den > 0.0) st3(s->vel, i, sub(scl(2.0, vw), scl(1.0 / den, num)));
        else st3(s->vel, i, vw);
    }
    bins_free(&b);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* SDPD force (Espanol & Revenga 2003), with d = rho/m:                      */
/*   f_i = sum_j (P_i/d_i^2 + P_j/d_j^2) F_ij r_ij                           */
/*         - F_ij/(d_i d_j) [A v_ij + B e (e.v_ij)]                           */
/*         + sqrt(2 kT F_ij/(d_i d_j dt)) [sqrt(A) xi + (sqrt(A+B)-sqrt(A)) e (e.xi)] */
/*   A = 5 eta/3 - zeta, B = 5 (zeta + eta/3).                               */
/* The random term has covariance 2 kT [A (1 - ee) + (A+B) ee] F/(d_i d_j),  */
/* the fluctuation-dissipation partner of the friction matrix.               */
/* ------------------------------------------------------------------------ */

int or_sdpd_force(or_state* s) {
    bins_t b;
    if (bins_build(&b, s, s->c.CutRadius, NULL)) return -1;
    long n = s->c.nTotalPar;
    float rc2 = rc2_f(s);
    double m = s->c.Mass, eta = s->c.ShearVis, zeta = s->c.BulkVis;
    double A = 5.0 * eta / 3.0 - zeta, B = 5.0 * (zeta + eta / 3.0);
    double sA = sqrt(A > 0 ? A : 0), sAB = sqrt(A + B > 0 ? A + B : 0);
    int noise = s->noise_on && s->c.Temp > 0.f;
    double pref = noise ? 2.0 * s->c.Temp / s->c.TimeStep : 0.0;
    set_threads(s);
#pragma omp parallel for schedule(dynamic, 256)
    for (long i = 0; i < n; ++i) {
        if (!is_mobile(s, (unsigned)i)) {
            st3(s->force, i, mk(0, 0, 0));
            continue;
        }
        double di = s->rho[i] / m, pi = s->press[i] / (di * di);
        v3 vi = ld3(s->vel, i), f = mk(0, 0, 0);
        FOR_CANDIDATES(&b, s, i, j, {
            if (j == i || !is_sdpd(s, (unsigned)j)) continue;
            if (r2_f32(s, i, j) >= rc2) continue;
            v3 d = disp(s, i, j);
            double r = nrm(d), F = wend_f(s, r);
            double dj = s->rho[j] / m;
            f = add(f, scl((pi + s->press[j] / (dj * dj)) * F, d));
            if (r <= 0.0) continue;
            v3 e = scl(1.0 / r, d), vij = sub(vi, ld3(s->vel, j));
            double ev = dot(e, vij), fdd = F / (di * dj);
            f = sub(f, scl(fdd, add(scl(A, vij), scl(B * ev, e))));
            if (noise) {
                double xi[3];
                or_pair_noise(s, (unsigned)i, (unsigned)j, xi);
                v3 x = mk(xi[0], xi[1], xi[2]);
                /* The pair passed the FP32 cut-off test (the GPU's predicate) but r is
                 * evaluated in FP64: at the cut-off, F can be a rounding-sized negative
                 * number.  Such a pair gets no noise, as on the GPU. */
                double q = fdd > 0.0 ? sqrt(pref * fdd) : 0.0;
                f = add(f, scl(q, add(scl(sA, x), scl((sAB - sA) * dot(e, x), e))));
            }
        });
        st3(s->force, i, f);
    }
    bins_free(&b);
    return 0;
}

/* Bound1 repulsion (Monaghan 1994, exponents 12 and 4), r0 = rc/3, D = c1^2. */
int or_rep_force(or_state* s) {
    if (s->c.nBound2Start == 0) return 0;
    bins_t b;
    if (bins_build(&b, s, s->c.CutRadius, NULL)) return -1;
    long n = s->c.nTotalPar;
    float r0f = (float)(s->c.CutRadius / 3.0);
    float r0sq = r0f * r0f;
    double r0 = s->c.CutRadius / 3.0, D = (double)s->c.SoundSpeed1 * s->c.SoundSpeed1;
    set_threads(s);
#pragma omp parallel for schedule(dynamic, 256)
    for (long i = 0; i < n; ++i) {
        if (!is_mobile(s, (unsigned)i)) continue;
        v3 f = mk(0, 0, 0);
        FOR_CANDIDATES(&b, s, i, j, {
            if (!is_b1(s, (unsigned)j)) continue;
            float r2f = r2_f32(s, i, j);
            if (r2f >= r0sq || r2f <= 0.f) continue;
            v3 d = disp(s, i, j);
            double r2 = dot(d, d), q2 = r0 * r0 / r2, q4 = q2 * q2, q12 = q4 * q4 * q4;
            f = add(f, scl(D * (q12 - q4) / r2, d));
        });
        acc3(s->force, i, f);
    }
    bins_free(&b);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Membranes (Fedosov, Caswell & Karniadakis 2010)                           */
/* ------------------------------------------------------------------------ */

static inline long memb_id(const or_state* s, int one_based) { return (long)s->c.nCellStart + one_based - 1; }

/* Unwrapped position x + nThroBound L. */
static inline v3 unwrapped(const or_state* s, long id) {
    v3 x = ld3(s->pos, id);
    if (s->pmask & 1) x.x += s->nthro[3 * id] * box_len(s, 0);
    if (s->pmask & 2) x.y += s->nthro[3 * id + 1] * box_len(s, 1);
    if (s->pmask & 4) x.z += s->nthro[3 * id + 2] * box_len(s, 2);
    return x;
}

int or_geo(or_state* s, int setup) {
    long ncp = s->c.nCellPar;
    for (long v = 0; v < ncp; ++v) s->pararea[v] = 0.0;
    set_threads(s);
#pragma omp parallel for schedule(dynamic, 1)
    for (int c = 0; c < s->ncell; ++c) {
        int t0 = s->betri[2 * c], t1 = s->betri[2 * c + 1];
        v3 xr = unwrapped(s, memb_id(s, s->tri[3 * t0]));
        double A = 0.0, V = 0.0;
        for (int t = t0; t <= t1; ++t) {
            const int* T = s->tri + 3 * t;
            v3 u1 = sub(unwrapped(s, memb_id(s, T[0])), xr);
            v3 u2 = sub(unwrapped(s, memb_id(s, T[1])), xr);
            v3 u3 = sub(unwrapped(s, memb_id(s, T[2])), xr);
            v3 xi = crs(sub(u2, u1), sub(u3, u1));
            double len = nrm(xi), At = 0.5 * len;
            s->triarea[t] = At;
            st3(s->trinormal, t, len > 0 ? scl(1.0 / len, xi) : mk(0, 0, 0));
            st3(s->tricenter, t, add(xr, scl(1.0 / 3.0, add(add(u1, u2), u3))));
            if (setup) s->reftriarea[t] = At;
            A += At;
            V += dot(u1, crs(u2, u3)) / 6.0;
            for (int k = 0; k < 3; ++k) s->pararea[T[k] - 1] += At / 3.0;   /* vertices belong to one cell */
        }
        s->area[c] = A;
        s->vol[c] = V;
        if (setup) {
            s->refarea[c] = A;
            s->refvol[c] = V;
        }
    }
    return 0;
}

/* Dihedral angle of (i, j, k, l) as the angle between planes ijk and jkl,
 * signed by r_ij . (r_kj x r_kl) (GROMACS-manual convention), and its
 * gradient d phi / d x. */
typedef struct { double c, s; v3 gi, gj, gk, gl; } dih_t;

static dih_t dihedral(v3 xi, v3 xj, v3 xk, v3 xl) {
    dih_t D;
    v3 rij = sub(xi, xj), rkj = sub(xk, xj), rkl = sub(xk, xl);
    v3 m = crs(rij, rkj), n = crs(rkj, rkl);
    double m2 = dot(m, m), n2 = dot(n, n), kj2 = dot(rkj, rkj), kj = sqrt(kj2), mn = sqrt(m2 * n2);
    D.c = mn > 0 ? dot(m, n) / mn : 1.0;
    D.s = mn > 0 ? dot(m, rkl) * kj / mn : 0.0;
    D.gi = m2 > 0 ? scl(kj / m2, m) : mk(0, 0, 0);
    D.gl = n2 > 0 ? scl(-kj / n2, n) : mk(0, 0, 0);
    double a = kj2 > 0 ? dot(rij, rkj) / kj2 : 0, b = kj2 > 0 ? dot(rkl, rkj) / kj2 : 0;
    D.gj = sub(scl(a - 1.0, D.gi), scl(b, D.gl));
    D.gk = sub(scl(b - 1.0, D.gl), scl(a, D.gi));
    return D;
}

#define OR_X0 (1.0 / 2.2)
#define OR_POWM 2.0

int or_mech_setup(or_state* s) {
    double kT = s->c.Temp, x0 = OR_X0, m = OR_POWM, u = 1.0 - x0;
    double kwlc = 1.0 / (4.0 * u * u) - 0.25 + x0;
    double kmod = x0 / (2.0 * u * u * u) - 1.0 / (4.0 * u * u) + 0.25;
    for (int e = 0; e < s->nedge; ++e) {
        const int* E = s->edge + 6 * e;
        v3 x1 = unwrapped(s, memb_id(s, E[0]));
        v3 b = sub(unwrapped(s, memb_id(s, E[1])), x1);
        v3 c = sub(unwrapped(s, memb_id(s, E[2])), x1);
        v3 d = sub(unwrapped(s, memb_id(s, E[3])), x1);
        double l0 = nrm(b);
        /* mu0 = (kT/p) C  (linear shear modulus of the WLC-POW network) */
        double C = sqrt(3.0) / (4.0 * l0) * (kmod + (m + 1.0) * kwlc);
        double mu0 = s->shearmod[e];
        double p = (mu0 > 0 && kT > 0) ? kT * C / mu0 : 0.0;
        s->refedgelen[e] = l0;
        s->maxrefedgelen[e] = l0 / x0;
        s->perlen[e] = p;
        s->hpow[e] = p > 0 ? (kT / p) * pow(l0, m) * kwlc : 0.0;   /* zero spring force at l0 */
        s->hbending[e] = 2.0 * s->bendmod[e] / sqrt(3.0);
        dih_t D = dihedral(c, mk(0, 0, 0), b, d);
        s->refangle[e] = atan2(D.s, D.c);
    }
    return 0;
}

/* spring force magnitude along the edge (positive = repulsive) */
static double spring_f(const or_state* s, int e, double r) {
    double p = s->perlen[e];
    if (!(p > 0) || !(r > 0)) return 0.0;
    double x = r / s->maxrefedgelen[e];
    if (x > 0.99) x = 0.99;
    double u = 1.0 - x;
    return -(s->c.Temp / p) * (1.0 / (4.0 * u * u) - 0.25 + x) + s->hpow[e] / pow(r, OR_POWM);
}

static double spring_u(const or_state* s, int e, double r) {
    double p = s->perlen[e];
    if (!(p > 0) || !(r > 0)) return 0.0;
    double lm = s->maxrefedgelen[e], x = r / lm;
    double uw = s->c.Temp * lm / (4.0 * p) * (3.0 * x * x - 2.0 * x * x * x) / (1.0 - x);
    double up = s->hpow[e] / ((OR_POWM - 1.0) * pow(r, OR_POWM - 1.0));
    return uw + up;
}

int or_def_force(or_state* s) {
    long ncp = s->c.nCellPar;
    for (long v = 0; v < 3 * ncp; ++v) s->defforce[v] = 0.0;
    for (int e = 0; e < s->nedge; ++e) {
        const int* E = s->edge + 6 * e;
        v3 x1 = unwrapped(s, memb_id(s, E[0]));
        v3 a = mk(0, 0, 0);
        v3 b = sub(unwrapped(s, memb_id(s, E[1])), x1);
        v3 c = sub(unwrapped(s, memb_id(s, E[2])), x1);
        v3 d = sub(unwrapped(s, memb_id(s, E[3])), x1);
        double r = nrm(b);
        double fm = spring_f(s, e, r);
        if (r > 0) {
            v3 eh = scl(-1.0 / r, b);
            acc3(s->defforce, E[0] - 1, scl(fm, eh));
            acc3(s->defforce, E[1] - 1, scl(-fm, eh));
        }
        double kb = s->hbending[e];
        if (kb != 0.0) {
            dih_t D = dihedral(c, a, b, d);
            double s0 = sin(s->refangle[e]), c0 = cos(s->refangle[e]);
            double dE = kb * (D.s * c0 - D.c * s0);
            acc3(s->defforce, E[2] - 1, scl(-dE, D.gi));
            acc3(s->defforce, E[0] - 1, scl(-dE, D.gj));
            acc3(s->defforce, E[1] - 1, scl(-dE, D.gk));
            acc3(s->defforce, E[3] - 1, scl(-dE, D.gl));
        }
    }
    for (int c = 0; c < s->ncell; ++c) {
        for (int t = s->betri[2 * c]; t <= s->betri[2 * c + 1]; ++t) {
            const int* T = s->tri + 3 * t;
            v3 x1 = unwrapped(s, memb_id(s, T[0]));
            v3 x2 = sub(unwrapped(s, memb_id(s, T[1])), x1);
            v3 x3 = sub(unwrapped(s, memb_id(s, T[2])), x1);
            v3 xi = crs(x2, x3);
            double len = nrm(xi);
            if (!(len > 0)) continue;
            double At = 0.5 * len;
            v3 nh = scl(1.0 / len, xi);
            double cA = s->hgarea[t] * (s->area[c] - s->refarea[c]) / s->refarea[c] +
                        s->hlarea[t] * (At - s->reftriarea[t]) / s->reftriarea[t];
            double cV = s->hvol[t] * (s->vol[c] - s->refvol[c]) / s->refvol[c] / 6.0;
            v3 g1 = scl(0.5, crs(nh, sub(x3, x2))), g2 = scl(0.5, crs(nh, scl(-1.0, x3))), g3 = scl(0.5, crs(nh, x2));
            v3 fv = scl(-cV, xi);
            acc3(s->defforce, T[0] - 1, sub(fv, scl(cA, g1)));
            acc3(s->defforce, T[1] - 1, sub(fv, scl(cA, g2)));
            acc3(s->defforce, T[2] - 1, sub(fv, scl(cA, g3)));
        }
    }
    for (long v = 0; v < ncp; ++v) acc3(s->force, (long)s->c.nCellStart + v, ld3(s->defforce, v));
    return 0;
}

double or_membrane_energy(const or_state* s) {
    double E = 0.0;
    for (int e = 0; e < s->nedge; ++e) {
        const int* E6 = s->edge + 6 * e;
        v3 x1 = unwrapped(s, memb_id(s, E6[0]));
        v3 b = sub(unwrapped(s, memb_id(s, E6[1])), x1);
        v3 c = sub(unwrapped(s, memb_id(s, E6[2])), x1);
        v3 d = sub(unwrapped(s, memb_id(s, E6[3])), x1);
        E += spring_u(s, e, nrm(b));
        dih_t D = dihedral(c, mk(0, 0, 0), b, d);
        E += s->hbending[e] * (1.0 - cos(atan2(D.s, D.c) - s->refangle[e]));
    }
    for (int c = 0; c < s->ncell; ++c) {
        int t0 = s->betri[2 * c], t1 = s->betri[2 * c + 1];
        v3 xr = unwrapped(s, memb_id(s, s->tri[3 * t0]));
        double A = 0.0, V = 0.0;
        for (int t = t0; t <= t1; ++t) {
            const int* T = s->tri + 3 * t;
            v3 u1 = sub(unwrapped(s, memb_id(s, T[0])), xr);
            v3 u2 = sub(unwrapped(s, memb_id(s, T[1])), xr);
            v3 u3 = sub(unwrapped(s, memb_id(s, T[2])), xr);
            double At = 0.5 * nrm(crs(sub(u2, u1), sub(u3, u1)));
            double dA = At - s->reftriarea[t];
            E += s->hlarea[t] * dA * dA / (2.0 * s->reftriarea[t]);
            A += At;
            V += dot(u1, crs(u2, u3)) / 6.0;
        }
        double dA = A - s->refarea[c], dV = V - s->refvol[c];
        E += s->hgarea[t0] * dA * dA / (2.0 * s->refarea[c]);
        E += s->hvol[t0] * dV * dV / (2.0 * s->refvol[c]);
    }
    return E;
}

/* ------------------------------------------------------------------------ */
/* Morse aggregation between vertices of different cells                     */
/* ------------------------------------------------------------------------ */

static int memb_member(const or_state* s, unsigned id) { return is_memb(s, id); }

int or_agg_force(or_state* s) {
    long ncp = s->c.nCellPar;
    for (long v = 0; v < 3 * ncp; ++v) s->aggforce[v] = 0.0;
    if (s->c.surEnergy == 0.f || !(s->c.MaxCut > 0.f) || ncp == 0) return 0;
    bins_t b;
    if (bins_build(&b, s, s->c.MaxCut, memb_member)) return -1;
    float mc2 = s->c.MaxCut * s->c.MaxCut;
    double De = s->c.surEnergy, beta = s->c.scaFac, r0 = s->c.zeroLen;
    long nc = s->c.nCellStart;
    set_threads(s);
#pragma omp parallel for schedule(dynamic, 64)
    for (long v = 0; v < ncp; ++v) {
        long i = nc + v;
        int ci = s->celltab[v];
        v3 f = mk(0, 0, 0);
        FOR_CANDIDATES(&b, s, i, j, {
            long w = j - nc;
            if (s->celltab[w] == ci) continue;
            float r2f = r2_f32(s, i, j);
            if (r2f >= mc2 || r2f <= 0.f) continue;
            v3 d = disp(s, i, j);
            double r = nrm(d), ex = exp(beta * (r0 - r));
            double fm = 2.0 * De * beta * (ex * ex - ex) * 0.5 * (s->pararea[v] + s->pararea[w]);
            f = add(f, scl(fm / r, d));
        });
        st3(s->aggforce, v, f);
    }
    bins_free(&b);
    for (long v = 0; v < ncp; ++v) acc3(s->force, nc + v, ld3(s->aggforce, v));
    return 0;
}

double or_morse_energy(const or_state* s) {
    long ncp = s->c.nCellPar, nc = s->c.nCellStart;
    double De = s->c.surEnergy, beta = s->c.scaFac, r0 = s->c.zeroLen, E = 0.0;
    float mc2 = s->c.MaxCut * s->c.MaxCut;
    for (long v = 0; v < ncp; ++v)
        for (long w = v + 1; w < ncp; ++w) {
            if (s->celltab[v] == s->celltab[w]) continue;
            if (r2_f32(s, nc + v, nc + w) >= mc2) continue;
            double r = nrm(disp(s, nc + v, nc + w)), ex = exp(beta * (r0 - r));
            E += De * 0.5 * (s->pararea[v] + s->pararea[w]) * (ex * ex - 2.0 * ex);
        }
    return E;
}

/* ------------------------------------------------------------------------ */
/* Force scale: per particle, the sum of the magnitudes of every term its    */
/* force adds up (SDPD conservative, dissipative and random pair terms, wall */
/* repulsion, body force, each spring, bending, area and volume term of a    */
/* membrane vertex, each Morse pair), on the state as it is; a term that is  */
/* itself a difference of larger quantities (the pressure c^2 (rho - rho0),  */
/* the WLC and POW parts of a spring, the area and volume penalties near     */
/* rest) counts with the size of those quantities.  The rounding error of an */
/* FP32 evaluation of the force is a small multiple of FP32's unit roundoff  */
/* times this scale, whatever the cancellation in the net.                   */
/* ------------------------------------------------------------------------ */

int or_force_scale(const or_state* s, int parts, double* scale) {
    long n = s->c.nTotalPar;
    for (long i = 0; i < n; ++i) scale[i] = 0.0;
    bins_t b;
    if (bins_build(&b, s, s->c.CutRadius, NULL)) return -1;
    float rc2 = rc2_f(s);
    double m = s->c.Mass, eta = s->c.ShearVis, zeta = s->c.BulkVis, rc = s->c.CutRadius;
    double A = 5.0 * eta / 3.0 - zeta, B = 5.0 * (zeta + eta / 3.0);
    double sA = sqrt(A > 0 ? A : 0), sAB = sqrt(A + B > 0 ? A + B : 0);
    int noise = s->noise_on && s->c.Temp > 0.f;
    double pref = noise ? 2.0 * s->c.Temp / s->c.TimeStep : 0.0;
    float r0f = (float)(s->c.CutRadius / 3.0);
    float r0sq = r0f * r0f;
    double r0 = s->c.CutRadius / 3.0, D = (double)s->c.SoundSpeed1 * s->c.SoundSpeed1;
    const double fnorm = 210.0 / (OR_PI * rc * rc * rc * rc * rc), wnorm = 21.0 / (2.0 * OR_PI * rc * rc * rc);
    const int eos = (parts & OR_SCALE_EOS) != 0;
    /* with the EOS bit: per particle, the rounding scale of its number
     * density, W(0) + sum_j (W_ij + |W'_ij| r_ij) -- each kernel value and its
     * sensitivity to the rounding of r */
    double* dscale = NULL;
    if (eos && (parts & OR_SCALE_SDPD)) {
        dscale = (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
        if (!dscale) {
            bins_free(&b);
            return -1;
        }
        set_threads(s);
#pragma omp parallel for schedule(dynamic, 256)
        for (long i = 0; i < n; ++i) {
            if (!is_mobile(s, (unsigned)i)) continue;
            double acc = wend_w(s, 0.0);
            FOR_CANDIDATES(&b, s, i, j, {
                if (j == i || !is_sdpd(s, (unsigned)j)) continue;
                if (r2_f32(s, i, j) >= rc2) continue;
                double r = nrm(disp(s, i, j)), q = r / rc, t = 1.0 - q;
                acc += wend_w(s, r) + wnorm * 20.0 * q * q * t * t * t;
            });
            dscale[i] = acc;
        }
    }
    set_threads(s);
#pragma omp parallel for schedule(dynamic, 256)
    for (long i = 0; i < n; ++i) {
        if (!is_mobile(s, (unsigned)i)) continue;
        double di = s->rho[i] / m;
        /* the size of P_i / d_i^2 for rounding: P = c^2 (rho - rho0) is the
         * difference of two terms of size c^2 rho, and rho is a sum of FP32
         * kernel values, so its rounding error reaches P as c^2 m (its
         * rounding scale) u */
        double ci = is_memb(s, (unsigned)i) ? s->c.SoundSpeed2 : s->c.SoundSpeed1;
        double pi = (fabs(s->press[i]) + (dscale ? ci * ci * m * dscale[i] : 0.0)) / (di * di);
        v3 vi = ld3(s->vel, i);
        double acc = (parts & OR_SCALE_BODY) && s->drive_on ? fabs((double)s->c.ConstExtForce) : 0.0;
        if (!(parts & (OR_SCALE_SDPD | OR_SCALE_REP))) {
            scale[i] = acc;
            continue;
        }
        FOR_CANDIDATES(&b, s, i, j, {
            if (j == i) continue;
            float r2f = r2_f32(s, i, j);
            if (is_b1(s, (unsigned)j)) {
                if (!(parts & OR_SCALE_REP) || r2f >= r0sq || r2f <= 0.f) continue;
                v3 d = disp(s, i, j);
                double r2 = dot(d, d), q2 = r0 * r0 / r2, q4 = q2 * q2, q12 = q4 * q4 * q4;
                /* the term and its sensitivity to r: |d/dr (r f(r))| r <= (12 q^12 + 4 q^4) D / r */
                acc += D * (fabs(q12 - q4) + 12.0 * q12 + 4.0 * q4) / sqrt(r2);
                continue;
            }
            if (!(parts & OR_SCALE_SDPD) || !is_sdpd(s, (unsigned)j) || r2f >= rc2) continue;
            v3 d = disp(s, i, j);
            double r = nrm(d), q = r / rc, t = 1.0 - q;
            double dj = s->rho[j] / m;
            /* Bound2 density is DenInit exactly: its pressure has no rounding */
            double cj = is_memb(s, (unsigned)j) ? s->c.SoundSpeed2 : s->c.SoundSpeed1;
            double pj = (fabs(s->press[j]) + (dscale && is_mobile(s, (unsigned)j) ? cj * cj * m * dscale[j] : 0.0)) /
                        (dj * dj);
            /* F = fnorm (1 - q)^3 with its sensitivity to the rounding of r:
             * |F| + |F'| r = fnorm (1 - q)^2 (1 + 2 q) */
            double Fc = fnorm * t * t * (1.0 + 2.0 * q);
            acc += (pi + pj) * Fc * r;
            if (r <= 0.0) continue;
            v3 vij = sub(vi, ld3(s->vel, j));
            double fddc = Fc / (di * dj);
            acc += fddc * (fabs(A) * nrm(vij) + fabs(B) * nrm(vij));
            if (noise && t > 0.0) {
                double xi[3];
                or_pair_noise(s, (unsigned)i, (unsigned)j, xi);
                v3 x = mk(xi[0], xi[1], xi[2]);
                /* the amplitude sqrt(pref F / (d_i d_j)) ~ (1 - q)^(3/2) with its sensitivity
                 * to the rounding of r: sqrt(pref fnorm (1 - q) / (d_i d_j)) (1 + q/2) */
                double qc = sqrt(pref * fnorm * t / (di * dj)) * (1.0 + 0.5 * q);
                acc += qc * (sA * nrm(x) + fabs(sAB - sA) * nrm(x));
            }
        });
        scale[i] = acc;
    }
    free(dscale);
    bins_free(&b);
    long nc = s->c.nCellStart, ncp = s->c.nCellPar;
    if (s->ncell <= 0) return 0;
    /* membrane terms, each added to its vertices as a magnitude */
    for (int e = 0; e < s->nedge && (parts & OR_SCALE_MEMB); ++e) {
        const int* E = s->edge + 6 * e;
        v3 x1 = unwrapped(s, memb_id(s, E[0]));
        v3 bb = sub(unwrapped(s, memb_id(s, E[1])), x1);
        v3 c = sub(unwrapped(s, memb_id(s, E[2])), x1);
        v3 d = sub(unwrapped(s, memb_id(s, E[3])), x1);
        double r = nrm(bb);
        /* the WLC and POW terms of the spring separately (they cancel at rest) */
        double p = s->perlen[e];
        if (p > 0 && r > 0) {
            double x = r / s->maxrefedgelen[e];
            if (x > 0.99) x = 0.99;
            double u = 1.0 - x;
            double t = fabs((s->c.Temp / p) * (1.0 / (4.0 * u * u) - 0.25 + x)) + fabs(s->hpow[e] / pow(r, OR_POWM));
            scale[nc + E[0] - 1] += t;
            scale[nc + E[1] - 1] += t;
        }
        double kb = s->hbending[e];
        if (kb != 0.0) {
            dih_t Dh = dihedral(c, mk(0, 0, 0), bb, d);
            double dE = fabs(kb) * (fabs(Dh.s) + fabs(Dh.c));
            scale[nc + E[2] - 1] += dE * nrm(Dh.gi);
            scale[nc + E[0] - 1] += dE * nrm(Dh.gj);
            scale[nc + E[1] - 1] += dE * nrm(Dh.gk);
            scale[nc + E[3] - 1] += dE * nrm(Dh.gl);
        }
    }
    for (int c = 0; c < s->ncell && (parts & OR_SCALE_MEMB); ++c) {
        for (int t = s->betri[2 * c]; t <= s->betri[2 * c + 1]; ++t) {
            const int* T = s->tri + 3 * t;
            v3 x1 = unwrapped(s, memb_id(s, T[0]));
            v3 x2 = sub(unwrapped(s, memb_id(s, T[1])), x1);
            v3 x3 = sub(unwrapped(s, memb_id(s, T[2])), x1);
            v3 xi = crs(x2, x3);
            double len = nrm(xi);
            if (!(len > 0)) continue;
            /* each of the area and volume coefficients is a difference of
             * nearly equal terms near rest: their rounding scales with the
             * larger term, k |A| / A0 */
            double cA = fabs(s->hgarea[t]) * s->area[c] / s->refarea[c] + fabs(s->hlarea[t]) * 0.5 * len / s->reftriarea[t];
            double cV = fabs(s->hvol[t]) * fabs(s->vol[c]) / fabs(s->refvol[c]) / 6.0;
            v3 nh = scl(1.0 / len, xi);
            double g[3] = {0.5 * nrm(crs(nh, sub(x3, x2))), 0.5 * nrm(x3), 0.5 * nrm(x2)};
            for (int k = 0; k < 3; ++k) scale[nc + T[k] - 1] += cV * len + cA * g[k];
        }
    }
    if ((parts & OR_SCALE_MORSE) && s->c.surEnergy != 0.f && s->c.MaxCut > 0.f && ncp > 0) {
        bins_t mb;
        if (bins_build(&mb, s, s->c.MaxCut, memb_member)) return -1;
        float mc2 = s->c.MaxCut * s->c.MaxCut;
        double De = s->c.surEnergy, beta = s->c.scaFac, rz = s->c.zeroLen;
#pragma omp parallel for schedule(dynamic, 64)
        for (long v = 0; v < ncp; ++v) {
            long i = nc + v;
            int ci = s->celltab[v];
            double acc = 0.0;
            FOR_CANDIDATES(&mb, s, i, j, {
                long w = j - nc;
                if (s->celltab[w] == ci) continue;
                float r2f = r2_f32(s, i, j);
                if (r2f >= mc2 || r2f <= 0.f) continue;
                double r = nrm(disp(s, i, j)), ex = exp(beta * (rz - r));
                acc += 2.0 * De * fabs(beta) * (ex * ex + ex) * 0.5 * (s->pararea[v] + s->pararea[w]);
            });
            scale[i] += acc;
        }
        bins_free(&mb);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Full step, Particle::UpdatePar order (src/Particle.cu:1310-1329)          */
/* ------------------------------------------------------------------------ */

int or_step(or_state* s) {
    int rc = 0;
    rc |= or_update_coor(s);
    rc |= or_periodic(s);
    rc |= or_density(s);
    rc |= or_predict(s);
    rc |= or_bound2_vel(s);
    rc |= or_eos(s);
    rc |= or_sdpd_force(s);
    rc |= or_rep_force(s);
    rc |= or_ext_force(s);
    if (s->ncell > 0) {
        rc |= or_geo(s, 0);
        rc |= or_def_force(s);
        rc |= or_agg_force(s);
    }
    rc |= or_correct(s);
    rc |= or_bound2_vel(s);
    s->step += 1;
    return rc;
}
