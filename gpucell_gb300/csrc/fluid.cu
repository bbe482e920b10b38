// fluid.cu -- the particle entry points of cupar:: (src/ParticleGPU.cuh:11-21):
// integrator stages, periodic wrap, density, equation of state, the SDPD
// pair force, wall repulsion, body force and the no-slip wall velocity.
//
// These are the reference-structured FP32 kernels behind the drop-in
// boundary: one kernel per entry point, one thread per slot, a 27-cube sweep
// over the caller's begin/end table for every neighbour pass, float3/float4
// arrays in the caller's layout.  Particle type is decided from the original
// id in d_sortpart (src/Particle.cu:432-435).
//
// The formulas (pinned because GPUCell's kernel bodies are absent):
//   density   rho_i = m (W(0) + sum_j W_ij), j over Bound2, fluid, membrane;
//             Bound2 keeps rho = DenInit (src/ParticleGPU.cuh:13 comment)
//   EOS       P_i = c_i^2 (rho_i - rho0), c = SoundSpeed1 (fluid, Bound2) or
//             SoundSpeed2 (membrane)
//   SDPD      Espanol & Revenga (2003), with d = rho/m:
//             f_i = sum_j (P_i/d_i^2 + P_j/d_j^2) F_ij r_ij
//                   - F_ij/(d_i d_j) [A v_ij + B e_ij (e_ij . v_ij)]
//                   + q_ij [sqrt(A) xi_ij + (sqrt(A+B) - sqrt(A)) e_ij (e_ij . xi_ij)]
//             A = 5 eta/3 - zeta, B = 5 (zeta + eta/3),
//             q_ij = sqrt(2 kT F_ij / (d_i d_j dt)), xi_ij the Philox pair noise
//   repulsion Monaghan (1994): f_i += D [(r0/r)^12 - (r0/r)^4] r_ij / r^2 from
//             Bound1 within r0 = rc/3, D = SoundSpeed1^2
//   walls     Adami, Hu & Adams (2012): v_w = 2 v_presc - sum_f v_f W / sum_f W,
//             v_presc = the wall's VelHalf (zero unless the caller sets it)
//   integrator Groot & Warren (1997) modified velocity-Verlet with lambda = VVsigma
#include "gc_internal.cuh"

namespace {

// Visits every slot j in the 27 cubes around cube c (periodic axes wrap,
// wall axes stop at the edge).  Cube counts per periodic axis are >= 3, so
// no cube is visited twice.
template <class Fn>
__device__ __forceinline__ void sweep27(const GcParams& p, int3 c, const int2* __restrict__ bec, Fn&& fn) {
    for (int dz = -1; dz <= 1; ++dz) {
        int z = cube_step(c.z, dz, 2, p.g);
        if (z < 0) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            int y = cube_step(c.y, dy, 1, p.g);
            if (y < 0) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                int x = cube_step(c.x, dx, 0, p.g);
                if (x < 0) continue;
                int2 be = bec[cube_key(x, y, z, p.g)];
                for (int j = be.x; j < be.y; ++j) fn(j);
            }
        }
    }
}

// K2 -- r += dt v + dt^2/2 F/m for fluid and membrane particles.
__global__ void k_update_coor(int n, GcParams p, const int* __restrict__ sortpart, const float3* __restrict__ force,
                              float3* __restrict__ coor, const float4* __restrict__ velrhop, unsigned* flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!is_mobile((unsigned)sortpart[i], p)) return;
    float3 x = coor[i], f = force[i];
    float4 v = velrhop[i];
    float h = 0.5f * p.dt * p.dt * p.inv_mass;
    x.x += p.dt * v.x + h * f.x;
    x.y += p.dt * v.y + h * f.y;
    x.z += p.dt * v.z + h * f.z;
    if (!(isfinite(x.x) && isfinite(x.y) && isfinite(x.z))) raise_flag(flags, GC_FLAG_NONFINITE);
    coor[i] = x;
}

// K3 -- wrap moving particles into the box on periodic axes and count the
// crossings (+1 for a crossing of the upper face) so that membranes can be
// unwrapped as x + nThroBound * L.
__global__ void k_periodic(int n, GcParams p, const int* __restrict__ sortpart, float3* __restrict__ coor,
                           int3* __restrict__ nthro, const float* __restrict__ bbox, unsigned* flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!is_mobile((unsigned)sortpart[i], p)) return;
    float3 x = coor[i];
    int3 t = nthro[i];
    float* xs[3] = {&x.x, &x.y, &x.z};
    int* ts[3] = {&t.x, &t.y, &t.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (!(p.g.pmask & (1 << a))) continue;
        float lo = bbox[2 * a], hi = bbox[2 * a + 1], L = hi - lo;
        float v = *xs[a];
        if (v >= hi) { v -= L; *ts[a] += 1; }
        else if (v < lo) { v += L; *ts[a] -= 1; }
        if (v >= hi || v < lo) raise_flag(flags, GC_FLAG_NONFINITE);
        *xs[a] = v;
    }
    coor[i] = x;
    nthro[i] = t;
}

// K8 -- kernel-sum density of fluid and membrane particles.
__global__ void k_density(int n, GcParams p, const float3* __restrict__ coor, float4* __restrict__ velrhop,
                          const int3* __restrict__ cc, const int* __restrict__ sortpart, const int2* __restrict__ bec) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!is_mobile((unsigned)sortpart[i], p)) return;
    float3 xi = coor[i];
    float sum = p.w0;
    sweep27(p, cc[i], bec, [&](int j) {
        if (j == i) return;
        float3 d = min_image(xi, coor[j], p.g);
        float r2 = norm2_rn(d);
        if (r2 >= p.rc2) return;
        if (!is_sdpd((unsigned)sortpart[j], p)) return;
        sum += wendland_w(sqrtf(r2), p);
    });
    velrhop[i].w = p.mass * sum;
}

// K9 -- predictor: VelHalf = v + dt/2 F/m, v <- v + lambda dt F/m.
__global__ void k_predict(int n, GcParams p, const int* __restrict__ sortpart, float4* __restrict__ velrhop,
                          float3* __restrict__ velhalf, const float3* __restrict__ force) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!is_mobile((unsigned)sortpart[i], p)) return;
    float4 v = velrhop[i];
    float3 f = force[i];
    float h = 0.5f * p.dt * p.inv_mass, l = p.lambda * p.dt * p.inv_mass;
    velhalf[i] = f3(v.x + h * f.x, v.y + h * f.y, v.z + h * f.z);
    v.x += l * f.x;
    v.y += l * f.y;
    v.z += l * f.z;
    velrhop[i] = v;
}

// K10 -- no-slip velocity of Bound2 wall particles.
__global__ void k_bound2vel(int n, GcParams p, const float3* __restrict__ coor, float4* __restrict__ velrhop,
                            const float3* __restrict__ velhalf, const int3* __restrict__ cc,
                            const int* __restrict__ sortpart, const int2* __restrict__ bec) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (ptype((unsigned)sortpart[i], p) != PT_B2) return;
    float3 xi = coor[i];
    float3 num = f3(0.f, 0.f, 0.f);
    float den = 0.f;
    sweep27(p, cc[i], bec, [&](int j) {
        float3 d = min_image(xi, coor[j], p.g);
        float r2 = norm2_rn(d);
        if (r2 >= p.rc2) return;
        if (!is_mobile((unsigned)sortpart[j], p)) return;
        float w = wendland_w(sqrtf(r2), p);
        float4 vj = velrhop[j];
        num += w * f3(vj.x, vj.y, vj.z);
        den += w;
    });
    float3 vw = velhalf ? velhalf[i] : f3(0.f, 0.f, 0.f);
    float4 v = velrhop[i];
    if (den > 0.f) {
        float inv = 1.f / den;
        v.x = 2.f * vw.x - num.x * inv;
        v.y = 2.f * vw.y - num.y * inv;
        v.z = 2.f * vw.z - num.z * inv;
    } else {
        v.x = vw.x; v.y = vw.y; v.z = vw.z;
    }
    velrhop[i] = v;
}

// K11 -- equation of state.
__global__ void k_eos(int n, GcParams p, const int* __restrict__ sortpart, const float4* __restrict__ velrhop,
                      float* __restrict__ press) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int t = ptype((unsigned)sortpart[i], p);
    float rho = velrhop[i].w;
    float P = 0.f;
    if (t == PT_MEMB) P = p.c2sq * (rho - p.rho0);
    else if (t != PT_B1) P = p.c1sq * (rho - p.rho0);
    press[i] = P;
}

// K12 -- SDPD pair force; writes the force of every slot (zero for walls).
__global__ void k_sdpd(int n, GcParams p, const float3* __restrict__ coor, const float4* __restrict__ velrhop,
                       const int3* __restrict__ cc, const int* __restrict__ sortpart, const int2* __restrict__ bec,
                       float3* __restrict__ force, const float* __restrict__ press) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned id = (unsigned)sortpart[i];
    if (!is_mobile(id, p)) {
        force[i] = f3(0.f, 0.f, 0.f);
        return;
    }
    float3 xi = coor[i];
    float4 vi = velrhop[i];
    float di = vi.w * p.inv_mass;
    float pi_term = press[i] / (di * di);
    bool noise = p.noise_pref > 0.f;
    float3 f = f3(0.f, 0.f, 0.f);
    sweep27(p, cc[i], bec, [&](int j) {
        if (j == i) return;
        float3 d = min_image(xi, coor[j], p.g);
        float r2 = norm2_rn(d);
        if (r2 >= p.rc2) return;
        unsigned idj = (unsigned)sortpart[j];
        if (!is_sdpd(idj, p)) return;
        float r = sqrtf(r2);
        float F = wendland_f(r, p);
        float4 vj = velrhop[j];
        float dj = vj.w * p.inv_mass;
        float cons = (pi_term + press[j] / (dj * dj)) * F;
        f += cons * d;
        if (r2 <= 0.f) return;
        float inv_r = 1.f / r;
        float3 e = inv_r * d;
        float3 vij = f3(vi.x - vj.x, vi.y - vj.y, vi.z - vj.z);
        float ev = dot3(e, vij);
        float fdd = F / (di * dj);
        f -= fdd * (p.visA * vij + (p.visB * ev) * e);
        if (noise) {
            // a pair at the cut-off can give F a rounding-sized negative value: no noise then
            float q = fdd > 0.f ? sqrtf(p.noise_pref * fdd) : 0.f;
            float3 xi_ = pair_noise(id, idj, p);
            float exi = dot3(e, xi_);
            f += q * (p.sqrtA * xi_ + ((p.sqrtAB - p.sqrtA) * exi) * e);
        }
    });
    force[i] = f;
}

// K13 -- repulsion of fluid and membrane particles by Bound1 walls.
__global__ void k_repulsion(int n, GcParams p, const float3* __restrict__ coor, const int3* __restrict__ cc,
                            const int* __restrict__ sortpart, const int2* __restrict__ bec,
                            float3* __restrict__ force) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!is_mobile((unsigned)sortpart[i], p)) return;
    float3 xi = coor[i];
    float3 f = f3(0.f, 0.f, 0.f);
    bool any = false;
    sweep27(p, cc[i], bec, [&](int j) {
        float3 d = min_image(xi, coor[j], p.g);
        float r2 = norm2_rn(d);
        if (r2 >= p.rep_r0sq || r2 <= 0.f) return;
        if (ptype((unsigned)sortpart[j], p) != PT_B1) return;
        float q2 = p.rep_r0sq / r2;
        float q4 = q2 * q2;
        float q12 = q4 * q4 * q4;
        f += (p.rep_D * (q12 - q4) / r2) * d;
        any = true;
    });
    if (any) {
        float3 t = force[i];
        force[i] = t + f;
    }
}

// K14 -- body force in x on fluid and membrane particles.
__global__ void k_ext(int n, GcParams p, const int* __restrict__ sortpart, float3* __restrict__ force) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!is_mobile((unsigned)sortpart[i], p)) return;
    force[i].x += p.gx;
}

// K19 -- corrector: v = VelHalf + dt/2 F/m.
__global__ void k_correct(int n, GcParams p, const int* __restrict__ sortpart, const float3* __restrict__ force,
                          const float3* __restrict__ velhalf, float4* __restrict__ velrhop, unsigned* flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!is_mobile((unsigned)sortpart[i], p)) return;
    float3 f = force[i], h = velhalf[i];
    float4 v = velrhop[i];
    float s = 0.5f * p.dt * p.inv_mass;
    v.x = h.x + s * f.x;
    v.y = h.y + s * f.y;
    v.z = h.z + s * f.z;
    if (!(isfinite(v.x) && isfinite(v.y) && isfinite(v.z))) raise_flag(flags, GC_FLAG_NONFINITE);
    velrhop[i] = v;
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void k_nbstats(int n, GcParams p, const float3* __restrict__ coor, const int* __restrict__ sortpart,
                          const int2* __restrict__ bec, int* __restrict__ count, unsigned long long* __restrict__ hash) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 xi = coor[i];
    int3 c = make_int3(cube_coord(xi.x, 0, p.g), cube_coord(xi.y, 1, p.g), cube_coord(xi.z, 2, p.g));
    int cnt = 0;
    unsigned long long h = 0;
    sweep27(p, c, bec, [&](int j) {
        if (j == i) return;
        float3 d = min_image(xi, coor[j], p.g);
        if (norm2_rn(d) >= p.rc2) return;
        ++cnt;
        h += mix64((unsigned long long)(unsigned)sortpart[j]);
    });
    count[i] = cnt;
    hash[i] = h;
}

}  // namespace

#define GC_PRE(name, need_grid)                                            \
    GcState& s = gc_state();                                               \
    if (n < 0) return gc_fail(GC_EINVAL, name ": n < 0");                  \
    GcParams p;                                                            \
    GC_TRY(gc_make_params(&p, need_grid));                                 \
    if ((unsigned)n != p.nT)                                               \
        return gc_fail(GC_EINVAL, name ": n = %d but nTotalPar = %u", n, p.nT); \
    if (n == 0) return GC_OK;                                              \
    const int nb = gc_blocks(n, SDPDSIZE);                                 \
    (void)nb

extern "C" {

int gc_cupar_UpdateFluidCoor(int n, int* d_sortpart, float* d_totalforce, float* d_totalcoor, float* d_velrhop) {
    GcState& s0 = gc_state();
    s0.ref.sortpart = d_sortpart;
    s0.ref.force = d_totalforce;
    s0.ref.coor = d_totalcoor;
    s0.ref.velrhop = d_velrhop;
    s0.step += 1;   // first call of every step (src/Particle.cu:1312)
    // With the fused engine, every step after the first is run whole at
    // SetFluidExtForce (which carries DriveOn); the other calls of the step
    // only record their buffers.
    s0.in_fused_step = s0.engine_mode == 1 && s0.plain_steps >= 1;
    if (s0.in_fused_step) return GC_OK;
    s0.plain_steps += 1;
    GC_PRE("UpdateFluidCoor", false);
    k_update_coor<<<nb, SDPDSIZE, 0, s.stream>>>(n, p, d_sortpart, (const float3*)d_totalforce, (float3*)d_totalcoor,
                                                (const float4*)d_velrhop, gc_flags_ptr());
    GC_CHECK_LAUNCH("UpdateFluidCoor");
    return GC_OK;
}

int gc_cupar_AppFluidPeriodicBC(int n, int* d_sortpart, float* d_totalcoor, int* d_nthrobound, float* d_bboxsdpd) {
    gc_state().ref.nthro = d_nthrobound;
    gc_state().ref.bbox = d_bboxsdpd;
    if (gc_state().in_fused_step) return GC_OK;
    GC_PRE("AppFluidPeriodicBC", false);
    p.g.pmask = s.periodic_mask;
    k_periodic<<<nb, SDPDSIZE, 0, s.stream>>>(n, p, d_sortpart, (float3*)d_totalcoor, (int3*)d_nthrobound, d_bboxsdpd,
                                             gc_flags_ptr());
    GC_CHECK_LAUNCH("AppFluidPeriodicBC");
    return GC_OK;
}

int gc_cupar_CalFluidDen(int n, float* d_totalcoor, float* d_velrhop, int* d_cc, int* d_ncube, float* d_outerregion,
                         int* d_sortpart, int* d_beginendcube) {
    if (gc_state().in_fused_step) return GC_OK;
    (void)d_ncube; (void)d_outerregion;
    GC_PRE("CalFluidDen", true);
    k_density<<<nb, SDPDSIZE, 0, s.stream>>>(n, p, (const float3*)d_totalcoor, (float4*)d_velrhop, (const int3*)d_cc,
                                            d_sortpart, (const int2*)d_beginendcube);
    GC_CHECK_LAUNCH("CalFluidDen");
    return GC_OK;
}

int gc_cupar_PredictFluidVel(int n, int* d_sortpart, float* d_velrhop, float* d_velhalf, float* d_totalforce) {
    gc_state().ref.velhalf = d_velhalf;
    if (gc_state().in_fused_step) return GC_OK;
    GC_PRE("PredictFluidVel", false);
    s.velhalf_ptr = d_velhalf;
    k_predict<<<nb, SDPDSIZE, 0, s.stream>>>(n, p, d_sortpart, (float4*)d_velrhop, (float3*)d_velhalf,
                                            (const float3*)d_totalforce);
    GC_CHECK_LAUNCH("PredictFluidVel");
    return GC_OK;
}

int gc_cupar_CalBound2Vel(int n, float* d_totalcoor, float* d_velrhop, int* d_cc, int* d_ncube, float* d_outerregion,
                          int* d_sortpart, int* d_beginendcube) {
    if (gc_state().in_fused_step) return GC_OK;
    (void)d_ncube; (void)d_outerregion;
    GC_PRE("CalBound2Vel", true);
    if (p.nF == p.nB2) return GC_OK;   // no Bound2 particles
    // The prescribed wall velocity lives in the wall's VelHalf, which the
    // reference sets to zero (src/Particle.cu:513-515).  The reference passes
    // no VelHalf here, so it is taken from the pointer the caller gave to
    // the latest PredictFluidVel / CorrectFliudVel (both precede every
    // CalBound2Vel in src/Particle.cu:1316-1327); without one the walls are
    // at rest.
    k_bound2vel<<<nb, SDPDSIZE, 0, s.stream>>>(n, p, (const float3*)d_totalcoor, (float4*)d_velrhop,
                                              (const float3*)s.velhalf_ptr, (const int3*)d_cc, d_sortpart,
                                              (const int2*)d_beginendcube);
    GC_CHECK_LAUNCH("CalBound2Vel");
    return GC_OK;
}

int gc_cupar_EOS(int n, int* d_sortpart, float* d_velrhop, float* d_press) {
    gc_state().ref.press = d_press;
    if (gc_state().in_fused_step) return GC_OK;
    GC_PRE("EOS", false);
    k_eos<<<nb, SDPDSIZE, 0, s.stream>>>(n, p, d_sortpart, (const float4*)d_velrhop, d_press);
    GC_CHECK_LAUNCH("EOS");
    return GC_OK;
}

int gc_cupar_CalFluidSDPDForce(int n, float* h_sdpdforce, float* d_totalcoor, float* d_velrhop, int* d_cc,
                               int* d_ncube, int* d_sortpart, float* d_outerregion, int* d_beginendcube,
                               float* d_totalforce, float* d_press) {
    if (gc_state().in_fused_step) return GC_OK;
    (void)h_sdpdforce; (void)d_ncube; (void)d_outerregion;
    GC_PRE("CalFluidSDPDForce", true);
    k_sdpd<<<nb, SDPDSIZE, 0, s.stream>>>(n, p, (const float3*)d_totalcoor, (const float4*)d_velrhop,
                                         (const int3*)d_cc, d_sortpart, (const int2*)d_beginendcube,
                                         (float3*)d_totalforce, d_press);
    GC_CHECK_LAUNCH("CalFluidSDPDForce");
    return GC_OK;
}

int gc_cupar_CalFluidRepForce(int n, float* d_totalcoor, int* d_cc, int* d_ncube, int* d_sortpart,
                              float* d_outerregion, int* d_beginendcube, float* d_totalforce) {
    if (gc_state().in_fused_step) return GC_OK;
    (void)d_ncube; (void)d_outerregion;
    GC_PRE("CalFluidRepForce", true);
    if (p.nB2 == 0) return GC_OK;   // no Bound1 particles
    k_repulsion<<<nb, SDPDSIZE, 0, s.stream>>>(n, p, (const float3*)d_totalcoor, (const int3*)d_cc, d_sortpart,
                                              (const int2*)d_beginendcube, (float3*)d_totalforce);
    GC_CHECK_LAUNCH("CalFluidRepForce");
    return GC_OK;
}

int gc_cupar_SetFluidExtForce(int driveon, int n, int* d_sortpart, float* d_totalforce) {
    if (gc_state().in_fused_step) return gc_engine_step(driveon);
    GC_PRE("SetFluidExtForce", false);
    if (!driveon || p.gx == 0.f) return GC_OK;
    k_ext<<<nb, SDPDSIZE, 0, s.stream>>>(n, p, d_sortpart, (float3*)d_totalforce);
    GC_CHECK_LAUNCH("SetFluidExtForce");
    return GC_OK;
}

int gc_cupar_CorrectFliudVel(int n, int* d_sortpart, float* d_totalforce, float* d_velhalf, float* d_velrhop,
                             float* d_totalcoor, int* d_cc, int* d_ncube, float* d_outerregion, int* d_beginendcube) {
    gc_state().ref.velhalf = d_velhalf;
    if (gc_state().in_fused_step) return GC_OK;
    (void)d_totalcoor; (void)d_cc; (void)d_ncube; (void)d_outerregion; (void)d_beginendcube;
    GC_PRE("CorrectFliudVel", false);
    s.velhalf_ptr = d_velhalf;
    k_correct<<<nb, SDPDSIZE, 0, s.stream>>>(n, p, d_sortpart, (const float3*)d_totalforce, (const float3*)d_velhalf,
                                            (float4*)d_velrhop, gc_flags_ptr());
    GC_CHECK_LAUNCH("CorrectFliudVel");
    return GC_OK;
}

int gc_debug_neighbor_stats(int n, float* d_totalcoor, int* d_sortpart, int* d_beginendcube, int* d_count,
                            unsigned long long* d_hash) {
    GC_PRE("debug_neighbor_stats", true);
    k_nbstats<<<nb, SDPDSIZE, 0, s.stream>>>(n, p, (const float3*)d_totalcoor, d_sortpart,
                                            (const int2*)d_beginendcube, d_count, d_hash);
    GC_CHECK_LAUNCH("debug_neighbor_stats");
    return GC_OK;
}

}  // extern "C"

