// membrane.cu -- the cell-membrane entry points of cupar::
// (src/ParticleGPU.cuh:25-35): geometry and per-cell area/volume (K15),
// per-edge mechanical parameters (K16), the deformation force (K17) and the
// Morse aggregation force between cells (K18).
//
// Topology conventions (src/Particle.cu:174-303): d_tri holds 1-based global
// membrane-vertex indices (global particle id = nCellStart + index - 1); an
// edge record is (p1, p2, p3, p4, t1, t2) with the shared edge p1-p2 and the
// opposite vertices p3 (in t1) and p4 (in t2), all 1-based; d_beginendtri
// holds each cell's first and last triangle (inclusive).  Membrane-only
// arrays (d_celltab, d_defforce, d_aggforce, d_pararea) are in original
// membrane order; particle arrays are in slot order, reached via d_curpos.
//
// Membrane model (Fedosov, Caswell & Karniadakis 2010):
//   WLC + POW spring per edge, x = l/l_max, x0 = l0/l_max = 1/2.2, m = 2:
//     f(l) = -(kT/p) [1/(4(1-x)^2) - 1/4 + x] + k_p / l^m   (along the edge)
//     p and k_p from the shear modulus mu0 and l0 (zero force at l0)
//   bending per edge: E = k_b [1 - cos(phi - phi0)], k_b = 2 kappa / sqrt(3),
//     phi the dihedral angle, phi0 its value at set-up
//   local area per triangle: k_d (A_t - A0_t)^2 / (2 A0_t)
//   global area and volume per cell: k_a (A - A0)^2/(2 A0), k_v (V - V0)^2/(2 V0)
// Aggregation (Morse), between vertices of different cells within MaxCut:
//   f_ij = 2 De beta [e^{2 beta (r0 - r)} - e^{beta (r0 - r)}] (a_i + a_j)/2 e_ij,
//   De = surEnergy (an energy per area), a = per-vertex area (ParArea).
#include "gc_internal.cuh"

#include <math.h>

namespace {

constexpr int kGeoBS = 256;

// Unwrapped difference x_k - x_r of two particles: (x_k - x_r) + (t_k - t_r) L
// on periodic axes, t the crossing counts.
__device__ __forceinline__ float3 unwrap_diff(float3 xk, int3 tk, float3 xr, int3 tr, const float L[3], int pmask) {
    float3 d = xk - xr;
    if (pmask & 1) d.x += (float)(tk.x - tr.x) * L[0];
    if (pmask & 2) d.y += (float)(tk.y - tr.y) * L[1];
    if (pmask & 4) d.z += (float)(tk.z - tr.z) * L[2];
    return d;
}

__device__ __forceinline__ bool memb_ok(int v1, const GcParams& p) { return v1 >= 1 && v1 <= (int)p.nCP; }

__device__ float block_sum(float v, float* sh) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    float t = 0.f;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.f;
#pragma unroll
        for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) sh[0] = t;
    }
    __syncthreads();
    t = sh[0];
    __syncthreads();
    return t;
}

// K15: one block per cell.  Per triangle: unit normal, area, unwrapped
// centroid; per cell: area and volume (volume by the divergence theorem
// relative to the cell's first vertex), copied to every triangle of the
// cell; at set-up also the reference values.  Per vertex: one third of the
// area of each incident triangle (d_pararea, cleared by the caller).
__global__ void k_geo_cell(GcParams p, int ncell, int ntri, const float* __restrict__ bbox, const int* __restrict__ curpos,
                           const int3* __restrict__ tri, const int2* __restrict__ betri,
                           const int3* __restrict__ nthro, const float3* __restrict__ coor,
                           float3* __restrict__ trinordir, float* __restrict__ triarea,
                           float* __restrict__ reftriarea, float3* __restrict__ tricenter,
                           float* __restrict__ refarea_para, float* __restrict__ refvol_para,
                           float* __restrict__ area_para, float* __restrict__ vol_para, float* __restrict__ area,
                           float* __restrict__ vol, float* __restrict__ pararea, int setup, unsigned* flags) {
    __shared__ float sh[32];
    int c = blockIdx.x;
    if (c >= ncell) return;
    int2 be = betri[c];
    if (be.x < 0 || be.y >= ntri || be.y < be.x) {
        if (threadIdx.x == 0) raise_flag(flags, GC_FLAG_BAD_INDEX);
        return;
    }
    float L[3] = {bbox[1] - bbox[0], bbox[3] - bbox[2], bbox[5] - bbox[4]};
    int pm = p.g.pmask;
    int vr = tri[be.x].x;
    if (!memb_ok(vr, p)) {
        if (threadIdx.x == 0) raise_flag(flags, GC_FLAG_BAD_INDEX);
        return;
    }
    int sr = curpos[p.nC + vr - 1];
    float3 xr = coor[sr];
    int3 tr = nthro ? nthro[sr] : make_int3(0, 0, 0);
    float accA = 0.f, accV = 0.f;
    for (int t = be.x + threadIdx.x; t <= be.y; t += blockDim.x) {
        int3 v = tri[t];
        if (!memb_ok(v.x, p) || !memb_ok(v.y, p) || !memb_ok(v.z, p)) {
            raise_flag(flags, GC_FLAG_BAD_INDEX);
            continue;
        }
        int s1 = curpos[p.nC + v.x - 1], s2 = curpos[p.nC + v.y - 1], s3 = curpos[p.nC + v.z - 1];
        float3 x1 = coor[s1], x2 = coor[s2], x3 = coor[s3];
        int3 t1 = nthro ? nthro[s1] : tr;
        float3 a = unwrap_diff(x1, t1, xr, tr, L, pm);
        float3 e1 = min_image(x2, x1, p.g), e2 = min_image(x3, x1, p.g);
        float3 xi = cross3(e1, e2);
        float len = sqrtf(dot3(xi, xi));
        float A = 0.5f * len;
        float3 nrm = len > 0.f ? (1.f / len) * xi : f3(0.f, 0.f, 0.f);
        float3 b = a + e1, cc3 = a + e2;
        float3 xru = xr;
        if (pm & 1) xru.x += (float)tr.x * L[0];
        if (pm & 2) xru.y += (float)tr.y * L[1];
        if (pm & 4) xru.z += (float)tr.z * L[2];
        trinordir[t] = nrm;
        triarea[t] = A;
        tricenter[t] = xru + (1.f / 3.f) * (a + b + cc3);
        if (setup) reftriarea[t] = A;
        accA += A;
        accV += dot3(a, cross3(b, cc3)) * (1.f / 6.f);
        float a3 = A * (1.f / 3.f);
        atomicAdd(&pararea[v.x - 1], a3);
        atomicAdd(&pararea[v.y - 1], a3);
        atomicAdd(&pararea[v.z - 1], a3);
    }
    float Ac = block_sum(accA, sh);
    float Vc = block_sum(accV, sh);
    if (threadIdx.x == 0) {
        area[c] = Ac;
        vol[c] = Vc;
    }
    for (int t = be.x + threadIdx.x; t <= be.y; t += blockDim.x) {
        area_para[t] = Ac;
        vol_para[t] = Vc;
        if (setup) {
            refarea_para[t] = Ac;
            refvol_para[t] = Vc;
        }
    }
}

// Dihedral angle of (i, j, k, l) in the convention of the GROMACS manual
// (angle between planes ijk and jkl, signed by r_ij . (r_kj x r_kl)), and
// its gradient.  Positions are relative to any common origin.
struct Dihedral {
    float phi_cos, phi_sin;
    float3 gi, gj, gk, gl;   // d phi / d x
};

__device__ __forceinline__ Dihedral dihedral(float3 xi, float3 xj, float3 xk, float3 xl) {
    Dihedral D;
    float3 rij = xi - xj, rkj = xk - xj, rkl = xk - xl;
    float3 m = cross3(rij, rkj), n = cross3(rkj, rkl);
    float m2 = dot3(m, m), n2 = dot3(n, n), kj2 = dot3(rkj, rkj);
    float kj = sqrtf(kj2);
    float mn = sqrtf(m2 * n2);
    float inv = mn > 0.f ? 1.f / mn : 0.f;
    D.phi_cos = dot3(m, n) * inv;
    D.phi_sin = dot3(m, rkl) * kj * inv;
    float im2 = m2 > 0.f ? 1.f / m2 : 0.f, in2 = n2 > 0.f ? 1.f / n2 : 0.f;
    D.gi = (kj * im2) * m;
    D.gl = -(kj * in2) * n;
    float ikj2 = kj2 > 0.f ? 1.f / kj2 : 0.f;
    float a = dot3(rij, rkj) * ikj2, b = dot3(rkl, rkj) * ikj2;
    D.gj = (a - 1.f) * D.gi - b * D.gl;
    D.gk = (b - 1.f) * D.gl - a * D.gi;
    return D;
}

// K16: per-edge reference length, WLC/POW and bending coefficients, and the
// reference dihedral angle.
__global__ void k_mech_setup(GcParams p, int nedge, const int6* __restrict__ edge, const int* __restrict__ curpos,
                             float* __restrict__ refedgelen, float* __restrict__ maxrefedgelen,
                             const float* __restrict__ bendmod, const float* __restrict__ shearmod,
                             float* __restrict__ hbending, float* __restrict__ powerindex, float* __restrict__ perlen,
                             float* __restrict__ hpow, float* __restrict__ refangle, const float3* __restrict__ coor,
                             unsigned* flags) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nedge) return;
    int6 E = edge[e];
    if (!memb_ok(E.x, p) || !memb_ok(E.y, p) || !memb_ok(E.z, p) || !memb_ok(E.k, p)) {
        raise_flag(flags, GC_FLAG_BAD_INDEX);
        return;
    }
    float3 x1 = coor[curpos[p.nC + E.x - 1]];
    float3 b = min_image(coor[curpos[p.nC + E.y - 1]], x1, p.g);
    float3 c = min_image(coor[curpos[p.nC + E.z - 1]], x1, p.g);
    float3 d = min_image(coor[curpos[p.nC + E.k - 1]], x1, p.g);
    float l0 = sqrtf(dot3(b, b));
    const float x0 = 1.f / 2.2f, m = 2.f;
    float u = 1.f - x0;
    float kwlc = 1.f / (4.f * u * u) - 0.25f + x0;               // f_WLC(x0) / (kT/p)
    float kmod = x0 / (2.f * u * u * u) - 1.f / (4.f * u * u) + 0.25f;
    float C = 1.7320508075688772f / (4.f * l0) * (kmod + (m + 1.f) * kwlc);   // mu0 = (kT/p) C
    float mu0 = shearmod[e];
    float pl = (mu0 > 0.f && p.kT > 0.f) ? p.kT * C / mu0 : 0.f;
    float kp = pl > 0.f ? (p.kT / pl) * l0 * l0 * kwlc : 0.f;
    refedgelen[e] = l0;
    maxrefedgelen[e] = l0 / x0;
    powerindex[e] = m;
    perlen[e] = pl;
    hpow[e] = kp;
    hbending[e] = 2.f * bendmod[e] / 1.7320508075688772f;
    Dihedral D = dihedral(c, f3(0.f, 0.f, 0.f), b, d);
    refangle[e] = atan2f(D.phi_sin, D.phi_cos);
}

// K17 part 1: spring and bending forces per edge, scattered to d_defforce.
__global__ void k_edge_force(GcParams p, int nedge, const int6* __restrict__ edge, const int* __restrict__ curpos,
                             const float3* __restrict__ coor, const float* __restrict__ maxlen,
                             const float* __restrict__ powerindex, const float* __restrict__ perlen,
                             const float* __restrict__ hpow, const float* __restrict__ refangle,
                             const float* __restrict__ hbending, float3* __restrict__ defforce, unsigned* flags) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nedge) return;
    int6 E = edge[e];
    if (!memb_ok(E.x, p) || !memb_ok(E.y, p) || !memb_ok(E.z, p) || !memb_ok(E.k, p)) {
        raise_flag(flags, GC_FLAG_BAD_INDEX);
        return;
    }
    float3 x1 = coor[curpos[p.nC + E.x - 1]];
    float3 b = min_image(coor[curpos[p.nC + E.y - 1]], x1, p.g);
    float3 c = min_image(coor[curpos[p.nC + E.z - 1]], x1, p.g);
    float3 d = min_image(coor[curpos[p.nC + E.k - 1]], x1, p.g);
    float3 z = f3(0.f, 0.f, 0.f);
    float3 f1 = z, f2 = z, f3v = z, f4 = z;
    // WLC + POW spring along p1-p2
    float pl = perlen[e];
    float r = sqrtf(dot3(b, b));
    if (pl > 0.f && r > 0.f) {
        float x = r / maxlen[e];
        if (x >= 0.99f) {
            raise_flag(flags, GC_FLAG_STRETCH);
            x = 0.99f;
        }
        float u = 1.f - x;
        float fm = -(p.kT / pl) * (1.f / (4.f * u * u) - 0.25f + x) + hpow[e] * powf(r, -powerindex[e]);
        float3 eh = (-1.f / r) * b;   // unit vector from p2 to p1
        f1 += fm * eh;
        f2 -= fm * eh;
    }
    // dihedral bending on (p3, p1, p2, p4)
    float kb = hbending[e];
    if (kb != 0.f) {
        Dihedral D = dihedral(c, z, b, d);
        float s0, c0;
        sincosf(refangle[e], &s0, &c0);
        float dEdphi = kb * (D.phi_sin * c0 - D.phi_cos * s0);   // k_b sin(phi - phi0)
        f3v -= dEdphi * D.gi;
        f1 -= dEdphi * D.gj;
        f2 -= dEdphi * D.gk;
        f4 -= dEdphi * D.gl;
    }
    float3* o1 = &defforce[E.x - 1];
    float3* o2 = &defforce[E.y - 1];
    float3* o3 = &defforce[E.z - 1];
    float3* o4 = &defforce[E.k - 1];
    atomicAdd(&o1->x, f1.x); atomicAdd(&o1->y, f1.y); atomicAdd(&o1->z, f1.z);
    atomicAdd(&o2->x, f2.x); atomicAdd(&o2->y, f2.y); atomicAdd(&o2->z, f2.z);
    atomicAdd(&o3->x, f3v.x); atomicAdd(&o3->y, f3v.y); atomicAdd(&o3->z, f3v.z);
    atomicAdd(&o4->x, f4.x); atomicAdd(&o4->y, f4.y); atomicAdd(&o4->z, f4.z);
}

// K17 part 2: local-area, global-area and volume forces per triangle.
__global__ void k_tri_force(GcParams p, int ntri, const int3* __restrict__ tri, const int* __restrict__ curpos,
                            const float3* __restrict__ coor, const float* __restrict__ reftriarea,
                            const float* __restrict__ hlarea, const float* __restrict__ hgarea,
                            const float* __restrict__ area_para, const float* __restrict__ refarea_para,
                            const float* __restrict__ hvol, const float* __restrict__ vol_para,
                            const float* __restrict__ refvol_para, float3* __restrict__ defforce, unsigned* flags) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    int3 v = tri[t];
    if (!memb_ok(v.x, p) || !memb_ok(v.y, p) || !memb_ok(v.z, p)) {
        raise_flag(flags, GC_FLAG_BAD_INDEX);
        return;
    }
    float3 x1 = coor[curpos[p.nC + v.x - 1]];
    float3 x2 = min_image(coor[curpos[p.nC + v.y - 1]], x1, p.g);
    float3 x3 = min_image(coor[curpos[p.nC + v.z - 1]], x1, p.g);
    float3 xi = cross3(x2, x3);
    float len = sqrtf(dot3(xi, xi));
    if (!(len > 0.f)) return;
    float At = 0.5f * len;
    float3 nh = (1.f / len) * xi;
    float A0t = reftriarea[t], A0 = refarea_para[t], V0 = refvol_para[t];
    float cA = hgarea[t] * (area_para[t] - A0) / A0 + hlarea[t] * (At - A0t) / A0t;
    float cV = hvol[t] * (vol_para[t] - V0) / V0 * (1.f / 6.f);
    // dA/dx1 = n x (x3 - x2)/2, dA/dx2 = n x (x1 - x3)/2, dA/dx3 = n x (x2 - x1)/2
    // dV/dxk = xi/6 for each vertex (the cell's closed-surface sum is exact)
    float3 g1 = 0.5f * cross3(nh, x3 - x2), g2 = 0.5f * cross3(nh, -x3), g3 = 0.5f * cross3(nh, x2);
    float3 fv = -cV * xi;
    float3 f1 = fv - cA * g1, f2 = fv - cA * g2, f3v = fv - cA * g3;
    float3* o1 = &defforce[v.x - 1];
    float3* o2 = &defforce[v.y - 1];
    float3* o3 = &defforce[v.z - 1];
    atomicAdd(&o1->x, f1.x); atomicAdd(&o1->y, f1.y); atomicAdd(&o1->z, f1.z);
    atomicAdd(&o2->x, f2.x); atomicAdd(&o2->y, f2.y); atomicAdd(&o2->z, f2.z);
    atomicAdd(&o3->x, f3v.x); atomicAdd(&o3->y, f3v.y); atomicAdd(&o3->z, f3v.z);
}

// K17 part 3: add the membrane force of every vertex to its slot.
__global__ void k_def_apply(GcParams p, const float3* __restrict__ defforce, const int* __restrict__ curpos,
                            float3* __restrict__ force) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= (int)p.nCP) return;
    int s = curpos[p.nC + v];
    float3 f = force[s];
    force[s] = f + defforce[v];
}

// K18: Morse aggregation.  One thread per slot (the entry point receives
// no id -> slot map); membrane slots sweep the cubes within MaxCut on the
// main grid.
__global__ void k_aggregate(int n, GcParams p, int R0, int R1, int R2, const float3* __restrict__ coor,
                            const int3* __restrict__ cc, const int* __restrict__ sortpart,
                            const int* __restrict__ celltab, const int2* __restrict__ bec,
                            const float* __restrict__ pararea, float3* __restrict__ aggforce,
                            float3* __restrict__ force) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    unsigned id = (unsigned)sortpart[s];
    if (id < p.nC) return;
    int v = (int)(id - p.nC);
    float3 xi = coor[s];
    int3 c = cc[s];
    int ci = celltab[v];
    float ai = pararea[v];
    float3 f = f3(0.f, 0.f, 0.f);
    for (int dz = -R2; dz <= R2; ++dz) {
        int zz = cube_step(c.z, dz, 2, p.g);
        if (zz < 0) continue;
        for (int dy = -R1; dy <= R1; ++dy) {
            int yy = cube_step(c.y, dy, 1, p.g);
            if (yy < 0) continue;
            for (int dx = -R0; dx <= R0; ++dx) {
                int xx = cube_step(c.x, dx, 0, p.g);
                if (xx < 0) continue;
                int2 be = bec[cube_key(xx, yy, zz, p.g)];
                for (int j = be.x; j < be.y; ++j) {
                    unsigned idj = (unsigned)sortpart[j];
                    if (idj < p.nC) continue;
                    int w = (int)(idj - p.nC);
                    if (celltab[w] == ci) continue;
                    float3 d = min_image(xi, coor[j], p.g);
                    float r2 = norm2_rn(d);
                    if (r2 >= p.maxcut2 || r2 <= 0.f) continue;
                    float r = sqrtf(r2);
                    float ex = __expf(p.beta * (p.r0m - r));
                    float fm = 2.f * p.De * p.beta * (ex * ex - ex) * 0.5f * (ai + pararea[w]);
                    f += (fm / r) * d;
                }
            }
        }
    }
    aggforce[v] = f;
    float3 t = force[s];
    force[s] = t + f;
}

}  // namespace

extern "C" {

int gc_cupar_CalGeoPara(long stepcount, int ntri, int ncell, float* d_bbox, int* d_curpos, int* d_tri,
                        int* d_beginendtri, int* d_nthrobound, float* d_totalcoor, float* d_trinordir,
                        float* d_triarea, float* d_reftriarea, float* d_tricenter, float* d_refarea_para,
                        float* d_refvol_para, float* d_area_para, float* d_vol_para, float* d_area, float* d_vol,
                        float* d_pararea) {
    {
        GcRefPtrs& r = gc_state().ref;
        r.ncell = ncell; r.ntri = ntri; r.curpos = d_curpos; r.tri = d_tri; r.betri = d_beginendtri;
        r.nthro = d_nthrobound; r.coor = d_totalcoor; r.trinordir = d_trinordir; r.triarea = d_triarea;
        r.reftriarea = d_reftriarea; r.tricenter = d_tricenter; r.refarea_para = d_refarea_para;
        r.refvol_para = d_refvol_para; r.area_para = d_area_para; r.vol_para = d_vol_para; r.area = d_area;
        r.vol = d_vol; r.pararea = d_pararea; r.bbox = d_bbox;
    }
    if (gc_state().in_fused_step) return GC_OK;
    GcState& s = gc_state();
    if (ncell < 0 || ntri < 0) return gc_fail(GC_EINVAL, "CalGeoPara: negative sizes");
    if (ncell == 0) return GC_OK;   // the reference calls it with nCell = 0 too (src/Particle.cu:476)
    GcParams p;
    GC_TRY(gc_make_params(&p, true));
    if (p.nCP == 0) return gc_fail(GC_EINVAL, "CalGeoPara: cells but nCellPar = 0");
    GC_CUDA(cudaMemsetAsync(d_pararea, 0, (size_t)p.nCP * sizeof(float), s.stream), "CalGeoPara: clear ParArea");
    k_geo_cell<<<ncell, kGeoBS, 0, s.stream>>>(
        p, ncell, ntri, d_bbox, d_curpos, (const int3*)d_tri, (const int2*)d_beginendtri, (const int3*)d_nthrobound,
        (const float3*)d_totalcoor, (float3*)d_trinordir, d_triarea, d_reftriarea, (float3*)d_tricenter,
        d_refarea_para, d_refvol_para, d_area_para, d_vol_para, d_area, d_vol, d_pararea, stepcount < 0 ? 1 : 0,
        gc_flags_ptr());
    GC_CHECK_LAUNCH("CalGeoPara");
    return GC_OK;
}

int gc_cupar_SetMechPara(int ncell, int nedge, int* d_edge, int* d_curpos, float* d_refedgelen,
                         float* d_maxrefedgelen, float* d_bendmodpara, float* d_shearmodpara, float* d_hbending,
                         float* d_powerindex, float* d_perlenWLC, float* d_hpow, float* d_reftriangle,
                         float* d_trinordir, float* d_tricenter, float* d_coor) {
    {
        GcRefPtrs& r = gc_state().ref;
        r.nedge = nedge; r.edge = d_edge; r.refedgelen = d_refedgelen; r.maxrefedgelen = d_maxrefedgelen;
        r.bendmod = d_bendmodpara; r.shearmod = d_shearmodpara; r.hbending = d_hbending; r.perlen = d_perlenWLC;
        r.hpow = d_hpow; r.reftriangle = d_reftriangle;
    }
    if (gc_state().in_fused_step) return GC_OK;
    (void)d_trinordir; (void)d_tricenter;
    GcState& s = gc_state();
    if (ncell <= 0 || nedge <= 0) return GC_OK;
    GcParams p;
    GC_TRY(gc_make_params(&p, true));
    k_mech_setup<<<gc_blocks(nedge, SDPDSIZE), SDPDSIZE, 0, s.stream>>>(
        p, nedge, (const int6*)d_edge, d_curpos, d_refedgelen, d_maxrefedgelen, d_bendmodpara, d_shearmodpara,
        d_hbending, d_powerindex, d_perlenWLC, d_hpow, d_reftriangle, (const float3*)d_coor, gc_flags_ptr());
    GC_CHECK_LAUNCH("SetMechPara");
    return GC_OK;
}

int gc_cupar_CalCellDefForce(int ncell, unsigned nedge, unsigned ntri, unsigned ntotalpar, unsigned ncellpar,
                             float* d_bbox, int* d_edge, int* d_tri, float* d_coor, float* h_defforce,
                             float* d_defforce, int* d_nthrobound, float* d_maxrefedgelen, float* d_powerindex,
                             float* d_perlenWLC, float* d_hpow, float* d_trinordir, float* d_tricenter,
                             float* d_reftriangle, float* d_hbending, float* d_triarea, float* d_reftriarea,
                             float* d_hlarea_para, float* d_hgarea_para, float* d_area_para, float* d_refarea_para,
                             float* d_hvol_para, float* d_vol_para, float* d_refvol_para, float* d_totalforce,
                             int* d_sortpart, int* d_curpos) {
    {
        GcRefPtrs& r = gc_state().ref;
        r.hlarea = d_hlarea_para; r.hgarea = d_hgarea_para; r.hvol = d_hvol_para; r.defforce = d_defforce;
        r.edge = d_edge; r.nedge = (int)nedge; r.tri = d_tri; r.ntri = (int)ntri;
    }
    if (gc_state().in_fused_step) return GC_OK;
    (void)d_bbox; (void)h_defforce; (void)d_nthrobound; (void)d_trinordir; (void)d_tricenter; (void)d_triarea;
    (void)d_sortpart;
    GcState& s = gc_state();
    if (ncell <= 0) return GC_OK;
    GcParams p;
    GC_TRY(gc_make_params(&p, true));
    if (ntotalpar != p.nT || ncellpar != p.nCP)
        return gc_fail(GC_EINVAL, "CalCellDefForce: counts disagree with ConstsDataUp");
    unsigned* flags = gc_flags_ptr();
    GC_CUDA(cudaMemsetAsync(d_defforce, 0, (size_t)ncellpar * 12, s.stream), "CalCellDefForce: clear");
    if (nedge) {
        k_edge_force<<<gc_blocks(nedge, SDPDSIZE), SDPDSIZE, 0, s.stream>>>(
            p, (int)nedge, (const int6*)d_edge, d_curpos, (const float3*)d_coor, d_maxrefedgelen, d_powerindex,
            d_perlenWLC, d_hpow, d_reftriangle, d_hbending, (float3*)d_defforce, flags);
        GC_CHECK_LAUNCH("CalCellDefForce: edges");
    }
    if (ntri) {
        k_tri_force<<<gc_blocks(ntri, SDPDSIZE), SDPDSIZE, 0, s.stream>>>(
            p, (int)ntri, (const int3*)d_tri, d_curpos, (const float3*)d_coor, d_reftriarea, d_hlarea_para,
            d_hgarea_para, d_area_para, d_refarea_para, d_hvol_para, d_vol_para, d_refvol_para, (float3*)d_defforce,
            flags);
        GC_CHECK_LAUNCH("CalCellDefForce: triangles");
    }
    k_def_apply<<<gc_blocks(ncellpar, SDPDSIZE), SDPDSIZE, 0, s.stream>>>(p, (const float3*)d_defforce, d_curpos,
                                                                        (float3*)d_totalforce);
    GC_CHECK_LAUNCH("CalCellDefForce");
    return GC_OK;
}

int gc_cupar_CalCellAggForce(unsigned ncell, unsigned n, unsigned ncellpar, float* d_totalcoor, float* d_aggforce,
                             int* d_cc, int* d_ncube, int* d_sortpart, int* d_celltab, float* d_outerregion,
                             int* d_beginendcube, float* d_totalforce, float* d_pararea) {
    {
        GcRefPtrs& r = gc_state().ref;
        r.celltab = d_celltab; r.aggforce = d_aggforce;
    }
    if (gc_state().in_fused_step) return GC_OK;
    (void)d_ncube; (void)d_outerregion;
    GcState& s = gc_state();
    if (ncell == 0 || ncellpar == 0) return GC_OK;
    GcParams p;
    GC_TRY(gc_make_params(&p, true));
    if (n != p.nT || ncellpar != p.nCP) return gc_fail(GC_EINVAL, "CalCellAggForce: counts disagree with ConstsDataUp");
    if (p.De == 0.f || !(p.maxcut > 0.f)) {
        GC_CUDA(cudaMemsetAsync(d_aggforce, 0, (size_t)ncellpar * 12, s.stream), "CalCellAggForce: clear");
        return GC_OK;
    }
    int R[3];
    for (int a = 0; a < 3; ++a) {
        R[a] = (int)ceilf(p.maxcut * p.g.invw[a]);
        if (R[a] < 1) R[a] = 1;
        if ((p.g.pmask >> a & 1) && p.g.n[a] < 2 * R[a] + 1)
            return gc_fail(GC_EINVAL, "CalCellAggForce: MaxCut spans the periodic box along axis %d", a);
    }
    k_aggregate<<<gc_blocks(n, SDPDSIZE), SDPDSIZE, 0, s.stream>>>(
        (int)n, p, R[0], R[1], R[2], (const float3*)d_totalcoor, (const int3*)d_cc, d_sortpart, d_celltab,
        (const int2*)d_beginendcube, d_pararea, (float3*)d_aggforce, (float3*)d_totalforce);
    GC_CHECK_LAUNCH("CalCellAggForce");
    return GC_OK;
}

}  // extern "C"
