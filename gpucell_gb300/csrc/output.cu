// output.cu -- GPUCell's output files, written from host arrays.
//
// The reference writes, per output step (Particle::OutputPar,
// src/Particle.cu:681-691), six Tecplot text files and appends one line per
// cell to two time series:
//
//   FluidCoor/<step>.plt   zones Bound1, Bound2, fluid, membrane: x y z id
//                          (OutputCoor, src/Particle.cu:712-790)
//   FluidField/<step>.plt  walls and fluid: x y z Den Press Vx Vy Vz
//                          (OutputField, src/Particle.cu:887-928)
//   CellCoor/<step>.plt    per cell an FE triangle zone: vertices x y z, then
//                          triangles as zone-local vertex numbers
//                          (OutPutCellCoor, src/Particle.cu:930-1005)
//   CellForce/<step>.plt   the same zones with DefForce and AggForce per
//                          vertex (OutPutCellForce, src/Particle.cu:1007-1081)
//   CellForce/TF_Cell<i>.plt  time, mean DefForce, mean AggForce of cell i
//                          (src/Particle.cu:1083-1133)
//   CellGeo/Geo_Cell<i>.plt   time, |mean velocity|, area, volume of cell i
//                          (OutPutCellGeo, src/Particle.cu:1139-1220)
//   CellNorDir/<step>.plt  per cell: triangle centre, normal, index
//                          (OutPutTriNorDir, src/Particle.cu:1222-1275)
//
// with the reference's layout: left-aligned fields, 20 characters wide (15
// in the two time series), floating point in scientific notation with five
// digits after the point.  The reference finds each cell's vertices by
// scanning all particles for every cell (O(cells x particles)) and sums the
// per-cell means on the host; here particles are written in original id
// order, each cell's vertices in membrane order (its zone-local numbering
// follows), the per-cell means arrive precomputed (the fused step reduces
// them on the GPU in FP64), and the text is formatted by several threads.
#include <errno.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "gc_internal.cuh"

namespace {

int mkdirs(const std::string& path) {
    std::string cur;
    for (size_t i = 0; i <= path.size(); ++i) {
        if (i == path.size() || path[i] == '/') {
            if (!cur.empty() && mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST)
                return gc_fail(GC_EINVAL, "output: cannot create directory %s", cur.c_str());
        }
        if (i < path.size()) cur.push_back(path[i]);
    }
    return GC_OK;
}

// "%.5e" of a float without snprintf.  The six significant digits come
// from one double division where that decides their rounding
// (digits_double; checked against the exact path on every float from 1e-15
// up), else exactly: a finite float is k * 2^q (k < 2^24), so
// m = floor(|v| / 10^(X - 5)) and the remainder are exact in 128-bit
// integers for 1e-15 <= |v| < 2^128, and the last digit is rounded to
// nearest with ties to even, as printf does with the exact binary value.
// Zeros are written directly; subnormals, values below 1e-15, infinities and
// NaNs go to snprintf (returns false).
typedef unsigned __int128 u128;

struct Pow10Table {
    u128 p[40];
    Pow10Table() {
        p[0] = 1;
        for (int i = 1; i < 40; ++i) p[i] = p[i - 1] * 10u;
    }
};
const Pow10Table kPow10;

// m = floor(k 2^q / 10^S) and the comparison of the remainder with half the
// divisor (-1 below, 0 equal, 1 above)
inline void scaled_digits(uint32_t k, int q, int S, uint64_t& m, int& half) {
    u128 N, D;
    if (S >= 0) {
        if (q >= 0) { N = (u128)k << q; D = kPow10.p[S]; }
        else { N = k; D = kPow10.p[S] << (-q); }
    } else {
        N = (u128)k * kPow10.p[-S];
        if (q >= 0) { N <<= q; D = 1; }
        else D = (u128)1 << (-q);
    }
    u128 quo = N / D, rem = N - quo * D;
    m = (uint64_t)quo;
    u128 r2 = rem << 1;
    half = r2 < D ? -1 : (r2 == D ? 0 : 1);
}

// The six rounded significant digits m (100000 <= m <= 1000000) and the
// decimal exponent X of |f| by double arithmetic: t = |f| / 10^(X-5) is one
// correctly rounded operation on exact operands (10^n is exact in double for
// n <= 22), so for 10^5 <= t < 10^6 it is within 1.2e-10 of the exact
// quotient, and rounding it to an integer gives the exact quotient's
// rounding unless its fraction lies within 1e-6 of one half (or t lies at the
// edge of the decade).  Returns false then, or when X is out of that range:
// the caller takes the exact path.
inline bool digits_double(double a, int ex, uint64_t& m, int& X) {
    static const double kP10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                    1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
    X = ((ex - 127) * 78913) >> 18;   // floor((ex - 127) log10 2): floor(log10 a) or one less
    for (int it = 0; it < 3; ++it) {
        const int S = X - 5;
        if (S < -22 || S > 22) return false;
        const double t = S >= 0 ? a / kP10[S] : a * kP10[-S];
        if (t >= 1e6) { ++X; continue; }
        if (t < 1e5) { --X; continue; }
        if (t < 100000.001 || t > 999999.999) return false;
        const uint64_t m0 = (uint64_t)t;
        const double fr = t - (double)m0;   // exact: t < 2^20
        if (fabs(fr - 0.5) < 1e-6) return false;
        m = m0 + (fr > 0.5 ? 1u : 0u);
        return true;
    }
    return false;
}

inline bool fast_e(float f, char* out, int& len) {
    uint32_t bits;
    memcpy(&bits, &f, 4);
    const bool neg = bits >> 31;
    const int ex = (int)((bits >> 23) & 0xFF);
    const uint32_t frac = bits & 0x7FFFFFu;
    char* p = out;
    if (ex == 0xFF) return false;
    if (ex == 0) {
        if (frac) return false;   // subnormal
        if (neg) *p++ = '-';
        memcpy(p, "0.00000e+00", 11);
        len = (int)(p - out) + 11;
        return true;
    }
    const double a = fabs((double)f);
    if (a < 1e-15) return false;
    uint64_t m = 0;
    int X = 0;
    if (!digits_double(a, ex, m, X)) {   // the exact path
        const uint32_t k = frac | 0x800000u;
        const int q = ex - 150;
        X = (int)floor(log10(a));
        int half = -1;
        for (int it = 0; it < 4; ++it) {
            scaled_digits(k, q, X - 5, m, half);
            if (m >= 1000000u) ++X;
            else if (m < 100000u) --X;
            else break;
        }
        if (m < 100000u || m >= 1000000u) return false;
        if (half > 0 || (half == 0 && (m & 1u))) ++m;
    }
    if (m == 1000000u) { m = 100000u; ++X; }
    if (neg) *p++ = '-';
    *p++ = (char)('0' + m / 100000u);
    *p++ = '.';
    uint32_t r = (uint32_t)(m % 100000u);
    for (int d = 4; d >= 0; --d) { p[d] = (char)('0' + r % 10u); r /= 10u; }
    p += 5;
    *p++ = 'e';
    *p++ = X < 0 ? '-' : '+';
    int ax = X < 0 ? -X : X;
    if (ax >= 100) { *p++ = (char)('0' + ax / 100); ax %= 100; }
    *p++ = (char)('0' + ax / 10);
    *p++ = (char)('0' + ax % 10);
    len = (int)(p - out);
    return true;
}

inline void put_e(std::string& s, float v, int width) {
    char b[64];
    int k;
    if (!fast_e(v, b, k)) k = snprintf(b, sizeof b, "%.5e", (double)v);
    s.append(b, (size_t)k);
    if (k < width) s.append((size_t)(width - k), ' ');
}

inline void put_d(std::string& s, long long v, int width) {
    char b[32];
    int k = 0;
    unsigned long long u = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
    char t[24];
    int n = 0;
    do { t[n++] = (char)('0' + u % 10u); u /= 10u; } while (u);
    if (v < 0) b[k++] = '-';
    while (n) b[k++] = t[--n];
    s.append(b, (size_t)k);
    if (k < width) s.append((size_t)(width - k), ' ');
}

inline void put_padded(std::string& s, const char* text, int width) {
    char b[256];
    int k = snprintf(b, sizeof b, "%-*s", width, text);
    s.append(b, (size_t)k);
}

struct File {
    FILE* fp = nullptr;
    bool ok = true;
    File(const std::string& path, const char* mode) { fp = fopen(path.c_str(), mode); ok = fp != nullptr; }
    ~File() { if (fp) fclose(fp); }
    void put(const std::string& s) {
        if (ok && !s.empty() && fwrite(s.data(), 1, s.size(), fp) != s.size()) ok = false;
    }
    bool close() {
        if (!fp) return false;
        bool r = fclose(fp) == 0 && ok;
        fp = nullptr;
        return r;
    }
};

// Formats `ntasks` pieces of text with `task(i, out)` on a pool of threads
// (taken in order from a shared counter) and writes them to f in order: the
// calling thread writes piece i as soon as it is done and formats pending
// pieces itself while it waits, so writing overlaps formatting and each
// piece's memory is released once written.
template <class F>
void emit_ordered(File& f, long long ntasks, int threads, F task) {
    if (ntasks <= 0) return;
    int t = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
    if (t < 1) t = 1;
    if ((long long)t > ntasks) t = (int)ntasks;
    std::vector<std::string> out((size_t)ntasks);
    std::unique_ptr<std::atomic<int>[]> done(new std::atomic<int>[(size_t)ntasks]);
    for (long long i = 0; i < ntasks; ++i) done[i].store(0, std::memory_order_relaxed);
    std::atomic<long long> next{0};
    auto run_one = [&]() -> bool {
        long long i = next.fetch_add(1);
        if (i >= ntasks) return false;
        task(i, out[(size_t)i]);
        done[i].store(1, std::memory_order_release);
        return true;
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < t; ++w)
        pool.emplace_back([&] {
            while (run_one()) {
            }
        });
    for (long long i = 0; i < ntasks; ++i) {
        while (!done[i].load(std::memory_order_acquire))
            if (!run_one()) std::this_thread::yield();
        f.put(out[(size_t)i]);
        std::string().swap(out[(size_t)i]);
    }
    for (auto& th : pool) th.join();
}

// Lines [0, count) as pieces of kLinesPerPiece lines, `line(i, s)` each.
constexpr long long kLinesPerPiece = 16384;

template <class F>
void emit_lines(File& f, long long count, int threads, size_t line_bytes, F line) {
    const long long pieces = (count + kLinesPerPiece - 1) / kLinesPerPiece;
    emit_ordered(f, pieces, threads, [&](long long p, std::string& s) {
        const long long b = p * kLinesPerPiece, e = std::min(count, b + kLinesPerPiece);
        s.reserve((size_t)(e - b) * line_bytes);
        for (long long i = b; i < e; ++i) line(i, s);
    });
}

int fail_write(const std::string& path) { return gc_fail(GC_EINVAL, "output: cannot write %s", path.c_str()); }

std::string step_file(const std::string& dir, const char* sub, long long step) {
    return dir + "/" + sub + "/" + std::to_string(step) + ".plt";
}

std::string zone_line() {
    std::string zone;
    put_padded(zone, "Zone", 20);
    zone += '\n';
    return zone;
}

int write_coor(const GcOutputFrame& fr, const std::string& dir, long long step, int threads) {
    std::string path = step_file(dir, "FluidCoor", step);
    File f(path, "w");
    if (!f.ok) return fail_write(path);
    f.put("Title=\"Particle Coordinate\"\n");
    f.put("Variables=\"x\",\"y\",\"z\",\"SP\"\n");
    const long long b12 = fr.n_b1 + fr.n_b2;
    const long long lo[4] = {0, fr.n_b1, b12, fr.n_cell_start};
    const long long hi[4] = {fr.n_b1, b12, fr.n_cell_start, fr.n};
    for (int z = 0; z < 4; ++z) {
        if (hi[z] <= lo[z]) continue;
        f.put(zone_line());
        const long long base = lo[z];
        emit_lines(f, hi[z] - lo[z], threads, 81, [&](long long k, std::string& s) {
            long long i = base + k;
            put_e(s, fr.pos[3 * i], 20);
            put_e(s, fr.pos[3 * i + 1], 20);
            put_e(s, fr.pos[3 * i + 2], 20);
            put_d(s, i, 20);
            s += '\n';
        });
    }
    return f.close() ? GC_OK : fail_write(path);
}

int write_field(const GcOutputFrame& fr, const std::string& dir, long long step, int threads) {
    std::string path = step_file(dir, "FluidField", step);
    File f(path, "w");
    if (!f.ok) return fail_write(path);
    f.put("Title=\"Particle Fluid\"\n");
    f.put("Variables=\"x\",\"y\",\"z\",\"Den\",\"Press\",\"Vx\",\"Vy\",\"Vz\"\n");
    emit_lines(f, fr.n_cell_start, threads, 161, [&](long long i, std::string& s) {
        put_e(s, fr.pos[3 * i], 20);
        put_e(s, fr.pos[3 * i + 1], 20);
        put_e(s, fr.pos[3 * i + 2], 20);
        put_e(s, fr.rho[i], 20);
        put_e(s, fr.press[i], 20);
        put_e(s, fr.vel[3 * i], 20);
        put_e(s, fr.vel[3 * i + 1], 20);
        put_e(s, fr.vel[3 * i + 2], 20);
        s += '\n';
    });
    return f.close() ? GC_OK : fail_write(path);
}

// CellCoor (forces = false) or CellForce (forces = true): one piece per cell
// (its zone line, vertices, then triangles as zone-local vertex numbers).
int write_cells(const GcOutputFrame& fr, const std::string& dir, long long step, int threads, bool forces) {
    std::string path = step_file(dir, forces ? "CellForce" : "CellCoor", step);
    File f(path, "w");
    if (!f.ok) return fail_write(path);
    f.put(forces ? "Title=\"Particle Force\"\n" : "Title=\"Particle Coordinate\"\n");
    f.put(forces ? "Variables=\"x\",\"y\",\"z\", \"DFx\",\"DFy\",\"DFz\",\"AFx\",\"AFy\",\"AFz\"\n"
                 : "Variables=\"x\",\"y\",\"z\"\n");
    emit_ordered(f, fr.ncell, threads, [&](long long c, std::string& s) {
        const int v0 = fr.cell_verts[2 * c], v1 = fr.cell_verts[2 * c + 1] + 1;
        const int t0 = fr.betri[2 * c], t1 = fr.betri[2 * c + 1];
        s.reserve((size_t)(v1 - v0) * (forces ? 181 : 61) + (size_t)(t1 - t0 + 1) * 61 + 64);
        char head[160];
        int k = snprintf(head, sizeof head, "Zone N=%d, E=%d, F=FEPOINT, ET=TRIANGLE\n", v1 - v0, t1 - t0 + 1);
        s.append(head, (size_t)k);
        for (long long m = v0; m < v1; ++m) {
            long long i = fr.n_cell_start + m;
            put_e(s, fr.pos[3 * i], 20);
            put_e(s, fr.pos[3 * i + 1], 20);
            put_e(s, fr.pos[3 * i + 2], 20);
            if (forces) {
                for (int a = 0; a < 3; ++a) put_e(s, fr.defforce[3 * m + a], 20);
                for (int a = 0; a < 3; ++a) put_e(s, fr.aggforce[3 * m + a], 20);
            }
            s += '\n';
        }
        for (long long t = t0; t <= t1; ++t) {
            for (int a = 0; a < 3; ++a) put_d(s, (long long)fr.tri[3 * t + a] - 1 - v0 + 1, 20);
            s += '\n';
        }
    });
    return f.close() ? GC_OK : fail_write(path);
}

int write_nordir(const GcOutputFrame& fr, const std::string& dir, long long step, int threads) {
    std::string path = step_file(dir, "CellNorDir", step);
    File f(path, "w");
    if (!f.ok) return fail_write(path);
    f.put("Title=\"Triangle information\"\n");
    f.put("Variables=\"Cenx\",\"Ceny\",\"Cenz\",\"Norx\",\"Nory\",\"Norz\",\"ID\"\n");
    const std::string zone = zone_line();
    emit_ordered(f, fr.ncell, threads, [&](long long c, std::string& s) {
        const int t0 = fr.betri[2 * c], t1 = fr.betri[2 * c + 1];
        s.reserve(zone.size() + (size_t)(t1 - t0 + 1) * 141);
        s += zone;
        for (long long t = t0; t <= t1; ++t) {
            for (int a = 0; a < 3; ++a) put_e(s, fr.tricenter[3 * t + a], 20);
            for (int a = 0; a < 3; ++a) put_e(s, fr.trinordir[3 * t + a], 20);
            put_d(s, t, 20);
            s += '\n';
        }
    });
    return f.close() ? GC_OK : fail_write(path);
}

// One line per cell appended to TF_Cell<i>.plt and Geo_Cell<i>.plt.
int write_series(const GcOutputFrame& fr, const std::string& dir, double time, int first) {
    for (int c = 0; c < fr.ncell; ++c) {
        const double* st = fr.cell_stats + 12 * (size_t)c;
        std::string tf, geo;
        put_e(tf, (float)time, 15);
        for (int a = 0; a < 6; ++a) put_e(tf, (float)st[a], 15);
        tf += '\n';
        put_e(geo, (float)time, 15);
        put_e(geo, (float)st[9], 15);
        put_e(geo, (float)st[10], 15);
        put_e(geo, (float)st[11], 15);
        geo += '\n';
        std::string p1 = dir + "/CellForce/TF_Cell" + std::to_string(c) + ".plt";
        std::string p2 = dir + "/CellGeo/Geo_Cell" + std::to_string(c) + ".plt";
        File a(p1, first ? "w" : "a");
        a.put(tf);
        if (!a.close()) return fail_write(p1);
        File b(p2, first ? "w" : "a");
        b.put(geo);
        if (!b.close()) return fail_write(p2);
    }
    return GC_OK;
}

}  // namespace

extern "C" int gc_output_write(const GcOutputFrame* fr, const char* dir, long long step_data, double time,
                               int first) {
    if (!fr || !dir) return gc_fail(GC_EINVAL, "output_write: NULL argument");
    if (fr->n < 0 || fr->n_b1 < 0 || fr->n_b2 < 0 || fr->n_b1 + fr->n_b2 > fr->n_cell_start ||
        fr->n_cell_start > fr->n)
        return gc_fail(GC_EINVAL, "output_write: inconsistent particle counts");
    if (fr->n > 0 && (!fr->pos || !fr->vel || !fr->rho || !fr->press))
        return gc_fail(GC_EINVAL, "output_write: NULL particle array");
    const long long ncp = fr->n - fr->n_cell_start;
    if (fr->ncell > 0) {
        if (!fr->cell_verts || !fr->tri || !fr->betri || !fr->defforce || !fr->aggforce || !fr->tricenter ||
            !fr->trinordir || !fr->cell_stats)
            return gc_fail(GC_EINVAL, "output_write: NULL membrane array");
        for (int c = 0; c < fr->ncell; ++c) {
            int v0 = fr->cell_verts[2 * c], v1 = fr->cell_verts[2 * c + 1] + 1;
            int t0 = fr->betri[2 * c], t1 = fr->betri[2 * c + 1];
            if (v0 < 0 || v1 < v0 || v1 > ncp || t0 < 0 || t1 < t0 || t1 >= fr->ntri)
                return gc_fail(GC_EINVAL, "output_write: bad vertex or triangle range of cell %d", c);
            for (int t = t0; t <= t1; ++t)
                for (int a = 0; a < 3; ++a) {
                    int v = fr->tri[3 * (size_t)t + a] - 1;
                    if (v < v0 || v >= v1)
                        return gc_fail(GC_EINVAL, "output_write: triangle %d of cell %d has a vertex of another cell",
                                       t, c);
                }
        }
    }
    std::string d(dir);
    for (const char* sub : {"FluidCoor", "FluidField", "CellCoor", "CellForce", "CellGeo", "CellNorDir"})
        GC_TRY(mkdirs(d + "/" + sub));
    const int th = fr->threads;
    GC_TRY(write_coor(*fr, d, step_data, th));
    GC_TRY(write_field(*fr, d, step_data, th));
    if (fr->ncell > 0) {
        GC_TRY(write_cells(*fr, d, step_data, th, false));
        GC_TRY(write_cells(*fr, d, step_data, th, true));
        GC_TRY(write_series(*fr, d, time, first));
        GC_TRY(write_nordir(*fr, d, step_data, th));
    }
    return GC_OK;
}
