// input.cu -- GPUCell's four input files, read without size caps, and a
// binary form of the same content for fast reloading.
//
// The reference's loaders (Particle::LoadFBPar, LoadSDPDPara, LoadCellStruct,
// LoadCellPara, src/Particle.cu:45-380) read fixed-width text: every value
// sits in a 20-character column and is converted with atoi/atof; every data
// block is preceded by one header line.  They copy into arrays of fixed
// size (2,000,000 wall + fluid particles and 4,000,000 membrane vertices,
// triangles and edges, src/Particle.cu:31-32, 200-202) and read line by
// line into a 200-character buffer.  Here each file is mapped whole, its line
// starts are found by all host threads, the numeric lines are converted by
// all host threads (the cells' rows in chunks shared out across cells), and
// the arrays are sized from the counts in the files.  The
// topology gets the reference's per-cell offsets (vertices of cell i
// follow those of cells 0..i-1; triangle indices in the edge records follow
// the triangles of cells 0..i-1), src/Particle.cu:252-284, and the per-type
// moduli are spread over edges and triangles as src/Particle.cu:355-375 does.
#include <errno.h>
#include <fcntl.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "gc_internal.cuh"

namespace {

// The decimal number in s[0, n) as strtod reads it, when that is m 10^e
// with at most 19 significant digits m < 2^53 and |e| <= 22 (surrounded by
// spaces only): m and 10^|e| are then exact doubles and one IEEE multiply
// or divide rounds their product or quotient correctly, as strtod does
// (Clinger 1990).  Returns false for anything else (more digits, larger
// exponents, inf/nan/hex, trailing text), which goes to strtod.
bool fast_decimal(const char* s, size_t n, double* out) {
    static const double kP10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                    1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
    size_t i = 0;
    while (i < n && s[i] == ' ') ++i;
    bool neg = false;
    if (i < n && (s[i] == '+' || s[i] == '-')) neg = s[i++] == '-';
    uint64_t m = 0;
    int digits = 0, exp10 = 0, seen = 0;
    bool point = false;
    for (; i < n; ++i) {
        char c = s[i];
        if (c >= '0' && c <= '9') {
            ++seen;
            if (m == 0 && c == '0') {   // leading zeros carry no digit
                if (point) --exp10;
                continue;
            }
            if (digits == 19) return false;
            m = m * 10u + (uint64_t)(c - '0');
            ++digits;
            if (point) --exp10;
        } else if (c == '.' && !point) {
            point = true;
        } else {
            break;
        }
    }
    if (seen == 0) return false;
    if (i < n && (s[i] == 'e' || s[i] == 'E')) {
        ++i;
        bool eneg = false;
        if (i < n && (s[i] == '+' || s[i] == '-')) eneg = s[i++] == '-';
        int e = 0, ed = 0;
        for (; i < n && s[i] >= '0' && s[i] <= '9'; ++i) {
            if (e < 10000) e = e * 10 + (s[i] - '0');
            ++ed;
        }
        if (ed == 0) return false;
        exp10 += eneg ? -e : e;
    }
    while (i < n && s[i] == ' ') ++i;
    if (i != n) return false;
    if (m >= (1ull << 53)) return false;
    double v = (double)m;
    if (m != 0) {
        if (exp10 > 22 || exp10 < -22) return false;
        v = exp10 >= 0 ? v * kP10[exp10] : v / kP10[-exp10];
    }
    *out = neg ? -v : v;
    return true;
}

// A text file mapped read-only, with the start of every line.
struct Text {
    const char* buf = nullptr;
    size_t size = 0;
    std::vector<size_t> line;   // start offset of every line
    Text() = default;
    Text(const Text&) = delete;
    Text& operator=(const Text&) = delete;
    ~Text() {
        if (buf) munmap((void*)buf, size);
    }
    size_t count() const { return line.size(); }
    // Column k (20 characters) of line r, converted like atof / atoi.
    double f(size_t r, int k) const { return atof_col(r, k); }
    long long i(size_t r, int k) const { return (long long)atof_col(r, k); }

  private:
    double atof_col(size_t r, int k) const {
        char tmp[24];
        size_t b = line[r], e = r + 1 < line.size() ? line[r + 1] - 1 : size;
        size_t s = b + 20 * (size_t)k;
        size_t m = 0;
        while (m < 20 && s + m < e) {
            tmp[m] = buf[s + m];
            ++m;
        }
        while (m > 0 && (tmp[m - 1] == '\r' || tmp[m - 1] == '\t')) --m;   // line ends and tabs: strtod's business
        double v;
        if (m > 0 && fast_decimal(tmp, m, &v)) return v;
        tmp[m] = '\0';
        m = 0;
        while (m < 20 && s + m < e) {   // the column as it was, for strtod
            tmp[m] = buf[s + m];
            ++m;
        }
        tmp[m] = '\0';
        return strtod(tmp, nullptr);
    }
};

// fn(w) for w in [0, nt) on nt threads (the caller's among them)
template <class F>
void run_threads(int nt, F fn) {
    std::vector<std::thread> pool;
    for (int w = 1; w < nt; ++w) pool.emplace_back(fn, w);
    fn(0);
    for (auto& th : pool) th.join();
}

int host_threads() {
    int nt = (int)std::thread::hardware_concurrency();
    return nt < 1 ? 1 : nt;
}

// Maps a file and finds its line starts: the text is cut into one piece per
// thread, each piece's newlines are found with memchr, and the pieces' line
// starts are joined in order.  (Mapped, the text is neither copied nor
// zero-filled first, and the threads that read it fault its pages in.)
int load_text(const std::string& path, Text* t) {
    const int fd = open(path.c_str(), O_RDONLY);
    if (fd < 0) return gc_fail(GC_EINVAL, "input: cannot open %s", path.c_str());
    struct stat st;
    if (fstat(fd, &st) != 0 || !S_ISREG(st.st_mode)) {
        close(fd);
        return gc_fail(GC_EINVAL, "input: %s is not a readable file", path.c_str());
    }
    t->size = (size_t)st.st_size;
    if (t->size > 0) {
        void* m = mmap(nullptr, t->size, PROT_READ, MAP_PRIVATE, fd, 0);
        if (m == MAP_FAILED) {
            t->size = 0;
            close(fd);
            return gc_fail(GC_EINVAL, "input: cannot read %s", path.c_str());
        }
        t->buf = (const char*)m;
    }
    close(fd);
    const size_t n = t->size;
    const char* b = t->buf;
    const int nt = n >= ((size_t)1 << 22) ? host_threads() : 1;
    std::vector<std::vector<size_t>> part(nt);
    run_threads(nt, [&](int w) {
        const char* p = b + n * w / nt;
        const char* e = b + n * (w + 1) / nt;
        while (p < e) {
            const char* q = (const char*)memchr(p, '\n', (size_t)(e - p));
            if (!q) break;
            const size_t k = (size_t)(q - b);
            if (k + 1 < n) part[w].push_back(k + 1);
            p = q + 1;
        }
    });
    size_t total = 1;
    for (const auto& v : part) total += v.size();
    t->line.clear();
    t->line.reserve(total);
    t->line.push_back(0);
    for (const auto& v : part) t->line.insert(t->line.end(), v.begin(), v.end());
    return GC_OK;
}

// fn(r) for r in [0, count), cut into one contiguous range per thread
template <class F>
void parallel_rows(size_t count, F fn) {
    const int nt = count < 50000 ? 1 : host_threads();
    run_threads(nt, [&](int w) {
        size_t b = count * w / nt, e = count * (w + 1) / nt;
        for (size_t r = b; r < e; ++r) fn(r);
    });
}

// fn(i) for i in [0, count) taken in order by all threads from one counter
// (tasks of uneven size)
template <class F>
void parallel_tasks(size_t count, F fn) {
    const int nt = count < 2 ? 1 : host_threads();
    std::atomic<size_t> next{0};
    run_threads(nt, [&](int) {
        for (size_t i = next++; i < count; i = next++) fn(i);
    });
}

template <class T>
T* alloc(size_t n) {
    return (T*)calloc(n ? n : 1, sizeof(T));
}

int need(const Text& t, size_t rows, const char* file) {
    if (rows > t.count()) return gc_fail(GC_EINVAL, "input: %s ends early (%zu lines, %zu needed)", file,
                                         t.count(), rows);
    return GC_OK;
}

}  // namespace

extern "C" int gc_input_free(GcInputSet* s) {
    if (!s) return GC_OK;
    void* ptrs[] = {s->sdpd_coor, s->cell_type, s->npar, s->ntri_cell, s->cell_coor, s->tri, s->edge, s->betri,
                    s->celltab, s->shear_mod, s->bending_mod, s->hgarea, s->hlarea, s->hvol, s->shear_e, s->bend_e,
                    s->hl_t, s->hg_t, s->hv_t};
    for (void* q : ptrs) free(q);
    memset(s, 0, sizeof(*s));
    return GC_OK;
}

static int input_read(const char* dir, GcInputSet* out) {
    std::string d(dir);
    GcInputSet& s = *out;
    int rc = GC_OK;
    // SDPDParCoor.txt: header, counts, then per type a header and its rows
    {
        Text t;
        GC_TRY(load_text(d + "/SDPDParCoor.txt", &t));
        GC_TRY(need(t, 2, "SDPDParCoor.txt"));
        s.n_b1 = t.i(1, 0);
        s.n_b2 = t.i(1, 1);
        s.n_fluid = t.i(1, 2);
        if (s.n_b1 < 0 || s.n_b2 < 0 || s.n_fluid < 0) return gc_fail(GC_EINVAL, "input: negative particle counts");
        const long long n = s.n_b1 + s.n_b2 + s.n_fluid;
        GC_TRY(need(t, (size_t)(2 + 3 + n), "SDPDParCoor.txt"));
        s.sdpd_coor = alloc<float>(3 * (size_t)n);
        const long long cnt[3] = {s.n_b1, s.n_b2, s.n_fluid};
        size_t r = 2, o = 0;
        for (int b = 0; b < 3; ++b) {
            r += 1;   // block header
            size_t r0 = r, o0 = o;
            parallel_rows((size_t)cnt[b], [&](size_t k) {
                for (int a = 0; a < 3; ++a) s.sdpd_coor[3 * (o0 + k) + a] = (float)t.f(r0 + k, a);
            });
            r += cnt[b];
            o += cnt[b];
        }
    }
    // SDPDPhyPara.txt
    {
        Text t;
        GC_TRY(load_text(d + "/SDPDPhyPara.txt", &t));
        GC_TRY(need(t, 11, "SDPDPhyPara.txt"));
        s.sound1 = (float)t.f(1, 0);
        s.sound2 = (float)t.f(2, 0);
        s.shear_vis = (float)t.f(4, 0);
        s.bulk_vis = (float)t.f(6, 0);
        s.den_init = (float)t.f(8, 0);
        s.ext_force = (float)t.f(10, 0);
    }
    // CELLParStruct.txt: nCell, then per cell: header, (Type nPar nTri
    // nEdgeInfo), header, vertices, header, triangles, header, edges
    Text cs;
    GC_TRY(load_text(d + "/CELLParStruct.txt", &cs));
    GC_TRY(need(cs, 2, "CELLParStruct.txt"));
    s.ncell = (int)cs.i(1, 0);
    if (s.ncell < 0) return gc_fail(GC_EINVAL, "input: negative cell count");
    s.cell_type = alloc<int>(s.ncell);
    s.npar = alloc<int>(s.ncell);
    s.ntri_cell = alloc<int>(s.ncell);
    std::vector<size_t> row_v(s.ncell), row_t(s.ncell), row_e(s.ncell);
    {
        size_t r = 2;
        for (int c = 0; c < s.ncell; ++c) {
            GC_TRY(need(cs, r + 2, "CELLParStruct.txt"));
            s.cell_type[c] = (int)cs.i(r + 1, 0);
            s.npar[c] = (int)cs.i(r + 1, 1);
            s.ntri_cell[c] = (int)cs.i(r + 1, 2);
            if (s.npar[c] < 0 || s.ntri_cell[c] < 0) return gc_fail(GC_EINVAL, "input: bad counts of cell %d", c);
            r += 2;
            row_v[c] = r + 1;
            r += 1 + s.npar[c];
            row_t[c] = r + 1;
            r += 1 + s.ntri_cell[c];
            row_e[c] = r + 1;
            r += 1 + (size_t)s.ntri_cell[c] * 3 / 2;   // nEdge = nTri * 3 / 2 (src/Particle.cu:217)
            s.ncp += s.npar[c];
            s.ntri += s.ntri_cell[c];
            s.nedge += (long long)s.ntri_cell[c] * 3 / 2;
        }
        GC_TRY(need(cs, r, "CELLParStruct.txt"));
    }
    s.cell_coor = alloc<float>(3 * (size_t)s.ncp);
    s.tri = alloc<int>(3 * (size_t)s.ntri);
    s.edge = alloc<int>(6 * (size_t)s.nedge);
    s.betri = alloc<int>(2 * (size_t)s.ncell);
    s.celltab = alloc<int>((size_t)s.ncp);
    {
        // each cell's vertex, triangle and edge offsets, then its rows in
        // chunks that all threads share out (cells are many and small, or few
        // and large)
        std::vector<long long> vo(s.ncell), to(s.ncell), eo(s.ncell);
        long long b = 0, a = 0, e = 0;
        for (int c = 0; c < s.ncell; ++c) {
            vo[c] = b;
            to[c] = a;
            eo[c] = e;
            s.betri[2 * c] = (int)a;
            s.betri[2 * c + 1] = (int)(a + s.ntri_cell[c] - 1);
            b += s.npar[c];
            a += s.ntri_cell[c];
            e += (long long)s.ntri_cell[c] * 3 / 2;
        }
        struct Chunk {
            int cell, kind;   // kind 0: vertices, 1: triangles, 2: edges
            size_t k0, k1;
        };
        constexpr size_t kRows = 4096;
        std::vector<Chunk> chunks;
        for (int c = 0; c < s.ncell; ++c) {
            const size_t rows[3] = {(size_t)s.npar[c], (size_t)s.ntri_cell[c], (size_t)s.ntri_cell[c] * 3 / 2};
            for (int kind = 0; kind < 3; ++kind)
                for (size_t k0 = 0; k0 < rows[kind]; k0 += kRows)
                    chunks.push_back(Chunk{c, kind, k0, std::min(rows[kind], k0 + kRows)});
        }
        parallel_tasks(chunks.size(), [&](size_t i) {
            const Chunk& ch = chunks[i];
            const int c = ch.cell;
            const long long b0 = vo[c], a0 = to[c], e0 = eo[c];
            if (ch.kind == 0) {
                for (size_t k = ch.k0; k < ch.k1; ++k) {
                    for (int q = 0; q < 3; ++q) s.cell_coor[3 * (b0 + k) + q] = (float)cs.f(row_v[c] + k, q);
                    s.celltab[b0 + k] = c;
                }
            } else if (ch.kind == 1) {
                for (size_t k = ch.k0; k < ch.k1; ++k)
                    for (int q = 0; q < 3; ++q) s.tri[3 * (a0 + k) + q] = (int)cs.i(row_t[c] + k, q) + (int)b0;
            } else {
                for (size_t k = ch.k0; k < ch.k1; ++k) {
                    for (int q = 0; q < 4; ++q) s.edge[6 * (e0 + k) + q] = (int)cs.i(row_e[c] + k, q) + (int)b0;
                    for (int q = 4; q < 6; ++q) s.edge[6 * (e0 + k) + q] = (int)cs.i(row_e[c] + k, q) + (int)a0;
                }
            }
        });
    }
    // CELLPhyPara.txt (read when there are cells, as the reference does):
    // nType, then per quantity a header and one line per type
    if (s.ncell > 0) {
        Text t;
        GC_TRY(load_text(d + "/CELLPhyPara.txt", &t));
        GC_TRY(need(t, 2, "CELLPhyPara.txt"));
        s.ntype = (int)t.i(1, 0);
        if (s.ntype <= 0) return gc_fail(GC_EINVAL, "input: CELLPhyPara.txt has %d types", s.ntype);
        GC_TRY(need(t, 2 + 5 * (1 + (size_t)s.ntype) + 8, "CELLPhyPara.txt"));
        float** per_type[5] = {&s.shear_mod, &s.bending_mod, &s.hgarea, &s.hlarea, &s.hvol};
        size_t r = 2;
        for (auto q : per_type) {
            *q = alloc<float>(s.ntype);
            r += 1;
            for (int k = 0; k < s.ntype; ++k) (*q)[k] = (float)t.f(r + k, 0);
            r += s.ntype;
        }
        s.max_cut = (float)t.f(r + 1, 0);
        s.zero_len = (float)t.f(r + 3, 0);
        s.sca_fac = (float)t.f(r + 5, 0);
        s.sur_energy = (float)t.f(r + 7, 0);
        s.shear_e = alloc<float>((size_t)s.nedge);
        s.bend_e = alloc<float>((size_t)s.nedge);
        s.hl_t = alloc<float>((size_t)s.ntri);
        s.hg_t = alloc<float>((size_t)s.ntri);
        s.hv_t = alloc<float>((size_t)s.ntri);
        long long e = 0, m = 0;
        for (int c = 0; c < s.ncell && rc == GC_OK; ++c) {
            int ty = s.cell_type[c] - 1;
            if (ty < 0 || ty >= s.ntype) {
                rc = gc_fail(GC_EINVAL, "input: cell %d has type %d of %d", c, ty + 1, s.ntype);
                break;
            }
            for (int k = 0; k < s.ntri_cell[c] * 3 / 2; ++k, ++e) {
                s.shear_e[e] = s.shear_mod[ty];
                s.bend_e[e] = s.bending_mod[ty];
            }
            for (int k = 0; k < s.ntri_cell[c]; ++k, ++m) {
                s.hl_t[m] = s.hlarea[ty];
                s.hg_t[m] = s.hgarea[ty];
                s.hv_t[m] = s.hvol[ty];
            }
        }
    }
    return rc;
}

extern "C" int gc_input_read(const char* dir, GcInputSet* out) {
    if (!dir || !out) return gc_fail(GC_EINVAL, "input_read: NULL argument");
    memset(out, 0, sizeof(*out));
    int rc = input_read(dir, out);
    if (rc != GC_OK) gc_input_free(out);   // nothing half-read is left behind
    return rc;
}

// ---- binary form ----------------------------------------------------------
// "GCINPUT1", then the scalar fields, then every array in a fixed order, all
// little-endian as the host stores them.
namespace {

struct BinHead {
    char magic[8];
    long long n_b1, n_b2, n_fluid, ncp, ntri, nedge;
    int ncell, ntype;
    float sound1, sound2, shear_vis, bulk_vis, den_init, ext_force, max_cut, zero_len, sca_fac, sur_energy;
};

template <class T>
struct Arr {
    T** p;
    size_t n;
};

}  // namespace

extern "C" int gc_input_write_binary(const char* path, const GcInputSet* s) {
    if (!path || !s) return gc_fail(GC_EINVAL, "input_write_binary: NULL argument");
    FILE* fp = fopen(path, "wb");
    if (!fp) return gc_fail(GC_EINVAL, "input: cannot open %s for writing", path);
    BinHead h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, "GCINPUT1", 8);
    h.n_b1 = s->n_b1; h.n_b2 = s->n_b2; h.n_fluid = s->n_fluid; h.ncp = s->ncp; h.ntri = s->ntri;
    h.nedge = s->nedge; h.ncell = s->ncell; h.ntype = s->ntype; h.sound1 = s->sound1; h.sound2 = s->sound2;
    h.shear_vis = s->shear_vis; h.bulk_vis = s->bulk_vis; h.den_init = s->den_init; h.ext_force = s->ext_force;
    h.max_cut = s->max_cut; h.zero_len = s->zero_len; h.sca_fac = s->sca_fac; h.sur_energy = s->sur_energy;
    bool ok = fwrite(&h, sizeof(h), 1, fp) == 1;
    const size_t n = (size_t)(s->n_b1 + s->n_b2 + s->n_fluid), nc = (size_t)s->ncell, nt = (size_t)s->ntype;
    const size_t ne = (size_t)s->nedge, ntr = (size_t)s->ntri, ncp = (size_t)s->ncp;
    auto put = [&](const void* p, size_t bytes) {
        if (ok && bytes) ok = p && fwrite(p, 1, bytes, fp) == bytes;
    };
    put(s->sdpd_coor, 12 * n);
    put(s->cell_type, 4 * nc); put(s->npar, 4 * nc); put(s->ntri_cell, 4 * nc);
    put(s->cell_coor, 12 * ncp); put(s->tri, 12 * ntr); put(s->edge, 24 * ne); put(s->betri, 8 * nc);
    put(s->celltab, 4 * ncp);
    if (nc) {
        put(s->shear_mod, 4 * nt); put(s->bending_mod, 4 * nt); put(s->hgarea, 4 * nt); put(s->hlarea, 4 * nt);
        put(s->hvol, 4 * nt);
        put(s->shear_e, 4 * ne); put(s->bend_e, 4 * ne); put(s->hl_t, 4 * ntr); put(s->hg_t, 4 * ntr);
        put(s->hv_t, 4 * ntr);
    }
    if (fclose(fp) != 0) ok = false;
    return ok ? GC_OK : gc_fail(GC_EINVAL, "input: write to %s failed", path);
}

extern "C" int gc_input_read_binary(const char* path, GcInputSet* out) {
    if (!path || !out) return gc_fail(GC_EINVAL, "input_read_binary: NULL argument");
    memset(out, 0, sizeof(*out));
    FILE* fp = fopen(path, "rb");
    if (!fp) return gc_fail(GC_EINVAL, "input: cannot open %s", path);
    BinHead h;
    if (fread(&h, sizeof(h), 1, fp) != 1 || memcmp(h.magic, "GCINPUT1", 8) != 0) {
        fclose(fp);
        return gc_fail(GC_EINVAL, "input: %s is not a binary input set", path);
    }
    GcInputSet& s = *out;
    s.n_b1 = h.n_b1; s.n_b2 = h.n_b2; s.n_fluid = h.n_fluid; s.ncp = h.ncp; s.ntri = h.ntri; s.nedge = h.nedge;
    s.ncell = h.ncell; s.ntype = h.ntype; s.sound1 = h.sound1; s.sound2 = h.sound2; s.shear_vis = h.shear_vis;
    s.bulk_vis = h.bulk_vis; s.den_init = h.den_init; s.ext_force = h.ext_force; s.max_cut = h.max_cut;
    s.zero_len = h.zero_len; s.sca_fac = h.sca_fac; s.sur_energy = h.sur_energy;
    bool ok = s.n_b1 >= 0 && s.n_b2 >= 0 && s.n_fluid >= 0 && s.ncp >= 0 && s.ntri >= 0 && s.nedge >= 0 &&
              s.ncell >= 0 && s.ntype >= 0;
    const size_t n = (size_t)(s.n_b1 + s.n_b2 + s.n_fluid), nc = (size_t)s.ncell, nt = (size_t)s.ntype;
    const size_t ne = (size_t)s.nedge, ntr = (size_t)s.ntri, ncp = (size_t)s.ncp;
    auto get = [&](auto** p, size_t count) {
        using T = typename std::remove_reference<decltype(**p)>::type;
        *p = alloc<T>(count);
        if (ok && count) ok = *p && fread(*p, sizeof(T), count, fp) == count;
    };
    if (ok) {
        get(&s.sdpd_coor, 3 * n);
        get(&s.cell_type, nc); get(&s.npar, nc); get(&s.ntri_cell, nc);
        get(&s.cell_coor, 3 * ncp); get(&s.tri, 3 * ntr); get(&s.edge, 6 * ne); get(&s.betri, 2 * nc);
        get(&s.celltab, ncp);
        if (nc) {
            get(&s.shear_mod, nt); get(&s.bending_mod, nt); get(&s.hgarea, nt); get(&s.hlarea, nt);
            get(&s.hvol, nt);
            get(&s.shear_e, ne); get(&s.bend_e, ne); get(&s.hl_t, ntr); get(&s.hg_t, ntr); get(&s.hv_t, ntr);
        }
    }
    fclose(fp);
    if (!ok) {
        gc_input_free(out);
        return gc_fail(GC_EINVAL, "input: %s is truncated or corrupt", path);
    }
    return GC_OK;
}
