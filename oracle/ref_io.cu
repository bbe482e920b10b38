// ref_io.cu -- GPUCell's own input loaders and output writers, run on the
// host, to pin this library's reader (gc_input_read) and writer
// (gc_output_write) against the reference itself rather than a
// restatement of it.
//
// Test infrastructure, built only where the reference's sources are present
// (oracle/ref_io.mk compiles src/Particle.cu and src/main.cu where they lie,
// with the reference's main renamed, and links this file against them into
// oracle/_ref/ref_io).  No CUDA call is made: the loaders
// (Particle::LoadParInfo and what it calls, src/Particle.cu:29-470) and the
// writers (Particle::OutputCoor ... OutPutTriNorDir, src/Particle.cu:712-1300)
// touch host memory and files only.
//
//   ref_io load  <dir> <dump>    LoadParInfo() on the four input files in
//                                <dir>; writes what it read to <dump>
//   ref_io write <dir> <frame>   LoadParInfo() on the files in <dir>, the host
//                                arrays from <frame>, then the six writers
//                                (files under <dir>/Result/)
//
// <dump>, little-endian: int64 nBound1Par, nBound2Par, nFluidPar, nCell,
// nAllTri, nAllEdge, nCellPar, nType; float SoundSpeed1, SoundSpeed2,
// ShearVis, BulkVis, DenInit, ConstExtForce, MaxCut, zeroLen, scaFac,
// surEnergy; float TotalCoor[nTotal][3]; then, with cells: int Type,
// nPar, nTri [nCell], BeginEndCoor, BeginEndTri [nCell][2], Tri[nAllTri][3],
// Edge[nAllEdge][6], CellTab[nCellPar]; float ShearMod_Para,
// BendingMod_Para [nAllEdge], HLarea_Para, HGarea_Para, HVol_Para [nAllTri],
// ShearMod, BendingMod, HGarea, HLarea, HVol [nType].
//
// <frame>, little-endian: int64 nTotal, nCellPar, nCell, nAllTri, StepData,
// StepCount; float TotalCoor[nTotal][3], Velrhop[nTotal][4], Press[nTotal];
// int SortPart[nTotal]; float h_DefForce[nCellPar][3],
// h_AggForce[nCellPar][3], h_Area[nCell], h_Vol[nCell],
// TriNorDir[nAllTri][3], TriCenter[nAllTri][3].
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <vector>

#include <cuda_runtime.h>

// in the order the reference's own sources include them
#include "main.cuh"
#include "TypesDef.cuh"
#include "Particle.cuh"

namespace {

struct Out {
    FILE* fp;
    bool ok = true;
    template <class T>
    void put(const T* p, size_t n) {
        if (n && fwrite(p, sizeof(T), n, fp) != n) ok = false;
    }
    void i64(long long v) { put(&v, 1); }
    void f32(float v) { put(&v, 1); }
};

struct In {
    FILE* fp;
    bool ok = true;
    template <class T>
    void get(T* p, size_t n) {
        if (n && fread(p, sizeof(T), n, fp) != n) ok = false;
    }
};

int load(const char* dump) {
    Particle p;
    p.LoadParInfo();
    FILE* fp = fopen(dump, "wb");
    if (!fp) return 2;
    Out o{fp};
    const long long ncell = p.nCell > 0 ? p.nCell : 0;
    const long long ntri = ncell ? p.nAllTri : 0, nedge = ncell ? p.nAllEdge : 0;
    const long long ntype = ncell ? p.nType : 0;
    for (long long v : {(long long)p.nBound1Par, (long long)p.nBound2Par, (long long)p.nFluidPar, ncell, ntri, nedge,
                        (long long)p.consts.nCellPar, ntype})
        o.i64(v);
    const Structconst& c = p.consts;
    for (float v : {c.SoundSpeed1, c.SoundSpeed2, c.ShearVis, c.BulkVis, p.DenInit, c.ConstExtForce, c.MaxCut,
                    c.zeroLen, c.scaFac, c.surEnergy})
        o.f32(v);
    for (int i = 0; i < c.nTotalPar; ++i) o.put(&p.TotalCoor[i].x, 3);
    if (ncell) {
        o.put(p.Type, ncell);
        o.put(p.nPar, ncell);
        o.put(p.nTri, ncell);
        for (int i = 0; i < ncell; ++i) o.put(&p.BeginEndCoor[i].x, 2);
        for (int i = 0; i < ncell; ++i) o.put(&p.BeginEndTri[i].x, 2);
        for (long long i = 0; i < ntri; ++i) o.put(&p.Tri[i].x, 3);
        for (long long i = 0; i < nedge; ++i) o.put(&p.Edge[i].x, 6);
        o.put(p.CellTab, (size_t)c.nCellPar);
        o.put(p.ShearMod_Para, nedge);
        o.put(p.BendingMod_Para, nedge);
        o.put(p.HLarea_Para, ntri);
        o.put(p.HGarea_Para, ntri);
        o.put(p.HVol_Para, ntri);
        o.put(p.ShearMod, ntype);
        o.put(p.BendingMod, ntype);
        o.put(p.HGarea, ntype);
        o.put(p.HLarea, ntype);
        o.put(p.HVol, ntype);
    }
    if (fclose(fp) != 0) o.ok = false;
    return o.ok ? 0 : 2;
}

int write(const char* frame) {
    Particle p;
    p.LoadParInfo();
    FILE* fp = fopen(frame, "rb");
    if (!fp) return 2;
    In in{fp};
    long long h[6];
    in.get(h, 6);
    const long long n = h[0], ncp = h[1], ncell = h[2], ntri = h[3];
    if (!in.ok || n != p.consts.nTotalPar || ncp != p.consts.nCellPar || ncell != (p.nCell > 0 ? p.nCell : 0) ||
        ntri != (ncell ? p.nAllTri : 0)) {
        fprintf(stderr, "ref_io: the frame does not match the input files\n");
        fclose(fp);
        return 2;
    }
    StepData = (long int)h[4];
    StepCount = (long int)h[5];
    std::vector<float> v4(4 * (size_t)n);
    for (long long i = 0; i < n; ++i) in.get(&p.TotalCoor[i].x, 3);
    in.get(v4.data(), v4.size());
    for (long long i = 0; i < n; ++i) {
        p.Velrhop[i].x = v4[4 * i];
        p.Velrhop[i].y = v4[4 * i + 1];
        p.Velrhop[i].z = v4[4 * i + 2];
        p.Velrhop[i].w = v4[4 * i + 3];
    }
    in.get(p.Press, n);
    in.get(p.SortPart, n);
    if (ncell) {
        for (long long i = 0; i < ncp; ++i) in.get(&p.h_DefForce[i].x, 3);
        for (long long i = 0; i < ncp; ++i) in.get(&p.h_AggForce[i].x, 3);
        in.get(p.h_Area, ncell);
        in.get(p.h_Vol, ncell);
        for (long long i = 0; i < ntri; ++i) in.get(&p.TriNorDir[i].x, 3);
        for (long long i = 0; i < ntri; ++i) in.get(&p.TriCenter[i].x, 3);
    }
    fclose(fp);
    if (!in.ok) {
        fprintf(stderr, "ref_io: the frame is truncated\n");
        return 2;
    }
    // the writers expect these folders (the reference ships them)
    mkdir("Result", 0755);
    for (const char* d : {"Result/FluidCoor", "Result/FluidField", "Result/CellCoor", "Result/CellForce",
                          "Result/CellGeo", "Result/CellNorDir"})
        mkdir(d, 0755);
    p.OutputCoor(StepData);
    p.OutputField(StepData);
    p.OutPutCellCoor(StepData);
    p.OutPutCellForce(StepData);
    p.OutPutCellGeo(StepData);
    p.OutPutTriNorDir(StepData);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 4 || (strcmp(argv[1], "load") != 0 && strcmp(argv[1], "write") != 0)) {
        fprintf(stderr, "usage: ref_io load|write <dir> <file>\n");
        return 1;
    }
    // the reference opens its files relative to the working directory
    char file[4096];
    if (argv[3][0] == '/') {
        snprintf(file, sizeof(file), "%s", argv[3]);
    } else {
        char cwd[2048];
        if (!getcwd(cwd, sizeof(cwd))) return 2;
        snprintf(file, sizeof(file), "%s/%s", cwd, argv[3]);
    }
    if (chdir(argv[2]) != 0) {
        fprintf(stderr, "ref_io: cannot enter %s\n", argv[2]);
        return 2;
    }
    return strcmp(argv[1], "load") == 0 ? load(file) : write(file);
}
