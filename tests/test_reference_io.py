"""The library's reader and writer of GPUCell's files against GPUCell's own
loaders and writers, run on the host.

oracle/_ref/ref_io is built by oracle/ref_io.mk from the reference's
src/Particle.cu and src/main.cu where they lie, only where the reference's
sources are present (the tests skip elsewhere).  It calls
Particle::LoadParInfo (src/Particle.cu:29-470) and the six writers of
Particle::OutputPar (src/Particle.cu:712-1300) on host memory; no GPU.

* gc_input_read reads the four input files as the reference's loaders do:
  every count, parameter, coordinate, topology index (with the per-cell
  offsets) and per-edge / per-triangle modulus, compared bit for bit, for a
  walled channel with cells of two types, a periodic suspension, a system
  without cells, the channel's files with CRLF line ends, and its
  coordinates in other spellings (%E, fixed point, explicit signs).
* gc_output_write writes the files the reference's writers write, byte for
  byte, from the same host arrays with the particles in id order (SortPart
  the identity), for a first output step and an appended one; the per-cell
  time series get the per-cell means the reference's writers form (FP32 sums
  in slot order).  With the slots permuted the reference writes the same
  particle rows in slot order: the same rows, zone by zone.
"""
import os
import subprocess

import numpy as np
import pytest

from gpucell_gb300 import generator as gen
from gpucell_gb300.inputs import read_inputs
from gpucell_gb300.output import write_frame

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_IO = os.path.join(ROOT, "oracle", "_ref", "ref_io")
TIME_STEP, STEP_OUTPUT = np.float32(1.0e-3), np.float32(100)   # src/main.cuh:8,16

pytestmark = pytest.mark.skipif(not os.path.exists(REF_IO),
                                reason="the reference's own loaders and writers are built only where its sources are")


def _ref(*args, cwd=None):
    res = subprocess.run([REF_IO, *map(str, args)], capture_output=True, text=True, cwd=cwd, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr


class _Reader:
    def __init__(self, path):
        self.b = open(path, "rb").read()
        self.o = 0

    def take(self, dtype, n):
        a = np.frombuffer(self.b, dtype=dtype, count=int(n), offset=self.o)
        self.o += a.nbytes
        return a


def _ref_load(directory, tmp_path):
    dump = tmp_path / "ref_load.bin"
    _ref("load", directory, dump)
    r = _Reader(dump)
    nb1, nb2, nfl, ncell, ntri, nedge, ncp, ntype = (int(v) for v in r.take("<i8", 8))
    par = r.take("<f4", 10)
    out = dict(n_b1=nb1, n_b2=nb2, n_fluid=nfl, ncell=ncell, ntri=ntri, nedge=nedge, ncp=ncp, ntype=ntype,
               params=par, coor=r.take("<f4", 3 * (nb1 + nb2 + nfl + ncp)).reshape(-1, 3))
    if ncell:
        for k, cnt in (("cell_type", ncell), ("npar", ncell), ("ntri_cell", ncell), ("verts", 2 * ncell),
                       ("betri", 2 * ncell), ("tri", 3 * ntri), ("edge", 6 * nedge), ("celltab", ncp)):
            out[k] = r.take("<i4", cnt)
        for k, cnt in (("shear_e", nedge), ("bend_e", nedge), ("hl_t", ntri), ("hg_t", ntri), ("hv_t", ntri),
                       ("shear_mod", ntype), ("bending_mod", ntype), ("hgarea", ntype), ("hlarea", ntype),
                       ("hvol", ntype)):
            out[k] = r.take("<f4", cnt)
    assert r.o == len(r.b)
    return out


def _two_types(directory, cfg):
    cfg.cell_type = np.array([2, 1], np.int32)
    gen.write_reference_inputs(cfg, str(directory))
    lines = ["nType", "2", "ShearMod", "100", "7.25", "BendingMod", "50", "3", "HGarea", "5000", "11", "HLarea",
             "100", "13", "HVol", "5000", "17", "MaxCut", "1.5", "zeroLen", "0.3", "scaFac", "1.25", "surEnergy",
             "0.002"]
    with open(os.path.join(directory, "CELLPhyPara.txt"), "w") as f:
        f.write("".join((x if not x[0].isdigit() else f"{x:<20}") + "\n" for x in lines))


def _same_bits(a, b, what):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    assert a.shape == b.shape, what
    assert a.tobytes() == b.tobytes(), what


CASES = ("channel_two_types", "suspension", "no_cells")
LOAD_CASES = CASES + ("crlf", "respelled")


def _respell(directory):
    """The coordinates of SDPDParCoor.txt and CELLParStruct.txt in other
    spellings of their values, one per column (%.7E, fixed with 8 decimals,
    an explicit plus sign with %.9g): every field still fits its 20
    characters."""
    fmts = ("{:<20.7E}", "{:<20.8f}", "{:<+20.9g}")
    for name in ("SDPDParCoor.txt", "CELLParStruct.txt"):
        path = os.path.join(directory, name)
        out = []
        for line in open(path).read().split("\n"):
            cols = [line[i:i + 20] for i in range(0, len(line), 20)]
            if len(cols) == 3 and all("." in c or "e" in c for c in cols):
                line = "".join(f.format(float(c)) for f, c in zip(fmts, cols))
            out.append(line)
        open(path, "w").write("\n".join(out))


def _crlf(directory):
    for name in os.listdir(directory):
        path = os.path.join(directory, name)
        data = open(path, "rb").read()
        open(path, "wb").write(data.replace(b"\n", b"\r\n"))


def _write_case(name, directory):
    os.makedirs(directory, exist_ok=True)
    if name == "channel_two_types":
        cfg = gen.channel(nx=24, ny=12, nz=18, wall_layers=3, cell_subdiv=1, cell_diameter=3.0,
                          cell_centers=[(0.0, -0.6, 0.0), (0.0, 0.6, 0.0)], seed=2)
        _two_types(directory, cfg)
    elif name == "suspension":
        cfg = gen.suspension(nx=16, ny=16, nz=16, ncells=2, subdiv=2, hematocrit=0.12, seed=3)
        gen.write_reference_inputs(cfg, str(directory))
    else:
        cfg = gen.suspension(nx=16, ny=16, nz=16, ncells=0, seed=5)
        gen.write_reference_inputs(cfg, str(directory))
    return cfg


@pytest.mark.parametrize("case", LOAD_CASES)
def test_reader_reads_what_the_reference_loaders_read(built_library, tmp_path, case):
    d = tmp_path / "in"
    _write_case("channel_two_types" if case in ("crlf", "respelled") else case, d)
    if case == "crlf":
        _crlf(d)
    elif case == "respelled":
        _respell(d)
    ref = _ref_load(d, tmp_path)
    ours = read_inputs(str(d))
    for k in ("n_b1", "n_b2", "n_fluid", "ncell", "ntri", "nedge", "ncp"):
        assert ours[k] == ref[k], k
    if ref["ncell"]:
        assert ours["ntype"] == ref["ntype"]
    names = ("sound1", "sound2", "shear_vis", "bulk_vis", "den_init", "ext_force", "max_cut", "zero_len",
             "sca_fac", "sur_energy")
    n_params = 10 if ref["ncell"] else 6   # the cell parameters are read only with cells
    for k, v in zip(names[:n_params], ref["params"][:n_params]):
        _same_bits(np.float32(ours[k]), v, k)
    _same_bits(np.concatenate([ours["sdpd_coor"], ours["cell_coor"]]).astype(np.float32), ref["coor"], "coordinates")
    if ref["ncell"]:
        for k in ("cell_type", "npar", "ntri_cell", "betri", "tri", "edge", "celltab"):
            _same_bits(ours[k].astype(np.int32).ravel(), ref[k], k)
        first = np.concatenate([[0], np.cumsum(ref["npar"])[:-1]])
        _same_bits(np.stack([first, first + ref["npar"] - 1], 1).astype(np.int32).ravel(), ref["verts"], "verts")
        for k in ("shear_e", "bend_e", "hl_t", "hg_t", "hv_t", "shear_mod", "bending_mod", "hgarea", "hlarea",
                  "hvol"):
            _same_bits(ours[k].astype(np.float32).ravel(), ref[k], k)


def _frame(cfg, rng):
    n, ncp, ncell, ntri = cfg.n, cfg.ncp, cfg.ncell, cfg.ntri
    f32 = lambda *s: (rng.normal(size=s) * 3).astype(np.float32)
    return dict(pos=f32(n, 3), vel=np.concatenate([f32(n, 3), rng.uniform(25, 29, (n, 1)).astype(np.float32)], 1),
                press=f32(n) * 30, defforce=f32(ncp, 3), aggforce=f32(ncp, 3) * 1e-3,
                area=rng.uniform(80, 90, ncell).astype(np.float32), vol=rng.uniform(50, 60, ncell).astype(np.float32),
                trinordir=f32(ntri, 3), tricenter=f32(ntri, 3))


def _ref_write(directory, fr, slot_ids, step_data, step_count):
    n = fr["pos"].shape[0]
    ncp, ncell, ntri = fr["defforce"].shape[0], fr["area"].shape[0], fr["tricenter"].shape[0]
    path = os.path.join(directory, "frame.bin")
    with open(path, "wb") as f:
        f.write(np.array([n, ncp, ncell, ntri, step_data, step_count], "<i8").tobytes())
        for a in (fr["pos"][slot_ids], fr["vel"][slot_ids], fr["press"][slot_ids]):
            f.write(np.ascontiguousarray(a, "<f4").tobytes())
        f.write(np.ascontiguousarray(slot_ids, "<i4").tobytes())
        for k in ("defforce", "aggforce", "area", "vol", "trinordir", "tricenter"):
            f.write(np.ascontiguousarray(fr[k], "<f4").tobytes())
    _ref("write", directory, path)


def _verts(cfg):
    """First and last membrane index of each cell (inclusive)."""
    first = np.concatenate([[0], np.cumsum(cfg.npar)[:-1]]).astype(np.int32)
    return np.stack([first, first + np.asarray(cfg.npar, np.int32) - 1], 1)


def _cell_means(cfg, fr, slot_ids):
    """Per-cell means as the reference's writers form them: FP32 sums over
    the slots in order, divided by the vertex count (src/Particle.cu:1036-1081,
    1175-1196); |mean velocity| from FP32 squares."""
    stats = np.zeros((cfg.ncell, 12))
    mem = slot_ids - cfg.n_cell_start   # membrane index of each slot
    verts = _verts(cfg)
    for c in range(cfg.ncell):
        a, b = verts[c]
        sel = np.flatnonzero((mem >= a) & (mem <= b))
        k = mem[sel]
        npar = np.float32(b - a + 1)

        def mean(v):
            return np.cumsum(v.astype(np.float32), axis=0, dtype=np.float32)[-1] / npar

        stats[c, 0:3] = mean(fr["defforce"][k])
        stats[c, 3:6] = mean(fr["aggforce"][k])
        v = mean(fr["vel"][slot_ids[sel], :3])
        stats[c, 6:9] = v
        stats[c, 9] = np.sqrt(np.float32(v[0] * v[0]) + np.float32(v[1] * v[1]) + np.float32(v[2] * v[2]),
                              dtype=np.float32)
        stats[c, 10], stats[c, 11] = fr["area"][c], fr["vol"][c]
    return stats


def _ours(cfg, fr, out_dir, step_data, first, stats):
    t = np.float32(np.float32(step_data) * TIME_STEP) * STEP_OUTPUT
    cells = cfg.ncell > 0
    write_frame(str(out_dir), step_data, float(t), first, pos=fr["pos"], vel=fr["vel"][:, :3],
                rho=fr["vel"][:, 3], press=fr["press"], n_b1=cfg.n_b1, n_b2=cfg.n_b2, n_cell_start=cfg.n_cell_start,
                cell_verts=_verts(cfg) if cells else None, tri=cfg.tri if cells else None,
                betri=cfg.betri if cells else None, defforce=fr["defforce"] if cells else None,
                aggforce=fr["aggforce"] if cells else None, tricenter=fr["tricenter"] if cells else None,
                trinordir=fr["trinordir"] if cells else None, cell_stats=stats if cells else None)


def _files(root):
    out = {}
    for r, _, fl in os.walk(root):
        for f in fl:
            p = os.path.join(r, f)
            out[os.path.relpath(p, root)] = open(p, "rb").read()
    return out


@pytest.mark.parametrize("case", CASES)
def test_writer_writes_what_the_reference_writers_write(built_library, tmp_path, case):
    d = tmp_path / "ref"
    cfg = _write_case(case, d)
    rng = np.random.default_rng(7)
    ids = np.arange(cfg.n, dtype=np.int32)   # SortPart: slot s holds particle s
    for step_data, step_count in ((0, 0), (3, 300)):   # a first output step, then one appended
        fr = _frame(cfg, rng)
        _ref_write(d, fr, ids, step_data, step_count)
        stats = _cell_means(cfg, fr, ids) if cfg.ncell else None
        _ours(cfg, fr, tmp_path / "ours", step_data, step_count == 0, stats)
    ref, ours = _files(d / "Result"), _files(tmp_path / "ours")
    assert sorted(ref) == sorted(ours)
    # per output step FluidCoor and FluidField, with cells CellCoor, CellForce
    # and CellNorDir too; one TF_Cell and one Geo_Cell series per cell
    assert len(ref) == 2 * (2 + (3 if cfg.ncell else 0)) + 2 * cfg.ncell
    for name in ref:
        assert ours[name] == ref[name], name


def _zones(text):
    zones, cur = [], None
    for line in text.decode().splitlines():
        if line.startswith("Zone"):
            cur = []
            zones.append(cur)
        elif cur is not None:
            cur.append(line)
    return [sorted(z) for z in zones]


def test_permuted_slots_give_the_same_rows(built_library, tmp_path):
    d = tmp_path / "ref"
    cfg = _write_case("channel_two_types", d)
    rng = np.random.default_rng(11)
    ids = rng.permutation(cfg.n).astype(np.int32)   # slot s holds particle ids[s]
    fr = _frame(cfg, rng)
    _ref_write(d, fr, ids, 1, 0)
    _ours(cfg, fr, tmp_path / "ours", 1, True, _cell_means(cfg, fr, np.arange(cfg.n, dtype=np.int32)))
    ref, ours = _files(d / "Result"), _files(tmp_path / "ours")
    coor = os.path.join("FluidCoor", "1.plt")
    assert _zones(ref[coor]) == _zones(ours[coor])
    field = os.path.join("FluidField", "1.plt")
    assert sorted(ref[field].splitlines()) == sorted(ours[field].splitlines())
    nordir = os.path.join("CellNorDir", "1.plt")
    assert ref[nordir] == ours[nordir]
