"""GPUCell's output files (OutputPar, src/Particle.cu:681-1300), written by
the library from host arrays, checked line by line against a restatement of
the reference's writers in this file (left-aligned fields 20 wide, 15 in the
per-cell time series, `%.5e` floats; zone layout as in
OutputCoor/OutputField/OutPutCellCoor/OutPutCellForce/OutPutCellGeo/
OutPutTriNorDir).  No GPU: only the host writer runs.
"""
import os

import numpy as np

from gpucell_gb300.output import read_plt, write_frame


def e20(v):
    return "%-20.5e" % float(np.float32(v))


def d20(v):
    return "%-20d" % int(v)


def e15(v):
    return "%-15.5e" % float(np.float32(v))


def _frame(seed=0):
    rng = np.random.default_rng(seed)
    n_b1, n_b2, n_fl = 3, 4, 9
    # two cells: a tetrahedron (4 vertices, 4 triangles) and a pyramid (5 vertices, 6 triangles)
    tri = np.array([[1, 2, 3], [1, 2, 4], [1, 3, 4], [2, 3, 4],
                    [5, 6, 7], [5, 7, 8], [5, 8, 9], [5, 9, 6], [6, 7, 8], [6, 8, 9]], np.int32)
    ncp = 9
    n = n_b1 + n_b2 + n_fl + ncp
    fr = dict(pos=rng.normal(size=(n, 3)) * 3, vel=rng.normal(size=(n, 3)), rho=rng.uniform(26, 28, n),
              press=rng.normal(size=n) * 100, n_b1=n_b1, n_b2=n_b2, n_cell_start=n_b1 + n_b2 + n_fl,
              cell_verts=np.array([[0, 3], [4, 8]], np.int32), tri=tri, betri=np.array([[0, 3], [4, 9]], np.int32),
              defforce=rng.normal(size=(ncp, 3)), aggforce=rng.normal(size=(ncp, 3)) * 1e-3,
              tricenter=rng.normal(size=(10, 3)), trinordir=rng.normal(size=(10, 3)),
              cell_stats=rng.normal(size=(2, 12)))
    return fr


def _expected_coor(fr):
    n, b1, b2, cs = fr["pos"].shape[0], fr["n_b1"], fr["n_b2"], fr["n_cell_start"]
    out = ["Title=\"Particle Coordinate\"", "Variables=\"x\",\"y\",\"z\",\"SP\""]
    for lo, hi in ((0, b1), (b1, b1 + b2), (b1 + b2, cs), (cs, n)):
        if hi > lo:
            out.append("%-20s" % "Zone")
            out += [e20(fr["pos"][i, 0]) + e20(fr["pos"][i, 1]) + e20(fr["pos"][i, 2]) + d20(i) for i in range(lo, hi)]
    return out


def _expected_field(fr):
    out = ["Title=\"Particle Fluid\"", "Variables=\"x\",\"y\",\"z\",\"Den\",\"Press\",\"Vx\",\"Vy\",\"Vz\""]
    for i in range(fr["n_cell_start"]):
        p, v = fr["pos"][i], fr["vel"][i]
        out.append("".join(e20(x) for x in (p[0], p[1], p[2], fr["rho"][i], fr["press"][i], v[0], v[1], v[2])))
    return out


def _expected_cells(fr, forces):
    out = ["Title=\"Particle Force\"" if forces else "Title=\"Particle Coordinate\"",
           "Variables=\"x\",\"y\",\"z\", \"DFx\",\"DFy\",\"DFz\",\"AFx\",\"AFy\",\"AFz\"" if forces
           else "Variables=\"x\",\"y\",\"z\""]
    cs = fr["n_cell_start"]
    for (v0, v1), (t0, t1) in zip(fr["cell_verts"], fr["betri"]):
        out.append(f"Zone N={v1 - v0 + 1}, E={t1 - t0 + 1}, F=FEPOINT, ET=TRIANGLE")
        for m in range(v0, v1 + 1):
            row = [fr["pos"][cs + m, a] for a in range(3)]
            if forces:
                row += list(fr["defforce"][m]) + list(fr["aggforce"][m])
            out.append("".join(e20(x) for x in row))
        for t in range(t0, t1 + 1):
            out.append("".join(d20(fr["tri"][t, a] - 1 - v0 + 1) for a in range(3)))
    return out


def _expected_nordir(fr):
    out = ["Title=\"Triangle information\"", "Variables=\"Cenx\",\"Ceny\",\"Cenz\",\"Norx\",\"Nory\",\"Norz\",\"ID\""]
    for t0, t1 in fr["betri"]:
        out.append("%-20s" % "Zone")
        for t in range(t0, t1 + 1):
            out.append("".join(e20(x) for x in list(fr["tricenter"][t]) + list(fr["trinordir"][t])) + d20(t))
    return out


def _lines(path):
    with open(path) as f:
        return f.read().split("\n")[:-1]


def test_step_files_match_the_reference_layout(built_library, tmp_path):
    fr = _frame()
    d = str(tmp_path / "Result")
    write_frame(d, 7, 0.5, True, **fr)
    assert _lines(os.path.join(d, "FluidCoor", "7.plt")) == _expected_coor(fr)
    assert _lines(os.path.join(d, "FluidField", "7.plt")) == _expected_field(fr)
    assert _lines(os.path.join(d, "CellCoor", "7.plt")) == _expected_cells(fr, False)
    assert _lines(os.path.join(d, "CellForce", "7.plt")) == _expected_cells(fr, True)
    assert _lines(os.path.join(d, "CellNorDir", "7.plt")) == _expected_nordir(fr)


def test_time_series_start_then_append(built_library, tmp_path):
    d = str(tmp_path / "Result")
    a, b = _frame(1), _frame(2)
    write_frame(d, 0, 0.0, True, **a)
    write_frame(d, 1, 0.25, False, **b)
    for c in range(2):
        tf = _lines(os.path.join(d, "CellForce", f"TF_Cell{c}.plt"))
        geo = _lines(os.path.join(d, "CellGeo", f"Geo_Cell{c}.plt"))
        assert tf == ["".join(e15(x) for x in [t] + list(fr["cell_stats"][c, :6])) for t, fr in ((0.0, a), (0.25, b))]
        assert geo == ["".join(e15(x) for x in [t] + list(fr["cell_stats"][c, 9:12])) for t, fr in ((0.0, a), (0.25, b))]
    write_frame(d, 2, 0.5, True, **a)                 # first again: the series start over
    assert len(_lines(os.path.join(d, "CellGeo", "Geo_Cell0.plt"))) == 1


def test_many_threads_give_the_same_text(built_library, tmp_path):
    rng = np.random.default_rng(3)
    n = 50000
    fr = dict(pos=rng.normal(size=(n, 3)), vel=rng.normal(size=(n, 3)), rho=rng.uniform(size=n),
              press=rng.normal(size=n), n_b1=100, n_b2=200, n_cell_start=n)
    write_frame(str(tmp_path / "a"), 0, 0.0, True, threads=1, **fr)
    write_frame(str(tmp_path / "b"), 0, 0.0, True, threads=8, **fr)
    for sub in ("FluidCoor", "FluidField"):
        assert open(tmp_path / "a" / sub / "0.plt").read() == open(tmp_path / "b" / sub / "0.plt").read()
    zones = read_plt(str(tmp_path / "b" / "FluidCoor" / "0.plt"))
    assert [z["rows"].shape[0] for z in zones] == [100, 200, n - 300]
    np.testing.assert_allclose(zones[2]["rows"][:, :3], fr["pos"][300:], rtol=1e-5)


def test_bad_frames_are_refused(built_library, tmp_path):
    import pytest
    from gpucell_gb300 import _lib
    fr = _frame()
    fr["tri"] = fr["tri"].copy()
    fr["tri"][0, 0] = 7           # a vertex of the other cell
    with pytest.raises(_lib.GcError, match="vertex of another cell"):
        write_frame(str(tmp_path), 0, 0.0, True, **fr)


def _hard_floats(seed=3):
    """Floats that stress a %.5e formatter: random bit patterns over the whole
    exponent range, decimal ties at the sixth digit (integers n*10+5 below
    2^24 and their binary scalings) and the floats next to them, powers of
    ten and their neighbours, log-uniform values over the range the double
    path serves (1e-12 to 1e16), the float extremes, subnormals, signed
    zeros, infinities and NaN."""
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 2**32, size=60000, dtype=np.uint64).astype(np.uint32)
    vals = [bits.view(np.float32)]
    ties = (rng.integers(100000, 1677721, size=4000) * 10 + 5).astype(np.float32)
    vals += [ties, ties * np.float32(2.0**-20), ties * np.float32(2.0**30), -ties]
    vals += [np.nextafter(ties, np.float32(np.inf)), np.nextafter(ties, np.float32(0))]
    vals.append((10.0 ** rng.uniform(-12, 16, size=100000)).astype(np.float32))
    p10 = np.array([10.0**e for e in range(-15, 39)], np.float64).astype(np.float32)
    vals += [p10, np.nextafter(p10, np.float32(np.inf)), np.nextafter(p10, np.float32(0)), -p10]
    fi = np.finfo(np.float32)
    vals.append(np.array([0.0, -0.0, fi.max, -fi.max, fi.tiny, fi.tiny * np.float32(0.5), 1e-16, 9.999995e-16,
                          np.inf, -np.inf, np.nan, 999999.5, 9.999995, 0.9999995, 1.0, -1.0], np.float32))
    return np.concatenate(vals).astype(np.float32)


def test_float_formatting_matches_printf(built_library, tmp_path):
    """The writer formats floats itself (six digits by double arithmetic where
    the rounding is certain, by exact integer arithmetic otherwise); every
    value must come out as printf's %-20.5e would write it."""
    v = _hard_floats()
    n = v.size // 3 * 3
    pos = v[:n].reshape(-1, 3)
    m = pos.shape[0]
    fr = dict(pos=pos, vel=np.zeros((m, 3), np.float32), rho=np.zeros(m, np.float32), press=np.zeros(m, np.float32),
              n_b1=0, n_b2=0, n_cell_start=m, cell_verts=np.zeros((0, 2), np.int32), tri=np.zeros((0, 3), np.int32),
              betri=np.zeros((0, 2), np.int32), defforce=np.zeros((0, 3), np.float32),
              aggforce=np.zeros((0, 3), np.float32), tricenter=np.zeros((0, 3), np.float32),
              trinordir=np.zeros((0, 3), np.float32), cell_stats=np.zeros((0, 12)))
    d = str(tmp_path / "Result")
    write_frame(d, 0, 0.0, True, **fr)
    got = _lines(os.path.join(d, "FluidCoor", "0.plt"))[3:]
    assert len(got) == m
    def c_e20(x):   # printf writes a NaN with its sign bit set as -nan (Python: nan)
        if np.isnan(x):
            return "%-20s" % ("-nan" if np.signbit(x) else "nan")
        return e20(x)

    for i in range(m):
        want = c_e20(pos[i, 0]) + c_e20(pos[i, 1]) + c_e20(pos[i, 2]) + d20(i)
        assert got[i] == want, (i, pos[i], got[i], want)
