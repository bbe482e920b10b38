"""The library's loader of GPUCell's four input files (gc_input_*), without
a GPU:

* the files the generator writes read back to the configuration exactly
  (positions are written with 9 significant digits, enough for FP32), and
  equal the Python restatement of the reference's parsing rules
  (generator.read_reference_inputs);
* several cell types spread their moduli over the cells' edges and
  triangles (src/Particle.cu:355-375);
* the binary form round-trips the set bit for bit;
* more wall + fluid particles than the reference's fixed 2,000,000-entry
  array (src/Particle.cu:31) load;
* truncated or missing files are refused.
"""
import os

import numpy as np
import pytest

from gpucell_gb300 import generator as gen
from gpucell_gb300.inputs import read_binary, read_inputs, to_config, write_binary


def test_text_files_read_back_exactly(built_library, tmp_path):
    cfg = gen.small_channel()
    gen.write_reference_inputs(cfg, str(tmp_path))
    d = read_inputs(str(tmp_path))
    assert (d["n_b1"], d["n_b2"], d["n_fluid"], d["ncell"]) == (cfg.n_b1, cfg.n_b2, cfg.n_fluid, cfg.ncell)
    np.testing.assert_array_equal(d["sdpd_coor"], cfg.coor[:cfg.n_cell_start])
    np.testing.assert_array_equal(d["cell_coor"], cfg.coor[cfg.n_cell_start:])
    for k in ("tri", "edge", "betri", "celltab"):
        np.testing.assert_array_equal(d[k], getattr(cfg, k), err_msg=k)
    py = gen.read_reference_inputs(str(tmp_path))
    for k in ("sdpd_coor", "cell_coor", "tri", "edge", "betri", "celltab"):
        np.testing.assert_array_equal(d[k], py[k], err_msg=k)
    assert d["den_init"] == pytest.approx(cfg.den_init, rel=1e-6)
    p = cfg.phys
    assert (d["shear_mod"][0], d["bending_mod"][0], d["hvol"][0]) == (p.shear_mod, p.bending_mod, p.hvol)
    back = to_config(d, phys=p, bbox=cfg.bbox, pmask=cfg.pmask)
    for a, b in zip(back.edge_params(), cfg.edge_params()):
        np.testing.assert_array_equal(a, b)
    ka, kb = back.consts(), cfg.consts()
    assert ka.keys() == kb.keys()
    for k in ka:   # the files carry FP32 values
        assert np.float32(ka[k]) == np.float32(kb[k]), k


def test_cell_types_spread_their_moduli(built_library, tmp_path):
    cfg = gen.channel(nx=24, ny=12, nz=18, wall_layers=3, cell_subdiv=1, cell_diameter=3.0,
                      cell_centers=[(0.0, -0.6, 0.0), (0.0, 0.6, 0.0)], seed=2)
    cfg.cell_type = np.array([2, 1], np.int32)
    gen.write_reference_inputs(cfg, str(tmp_path))
    lines = ["nType", "2", "ShearMod", "100", "7", "BendingMod", "50", "3", "HGarea", "5000", "11", "HLarea",
             "100", "13", "HVol", "5000", "17", "MaxCut", "0", "zeroLen", "0", "scaFac", "0", "surEnergy", "0"]
    with open(tmp_path / "CELLPhyPara.txt", "w") as f:
        f.write("".join((x if not x[0].isdigit() else f"{x:<20}") + "\n" for x in lines))
    d = read_inputs(str(tmp_path))
    ne0, nt0 = cfg.ntri_cell[0] * 3 // 2, cfg.ntri_cell[0]
    assert np.all(d["shear_e"][:ne0] == 7) and np.all(d["shear_e"][ne0:] == 100)
    assert np.all(d["hv_t"][:nt0] == 17) and np.all(d["hv_t"][nt0:] == 5000)
    assert np.all(d["bend_e"][:ne0] == 3) and np.all(d["hg_t"][nt0:] == 5000)


def test_binary_round_trip(built_library, tmp_path):
    cfg = gen.small_channel()
    gen.write_reference_inputs(cfg, str(tmp_path / "txt"))
    write_binary(str(tmp_path / "txt"), str(tmp_path / "set.bin"))
    a, b = read_inputs(str(tmp_path / "txt")), read_binary(str(tmp_path / "set.bin"))
    for k in a:
        if isinstance(a[k], np.ndarray):
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
        else:
            assert a[k] == b[k], k
    write_binary(a, str(tmp_path / "set2.bin"))
    assert open(tmp_path / "set.bin", "rb").read() == open(tmp_path / "set2.bin", "rb").read()


def test_more_particles_than_the_reference_arrays_hold(built_library, tmp_path):
    n = 2_000_100
    rng = np.random.default_rng(0)
    pos = rng.uniform(0, 20, size=(n, 3)).astype(np.float32)
    with open(tmp_path / "SDPDParCoor.txt", "w") as f:
        f.write("nBound1 nBound2 nFluid\n" + f"{0:<20}{0:<20}{n:<20}\n" + "Bound1 x y z\nBound2 x y z\nFluid x y z\n")
        np.savetxt(f, pos, fmt="%-20.9g%-20.9g%-20.9g", delimiter="")
    for name, body in (("SDPDPhyPara.txt", "S\n20\n20\nV\n10\nB\n0\nD\n27\nF\n0.02\n"),
                       ("CELLParStruct.txt", "nCell\n0\n")):
        (tmp_path / name).write_text(body)
    d = read_inputs(str(tmp_path))
    assert d["n_fluid"] == n
    np.testing.assert_array_equal(d["sdpd_coor"][[0, n // 2, n - 1]], pos[[0, n // 2, n - 1]])


def test_bad_files_are_refused(built_library, tmp_path):
    from gpucell_gb300 import _lib
    with pytest.raises(_lib.GcError, match="cannot open"):
        read_inputs(str(tmp_path))
    cfg = gen.small_channel()
    gen.write_reference_inputs(cfg, str(tmp_path))
    text = open(tmp_path / "CELLParStruct.txt").read().split("\n")
    (tmp_path / "CELLParStruct.txt").write_text("\n".join(text[: len(text) // 2]))
    with pytest.raises(_lib.GcError, match="ends early"):
        read_inputs(str(tmp_path))
    (tmp_path / "x.bin").write_bytes(b"GCINPUT1" + b"\0" * 20)
    with pytest.raises(_lib.GcError, match="truncated|corrupt|not a binary"):
        read_binary(str(tmp_path / "x.bin"))


def _field_strings(seed=11, n=30000):
    """Numbers as GPUCell's 20-character columns may hold them: printf
    formats of many widths and precisions, magnitudes from 1e-40 to 1e38,
    signs, leading spaces, integers, long mantissas and exponents beyond
    the exact fast path, and inf/nan."""
    rng = np.random.default_rng(seed)
    mags = 10.0 ** rng.uniform(-40, 38, n)
    vals = mags * rng.choice([-1.0, 1.0], n)
    fmts = ["%.5e", "%.9g", "%.17g", "%f", "%.3E", "%+.7e", "%.12f", "%g", "%.0f", "%.1e", "%.19g"]
    out = []
    for k, v in enumerate(vals):
        s = fmts[k % len(fmts)] % v
        if len(s) > 19:
            s = "%.9g" % v
        out.append(s)
    out += ["0", "-0", "0.0", "-0.000", "1", "-1", "123456789012345678", "1e22", "1e23", "9007199254740993",
            "0.1", "0.30000000000000004", "1.7976931348623e308", "4.9e-324", "2.225073858507e-308",
            "inf", "-inf", "nan", "1e-400", "1e400", "  3.5", "+2.5", "1.e5", ".5", "5.", "00012.5000"]
    return out


def test_decimal_fields_read_like_atof(built_library, tmp_path):
    """Every 20-character field converts to the float32 of the correctly
    rounded double, as the reference's atof followed by the assignment to a
    float does (the loader takes an exact fast path for short decimals and
    strtod for the rest)."""
    cfg = gen.small_channel()
    gen.write_reference_inputs(cfg, str(tmp_path))
    strs = _field_strings()
    n = (len(strs) + 2) // 3
    strs += ["0"] * (3 * n - len(strs))
    with open(tmp_path / "SDPDParCoor.txt", "w") as f:
        f.write("nBound1 nBound2 nFluid\n")
        f.write("%-20d%-20d%-20d\n" % (0, 0, n))
        f.write("Bound1 x y z\nBound2 x y z\nFluid x y z\n")
        for r in range(n):
            f.write("".join("%-20s" % s for s in strs[3 * r:3 * r + 3]) + "\n")
    got = read_inputs(str(tmp_path))["sdpd_coor"].reshape(-1)
    assert max(len(s) for s in strs) <= 20   # a column holds 20 characters
    with np.errstate(over="ignore"):
        want = np.array([np.float32(float(s)) for s in strs], np.float32)
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan)
    assert np.array_equal(got[~nan].view(np.uint32), want[~nan].view(np.uint32))
