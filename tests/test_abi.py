"""The C ABI and the C++ drop-in symbols, checked without a GPU."""
import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gpucell_gb300.h")

# The 20 entry points of src/ParticleGPU.cuh:10-35 and src/ConfigDomain.cuh:11-17.
CUPAR = ["ConstsDataUp", "UpdateFluidCoor", "AppFluidPeriodicBC", "CalFluidDen", "PredictFluidVel", "CalBound2Vel",
         "EOS", "CalFluidSDPDForce", "CalFluidRepForce", "SetFluidExtForce", "CorrectFliudVel", "CalGeoPara",
         "SetMechPara", "CalCellDefForce", "CalCellAggForce"]
CUDIV = ["PreConList", "Sort", "CalBeginEndCube", "SortBasicArrays", "SortArraysWithCells", "Printf"]


def declared_c_functions():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*|long long|unsigned long long)\s+(gc_\w+)\s*\(", txt, re.M)))


def test_structconst_layout():
    from gpucell_gb300._lib import Structconst
    assert C.sizeof(Structconst) == 96
    assert Structconst.iSeed.offset == 24
    assert Structconst.CutRadius.offset == 32
    assert Structconst.Temp.offset == 88


def test_option_and_system_records_match_the_header():
    from gpucell_gb300._lib import GcFusedOptions, GcSystemDesc
    assert C.sizeof(GcFusedOptions) == 32 and GcFusedOptions.graph.offset == 16
    assert C.sizeof(GcSystemDesc) == 128
    assert GcSystemDesc.bbox.offset == 96 and GcSystemDesc.periodic_mask.offset == 120
    txt = open(HEADER).read()
    assert GcFusedOptions.tiles.offset == 20 and GcFusedOptions.half_velocity.offset == 28
    assert "int graph;" in txt and "int tiles;" in txt and "int fp32_positions;" in txt and "int half_velocity;" in txt
    assert "Structconst consts;" in txt


def test_library_exports_every_declared_function(built_library):
    lib = C.CDLL(built_library)
    names = declared_c_functions()
    assert len(names) >= 33   # 11 controls, 15 cupar, 6 cudiv, 1 test hook
    for n in names:
        assert hasattr(lib, n), n
    from gpucell_gb300 import _lib
    assert set(_lib.exported_symbols()) == set(names)


def test_controls_without_gpu(built_library):
    from gpucell_gb300 import _lib
    lib = _lib.load()
    assert lib.gc_version() > 0
    assert lib.gc_set_periodic(5) == 0 and lib.gc_get_periodic() == 5
    assert lib.gc_set_periodic(9) != 0 and b"mask" in lib.gc_last_error()
    assert lib.gc_set_periodic(1) == 0
    # entry points validate before touching the device
    assert lib.gc_cupar_ConstsDataUp(None) == -1
    assert lib.gc_cudiv_Sort(-1, None, None) == -1


def test_cpp_symbols_link(built_library, tmp_path):
    """A C++ caller of the 20 cupar::/cudiv:: functions, declared by
    include/gpucell/cupar.h, links against the library."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "caller.cu"
    refs = "\n".join(f"    (void*)&cupar::{n}," for n in CUPAR) + "\n" + \
           "\n".join(f"    (void*)&cudiv::{n}," for n in CUDIV)
    src.write_text('#include "gpucell/cupar.h"\n#include <cstdio>\nint main(){ void* f[] = {\n' + refs +
                   '\n  };\n  printf("%d\\n", (int)(sizeof(f)/sizeof(f[0])));\n  return 0; }\n')
    libdir = os.path.dirname(built_library)
    subprocess.run([nvcc, "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(tmp_path / "caller"),
                    "-L" + libdir, "-lgpucell_gb300", "-Xlinker", "-rpath=" + libdir], check=True,
                   capture_output=True)
    out = subprocess.run([str(tmp_path / "caller")], capture_output=True, text=True)
    assert out.stdout.strip() == "21"
