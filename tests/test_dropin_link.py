"""GPUCell's own host frame links against the library with nothing missing.

The reference's src/main.cu and src/Particle.cu are compiled where they lie
(only in the development container; the reference is not shipped) and
linked against libgpucell_gb300.so in place of the absent ParticleGPU.o and
ConfigDomain.o (src/makefile:7-18).  Nothing is run: that needs the
reference's input files and a GPU.
"""
import os
import shutil
import subprocess

import pytest

from gpucell_gb300.build import reference_src

REF_SRC = reference_src()


@pytest.mark.slow
def test_reference_host_frame_links(built_library, tmp_path):
    if not os.path.isdir(REF_SRC):
        pytest.skip("reference sources are not present on this machine")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    objs = []
    for name in ("main.cu", "Particle.cu"):
        obj = tmp_path / (name[:-3] + ".o")
        subprocess.run([nvcc, "-w", "-c", os.path.join(REF_SRC, name), "-o", str(obj)], check=True,
                       capture_output=True)
        objs.append(str(obj))
    nm = subprocess.run(["nm", "-C", "--undefined-only"] + objs, capture_output=True, text=True).stdout
    boundary = sorted({ln.split("U ", 1)[1] for ln in nm.splitlines() if "cupar::" in ln or "cudiv::" in ln})
    assert len(boundary) == 20, boundary
    libdir = os.path.dirname(built_library)
    exe = tmp_path / "sdpdgpu"
    res = subprocess.run([nvcc] + objs + ["-o", str(exe), "-L" + libdir, "-lgpucell_gb300",
                                          "-Xlinker", "-rpath=" + libdir, "-Xlinker", "--no-undefined"],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    assert exe.exists()
