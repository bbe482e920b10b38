"""GPUCell's own step driver, run on the host against recording entry
points, against what this repository assumes of it.

oracle/_ref/ref_calls (built by oracle/ref_io.mk from the reference's
src/Particle.cu and src/main.cu where they lie, only where the reference's
sources are present; the tests skip elsewhere) links Particle.cu against
recorders of the 20 boundary entry points and runs Particle::DrivePar +
Particle::UpdatePar (src/Particle.cu:1302-1329), after the parts of the
set-up that touch no device memory.  The trace is the sequence of boundary
calls the reference makes, with the counts it passes.

* The fused engine behind the entry points (GPUCELL_ENGINE=fused) takes
  UpdateFluidCoor as the first call of every step and runs the whole step at
  SetFluidExtForce, which carries DriveOn; the calls after it only record
  their buffers.  The reference's trace has that shape at every step.
* The host-frame mirror (gpucell_gb300/host.py, which the GPU tests drive)
  makes the reference's calls in the reference's order with the same counts,
  recorded here without a GPU.  It differs in two ways, both asserted: its
  set-up also makes the CalGeoPara and SetMechPara calls that SetPar makes
  itself (src/Particle.cu:476-480), which the recorder cannot run because
  SetPar allocates device memory first; and without cells it leaves out the
  membrane calls (CalGeoPara, SetMechPara, CalCellDefForce,
  CalCellAggForce) that the entry points return from at once with nCell 0.
"""
import numbers
import os
import subprocess

import pytest

from gpucell_gb300 import generator as gen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_CALLS = os.path.join(ROOT, "oracle", "_ref", "ref_calls")
STEPS = 3
MEMBRANE = ("CalGeoPara", "SetMechPara", "CalCellDefForce", "CalCellAggForce")
AFTER_EXT_FORCE = ["CalGeoPara", "CalCellDefForce", "CalCellAggForce", "CorrectFliudVel", "CalBound2Vel"]

pytestmark = pytest.mark.skipif(not os.path.exists(REF_CALLS),
                                reason="the reference's step driver is built only where its sources are")


def _config(name):
    if name == "channel":
        return gen.small_channel()
    if name == "suspension":
        return gen.suspension(nx=16, ny=16, nz=16, ncells=2, subdiv=2, hematocrit=0.12, seed=3)
    return gen.suspension(nx=16, ny=16, nz=16, ncells=0, seed=5)


def _sections(lines):
    """{"setup": [...], "steps": [[...], ...]} from a trace."""
    out = {"setup": [], "steps": []}
    cur = None
    for ln in lines:
        if ln == "setup":
            cur = out["setup"]
        elif ln == "step":
            out["steps"].append([])
            cur = out["steps"][-1]
        else:
            cur.append(ln)
    return out


def _reference_trace(cfg, tmp_path):
    d = tmp_path / "in"
    gen.write_reference_inputs(cfg, str(d))
    trace = tmp_path / "trace.txt"
    res = subprocess.run([REF_CALLS, str(d), str(STEPS), str(trace)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    return _sections(trace.read_text().splitlines())


def _mirror_trace(cfg, monkeypatch):
    import torch

    from gpucell_gb300 import _lib, host
    lines = []

    def record(name, *args):
        if name.startswith(("gc_cupar_", "gc_cudiv_")):
            short = name.split("_", 2)[2]
            ints = [int(a) for a in args if isinstance(a, numbers.Integral)]
            if short == "CalBeginEndCube":
                ints = ints[:1]   # the recorder leaves SizeCube out (ConfigDomain sets it)
            lines.append(" ".join([short] + [str(v) for v in ints]))
        return 0

    monkeypatch.setattr(_lib, "call", record)
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    lines.append("setup")
    ps = host.ParticleSystem(cfg, device="cpu", noise=False)
    for _ in range(STEPS):
        lines.append("step")
        ps.update()
    return _sections(lines)


@pytest.mark.parametrize("case", ("channel", "suspension", "no_cells"))
def test_reference_steps_have_the_shape_the_engine_relies_on(built_library, tmp_path, case):
    cfg = _config(case)
    ref = _reference_trace(cfg, tmp_path)
    assert len(ref["steps"]) == STEPS
    for k, step in enumerate(ref["steps"]):
        names = [ln.split()[0] for ln in step]
        assert names[0] == "UpdateFluidCoor"
        assert names.count("UpdateFluidCoor") == 1 and names.count("SetFluidExtForce") == 1
        at = names.index("SetFluidExtForce")
        assert step[at] == f"SetFluidExtForce 1 {cfg.n}"   # DriveOn from DrivePar (StepEquil 0)
        assert names[at + 1:] == AFTER_EXT_FORCE
        assert step[names.index("CalGeoPara")].split()[1] == str(k)   # StepCount of the step


@pytest.mark.parametrize("case", ("channel", "suspension", "no_cells"))
def test_host_mirror_makes_the_reference_calls(built_library, tmp_path, monkeypatch, case):
    cfg = _config(case)
    ref = _reference_trace(cfg, tmp_path)
    mirror = _mirror_trace(cfg, monkeypatch)
    if cfg.ncell:
        # the set-up calls SetPar makes itself come last in the mirror's set-up
        assert [ln.split()[0] for ln in mirror["setup"][-2:]] == ["CalGeoPara", "SetMechPara"]
        assert mirror["setup"][-2] == f"CalGeoPara -1 {cfg.ntri} {cfg.ncell}"
        assert mirror["setup"][:-2] == ref["setup"]
        assert mirror["steps"] == ref["steps"]
    else:
        assert mirror["setup"] == ref["setup"]
        for got, want in zip(mirror["steps"], ref["steps"]):
            assert got == [ln for ln in want if ln.split()[0] not in MEMBRANE]
        assert len(mirror["steps"]) == len(ref["steps"])
