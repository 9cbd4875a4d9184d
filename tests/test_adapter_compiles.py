"""The C++ adapter include/adapter/SimulationEngineCUDA.h (`SimulationEngineCUDA
: SPH::SimulationEngine`) compiles against the reference's own engine headers
(SPHFluidSimulation/include/SPH/Core/SimulationEngine.h, SceneBlueprint.h,
ParticleBufferManager.h, ResourceLockGuard.h, Particles.h) and this
library's C ABI (include/sph_gb300.h).

The headers need the Blaze Engine, an un-vendored dependency of the
reference; tests/adapter_shim declares the names they use, and
oracle/ref_shim the integer and vector types.  The check is
`g++ -std=c++20 -fsyntax-only`, so nothing is linked or run.  It needs the
reference tree (SPH_REFERENCE_ROOT, default /root/reference) and is skipped
where that is absent.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE_ROOT = os.environ.get("SPH_REFERENCE_ROOT", "/root/reference")
REFERENCE_INCLUDE = os.path.join(REFERENCE_ROOT, "SPHFluidSimulation", "include")
ADAPTER = os.path.join(ROOT, "include", "adapter", "SimulationEngineCUDA.h")


def adapter_source() -> str:
    src = open(ADAPTER).read()
    assert "class SimulationEngineCUDA : public SimulationEngine" in src
    return src


def test_adapter_declares_every_engine_member():
    src = adapter_source()
    for member in ("void Clear()", "void Initialize(", "void Update(", "SystemImplementationName()",
                   "GetDynamicParticlesBufferManager()", "GetStaticParticlesBufferManager()",
                   "GetSimulationTime()"):
        assert member in src, member


@pytest.mark.skipif(not os.path.isdir(REFERENCE_INCLUDE), reason="reference tree not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not present")
def test_adapter_compiles_against_reference_headers(tmp_path):
    unit = tmp_path / "adapter.cpp"
    unit.write_text('#include "SimulationEngineCUDA.h"\n'
                    "// the class is complete and concrete: every pure virtual is overridden\n"
                    "SPH::SimulationEngine* make_engine() { return new SPH::SimulationEngineCUDA(0); }\n")
    cmd = ["g++", "-std=c++20", "-fsyntax-only", "-Wall", "-Wno-unused-variable",
           "-I", os.path.dirname(ADAPTER),
           "-I", os.path.join(ROOT, "tests", "adapter_shim"),
           "-I", os.path.join(ROOT, "oracle", "ref_shim"),
           "-I", REFERENCE_INCLUDE,
           "-I", os.path.join(ROOT, "include"),
           str(unit)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
