"""PD's side of the boundary: the C++ components of pd_gb300/pd_plugin/ff_gpu.h
(FF_NonBonded_GPU, FF_GeneralizedBorn_Still_GPU, FF_SASA_LCPO_GPU) inside PD.

plugin_check builds a peptide with PD, evaluates it with PD's own components
and with these ones on the same WorkSpace (Forcefield::calcForces and
calcEnergies, forcefield.cpp:229-264) and requires every Hamiltonian field and
force to agree.  Here it is linked against PD's libmmlib (the oracle's
out-of-tree build of the PD sources) and the FP64 test double of the C ABI
(oracle/pdgpu_abi_double.c), so the components' own code — what they gather
from the WorkSpace, the parameters they set, how they add energies and forces
back — is checked to 1e-9 without a GPU.  The same program also links against
the real libpdgpu (the GPU leg is tests/test_gpu_plugin_replay.py, which
replays the calls recorded here on the GPU).  Skipped without the PD build."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref")


def _pd_build():
    if not (os.path.exists(os.path.join(REF, "libmmlib.a")) and os.path.exists(os.path.join(REF, "REF"))):
        pytest.skip("needs the PD reference build (make -C oracle ref REF=<PD checkout>)")
    src = open(os.path.join(REF, "REF")).read().strip()
    if not os.path.isdir(os.path.join(src, "param")):
        pytest.skip("the PD checkout recorded in oracle/_ref/REF is not present")
    return src


def test_pd_components_match_pd_components():
    src = _pd_build()
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "plugin-check"], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    env = dict(os.environ, PD_PARAM_PATH=os.path.join(src, "param"))
    out = subprocess.run([os.path.join(REF, "plugin_check")], capture_output=True, text=True, timeout=600, env=env)
    lines = [ln for ln in out.stdout.splitlines() if "agree" in ln or "MISMATCH" in ln or "match" in ln]
    assert out.returncode == 0, "\n".join(lines)
    assert "pdgpu PD components match PD" in out.stdout
    assert sum("agree" in ln for ln in lines) == 3


def test_pd_components_link_against_the_library():
    _pd_build()
    from pd_gb300 import build
    build.build()
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "plugin-gpu"], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    assert os.path.exists(os.path.join(REF, "plugin_gpu"))
