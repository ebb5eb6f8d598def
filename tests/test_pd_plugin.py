"""PD's side of the boundary: the C++ components of pd_gb300/pd_plugin/ff_gpu.h
(FF_NonBonded_GPU, FF_GeneralizedBorn_Still_GPU) compile against PD's own
headers and link with PD's libmmlib (the oracle's out-of-tree build of the PD
sources) and libpdgpu.  No GPU: the program only reports that it linked."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_pd_components_build_against_pd():
    mmlib = os.path.join(ROOT, "oracle", "_ref", "libmmlib.a")
    lib = os.path.join(ROOT, "pd_gb300", "_build", "libpdgpu.so")
    if not (os.path.exists(mmlib) and os.path.exists(lib)):
        pytest.skip("needs the PD reference build (oracle/_ref) and libpdgpu")
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "plugin-check"], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "plugin_check")], capture_output=True, text=True,
                         timeout=60)
    assert out.returncode == 0 and "linked" in out.stdout, out.stderr
