"""Record what PD's side of the boundary passes through the C ABI.

Runs oracle/_ref/plugin_check (pd_gb300/pd_plugin/plugin_check.cpp linked
against PD and against the oracle-backed test double of the C ABI,
oracle/pdgpu_abi_double.c) with PDGPU_DOUBLE_RECORD set: the double writes
every context the PD components create — the system description they
gathered from PD's WorkSpace, the parameters they set, the positions — and the
result of every compute call.  plugin_check itself checks that those
components reproduce PD's own components (FF_GeneralizedBorn_Still,
FF_SASA_LCPO, FF_NonBonded) on the same WorkSpace.  The recording becomes
tests/golden/plugin_peptide.npz, which tests/test_gpu_plugin_replay.py feeds to
the real library on the GPU.

    make -C oracle plugin-check REF=<PD checkout>
    PD_SOURCES=<PD checkout> python tests/golden/make_plugin_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PROGRAM = os.path.join(ROOT, "oracle", "_ref", "plugin_check")
sys.path.insert(0, HERE)
from make_golden import param_path  # noqa: E402
from refbin import read_container  # noqa: E402


def record():
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "abi.bin")
        env = dict(os.environ, PDGPU_DOUBLE_RECORD=out, PD_PARAM_PATH=param_path())
        r = subprocess.run([PROGRAM], env=env, capture_output=True, text=True)
        if r.returncode != 0:
            sys.exit("plugin_check failed:\n" + r.stdout[-3000:])
        return read_container(out)


def main():
    if not os.path.exists(PROGRAM):
        sys.exit("build it first: make -C oracle plugin-check REF=<PD checkout>")
    d = record()
    path = os.path.join(HERE, "plugin_peptide.npz")
    np.savez_compressed(path, **d)
    nctx = len({k.split("_")[0] for k in d})
    print("%s: %d contexts, %d arrays, %.1f kB" % (path, nctx, len(d), os.path.getsize(path) / 1024))


if __name__ == "__main__":
    main()
