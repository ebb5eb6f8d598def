"""Writes tests/golden/peptide30_remd.mime with PD's own SnapShot::writeMIME
(oracle/_ref/mime_driver, built by `make -C oracle ref`) for the peptide30
fixture: positions from the fixture, seeded velocities and forces, epot and
status words, so the checkpoint reader/writer in pd_gb300/checkpoint.py can be
checked against PD's bytes.  Run from the repository root."""
import os
import struct
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "mime_driver")
OUT = os.path.join(ROOT, "tests", "golden", "peptide30_remd.mime")
NAME = "remd3"


def golden_inputs():
    d = np.load(os.path.join(ROOT, "tests", "golden", "peptide30.npz"))
    rng = np.random.default_rng(30)
    pos = d["pos"]
    vel = rng.normal(0.0, 400.0, pos.shape)        # m/s, thermal scale
    force = rng.normal(0.0, 1e-10, pos.shape)      # N
    return pos, vel, force, -5.59e-18, (7, -1, 0, 123456)


def main():
    pos, vel, force, epot, status = golden_inputs()
    n = len(pos)
    tmp = OUT + ".bin"
    with open(tmp, "wb") as f:
        f.write(struct.pack("<id4i", n, epot, *status))
        f.write(np.concatenate([pos, vel, force], axis=1).astype("<f8").tobytes())
    subprocess.run([DRIVER, "write", tmp, OUT, NAME], check=True)
    os.remove(tmp)
    print("wrote", OUT)


if __name__ == "__main__":
    sys.exit(main())
