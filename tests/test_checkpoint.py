"""PD's MIME snapshot format (REMD checkpoints) against PD's own writer/reader.

The golden file tests/golden/peptide30_remd.mime was written by PD's
SnapShot::writeMIME (tests/golden/make_mime_golden.py); when the reference
build is present (oracle/_ref/mime_driver) PD's reader also reads ours back."""
import io
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

MIME = os.path.join(GOLDEN, "peptide30_remd.mime")
DRIVER = os.path.join(ROOT, "oracle", "_ref", "mime_driver")


def _inputs():
    from tests.golden.make_mime_golden import golden_inputs
    return golden_inputs()


def test_reads_pd_written_snapshot():
    from pd_gb300 import checkpoint as C
    pos, vel, force, epot, status = _inputs()
    s = C.read_snapshot(MIME, "remd3")
    assert np.array_equal(s["pos"], pos) and np.array_equal(s["vel"], vel) and np.array_equal(s["force"], force)
    assert s["epot"] == epot and s["status"] == status


def test_writes_pd_bytes():
    """Our writer reproduces PD's file character for character (PD leaves header
    bytes 28-127 unset; in the golden they are zero, as we write them)."""
    from pd_gb300 import checkpoint as C
    pos, vel, force, epot, status = _inputs()
    b = io.StringIO()
    C.write_snapshot(b, "remd3", pos, vel, force, epot, status)
    assert b.getvalue() == open(MIME).read()


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 64, 65])
def test_6bit_round_trip_and_line_breaks(n):
    from pd_gb300 import checkpoint as C
    data = bytes(np.random.default_rng(n).integers(0, 256, 3 * n + n % 3, dtype=np.uint8))
    text = C.encode6bit(data)
    groups = (len(data) + 2) // 3
    lines = text.split("\n")
    assert all(len(l) == 64 for l in lines[:groups // 16])
    assert text.endswith("\n") and text.replace("\n", "").__len__() == 4 * groups
    assert C.decode6bit(text)[:len(data)] == data


def test_named_sections_and_missing_name(tmp_path):
    from pd_gb300 import checkpoint as C
    p = tmp_path / "two.mime"
    with open(p, "w") as f:
        C.write_snapshot(f, "remd0", np.ones((3, 3)), epot=1.0)
        C.write_snapshot(f, "remd1", 2 * np.ones((5, 3)), epot=2.0)
    assert C.read_snapshot(str(p), "remd1")["pos"].shape == (5, 3)
    assert C.read_snapshot(str(p))["epot"] == 1.0       # empty name: the first section
    with pytest.raises(KeyError):
        C.read_snapshot(str(p), "remd7")


@pytest.mark.skipif(not os.path.exists(DRIVER), reason="reference build (make -C oracle ref) not present")
def test_pd_reads_our_snapshot(tmp_path):
    from pd_gb300 import checkpoint as C
    pos, vel, force, epot, status = _inputs()
    p = tmp_path / "ours.mime"
    with open(p, "w") as f:
        C.write_snapshot(f, "other", pos[:3], epot=0.5)
        C.write_snapshot(f, "remd2", pos, vel, force, epot, status)
    out = tmp_path / "back.bin"
    subprocess.run([DRIVER, "read", str(p), "remd2", str(out)], check=True, capture_output=True)
    raw = out.read_bytes()
    n, e, *st = struct.unpack_from("<id4i", raw, 0)
    a = np.frombuffer(raw, "<f8", offset=28).reshape(n, 9)
    assert n == len(pos) and e == epot and tuple(st) == status
    assert np.array_equal(a[:, :3], pos) and np.array_equal(a[:, 3:6], vel) and np.array_equal(a[:, 6:], force)
