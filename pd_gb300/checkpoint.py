"""PD's MIME snapshot format: REMD checkpoints that PD itself can read back.

``REX_Local::printCheckPointMIME`` writes every replica's SnapShot as a section
``!PSP remd<r>`` ... ``!ENDPSP`` and ``readCheckPointMIME`` reads them back
(src/mmlib/protocols/remd.cpp:319-331).  A section holds a binary record in
PD's 6-bit text coding (src/mmlib/workspace/snapshot.cpp:322-379,
src/mmlib/tools/io.cpp:95-201):

* record: 128-byte header (int32 natoms at 0, float64 epot at 4, int32
  status1..4 at 12..27; PD leaves the other header bytes unset, written as
  zeros here), then per atom 9 float64: position (A), velocity, force;
* coding: every 3 bytes b0 b1 b2 become 4 characters of the alphabet
  ``A-Z a-z 0-9 + /`` carrying, in order, the low 6 bits of b0; the top 2 bits
  of b0 with the low 4 of b1; the top 4 bits of b1 with the low 2 of b2; the
  top 6 bits of b2 (a little-endian bit order, not RFC 4648's); a short last
  group is zero-padded; a newline follows every 16 groups and the end.

All values are little-endian, as PD writes them on the machines it runs on.
"""
import io
import struct

import numpy as np

ALPHABET = b"ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/"
_DECODE = np.full(256, 63, np.uint8)
for _i, _c in enumerate(ALPHABET):
    _DECODE[_c] = _i
HEADER_BYTES = 128
GROUPS_PER_LINE = 16


def encode6bit(data):
    """PD's IO::encode6bit: bytes -> text (with its line breaks and final newline)."""
    b = np.frombuffer(bytes(data), np.uint8)
    pad = (-len(b)) % 3
    if pad:
        b = np.concatenate([b, np.zeros(pad, np.uint8)])
    g = b.reshape(-1, 3).astype(np.uint16)
    i0, i1, i2 = g[:, 0], g[:, 1], g[:, 2]
    q = np.stack([i0 & 63, ((i1 << 2) | (i0 >> 6)) & 63, ((i1 >> 4) | ((i2 << 4) & 63)) & 63, i2 >> 2], axis=1)
    chars = np.frombuffer(ALPHABET, np.uint8)[q.astype(np.uint8)]
    out = io.BytesIO()
    n = len(chars)
    for start in range(0, n, GROUPS_PER_LINE):
        out.write(chars[start:start + GROUPS_PER_LINE].tobytes())
        if start + GROUPS_PER_LINE <= n:
            out.write(b"\n")
    out.write(b"\n")
    return out.getvalue().decode("ascii")


def decode6bit(text):
    """PD's IO::decode6bit: characters below 32 are skipped; a short last group
    reads as if filled with code 63 (PD's behaviour; its own writer never makes one)."""
    raw = np.frombuffer(text.encode("ascii") if isinstance(text, str) else bytes(text), np.uint8)
    raw = raw[raw >= 32]
    pad = (-len(raw)) % 4
    codes = _DECODE[raw]
    if pad:
        codes = np.concatenate([codes, np.full(pad, 63, np.uint8)])
    c = codes.reshape(-1, 4).astype(np.uint16)
    o0 = (c[:, 0] | (c[:, 1] << 6)) & 255
    o1 = ((c[:, 1] >> 2) | (c[:, 2] << 4)) & 255
    o2 = ((c[:, 3] << 2) | (c[:, 2] >> 4)) & 255
    return np.stack([o0, o1, o2], axis=1).astype(np.uint8).tobytes()


def snapshot_record(pos, vel=None, force=None, epot=0.0, status=(0, 0, 0, 0)):
    pos = np.asarray(pos, np.float64).reshape(-1, 3)
    n = len(pos)
    z = np.zeros((n, 3))
    vel = z if vel is None else np.asarray(vel, np.float64).reshape(n, 3)
    force = z if force is None else np.asarray(force, np.float64).reshape(n, 3)
    head = bytearray(HEADER_BYTES)
    struct.pack_into("<id4i", head, 0, n, float(epot), *[int(s) for s in status])
    body = np.concatenate([pos, vel, force], axis=1).astype("<f8").tobytes()
    return bytes(head) + body


def write_snapshot(f, name, pos, vel=None, force=None, epot=0.0, status=(0, 0, 0, 0)):
    """SnapShot::writeMIME into an open text file."""
    f.write("!PSP %s\n" % name)
    f.write(encode6bit(snapshot_record(pos, vel, force, epot, status)))
    f.write("\n!ENDPSP\n")


def read_snapshots(f):
    """Every section of an open text file: {name: dict(pos, vel, force, epot, status)}."""
    out = {}
    name, chunks = None, None
    for line in f:
        if name is None:
            if line.startswith("!PSP"):
                tok = line.split()
                name = tok[1] if len(tok) > 1 else ""
                chunks = []
            continue
        if line.startswith("!ENDPSP"):
            out[name] = _parse(decode6bit("".join(chunks)))
            name = None
            continue
        chunks.append(line)
    return out


def read_snapshot(path, name=""):
    """SnapShot::readMIME: the section called ``name`` (the first one if empty)."""
    with open(path) as f:
        secs = read_snapshots(f)
    if not secs:
        raise ValueError("no MIME snapshot in %s" % path)
    if name == "":
        return next(iter(secs.values()))
    if name not in secs:
        raise KeyError("MIME snapshot '%s' not found in %s" % (name, path))
    return secs[name]


def _parse(rec):
    n, epot, s1, s2, s3, s4 = struct.unpack_from("<id4i", rec, 0)
    if n <= 0:
        raise ValueError("corrupt MIME snapshot: natoms <= 0")
    a = np.frombuffer(rec, "<f8", count=9 * n, offset=HEADER_BYTES).reshape(n, 9).astype(np.float64)
    return {"pos": a[:, 0:3].copy(), "vel": a[:, 3:6].copy(), "force": a[:, 6:9].copy(), "epot": epot,
            "status": (s1, s2, s3, s4)}
