"""Trajectory output for device dynamics.

PD appends a frame every UpdateTra steps (md.cpp:277) through its OutTra
writers (fileio/tra.h:78-87), one of which writes PDB models (fileio/pdb.h,
MODEL/ENDMDL).  Here the frames come from the device without stalling the
step stream (pdgpu_md_set_trajectory copies them asynchronously into a
page-locked ring) and are written as a multi-model PDB file."""
import numpy as np

ELEMENT = {1: "H", 6: "C", 7: "N", 8: "O", 15: "P", 16: "S"}


class PDBTrajectory:
    """Appends frames of a batch as PDB models (one model per frame; systems of a
    batch are chains A, B, ... when there are at most 26 of them)."""

    def __init__(self, path, image, Z=None, residue=None, append=False):
        self.path = path
        self.image = image
        n = image.natom
        self.names = [ELEMENT.get(int(z), "X") for z in Z] if Z is not None else ["X"] * n
        self.residue = np.asarray(residue, np.int64) if residue is not None else np.zeros(n, np.int64)
        sys_of = np.repeat(np.arange(image.nsystems), image.natoms)
        self.chain = [chr(65 + s) if image.nsystems <= 26 else "A" for s in sys_of]
        self.model = 0
        if not append:
            open(path, "w").close()

    def append(self, frames):
        frames = np.asarray(frames, np.float64).reshape(-1, self.image.natom, 3)
        with open(self.path, "a") as f:
            for fr in frames:
                self.model += 1
                f.write("MODEL     %4d\n" % self.model)
                for i, (x, y, z) in enumerate(fr):
                    f.write("ATOM  %5d %-4s UNK %1s%4d    %8.3f%8.3f%8.3f  1.00  0.00          %2s\n" % (
                        (i + 1) % 100000, self.names[i], self.chain[i], (self.residue[i] + 1) % 10000, x, y, z,
                        self.names[i]))
                f.write("ENDMDL\n")


def read_pdb_models(path):
    """Coordinates of every MODEL of a PDB file, shape (models, atoms, 3)."""
    models, cur = [], None
    for line in open(path):
        if line.startswith("MODEL"):
            cur = []
        elif line.startswith("ATOM") or line.startswith("HETATM"):
            cur.append((float(line[30:38]), float(line[38:46]), float(line[46:54])))
        elif line.startswith("ENDMDL"):
            models.append(cur)
    return np.asarray(models)
