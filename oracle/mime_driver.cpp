// mime_driver.cpp — test infrastructure: PD's own SnapShot MIME writer and
// reader (src/mmlib/workspace/snapshot.cpp:322-466, 6-bit coding in
// src/mmlib/tools/io.cpp:95-201), run on given data so the Python restatement
// of the checkpoint format can be checked byte for byte.
//
//   mime_driver write <in.bin> <out.mime> <name>
//   mime_driver read  <in.mime> <name> <out.bin>
//
// bin layout: int32 natoms, f64 epot, int32 status[4], f64 [natoms][9] (p, v, f)
#include <cstdio>
#include <cstring>
#include <vector>

#include "workspace/snapshot.h"

static int fail(const char *msg) {
    fprintf(stderr, "mime_driver: %s\n", msg);
    return 1;
}

int main(int argc, char **argv) {
    if (argc < 5) return fail("usage: write <in.bin> <out.mime> <name> | read <in.mime> <name> <out.bin>");
    if (!strcmp(argv[1], "write")) {
        FILE *f = fopen(argv[2], "rb");
        if (!f) return fail("cannot open input");
        int n = 0;
        double epot = 0;
        int st[4];
        if (fread(&n, 4, 1, f) != 1 || fread(&epot, 8, 1, f) != 1 || fread(st, 4, 4, f) != 4 || n <= 0)
            return fail("bad header");
        std::vector<double> d((size_t)n * 9);
        if (fread(&d[0], 8, d.size(), f) != d.size()) return fail("short input");
        fclose(f);
        SnapShot s((size_t)n);
        s.epot = epot;
        s.status1 = st[0];
        s.status2 = st[1];
        s.status3 = st[2];
        s.status4 = st[3];
        for (int i = 0; i < n; i++) {
            const double *r = &d[(size_t)i * 9];
            s.atom[i].p.setTo(r[0], r[1], r[2]);
            s.atom[i].v.setTo(r[3], r[4], r[5]);
            s.atom[i].f.setTo(r[6], r[7], r[8]);
        }
        return s.writeMIME(std::string(argv[3]), std::string(argv[4]), "w") == 0 ? 0 : fail("write failed");
    }
    if (!strcmp(argv[1], "read")) {
        SnapShot s(1);
        s.readMIME(std::string(argv[2]), std::string(argv[3]));
        FILE *f = fopen(argv[4], "wb");
        if (!f) return fail("cannot open output");
        int n = (int)s.natoms;
        int st[4] = {s.status1, s.status2, s.status3, s.status4};
        fwrite(&n, 4, 1, f);
        fwrite(&s.epot, 8, 1, f);
        fwrite(st, 4, 4, f);
        for (int i = 0; i < n; i++) {
            double r[9] = {s.atom[i].p.x, s.atom[i].p.y, s.atom[i].p.z, s.atom[i].v.x, s.atom[i].v.y,
                           s.atom[i].v.z, s.atom[i].f.x, s.atom[i].f.y, s.atom[i].f.z};
            fwrite(r, 8, 9, f);
        }
        fclose(f);
        return 0;
    }
    return fail("unknown mode");
}
