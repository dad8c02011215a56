"""Generate tests/golden/diag_layout.json from the REFERENCE runtime.

The diagonal layout of a transformed device array (two axes renumbered along
anti-diagonals, the order in which an ACROSS loop with two dependences sweeps
them) is a format the runtime and the generated kernels must agree on.  This
script links a small driver against the reference runtime built from its
sources (oracle/_ref/libdvmh.a, see oracle/ref.mk) and records, for a set of
plane shapes Rx x Ry and both orientations, the position the reference gives
every (x, y): libdvmh::dvmhXYToDiagonal (rts/dvmh/util.cpp:1009-1055).

Run here (needs oracle/_ref built):  python tests/golden/make_diag_golden.py
"""
import json
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF = os.path.join(ROOT, "oracle", "_ref")

SHAPES = [(1, 1), (1, 4), (4, 1), (2, 2), (3, 3), (2, 5), (5, 2), (4, 4), (3, 7), (7, 3), (6, 6), (8, 13), (13, 8),
          (16, 16)]

DRIVER = r"""
#include <cstdio>
#include <cstdlib>
namespace libdvmh { long dvmhXYToDiagonal(long x, long y, long Rx, long Ry, bool slash); }
int main(int argc, char **argv) {
    long Rx = atol(argv[1]), Ry = atol(argv[2]);
    int slash = atoi(argv[3]);
    for (long y = 0; y < Ry; y++)
        for (long x = 0; x < Rx; x++) printf("%ld\n", libdvmh::dvmhXYToDiagonal(x, y, Rx, Ry, slash != 0));
    return 0;
}
"""


def main():
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "diag.cpp")
        exe = os.path.join(tmp, "diag")
        with open(src, "w") as f:
            f.write(DRIVER)
        subprocess.run(["g++", "-O1", src, os.path.join(REF, "libdvmh.a"), os.path.join(REF, "libdvm.a"),
                        os.path.join(REF, "pstub.o"), "-fopenmp", "-lpthread", "-o", exe], check=True)
        cases = []
        for rx, ry in SHAPES:
            for slash in (0, 1):
                out = subprocess.run([exe, str(rx), str(ry), str(slash)], check=True, capture_output=True,
                                     text=True).stdout.split()
                # table[y][x] = position of (x, y) in the diagonal order
                flat = [int(v) for v in out]
                cases.append({"Rx": rx, "Ry": ry, "slash": slash,
                              "table": [flat[y * rx:(y + 1) * rx] for y in range(ry)]})
    with open(os.path.join(ROOT, "tests", "golden", "diag_layout.json"), "w") as f:
        f.write('{"source": "reference runtime libdvmh::dvmhXYToDiagonal (rts/dvmh/util.cpp:1009-1055)",\n')
        f.write(' "cases": [\n')
        f.write(",\n".join("  " + json.dumps(c, separators=(",", ":")) for c in cases))
        f.write("\n]}\n")


if __name__ == "__main__":
    main()
