"""Diagonal numbering of transformed device arrays, on the CPU.

The numbering is a format shared by the runtime and the generated kernels:
golden tables from the reference runtime (tests/golden/diag_layout.json, made by
tests/golden/make_diag_golden.py from libdvmh::dvmhXYToDiagonal) pin both the
public header's closed form (include/dvmh_gb_layout.h, compiled here with gcc
and g++) and the oracle's independent counting restatement."""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = json.load(open(os.path.join(ROOT, "tests", "golden", "diag_layout.json")))

DRIVER = r"""
#include <stdio.h>
#include <stdlib.h>
#include "dvmh_gb_layout.h"
int main(int argc, char **argv) {
    long Rx = atol(argv[1]), Ry = atol(argv[2]);
    int slash = atoi(argv[3]);
    for (long y = 0; y < Ry; y++)
        for (long x = 0; x < Rx; x++) printf("%ld\n", dvmhgb_diag_index(x, y, Rx, Ry, slash));
    return 0;
}
"""


@pytest.fixture(scope="module", params=["gcc", "g++"])
def header_exe(request, tmp_path_factory):
    d = tmp_path_factory.mktemp("layout")
    src = d / ("drv.c" if request.param == "gcc" else "drv.cpp")
    src.write_text(DRIVER)
    exe = d / "drv"
    subprocess.run([request.param, "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    return str(exe)


def test_golden_cover_shapes():
    shapes = {(c["Rx"], c["Ry"], c["slash"]) for c in GOLDEN["cases"]}
    # square, wide, tall, single row / column, both orientations
    for need in [(4, 4, 0), (4, 4, 1), (7, 3, 0), (3, 7, 1), (1, 4, 0), (4, 1, 1)]:
        assert need in shapes
    for c in GOLDEN["cases"]:  # each table is a permutation of 0 .. Rx*Ry-1
        t = np.array(c["table"]).ravel()
        assert sorted(t.tolist()) == list(range(c["Rx"] * c["Ry"]))


def test_header_matches_reference(header_exe):
    for c in GOLDEN["cases"]:
        out = subprocess.run([header_exe, str(c["Rx"]), str(c["Ry"]), str(c["slash"])], check=True,
                             capture_output=True, text=True).stdout.split()
        assert [int(v) for v in out] == np.array(c["table"]).ravel().tolist(), c


def test_oracle_matches_reference():
    L = orc.lib()
    for c in GOLDEN["cases"]:
        for y, row in enumerate(c["table"]):
            for x, v in enumerate(row):
                assert L.orc_diag_index(x, y, c["Rx"], c["Ry"], c["slash"]) == v, (c["Rx"], c["Ry"], x, y)


def test_header_matches_oracle_on_larger_planes(header_exe):
    # beyond the golden shapes: the closed form against the counting restatement
    L = orc.lib()
    for rx, ry in [(31, 17), (17, 31), (24, 24), (64, 5)]:
        for slash in (0, 1):
            out = subprocess.run([header_exe, str(rx), str(ry), str(slash)], check=True, capture_output=True,
                                 text=True).stdout.split()
            want = [L.orc_diag_index(x, y, rx, ry, slash) for y in range(ry) for x in range(rx)]
            assert [int(v) for v in out] == want, (rx, ry, slash)
