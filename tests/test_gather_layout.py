"""CPU checks of the FP64 gather's accumulator placement (csrc/assemble.cu, pos27).

A row of 27 slots (the 3 x 3 x 3 neighbourhood of a structured hex mesh node, slot
s = x + 3 y + 9 z in ascending column order) keeps slot s's accumulator at position pos27(s).
Any one-to-one placement gives the same sums; this one puts the 8 slots of every 2 x 2 x 2
sub-cube -- the corners of one incident element -- at distinct positions mod 8, so the 16-byte
shared-memory accesses of a row's 8 lanes use 8 different bank groups.  The test decodes the
packed constants from the kernel source and checks those properties, and that the table fits
the accumulator size the kernel allocates.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "fem_taichi_gb300", "csrc", "assemble.cu")


def _source():
    with open(SRC) as f:
        return f.read()


def _table():
    src = _source()
    body = src[src.index("int pos27(int s)"):]
    body = body[:body.index("}")]
    words = [int(w, 16) for w in re.findall(r"0x([0-9a-fA-F]+)ull", body)]
    assert len(words) == 3
    return [(words[s // 12] >> (5 * (s % 12))) & 31 for s in range(27)]


def test_pos27_is_one_to_one_and_fits_the_row():
    t = _table()
    npos = int(re.search(r"constexpr int kG64Pos = (\d+);", _source()).group(1))
    assert len(set(t)) == 27
    assert max(t) < npos


def test_pos27_separates_every_element_sub_cube():
    t = _table()
    for x0 in (0, 1):
        for y0 in (0, 1):
            for z0 in (0, 1):
                res = {t[(x0 + dx) + 3 * (y0 + dy) + 9 * (z0 + dz)] % 8
                       for dx in (0, 1) for dy in (0, 1) for dz in (0, 1)}
                assert len(res) == 8, (x0, y0, z0)


def test_no_27_position_placement_exists():
    """The reason the row holds 29 positions: the centre slot lies in all 8 sub-cubes, so no
    other slot may share its residue mod 8, while 27 positions give every residue at least 3."""
    subcubes_of_centre = sum(1 for x0 in (0, 1) for y0 in (0, 1) for z0 in (0, 1)
                             if x0 <= 1 <= x0 + 1 and y0 <= 1 <= y0 + 1 and z0 <= 1 <= z0 + 1)
    assert subcubes_of_centre == 8
    assert min(sum(1 for p in range(27) if p % 8 == r) for r in range(8)) == 3
