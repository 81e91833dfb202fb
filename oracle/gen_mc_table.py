"""Generate lvr2_gb300/csrc/mc_table.inc from the reference's marching-cubes table.

The triangulation table has to be value-identical to the reference's
(include/lvr2/reconstruction/MCTable.hpp:41, the lvr2 variant of Paul
Bourke's table) for the mesh topology to match.  This script parses that
header once and writes the table in this project's own packed encoding:
one uint64 per cube index, bits [4*j, 4*j+4) = j-th edge index of the
triangle list (up to 12 edges), bits [60, 64) = number of triangles.

Usage: python oracle/gen_mc_table.py <lvr2 source tree>
The generated file is committed; tests/test_tables.py re-checks it against
the reference header (compiled by oracle/Makefile into oracle/_ref/).
"""
import re
import sys
from pathlib import Path


def parse_mc_table(text):
    body = text[text.index("MCTable[256][13]"):]
    body = body[body.index("{") + 1:]
    rows = re.findall(r"\{([^{}]*)\}", body)[:256]
    table = [[int(v) for v in r.split(",")] for r in rows]
    assert len(table) == 256 and all(len(r) == 13 for r in table)
    return table


def pack(row):
    edges = []
    for v in row:
        if v == -1:
            break
        edges.append(v)
    assert len(edges) % 3 == 0 and len(edges) <= 12
    word = 0
    for j, e in enumerate(edges):
        assert 0 <= e < 12
        word |= e << (4 * j)
    word |= (len(edges) // 3) << 60
    return word


def main(ref_root):
    hdr = Path(ref_root) / "include/lvr2/reconstruction/MCTable.hpp"
    table = parse_mc_table(hdr.read_text())
    words = [pack(r) for r in table]
    out = Path(__file__).resolve().parent.parent / "lvr2_gb300/csrc/mc_table.inc"
    lines = ["/* Marching-cubes triangle table, packed: bits [4j,4j+4) = j-th edge of the",
             " * triangle list, bits [60,64) = triangle count.  Generated by",
             " * oracle/gen_mc_table.py; value-identical to the lvr2 table",
             " * (include/lvr2/reconstruction/MCTable.hpp:41). */"]
    for i in range(0, 256, 4):
        lines.append("    " + ", ".join("0x%016xULL" % w for w in words[i:i + 4]) + ",")
    out.write_text("\n".join(lines) + "\n")
    print("wrote", out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python oracle/gen_mc_table.py <lvr2 source tree>")
    main(sys.argv[1])
