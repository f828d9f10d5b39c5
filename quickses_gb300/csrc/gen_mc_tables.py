"""Generate the marching-cubes triangle tables used by the CUDA kernels and the oracle.

The triangle table must be identical to QuickSES's (MarchingCubes.cu:64-343, the classic
Lorensen-Cline / Bourke 256-case table) because triangle topology and emission order are
part of the parity contract.  This script parses that table from the reference source and
writes two representations:

* ``quickses_gb300/csrc/mc_tables.h`` - one ``uint64_t`` per case: nibble ``v`` (v < 15)
  holds the edge index of triangle vertex ``v``; the top nibble holds the triangle count.
  One 8-byte constant load per cell replaces the reference's 16 ``int`` loads.
* ``oracle/mc_table.h`` - the plain ``int[256][16]`` layout (``-1`` terminated) for the
  CPU oracle, so the oracle does not share the packed decoding with the kernels.

Usage: ``python quickses_gb300/csrc/gen_mc_tables.py path/to/MarchingCubes.cu`` (the file
from a reference checkout).  Both outputs are committed.
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def parse_int_table(src: str, marker: str):
    i = src.index(marker)
    j = src.index("{", i)
    depth = 0
    for k in range(j, len(src)):
        if src[k] == "{":
            depth += 1
        elif src[k] == "}":
            depth -= 1
            if depth == 0:
                break
    body = src[j:k + 1]
    return [int(x, 0) for x in re.findall(r"-?0x[0-9a-fA-F]+|-?\d+", body)]


def load_reference(path: str):
    src = open(path).read()
    flat = parse_int_table(src, "triTable[256][16]")
    nb = parse_int_table(src, "nbTriTable[256]")
    assert len(flat) == 4096 and len(nb) == 256
    tri = [flat[c * 16:(c + 1) * 16] for c in range(256)]
    return tri, nb


def pack(tri):
    packed = []
    for row in tri:
        n = 0
        while n < 16 and row[n] != -1:
            n += 1
        assert n % 3 == 0 and n <= 15
        word = 0
        for v in range(n):
            assert 0 <= row[v] < 12
            word |= row[v] << (4 * v)
        word |= (n // 3) << 60
        packed.append(word)
    return packed


def main():
    if len(sys.argv) < 2:
        raise SystemExit("usage: gen_mc_tables.py path/to/MarchingCubes.cu")
    ref = sys.argv[1]
    tri, nb = load_reference(ref)
    packed = pack(tri)
    for c in range(256):
        assert (packed[c] >> 60) * 3 == nb[c]

    lines = [
        "// Generated by gen_mc_tables.py - do not edit.",
        "// Marching-cubes triangle table, identical in content to QuickSES",
        "// MarchingCubes.cu:64-343 (classic 256-case table).  Packed: nibble v (v < 15) is",
        "// the edge of triangle vertex v, the top nibble is the triangle count.",
        "#pragma once",
        "#include <stdint.h>",
        "#define QSES_MC_TABLE_INIT { \\",
    ]
    for c in range(0, 256, 4):
        lines.append("    " + ", ".join("0x%016xULL" % packed[c + d] for d in range(4)) + ", \\")
    lines.append("}")
    with open(os.path.join(HERE, "mc_tables.h"), "w") as f:
        f.write("\n".join(lines) + "\n")

    olines = [
        "// Generated by quickses_gb300/csrc/gen_mc_tables.py - do not edit.",
        "// Marching-cubes triangle table as laid out in QuickSES MarchingCubes.cu:64-343",
        "// (-1 terminated rows).  TEST INFRASTRUCTURE: used only by the CPU oracle.",
        "#pragma once",
        "static const int ORACLE_TRI_TABLE[256][16] = {",
    ]
    for row in tri:
        olines.append("    {" + ", ".join("%d" % v for v in row) + "},")
    olines.append("};")
    with open(os.path.join(ROOT, "oracle", "mc_table.h"), "w") as f:
        f.write("\n".join(olines) + "\n")
    print("wrote mc_tables.h and oracle/mc_table.h")


if __name__ == "__main__":
    main()
