"""Generate the PDB-reading golden case from QuickSES's own parser.

Writes tests/golden/sample.pdb (synthetic, seeded; exercises the record rules the QuickSES
executable depends on) and tests/golden/ref_pdb.npz with what the reference's parsePDB
(cpdb/cpdb.cpp:35-158), walked as CudaSurf.cu:942-968 walks it, returns for that file:
coordinates and the first byte of each atom's element field.

Usage: python tests/golden/gen_pdb_golden.py   (needs the reference checkout; run in the
build container).
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as ob  # noqa: E402

PDB = os.path.join(HERE, "sample.pdb")
OUT = os.path.join(HERE, "ref_pdb.npz")


def atom_line(rec, serial, name, alt, res, chain, resi, x, y, z, elem, charge="  "):
    # PDB fixed columns: coordinates at 31-54, element at 77-78, charge at 79-80 (1-based)
    return "%-6s%5d %-4s%c%3s %c%4d    %8.3f%8.3f%8.3f%6.2f%6.2f          %2s%2s\n" % (
        rec, serial, name, alt, res, chain, resi, x, y, z, 1.0, 20.0, elem, charge)


def make_pdb(seed=5):
    rng = np.random.default_rng(seed)
    lines = ["REMARK   1 " + "synthetic structure for parser parity ".ljust(100, "-") + "\n"]
    elems = ["C", "N", "O", "S", "H", "P", "FE", "CL", "SE", "ZN", "X", "MG"]
    serial = 1
    for chain, nres in (("A", 6), ("B", 3), ("A", 2)):  # chain A appears twice
        for r in range(nres):
            for k in range(5):
                x, y, z = rng.uniform(-120, 120, 3)
                alt = " " if k != 3 else "AB"[r % 2]   # altLoc B records are skipped
                rec = "ATOM" if (serial % 11) else "HETATM"  # HETATM is not an atom here
                e = elems[int(rng.integers(len(elems)))]
                lines.append(atom_line(rec, serial, "CA", alt, "ALA", chain, r + 1, x, y, z, e.rjust(2)))
                serial += 1
        lines.append("TER\n")  # TER does not stop reading
    # adjacent negative fields with no separating blank
    lines.append(atom_line("ATOM", serial, "N", " ", "GLY", "C", 1, -100.125, -200.5, -9.0625, " N"))
    serial += 1
    # a short record: bytes 77-79 still hold the previous (longer) line's element
    lines.append(atom_line("ATOM", serial, "O", " ", "GLY", "C", 1, 1.5, 2.5, 3.5, " O")[:66] + "\n")
    serial += 1
    # a record longer than 127 bytes: its tail is read as a separate line, here another ATOM
    tail = atom_line("ATOM", serial, "S", " ", "CYS", "C", 2, 7.0, 8.0, 9.0, " S")
    lines.append("REMARK 999 " + "x" * 116 + tail)
    serial += 1
    lines.append(atom_line("ATOM", serial, "C", " ", "CYS", "C", 2, 4.0, 5.0, 6.0, " C"))
    serial += 1
    lines.append("ENDMDL\n")  # reading stops here
    lines.append(atom_line("ATOM", serial, "C", " ", "CYS", "C", 3, 0.0, 0.0, 0.0, " C"))
    lines.append("END\n")
    return "".join(lines)


def main():
    with open(PDB, "w") as f:
        f.write(make_pdb())
    path = ob.build_ref_pdb()
    if path is None:
        raise SystemExit("reference checkout not found")
    L = ctypes.CDLL(path)
    L.ref_read_pdb.restype = ctypes.c_int
    L.ref_read_pdb.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    cap = 1000
    xyz = np.zeros((cap, 3), np.float32)
    el = np.zeros(cap, np.uint8)
    n = L.ref_read_pdb(PDB.encode(), xyz.ctypes.data, el.ctypes.data, cap)
    assert 0 < n <= cap
    np.savez_compressed(OUT, xyz=xyz[:n], element0=el[:n])
    print("%d atoms -> %s" % (n, OUT))


if __name__ == "__main__":
    main()
