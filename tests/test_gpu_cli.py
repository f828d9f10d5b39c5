"""The QuickSES-compatible executable end to end on the GPU: PDB in, OBJ out, compared byte
for byte with the oracle's mesh written in the reference's OBJ format."""
import os
import subprocess

import numpy as np
import pytest

import quickses_gb300 as q
from oracle import oracle as O
from tests.golden.gen_pdb_golden import atom_line
from tests.test_io import _expected_obj

pytestmark = pytest.mark.gpu

CLI = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "quickses_gb300", "bin", "QuickSES")


def _write_pdb(path, xyz, elem):
    with open(path, "w") as f:
        for k, (p, e) in enumerate(zip(xyz, elem)):
            f.write(atom_line("ATOM", k + 1, "X", " ", "UNK", "A", k // 10 + 1, *p, e.rjust(2)))
        f.write("END\n")


@pytest.mark.parametrize("voxel,passes", [(0.5, 1), (0.4, 0), (0.3, 2)])
def test_cli_obj_matches_oracle(tmp_path, voxel, passes):
    xyz, _, el = q.molecules.ball(300, seed=17)
    names = [chr(int(c)) for c in el]  # element letters as ASCII codes
    pdb, obj = tmp_path / "m.pdb", tmp_path / "m.obj"
    _write_pdb(pdb, xyz, names)
    r = subprocess.run([CLI, "-i", str(pdb), "-o", str(obj), "-l", str(passes), "-v", str(voxel)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    pxyz, prad = q.read_pdb(pdb)
    ref = O.compute_ses(pxyz, prad, voxel, smooth=passes, fp64=False)
    # the OBJ path keeps degenerate triangles (CudaSurf.cu:363-368 writes every triangle)
    assert obj.read_text() == _expected_obj(ref.vertices.astype(np.float32), ref.triangles)


def test_cli_reference_slices_obj_matches_oracle(tmp_path):
    """-r -s 20: the reference's sliced output (one mesh per slice, concatenated), written
    byte for byte as the oracle's restatement of that slicing gives it."""
    xyz, _, el = q.molecules.ball(300, seed=18)
    names = [chr(int(c)) for c in el]
    pdb, obj = tmp_path / "m.pdb", tmp_path / "m.obj"
    _write_pdb(pdb, xyz, names)
    r = subprocess.run([CLI, "-i", str(pdb), "-o", str(obj), "-l", "1", "-v", "0.5", "-s", "20", "-r"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    pxyz, prad = q.read_pdb(pdb)
    ref = O.compute_ses_slices(pxyz, prad, 0.5, 20, smooth=1)
    assert len(ref.slice_v) > 2
    assert obj.read_text() == _expected_obj(ref.vertices.astype(np.float32), ref.triangles)
    bad = subprocess.run([CLI, "-i", str(pdb), "-o", str(obj), "-s", "0", "-r"], capture_output=True, text=True,
                         timeout=60)
    assert bad.returncode != 0
