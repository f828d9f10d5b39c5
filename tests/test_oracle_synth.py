"""The oracle's molecule generator (oracle/oracle_synth.cpp) against the library's
(qses_synth_ball / qses_synth_shell): the benchmark's CPU legs build their inputs with the
oracle's, so both must give the same atoms, bit for bit, for the same seed."""
import numpy as np
import pytest

import quickses_gb300 as q
from oracle import oracle as O


@pytest.mark.parametrize("n,seed", [(2, 1), (150, 3), (1000, 1), (20000, 1)])
def test_ball_same_atoms(n, seed):
    a_xyz, a_rad = O.synth_ball(n, seed)
    b_xyz, b_rad, _ = q.molecules.ball(n, seed)
    assert np.array_equal(a_xyz, b_xyz) and np.array_equal(a_rad, b_rad)


def test_sparse_ball_and_no_spacing_same_atoms():
    for kw in ({"density": 0.0045}, {"min_dist": 0.0}):
        a_xyz, a_rad = O.synth_ball(800, 5, **kw)
        b_xyz, b_rad, _ = q.molecules.ball(800, 5, **kw)
        assert np.array_equal(a_xyz, b_xyz) and np.array_equal(a_rad, b_rad)


@pytest.mark.parametrize("n,seed", [(3000, 4), (1000, 1)])
def test_shell_same_atoms(n, seed):
    a_xyz, a_rad = O.synth_shell(n, seed)
    b_xyz, b_rad, _ = q.molecules.shell(n, seed)
    assert np.array_equal(a_xyz, b_xyz) and np.array_equal(a_rad, b_rad)
