"""Input formats of the optional terms (CPU): restraint files
(read_restraint.F90), the [Tweezers] tables (read_input.F90:973-1160,
init_tweezers.F90) and the restart file's force-ramp block
(write_rst.F90:98-111, read_rst.F90:339-360)."""
import struct

import numpy as np
import pytest

from sis_gb300.inputs import (PN_TO_KCAL_MOL_A, InputError, constant_force_pairs, force_ramp_pairs,
                              parse_restraints)
from sis_gb300.model import Restraint
from sis_gb300.outputs import RST_TWZ, read_rst, write_rst

RESTRAINT_FILE = """# restraints of a test hairpin
# Sigmoid  i  j  epsilon  d  s  r_cut

Sigmoid          3     40     4.0    6.0    1.5    14.0
Sigmoid-to-bead  7, 22, 2.5, 8.0, 2.0, 20.0
#Sigmoid         1      2     1.0    1.0    1.0     1.0
Sigmoid 1 9 1e0 5 0.5 9.5 trailing text is ignored
"""


def test_restraint_file():
    r = parse_restraints(RESTRAINT_FILE)
    assert r == [Restraint(3, 40, 4.0, 6.0, 1.5, 14.0), Restraint(7, 22, 2.5, 8.0, 2.0, 20.0, to_bead=True),
                 Restraint(1, 9, 1.0, 5.0, 0.5, 9.5)]


@pytest.mark.parametrize("bad", ["Harmonic 1 2 1.0 1.0 1.0 1.0\n", "Sigmoid 1 2 1.0\n", "Sigmoid 1 x 1 1 1 1\n",
                                 " Sigmoid 1 2 1 1 1 1\n"])
def test_restraint_file_errors(bad):
    with pytest.raises(InputError):
        parse_restraints(bad)


def test_constant_force_pairs_in_kcal_per_mol_per_angstrom():
    p = constant_force_pairs([[1, 5]], [[5.0, 0.0, -2.0]])
    assert p[0].i == 1 and p[0].j == 5
    assert np.allclose(p[0].force, [5.0 * PN_TO_KCAL_MOL_A, 0.0, -2.0 * PN_TO_KCAL_MOL_A], rtol=1e-15)
    # 1 pN is 0.0143933 kcal/mol/A
    assert PN_TO_KCAL_MOL_A == pytest.approx(0.0143933, rel=1e-5)
    with pytest.raises(InputError):
        constant_force_pairs([[1, 5]], [])
    with pytest.raises(InputError):
        constant_force_pairs([[0, 5]], [[1.0, 0.0, 0.0]])


def test_force_ramp_traps_start_on_the_beads_and_move_apart():
    x = np.zeros((6, 3))
    x[1] = [1.0, 2.0, 3.0]
    x[4] = [4.0, 6.0, 3.0]  # 5 A from bead 2 along (0.6, 0.8, 0)
    p = force_ramp_pairs(x, [[2, 5]], [[0.003, 0.004]], [[0.0, 1.5e-6]])[0]
    assert (p.i, p.j, p.k) == (2, 5, (0.003, 0.004))
    assert np.array_equal(p.init, [x[1], x[4]])
    assert np.allclose(p.velo[0], [0.0, 0.0, 0.0]) and np.allclose(p.velo[1], [0.9e-6, 1.2e-6, 0.0], rtol=1e-12)
    q = force_ramp_pairs(x, [[2, 5]], [[0.003, 0.004]], [[2.0, 1.0]])[0]
    assert np.allclose(q.velo[0], [-1.2, -1.6, 0.0]) and np.allclose(q.velo[1], [0.6, 0.8, 0.0])
    # on a restart the traps start where the file says
    init = np.array([[[0.0, 0.0, 0.0], [0.0, 0.0, 10.0]]])
    r = force_ramp_pairs(x, [[2, 5]], [[0.003, 0.004]], [[1.0, 1.0]], init=init)[0]
    assert np.array_equal(r.init, init[0]) and np.allclose(r.velo[1], [0.0, 0.0, 1.0])
    with pytest.raises(InputError):
        force_ramp_pairs(x, [[2, 7]], [[0.003, 0.004]], [[1.0, 1.0]])


def test_restart_file_keeps_the_trap_starts(tmp_path):
    x = np.arange(15.0).reshape(5, 3)
    init = np.arange(12.0).reshape(2, 2, 3) + 0.5
    p = tmp_path / "a.rst"
    write_rst(p, 99, x, x, x, grep=3, twz_init=init, box=[50.0, 50.0, 50.0])
    b = p.read_bytes()
    off = 20 + 3 * (16 + 8 * 15)  # step block, then xyz, velo, accel
    assert struct.unpack_from("<iiii", b, off) == (RST_TWZ, 8 + 8 * 12, 3, 2)
    r = read_rst(p)
    assert np.array_equal(r.twz_init[3], init) and np.array_equal(r.box, [50.0] * 3)
    bad = bytearray(b)
    struct.pack_into("<i", bad, off + 12, 3)  # three pairs claimed, two stored
    (tmp_path / "bad.rst").write_bytes(bytes(bad))
    with pytest.raises(ValueError, match="trap pairs"):
        read_rst(tmp_path / "bad.rst")
