"""[Freeze] on the GPU (set_md_coef, job_md.F90:713-729,745-748): the
frozen beads' coefficients against the oracle's, and fed-noise runs of both
integrators in which the frozen beads keep their places exactly and the
rest follows the oracle."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from sis_gb300 import BD_EM, FP64, GJF2GJ
from sis_gb300._abi import SisError
from sis_gb300.coil import random_coil
from sis_gb300.engine import Engine
from sis_gb300.model import Chain, Instance, Options, System

pytestmark = pytest.mark.gpu

FROZEN = [1, 6, 7, 24]


def _chain(sis_ff, integrator):
    rng = np.random.default_rng(1001)
    x = random_coil(rng, 24, rmin=10.0)
    sysm = System(sis_ff, Options(bp_model=1), [Instance([Chain(rng.integers(0, 4, 24).astype(np.int32))],
                                                         tempK=300.0, ionic_strength=0.15, xyz=x)])
    sysm.opts.integrator = integrator
    if integrator == BD_EM:
        # water viscosity keeps the explicit BD step stable (h/gamma * k_bond < 1)
        sysm.opts.viscosity_Pas = 8.9e-4
    return sysm


@pytest.mark.parametrize("integrator", [GJF2GJ, BD_EM])
def test_frozen_beads_match_oracle_and_stay(integrator, sis_ff):
    sysm = _chain(sis_ff, integrator)
    n = sysm.nmp
    rng = np.random.default_rng(7)
    v0 = rng.normal(size=(n, 3)) * 0.05 if integrator == GJF2GJ else np.zeros((n, 3))
    a0 = rng.normal(size=(n, 3)) * 0.01 if integrator == GJF2GJ else np.zeros((n, 3))
    noise = rng.normal(size=(10, 1, n, 3))
    orc = Oracle.from_instance(sysm, 0)
    orc.set_frozen(FROZEN)
    orc.set_velos(0, v0)
    orc.set_accels(0, a0)
    orc.md_init()
    eng = Engine(sysm, precision=FP64)
    eng.set_frozen(0, FROZEN)
    assert np.allclose(eng.get_md_coef(0), orc.get_md_coef(0), rtol=1e-14, atol=0)
    orc.run(10, noise)
    eng.set_state(0, None, v0, a0)
    eng.step(10, noise.reshape(10, n, 3))
    x = eng.get_state(0)[0]
    idx = np.array(FROZEN) - 1
    assert np.array_equal(x[idx], sysm.instances[0].xyz[idx])
    assert np.abs(x - orc.get_xyz(0)).max() <= 1e-10 * np.abs(orc.get_xyz(0)).max()
    # an empty set frees every bead again; a bead number out of range is refused
    eng.set_frozen(0, [])
    orc.set_frozen([])
    assert np.allclose(eng.get_md_coef(0), orc.get_md_coef(0), rtol=1e-14, atol=0)
    with pytest.raises(SisError):
        eng.set_frozen(0, [n + 1])
