"""Optional terms of force.F90:62-75 on the GPU against the oracle's
restatement: the stage wall (force_stage.F90), tweezers with constant-force
and force-ramp trap pairs (force_tweezers.F90), the Rg bias (force_rg.F90)
and sigmoid restraints (force_restraint.F90).

* force term 7 and the full force: FP64 path to 1e-12, mixed path to the
  1e-5 bar (the terms are evaluated in FP64 there too; only the fixed-point
  scatter rounds them);
* energy slots 7-10 to 1e-12 in both paths;
* a fed-noise Langevin run with every term on follows the oracle to 1e-10
  after 10 steps, which also checks that the force-ramp traps move with the
  step being taken;
* a flat-bottomed Rg bias exerts nothing while Rg <= rg0.
"""
import numpy as np
import pytest

from helpers import max_rel, rms_rel
from oracle.oracle import Oracle
from sis_gb300 import FP64, MIXED
from sis_gb300.coil import single_chain
from sis_gb300.engine import Engine
from sis_gb300.model import ConstantForcePair, ForceRampPair, Restraint

pytestmark = pytest.mark.gpu

RESTRAINTS = [Restraint(1, 20, 3.0, 15.0, 2.0, 60.0), Restraint(3, 12, 2.0, 20.0, 3.0, 100.0, to_bead=True)]
DCF = [ConstantForcePair(1, 20, (0.5, -0.3, 0.2))]
FR = [ForceRampPair(2, 19, (0.3, 0.2), ((0.0, 0.0, 20.0), (60.0, 5.0, 25.0)), ((0.01, 0.0, 0.0), (-0.02, 0.01, 0.0)))]


def lifted_chain(sis_ff):
    sysm = single_chain(sis_ff, n=20, seed=3)
    x = sysm.instances[0].xyz.copy()
    x[:, 2] += 9.0 - x[:, 2].min()
    sysm.instances[0].xyz = x
    return sysm


def with_terms(obj, rg0, oracle):
    obj.set_stage(5.0, 1.2)
    if oracle:
        obj.set_rg_bias(2.0, rg0)
        obj.set_restraints(RESTRAINTS)
        obj.set_tweezers(dcf=DCF, fr=FR)
    else:
        obj.set_rg_bias(0, 2.0, rg0)
        obj.set_restraints(0, RESTRAINTS)
        obj.set_tweezers(0, dcf=DCF, fr=FR)
    return obj


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_optional_terms_match_oracle(prec, sis_ff):
    sysm = lifted_chain(sis_ff)
    orc = Oracle.from_instance(sysm, 0)
    orc.neighbor_list(0)
    rg0 = 0.6 * orc.rg(0)
    with_terms(orc, rg0, True)
    eng = with_terms(Engine(sysm, precision=prec), rg0, False)
    ref7 = orc.force_term(0, 7)
    assert np.abs(ref7).max() > 0.1
    got7 = eng.force_term(0, 7)
    tol = 1e-12 if prec == FP64 else 1e-5
    assert max_rel(got7, ref7) < tol, max_rel(got7, ref7)
    ref = orc.force(0)
    got = eng.force(0)
    assert (max_rel(got, ref) if prec == FP64 else rms_rel(got, ref)) < tol
    orc.set_bp_energy_flag(0)
    eref = orc.energy_sumup(0)
    eng.invalidate_bp_cache()
    e = eng.energy_sumup(0)
    for k in (7, 8, 9, 10):
        assert abs(e[k] - eref[k]) <= 1e-12 * max(1.0, abs(eref[k])), (k, e[k], eref[k])


def test_fed_noise_trajectory_with_optional_terms(sis_ff):
    sysm = lifted_chain(sis_ff)
    n = sysm.nmp
    rng = np.random.default_rng(42)
    v0 = rng.normal(size=(n, 3)) * 0.04
    a0 = rng.normal(size=(n, 3)) * 0.01
    noise = rng.normal(size=(10, 1, n, 3))
    orc = Oracle.from_instance(sysm, 0)
    rg0 = 0.6 * orc.rg(0)
    with_terms(orc, rg0, True)
    orc.set_velos(0, v0)
    orc.set_accels(0, a0)
    orc.md_init()
    orc.run(10, noise)
    eng = with_terms(Engine(sysm, precision=FP64), rg0, False)
    eng.set_state(0, None, v0, a0)
    eng.step(10, noise.reshape(10, n, 3))
    x, v, a = eng.get_state(0)
    scale = np.abs(orc.get_xyz(0)).max()
    assert np.abs(x - orc.get_xyz(0)).max() <= 1e-10 * scale
    assert np.abs(v - orc.get_velos(0)).max() <= 1e-10 * np.abs(orc.get_velos(0)).max()


def test_flat_bottomed_rg_bias_is_off_inside(sis_ff):
    sysm = lifted_chain(sis_ff)
    orc = Oracle.from_instance(sysm, 0)
    rg = orc.rg(0)
    eng = Engine(sysm, precision=FP64)
    eng.set_rg_bias(0, 2.0, 1.5 * rg, flat=True)
    assert np.abs(eng.force_term(0, 7)).max() == 0.0
    assert eng.energy_sumup(0)[9] == 0.0
    eng.set_rg_bias(0, 2.0, 0.5 * rg, flat=True)
    assert np.abs(eng.force_term(0, 7)).max() > 0.0
    assert eng.energy_sumup(0)[9] > 0.0
    eng.set_rg_bias(0, 0.0, 0.0, off=True)
    assert np.abs(eng.force_term(0, 7)).max() == 0.0
