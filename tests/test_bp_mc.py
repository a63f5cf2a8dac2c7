"""Base-pair Monte Carlo removal (force_bp_limit_triplet.F90; job_md.F90
scheduling) on the GPU against the oracle's restatement.

Fed the uniforms the oracle drew from its MT stream, the device pass removes
the same pairs and gives the same forces (FP64 path).  The survivors are the
mask of the following evaluations.  On device Philox uniforms, no nucleotide
keeps more than max_bp_per_nt pairs through dynamics.
"""
import numpy as np
import pytest

from helpers import max_rel
from oracle.oracle import Oracle
from sis_gb300 import FP64, MIXED
from sis_gb300.coil import random_coil
from sis_gb300.engine import Engine
from sis_gb300.model import Chain, Instance, Options, System

pytestmark = pytest.mark.gpu
SEQ = "GGGGCAAAAGCCCCAAAAGGGGAAAACCCC"


def hairpin(ff, model, seed, nstep_mc=1):
    rng = np.random.default_rng(seed)
    x = random_coil(rng, 30, amin_deg=60.0, amax_deg=100.0, rmin=3.0)
    inst = Instance([Chain.from_string(SEQ)], tempK=300.0, ionic_strength=0.15, xyz=x)
    opts = Options(bp_model=model, nstep_bp_mc=nstep_mc, max_bp_per_nt=1)
    if model == 5:
        opts.ele_cutoff_type, opts.ele_cutoff = 2, 20.0
    return System(ff, opts, [inst])


def survivors(records, status):
    return {tuple(r[:2]) for r, s in zip(np.asarray(records).tolist(), status) if s}


@pytest.mark.parametrize("model,seed", [(1, 5), (5, 5), (5, 9)])
def test_mc_pass_matches_oracle_with_its_draws(model, seed, sis_ff, nn_ff):
    sysm = hairpin(nn_ff if model == 5 else sis_ff, model, seed)
    orc = Oracle.from_instance(sysm, 0)
    orc.seed(3)
    orc.neighbor_list(0)
    f_ref = orc.force_mc(0)
    draws = orc.mc_draws()
    ref = survivors(orc.get_list(0, 2), orc.bp_status(0))
    assert len(draws) > 0
    eng = Engine(sysm, precision=FP64)
    eng.bp_mc(0, draws)
    f = eng.force(0)
    got = survivors(eng.get_list(0, 2), eng.get_bp_status(0))
    assert got == ref
    assert max_rel(f, f_ref) < 1e-12
    # the survivors mask the next (plain) evaluations, on both sides
    assert max_rel(eng.force(0), orc.force(0)) < 1e-12
    assert survivors(eng.get_list(0, 2), eng.get_bp_status(0)) <= ref


@pytest.mark.parametrize("nstep_mc", [1, 5])
def test_mc_limit_holds_through_dynamics(nstep_mc, nn_ff):
    sysm = hairpin(nn_ff, 5, 7, nstep_mc=nstep_mc)
    eng = Engine(sysm, precision=MIXED, seed=4)
    eng.init_velocities()
    for _ in range(6):
        eng.step(25)
        eng.bp_mc(0)
        eng.force(0)
        rec = np.asarray(eng.get_list(0, 2))
        st = eng.get_bp_status(0)
        pairs = rec[st == 1][:, :2].ravel()
        if pairs.size:
            assert np.bincount(pairs).max() <= 1
