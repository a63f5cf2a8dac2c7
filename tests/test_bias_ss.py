"""Base pairs restricted to a given secondary structure (read_ss.F90, the
ct/bpseq/bpl inputs of [Files.In]; init_bp.F90:207-209) and the [Bias_SS]
constant pull (force_bp_triplet.F90:85-92, neighbor_list.F90:89-93).

CPU: the file readers and read_ss's checks; the oracle's restatement (only
allowed pairs become records; with the bias every allowed pair is listed at
any distance, and a pair outside its distance window is pulled together by
the bias force along its separation).  GPU (through the C ABI): records
bit-exact against the oracle, FP64 forces per term to 1e-12 and the mixed
path to the mixed-path bar, with the general kernels and after steps of the
per-block kernel of small instances.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from sis_gb300.coil import random_coil
from sis_gb300.inputs import filter_ss_pairs, parse_bpl, parse_bpseq, parse_ct
from sis_gb300.model import Chain, Instance, Options, System

SEQ = "GGGGCAAAAGCCCCAAAAGGGGAAAACCCC"
# the two stems, a pair at a chain end and an isolated pair of no known type
PAIRS = [(1, 14), (2, 13), (3, 12), (4, 11), (5, 10), (20, 29), (21, 28), (22, 27), (6, 15)]
KEPT = [(2, 13), (3, 12), (4, 11), (5, 10), (20, 29), (21, 28), (22, 27)]
PULL = 10.0 * 6.02214076e23 / 4184.0 * 1e-22  # 10 pN in kcal/mol/A (read_input.F90:1217)


def two_hairpins(ff, model, seed=3):
    x = random_coil(np.random.default_rng(seed), len(SEQ))
    inst = Instance([Chain.from_string(SEQ)], tempK=300.0, ionic_strength=0.15, xyz=x)
    opts = Options(bp_model=model)
    if model == 5:
        opts.ele_cutoff_type, opts.ele_cutoff = 2, 20.0
    return System(ff, opts, [inst])


def as_set(a):
    return set(map(tuple, np.asarray(a).tolist()))


# ------------------------------------------------------------------- CPU
def test_ss_file_readers():
    n = 6
    ct = "6 test\n1 G 0 2 6 1\n2 G 1 3 0 2\n3 A 2 4 0 3\n4 A 3 5 0 4\n5 C 4 6 0 5\n6 C 5 0 1 6\n"
    assert parse_ct(ct, n) == [(1, 6), (6, 1)]
    bpseq = "1 G 6\n2 G 5\n3 A 0\n4 A 0\n5 C 2\n6 C 1\n"
    assert parse_bpseq(bpseq, n) == [(1, 6), (2, 5), (5, 2), (6, 1)]
    assert parse_bpl("2 5\n3 4\n") == [(2, 5), (3, 4)]
    with pytest.raises(ValueError):
        parse_ct("7 x\n", n)
    with pytest.raises(ValueError):
        parse_bpseq("1 G 6\n3 G 5\n", 2)


def test_read_ss_checks(nn_ff):
    inst = two_hairpins(nn_ff, 5).instances[0]
    kept, warn = filter_ss_pairs(inst, PAIRS, bp_model=5)
    assert kept == KEPT
    # in models 3-5 the isolation check comes first (read_ss.F90)
    assert len(warn) == 2 and "chain end" in warn[0] and "isolated" in warn[1]
    kept, warn = filter_ss_pairs(inst, PAIRS, bp_model=1)
    assert kept == KEPT and "known type" in warn[1]
    # the minimum loop and, in models 3-5, isolated pairs
    kept, warn = filter_ss_pairs(inst, [(10, 13), (3, 24)], bp_model=5)
    assert kept == [] and "minimum loop" in warn[0] and "isolated" in warn[1]
    kept, _ = filter_ss_pairs(inst, [(3, 24)], bp_model=1)
    assert kept == []  # G-A: no known type


def test_oracle_lists_only_allowed_pairs(nn_ff):
    sysm = two_hairpins(nn_ff, 5)
    o = Oracle.from_instance(sysm, 0)
    o.set_ss_pairs(KEPT)
    o.neighbor_list(0)
    got = {tuple(r[:2]) for r in np.asarray(o.get_list(0, 2)).tolist()}
    assert got <= set(KEPT)
    o.set_bias_ss(PULL)
    o.neighbor_list(0)
    got = {tuple(r[:2]) for r in np.asarray(o.get_list(0, 2)).tolist()}
    assert got == set(KEPT)  # every allowed pair, at any distance


def test_oracle_bias_pull_outside_the_window(nn_ff):
    """A stretched start: every allowed pair lies outside its distance window,
    so the base-pair force is the pull alone, bias_ss_force along each pair's
    separation (pair types with dG < 0)."""
    sysm = two_hairpins(nn_ff, 5)
    x = np.stack([np.arange(len(SEQ)) * 5.9, np.zeros(len(SEQ)), np.zeros(len(SEQ))], axis=1)
    sysm.instances[0].xyz = x
    o = Oracle.from_instance(sysm, 0)
    o.set_ss_pairs(KEPT)
    o.set_bias_ss(PULL)
    o.neighbor_list(0)
    f = o.force_term(0, 4)
    ref = np.zeros_like(f)
    rec = np.asarray(o.get_list(0, 2))
    coef = o.get_bp_coef(0)  # (dH, dS) of every record
    for k, r in enumerate(rec.tolist()):
        i, j = r[0] - 1, r[1] - 1
        if coef[k][0] - 300.0 * coef[k][1] >= 0.0:
            continue
        v = x[i] - x[j]
        pull = PULL / np.linalg.norm(v) * v
        ref[i] -= pull
        ref[j] += pull
    assert np.abs(f - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
    assert np.abs(ref).max() > 0.5 * PULL


# ------------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("model", [1, 5])
@pytest.mark.parametrize("bias", [False, True])
def test_ss_records_and_forces_match_oracle(model, bias, sis_ff, nn_ff):
    from helpers import max_rel, rms_rel
    from sis_gb300 import FP64, MIXED
    from sis_gb300.engine import Engine

    sysm = two_hairpins(nn_ff if model == 5 else sis_ff, model)
    o = Oracle.from_instance(sysm, 0)
    o.set_ss_pairs(KEPT)
    if bias:
        o.set_bias_ss(PULL)
    o.neighbor_list(0)
    for prec in (FP64, MIXED):
        eng = Engine(sysm, precision=prec)
        eng.set_ss_pairs(0, KEPT)
        if bias:
            eng.set_bias_ss(PULL)
        eng.neighbor_list(0)
        assert as_set(eng.get_list(0, 2)) == as_set(o.get_list(0, 2))
        if prec == FP64:
            fb, fo = eng.force_term(0, 4), o.force_term(0, 4)
            assert np.abs(fb - fo).max() <= 1e-12 * max(1.0, np.abs(fo).max())
            assert max_rel(eng.force(0), o.force(0)) < 1e-12
        else:
            assert rms_rel(eng.force(0), o.force(0)) < 1e-5
        eng.close()


@pytest.mark.gpu
def test_ss_records_after_small_kernel_steps(nn_ff):
    """The per-block kernel's rebuilds take the records of an instance with a
    structure from its partner table: with no list margin the lists after
    the steps belong to the final positions and equal the oracle's."""
    from sis_gb300 import MIXED
    from sis_gb300.engine import Engine

    sysm = two_hairpins(nn_ff, 5)
    sysm.opts.nl_margin = 0.0
    eng = Engine(sysm, precision=MIXED, seed=2)
    eng.set_ss_pairs(0, KEPT)
    eng.set_bias_ss(PULL)
    eng.init_velocities()
    eng.step(40)
    assert eng.stats()["small_blocks"] > 0
    x = eng.get_state(0)[0]
    o = Oracle.from_instance(sysm, 0)
    o.set_xyz(0, x)
    o.set_ss_pairs(KEPT)
    o.set_bias_ss(PULL)
    o.neighbor_list(0)
    for kind in (0, 1, 2):
        assert as_set(eng.get_list(0, kind)) == as_set(o.get_list(0, kind)), kind
