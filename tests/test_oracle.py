"""CPU checks of the FP64 oracle against the reference's golden vectors and
known-answer tests.

* CAG47 energies of the reference's regression test
  (check/test_DCD_CAG47: OpenMM energies of 25 DCD frames);
* MT19937 known answers (the C++ standard's mt19937 requirement: the 10000th
  output of the default seed 5489 is 4123659995);
* force = -grad(energy) by central differences, the reference's own
  consistency check (src/job_check_force.F90:57-82);
* neighbour-list membership recomputed independently with numpy.
"""
import numpy as np
import pytest

from helpers import cag47_system, t2s2hp_system, pbc_md_system
from oracle.oracle import MT, Oracle
from sis_gb300.coil import random_coil, single_chain
from sis_gb300.model import Chain, Instance, Options, System


def test_cag47_energies_match_openmm_golden():
    z = np.load(__import__("helpers").GOLDEN / "cag47.npz")
    sysm = cag47_system(0)
    orc = Oracle.from_instance(sysm, 0)
    for f in range(len(z["xyz"])):
        orc.set_xyz(0, z["xyz"][f].astype(np.float64))
        orc.neighbor_list(0)
        orc.set_bp_energy_flag(0)
        e = orc.energy_sumup(0)
        g = z["energy"][f]
        # columns: step, Ebond, Eangl, Eexv, Eele, -, Ebp, -; coordinates are float32
        assert abs(e[1] - g[1]) <= 1e-4 * abs(g[1]) + 1e-4
        assert abs(e[2] - g[2]) <= 1e-4 * abs(g[2]) + 1e-4
        assert abs(e[5] - g[3]) <= 2e-3 * abs(g[3]) + 1e-5
        # OpenMM used slightly different electrostatic constants (closer to the
        # reference's _HTN_CONSISTENT build): agreement to 0.6 %
        assert abs(e[6] - g[4]) <= 6e-3 * abs(g[4])


def test_mt19937_known_answers():
    m = MT(5489)
    first = m.int32()
    assert first == 3499211612
    for _ in range(9998):
        m.int32()
    assert m.int32() == 4123659995


def test_mt_double_ranges_and_boxmuller_moments():
    m = MT(123)
    u = np.array([m.double1() for _ in range(20000)])
    assert u.min() >= 0.0 and u.max() <= 1.0 and abs(u.mean() - 0.5) < 0.01
    g = np.array([m.boxmuller() for _ in range(100000)])
    assert abs(g.mean()) < 0.015 and abs(g.var() - 1.0) < 0.015


def _fd_check(orc, beads, h=1e-5):
    x0 = orc.get_xyz(0)
    orc.set_bp_energy_flag(0)
    f = orc.force(0)
    worst = 0.0
    scale = np.sqrt(np.mean(np.sum(f ** 2, axis=1)))
    for i in beads:
        for k in range(3):
            xp = x0.copy()
            xp[i, k] += h
            orc.set_xyz(0, xp)
            orc.set_bp_energy_flag(0)
            ep = orc.energy_sumup(0)[0]
            xp[i, k] -= 2 * h
            orc.set_xyz(0, xp)
            orc.set_bp_energy_flag(0)
            em = orc.energy_sumup(0)[0]
            fd = -(ep - em) / (2 * h)
            worst = max(worst, abs(fd - f[i, k]) / max(abs(f[i, k]), scale))
    orc.set_xyz(0, x0)
    return worst


def test_force_is_minus_energy_gradient_model1(sis_ff):
    sysm = single_chain(sis_ff, n=40, seed=11)
    orc = Oracle.from_instance(sysm, 0)
    orc.neighbor_list(0)
    assert _fd_check(orc, range(0, 40, 3)) < 2e-5


def test_force_is_minus_energy_gradient_model5_reb_expdih(nn_ff):
    sysm = t2s2hp_system(nn_ff)
    orc = Oracle.from_instance(sysm, 0)
    orc.neighbor_list(0)
    assert _fd_check(orc, range(27)) < 2e-5


def _biased_chain(sis_ff):
    """A 20-nt chain lifted above a stage wall at z = 0, with an Rg bias, two
    sigmoid restraints (one on both beads, one to a reference bead) and a
    constant-force trap pair."""
    from sis_gb300.model import ConstantForcePair, Restraint

    sysm = single_chain(sis_ff, n=20, seed=3)
    x = sysm.instances[0].xyz.copy()
    x[:, 2] += 9.0 - x[:, 2].min()
    sysm.instances[0].xyz = x
    orc = Oracle.from_instance(sysm, 0)
    orc.neighbor_list(0)
    orc.set_stage(5.0, 1.2)
    orc.set_rg_bias(2.0, 0.6 * orc.rg(0))
    orc.set_restraints([Restraint(1, 20, 3.0, 15.0, 2.0, 60.0), Restraint(3, 12, 2.0, 20.0, 3.0, 100.0, to_bead=True)])
    orc.set_tweezers(dcf=[ConstantForcePair(1, 20, (0.5, -0.3, 0.2))])
    return orc


def test_optional_terms_are_minus_energy_gradient(sis_ff):
    """Stage wall, Rg bias, sigmoid restraints and constant-force traps
    (force_stage/rg/restraint/tweezers.F90 against their energy routines).
    The reference bead of a to-bead restraint (bead 12) feels no force by
    design (force_restraint.F90:36-39), so its energy gradient is left out."""
    orc = _biased_chain(sis_ff)
    f7 = orc.force_term(0, 7)
    assert np.abs(f7).max() > 0.1
    e = orc.energy_sumup(0)
    assert all(abs(e[k]) > 1e-6 for k in (7, 8, 9, 10))
    assert _fd_check(orc, [b for b in range(20) if b != 11]) < 2e-5


def test_flat_bottomed_rg_bias_is_off_inside(sis_ff):
    orc = _biased_chain(sis_ff)
    orc.set_stage(0.0, 0.0)
    orc.set_restraints([])
    orc.set_tweezers()
    orc.set_rg_bias(2.0, 1.5 * orc.rg(0), flat=True)
    assert np.abs(orc.force_term(0, 7)).max() == 0.0 and orc.energy_sumup(0)[9] == 0.0
    orc.set_rg_bias(2.0, 0.5 * orc.rg(0), flat=True)
    assert np.abs(orc.force_term(0, 7)).max() > 0.0 and orc.energy_sumup(0)[9] > 0.0


def test_force_is_minus_energy_gradient_with_pairs(sis_ff):
    """A compact structure so that WCA, DH and base pairs all contribute."""
    rng = np.random.default_rng(5)
    n = 30
    x = random_coil(rng, n, amin_deg=60.0, amax_deg=100.0, rmin=3.0)
    inst = Instance([Chain.from_string("GGGGCAAAAGCCCCAAAAGGGGAAAACCCC")], tempK=300.0, ionic_strength=0.15, xyz=x)
    orc = Oracle.from_instance(System(sis_ff, Options(bp_model=1), [inst]), 0)
    orc.neighbor_list(0)
    assert len(orc.get_list(0, 0)) > 0
    assert _fd_check(orc, range(n)) < 5e-5


def _ref_lists(sysm):
    """neighbor_list.F90 membership recomputed with numpy (no bp)."""
    inst = sysm.instances[0]
    o = sysm.opts
    x = np.array(inst.xyz, dtype=np.float64)
    n = len(x)
    if inst.box is not None:
        L = np.array(inst.box)
        for k in range(3):
            hi = x[:, k] > L[k]
            lo = x[:, k] < 0
            x[hi, k] = x[hi, k] - L[k] * (np.trunc((x[hi, k] - L[k]) / L[k]) + 1)
            x[lo, k] = x[lo, k] + L[k] * (np.trunc((0 - x[lo, k]) / L[k]) + 1)
    chain = np.concatenate([[c] * len(ch) for c, ch in enumerate(inst.chains)])
    loc = np.concatenate([np.arange(1, len(ch) + 1) for ch in inst.chains])
    wca, ele = set(), set()
    wc2 = (sysm.ff.wca_sigma + o.nl_margin) ** 2
    ec2 = (o.ele_cutoff + o.nl_margin) ** 2
    for i in range(n):
        v = x[i] - x[i + 1:]
        if inst.box is not None:
            for k in range(3):
                c = v[:, k]
                c[c > L[k] / 2] -= L[k]
                c[c < -L[k] / 2] += L[k]
        d2 = v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2]
        for jj in np.nonzero(d2 <= max(wc2, ec2))[0]:
            j = i + 1 + jj
            same = chain[i] == chain[j]
            if d2[jj] <= wc2 and not (same and loc[i] + 2 >= loc[j]):
                wca.add((i + 1, j + 1))
            if d2[jj] <= ec2 and not (same and loc[j] - loc[i] in (1, 2)):
                ele.add((i + 1, j + 1))
    return wca, ele


@pytest.mark.parametrize("which", ["cag47", "test_md_pbc"])
def test_neighbor_list_membership_matches_numpy(which, sis_ff):
    sysm = cag47_system(3) if which == "cag47" else pbc_md_system(sis_ff, 1)
    orc = Oracle.from_instance(sysm, 0)
    orc.neighbor_list(0)
    wca, ele = _ref_lists(sysm)
    assert set(map(tuple, orc.get_list(0, 0).tolist())) == wca
    assert set(map(tuple, orc.get_list(0, 1).tolist())) == ele


def test_gjf2gj_one_step_matches_update_formula(sis_ff):
    sysm = single_chain(sis_ff, n=32, seed=3)
    orc = Oracle.from_instance(sysm, 0)
    orc.md_init()
    rng = np.random.default_rng(0)
    v0 = rng.normal(size=(32, 3)) * 0.03
    a0 = rng.normal(size=(32, 3)) * 0.01
    orc.set_velos(0, v0)
    orc.set_accels(0, a0)
    x0 = orc.get_xyz(0)
    f = orc.force(0)
    xi = rng.normal(size=(1, 1, 32, 3))
    orc.run(1, xi)
    c = orc.get_md_coef(0)
    bn = c[:, 3:4] * xi[0, 0]
    v1 = c[:, 0:1] * v0 + c[:, 1:2] * f + (a0 + bn)
    x1 = x0 + c[:, 2:3] * v1
    assert np.allclose(orc.get_velos(0), v1, rtol=1e-14, atol=0)
    assert np.allclose(orc.get_xyz(0), x1, rtol=1e-15, atol=0)
    assert np.allclose(orc.get_accels(0), bn, rtol=0, atol=0)


def test_set_ele_values_are_physical(sis_ff):
    sysm = single_chain(sis_ff, n=8, seed=1)
    orc = Oracle.from_instance(sysm, 0)
    ele_coef, lam, cut, diele = orc.get_ele(0)
    assert 77.0 < diele < 78.5  # water at 300 K (Malmberg-Maryott)
    assert 7.6 < lam < 8.2  # Debye length at 150 mM
    assert cut == 50.0
    kB = orc.L.or_const(1)
    assert abs(kB - 0.0019872) < 1e-6


@pytest.mark.parametrize("integ", ["GJF2GJ", "BD_EM"])
def test_frozen_beads_stay_where_they_are(integ, sis_ff):
    """[Freeze] (job_md.F90:713-729,745-748): the position coefficient of a
    frozen bead is zero, so it keeps its place through a run while the
    others move; GJF-2GJ velocities of frozen beads still evolve."""
    from sis_gb300 import model
    from sis_gb300.coil import single_chain

    sysm = single_chain(sis_ff, n=16, seed=12)
    sysm.opts.integrator = getattr(model, integ)
    orc = Oracle.from_instance(sysm, 0)
    md0 = orc.get_md_coef(0)
    frozen = [1, 6, 7, 16]
    orc.set_frozen(frozen)
    md = orc.get_md_coef(0)
    idx = np.array(frozen) - 1
    other = np.setdiff1d(np.arange(16), idx)
    if integ == "GJF2GJ":
        keep = np.ix_(idx, [0, 1, 3])
        assert np.all(md[idx, 2] == 0.0) and np.array_equal(md[keep], md0[keep])
    else:
        assert np.all(md[idx, 0] == 0.0) and np.all(md[idx, 3] == 0.0)
    assert np.array_equal(md[other], md0[other])
    x0 = orc.get_xyz(0)
    rng = np.random.default_rng(4)
    orc.set_velos(0, rng.normal(size=(16, 3)) * 0.05)
    orc.md_init()
    orc.run(20, rng.normal(size=(20, 1, 16, 3)))
    x1 = orc.get_xyz(0)
    assert np.array_equal(x1[idx], x0[idx])
    assert np.all(np.abs(x1[other] - x0[other]).max(axis=1) > 0)
    if integ == "GJF2GJ":
        assert np.abs(orc.get_velos(0)[idx]).max() > 0


@pytest.mark.parametrize("seq,lists,terms", [
    ("A", (0, 0, 0), ()),
    ("AC", (0, 0, 0), (1,)),
    ("ACG", (0, 0, 0), (1, 2)),
    ("ACGU", (1, 1, 0), (1, 2, 3, 5, 6)),  # (1,4): WCA and Debye-Hueckel; no base pair within min_loop
    ("DDDD", (0, 0, 0), (1, 2, 3)),  # dummy beads: no WCA (neighbor_list.F90:123), no charge
    ("AAAAAAAAAA", (22, 28, 0), (1, 2, 3, 5, 6)),  # A-A never pairs; |i-j| >= 3 for WCA and ele
])
def test_short_and_dummy_chains(seq, lists, terms, sis_ff):
    """Edge cases of the list rules and term counts: chains of one to four
    beads, a chain of dummy beads and one that cannot pair; forces stay
    finite and equal minus the energy gradient."""
    n = len(seq)
    # a helix (bond 6.8 A, bend 98 degrees): no angle comes near straight,
    # where force_angl.F90:57-60 clamps |v21 x v32|^2 to 1 on purpose
    ph = np.radians(100.0) * np.arange(n)
    x = np.stack([4.0 * np.cos(ph), 4.0 * np.sin(ph), 3.0 * np.arange(n)], axis=1)
    sysm = System(sis_ff, Options(bp_model=1), [Instance([Chain.from_string(seq)], xyz=x)])
    o = Oracle.from_instance(sysm, 0)
    o.neighbor_list(0)
    assert tuple(len(o.get_list(0, k)) for k in range(3)) == lists
    e = o.energy_sumup(0)
    assert [k for k in range(1, 7) if e[k] != 0.0] == list(terms)
    f = o.force(0)
    assert np.all(np.isfinite(f))
    h = 1e-5
    for i in range(n):
        for a in range(3):
            ep = []
            for s in (h, -h):
                y = x.copy()
                y[i, a] += s
                o.set_xyz(0, y)
                o.set_bp_energy_flag(0)
                ep.append(o.energy_sumup(0)[0])
            assert abs(-(ep[0] - ep[1]) / (2 * h) - f[i, a]) <= 1e-5 * max(1.0, abs(f[i, a]))
    o.set_xyz(0, x)


def test_near_straight_angle_force_is_clamped_as_the_reference_does(sis_ff):
    """force_angl.F90:50-64: below |v21 x v32|^2 = 1 A^4 the denominator is
    held at 1, so near 180 degrees the force is smaller than minus the energy
    gradient, by design.  Checked against the formula written out here."""
    x = np.array([[0.0, 0.0, 0.0], [5.9, 0.05, 0.0], [11.8, 0.0, 0.08]])
    sysm = System(sis_ff, Options(bp_model=1), [Instance([Chain.from_string("ACG")], xyz=x)])
    o = Oracle.from_instance(sysm, 0)
    o.neighbor_list(0)
    f = o.force_term(0, 2)
    v21, v32 = x[1] - x[0], x[2] - x[1]
    d21, d32, d2132 = v21 @ v21, v32 @ v32, v32 @ v21
    assert d21 * d32 - d2132 ** 2 < 1.0
    k, t0 = sis_ff.angl_k, sis_ff.angl_t0
    delta = np.arccos(max(-1.0, min(1.0, -d2132 / np.sqrt(d21 * d32)))) - t0
    g = k * delta / 1.0
    f21 = g * (v21 * (d2132 / d21) - v32)
    f32 = g * (v32 * (d2132 / d32) - v21)
    want = np.array([-f21, f21 - f32, f32])
    assert np.allclose(f, want, rtol=1e-12, atol=1e-14)


# ------------------------------------------------------ MT jump-ahead streams
def test_mt_jump_ahead_matches_stepping():
    """mt_create_stream at the library's _DEBUG_ distance 2^16
    (mt_stream.F90:96-97): stream id starts id * 65536 outputs after the base
    (whose pointer is at 624, right after init_by_scalar)."""
    from oracle.oracle import MT

    base = MT(4357)
    outs = [base.int32() for _ in range(3 * 65536 + 16)]
    for sid in (1, 2, 3):
        s = MT(4357).jumped(16, sid)
        assert [s.int32() for _ in range(16)] == outs[sid * 65536: sid * 65536 + 16], sid


def test_reference_replica_streams():
    """init_mts.F90:21-43: replica r draws from stream (r + 1 + replica_run)
    * 2^256; with the seed and a replica run, replicas differ and restarting
    the derivation gives the same draws."""
    from oracle.oracle import MT

    a = MT(1234).jumped(256, 2)
    b = MT(1234).jumped(256, 2)
    assert [a.int32() for _ in range(8)] == [b.int32() for _ in range(8)]
    c = MT(1234).jumped(256, 3)
    assert [MT(1234).jumped(256, 2).int32() for _ in range(1)] != [c.int32()]
