"""GPU parity: libsisgpu (through the C ABI) against the FP64 oracle.

Bars (from the engine's specification):
* list membership (WCA, DH, base-pair records and their dH/dS) bit-exact;
* FP64 path: forces per term within 1e-12 (norm-wise, per bead relative to
  max(|F_ref|, rms F_ref)), energies within 1e-12 relative;
* mixed path (FP32 terms, FP64 accumulation/integration): force RMS relative
  error <= 1e-5;
* a Langevin run fed the oracle's noise array matches its positions to 1e-10
  after 10 steps (FP64 path).
"""
import numpy as np
import pytest

from helpers import cag47_system, max_rel, pbc_md_system, rms_rel, t2s2hp_system
from oracle.oracle import Oracle
from sis_gb300 import BD_EM, FP64, GJF2GJ, MIXED
from sis_gb300._abi import SisError
from sis_gb300.coil import crowded_box, random_coil, single_chain, uneven_batch
from sis_gb300.engine import Engine
from sis_gb300.model import MOLT_CIRC, Chain, Instance, Options, System

pytestmark = pytest.mark.gpu

FORCE_TOL_FP64 = 1e-12
ENERGY_TOL_FP64 = 1e-12
FORCE_RMS_TOL_MIXED = 1e-5


def compact_system(ff):
    rng = np.random.default_rng(5)
    x = random_coil(rng, 30, amin_deg=60.0, amax_deg=100.0, rmin=3.0)
    inst = Instance([Chain.from_string("GGGGCAAAAGCCCCAAAAGGGGAAAACCCC")], tempK=300.0, ionic_strength=0.15, xyz=x)
    return System(ff, Options(bp_model=1), [inst])


def near_collinear_bp_system(ff, sin_theta):
    """One G-C base-pair record (strands GGG / CCC, middle beads paired) whose
    flanking bond angle imp+1 -- imp -- jmp has sine sin_theta (nearly 0 deg);
    the other three flanking angles sit near their minima."""
    u12 = np.array([-1.0, 0.0, 0.0])

    def arm(theta, e):
        e = np.asarray(e, float) / np.linalg.norm(e)
        return 5.84 * (np.cos(theta) * u12 + np.sin(theta) * e)

    x1, x2 = np.zeros(3), np.array([13.8, 0.0, 0.0])
    xyz = np.stack([x1 - arm(1.83, [0, 0.6, 0.8]), x1, x1 - arm(np.arcsin(sin_theta), [0, 1, 0.3]),
                    x2 + arm(1.83, [0, -0.8, 0.6]), x2, x2 + arm(0.94, [0, 0.28, -0.96])])
    inst = Instance([Chain.from_string("GGG"), Chain.from_string("CCC")], tempK=300.0, ionic_strength=0.15, xyz=xyz)
    return System(ff, Options(bp_model=1), [inst])


def near_straight_chain_system(ff, sin_theta):
    """Five beads whose middle bond angle 1-2-3 has sine sin_theta (nearly
    180 deg): it is the angle term's own angle and a flanking angle of both
    dihedrals; the outer angles sit near 150 deg, out of plane."""
    ex, ey = np.array([1.0, 0.0, 0.0]), np.array([0.0, 1.0, 0.0])
    phi = np.arcsin(sin_theta)
    x2 = np.zeros(3)
    x1 = x2 - 5.84 * ex
    x3 = x2 + 5.84 * (np.cos(phi) * ex + np.sin(phi) * ey)

    def arm(a, b, e):
        u = (b - a) / np.linalg.norm(b - a)
        e = np.asarray(e, float) - (np.asarray(e, float) @ u) * u
        e /= np.linalg.norm(e)
        t = np.pi - 2.6
        return b + 5.84 * (np.cos(t) * u + np.sin(t) * e)

    x0 = arm(x2, x1, [0.0, 0.6, 0.8])
    x4 = arm(x2, x3, [0.0, -0.3, 0.95])
    inst = Instance([Chain.from_string("AAAAA")], tempK=300.0, ionic_strength=0.15, xyz=np.stack([x0, x1, x2, x3, x4]))
    return System(ff, Options(bp_model=1), [inst])


def circ_system(ff):
    rng = np.random.default_rng(9)
    seq = rng.integers(0, 4, 48).astype(np.int32)
    t = np.linspace(0, 2 * np.pi, 48, endpoint=False)
    x = np.stack([45 * np.cos(t), 45 * np.sin(t), 8 * np.sin(3 * t)], axis=1) + rng.normal(scale=0.3, size=(48, 3))
    inst = Instance([Chain(seq, MOLT_CIRC)], tempK=310.0, ionic_strength=0.1, xyz=x)
    return System(ff, Options(bp_model=3), [inst])


def cell_system(ff):
    return crowded_box(ff, n_chains=12, n=500, molar=0.05, seed=21)


SYSTEMS = {
    "cag47": lambda ff, nn: cag47_system(7),
    "chain64": lambda ff, nn: single_chain(ff, n=64, seed=1001),
    "pbc564": lambda ff, nn: pbc_md_system(ff, 1),
    "t2s2hp_model5": lambda ff, nn: t2s2hp_system(nn),
    "compact_bp": lambda ff, nn: compact_system(ff),
    "circ": lambda ff, nn: circ_system(ff),
    "cells6000": lambda ff, nn: cell_system(ff),
}


@pytest.fixture(scope="module")
def systems(sis_ff, nn_ff):
    return {k: f(sis_ff, nn_ff) for k, f in SYSTEMS.items()}


def oracle_for(sysm, k=0):
    o = Oracle.from_instance(sysm, k)
    o.neighbor_list(0)
    return o


def as_set(a):
    return set(map(tuple, np.asarray(a).tolist()))


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_lists_bit_exact(name, systems):
    sysm = systems[name]
    orc = oracle_for(sysm)
    eng = Engine(sysm, precision=FP64)
    eng.neighbor_list(-1)
    for kind in (0, 1, 2):
        assert as_set(eng.get_list(0, kind)) == as_set(orc.get_list(0, kind)), (name, kind)
    # dH/dS of each base-pair record
    g = {tuple(r): tuple(c) for r, c in zip(eng.get_list(0, 2).tolist(), eng.get_bp_coef(0).tolist())}
    o = {tuple(r): tuple(c) for r, c in zip(orc.get_list(0, 2).tolist(), orc.get_bp_coef(0).tolist())}
    assert g == o
    # wrapped coordinates after the rebuild (pbc_wrap) are bit-identical
    assert np.array_equal(eng.get_state(0)[0], orc.get_xyz(0))


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_fp64_forces_per_term(name, systems):
    sysm = systems[name]
    orc = oracle_for(sysm)
    eng = Engine(sysm, precision=FP64)
    for term in range(1, 7):
        ref = orc.force_term(0, term)
        got = eng.force_term(0, term)
        if not np.any(ref):
            assert not np.any(got), (name, term)
            continue
        assert max_rel(got, ref) < FORCE_TOL_FP64, (name, term, max_rel(got, ref))
    ref = orc.force(0)
    assert max_rel(eng.force(0), ref) < FORCE_TOL_FP64


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_fp64_energies(name, systems):
    sysm = systems[name]
    orc = oracle_for(sysm)
    eng = Engine(sysm, precision=FP64)
    orc.set_bp_energy_flag(0)
    ref = orc.energy_sumup(0)
    eng.invalidate_bp_cache()
    got = eng.energy_sumup(0)
    scale = np.abs(ref[1:7]).sum()
    for k in range(1, 7):
        assert abs(got[k] - ref[k]) <= ENERGY_TOL_FP64 * max(abs(ref[k]), 1e-3 * scale), (name, k, got[k], ref[k])
    # bp energies cached by the force call (flg_bp_energy) equal the recomputed ones
    eng.force(0)
    assert abs(eng.energy_sumup(0)[4] - ref[4]) <= 1e-12 * max(1.0, abs(ref[4]))


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_mixed_precision_force_error(name, systems):
    sysm = systems[name]
    orc = oracle_for(sysm)
    eng = Engine(sysm, precision=MIXED)
    ref = orc.force(0)
    err = rms_rel(eng.force(0), ref)
    assert err <= FORCE_RMS_TOL_MIXED, (name, err)
    orc.set_bp_energy_flag(0)
    eref = orc.energy_sumup(0)
    eng.invalidate_bp_cache()
    e = eng.energy_sumup(0)
    assert abs(e[0] - eref[0]) <= 1e-5 * np.abs(eref[1:7]).sum()


@pytest.mark.parametrize("sin_theta", [0.02, 1e-2, 1e-3, 1e-4, 1e-5])
def test_bonded_near_straight_angle(sin_theta, sis_ff):
    """A bond angle within 0.8 deg of 180 deg: the mixed path evaluates the
    angle term and the two dihedrals it flanks again from cross products
    formed exactly from the fixed-point mirror (cross_fx) and keeps the 1e-5
    bar down to sin = 1e-5 without FP64.  The dihedral forces grow as
    1/sin there.  The FP64 tolerance follows the eps / sin^2 conditioning of
    the reference's formulas, as for the base-pair angles."""
    sysm = near_straight_chain_system(sis_ff, sin_theta)
    orc = oracle_for(sysm)
    tol64 = max(FORCE_TOL_FP64, 2.2e-16 / sin_theta ** 2)
    for term in (2, 3):
        ref = orc.force_term(0, term)
        assert np.abs(ref).max() > 1e-3
        for prec, tol in ((FP64, tol64), (MIXED, FORCE_RMS_TOL_MIXED)):
            got = Engine(sysm, precision=prec).force_term(0, term)
            assert max_rel(got, ref) < tol, (term, prec, max_rel(got, ref))


@pytest.mark.parametrize("sin_theta", [0.1, 0.031, 0.029, 1e-3, 3e-5])
def test_base_pair_near_collinear_angle(sin_theta, sis_ff):
    """sin >= 0.03: the FP32 base-pair term (atan2 angles, compensated cross
    products of FP32 separations) keeps the 1e-5 bar where acos would not;
    below, the mixed path recomputes the four cross products exactly from the
    fixed-point mirror and its residuals.  The reference's angle forces divide
    by sqrt(|a|^2 |b|^2 - (a.b)^2), whose rounding error grows as
    eps / sin^2: FP64 results that round differently (FMA contraction) agree
    with the oracle to that bound, not to 1e-12, at the smallest angles."""
    sysm = near_collinear_bp_system(sis_ff, sin_theta)
    orc = oracle_for(sysm)
    ref = orc.force_term(0, 4)
    assert len(orc.get_list(0, 2)) == 1 and np.abs(ref).max() > 1e-3
    tol64 = max(FORCE_TOL_FP64, 2.2e-16 / sin_theta ** 2)
    for prec, tol in ((FP64, tol64), (MIXED, FORCE_RMS_TOL_MIXED)):
        eng = Engine(sysm, precision=prec)
        got = eng.force_term(0, 4)
        assert max_rel(got, ref) < tol, (prec, max_rel(got, ref))


def test_radius_of_gyration_matches_oracle(sis_ff):
    """energy_rg.F90:17-26 for every instance of an uneven batch, after steps."""
    sysm = uneven_batch(sis_ff, n_inst=8, lmin=20, lmax=120, seed=78)
    eng = Engine(sysm, precision=FP64, seed=4)
    eng.step(30)
    x = eng.get_state(-1)[0]
    off = sysm.offsets()
    rg = eng.rg()
    for k in range(len(sysm.instances)):
        orc = Oracle.from_instance(sysm, k)
        orc.set_xyz(0, x[off[k]:off[k + 1]])
        assert abs(rg[k] - orc.rg(0)) <= 1e-12 * orc.rg(0), k
        assert eng.rg(k)[0] == rg[k]


def test_batched_instances_match_their_own_oracles(sis_ff):
    sysm = uneven_batch(sis_ff, n_inst=8, lmin=20, lmax=120, seed=77)
    eng = Engine(sysm, precision=FP64)
    for k in range(len(sysm.instances)):
        orc = oracle_for(sysm, k)
        for kind in (0, 1, 2):
            assert as_set(eng.get_list(k, kind)) == as_set(orc.get_list(0, kind))
        assert max_rel(eng.force(k), orc.force(0)) < FORCE_TOL_FP64
        assert np.allclose(eng.get_ele(k), orc.get_ele(0), rtol=1e-15, atol=0)


@pytest.mark.parametrize("name", ["chain64", "pbc564", "t2s2hp_model5", "compact_bp"])
def test_fed_noise_trajectory_matches_oracle(name, systems):
    sysm = systems[name]
    n = sysm.nmp
    rng = np.random.default_rng(42)
    v0 = rng.normal(size=(n, 3)) * 0.04
    a0 = rng.normal(size=(n, 3)) * 0.01
    noise = rng.normal(size=(10, 1, n, 3))
    orc = Oracle.from_instance(sysm, 0)
    orc.set_velos(0, v0)
    orc.set_accels(0, a0)
    orc.md_init()
    orc.run(10, noise)
    eng = Engine(sysm, precision=FP64)
    eng.set_state(0, None, v0, a0)
    eng.step(10, noise.reshape(10, n, 3))
    x, v, a = eng.get_state(0)
    scale = np.abs(orc.get_xyz(0)).max()
    assert np.abs(x - orc.get_xyz(0)).max() <= 1e-10 * scale
    assert np.abs(v - orc.get_velos(0)).max() <= 1e-10 * np.abs(orc.get_velos(0)).max()
    assert np.array_equal(a, orc.get_accels(0))


@pytest.mark.parametrize("name", ["chain64", "pbc564", "compact_bp"])
def test_one_fed_noise_step_matches_oracle(name, systems):
    """One GJF-2GJ step fed the oracle's Gaussian array: positions to 1e-12."""
    sysm = systems[name]
    n = sysm.nmp
    rng = np.random.default_rng(8)
    v0 = rng.normal(size=(n, 3)) * 0.04
    a0 = rng.normal(size=(n, 3)) * 0.01
    noise = rng.normal(size=(1, 1, n, 3))
    orc = Oracle.from_instance(sysm, 0)
    orc.set_velos(0, v0)
    orc.set_accels(0, a0)
    orc.md_init()
    orc.run(1, noise)
    eng = Engine(sysm, precision=FP64)
    eng.set_state(0, None, v0, a0)
    eng.step(1, noise.reshape(1, n, 3))
    x = eng.get_state(0)[0]
    assert np.abs(x - orc.get_xyz(0)).max() <= 1e-12 * np.abs(orc.get_xyz(0)).max()


@pytest.mark.parametrize("name", ["chain64", "pbc564"])
def test_fed_noise_ermak_mccammon_matches_oracle(name, sis_ff):
    """Ermak-McCammon Brownian dynamics (job_md.F90:446-456), 10 fed steps, at
    water viscosity: with the MD default (1e-5 Pa s) the explicit BD step
    h/gamma * k_bond exceeds 1 and amplifies every rounding difference.
    Positions compare modulo the box: the engine wraps when it rebuilds after
    a step, the oracle when it rebuilds before the next one."""
    if name == "chain64":  # a coil without WCA overlap (the 4 A contacts of the recipe kick beads far)
        rng = np.random.default_rng(1001)
        x = random_coil(rng, 64, rmin=10.0)
        sysm = System(sis_ff, Options(bp_model=1), [Instance([Chain(rng.integers(0, 4, 64).astype(np.int32))],
                                                             tempK=300.0, ionic_strength=0.15, xyz=x)])
    else:
        sysm = pbc_md_system(sis_ff, 1)
    sysm.opts.integrator = BD_EM
    sysm.opts.viscosity_Pas = 8.9e-4
    n = sysm.nmp
    noise = np.random.default_rng(4).normal(size=(10, 1, n, 3))
    orc = Oracle.from_instance(sysm, 0)
    orc.md_init()
    orc.run(10, noise)
    eng = Engine(sysm, precision=FP64)
    eng.step(10, noise.reshape(10, n, 3))
    d = eng.get_state(0)[0] - orc.get_xyz(0)
    box = sysm.instances[0].box
    if box is not None and box[0] > 0:
        d -= np.asarray(box) * np.round(d / np.asarray(box))
    assert np.abs(d).max() <= 1e-10 * np.abs(orc.get_xyz(0)).max()


@pytest.mark.parametrize("integrator", [GJF2GJ, BD_EM])
def test_md_coefficients_match_oracle(integrator, sis_ff):
    """set_md_coef (job_md.F90:700-767): per-bead coefficients of every instance."""
    sysm = uneven_batch(sis_ff, n_inst=3, lmin=20, lmax=60, seed=9)
    sysm.opts.integrator = integrator
    eng = Engine(sysm, precision=FP64)
    for k in range(3):
        orc = Oracle.from_instance(sysm, k)
        orc.md_init()
        assert np.allclose(eng.get_md_coef(k), orc.get_md_coef(0), rtol=1e-14, atol=0), k


def test_rebuild_trigger_matches_oracle(sis_ff):
    """Large early displacements from a 4 A random-coil contact set force several
    displacement-triggered rebuilds; positions still agree with the oracle."""
    sysm = single_chain(sis_ff, n=64, seed=1001)
    n = sysm.nmp
    rng = np.random.default_rng(1)
    noise = rng.normal(size=(60, 1, n, 3))
    orc = Oracle.from_instance(sysm, 0)
    orc.md_init()
    nreb = orc.run(60, noise)
    eng = Engine(sysm, precision=FP64)
    eng.step(60, noise.reshape(60, n, 3))
    st = eng.stats()
    assert st["rebuilds"] - 1 == nreb  # minus the initial build
    x = eng.get_state(0)[0]
    assert np.abs(x - orc.get_xyz(0)).max() <= 1e-8 * np.abs(x).max()


@pytest.mark.parametrize("name", ["chain64", "cells6000"])
@pytest.mark.parametrize("prec", [MIXED, FP64])
def test_step_graph_equals_single_steps(name, prec, systems, sis_ff):
    """sis_gpu_step runs 20-step graphs whose rebuilds sit behind conditional
    nodes; single-step calls launch every kernel.  Same state, same rebuilds.
    Both starts carry 4 A contacts, so the trigger fires within the run (the
    cell-list box under the force cap that guards such starts)."""
    sysm = systems[name] if name == "chain64" else crowded_box(sis_ff, n_chains=12, n=500, molar=0.05, seed=22, rmin=4.0)
    a = Engine(sysm, precision=prec, seed=5)
    b = Engine(sysm, precision=prec, seed=5)
    for e in (a, b):
        e.set_small(0)  # the general kernels, whose graphs are under test
        e.set_lanes(8)
        e.set_force_cap(1000.0)
        e.init_velocities()
    nsteps = 60 if name == "chain64" else 100
    a.step(nsteps)
    for _ in range(nsteps):
        b.step(1)
    for u, w in zip(a.get_state(-1), b.get_state(-1)):
        if prec == MIXED:
            assert np.array_equal(u, w)
        else:  # FP64 base-pair scatter: atomic arrival order moves the last bits
            assert np.abs(u - w).max() <= 1e-12 * np.abs(w).max()
    sa, sb = a.stats(), b.stats()
    assert sa["rebuilds"] == sb["rebuilds"] and sa["rebuilds"] > 1
    assert a.get_step() == b.get_step() == nsteps


@pytest.mark.parametrize("graphs", [True, False])
def test_overlapped_step_equals_fused_step(graphs, sis_ff):
    """Pair forces in their own kernel on another stream or inside the step
    kernel: the same trajectory bit for bit."""
    sysm = crowded_box(sis_ff, n_chains=12, n=500, molar=0.05, seed=23, rmin=4.0)
    a = Engine(sysm, precision=MIXED, seed=6)
    b = Engine(sysm, precision=MIXED, seed=6)
    a.set_overlap(True)
    b.set_overlap(False)
    for e in (a, b):
        e.set_lanes(8)
        e.set_graphs(graphs)
        e.set_force_cap(1000.0)
        e.init_velocities()
        e.step(80)
    for u, w in zip(a.get_state(-1), b.get_state(-1)):
        assert np.array_equal(u, w)
    assert a.stats()["rebuilds"] == b.stats()["rebuilds"] > 1


@pytest.mark.parametrize("name", ["uneven", "cells"])
def test_autotune_leaves_the_state_as_it_was(name, sis_ff):
    """The autotuner times the real step kernels of every candidate (lanes
    per bead, pair kernel beside the bonded pass or not) and restores what
    they update in place.  A run that tuned first equals, bit for bit, a run
    fixed at the configuration it chose.  The uneven batch has blocks that
    span many instances, whose displacement maxima go straight to the
    per-instance words the tuning also restores."""
    if name == "uneven":
        sysm = uneven_batch(sis_ff, n_inst=24, lmin=8, lmax=120, seed=5)
    else:
        sysm = crowded_box(sis_ff, n_chains=12, n=500, molar=0.05, seed=23, rmin=4.0)
    a = Engine(sysm, precision=MIXED, seed=9)
    a.set_small(0)  # the general kernels, whose tuner is under test
    a.set_force_cap(1000.0)
    a.init_velocities()
    a.step(80)
    st = a.stats()
    b = Engine(sysm, precision=MIXED, seed=9)
    b.set_small(0)
    b.set_lanes(st["lanes_per_bead"])
    b.set_overlap(bool(st["overlap"]))
    b.set_force_cap(1000.0)
    b.init_velocities()
    b.step(80)
    for u, w in zip(a.get_state(-1), b.get_state(-1)):
        assert np.array_equal(u, w)
    assert a.stats()["rebuilds"] == b.stats()["rebuilds"]
    assert a.stats()["capped"] == b.stats()["capped"]


@pytest.mark.parametrize("small", [-1, 0])
def test_instance_alone_equals_instance_in_batch(small, sis_ff):
    """With the per-block kernel of small instances (-1) and the general
    kernels (0)."""
    big = uneven_batch(sis_ff, n_inst=6, lmin=30, lmax=80, seed=5)
    alone = System(big.ff, big.opts, [big.instances[3]])
    e1 = Engine(big, precision=MIXED, seed=99)
    # the noise of an instance is keyed by its stream id (here the batch index)
    e2 = Engine(alone, precision=MIXED, seed=99, streams=[3])
    e1.set_small(small)
    e2.set_small(small)
    e1.step(50)
    e2.step(50)
    x1 = e1.get_state(3)[0]
    x2 = e2.get_state(0)[0]
    assert np.array_equal(x1, x2)


def test_philox_thermostat_free_particles(sis_ff):
    """512 force-free beads: the GJF-2GJ half-step velocity samples the
    Maxwell-Boltzmann distribution, so <Ekin> = 3/2 kB T per bead."""
    kB = 0.0019872042586408316
    insts = [Instance([Chain.from_string("A")], tempK=300.0, ionic_strength=0.15, xyz=np.zeros((1, 3))) for _ in range(512)]
    for prec in (FP64, MIXED):
        eng = Engine(System(sis_ff, Options(bp_model=1), insts), precision=prec, seed=5)
        eng.init_velocities()
        eng.step(500)
        ek = []
        for _ in range(20):
            eng.step(20)
            ek.append(sum(eng.energy_kinetic(k) for k in range(512)) / 512)
        T = np.mean(ek) / (1.5 * kB)
        assert abs(T - 300.0) < 12.0, (prec, T)
        v = eng.get_state(-1)[1]
        assert abs(v.mean()) < 0.01 * v.std()


def test_philox_thermostat_relaxed_chain(sis_ff):
    """A coil without WCA overlaps (no non-bonded pair closer than sigma)."""
    rng = np.random.default_rng(8)
    x = random_coil(rng, 64, rmin=10.0)
    inst = Instance([Chain(rng.integers(0, 4, 64).astype(np.int32))], tempK=300.0, ionic_strength=0.15, xyz=x)
    eng = Engine(System(sis_ff, Options(bp_model=1), [inst]), precision=MIXED, seed=3)
    eng.init_velocities()
    eng.step(4000)
    kB = 0.0019872042586408316
    ek = []
    for _ in range(100):
        eng.step(40)
        ek.append(eng.energy_kinetic(0))
    T = np.mean(ek) / (1.5 * 64 * kB)
    assert abs(T - 300.0) < 30.0, T


def test_nonfinite_coordinates_are_reported(sis_ff):
    sysm = single_chain(sis_ff, n=32, seed=2)
    eng = Engine(sysm, precision=MIXED)
    x = eng.get_state(0)[0]
    x[5, 1] = np.nan
    eng.set_state(0, x)
    with pytest.raises(SisError) as ei:
        eng.step(2)
    assert ei.value.code == -4


def test_pair_list_overflow_is_reported(sis_ff):
    sysm = compact_system(sis_ff)
    eng = Engine(sysm, precision=MIXED, nbr_cap=4)
    with pytest.raises(SisError) as ei:
        eng.neighbor_list(-1)
    assert ei.value.code == -3
