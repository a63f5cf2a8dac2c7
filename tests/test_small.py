"""The per-block MD kernel of small instances (kernels.cu k_md_small), mixed
path, through the C ABI.

It runs every phase of job_md's step (job_md.F90:360-460) for buckets of
whole instances, one block each.  Checked here:
* it is the path sis_gpu_step takes for small instances (stats);
* its in-kernel list rebuilds give the oracle's lists bit for bit;
* fed the oracle's noise, 10 steps agree with the oracle as closely as the
  general kernels' mixed path does (FP32 terms: positions to 1e-6 of their
  scale, velocities to 1e-4 of theirs);
* it follows the general kernels' trajectory to FP32 rounding;
* the trajectory does not depend on how the steps are split into calls or
  launches, nor on the buckets (the first long call times several bucket
  counts and block widths on real steps);
* it keeps the displacement trigger: lists rebuilt as often as the general
  kernels rebuild them.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from sis_gb300 import MIXED
from sis_gb300.coil import random_coil, random_sequence, single_chain, sis_options, uneven_batch
from sis_gb300.engine import Engine
from sis_gb300.model import Chain, Instance, System

pytestmark = pytest.mark.gpu


def _batch(ff, n_inst=12, seed=5, lmin=20, lmax=200, clean=False):
    if not clean:
        return uneven_batch(ff, n_inst=n_inst, lmin=lmin, lmax=lmax, seed=seed)
    # coils without WCA overlaps (no pair closer than 10 A), so that short
    # trajectories of two paths whose FP32 sums differ stay comparable
    rng = np.random.default_rng(seed)
    insts = []
    for _ in range(n_inst):
        n = int(rng.integers(lmin, lmax + 1))
        insts.append(Instance([Chain(random_sequence(rng, n))], tempK=float(rng.uniform(280.0, 340.0)),
                              ionic_strength=float(rng.uniform(0.02, 0.5)), xyz=random_coil(rng, n, rmin=10.0)))
    return System(ff, sis_options(), insts)


# chain lengths of the batches: short chains walk their lists; chains of 256
# moving beads and more walk inner lists (kernels.cu kInnerMinBeads)
LENGTHS = [pytest.param((20, 200), id="short"), pytest.param((256, 400), id="inner")]


def as_set(a):
    return set(map(tuple, np.asarray(a).tolist()))


def test_small_kernel_is_the_step_path(sis_ff):
    eng = Engine(_batch(sis_ff), precision=MIXED, seed=3)
    eng.init_velocities()
    eng.step(10)
    st = eng.stats()
    assert st["small_blocks"] > 0 and st["small_threads"] > 0
    eng.set_small(0)
    assert eng.stats()["small_blocks"] == 0


def test_small_rebuilds_give_the_oracle_lists(sis_ff):
    """With no list margin the trigger fires after every step, so the lists
    the kernel rebuilt last belong to the final positions: they equal the
    oracle's lists built from the same positions, bit for bit."""
    sysm = single_chain(sis_ff, n=64, seed=1001)
    sysm.opts.nl_margin = 0.0
    eng = Engine(sysm, precision=MIXED, seed=4)
    eng.set_force_cap(1000.0)
    eng.init_velocities()
    eng.step(30)
    assert eng.stats()["rebuilds"] >= 30
    assert eng.stats()["small_blocks"] > 0
    x, _, _ = eng.get_state(0)
    orc = Oracle.from_instance(sysm, 0)
    orc.set_xyz(0, x)
    orc.neighbor_list(0)
    for kind in (0, 1, 2):
        assert as_set(eng.get_list(0, kind)) == as_set(orc.get_list(0, kind)), kind


@pytest.mark.parametrize("small", [-1, 0])
def test_fed_noise_mixed_trajectory_matches_oracle(small, sis_ff):
    sysm = single_chain(sis_ff, n=64, seed=1001)
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
    eng = Engine(sysm, precision=MIXED)
    eng.set_small(small)
    eng.set_state(0, None, v0, a0)
    eng.step(10, noise.reshape(10, n, 3))
    x, v, _ = eng.get_state(0)
    assert np.abs(x - orc.get_xyz(0)).max() <= 1e-6 * np.abs(orc.get_xyz(0)).max()
    assert np.abs(v - orc.get_velos(0)).max() <= 1e-4 * np.abs(orc.get_velos(0)).max()


@pytest.mark.parametrize("lengths", LENGTHS)
def test_small_follows_the_general_kernels(lengths, sis_ff):
    """Same state, same Philox noise: the two paths differ in the order of
    FP32 sums only, so over 20 steps they stay within FP32 rounding."""
    long = lengths[1] > 200
    sysm = _batch(sis_ff, n_inst=6 if long else 12, lmin=lengths[0], lmax=lengths[1], clean=long)
    a = Engine(sysm, precision=MIXED, seed=8)
    b = Engine(sysm, precision=MIXED, seed=8)
    b.set_small(0)
    for e in (a, b):
        e.init_velocities()
        e.step(20)
    xa, xb = a.get_state(-1)[0], b.get_state(-1)[0]
    assert np.abs(xa - xb).max() <= 1e-4
    assert a.stats()["small_blocks"] > 0 and b.stats()["small_blocks"] == 0


@pytest.mark.parametrize("lengths", LENGTHS)
def test_small_trajectory_independent_of_calls_and_buckets(lengths, sis_ff):
    """One 400-step call (whose first steps time several bucket plans and
    block widths), 40 calls of 10 steps (the default plan) and 400 calls of
    one step give the same state bit for bit, with the same rebuilds (and,
    for long chains, the same inner-list filterings)."""
    sysm = _batch(sis_ff, n_inst=40 if lengths[1] <= 200 else 12, seed=7, lmin=lengths[0], lmax=lengths[1])
    runs = []
    for calls, per in ((1, 400), (40, 10), (400, 1)):
        e = Engine(sysm, precision=MIXED, seed=11)
        e.set_force_cap(1000.0)
        e.init_velocities()
        for _ in range(calls):
            e.step(per)
        runs.append((e.get_state(-1), e.stats(), e.get_step()))
    (s0, st0, k0) = runs[0]
    for s, st, k in runs[1:]:
        for u, w in zip(s0, s):
            assert np.array_equal(u, w)
        assert st["rebuilds"] == st0["rebuilds"] and k == k0 == 400
    assert st0["rebuilds"] > len(sysm.instances)


def test_small_rebuild_rate_matches_general_kernels(sis_ff):
    """The trigger of the per-block kernel fires as often as the general
    kernels' on the same system (within a few rebuilds over 600 steps)."""
    sysm = _batch(sis_ff, n_inst=16, seed=9)
    out = []
    for small in (-1, 0):
        e = Engine(sysm, precision=MIXED, seed=12)
        e.set_small(small)
        e.set_force_cap(1000.0)
        e.init_velocities()
        e.step(600)
        out.append(e.stats()["rebuilds"])
    assert abs(out[0] - out[1]) <= max(3, 0.1 * out[1]), out


def test_inner_lists_hold_every_pair_within_its_cutoff(sis_ff):
    """After 400 steps of chains of 256-400 beads from coils with WCA
    overlaps (fast motion: many inner filterings and list rebuilds), every
    listed pair within its cutoff at the current positions is in the inner
    lists, the inner lists are part of the lists, and they leave out the
    pairs well beyond the cutoffs."""
    sysm = _batch(sis_ff, n_inst=6, seed=13, lmin=256, lmax=400)
    eng = Engine(sysm, precision=MIXED, seed=17)
    eng.set_force_cap(1000.0)
    eng.init_velocities()
    eng.step(400)
    assert eng.stats()["small_blocks"] > 0
    x = eng.get_state(-1)[0]
    off, left_out, total = 0, 0, 0
    for k, inst in enumerate(sysm.instances):
        n = inst.nmp
        xk = x[off:off + n]
        cut = {0: 10.0, 1: eng.get_ele(k)[2]}  # WCA sigma (sis.ff), electrostatic cutoff
        for kind, kind_in in ((0, 3), (1, 4)):
            outer = as_set(eng.get_list(k, kind))
            inner = as_set(eng.get_list(k, kind_in))
            assert inner <= outer, (k, kind)
            for i, j in outer:
                d = np.linalg.norm(xk[i - 1] - xk[j - 1])
                if d <= cut[kind]:
                    assert (i, j) in inner, (k, kind, i, j, d)
            left_out += len(outer) - len(inner)
            total += len(outer)
        off += n
    assert left_out > 0.05 * total, (left_out, total)
