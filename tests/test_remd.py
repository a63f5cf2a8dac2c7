"""Temperature replica exchange on the device (sis_gpu_remd_init /
sis_gpu_remd_exchange) against a restatement of replica_exchange.F90 and
energy_replica.F90 fed with FP64 oracle energies:

* own- and partner-temperature total energies from the oracle (an oracle
  built at the partner's temperature is set_ele at that temperature);
* delta = ((E_j(T_m) - E_i(T_m)) / T_m - (E_j(T_n) - E_i(T_n)) / T_n) / k_B,
  accepted if delta < 0 or u <= exp(-delta), with the caller's uniforms;
* accepted pairs swap labels, their velocities are scaled by sqrt(T_n/T_m)
  (times for the colder replica, divided for the hotter one), and every
  temperature-dependent coefficient follows the new temperature.
"""
import dataclasses

import numpy as np
import pytest

from oracle.oracle import Oracle
from sis_gb300 import FP64
from sis_gb300.coil import remd_batch
from sis_gb300.engine import Engine
from sis_gb300.model import System

pytestmark = pytest.mark.gpu

# const_phys.F90: BOLTZ_KCAL_MOL = BOLTZ_J * JOUL2KCAL_MOL
KB = 1.380649e-23 * ((1.0 / 4184.0) * 6.02214076e23)
N_REP = 6


def oracle_at(sysm, k, x, T):
    inst = dataclasses.replace(sysm.instances[k], tempK=T, xyz=x)
    o = Oracle.from_instance(System(sysm.ff, sysm.opts, [inst]), 0)
    o.neighbor_list(0)
    return o


def total_energy(sysm, k, x, T):
    o = oracle_at(sysm, k, x, T)
    o.set_bp_energy_flag(0)
    return o.energy_sumup(0)[0]


def partner(l, parity, n):
    if l - parity < 0:
        return -1
    p = l + 1 if (l - parity) % 2 == 0 else l - 1
    return p if p < n else -1


@pytest.fixture(scope="module")
def ladder(sis_ff):
    sysm = remd_batch(sis_ff, n_rep=N_REP, n=40, seed=31)
    return sysm, [inst.tempK for inst in sysm.instances]


def stepped_engine(sysm, temps, steps=300):
    eng = Engine(sysm, precision=FP64, seed=7)
    eng.remd_init(temps)
    eng.init_velocities()
    eng.step(steps)
    return eng


@pytest.mark.parametrize("parity", [0, 1])
def test_exchange_matches_restatement(parity, ladder):
    sysm, temps = ladder
    eng = stepped_engine(sysm, temps)
    state = [eng.get_state(k) for k in range(N_REP)]
    own = [total_energy(sysm, k, state[k][0], temps[k]) for k in range(N_REP)]
    par = [total_energy(sysm, k, state[k][0], temps[partner(k, parity, N_REP)]) if partner(k, parity, N_REP) >= 0 else 0.0
           for k in range(N_REP)]
    # the labels start as the instance indices; u forces "accept unless delta
    # is huge" on even pairs and "accept only if delta <= 0" on odd ones
    u = np.array([1e-300 if q % 2 == 0 else 1.0 for q in range(N_REP // 2 + 1)])
    labels = list(range(N_REP))
    scale = {}
    for q in range(N_REP):
        li, lj = 2 * q + parity, 2 * q + parity + 1
        if lj >= N_REP:
            break
        tm, tn = temps[li], temps[lj]
        delta = ((par[lj] - own[li]) / tm - (own[lj] - par[li]) / tn) / KB
        if delta < 0.0 or u[q] <= np.exp(-delta):
            labels[li], labels[lj] = lj, li
            sf = np.sqrt(tn / tm)
            scale[li] = ("mul", sf)
            scale[lj] = ("div", sf)
    r2l, nacc = eng.remd_exchange(parity, u)
    assert list(r2l) == labels
    assert nacc == len(scale) // 2
    assert nacc >= 1
    for k in range(N_REP):
        x, v, a = eng.get_state(k)
        assert np.array_equal(x, state[k][0]) and np.array_equal(a, state[k][2])
        if k in scale:
            how, sf = scale[k]
            assert np.array_equal(v, state[k][1] * sf if how == "mul" else state[k][1] / sf), k
        else:
            assert np.array_equal(v, state[k][1])
        # every temperature-dependent coefficient follows the new label
        T = temps[labels[k]]
        o = oracle_at(sysm, k, x, T)
        assert np.allclose(eng.get_ele(k), o.get_ele(0), rtol=1e-15, atol=0)
        o.md_init()
        assert np.allclose(eng.get_md_coef(k), o.get_md_coef(0), rtol=1e-14, atol=0), k
        o.set_bp_energy_flag(0)
        assert abs(eng.energy_sumup(k)[0] - o.energy_sumup(0)[0]) <= 1e-12 * max(1.0, abs(o.energy_sumup(0)[0]))


def test_swapped_replica_steps_like_a_fresh_instance(ladder):
    """After a swap, a replica's next fed-noise steps equal those of an
    instance created at its new temperature from the same state."""
    sysm, temps = ladder
    eng = stepped_engine(sysm, temps, steps=200)
    r2l, nacc = eng.remd_exchange(0, np.full(N_REP // 2 + 1, 1e-300))
    assert nacc >= 1
    k = int(np.flatnonzero(r2l != np.arange(N_REP))[0])
    x, v, a = eng.get_state(k)
    fresh = Engine(System(sysm.ff, sysm.opts, [dataclasses.replace(sysm.instances[k], tempK=temps[r2l[k]], xyz=x)]),
                   precision=FP64)
    fresh.set_state(0, x, v, a)
    noise = np.random.default_rng(3).normal(size=(5, sysm.nmp, 3))
    eng.step(5, noise)
    off = sysm.offsets()
    fresh.step(5, np.ascontiguousarray(noise[:, off[k]:off[k + 1]]))
    got, want = eng.get_state(k)[0], fresh.get_state(0)[0]
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


def test_device_uniforms_give_a_permutation(ladder):
    sysm, temps = ladder
    eng = stepped_engine(sysm, temps, steps=100)
    for parity in (0, 1, 0, 1):
        r2l, nacc = eng.remd_exchange(parity)
        assert sorted(r2l) == list(range(N_REP))
        assert 0 <= nacc <= N_REP // 2
        eng.step(50)
