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


# ------------------------------------------------ other replica variables
def _same_temperature(sysm, T=300.0):
    insts = [dataclasses.replace(i, tempK=T) for i in sysm.instances]
    return System(sysm.ff, sysm.opts, insts)


def _oracle_with(sysm, k, x, T, ion=None, rg=None, twz=None):
    """An oracle of replica k at the given variables: ionic strength, Rg bias
    (k_rg, rg0) and a constant-force trap pair (i, j, force vector)."""
    from sis_gb300.model import ConstantForcePair

    inst = dataclasses.replace(sysm.instances[k], tempK=T, xyz=x)
    if ion is not None:
        inst = dataclasses.replace(inst, ionic_strength=ion)
    o = Oracle.from_instance(System(sysm.ff, sysm.opts, [inst]), 0)
    if rg is not None:
        o.set_rg_bias(rg[0], rg[1])
    if twz is not None:
        o.set_tweezers(dcf=[ConstantForcePair(twz[0], twz[1], list(twz[2]))])
    o.neighbor_list(0)
    o.set_bp_energy_flag(0)
    return o


@pytest.mark.parametrize("var", ["ion", "rg", "twz"])
@pytest.mark.parametrize("parity", [0, 1])
def test_replica_variable_exchange_matches_restatement(var, parity, ladder):
    """Ionic strength (REPT%ION), Rg target (REPT%RG) and trap force
    (REPT%TWZDCF) as the replica variable at one temperature: partner
    energies at the partner label's value (energy_replica.F90:95-107),
    delta with T_m = T_n, no velocity scaling (replica_exchange.F90:132-147)."""
    from sis_gb300.model import ConstantForcePair

    base, _ = ladder
    sysm = _same_temperature(base)
    T = 300.0
    vals = {"ion": [0.02, 0.05, 0.1, 0.2, 0.35, 0.5], "rg": [14.0, 15.0, 16.0, 17.0, 18.0, 19.0],
            "twz": [0.0, 0.1, 0.2, 0.3, 0.4, 0.5]}[var]
    kind = {"ion": 2, "rg": 4, "twz": 3}[var]
    direction = np.array([0.6, 0.0, 0.8])
    eng = Engine(sysm, precision=FP64, seed=7)
    if var == "rg":
        eng.set_rg_bias(-1, 2.0, 15.0)
    if var == "twz":
        for k in range(N_REP):
            eng.set_tweezers(k, dcf=[ConstantForcePair(1, 40, list(direction))])
    eng.remd_init_vars([kind], np.array(vals).reshape(N_REP, 1))
    eng.init_velocities()
    eng.step(300)
    state = [eng.get_state(k) for k in range(N_REP)]

    def energy(k, l):
        x = state[k][0]
        if var == "ion":
            return _oracle_with(sysm, k, x, T, ion=vals[l]).energy_sumup(0)[0]
        if var == "rg":
            return _oracle_with(sysm, k, x, T, rg=(2.0, vals[l])).energy_sumup(0)[0]
        return _oracle_with(sysm, k, x, T, twz=(1, 40, vals[l] * direction)).energy_sumup(0)[0]

    own = [energy(k, k) for k in range(N_REP)]
    par = [energy(k, partner(k, parity, N_REP)) if partner(k, parity, N_REP) >= 0 else 0.0 for k in range(N_REP)]
    u = np.array([1e-300 if q % 2 == 0 else 1.0 for q in range(N_REP // 2 + 1)])
    labels = list(range(N_REP))
    for q in range(N_REP):
        li, lj = 2 * q + parity, 2 * q + parity + 1
        if lj >= N_REP:
            break
        delta = ((par[lj] - own[li]) / T - (own[lj] - par[li]) / T) / KB
        if delta < 0.0 or u[q] <= np.exp(-delta):
            labels[li], labels[lj] = lj, li
    r2l, nacc = eng.remd_exchange(parity, u)
    assert list(r2l) == labels and nacc >= 1
    for k in range(N_REP):
        x, v, a = eng.get_state(k)
        assert np.array_equal(v, state[k][1])  # no temperature variable: no scaling
        l = labels[k]
        o = (_oracle_with(sysm, k, x, T, ion=vals[l]) if var == "ion" else
             _oracle_with(sysm, k, x, T, rg=(2.0, vals[l])) if var == "rg" else
             _oracle_with(sysm, k, x, T, twz=(1, 40, vals[l] * direction)))
        e = o.energy_sumup(0)[0]
        assert abs(eng.energy_sumup(k)[0] - e) <= 1e-12 * max(1.0, abs(e)), (k, l)
