"""The force check (sis_gb300.job_check_force, job_check_force.F90).

CPU, with a stand-in engine over an analytic potential: the central
differences, the batching of displaced copies, the report lines and the
beads flagged when force and energy disagree by more than ``small``.
GPU: forces and energy differences of a chain against the oracle's.
"""
import io

import numpy as np
import pytest

from sis_gb300 import job_check_force as jcf
from sis_gb300.model import Chain, Instance, Options, System
from sis_gb300.outputs import fortran_f, fortran_g


class AnalyticEngine:
    """E = sum_i a (x_i . w)^3 + b |x_i|^2; one bead's force can be made
    wrong on purpose (the stand-in, not the product, carries the mistake)."""
    a, b = 0.01, 0.5
    w = np.array([0.3, -0.2, 0.5])
    wrong_bead = None
    made = []

    def __init__(self, system, precision=0):
        self.x = [np.asarray(i.xyz, dtype=np.float64) for i in system.instances]
        self.n_inst = len(self.x)
        AnalyticEngine.made.append(self.n_inst)

    def neighbor_list(self, inst=-1):
        pass

    def energy(self, x):
        return float(np.sum(self.a * (x @ self.w) ** 3 + self.b * np.sum(x * x, axis=1)))

    def force(self, inst):
        x = self.x[inst]
        f = -(3 * self.a * (x @ self.w)[:, None] ** 2 * self.w[None, :] + 2 * self.b * x)
        if self.wrong_bead is not None:
            f[self.wrong_bead] += [0.0, 0.01, 0.0]
        return f

    def energy_sumup(self, k):
        e = np.zeros(11)
        e[0] = self.energy(self.x[k])
        return e

    def close(self):
        pass


def _system(n=7):
    rng = np.random.default_rng(3)
    inst = Instance([Chain.from_string("ACGUACGUACGU"[:n])], xyz=rng.normal(size=(n, 3)) * 5.0)
    return System(None, Options(), [inst])


def test_central_differences_and_report(monkeypatch):
    monkeypatch.setattr(jcf, "Engine", AnalyticEngine)
    AnalyticEngine.made = []
    sysm = _system()
    jit = np.full((7, 3), 0.5)
    out = io.StringIO()
    logged = []
    fe, ff = jcf.check_force(sysm, jitter=jit, out=out, log=logged.append)
    # one context for the forces, one for the 42 displaced copies
    assert AnalyticEngine.made == [1, 42]
    x = sysm.instances[0].xyz + 0.0005
    eng = AnalyticEngine(System(None, Options(), [Instance(sysm.instances[0].chains, xyz=x)]))
    assert np.allclose(ff, eng.force(0), rtol=1e-15, atol=0)
    # the central difference of a cubic is exact up to a^small^2 terms
    assert np.abs(fe - ff).max() < 1e-6
    assert logged == []
    lines = out.getvalue().splitlines()
    assert len(lines) == 14
    assert lines[0] == ("imp=     1  f_energy" + "".join(" " + fortran_g(v, 11, 4) for v in fe[0])
                        + "  f_force=" + "".join(" " + fortran_g(v, 11, 4) for v in ff[0]))
    assert lines[1] == "f_energy - f_force     1" + "".join(fortran_f(v, 11, 4) for v in fe[0] - ff[0])


def test_batches_give_the_same_differences(monkeypatch):
    monkeypatch.setattr(jcf, "Engine", AnalyticEngine)
    AnalyticEngine.made = []
    sysm = _system()
    a = jcf.check_force(sysm, seed=5, log=lambda s: None)
    b = jcf.check_force(sysm, seed=5, log=lambda s: None, max_beads=7 * 5)
    assert AnalyticEngine.made[:2] == [1, 42] and AnalyticEngine.made[3:] == [5] * 8 + [2]
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_a_wrong_force_is_flagged(monkeypatch):
    monkeypatch.setattr(jcf, "Engine", AnalyticEngine)
    monkeypatch.setattr(AnalyticEngine, "wrong_bead", 3)
    logged = []
    fe, ff = jcf.check_force(_system(), seed=1, log=logged.append)
    assert len(logged) == 1 and logged[0].startswith("f_energy - f_force      4")
    assert float(logged[0].split()[-2]) == pytest.approx(-0.01, abs=1e-4)


@pytest.mark.gpu
def test_check_force_matches_the_oracle(sis_ff):
    """Forces to 1e-12 of the oracle's; the central differences to 1e-6
    of the oracle's energies at the same displaced coordinates."""
    from oracle.oracle import Oracle
    from sis_gb300.coil import single_chain

    sysm = single_chain(sis_ff, n=12, seed=9)
    jit = np.random.default_rng(2).random((12, 3))
    fe, ff = jcf.check_force(sysm, jitter=jit, log=lambda s: None)
    x = sysm.instances[0].xyz + 0.001 * jit
    orc = Oracle.from_instance(sysm, 0)
    orc.set_xyz(0, x)
    orc.neighbor_list(0)
    ref = orc.force(0)
    assert np.abs(ff - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
    fd = np.empty((12, 3))
    for i in range(12):
        for a in range(3):
            e = []
            for s in (0.001, -0.001):
                y = x.copy()
                y[i, a] += s
                orc.set_xyz(0, y)
                orc.neighbor_list(0)
                orc.set_bp_energy_flag(0)
                e.append(orc.energy_sumup(0)[0])
            fd[i, a] = -(e[0] - e[1]) / 0.002
    assert np.abs(fe - fd).max() < 1e-6
