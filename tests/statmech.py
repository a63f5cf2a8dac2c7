"""Long-run observables and two-sample tests for the statistical parity of
the device noise (Philox4x32-10 + Box-Muller) against the reference's noise
(MT19937 + polar Box-Muller, rnd_boxmuller.F90:1-49, restated in the oracle).

Observables, sampled every `every` MD steps of each independent copy:
  rg   unweighted radius of gyration (energy_rg.F90:17-26)
  T    kinetic temperature 2 Ekin / (3 N kB) (energy_kinetic.F90:15-29)
  nbp  formed base pairs: records on with E <= -kT, the pairs write_bp.F90:36-49
       writes to the .bp file
  nbp_on  base-pair records on (E <= cutoff_energy: bp_status of force_bp.F90),
       the pairs whose forces act in the step

Samples of one copy are correlated.  The integrated autocorrelation time
tau (in samples, Sokal's automatic window, c = 5) is estimated from the
copies' autocovariance; the tests then use n_eff = n / tau samples: the
two-sample Kolmogorov-Smirnov statistic D of all samples, with the
asymptotic p-value of sqrt(n1e n2e / (n1e + n2e)) D, and a z-test of the
means with variances over n_eff.
"""
from __future__ import annotations

import os

import numpy as np

KB = 1.380649e-23 * 6.02214076e23 / 4184.0  # kcal/mol/K (const_phys.F90)
OBS = ("rg", "T", "nbp", "nbp_on")


def tau_int(series: np.ndarray, c: float = 5.0) -> float:
    """Integrated autocorrelation time (in samples) of series[copy, sample]."""
    x = np.asarray(series, dtype=np.float64)
    x = x - x.mean()
    n = x.shape[1]
    var = np.mean(x * x)
    if var <= 0.0:
        return 1.0
    f = np.fft.rfft(x, 2 * n, axis=1)
    acov = np.fft.irfft(f * np.conj(f), axis=1)[:, :n].sum(axis=0)
    acov /= (x.shape[0] * (n - np.arange(n)))
    rho = acov / acov[0]
    tau = 1.0
    for w in range(1, n):
        tau += 2.0 * rho[w]
        if w >= c * tau:
            break
    return max(1.0, float(tau))


def compare(a: np.ndarray, b: np.ndarray) -> dict:
    """Two arms' samples [copy, sample] of one observable: KS and mean z-test
    p-values with effective sample sizes."""
    from scipy.stats import kstwobign, ks_2samp, norm

    ta, tb = tau_int(a), tau_int(b)
    na, nb = a.size / ta, b.size / tb
    D = float(ks_2samp(a.ravel(), b.ravel()).statistic)
    p_ks = float(kstwobign.sf(D * np.sqrt(na * nb / (na + nb))))
    va, vb = a.var(), b.var()
    se = np.sqrt(va / na + vb / nb)
    if se == 0.0:
        p_mean = 1.0 if a.mean() == b.mean() else 0.0
    else:
        p_mean = float(2.0 * norm.sf(abs(a.mean() - b.mean()) / se))
    return {"mean": (float(a.mean()), float(b.mean())), "sd": (float(a.std()), float(b.std())), "tau": (ta, tb),
            "n_eff": (na, nb), "D": D, "p_ks": p_ks, "p_mean": p_mean}


def formed_pairs(ene: np.ndarray, status: np.ndarray, tempK: float) -> int:
    return int(np.count_nonzero((status != 0) & (ene <= -KB * tempK)))


def _worker_init():
    # one OpenMP thread per worker process: the copies run side by side
    os.environ["OMP_NUM_THREADS"] = "1"


def oracle_copy(args) -> dict:
    """One oracle copy of instance 0 of `system` with its own MT stream, from
    the system's start: md_init, velocities from the noise, n_equil steps,
    then n_sample samples every `every` steps."""
    system, seed, n_equil, n_sample, every = args
    from oracle.oracle import Oracle

    T = system.instances[0].tempK
    o = Oracle.from_instance(system, 0)
    o.seed_streams(seed)  # the reference's noise stream of a run with rng_seed = seed
    o.md_init()
    o.init_velocities()
    o.run(n_equil)
    out = {k: np.zeros(n_sample) for k in OBS}
    for s in range(n_sample):
        o.run(every)
        out["rg"][s] = o.rg(0)
        out["T"][s] = 2.0 * o.energy_kinetic(0) / (3.0 * o.nmp * KB)
        e, st = o.bp_state(0)
        out["nbp"][s] = formed_pairs(e, st, T)
        out["nbp_on"][s] = np.count_nonzero(st)
    return out


def oracle_runs(system, copies: int, seed0: int, n_equil: int, n_sample: int, every: int) -> dict:
    """`copies` oracle copies in a pool of spawned processes (spawn: the
    parent may already hold a CUDA context, which a forked child must not
    inherit)."""
    import multiprocessing as mp

    procs = max(1, min(copies, os.cpu_count() or 1))
    with mp.get_context("spawn").Pool(procs, initializer=_worker_init) as pool:
        res = pool.map(oracle_copy, [(system, seed0 + k, n_equil, n_sample, every) for k in range(copies)])
    return {k: np.stack([r[k] for r in res]) for k in OBS}


def gpu_runs(system, copies: int, precision: int, seed: int, n_equil: int, n_sample: int, every: int) -> dict:
    """`copies` copies of instance 0 of `system` as instances of one context,
    each with its own Philox stream, from the same start as the oracle's."""
    from sis_gb300.engine import Engine
    from sis_gb300.model import System

    inst = system.instances[0]
    T = inst.tempK
    batch = System(system.ff, system.opts, [inst] * copies)
    eng = Engine(batch, precision=precision, seed=seed)
    eng.init_velocities()
    eng.step(n_equil)
    out = {k: np.zeros((copies, n_sample)) for k in OBS}
    n = inst.nmp
    for s in range(n_sample):
        eng.step(every)
        out["rg"][:, s] = eng.rg(-1)
        for k in range(copies):
            out["T"][k, s] = 2.0 * eng.energy_kinetic(k) / (3.0 * n * KB)
            st = eng.get_bp_status(k)
            out["nbp"][k, s] = formed_pairs(eng.get_bp_energies(k), st, T)
            out["nbp_on"][k, s] = np.count_nonzero(st)
    eng.close()
    return out
