"""Statistical parity of long Langevin runs: the device's Philox noise (mixed
and FP64 paths) against the reference's MT19937 + polar Box-Muller noise
(rnd_boxmuller.F90:1-49) run by the oracle, and the mixed path against the
FP64 path.

Every arm runs independent copies of one system from the same start through
the same protocol (velocities from the noise, n_equil steps, then a sample
every `every` steps), so the arms' sample distributions agree exactly when
their dynamics are equivalent in distribution.  Observables: radius of
gyration (energy_rg.F90), kinetic temperature (energy_kinetic.F90), the
count of formed base pairs (E <= -kT, write_bp.F90:36-49) and the count of
base-pair records on (bp_status, E <= cutoff_energy).  A pair of arms
passes when, for every observable, both the Kolmogorov-Smirnov and the
mean z-test p-values, computed with effective sample sizes n / tau_int, are
at least P_MIN.  Seeds are fixed, so every run gives the same p-values.

Systems:
  chain64  the 64-nt chain of the single-chain benchmark (sis.ff, base-pair
           model 1, 300 K, 150 mM, no PBC)
  hairpin  a 30-nt two-hairpin sequence with the nearest-neighbour base-pair
           model 5, the ReB angle, the exp dihedral and the base-pair Monte
           Carlo removal every step (at most one pair per nucleotide)
"""
import numpy as np
import pytest

from statmech import OBS, compare, gpu_runs, oracle_runs, tau_int

P_MIN = 1e-3

# copies and run lengths of each arm (MD steps)
GPU_COPIES, ORACLE_COPIES = 128, 48
N_EQUIL, N_SAMPLE, EVERY = 50000, 200, 500


def _chain64():
    from sis_gb300.coil import single_chain
    from sis_gb300.inputs import read_ff
    from sis_gb300.model import System
    from conftest import ROOT

    ff = read_ff(ROOT / "sis_gb300" / "data" / "sis.ff")
    return single_chain(ff, 64, seed=1001)


def _hairpin():
    from sis_gb300.coil import random_coil
    from sis_gb300.inputs import read_ff
    from sis_gb300.model import Chain, Instance, Options, System
    from conftest import ROOT

    nn = read_ff(ROOT / "sis_gb300" / "data" / "sis_dih_ReB_NN.ff", bp_model=5)
    seq = "GGGGCAAAAGCCCCAAAAGGGGAAAACCCC"
    # a coil without WCA overlaps: both arms start at rest, not from a kick
    x = random_coil(np.random.default_rng(5), len(seq), rmin=10.0)
    inst = Instance([Chain.from_string(seq)], tempK=300.0, ionic_strength=0.15, xyz=x)
    opts = Options(bp_model=5, nstep_bp_mc=1, max_bp_per_nt=1, ele_cutoff_type=2, ele_cutoff=20.0)
    return System(nn, opts, [inst])


SYSTEMS = {"chain64": _chain64, "hairpin": _hairpin}
_cache = {}


def _arm(system_name, arm):
    key = (system_name, arm)
    if key not in _cache:
        sysm = SYSTEMS[system_name]()
        if arm == "oracle":
            _cache[key] = oracle_runs(sysm, ORACLE_COPIES, 7001, N_EQUIL, N_SAMPLE, EVERY)
        else:
            from sis_gb300 import FP64, MIXED

            _cache[key] = gpu_runs(sysm, GPU_COPIES, MIXED if arm == "mixed" else FP64, 9001, N_EQUIL, N_SAMPLE, EVERY)
    return _cache[key]


def _check(a, b, label):
    report = {}
    for obs in OBS:
        x, y = a[obs], b[obs]
        if x.var() == 0.0 and y.var() == 0.0:
            # an observable that never moves (no pair forms): equal constants
            assert x.mean() == y.mean(), (label, obs)
            continue
        r = compare(x, y)
        report[obs] = r
        assert r["p_ks"] >= P_MIN and r["p_mean"] >= P_MIN, (label, obs, r)
    print(label, report)
    return report


# ------------------------------------------------------------- CPU: the tests' machinery
def _ar1(rng, copies, n, phi, mu=0.0):
    x = np.zeros((copies, n))
    x[:, 0] = rng.normal(size=copies) / np.sqrt(1 - phi * phi)
    e = rng.normal(size=(copies, n))
    for t in range(1, n):
        x[:, t] = phi * x[:, t - 1] + e[:, t]
    return x * np.sqrt(1 - phi * phi) + mu


def test_tau_int_of_ar1_series():
    """tau_int of an AR(1) series is (1 + phi) / (1 - phi)."""
    rng = np.random.default_rng(1)
    for phi in (0.0, 0.5, 0.9):
        t = tau_int(_ar1(rng, 64, 2000, phi))
        assert abs(t - (1 + phi) / (1 - phi)) < 0.15 * (1 + phi) / (1 - phi) + 0.1, (phi, t)


def test_effective_sample_tests_are_calibrated():
    """Correlated samples of one distribution pass (the p-values are not
    inflated by the correlation); a shift of 0.3 standard deviations fails."""
    rng = np.random.default_rng(2)
    small = 0
    for _ in range(40):
        r = compare(_ar1(rng, 32, 400, 0.9), _ar1(rng, 48, 400, 0.9))
        small += min(r["p_ks"], r["p_mean"]) < 0.01
    assert small <= 3
    r = compare(_ar1(rng, 32, 400, 0.9), _ar1(rng, 48, 400, 0.9, mu=0.3))
    assert r["p_mean"] < 1e-6


# ------------------------------------------------------------- GPU: the parity itself
@pytest.mark.gpu
@pytest.mark.parametrize("system_name", list(SYSTEMS))
@pytest.mark.parametrize("arm", ["mixed", "fp64"])
def test_philox_runs_match_reference_noise(system_name, arm):
    """Device Philox noise against the oracle's MT19937 + polar Box-Muller."""
    _check(_arm(system_name, arm), _arm(system_name, "oracle"), f"{system_name} {arm} vs oracle")


@pytest.mark.gpu
@pytest.mark.parametrize("system_name", list(SYSTEMS))
def test_mixed_runs_match_fp64_runs(system_name):
    """The mixed path (FP32 terms) against the FP64 path, both on Philox."""
    _check(_arm(system_name, "mixed"), _arm(system_name, "fp64"), f"{system_name} mixed vs fp64")


@pytest.mark.gpu
def test_chain64_forms_base_pairs():
    """The chain's base-pair comparisons have something to compare."""
    a = _arm("chain64", "oracle")
    assert a["nbp"].var() > 0.0 and a["nbp_on"].mean() > 1.0
