"""Failure detection of the device waits, without a GPU fault.

The trigger/rebuild kernel (k_trigger_rebuild) separates its phases with a
grid barrier whose wait is bounded.  sis_gpu_probe_barrier_timeout runs that
barrier with one block of the cooperative launch absent: nothing ever
completes it, the other blocks' waits run out after about a second, the
kernel reports the timeout through the error word, and the host answers
SIS_ERR_TIMEOUT and resets the barrier.  The context then steps on, its
rebuilds (which use the same barrier) included.
"""
import numpy as np
import pytest

from sis_gb300 import MIXED
from sis_gb300._abi import SIS_ERR_TIMEOUT
from sis_gb300.coil import crowded_box
from sis_gb300.engine import Engine

pytestmark = pytest.mark.gpu


def test_barrier_wait_runs_out_and_the_context_recovers(sis_ff):
    sysm = crowded_box(sis_ff, n_chains=12, n=500, molar=0.05, seed=23, rmin=4.0)
    eng = Engine(sysm, precision=MIXED, seed=2)
    eng.set_force_cap(1000.0)
    eng.init_velocities()
    eng.step(40)
    before = eng.stats()["rebuilds"]
    assert eng.L.sis_gpu_probe_barrier_timeout(eng.h) == SIS_ERR_TIMEOUT
    assert "timed out" in eng.L.sis_gpu_last_error(eng.h).decode()
    eng.step(200)
    x = eng.get_state(-1)[0]
    assert np.all(np.isfinite(x))
    assert eng.stats()["rebuilds"] > before
    assert eng.stats()["error_flags"] == 0
