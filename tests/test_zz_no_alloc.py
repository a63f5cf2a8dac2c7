"""sis_gpu_step_noise_static (fed noise staged through a static device
buffer, no allocation) against sis_gpu_step (fed noise through the context's
own buffer), both called through the C ABI.

Two contexts of the same system take the same noise; after each of two
calls in a row their states agree.  The mixed path is deterministic (FP32
lanes reduced in a fixed order, base-pair forces as exact fixed-point sums),
so it matches bit for bit; the FP64 path scatters base-pair forces with FP64
atomics, whose arrival order moves the last bits, hence a 1e-12 relative bar.
"""
import ctypes as C

import numpy as np
import pytest

from sis_gb300 import FP64, MIXED, _abi
from sis_gb300.coil import sis_options, uneven_batch
from sis_gb300.engine import Engine
from sis_gb300.model import Chain, Instance, Options, System

pytestmark = pytest.mark.gpu

STATIC_NOISE_BEADS = 65536


def _static_step(eng, noise):
    L = _abi.lib()
    rc = L.sis_gpu_step_noise_static(eng.h, noise.shape[0], noise.ctypes.data_as(C.c_void_p))
    return rc, L.sis_gpu_last_error(eng.h)


@pytest.mark.parametrize("prec", [MIXED, FP64])
def test_static_noise_step_matches_step(prec, sis_ff):
    sysm = uneven_batch(sis_ff, n_inst=4, lmin=40, lmax=120, seed=17)
    n = sysm.nmp
    rng = np.random.default_rng(23)
    ref = Engine(sysm, precision=prec, seed=3)
    got = Engine(sysm, precision=prec, seed=3)
    for call in range(2):
        noise = np.ascontiguousarray(rng.normal(size=(25, n, 3)))
        ref.step(25, noise)
        rc, msg = _static_step(got, noise)
        assert rc == 0, msg
        for a, b in zip(ref.get_state(-1), got.get_state(-1)):
            if prec == MIXED:
                assert np.array_equal(a, b), call
            else:
                assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max(), call
    assert ref.stats()["steps"] == got.stats()["steps"] == 50


@pytest.mark.parametrize("prec", [MIXED, FP64])
def test_static_noise_step_releases_monte_carlo_draws(prec, nn_ff):
    """Uniforms given to sis_gpu_bp_mc serve the next call only: a second
    call whose Monte Carlo passes (every 5 steps) find no caller uniforms
    draws from Philox, in both entry points alike."""
    from sis_gb300.coil import random_coil

    rng = np.random.default_rng(5)
    x = random_coil(rng, 30, amin_deg=60.0, amax_deg=100.0, rmin=3.0)
    inst = Instance([Chain.from_string("GGGGCAAAAGCCCCAAAAGGGGAAAACCCC")], tempK=300.0, ionic_strength=0.15, xyz=x)
    opts = Options(bp_model=5, nstep_bp_mc=5, max_bp_per_nt=1, ele_cutoff_type=2, ele_cutoff=20.0)
    sysm = System(nn_ff, opts, [inst])
    ref = Engine(sysm, precision=prec, seed=3)
    got = Engine(sysm, precision=prec, seed=3)
    draws = np.random.default_rng(11).uniform(size=100000)
    ref.bp_mc(0, draws)
    got.bp_mc(0, draws)
    for call in range(2):
        noise = np.ascontiguousarray(rng.normal(size=(12, sysm.nmp, 3)))
        ref.step(12, noise)
        rc, msg = _static_step(got, noise)
        assert rc == 0, msg
        for a, b in zip(ref.get_state(-1), got.get_state(-1)):
            if prec == MIXED:
                assert np.array_equal(a, b), call
            else:
                assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max(), call
    # and a plain call afterwards runs as it does after sis_gpu_step
    ref.step(20)
    got.step(20)
    for a, b in zip(ref.get_state(-1), got.get_state(-1)):
        if prec == MIXED:
            assert np.array_equal(a, b)
        else:
            assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()


def test_static_noise_step_rejects_too_many_beads(sis_ff):
    line = np.stack([np.arange(500) * 5.84, np.zeros(500), np.zeros(500)], axis=1)
    insts = [Instance([Chain.from_string("A" * 500)], tempK=300.0, ionic_strength=0.15, xyz=line)
             for _ in range(STATIC_NOISE_BEADS // 500 + 1)]
    sysm = System(sis_ff, sis_options(), insts)
    assert sysm.nmp > STATIC_NOISE_BEADS
    eng = Engine(sysm, precision=MIXED)
    noise = np.zeros((1, sysm.nmp, 3))
    rc, msg = _static_step(eng, noise)
    assert rc == -1
    assert b"static noise buffer" in msg
    assert eng.stats()["steps"] == 0
