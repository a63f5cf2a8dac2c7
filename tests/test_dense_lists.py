"""The mixed path's force error on dense states, whose pair lists are several
times longer than the crowded benchmark box's (about 100 entries per bead).

The mixed path evaluates every pair term in FP32 and sums a bead's pair
forces in FP32 partial sums (at most a few dozen terms each: one lane's share
of its cluster-pair list, or of its per-bead list), which are then added in
FP32 and converted to FP64 once per bead.  A fully FP64 accumulation (one
FP64 addition per pair) would cost more FP64 instructions than the whole
update on this part.  These tests bound what the shorter FP32 accumulation
costs where it matters most: many pairs per bead, with large cancelling
contributions.  The bar is the mixed path's 1e-5 force RMS error against
the FP64 path (itself checked against the oracle to 1e-12).
"""
import numpy as np
import pytest

from helpers import rms_rel
from sis_gb300 import FP64, MIXED
from sis_gb300.coil import crowded_box
from sis_gb300.engine import Engine
from sis_gb300.model import Chain, Instance, System

pytestmark = pytest.mark.gpu

FORCE_RMS_TOL_MIXED = 1e-5


def _full_entries(eng):
    n = eng.nmp(-1)
    return 2 * sum(len(eng.get_list(k, kind)) for k in range(eng.n_inst) for kind in (0, 1)) / n


def _compare(sysm, min_entries):
    e64 = Engine(sysm, precision=FP64)
    e32 = Engine(sysm, precision=MIXED)
    f64 = np.concatenate([e64.force(k) for k in range(e64.n_inst)])
    f32 = np.concatenate([e32.force(k) for k in range(e32.n_inst)])
    entries = _full_entries(e64)
    assert entries >= min_entries, entries
    err = rms_rel(f32, f64)
    assert err <= FORCE_RMS_TOL_MIXED, (entries, err)
    return entries, err


def test_crowded_box_ten_times_denser(sis_ff):
    """The crowded benchmark box at 100 mM nucleotide (ten times
    denser): about twice the list entries per bead."""
    sysm = crowded_box(sis_ff, n_chains=12, n=500, molar=0.1, seed=31)
    _compare(sysm, 90)


def test_dense_charged_lattice(sis_ff):
    """2744 charged beads on a jittered 13 A lattice in a periodic box: about
    400 list entries per bead whose Debye-Hueckel forces nearly cancel, the
    hardest case for a short FP32 accumulation."""
    k = 14
    rng = np.random.default_rng(3)
    g = np.stack(np.meshgrid(*[np.arange(k)] * 3, indexing="ij"), axis=-1).reshape(-1, 3) * 13.0
    x = g + rng.uniform(-1.5, 1.5, size=g.shape)
    seq = rng.integers(0, 4, len(x)).astype(np.int32)
    chains = [Chain(seq[i:i + 1]) for i in range(len(x))]
    L = 13.0 * k
    opts = crowded_box(sis_ff, 1, 20, 0.01, seed=1).opts
    sysm = System(sis_ff, opts, [Instance(chains, tempK=300.0, ionic_strength=0.15, box=(L, L, L), xyz=x)])
    _compare(sysm, 350)
