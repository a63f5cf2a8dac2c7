"""Input checks of sis_gpu_create (CPU: they run before any CUDA call).

Every system the GPU tests and the benchmark build passes them (on a machine
without a GPU, creation then fails only at the first CUDA call), and a
sequence code, molecule type, temperature, salt, box or parameter that would
index a device table out of range or divide by zero is refused with
SIS_ERR_ARG."""
import ctypes as C

import numpy as np
import pytest

from sis_gb300 import BD_EM, FP64, MIXED, _abi
from sis_gb300.coil import crowded_box, remd_batch, single_chain, uneven_batch
from sis_gb300.model import Chain, Instance, Options, System
from test_gpu_parity import SYSTEMS


def try_create(sysm, precision=MIXED, mutate=None):
    from sis_gb300.build import build_lib

    build_lib()
    L = _abi.lib()
    topo = _abi.TopologyArrays(sysm)
    par = _abi.pack_params(sysm, precision)
    if mutate is not None:
        mutate(topo, par)
    h = C.c_void_p()
    rc = L.sis_gpu_create(C.byref(topo.struct), C.byref(par), C.byref(h))
    if rc == 0:
        L.sis_gpu_destroy(h)
    return rc


def _filler(capacity=8, n_slots=2):
    chains = [Chain(np.array([4], dtype=np.int32)) for _ in range(capacity)]
    insts = [Instance(list(chains), xyz=np.zeros((capacity, 3)), has_charge=np.zeros(capacity, dtype=bool))
             for _ in range(n_slots)]
    return insts


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_parity_systems_pass(name, sis_ff, nn_ff):
    sysm = SYSTEMS[name](sis_ff, nn_ff)
    for prec in (FP64, MIXED):
        assert try_create(sysm, prec) != _abi.SIS_ERR_ARG


def test_workloads_pass(sis_ff):
    for sysm in (single_chain(sis_ff, n=64), uneven_batch(sis_ff, n_inst=6, lmin=20, lmax=80),
                 remd_batch(sis_ff, n_rep=4, n=40), crowded_box(sis_ff, n_chains=3, n=50, molar=0.01),
                 System(sis_ff, Options(), _filler())):
        assert try_create(sysm) != _abi.SIS_ERR_ARG
    bd = single_chain(sis_ff, n=16)
    bd.opts.integrator = BD_EM
    assert try_create(bd) != _abi.SIS_ERR_ARG
    mc = single_chain(sis_ff, n=16)
    mc.opts.nstep_bp_mc, mc.opts.max_bp_per_nt = 1, 1
    assert try_create(mc) != _abi.SIS_ERR_ARG


def _set(arr_name, index, value):
    def f(topo, par):
        getattr(topo, arr_name)[index] = value
    return f


def _par(**kw):
    def f(topo, par):
        for k, v in kw.items():
            setattr(par, k, v)
    return f


@pytest.mark.parametrize("mutate", [
    _set("seq", 3, 5), _set("seq", 0, -1), _set("types", 0, 0), _set("types", 0, 3), _set("lens", 0, 0),
    _set("temps", 0, 0.0), _set("temps", 0, float("nan")), _set("salts", 0, 0.0), _set("boxes", 0, -1.0),
    _set("boxes", 2, float("inf")),
    _par(dt=0.0), _par(dt=float("nan")), _par(precision=2), _par(integrator=0), _par(viscosity_Pas=-1.0),
    _par(nl_margin=-1.0), _par(bp_model=6), _par(ele_cutoff_type=3), _par(nbr_cap=-1),
    _par(nstep_bp_mc=1, max_bp_per_nt=0),
], ids=["seq5", "seq-1", "moltype0", "moltype3", "len0", "T0", "Tnan", "salt0", "box-1", "boxinf", "dt0", "dtnan",
        "prec2", "integ0", "visc-1", "margin-1", "bp6", "cut3", "cap-1", "mc0"])
def test_bad_inputs_are_refused(mutate, sis_ff):
    sysm = single_chain(sis_ff, n=12)
    assert try_create(sysm, mutate=mutate) == _abi.SIS_ERR_ARG
