"""ctypes binding of libsisgpu.so (include/sis_gpu.h).

The library is built in-tree by ``__graft_entry__.build()`` into
``sis_gb300/_lib/libsisgpu.so``.  There is no fallback: if the library is
missing or fails to load, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .model import System

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libsisgpu.so"

SIS_OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "list overflow", -4: "non-finite values", -5: "out of device memory",
          -6: "call out of order", -7: "device wait timed out"}
SIS_ERR_ARG = -1
SIS_ERR_TIMEOUT = -7


class SisError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class sis_params(C.Structure):
    _fields_ = [
        ("bond_k", C.c_double), ("bond_r0", C.c_double),
        ("angl_reb", C.c_int32), ("angl_k", C.c_double), ("angl_t0", C.c_double),
        ("dih_type", C.c_int32), ("dih_k", C.c_double), ("dih_w", C.c_double), ("dih_p0", C.c_double),
        ("wca_sigma", C.c_double), ("wca_eps", C.c_double),
        ("bp_model", C.c_int32), ("bp_min_loop", C.c_int32), ("bp_jnext_compat", C.c_int32),
        ("bp_cutoff_energy", C.c_double),
        ("bp_ff", (C.c_double * 15) * 3),
        ("nn_dH", C.c_double * 21), ("nn_dS", C.c_double * 21), ("dH0", C.c_double), ("dS0", C.c_double),
        ("nnend", C.c_int32), ("nnend_dH", C.c_double * 6), ("nnend_dS", C.c_double * 6),
        ("dHend0", C.c_double), ("dSend0", C.c_double),
        ("flg_ele", C.c_int32), ("ele_cutoff_type", C.c_int32),
        ("ele_cutoff_inp", C.c_double), ("length_per_charge", C.c_double),
        ("ele_excl_bond", C.c_int32), ("ele_excl_angle", C.c_int32),
        ("temp_independent", C.c_int32), ("tempK_ref", C.c_double),
        ("integrator", C.c_int32), ("dt", C.c_double), ("viscosity_Pas", C.c_double), ("nl_margin", C.c_double),
        ("nstep_bp_mc", C.c_int32), ("max_bp_per_nt", C.c_int32),
        ("precision", C.c_int32), ("seed", C.c_uint64), ("nbr_cap", C.c_int32), ("bp_cap", C.c_int32),
    ]


class sis_topology(C.Structure):
    _fields_ = [
        ("n_inst", C.c_int32),
        ("inst_chain_off", C.POINTER(C.c_int32)), ("chain_len", C.POINTER(C.c_int32)),
        ("chain_moltype", C.POINTER(C.c_int32)), ("seq", C.POINTER(C.c_int32)),
        ("has_charge", C.POINTER(C.c_uint8)), ("tempK", C.POINTER(C.c_double)),
        ("ionic_strength", C.POINTER(C.c_double)), ("box", C.POINTER(C.c_double)),
        ("stream", C.POINTER(C.c_uint32)),
    ]


class sis_stats(C.Structure):
    _fields_ = [
        ("steps", C.c_int64), ("rebuilds", C.c_int64), ("pair_entries", C.c_int64), ("wca_pairs", C.c_int64),
        ("ele_pairs", C.c_int64), ("bp_pairs", C.c_int64), ("error_flags", C.c_int32), ("n_beads", C.c_int32),
        ("n_inst", C.c_int32), ("lanes_per_bead", C.c_int32), ("capped", C.c_int64),
        ("bp_blocks", C.c_int32), ("overlap", C.c_int32), ("small_blocks", C.c_int32), ("small_threads", C.c_int32),
        ("cluster_pairs", C.c_int64), ("i_clusters", C.c_int32), ("reserved", C.c_int32),
    ]


EXPORTS = {
    "sis_gpu_create": (C.c_int, [C.POINTER(sis_topology), C.POINTER(sis_params), C.POINTER(C.c_void_p)]),
    "sis_gpu_destroy": (None, [C.c_void_p]),
    "sis_gpu_nmp": (C.c_int, [C.c_void_p, C.c_int32]),
    "sis_gpu_set_state": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sis_gpu_get_state": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sis_gpu_init_velocities": (C.c_int, [C.c_void_p]),
    "sis_gpu_neighbor_list": (C.c_int, [C.c_void_p, C.c_int32]),
    "sis_gpu_get_list": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    "sis_gpu_get_bp_coef": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    "sis_gpu_force": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "sis_gpu_force_term": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    "sis_gpu_energy_sumup": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_void_p]),
    "sis_gpu_energy_kinetic": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]),
    "sis_gpu_rg": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "sis_gpu_invalidate_bp_cache": (C.c_int, [C.c_void_p]),
    "sis_gpu_step": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p]),
    "sis_gpu_set_condition": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double]),
    "sis_gpu_set_temperature": (C.c_int, [C.c_void_p, C.c_int32, C.c_double]),
    "sis_gpu_set_frozen": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32]),
    "sis_gpu_get_ele": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "sis_gpu_get_md_coef": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "sis_gpu_set_force_cap": (C.c_int, [C.c_void_p, C.c_double]),
    "sis_gpu_get_stats": (C.c_int, [C.c_void_p, C.POINTER(sis_stats)]),
    "sis_gpu_get_step": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "sis_gpu_set_lanes": (C.c_int, [C.c_void_p, C.c_int32]),
    "sis_gpu_set_graphs": (C.c_int, [C.c_void_p, C.c_int32]),
    "sis_gpu_set_overlap": (C.c_int, [C.c_void_p, C.c_int32]),
    "sis_gpu_set_small": (C.c_int, [C.c_void_p, C.c_int32]),
    "sis_gpu_set_ss_pairs": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    "sis_gpu_set_bias_ss": (C.c_int, [C.c_void_p, C.c_int32, C.c_double]),
    "sis_gpu_set_step": (C.c_int, [C.c_void_p, C.c_uint64]),
    "sis_gpu_last_error": (C.c_char_p, [C.c_void_p]),
    "sis_gpu_event_record": (C.c_int, [C.c_void_p, C.c_int32]),
    "sis_gpu_event_elapsed": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_float)]),
    "sis_gpu_synchronize": (C.c_int, [C.c_void_p]),
    "sis_gpu_flush_l2": (C.c_int, [C.c_void_p]),
    "sis_gpu_probe_barrier_timeout": (C.c_int, [C.c_void_p]),
    "sis_gpu_set_stage": (C.c_int, [C.c_void_p, C.c_double, C.c_double]),
    "sis_gpu_set_rg_bias": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_double, C.c_double]),
    "sis_gpu_set_bias_items": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "sis_gpu_kernel_launches": (C.c_int64, [C.c_void_p]),
    "sis_gpu_step_profiled": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_float)]),
    "sis_gpu_step_noise_static": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p]),
    "sis_gpu_remd_init": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sis_gpu_remd_init_vars": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "sis_gpu_bp_mc": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32]),
    "sis_gpu_get_bp_status": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    "sis_gpu_get_bp_energies": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    "sis_gpu_load_slot": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                    C.c_double, C.c_uint32, C.c_void_p, C.c_int32]),
    "sis_gpu_remd_exchange": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.POINTER(C.c_int32)]),
}

_lib = None


def lib() -> C.CDLL:
    """Loads libsisgpu.so; raises if it is missing (no CPU fallback exists)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in EXPORTS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def pack_params(system: System, precision: int, seed: int = 12345, nbr_cap: int = 0, bp_cap: int = 0) -> sis_params:
    ff, o = system.ff, system.opts
    p = sis_params()
    p.bond_k, p.bond_r0 = ff.bond_k, ff.bond_r0
    p.angl_reb, p.angl_k, p.angl_t0 = int(ff.angl_reb), ff.angl_k, ff.angl_t0
    p.dih_type, p.dih_k, p.dih_w, p.dih_p0 = ff.dih_type, ff.dih_k, ff.dih_w, ff.dih_p0
    p.wca_sigma, p.wca_eps = ff.wca_sigma, ff.wca_eps
    p.bp_model, p.bp_min_loop, p.bp_jnext_compat = o.bp_model, o.bp_min_loop, int(o.bp_jnext_compat)
    p.bp_cutoff_energy = ff.bp_cutoff_energy
    bpa = ff.bp_array()
    for t in range(3):
        for k in range(15):
            p.bp_ff[t][k] = bpa[t, k]
    for k in range(21):
        p.nn_dH[k], p.nn_dS[k] = ff.nn_dH[k], ff.nn_dS[k]
    p.dH0, p.dS0 = ff.dH0, ff.dS0
    p.nnend = int(ff.nnend)
    for k in range(6):
        p.nnend_dH[k], p.nnend_dS[k] = ff.nnend_dH[k], ff.nnend_dS[k]
    p.dHend0, p.dSend0 = ff.dHend0, ff.dSend0
    p.flg_ele, p.ele_cutoff_type = int(o.flg_ele), o.ele_cutoff_type
    p.ele_cutoff_inp, p.length_per_charge = o.ele_cutoff, o.length_per_charge
    p.ele_excl_bond, p.ele_excl_angle = int(o.ele_excl_bond), int(o.ele_excl_angle)
    p.temp_independent, p.tempK_ref = o.temp_independent, o.tempK_ref
    p.integrator, p.dt, p.viscosity_Pas, p.nl_margin = o.integrator, o.dt, o.viscosity_Pas, o.nl_margin
    p.nstep_bp_mc, p.max_bp_per_nt = o.nstep_bp_mc, o.max_bp_per_nt
    p.precision, p.seed, p.nbr_cap, p.bp_cap = precision, seed, nbr_cap, bp_cap
    return p


class TopologyArrays:
    """Keeps the numpy arrays behind a sis_topology alive."""

    def __init__(self, system: System, streams=None):
        ch_off, lens, types, seqs, charges, temps, salts, boxes = [0], [], [], [], [], [], [], []
        for inst in system.instances:
            for c in inst.chains:
                lens.append(len(c))
                types.append(c.moltype)
            ch_off.append(len(lens))
            seqs.append(inst.seq())
            charges.append(inst.charges())
            temps.append(inst.tempK)
            salts.append(inst.ionic_strength)
            boxes.append(list(inst.box) if inst.box is not None else [0.0, 0.0, 0.0])
        self.ch_off = np.asarray(ch_off, dtype=np.int32)
        self.lens = np.asarray(lens, dtype=np.int32)
        self.types = np.asarray(types, dtype=np.int32)
        self.seq = np.ascontiguousarray(np.concatenate(seqs), dtype=np.int32)
        self.charge = np.ascontiguousarray(np.concatenate(charges), dtype=np.uint8)
        self.temps = np.asarray(temps, dtype=np.float64)
        self.salts = np.asarray(salts, dtype=np.float64)
        self.boxes = np.asarray(boxes, dtype=np.float64).reshape(-1)
        t = sis_topology()
        t.n_inst = len(system.instances)
        P = lambda a, ty: a.ctypes.data_as(C.POINTER(ty))
        t.inst_chain_off = P(self.ch_off, C.c_int32)
        t.chain_len = P(self.lens, C.c_int32)
        t.chain_moltype = P(self.types, C.c_int32)
        t.seq = P(self.seq, C.c_int32)
        t.has_charge = P(self.charge, C.c_uint8)
        t.tempK = P(self.temps, C.c_double)
        t.ionic_strength = P(self.salts, C.c_double)
        t.box = P(self.boxes, C.c_double)
        if streams is not None:
            self.streams = np.asarray(streams, dtype=np.uint32)
            t.stream = P(self.streams, C.c_uint32)
        self.struct = t


def ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None
