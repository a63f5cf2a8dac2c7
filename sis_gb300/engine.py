"""Host-side mirror of the reference's hot-path interface over libsisgpu.

The reference's Fortran routines act on module state for replica ``irep``:
``force(irep, forces)`` (src/force.F90:1), ``energy_sumup(irep, tempK_in,
energies)`` (src/energy_sumup.F90:1), ``neighbor_list(irep)``
(src/neighbor_list.F90:1) and the time loop of ``job_md``
(src/job_md.F90:360-460).  :class:`Engine` exposes the same operations with
0-based instance indices; arrays are numpy, shaped (nmp, 3) where the
reference uses (3, nmp).  Every call goes through the C ABI of
include/sis_gpu.h; a failing call raises :class:`SisError`.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _abi
from ._abi import SisError, ptr
from .model import MIXED, System

ENE_NAMES = ["total", "bond", "angl", "dihe", "bp", "exv", "ele", "stage", "twz", "rg", "rest"]


class Engine:
    def __init__(self, system: System, precision: int = MIXED, seed: int = 12345, nbr_cap: int = 0, bp_cap: int = 0,
                 streams: Optional[Sequence[int]] = None):
        self.L = _abi.lib()
        self.system = system
        self.precision = precision
        # the Philox key and the noise stream of every instance: with the
        # step counter they determine the noise (restart files keep them)
        self.seed = int(seed)
        self.streams = [int(v) for v in streams] if streams is not None else list(range(len(system.instances)))
        self._topo = _abi.TopologyArrays(system, streams)
        self._par = _abi.pack_params(system, precision, seed, nbr_cap, bp_cap)
        h = C.c_void_p()
        rc = self.L.sis_gpu_create(C.byref(self._topo.struct), C.byref(self._par), C.byref(h))
        if rc != 0:
            raise SisError(rc, "sis_gpu_create failed")
        self.h = h
        self.n_inst = len(system.instances)
        self.offsets = system.offsets()
        self.n = int(self.offsets[-1])
        if all(i.xyz is not None for i in system.instances):
            self.set_state(-1, np.concatenate([np.asarray(i.xyz, dtype=np.float64) for i in system.instances]))

    # ------------------------------------------------------------- plumbing
    def _ck(self, rc: int):
        if rc != 0:
            raise SisError(rc, self.L.sis_gpu_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.sis_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def nmp(self, inst: int = -1) -> int:
        return self.n if inst < 0 else int(self.offsets[inst + 1] - self.offsets[inst])

    # ---------------------------------------------------------------- state
    def set_state(self, inst: int, xyz=None, velos=None, accels=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (xyz, velos, accels)]
        for a in arrs:
            if a is not None and a.size != 3 * self.nmp(inst):
                raise ValueError("state array size does not match the instance")
        self._ck(self.L.sis_gpu_set_state(self.h, inst, *(ptr(a) for a in arrs)))

    def get_state(self, inst: int = -1):
        n = self.nmp(inst)
        x, v, a = (np.empty((n, 3)) for _ in range(3))
        self._ck(self.L.sis_gpu_get_state(self.h, inst, ptr(x), ptr(v), ptr(a)))
        return x, v, a

    def init_velocities(self):
        self._ck(self.L.sis_gpu_init_velocities(self.h))

    # ---------------------------------------------------- reference interface
    def neighbor_list(self, inst: int = -1):
        self._ck(self.L.sis_gpu_neighbor_list(self.h, inst))

    def get_list(self, inst: int, kind: int) -> np.ndarray:
        """kind 0 wca (n,2), 1 ele (n,2), 2 bp (n,7), 3 / 4 the wca / ele pairs
        of the per-block kernel's inner lists (n,2); 1-based local indices."""
        w = 7 if kind == 2 else 2
        n = C.c_int32()
        self._ck(self.L.sis_gpu_get_list(self.h, inst, kind, None, 0, C.byref(n)))
        out = np.zeros((max(n.value, 1), w), dtype=np.int32)
        self._ck(self.L.sis_gpu_get_list(self.h, inst, kind, ptr(out), n.value, C.byref(n)))
        return out[: n.value]

    def get_bp_coef(self, inst: int) -> np.ndarray:
        n = C.c_int32()
        self._ck(self.L.sis_gpu_get_bp_coef(self.h, inst, None, 0, C.byref(n)))
        out = np.zeros((max(n.value, 1), 2))
        self._ck(self.L.sis_gpu_get_bp_coef(self.h, inst, ptr(out), n.value, C.byref(n)))
        return out[: n.value]

    def force(self, inst: int = 0) -> np.ndarray:
        out = np.empty((self.nmp(inst), 3))
        self._ck(self.L.sis_gpu_force(self.h, inst, ptr(out)))
        return out

    def force_term(self, inst: int, term: int) -> np.ndarray:
        out = np.empty((self.nmp(inst), 3))
        self._ck(self.L.sis_gpu_force_term(self.h, inst, term, ptr(out)))
        return out

    def energy_sumup(self, inst: int = 0, tempK: Optional[float] = None) -> np.ndarray:
        T = self.system.instances[inst].tempK if tempK is None else tempK
        out = np.zeros(11)
        self._ck(self.L.sis_gpu_energy_sumup(self.h, inst, float(T), ptr(out)))
        return out

    def energy_kinetic(self, inst: int = 0) -> float:
        e = C.c_double()
        self._ck(self.L.sis_gpu_energy_kinetic(self.h, inst, C.byref(e)))
        return e.value

    def invalidate_bp_cache(self):
        self._ck(self.L.sis_gpu_invalidate_bp_cache(self.h))

    def step(self, nsteps: int, noise: Optional[np.ndarray] = None):
        if noise is not None:
            noise = np.ascontiguousarray(noise, dtype=np.float64)
            if noise.size != nsteps * self.n * 3:
                raise ValueError("noise must hold nsteps * n_beads * 3 values")
        self._ck(self.L.sis_gpu_step(self.h, int(nsteps), ptr(noise)))

    def set_condition(self, inst: int, tempK: float, ionic_strength: float):
        self._ck(self.L.sis_gpu_set_condition(self.h, inst, float(tempK), float(ionic_strength)))
        self.system.instances[inst].tempK = tempK
        self.system.instances[inst].ionic_strength = ionic_strength

    def set_temperature(self, inst: int, tempK: float):
        """The annealing update (job_md.F90:597-611): noise coefficients and
        base-pair free energies at tempK, Debye-Hueckel left as it was set;
        inst = -1 for every instance."""
        self._ck(self.L.sis_gpu_set_temperature(self.h, int(inst), float(tempK)))
        for k in (range(self.n_inst) if inst < 0 else [inst]):
            self.system.instances[k].tempK = tempK

    def set_frozen(self, inst: int, beads):
        """[Freeze]: 1-based bead numbers of an instance whose positions stay
        fixed; replaces the instance's earlier set (an empty list frees all)."""
        b = np.ascontiguousarray(beads, dtype=np.int32).ravel()
        self._ck(self.L.sis_gpu_set_frozen(self.h, int(inst), b.ctypes.data_as(C.c_void_p), b.size))

    def set_force_cap(self, fmax: float):
        """Equilibration aid: caps each bead's force magnitude (0 = off)."""
        self._ck(self.L.sis_gpu_set_force_cap(self.h, float(fmax)))

    def relax(self, capped_steps: int = 3000, fmax: float = 1000.0, free_steps: int = 2000):
        """Force-capped dynamics followed by uncapped dynamics; removes the
        bead overlaps of random-coil starts before production steps."""
        self.set_force_cap(fmax)
        self.step(capped_steps)
        self.set_force_cap(0.0)
        self.step(free_steps)

    def get_md_coef(self, inst: int = -1) -> np.ndarray:
        out = np.zeros((self.nmp(inst), 4))
        self._ck(self.L.sis_gpu_get_md_coef(self.h, inst, ptr(out)))
        return out

    def get_ele(self, inst: int) -> np.ndarray:
        out = np.zeros(4)
        self._ck(self.L.sis_gpu_get_ele(self.h, inst, ptr(out)))
        return out

    def set_lanes(self, lanes: int):
        """Lanes per bead of the step kernel; 0 lets the autotuner choose."""
        self._ck(self.L.sis_gpu_set_lanes(self.h, int(lanes)))

    def set_graphs(self, enable: bool):
        """Run steady-state steps as CUDA graphs (default) or launch by launch."""
        self._ck(self.L.sis_gpu_set_graphs(self.h, int(bool(enable))))

    def rg(self, inst: int = -1) -> np.ndarray:
        """Radius of gyration of one instance or (inst = -1) of every instance."""
        out = np.zeros(self.n_inst if inst < 0 else 1)
        self._ck(self.L.sis_gpu_rg(self.h, int(inst), ptr(out)))
        return out

    def load_slot(self, inst: int, chains, tempK: float, ionic_strength: float, stream: int, xyz,
                  init_velocities: bool = False):
        """Replace instance `inst` by a job (list of Chain) that fits its bead count."""
        lens = np.array([len(c) for c in chains], dtype=np.int32)
        molt = np.array([c.moltype for c in chains], dtype=np.int32)
        seq = np.ascontiguousarray(np.concatenate([c.seq for c in chains]) if len(chains) else np.zeros(0), dtype=np.int32)
        x = np.ascontiguousarray(xyz, dtype=np.float64) if len(chains) else np.zeros((0, 3))
        vp = C.c_void_p
        self._ck(self.L.sis_gpu_load_slot(self.h, int(inst), len(chains), lens.ctypes.data_as(vp), molt.ctypes.data_as(vp),
                                          seq.ctypes.data_as(vp), None, float(tempK), float(ionic_strength), int(stream),
                                          x.ctypes.data_as(vp), int(bool(init_velocities))))
        self.streams[inst] = int(stream)

    def bp_mc(self, inst: int = -1, draws: Optional[np.ndarray] = None):
        """Request a base-pair Monte Carlo pass at the next force or step evaluation."""
        d = None if draws is None else np.ascontiguousarray(draws, dtype=np.float64)
        self._ck(self.L.sis_gpu_bp_mc(self.h, int(inst), ptr(d), 0 if d is None else d.size))

    # optional terms (force.F90:62-75): force term 7, energy slots 7-10
    def set_stage(self, sigma: float, eps: float):
        """Stage wall at z = 0 (force_stage.F90); sigma = 0 turns it off."""
        self._ck(self.L.sis_gpu_set_stage(self.h, float(sigma), float(eps)))
        self._stage = float(sigma) > 0.0

    def set_rg_bias(self, inst: int, k: float, rg0: float, flat: bool = False, off: bool = False):
        """Bias on the radius of gyration (force_rg.F90); inst -1: all."""
        self._ck(self.L.sis_gpu_set_rg_bias(self.h, int(inst), 0 if off else (2 if flat else 1), float(k), float(rg0)))
        if not hasattr(self, "_rg"):
            self._rg = {}
        for q in (range(self.n_inst) if inst < 0 else [inst]):
            self._rg[q] = None if off else (float(k), float(rg0), bool(flat))

    def rg_bias(self, inst: int):
        """(k, rg0, flat) of an instance's Rg bias, or None when it is off."""
        return getattr(self, "_rg", {}).get(inst)

    def tweezers(self, inst: int):
        """(ConstantForcePair list, ForceRampPair list) of an instance."""
        return getattr(self, "_bias", {}).get(inst, {"twz": ([], [])})["twz"]

    def optional_terms(self) -> dict:
        """Which optional terms are on in any instance (the flg_stage,
        flg_twz, flg_bias_rg and flg_restraint of var_potential.F90)."""
        b = getattr(self, "_bias", {})
        return {"stage": getattr(self, "_stage", False),
                "twz": any(len(v["twz"][0]) + len(v["twz"][1]) > 0 for v in b.values()),
                "rg": any(v is not None for v in getattr(self, "_rg", {}).values()),
                "rest": any(len(v["rest"]) > 0 for v in b.values())}

    def set_restraints(self, inst: int, restraints):
        """Sigmoid restraints (sis_gb300.model.Restraint) of one instance."""
        self._bias_items(inst)["rest"] = list(restraints)
        self._upload_bias(inst)

    def set_tweezers(self, inst: int, dcf=(), fr=()):
        """Trap pairs of one instance: ConstantForcePair and ForceRampPair."""
        self._bias_items(inst)["twz"] = (list(dcf), list(fr))
        self._upload_bias(inst)

    def _bias_items(self, inst):
        if not hasattr(self, "_bias"):
            self._bias = {}
        return self._bias.setdefault(inst, {"rest": [], "twz": ([], [])})

    def _upload_bias(self, inst):
        b = self._bias_items(inst)
        kij, par = [], []
        for q in b["rest"]:
            kij.append((2 if q.to_bead else 1, q.i, q.j))
            par.append([q.eps, q.d, q.s, q.rcut] + [0.0] * 10)
        dcf, fr = b["twz"]
        for q in dcf:
            kij.append((3, q.i, q.j))
            par.append(list(np.asarray(q.force, dtype=np.float64).reshape(3)) + [0.0] * 11)
        for q in fr:
            kij.append((4, q.i, q.j))
            par.append(list(np.asarray(q.k, dtype=np.float64).reshape(2)) + list(np.asarray(q.init, dtype=np.float64).reshape(6))
                       + list(np.asarray(q.velo, dtype=np.float64).reshape(6)))
        kij = np.ascontiguousarray(np.array(kij, dtype=np.int32).reshape(-1, 3))
        par = np.ascontiguousarray(np.array(par, dtype=np.float64).reshape(-1, 14))
        self._ck(self.L.sis_gpu_set_bias_items(self.h, int(inst), kij.shape[0], kij.ctypes.data_as(C.c_void_p),
                                               par.ctypes.data_as(C.c_void_p)))

    def get_bp_energies(self, inst: int) -> np.ndarray:
        """Cached energy of every base-pair record (order of get_list(inst, 2))."""
        n = C.c_int32()
        self._ck(self.L.sis_gpu_get_bp_energies(self.h, inst, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=np.float64)
        self._ck(self.L.sis_gpu_get_bp_energies(self.h, inst, out.ctypes.data_as(C.c_void_p), n.value, C.byref(n)))
        return out

    def get_bp_status(self, inst: int) -> np.ndarray:
        n = C.c_int32()
        self._ck(self.L.sis_gpu_get_bp_status(self.h, inst, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=np.uint8)
        self._ck(self.L.sis_gpu_get_bp_status(self.h, inst, out.ctypes.data_as(C.c_void_p), n.value, C.byref(n)))
        return out

    def remd_init(self, temps):
        """Temperature replica exchange over the instances; temps: the ladder by label."""
        t = np.ascontiguousarray(temps, dtype=np.float64)
        if t.size != self.n_inst:
            raise ValueError("one temperature per instance")
        self._ck(self.L.sis_gpu_remd_init(self.h, ptr(t)))

    def remd_init_vars(self, kinds, values):
        """Replica exchange over replica variables (1 T, 2 ionic strength,
        3 trap force, 4 Rg target); values[label][variable]."""
        k = np.ascontiguousarray(kinds, dtype=np.int32)
        v = np.ascontiguousarray(np.asarray(values, dtype=np.float64).reshape(self.n_inst, k.size))
        self._ck(self.L.sis_gpu_remd_init_vars(self.h, k.size, ptr(k), ptr(v)))

    def remd_exchange(self, parity: int, uniforms: Optional[np.ndarray] = None):
        """One exchange attempt; returns (label of every instance, accepted pairs)."""
        u = None
        if uniforms is not None:
            u = np.zeros(self.n_inst // 2 + 1)
            uu = np.asarray(uniforms, dtype=np.float64).ravel()
            u[:min(u.size, uu.size)] = uu[:u.size]
        r2l = np.zeros(self.n_inst, dtype=np.int32)
        acc = C.c_int32()
        self._ck(self.L.sis_gpu_remd_exchange(self.h, int(parity), ptr(u), r2l.ctypes.data_as(C.c_void_p), C.byref(acc)))
        return r2l, int(acc.value)

    def set_ss_pairs(self, inst: int, pairs):
        """Base pairs of instance inst only between these (imp, jmp), 1-based."""
        a = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        self._ck(self.L.sis_gpu_set_ss_pairs(self.h, int(inst), a.shape[0], a.ctypes.data_as(C.c_void_p)))

    def set_bias_ss(self, force_kcal_per_mol_A: float, on: bool = True):
        """[Bias_SS]: constant pull of allowed pairs outside their distance window."""
        self._ck(self.L.sis_gpu_set_bias_ss(self.h, int(on), float(force_kcal_per_mol_A)))

    def set_small(self, mode: int):
        """Per-block kernel of small instances: -1 where eligible (default), 0 never."""
        self._ck(self.L.sis_gpu_set_small(self.h, int(mode)))

    def set_overlap(self, enable):
        """Pair forces in their own kernel beside the bonded/base-pair pass
        (True) or in the step kernel (False); None lets the autotuner choose."""
        self._ck(self.L.sis_gpu_set_overlap(self.h, -1 if enable is None else int(bool(enable))))

    def get_step(self) -> int:
        v = C.c_uint64()
        self._ck(self.L.sis_gpu_get_step(self.h, C.byref(v)))
        return int(v.value)

    def set_step(self, step: int):
        self._ck(self.L.sis_gpu_set_step(self.h, int(step)))

    def stats(self) -> dict:
        s = _abi.sis_stats()
        self._ck(self.L.sis_gpu_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    # --------------------------------------------------------------- timing
    def event(self, slot: int):
        self._ck(self.L.sis_gpu_event_record(self.h, slot))

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_float()
        self._ck(self.L.sis_gpu_event_elapsed(self.h, a, b, C.byref(ms)))
        return ms.value

    def synchronize(self):
        self._ck(self.L.sis_gpu_synchronize(self.h))

    def flush_l2(self):
        self._ck(self.L.sis_gpu_flush_l2(self.h))

    def step_profiled(self, nsteps: int):
        ms = (C.c_float * 3)()
        self._ck(self.L.sis_gpu_step_profiled(self.h, int(nsteps), ms))
        return list(ms)

    def kernel_launches(self) -> int:
        return int(self.L.sis_gpu_kernel_launches(self.h))
