"""lulesh_gb300 -- the LULESH Lagrange leap-frog timestep on one GB300.

Python mirror of the reference's Domain surface (lulesh.h:148-595) over the C
ABI in include/lulesh_gb300.h.  Every compute call runs the native CUDA
library ``lib/liblulesh_gb300.so``; there is no CPU fallback, and importing a
``Domain`` without the built library raises.

    from lulesh_gb300 import Domain
    d = Domain(nx=30, numReg=11, balance=1, cost=1, its=100)
    d.run()                      # the reference main loop on the GPU
    print(d.report(elapsed))     # VerifyAndWriteFinalOutput text
    e = d.field("e")             # numpy copy of an accessor array

Errors the reference turns into exit(-1)/exit(-2) (lulesh.h:42) are returned
as status codes by ``step``/``run`` (or raised as VolumeError/QStopError with
``check=True``); API and CUDA failures raise LuleshError.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

__all__ = ["Domain", "LuleshError", "VolumeError", "QStopError", "library_path", "load",
           "FP64", "FP64_FMA", "MIXED", "NODE_FIELDS", "ELEM_FIELDS", "measure_pipe", "Ensemble",
           "sample_ensemble", "HaloPlan", "HALO_KINDS"]

_PKG = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_PKG, "lib", "liblulesh_gb300.so")

FP64, FP64_FMA, MIXED = 0, 1, 2
_PRECISION = {"fp64": FP64, "fp64-fma": FP64_FMA, "fp64_fma": FP64_FMA, "mixed": MIXED}

NODE_FIELDS = ["x", "y", "z", "xd", "yd", "zd", "xdd", "ydd", "zdd", "fx", "fy", "fz",
               "nodalMass"]
ELEM_FIELDS = ["e", "p", "q", "ql", "qq", "v", "volo", "vnew", "delv", "vdov", "arealg",
               "ss", "elemMass"]
# the state the adjoint carries, in lg_adjoint_vjp's seed / gradient order
ADJOINT_FIELDS = ["x", "y", "z", "xd", "yd", "zd", "e", "p", "q", "v", "ss"]


class LuleshError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class VolumeError(LuleshError):
    """The reference's exit(VolumeError): a non-positive element volume."""


class QStopError(LuleshError):
    """The reference's exit(QStopError): artificial viscosity above qstop."""


class _Opts(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("numReg", ctypes.c_int), ("balance", ctypes.c_int),
                ("cost", ctypes.c_int), ("its", ctypes.c_int), ("precision", ctypes.c_int),
                ("hgcoef", ctypes.c_double), ("einit_factor", ctypes.c_double),
                ("device", ctypes.c_int)]


class _HaloInfo(ctypes.Structure):
    _fields_ = [("buffer_doubles", ctypes.c_size_t), ("send_messages", ctypes.c_int),
                ("recv_messages", ctypes.c_int), ("send_values", ctypes.c_int),
                ("recv_values", ctypes.c_int), ("recv_targets", ctypes.c_int),
                ("ghost_elems", ctypes.c_int), ("field_length", ctypes.c_int)]


_lib = None


def library_path() -> str:
    return _LIB_PATH


def load() -> ctypes.CDLL:
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise ImportError(
            f"{_LIB_PATH} is missing: build it with `python -m lulesh_gb300.build` "
            "(or __graft_entry__.build()); there is no CPU fallback")
    lib = ctypes.CDLL(_LIB_PATH)
    H = ctypes.c_void_p
    lib.lg_default_opts.argtypes = [ctypes.POINTER(_Opts)]
    lib.lg_create.argtypes = [ctypes.POINTER(_Opts), ctypes.POINTER(H)]
    lib.lg_destroy.argtypes = [H]
    lib.lg_step.argtypes = [H, ctypes.c_int]
    lib.lg_run.argtypes = [H]
    lib.lg_step_timed.argtypes = [H, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    lib.lg_phase.argtypes = [H, ctypes.c_int]
    lib.lg_field_info.argtypes = [H, ctypes.c_char_p, ctypes.POINTER(ctypes.c_size_t),
                                  ctypes.POINTER(ctypes.c_int)]
    lib.lg_get_field.argtypes = [H, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_size_t]
    lib.lg_set_field.argtypes = [H, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_size_t]
    lib.lg_get_scalar.argtypes = [H, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)]
    lib.lg_set_scalar.argtypes = [H, ctypes.c_char_p, ctypes.c_double]
    lib.lg_region_rep.argtypes = [H, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    lib.lg_report.argtypes = [H, ctypes.c_double, ctypes.c_char_p, ctypes.c_size_t]
    lib.lg_verify.argtypes = [H, ctypes.POINTER(ctypes.c_double)]
    lib.lg_profile.argtypes = [H, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                               ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_int)]
    lib.lg_reset.argtypes = [H]
    lib.lg_dt_record.argtypes = [H, ctypes.c_int]
    lib.lg_dt_get.argtypes = [H, ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    lib.lg_dt_freeze.argtypes = [H, ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    lib.lg_adjoint.argtypes = [H, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_ubyte),
                               ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                               ctypes.POINTER(ctypes.c_double)]
    P11 = ctypes.c_void_p * 11
    lib.lg_adjoint_vjp.argtypes = [H, ctypes.c_int, ctypes.c_int, P11, P11,
                                   ctypes.POINTER(ctypes.c_double)]
    lib.lg_ensemble_sample.argtypes = [ctypes.c_int, ctypes.c_ulonglong, ctypes.POINTER(_Opts)]
    lib.lg_ensemble_create.argtypes = [ctypes.c_int, ctypes.POINTER(_Opts), ctypes.POINTER(H)]
    lib.lg_ensemble_destroy.argtypes = [H]
    lib.lg_ensemble_step.argtypes = [H, ctypes.c_int]
    lib.lg_ensemble_step_timed.argtypes = [H, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    lib.lg_ensemble_reset.argtypes = [H]
    lib.lg_ensemble_info.argtypes = [H] + [ctypes.POINTER(ctypes.c_longlong)] * 3
    lib.lg_ensemble_get_field.argtypes = [H, ctypes.c_int, ctypes.c_char_p, ctypes.c_void_p,
                                          ctypes.c_size_t]
    lib.lg_ensemble_set_field.argtypes = [H, ctypes.c_int, ctypes.c_char_p, ctypes.c_void_p,
                                          ctypes.c_size_t]
    lib.lg_ensemble_get_scalar.argtypes = [H, ctypes.c_int, ctypes.c_char_p,
                                           ctypes.POINTER(ctypes.c_double)]
    lib.lg_ensemble_autotune.argtypes = [H, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(ctypes.c_int)]
    lib.lg_measure_pipe.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    lib.lg_halo_plan_create.argtypes = [ctypes.c_int] * 5 + [ctypes.POINTER(H)]
    lib.lg_halo_plan_destroy.argtypes = [H]
    lib.lg_halo_plan_info.argtypes = [H, ctypes.POINTER(_HaloInfo)]
    lib.lg_halo_plan_message.argtypes = [H, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(ctypes.c_size_t)]
    lib.lg_halo_plan_entries.argtypes = [H, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_size_t]
    lib.lg_halo_pack.argtypes = [H, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.lg_halo_unpack.argtypes = [H, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.lg_last_error.restype = ctypes.c_char_p
    _lib = lib
    return lib


def measure_pipe(op: str = "fma", fp32: bool = False) -> float:
    """Measured issue rate of one arithmetic pipe, in 1e9 thread-instructions/s."""
    lib = load()
    v = ctypes.c_double()
    st = lib.lg_measure_pipe({"fma": 0, "add": 1, "mul": 2}[op], int(fp32), ctypes.byref(v))
    if st:
        _raise(st, lib)
    return v.value


def _raise(code: int, lib) -> None:
    msg = (lib.lg_last_error() or b"").decode()
    if code == -1:
        raise VolumeError(code, msg or "VolumeError")
    if code == -2:
        raise QStopError(code, msg or "QStopError")
    raise LuleshError(code, msg)


class Domain:
    """A Sedov problem resident on the GPU, driven through the C ABI.

    Constructor arguments are the reference's -s -r -b -c -i options
    (lulesh.cc:2682-2690 defaults) plus the device-path choices.
    """

    def __init__(self, nx: int = 30, numReg: int = 11, balance: int = 1, cost: int = 1,
                 its: int = 9999999, precision: str | int = "fp64", hgcoef: float = 3.0,
                 einit_factor: float = 1.0, device: int = 0):
        lib = load()
        self._lib = lib
        o = _Opts()
        lib.lg_default_opts(ctypes.byref(o))
        o.nx, o.numReg, o.balance, o.cost, o.its = nx, numReg, balance, cost, its
        o.precision = _PRECISION[precision] if isinstance(precision, str) else int(precision)
        o.hgcoef, o.einit_factor, o.device = hgcoef, einit_factor, device
        h = ctypes.c_void_p()
        st = lib.lg_create(ctypes.byref(o), ctypes.byref(h))
        if st:
            _raise(st, lib)
        self._h = h
        self.nx = nx
        self.numElem = nx ** 3
        self.numNode = (nx + 1) ** 3

    # lifetime -------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.lg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # time stepping -------------------------------------------------------
    def _status(self, st: int, check: bool) -> int:
        if st > 0 or (check and st < 0):
            _raise(st, self._lib)
        return st

    def step(self, ncycles: int = 1, check: bool = False) -> int:
        """Up to ncycles of TimeIncrement + LagrangeLeapFrog; returns 0/-1/-2."""
        return self._status(self._lib.lg_step(self._h, int(ncycles)), check)

    def run(self, check: bool = False) -> int:
        """The reference main loop until stoptime or its (lulesh.cc:2745)."""
        return self._status(self._lib.lg_run(self._h), check)

    def step_timed(self, ncycles: int) -> tuple[int, float]:
        ms = ctypes.c_double()
        st = self._lib.lg_step_timed(self._h, int(ncycles), ctypes.byref(ms))
        self._status(st, False)
        return st, ms.value

    def reset(self) -> None:
        """Restore the state built at creation (lg_reset)."""
        st = self._lib.lg_reset(self._h)
        if st:
            _raise(st, self._lib)

    # frozen time steps and the adjoint ------------------------------------
    def dt_record(self, capacity: int) -> None:
        """Record every following cycle's time step (index = cycle number)."""
        st = self._lib.lg_dt_record(self._h, int(capacity))
        if st:
            _raise(st, self._lib)

    def dt_get(self, n: int) -> np.ndarray:
        out = np.empty(n, dtype=np.float64)
        st = self._lib.lg_dt_get(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n)
        if st:
            _raise(st, self._lib)
        return out

    def dt_freeze(self, dts) -> None:
        """Cycle c uses dts[c] instead of TimeIncrement (empty: unfreeze)."""
        a = np.ascontiguousarray(dts, dtype=np.float64)
        st = self._lib.lg_dt_freeze(self._h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                    a.size)
        if st:
            _raise(st, self._lib)

    def adjoint(self, ncycles: int, mask, ckpt: int = 20) -> tuple[float, np.ndarray, float]:
        """J = sum(e * volo over mask) after ncycles frozen-dt cycles from the
        current state, and its gradients with respect to the current energy
        field and hgcoef (lg_adjoint)."""
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        if m.size != self.numElem:
            raise ValueError("mask needs one entry per element")
        J = ctypes.c_double()
        ge = np.empty(self.numElem, dtype=np.float64)
        gh = ctypes.c_double()
        st = self._lib.lg_adjoint(self._h, int(ncycles), int(ckpt),
                                  m.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)),
                                  ctypes.byref(J),
                                  ge.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                  ctypes.byref(gh))
        if st:
            _raise(st, self._lib)
        return J.value, ge, gh.value

    def adjoint_vjp(self, ncycles: int, seeds: dict, want=ADJOINT_FIELDS,
                    ckpt: int = 20) -> tuple[dict, float]:
        """Reverse-mode product of ncycles frozen-dt cycles from the current
        state (lg_adjoint_vjp): seeds maps final-state field names (of
        ADJOINT_FIELDS) to dJ/d(final field); returns {name: dJ/d(initial
        field)} for the names in `want`, and dJ/dhgcoef."""
        seed_arr = (ctypes.c_void_p * 11)()
        keep = []
        for name, v in seeds.items():
            if name not in ADJOINT_FIELDS:
                raise KeyError(f"{name} is not one of {ADJOINT_FIELDS}")
            n = self.numNode if name in NODE_FIELDS else self.numElem
            a = np.ascontiguousarray(v, dtype=np.float64)
            if a.size != n:
                raise ValueError(f"seed {name}: expected {n} values, got {a.size}")
            keep.append(a)
            seed_arr[ADJOINT_FIELDS.index(name)] = a.ctypes.data
        grad_arr = (ctypes.c_void_p * 11)()
        grads = {}
        for name in want:
            n = self.numNode if name in NODE_FIELDS else self.numElem
            grads[name] = np.empty(n, dtype=np.float64)
            grad_arr[ADJOINT_FIELDS.index(name)] = grads[name].ctypes.data
        gh = ctypes.c_double()
        st = self._lib.lg_adjoint_vjp(self._h, int(ncycles), int(ckpt), seed_arr, grad_arr,
                                      ctypes.byref(gh))
        if st:
            _raise(st, self._lib)
        return grads, gh.value

    def phase(self, which: int) -> int:
        return self._status(self._lib.lg_phase(self._h, int(which)), False)

    def profile(self, ncycles: int) -> dict:
        cap = 16
        ms = (ctypes.c_double * cap)()
        names = (ctypes.c_char_p * cap)()
        n = ctypes.c_int(cap)
        st = self._lib.lg_profile(self._h, int(ncycles), ms, names, ctypes.byref(n))
        self._status(st, False)
        return {names[i].decode(): ms[i] for i in range(n.value)}

    # fields --------------------------------------------------------------
    def field_info(self, name: str) -> tuple[int, np.dtype]:
        n = ctypes.c_size_t()
        dt = ctypes.c_int()
        st = self._lib.lg_field_info(self._h, name.encode(), ctypes.byref(n), ctypes.byref(dt))
        if st:
            _raise(st, self._lib)
        return n.value, (np.float64 if dt.value == 0 else np.int32)

    def field(self, name: str, out: np.ndarray | None = None) -> np.ndarray:
        """Copy of the accessor array `name` (lulesh.h:263-367)."""
        n, dt = self.field_info(name)
        if out is None:
            out = np.empty(n, dtype=dt)
        if out.dtype != dt or out.size != n or not out.flags.c_contiguous:
            raise ValueError(f"{name}: need a contiguous {np.dtype(dt)}[{n}] buffer")
        st = self._lib.lg_get_field(self._h, name.encode(), out.ctypes.data, n)
        if st:
            _raise(st, self._lib)
        return out

    def set_field(self, name: str, values) -> None:
        n, dt = self.field_info(name)
        a = np.ascontiguousarray(values, dtype=dt)
        if a.size != n:
            raise ValueError(f"{name}: expected {n} entries, got {a.size}")
        st = self._lib.lg_set_field(self._h, name.encode(), a.ctypes.data, n)
        if st:
            _raise(st, self._lib)

    def scalar(self, name: str) -> float:
        v = ctypes.c_double()
        st = self._lib.lg_get_scalar(self._h, name.encode(), ctypes.byref(v))
        if st:
            _raise(st, self._lib)
        return v.value

    def set_scalar(self, name: str, value: float) -> None:
        st = self._lib.lg_set_scalar(self._h, name.encode(), float(value))
        if st:
            _raise(st, self._lib)

    @property
    def cycle(self) -> int:
        return int(self.scalar("cycle"))

    @property
    def time(self) -> float:
        return self.scalar("time")

    @property
    def deltatime(self) -> float:
        return self.scalar("deltatime")

    def region_rep(self, r: int) -> int:
        v = ctypes.c_int()
        st = self._lib.lg_region_rep(self._h, r, ctypes.byref(v))
        if st:
            _raise(st, self._lib)
        return v.value

    def state(self) -> dict:
        out = {f: self.field(f) for f in NODE_FIELDS + ELEM_FIELDS}
        for s in ("time", "deltatime", "dtcourant", "dthydro", "cycle"):
            out[s] = self.scalar(s)
        return out

    # report --------------------------------------------------------------
    def verify(self) -> dict:
        v = (ctypes.c_double * 4)()
        st = self._lib.lg_verify(self._h, v)
        if st:
            _raise(st, self._lib)
        return {"origin_energy": v[0], "MaxAbsDiff": v[1], "TotalAbsDiff": v[2],
                "MaxRelDiff": v[3]}

    def report(self, elapsed: float) -> str:
        buf = ctypes.create_string_buffer(8192)
        st = self._lib.lg_report(self._h, float(elapsed), buf, len(buf))
        if st:
            _raise(st, self._lib)
        return buf.value.decode()


_OPT_KEYS = ("nx", "numReg", "balance", "cost", "its", "hgcoef", "einit_factor")


def sample_ensemble(nprob: int = 64, seed: int = 0) -> list[dict]:
    """The ensemble study's problem set (lg_ensemble_sample): nx in 16..64,
    log-uniform energy factor in [0.5, 2], hgcoef in [1, 3], 4..16 regions,
    balance 1, cost 1, 300 cycles."""
    lib = load()
    arr = (_Opts * nprob)()
    st = lib.lg_ensemble_sample(nprob, seed, arr)
    if st:
        _raise(st, lib)
    return [{k: getattr(o, k) for k in _OPT_KEYS} for o in arr]


class Ensemble:
    """Many independent Sedov problems advanced together on one GPU
    (lg_ensemble_*): each member keeps its own time step, cycle count and stop
    test, while every phase of the cycle is one launch over all members."""

    def __init__(self, members: list[dict], precision: str | int = "fp64", device: int = 0):
        lib = load()
        self._lib = lib
        n = len(members)
        arr = (_Opts * n)()
        prec = _PRECISION[precision] if isinstance(precision, str) else int(precision)
        for o, m in zip(arr, members):
            lib.lg_default_opts(ctypes.byref(o))
            for k, v in m.items():
                setattr(o, k, v)
            o.precision, o.device = prec, device
        h = ctypes.c_void_p()
        st = lib.lg_ensemble_create(n, arr, ctypes.byref(h))
        if st:
            _raise(st, lib)
        self._h = h
        self.members = [dict(m) for m in members]

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.lg_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, ncycles: int) -> int:
        st = self._lib.lg_ensemble_step(self._h, int(ncycles))
        if st > 0:
            _raise(st, self._lib)
        return st

    def step_timed(self, ncycles: int) -> tuple[int, float]:
        ms = ctypes.c_double()
        st = self._lib.lg_ensemble_step_timed(self._h, int(ncycles), ctypes.byref(ms))
        if st > 0:
            _raise(st, self._lib)
        return st, ms.value

    def reset(self) -> None:
        st = self._lib.lg_ensemble_reset(self._h)
        if st:
            _raise(st, self._lib)

    def info(self) -> dict:
        e, n, l = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        self._lib.lg_ensemble_info(self._h, ctypes.byref(e), ctypes.byref(n), ctypes.byref(l))
        return {"elements": e.value, "nodes": n.value, "launches": l.value}

    def autotune(self, ncycles: int = 3) -> dict:
        bs = (ctypes.c_int * 4)()
        pers = (ctypes.c_int * 4)()
        st = self._lib.lg_ensemble_autotune(self._h, int(ncycles), bs, pers)
        if st:
            _raise(st, self._lib)
        names = ("k_forces", "k_nodes", "k_kinematics", "k_material")
        return {n: {"block": bs[i], "persistent": bool(pers[i])} for i, n in enumerate(names)}

    def scalar(self, member: int, name: str) -> float:
        v = ctypes.c_double()
        st = self._lib.lg_ensemble_get_scalar(self._h, member, name.encode(), ctypes.byref(v))
        if st:
            _raise(st, self._lib)
        return v.value

    def field(self, member: int, name: str) -> np.ndarray:
        nx = self.members[member]["nx"]
        n = (nx + 1) ** 3 if name in NODE_FIELDS else nx ** 3
        if name == "nodelist":
            n = 8 * nx ** 3
        dt = np.int32 if name in ("nodelist", "regNumList", "elemBC") else np.float64
        out = np.empty(n, dtype=dt)
        st = self._lib.lg_ensemble_get_field(self._h, member, name.encode(), out.ctypes.data, n)
        if st:
            _raise(st, self._lib)
        return out

    def set_field(self, member: int, name: str, values) -> None:
        """Replace a member's double field (lg_ensemble_set_field)."""
        a = np.ascontiguousarray(values, dtype=np.float64)
        st = self._lib.lg_ensemble_set_field(self._h, member, name.encode(), a.ctypes.data, a.size)
        if st:
            _raise(st, self._lib)


HALO_KINDS = {"sbn": 0, "sync_pos_vel": 1, "monoq": 2}


def _dev_ptr(a) -> int:
    """Device address of a torch tensor, or an integer address as is."""
    return a.data_ptr() if hasattr(a, "data_ptr") else int(a)


class HaloPlan:
    """One rank's halo messages of a tp^3 block decomposition (lg_halo_*):
    kind "sbn" (CommSBN: node fields summed), "sync_pos_vel" (CommSyncPosVel:
    node fields copied from higher ranks) or "monoq" (CommMonoQ: element
    fields into ghost elements), in the reference's message order and buffer
    layout (lulesh-comm.cc).  pack / unpack take device arrays (torch
    tensors or addresses) and run on the GPU; the plan itself is host data."""

    def __init__(self, kind, nx: int, tp: int, rank: int, nfields: int):
        lib = load()
        self._lib = lib
        h = ctypes.c_void_p()
        k = HALO_KINDS[kind] if isinstance(kind, str) else int(kind)
        st = lib.lg_halo_plan_create(k, nx, tp, rank, nfields, ctypes.byref(h))
        if st:
            _raise(st, lib)
        self._h = h
        self.kind, self.nx, self.tp, self.rank, self.nfields = k, nx, tp, rank, nfields

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.lg_halo_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> dict:
        i = _HaloInfo()
        st = self._lib.lg_halo_plan_info(self._h, ctypes.byref(i))
        if st:
            _raise(st, self._lib)
        return {k: getattr(i, k) for k, _ in _HaloInfo._fields_}

    def messages(self, side: str) -> list[dict]:
        """side "send" or "recv": [{peer, count, offset}] in order."""
        d = 0 if side == "send" else 1
        n = self.info()["send_messages" if d == 0 else "recv_messages"]
        out = []
        for m in range(n):
            peer, count, off = ctypes.c_int(), ctypes.c_int(), ctypes.c_size_t()
            st = self._lib.lg_halo_plan_message(self._h, d, m, ctypes.byref(peer),
                                                ctypes.byref(count), ctypes.byref(off))
            if st:
                _raise(st, self._lib)
            out.append({"peer": peer.value, "count": count.value, "offset": off.value})
        return out

    def entries(self, side: str) -> dict:
        """The plan's value list: index, bufpos, stride (numpy int32)."""
        d = 0 if side == "send" else 1
        n = self.info()["send_values" if d == 0 else "recv_values"]
        out = {k: np.empty(n, dtype=np.int32) for k in ("index", "bufpos", "stride")}
        st = self._lib.lg_halo_plan_entries(self._h, d, out["index"].ctypes.data,
                                            out["bufpos"].ctypes.data, out["stride"].ctypes.data, n)
        if st:
            _raise(st, self._lib)
        return out

    def _ptrs(self, fields):
        if len(fields) != self.nfields:
            raise ValueError(f"need {self.nfields} fields")
        return (ctypes.c_void_p * self.nfields)(*[_dev_ptr(f) for f in fields])

    def pack(self, fields, send_buf, stream=None) -> None:
        st = self._lib.lg_halo_pack(self._h, self._ptrs(fields), _dev_ptr(send_buf), stream)
        if st:
            _raise(st, self._lib)

    def unpack(self, fields, recv_buf, stream=None) -> None:
        st = self._lib.lg_halo_unpack(self._h, self._ptrs(fields), _dev_ptr(recv_buf), stream)
        if st:
            _raise(st, self._lib)
