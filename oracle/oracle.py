"""ctypes bindings for the CPU checkers (test infrastructure only).

``OracleDomain`` wraps ``build/liblulesh_oracle.so`` (the C restatement of the
reference path, lulesh_oracle.c).  ``RefDomain`` wraps ``_ref/liblulesh_ref.so``
(the unchanged reference sources behind C entry points, ref_driver.cc); it only
exists where the reference sources were available at build time.

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use
this module.  The product package never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "build", "liblulesh_oracle.so")
FAST_LIB = os.path.join(HERE, "build", "liblulesh_oracle_fast.so")
TAPE_LIB = os.path.join(HERE, "build", "liblulesh_oracle_tape.so")
TAPE_LD_LIB = os.path.join(HERE, "build", "liblulesh_oracle_tape_ld.so")
REF_LIB = os.path.join(HERE, "_ref", "liblulesh_ref.so")
REF_BIN = os.path.join(HERE, "_ref", "lulesh_ref")

NODE_FIELDS = ["x", "y", "z", "xd", "yd", "zd", "xdd", "ydd", "zdd", "fx", "fy", "fz",
               "nodalMass"]
ELEM_FIELDS = ["e", "p", "q", "ql", "qq", "v", "volo", "vnew", "delv", "vdov", "arealg",
               "ss", "elemMass"]
SCALARS = ["time", "deltatime", "dtcourant", "dthydro", "cycle"]


def build(ref: bool = True) -> None:
    """Compile the restatement (parity, fast, tape and long double builds) and
    the reference build when its sources exist."""
    targets = ["port", "ld"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


_libs: dict[str, ctypes.CDLL] = {}


def _view(ptr, n: int, dtype) -> np.ndarray:
    """writable numpy view of n values of dtype at a ctypes pointer"""
    addr = ctypes.cast(ptr, ctypes.c_void_p).value
    buf = (ctypes.c_char * (n * np.dtype(dtype).itemsize)).from_address(addr)
    return np.frombuffer(buf, dtype=dtype, count=n)


def _load(path: str) -> ctypes.CDLL:
    if path in _libs:
        return _libs[path]
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} not built; run `make -C {HERE}`")
    lib = ctypes.CDLL(path)
    _libs[path] = lib
    return lib


def _port(lib_path: str = PORT_LIB, real=ctypes.c_double) -> ctypes.CDLL:
    """The restatement's entry points; real: the build's floating type."""
    lib = _load(lib_path)
    R = ctypes.POINTER(real)
    lib.orc_create_ex.restype = ctypes.c_void_p
    lib.orc_create_ex.argtypes = [ctypes.c_int] * 4 + [real] * 2
    lib.orc_destroy.argtypes = [ctypes.c_void_p]
    lib.orc_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.orc_phase.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.orc_field_f64.restype = R
    lib.orc_field_f64.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_size_t)]
    lib.orc_field_i32.restype = ctypes.POINTER(ctypes.c_int)
    lib.orc_field_i32.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_size_t)]
    lib.orc_get_scalar.restype = real
    lib.orc_get_scalar.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    lib.orc_set_scalar.argtypes = [ctypes.c_void_p, ctypes.c_char_p, real]
    lib.orc_region_rep.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.orc_dt_freeze.argtypes = [ctypes.c_void_p, R, ctypes.c_int]
    lib.orc_dt_record.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.orc_dt_recorded.restype = R
    lib.orc_dt_recorded.argtypes = [ctypes.c_void_p]
    lib.orc_tape_record.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.orc_tape_replay.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.orc_tape_stop.argtypes = [ctypes.c_void_p]
    return lib


class OracleDomain:
    """The C restatement: build the Sedov problem and advance it on the CPU."""

    def __init__(self, nx: int, numReg: int = 11, balance: int = 1, cost: int = 1,
                 hgcoef: float = 3.0, einit_factor: float = 1.0, fast: bool = False,
                 tape: bool = False, extended: bool = False):
        """fast: the default-contraction build (timing); tape: the parity
        build with the decision tape (tape_record / tape_replay); extended:
        the tape build in long double (fields are np.longdouble)."""
        self._real = ctypes.c_longdouble if extended else ctypes.c_double
        self._dtype = np.longdouble if extended else np.float64
        self._lib = _port(TAPE_LD_LIB if extended else TAPE_LIB if tape else
                          FAST_LIB if fast else PORT_LIB, self._real)
        self._h = self._lib.orc_create_ex(nx, numReg, balance, cost, hgcoef, einit_factor)
        if not self._h:
            raise ValueError("invalid problem size")
        self.nx = nx

    def close(self) -> None:
        if self._h:
            self._lib.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, ncycles: int) -> int:
        """Run up to ncycles cycles; returns 0, -1 (VolumeError) or -2 (QStopError)."""
        return self._lib.orc_step(self._h, ncycles)

    def phase(self, which: int) -> int:
        return self._lib.orc_phase(self._h, which)

    def field(self, name: str) -> np.ndarray:
        n = ctypes.c_size_t()
        p = self._lib.orc_field_f64(self._h, name.encode(), ctypes.byref(n))
        if p:
            return _view(p, n.value, self._dtype)
        p = self._lib.orc_field_i32(self._h, name.encode(), ctypes.byref(n))
        if p:
            return np.ctypeslib.as_array(p, shape=(n.value,))
        raise KeyError(name)

    def scalar(self, name: str) -> float:
        return self._lib.orc_get_scalar(self._h, name.encode())

    def set_scalar(self, name: str, value: float) -> None:
        if self._lib.orc_set_scalar(self._h, name.encode(), float(value)):
            raise KeyError(name)

    def region_rep(self, r: int) -> int:
        return self._lib.orc_region_rep(self._h, r)

    def dt_freeze(self, dts) -> None:
        a = np.ascontiguousarray(dts, dtype=self._dtype)
        self._lib.orc_dt_freeze(self._h, a.ctypes.data_as(ctypes.POINTER(self._real)), a.size)

    def dt_record(self, capacity: int) -> None:
        self._lib.orc_dt_record(self._h, capacity)

    def dt_recorded(self, n: int) -> np.ndarray:
        return _view(self._lib.orc_dt_recorded(self._h), n, self._dtype).copy()

    def tape_record(self, ncycles: int) -> None:
        """Record the branch outcomes of the next ncycles cycles."""
        if self._lib.orc_tape_record(self._h, ncycles):
            raise RuntimeError("decision tape unavailable (build with tape=True)")

    def tape_replay(self, src: "OracleDomain") -> None:
        """Replay src's recorded branches in this domain's next cycles; src
        must stay alive while this domain steps."""
        if self._lib.orc_tape_replay(self._h, src._h):
            raise RuntimeError("no recorded tape in src, or a different mesh")
        self._tape_src = src

    def tape_stop(self) -> None:
        self._lib.orc_tape_stop(self._h)
        self._tape_src = None

    def state(self) -> dict:
        out = {f: self.field(f).copy() for f in NODE_FIELDS + ELEM_FIELDS}
        for s in SCALARS:
            out[s] = self.scalar(s)
        return out


def _ref(path: str = REF_LIB) -> ctypes.CDLL:
    lib = _load(path)
    lib.ref_create.restype = ctypes.c_void_p
    lib.ref_create.argtypes = [ctypes.c_int] * 4 + [ctypes.c_double] * 2
    lib.ref_destroy.argtypes = [ctypes.c_void_p]
    lib.ref_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.ref_step_frozen.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    lib.ref_field_f64.restype = ctypes.POINTER(ctypes.c_double)
    lib.ref_field_f64.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_size_t)]
    lib.ref_field_i32.restype = ctypes.POINTER(ctypes.c_int)
    lib.ref_field_i32.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_size_t)]
    lib.ref_get_scalar.restype = ctypes.c_double
    lib.ref_get_scalar.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    lib.ref_set_e.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_size_t]
    lib.ref_report.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int]
    return lib


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


class RefDomain:
    """The reference's own Domain and timestep (unchanged sources)."""

    def __init__(self, nx: int, numReg: int = 11, balance: int = 1, cost: int = 1,
                 hgcoef: float = 3.0, einit_factor: float = 1.0, lib_path: str = REF_LIB):
        self._lib = _ref(lib_path)
        self._h = self._lib.ref_create(nx, numReg, balance, cost, hgcoef, einit_factor)
        self.nx = nx

    def close(self) -> None:
        if self._h:
            self._lib.ref_destroy(self._h)
            self._h = None

    def step(self, ncycles: int) -> int:
        return self._lib.ref_step(self._h, ncycles)

    def step_frozen(self, dts) -> int:
        """len(dts) cycles, cycle c advancing by dts[c]."""
        a = np.ascontiguousarray(dts, dtype=np.float64)
        return self._lib.ref_step_frozen(self._h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                         a.size)

    def field(self, name: str) -> np.ndarray:
        n = ctypes.c_size_t()
        p = self._lib.ref_field_f64(self._h, name.encode(), ctypes.byref(n))
        if p:
            return np.ctypeslib.as_array(p, shape=(n.value,))
        p = self._lib.ref_field_i32(self._h, name.encode(), ctypes.byref(n))
        if p:
            return np.ctypeslib.as_array(p, shape=(n.value,))
        raise KeyError(name)

    def scalar(self, name: str) -> float:
        return self._lib.ref_get_scalar(self._h, name.encode())

    def set_e(self, e: np.ndarray) -> None:
        e = np.ascontiguousarray(e, dtype=np.float64)
        self._lib.ref_set_e(self._h, e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), e.size)

    def state(self) -> dict:
        out = {f: self.field(f).copy() for f in NODE_FIELDS + ELEM_FIELDS}
        for s in SCALARS:
            out[s] = self.scalar(s)
        return out
