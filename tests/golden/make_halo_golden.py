"""Generate the halo fixture from the reference's own exchange.

Run where the reference sources exist (they are read, never copied):
    make -C oracle ref && python tests/golden/make_halo_golden.py

Writes halo_tp2_nx3.npz next to this script: for each call site of the
reference's halo exchange (forces and nodal mass through CommSBN, positions
and velocities through CommSyncPosVel, velocity gradients through CommMonoQ;
lulesh.cc:1109-1133, 2723-2729, 2621-2642, 1963-1985), seeded random fields
on the 8 ranks of a 2x2x2 decomposition of cubes of 3 elements, and the
fields after the reference's CommRecv / CommSend / unpack ran for every rank
in one process (oracle/halo_ref_driver.cc over oracle/mpi_stub/mpi.h).
Keys: <site>_in_r<rank>_f<field>, <site>_out_r<rank>_f<field>.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(ROOT, "oracle", "_ref", "liblulesh_halo_ref.so")
SITES = {"forces": (0, ["fx", "fy", "fz"]), "pos_vel": (1, ["x", "y", "z", "xd", "yd", "zd"]),
         "monoq": (2, ["delv_xi", "delv_eta", "delv_zeta"]), "nodal_mass": (3, ["nodalMass"])}
TP, NX = 2, 3


def main() -> None:
    if not os.path.exists(LIB):
        sys.exit(f"{LIB} missing: run `make -C oracle ref` where the reference sources exist")
    lib = ctypes.CDLL(LIB)
    lib.hr_create.argtypes = [ctypes.c_int, ctypes.c_int]
    lib.hr_field.restype = ctypes.POINTER(ctypes.c_double)
    lib.hr_field.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.POINTER(ctypes.c_size_t)]
    lib.hr_exchange.argtypes = [ctypes.c_int]
    out = {"tp": np.int32(TP), "nx": np.int32(NX)}
    for site, (kind, names) in SITES.items():
        nr = lib.hr_create(TP, NX)
        if site == "monoq":
            lib.hr_alloc_gradients()
        rng = np.random.default_rng(2024 + kind)
        views = {}
        for r in range(nr):
            for f, name in enumerate(names):
                n = ctypes.c_size_t()
                a = np.ctypeslib.as_array(lib.hr_field(r, name.encode(), ctypes.byref(n)),
                                          shape=(n.value,))
                a[:] = rng.standard_normal(n.value)
                out[f"{site}_in_r{r}_f{f}"] = a.copy()
                views[(r, f)] = a
        lib.hr_exchange(kind)
        for (r, f), a in views.items():
            out[f"{site}_out_r{r}_f{f}"] = a.copy()
    lib.hr_destroy()
    np.savez_compressed(os.path.join(HERE, f"halo_tp{TP}_nx{NX}.npz"), **out)
    print("wrote", os.path.join(HERE, f"halo_tp{TP}_nx{NX}.npz"))


if __name__ == "__main__":
    main()
