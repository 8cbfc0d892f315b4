"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle is the checker of the GPU library; only tests, the smoke check and
the CPU-baseline leg of bench.py load it. It shares the deck reader of the
product (include/mpm_deck.h) but derives the set-up and runs the step with
its own sequential restatement of the reference (mpm_oracle.c).

Parity status: unpinned against the reference binary (no Fortran compiler is
available); pinned end-to-end by the published Cook-membrane tip displacement.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmpm_oracle.so")
CLI_PATH = os.path.join(HERE, "_build", "mpm3d_oracle")

FIELDS = {
    "Xp": 1, "XX": 2, "VXp": 3, "FXp": 4, "XN": 5, "XXN": 6, "VOL": 7, "VOL0": 8, "sig_y": 9,
    "SM": 10, "Seqv": 11, "SD": 12, "Fp": 13, "epeff": 14, "celsius_t": 15, "DMG": 16, "LT": 17,
    "ie": 18, "mass": 19, "cp": 20, "q": 21, "failure": 22, "icell": 23, "centericell": 24,
    "inode": 25, "Spre": 26, "PK": 27, "Mg": 40, "PXg": 41, "FXg": 42, "Cmg": 50, "Cpxg": 51,
}
COMPONENTS = {"Xp": 3, "XX": 3, "VXp": 3, "FXp": 3, "XN": 3, "XXN": 3, "SD": 6, "Fp": 9, "PK": 9,
              "PXg": 3, "FXg": 3, "Cpxg": 3}
GRID_FIELDS = {"Mg", "PXg", "FXg"}
CELL_FIELDS = {"Cmg", "Cpxg"}
PHASES = {
    "GridMomentumInitial": 1, "ApplyBoundaryConditions": 2, "ParticleStressUpdate": 3,
    "GridMomentumUpdate": 4, "IntegrateMomentum": 5, "ParticlePositionUpdate": 6,
    "GridMomentumMUSL": 7, "calcEnergy": 8, "UpdateDT": 9, "dynamicRelaxationDamping": 10,
    "BeginStep": 11, "SmoothStressbyGrid": 12, "Lagr_NodContact": 13,
}
SCALARS = ("istep", "CurrentTime", "DT", "EngKinetic", "EngInternal", "Momentum_x",
           "Momentum_y", "Momentum_z", "EngKinetic_prev", "nb_gridnode", "nb_particle",
           "CutOff", "DCell", "active_nodes", "status", "reserved")

_lib = None


def library() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"oracle not built ({LIB_PATH})")
        lib = ctypes.CDLL(LIB_PATH)
        vp, i, i64, d, c = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_char_p
        P = ctypes.POINTER
        for name, res, args in [
            ("mpm_deck_load", i, [c, P(vp), c, i]),
            ("mpm_deck_parse", i, [c, P(vp), c, i]),
            ("mpm_deck_free", None, [vp]),
            ("orc_create", i, [vp, i, P(vp)]),
            ("orc_destroy", None, [vp]),
            ("orc_error", c, [vp]),
            ("orc_phase", i, [vp, i]),
            ("orc_step", i, [vp]),
            ("orc_run", i, [vp, i]),
            ("orc_get_scalars", i, [vp, P(d)]),
            ("orc_download", i, [vp, i, P(d)]),
            ("orc_upload", i, [vp, i, P(d)]),
            ("orc_nb_particle", i64, [vp]),
            ("orc_nb_gridnode", i64, [vp]),
            ("orc_nb_cell", i64, [vp]),
            ("orc_nb_component", i, [vp]),
            ("orc_contact_force", i, [vp, P(d)]),
        ]:
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """Sequential CPU restatement of the step for one deck."""

    def __init__(self, deck_text: str = None, deck_path: str = None, libm: str = "system"):
        lib = library()
        d = ctypes.c_void_p()
        err = ctypes.create_string_buffer(256)
        if deck_path is not None:
            st = lib.mpm_deck_load(deck_path.encode(), ctypes.byref(d), err, 256)
        else:
            st = lib.mpm_deck_parse(deck_text.encode(), ctypes.byref(d), err, 256)
        if st:
            raise RuntimeError(f"deck error {st}: {err.value.decode()}")
        h = ctypes.c_void_p()
        st = lib.orc_create(d, 1 if libm == "project" else 0, ctypes.byref(h))
        lib.mpm_deck_free(d)
        if st:
            msg = lib.orc_error(h).decode() if h.value else ""
            if h.value:
                lib.orc_destroy(h)
            raise RuntimeError(f"oracle error {st}: {msg}")
        self._h = h
        self.nb_particle = int(lib.orc_nb_particle(h))
        self.nb_gridnode = int(lib.orc_nb_gridnode(h))
        self.nb_cell = int(lib.orc_nb_cell(h))
        self.nb_component = int(lib.orc_nb_component(h))

    def close(self):
        if self._h and self._h.value:
            library().orc_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st:
            raise RuntimeError(f"oracle error {st}: {library().orc_error(self._h).decode()}")

    def phase(self, name: str):
        self._check(library().orc_phase(self._h, PHASES[name]))

    def step(self):
        self._check(library().orc_step(self._h))

    def run(self, n: int):
        self._check(library().orc_run(self._h, int(n)))

    def scalars(self) -> dict:
        o = np.zeros(16)
        self._check(library().orc_get_scalars(self._h, _dptr(o)))
        return dict(zip(SCALARS, o.tolist()))

    def download(self, field: str) -> np.ndarray:
        ncomp = COMPONENTS.get(field, 1)
        n = (self.nb_gridnode * self.nb_component if field in GRID_FIELDS
             else (self.nb_cell if field in CELL_FIELDS else self.nb_particle))
        out = np.zeros(ncomp * n)
        self._check(library().orc_download(self._h, FIELDS[field], _dptr(out)))
        return out.reshape(ncomp, n) if ncomp > 1 else out

    def contact_force(self) -> np.ndarray:
        """Total contact force of the last step (Lagr_NodContact's tot_cont_for)."""
        f = np.zeros(3)
        self._check(library().orc_contact_force(self._h, _dptr(f)))
        return f

    def upload(self, field: str, values):
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        self._check(library().orc_upload(self._h, FIELDS[field], _dptr(a)))
