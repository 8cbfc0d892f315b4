"""Python host binding of libmpm3d_gpu, the GB300 explicit MPM time step.

The module mirrors the reference's step interface: a :class:`MpmStep` object
owns one device context and exposes one method per reference subroutine
(``GridMomentumInitial``, ``ApplyBoundaryConditions``, ``ParticleStressUpdate``,
``GridMomentumUpdate``, ``IntegrateMomentum``, ``ParticlePositionUpdate``,
``GridMomentumMUSL``, ``calcEnergy``, ``UpdateDT``,
``dynamicRelaxationDamping`` -- update_step.f90 / Particle.f90), plus
``step()`` for one whole pass of the MPM3D.f90 time loop.

Errors raise :class:`MpmError` carrying the C status code; there is no CPU
fallback: if the compiled library is missing, importing the binding fails.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_PKG)
LIB_PATH = os.path.join(_ROOT, "_build", "libmpm3d_gpu.so")

STATUS = {
    0: "ok", 1: "bad argument", 2: "out of memory", 3: "parse error", 4: "unsupported",
    5: "CUDA error", 6: "particle out of grid", 7: "non-finite state", 8: "timeout",
    9: "bad state", 10: "I/O error",
}

PRECISION = {"fp64": 0, "strict": 0, "fp64-strict": 0, "native": 1, "fp64-native": 1, "mixed": 2}

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

FLAG_BITS = {"MUSL": 1 << 0, "USL": 1 << 1, "USF": 1 << 2, "GIMP": 1 << 3, "Bspline": 1 << 4,
             "SGMP": 1 << 5, "QuasiLoad": 1 << 6, "QuasiDamp": 1 << 7, "SmoothStress": 1 << 8,
             "UpdateVbyFp": 1 << 9, "TLMPM": 1 << 10, "contact": 1 << 11, "Gravity": 1 << 12,
             "DR_DAMPING": 1 << 13}


class MpmError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code} {STATUS.get(code, '?')}] {message}")
        self.code = code


_lib: Optional[ctypes.CDLL] = None


def library() -> ctypes.CDLL:
    """Load libmpm3d_gpu.so (built in-tree by build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libmpm3d_gpu.so is not built ({LIB_PATH}); run build.py first")
    lib = ctypes.CDLL(LIB_PATH)
    vp, i, i64, d, c = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_char_p
    P = ctypes.POINTER
    sig = {
        "mpm_deck_load": (i, [c, P(vp), c, i]),
        "mpm_deck_parse": (i, [c, P(vp), c, i]),
        "mpm_deck_free": (None, [vp]),
        "mpm_deck_nb_particle": (i64, [vp]),
        "mpm_deck_flags": (ctypes.c_int32, [vp]),
        "mpm_deck_get_particles": (i, [vp, P(d), P(d), P(d), P(d)]),
        "mpm_deck_scalars": (i, [vp, P(d)]),
        "mpm_field_components": (i, [i]),
        "mpm_create": (i, [vp, i, i, P(vp)]),
        "mpm_destroy": (None, [vp]),
        "mpm_last_error": (c, [vp]),
        "mpm_step_phase": (i, [vp, i]),
        "mpm_step": (i, [vp]),
        "mpm_run": (i, [vp, i, i]),
        "mpm_sync": (i, [vp]),
        "mpm_get_scalars": (i, [vp, P(d)]),
        "mpm_download": (i, [vp, i, P(d)]),
        "mpm_upload": (i, [vp, i, P(d)]),
        "mpm_host_alloc": (vp, [i64]),
        "mpm_host_free": (None, [vp]),
        "mpm_host_register": (i, [vp, i64]),
        "mpm_host_unregister": (i, [vp]),
        "mpm_deck_pin": (i, [vp, i]),
        "mpm_nb_particle": (i64, [vp]),
        "mpm_nb_gridnode": (i64, [vp]),
        "mpm_nb_cell": (i64, [vp]),
        "mpm_nb_component": (i, [vp]),
        "mpm_contact_force": (i, [vp, P(d)]),
        "mpm_time_steps": (i, [vp, i, i, P(d)]),
        "mpm_profile_enable": (i, [vp, i]),
        "mpm_kernel_count": (i, [vp]),
        "mpm_kernel_stats": (i, [vp, i, c, i, P(i64), P(d)]),
        "mpm_algorithmic_bytes": (i, [vp, P(d)]),
        "mpm_device_bytes": (i64, [vp]),
        "mpm_energy_reduce_noalloc": (i, [vp, vp, vp, i64, vp, vp]),
        "mpm_fp64_ceiling": (i, [i, i, P(d), P(d)]),
        "mpm_batch_create": (i, [i, P(vp)]),
        "mpm_batch_destroy": (None, [vp]),
        "mpm_batch_add": (i, [vp, vp, i, P(i)]),
        "mpm_batch_remove": (i, [vp, i]),
        "mpm_batch_commit": (i, [vp]),
        "mpm_scene_device_bytes": (i64, [vp]),
        "mpm_batch_device_bytes": (i64, [vp]),
        "mpm_batch_scene_count": (i, [vp]),
        "mpm_batch_run": (i, [vp, i, i]),
        "mpm_batch_run_loop": (i, [vp, i, P(i)]),
        "mpm_serve_launch_shape": (i, [vp, P(i), P(i), P(i)]),
        "mpm_batch_interrupt": (i, [vp]),
        "mpm_batch_sync": (i, [vp]),
        "mpm_batch_time_steps": (i, [vp, i, i, P(d)]),
        "mpm_batch_scene_scalars": (i, [vp, i, P(d)]),
        "mpm_batch_scene_download": (i, [vp, i, i, P(d)]),
        "mpm_batch_last_error": (c, [vp]),
        "mpm_batch_set_blocks": (i, [vp, i, i]),
        "mpm_batch_set_option": (i, [vp, i, i]),
        "mpm_batch_get_option": (i, [vp, i]),
        "mpm_batch_profile_enable": (i, [vp, i]),
        "mpm_batch_kernel_stats": (i, [vp, i, c, i, P(i64), P(d)]),
        "mpm_snapshot_save": (i, [vp, c]),
        "mpm_snapshot_load": (i, [vp, c]),
        "mpm_gather_async": (i, [vp, i, P(i64), P(i), P(i)]),
        "mpm_gather_wait": (i, [vp, P(d)]),
        "mpm_gather": (i, [vp, i, P(i64), P(i), P(i), P(d)]),
        "mpm_batch_scene_gather_async": (i, [vp, i, i, P(i64), P(i), P(i)]),
        "mpm_batch_scene_gather_wait": (i, [vp, P(d)]),
        "mpm_output_open": (i, [vp, c, c, P(vp)]),
        "mpm_output_close": (None, [vp]),
        "mpm_output_curve_count": (i, [vp]),
        "mpm_output_curve_items": (i, [vp, P(i64), P(i), P(i), i]),
        "mpm_output_curve": (i, [vp, P(d), P(d)]),
        "mpm_output_contact": (i, [vp, d, P(d)]),
        "mpm_output_anim": (i, [vp, P(d), vp]),
        "mpm_format_e": (i, [c, i, i, i, d]),
        "mpm_serve_create": (i, [vp, P(vp)]),
        "mpm_serve_destroy": (None, [vp]),
        "mpm_serve_last_error": (c, [vp]),
        "mpm_serve_submit": (i, [vp, vp, i, ctypes.c_uint32, P(i64)]),
        "mpm_serve_wait": (i, [vp, i64, i]),
        "mpm_serve_result": (i, [vp, i64, P(d), P(d)]),
        "mpm_serve_field": (i, [vp, i64, i, P(d)]),
        "mpm_serve_release": (i, [vp, i64]),
        "mpm_serve_stats": (i, [vp, P(d)]),
        "mpm_serve_drain": (i, [vp, i]),
        "mpm_serve_plan": (i, [vp, i, P(i64), P(i), P(i64), i, i64, i64, P(i), P(i), P(i)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class _PinnedBuffer:
    """Owner of a page-locked host allocation (mpm_host_alloc), freed when
    the last array viewing it goes away."""

    def __init__(self, nbytes: int):
        lib = library()
        self.p = lib.mpm_host_alloc(int(nbytes))
        if not self.p:
            raise MpmError(2, lib.mpm_last_error(None).decode(errors="replace"))

    def __del__(self):
        if getattr(self, "p", None):
            library().mpm_host_free(self.p)
            self.p = None


class _PinnedArray(np.ndarray):
    """ndarray in page-locked host memory; its views keep it (and so the
    allocation) alive through their base."""
    _owner = None


def _out_buffer(out: Optional[np.ndarray], n: int) -> np.ndarray:
    if out is None:
        return np.empty(n)
    if out.dtype != np.float64 or out.size != n or not out.flags.c_contiguous:
        raise MpmError(1, f"out must be a contiguous float64 array of {n} values")
    return out.reshape(n)


def fp64_ceiling(device: int = 0, repeats: int = 5) -> dict:
    """Measured FP64 arithmetic ceiling of a device (mpm_fp64_ceiling): FP64
    fused multiply-adds per second (flop/s = 2 x) and FP64 divisions per
    second, each the best of `repeats` timed launches."""
    fma, div = ctypes.c_double(), ctypes.c_double()
    st = library().mpm_fp64_ceiling(int(device), int(repeats), ctypes.byref(fma), ctypes.byref(div))
    if st:
        raise MpmError(st, "FP64 ceiling probe failed")
    return {"dfma_per_s": fma.value, "fp64_tflops": 2.0 * fma.value / 1e12, "ddiv_per_s": div.value}


def pinned_empty(shape, dtype=np.float64) -> np.ndarray:
    """An uninitialised array in page-locked host memory: device copies into
    and out of it run at the link's bandwidth (downloads accept it as out=)."""
    shape = (int(shape),) if np.isscalar(shape) else tuple(int(x) for x in shape)
    dt = np.dtype(dtype)
    n = int(np.prod(shape))
    nbytes = max(1, n * dt.itemsize)
    buf = _PinnedBuffer(nbytes)
    raw = (ctypes.c_char * nbytes).from_address(buf.p)
    a = np.frombuffer(raw, dtype=dt, count=n).reshape(shape).view(_PinnedArray)
    a._owner = buf
    return a


class Deck:
    """A parsed .mpm deck (the reference's input format, FFI.f90 / DataIn.f90)."""

    def __init__(self, handle: int):
        self._h = ctypes.c_void_p(handle)

    @classmethod
    def load(cls, path: str) -> "Deck":
        lib = library()
        h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(256)
        st = lib.mpm_deck_load(path.encode(), ctypes.byref(h), err, 256)
        if st:
            raise MpmError(st, err.value.decode(errors="replace"))
        return cls(h.value)

    @classmethod
    def parse(cls, text: str) -> "Deck":
        lib = library()
        h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(256)
        st = lib.mpm_deck_parse(text.encode(), ctypes.byref(h), err, 256)
        if st:
            raise MpmError(st, err.value.decode(errors="replace"))
        return cls(h.value)

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    @property
    def nb_particle(self) -> int:
        return int(library().mpm_deck_nb_particle(self._h))

    @property
    def flags(self) -> dict:
        f = int(library().mpm_deck_flags(self._h))
        return {k: bool(f & v) for k, v in FLAG_BITS.items()}

    def particles(self) -> dict:
        n = self.nb_particle
        m = np.zeros(n)
        x = np.zeros(3 * n)
        v = np.zeros(3 * n)
        f = np.zeros(3 * n)
        library().mpm_deck_get_particles(self._h, _dptr(m), _dptr(x), _dptr(v), _dptr(f))
        return {"mass": m, "Xp": x.reshape(3, n), "VXp": v.reshape(3, n), "FXp": f.reshape(3, n)}

    def scalars(self) -> dict:
        o = np.zeros(16)
        library().mpm_deck_scalars(self._h, _dptr(o))
        names = ("spx0", "spx1", "spy0", "spy1", "spz0", "spz1", "DCell", "CutOff", "DTScale",
                 "EndTime", "OutTime", "ReportTime", "QuasiLoadTime", "DampFactor", "bq1", "bq2")
        return dict(zip(names, o.tolist()))

    def pin(self, on: bool = True) -> None:
        """Page-lock (or unlock) the deck's particle arrays, from which a
        context is uploaded: the upload then runs at the link's bandwidth."""
        if bool(on) == getattr(self, "_pinned", False):
            return
        st = library().mpm_deck_pin(self._h, int(bool(on)))
        if st:
            raise MpmError(st, library().mpm_last_error(None).decode(errors="replace"))
        self._pinned = bool(on)

    def close(self) -> None:
        if self._h and self._h.value:
            if getattr(self, "_pinned", False):
                library().mpm_deck_pin(self._h, 0)
                self._pinned = False
            library().mpm_deck_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MpmStep:
    """One device context: the explicit step of one scene on one GPU."""

    def __init__(self, deck: Deck, precision: str = "fp64", device: int = -1):
        lib = library()
        h = ctypes.c_void_p()
        st = lib.mpm_create(deck.handle, PRECISION[precision], device, ctypes.byref(h))
        if st:
            raise MpmError(st, lib.mpm_last_error(None).decode(errors="replace"))
        self._h = h
        self.precision = precision
        self.nb_particle = int(lib.mpm_nb_particle(h))
        self.nb_gridnode = int(lib.mpm_nb_gridnode(h))
        self.nb_cell = int(lib.mpm_nb_cell(h))
        self.nb_component = int(lib.mpm_nb_component(h))

    # -- plumbing
    def _check(self, st: int) -> None:
        if st:
            raise MpmError(st, library().mpm_last_error(self._h).decode(errors="replace"))

    def close(self) -> None:
        if self._h and self._h.value:
            library().mpm_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- the reference's subroutines (one phase each)
    def phase(self, name: str) -> None:
        self._check(library().mpm_step_phase(self._h, PHASES[name]))

    def BeginStep(self):
        self.phase("BeginStep")

    def GridMomentumInitial(self):
        self.phase("GridMomentumInitial")

    def ApplyBoundaryConditions(self):
        self.phase("ApplyBoundaryConditions")

    def ParticleStressUpdate(self):
        self.phase("ParticleStressUpdate")

    def GridMomentumUpdate(self):
        self.phase("GridMomentumUpdate")

    def IntegrateMomentum(self):
        self.phase("IntegrateMomentum")

    def ParticlePositionUpdate(self):
        self.phase("ParticlePositionUpdate")

    def GridMomentumMUSL(self):
        self.phase("GridMomentumMUSL")

    def calcEnergy(self):
        self.phase("calcEnergy")

    def UpdateDT(self):
        self.phase("UpdateDT")

    def dynamicRelaxationDamping(self):
        self.phase("dynamicRelaxationDamping")

    def SmoothStressbyGrid(self):
        self.phase("SmoothStressbyGrid")

    def Lagr_NodContact(self):
        self.phase("Lagr_NodContact")

    # -- whole steps
    def step(self) -> None:
        self._check(library().mpm_step(self._h))

    def run(self, nsteps: int, graph: bool = True) -> None:
        self._check(library().mpm_run(self._h, int(nsteps), int(bool(graph))))

    def sync(self) -> None:
        self._check(library().mpm_sync(self._h))

    def time_steps(self, nsteps: int, graph: bool = True) -> float:
        ms = ctypes.c_double()
        self._check(library().mpm_time_steps(self._h, int(nsteps), int(bool(graph)), ctypes.byref(ms)))
        return ms.value

    # -- data
    def scalars(self) -> dict:
        o = np.zeros(16)
        self._check(library().mpm_get_scalars(self._h, _dptr(o)))
        return dict(zip(SCALARS, o.tolist()))

    def download(self, field: str, out: Optional[np.ndarray] = None) -> np.ndarray:
        """A field in host memory; out (contiguous float64 of the field's size,
        e.g. from pinned_empty) receives it in place of a new array."""
        ncomp = COMPONENTS.get(field, 1)
        if field in GRID_FIELDS:
            n = self.nb_gridnode * self.nb_component  # every grid component, component-major
        elif field in CELL_FIELDS:
            n = self.nb_cell
        else:
            n = self.nb_particle
        out = _out_buffer(out, ncomp * n)
        self._check(library().mpm_download(self._h, FIELDS[field], _dptr(out)))
        return out.reshape(ncomp, n) if ncomp > 1 else out.reshape(n)

    def contact_force(self) -> np.ndarray:
        """Total contact force of the last step (Lagr_NodContact's tot_cont_for)."""
        f = np.zeros(3)
        self._check(library().mpm_contact_force(self._h, _dptr(f)))
        return f

    def upload(self, field: str, values: np.ndarray) -> None:
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        self._check(library().mpm_upload(self._h, FIELDS[field], _dptr(a)))

    # -- measurement
    def profile(self, on: bool = True) -> None:
        self._check(library().mpm_profile_enable(self._h, int(bool(on))))

    def kernel_stats(self) -> list:
        lib = library()
        out = []
        for k in range(lib.mpm_kernel_count(self._h)):
            name = ctypes.create_string_buffer(64)
            n = ctypes.c_int64()
            ms = ctypes.c_double()
            self._check(lib.mpm_kernel_stats(self._h, k, name, 64, ctypes.byref(n), ctypes.byref(ms)))
            out.append({"kernel": name.value.decode(), "launches": n.value, "total_ms": ms.value})
        return out

    def algorithmic_bytes(self) -> float:
        b = ctypes.c_double()
        self._check(library().mpm_algorithmic_bytes(self._h, ctypes.byref(b)))
        return b.value

    # -- restart snapshot (every form)
    def save(self, path: str) -> None:
        self._check(library().mpm_snapshot_save(self._h, path.encode()))

    def load(self, path: str) -> None:
        self._check(library().mpm_snapshot_load(self._h, path.encode()))

    # -- a few particles' values (curve output)
    @staticmethod
    def _items(items):
        n = len(items)
        p = (ctypes.c_int64 * max(1, n))(*[int(x[0]) for x in items])
        f = (ctypes.c_int * max(1, n))(*[FIELDS[x[1]] if isinstance(x[1], str) else int(x[1]) for x in items])
        c = (ctypes.c_int * max(1, n))(*[int(x[2]) if len(x) > 2 else 0 for x in items])
        return n, p, f, c

    def gather_async(self, items) -> None:
        """Enqueue a gather of (particle, field[, component]) values behind the
        work on the context's stream."""
        n, p, f, c = self._items(items)
        self._n_gather = n
        self._check(library().mpm_gather_async(self._h, n, p, f, c))

    def gather_wait(self) -> np.ndarray:
        out = np.zeros(max(1, self._n_gather))
        self._check(library().mpm_gather_wait(self._h, _dptr(out)))
        return out[: self._n_gather]

    def gather(self, items) -> np.ndarray:
        self.gather_async(items)
        return self.gather_wait()

    def device_bytes(self) -> int:
        return int(library().mpm_device_bytes(self._h))


BATCH_OPTIONS = {"particle_block": 1, "node_block": 2, "scatter_blocks": 3, "loop_min_steps": 4}


class Batch:
    """Many independent scenes advanced together by the mixed-precision step.

    Scenes are added (with a step count; 0 = until removed) and removed at any
    time; the composition takes effect at the next :meth:`commit` or run.
    Results of a scene do not depend on which other scenes share the batch.
    """

    def __init__(self, device: int = -1):
        lib = library()
        h = ctypes.c_void_p()
        st = lib.mpm_batch_create(device, ctypes.byref(h))
        if st:
            raise MpmError(st, "mpm_batch_create failed")
        self._h = h
        self._scenes = {}

    def _check(self, st: int) -> None:
        if st:
            raise MpmError(st, library().mpm_batch_last_error(self._h).decode(errors="replace"))

    def close(self) -> None:
        if self._h and self._h.value:
            library().mpm_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def scene_bytes(deck: Deck) -> int:
        """Device memory a scene adds to a batch (admission estimate)."""
        return int(library().mpm_scene_device_bytes(deck.handle))

    def add(self, deck: Deck, steps: int = 0) -> int:
        sid = ctypes.c_int()
        self._check(library().mpm_batch_add(self._h, deck.handle, int(steps), ctypes.byref(sid)))
        self._scenes[sid.value] = (deck.nb_particle, deck)
        return sid.value

    def remove(self, scene: int) -> None:
        self._check(library().mpm_batch_remove(self._h, int(scene)))
        self._scenes.pop(scene, None)

    def commit(self) -> None:
        self._check(library().mpm_batch_commit(self._h))

    def run(self, nsteps: int, graph: bool = True) -> None:
        self._check(library().mpm_batch_run(self._h, int(nsteps), int(bool(graph))))

    def sync(self) -> None:
        self._check(library().mpm_batch_sync(self._h))

    def run_loop(self, max_steps: int) -> int:
        """Device-resident run: the device repeats steps until a scene takes
        its last step, max_steps are taken, or :meth:`interrupt` is called;
        returns the steps taken."""
        n = ctypes.c_int()
        self._check(library().mpm_batch_run_loop(self._h, int(max_steps), ctypes.byref(n)))
        return n.value

    def interrupt(self) -> None:
        """Ask a running :meth:`run_loop` (on another thread) to return."""
        self._check(library().mpm_batch_interrupt(self._h))

    def time_steps(self, nsteps: int, graph: bool = True) -> float:
        ms = ctypes.c_double()
        self._check(library().mpm_batch_time_steps(self._h, int(nsteps), int(bool(graph)), ctypes.byref(ms)))
        return ms.value

    def scalars(self, scene: int) -> dict:
        o = np.zeros(16)
        self._check(library().mpm_batch_scene_scalars(self._h, int(scene), _dptr(o)))
        return dict(zip(SCALARS, o.tolist()))

    def download(self, scene: int, field: str, out: Optional[np.ndarray] = None) -> np.ndarray:
        ncomp = COMPONENTS.get(field, 1)
        sc = self.scalars(scene)
        if field in GRID_FIELDS:
            n = int(sc["nb_gridnode"])
        elif field in CELL_FIELDS:
            raise MpmError(1, "cell fields are read per scene through MpmStep")
        else:
            n = int(sc["nb_particle"])
        out = _out_buffer(out, ncomp * n)
        self._check(library().mpm_batch_scene_download(self._h, int(scene), FIELDS[field], _dptr(out)))
        return out.reshape(ncomp, n) if ncomp > 1 else out.reshape(n)

    def set_blocks(self, particle_block: int = 0, node_block: int = 0) -> None:
        self._check(library().mpm_batch_set_blocks(self._h, int(particle_block), int(node_block)))

    def set_option(self, name: str, value: int) -> None:
        self._check(library().mpm_batch_set_option(self._h, BATCH_OPTIONS[name], int(value)))

    def option(self, name: str) -> int:
        return int(library().mpm_batch_get_option(self._h, BATCH_OPTIONS[name]))

    def profile(self, on: bool = True) -> None:
        self._check(library().mpm_batch_profile_enable(self._h, int(bool(on))))

    def kernel_stats(self) -> list:
        lib = library()
        out = []
        for k in range(lib.mpm_kernel_count(None)):
            name = ctypes.create_string_buffer(64)
            n = ctypes.c_int64()
            ms = ctypes.c_double()
            self._check(lib.mpm_batch_kernel_stats(self._h, k, name, 64, ctypes.byref(n), ctypes.byref(ms)))
            out.append({"kernel": name.value.decode(), "launches": n.value, "total_ms": ms.value})
        return out

    def device_bytes(self) -> int:
        return int(library().mpm_batch_device_bytes(self._h))

    @property
    def scene_count(self) -> int:
        return int(library().mpm_batch_scene_count(self._h))


class _ParticleView(ctypes.Structure):
    _fields_ = [(n, ctypes.POINTER(ctypes.c_double)) for n in
                ("xp", "vxp", "fxp", "mass", "seqv", "epeff", "sm", "vol", "ie", "celsius", "cp", "dmg", "sd",
                 "failure", "icell", "spre")]


def format_e(w: int, d: int, x: float) -> str:
    """Fortran Ew.d as gfortran writes it."""
    b = ctypes.create_string_buffer(64)
    library().mpm_format_e(b, 64, int(w), int(d), float(x))
    return b.value.decode()


class Output:
    """The reference's result files (curves, energy / momentum plots,
    Tecplot or ParaView animation) for a deck, written from host arrays."""

    VIEW_FIELDS = {"xp": "Xp", "vxp": "VXp", "fxp": "FXp", "mass": "mass", "seqv": "Seqv", "epeff": "epeff",
                   "sm": "SM", "vol": "VOL", "ie": "ie", "celsius": "celsius_t", "cp": "cp", "dmg": "DMG",
                   "sd": "SD", "failure": "failure", "icell": "icell", "spre": "Spre"}

    def __init__(self, deck: Deck, job: str, plot_dir: Optional[str] = None):
        h = ctypes.c_void_p()
        st = library().mpm_output_open(deck.handle, job.encode(), plot_dir.encode() if plot_dir else None,
                                       ctypes.byref(h))
        if st:
            raise MpmError(st, f"cannot open the result files of {job}")
        self._h = h
        self._deck = deck

    def close(self) -> None:
        if self._h and self._h.value:
            library().mpm_output_close(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def curve_items(self) -> list:
        n = library().mpm_output_curve_items(self._h, None, None, None, 0)
        p = (ctypes.c_int64 * max(1, n))()
        f = (ctypes.c_int * max(1, n))()
        c = (ctypes.c_int * max(1, n))()
        library().mpm_output_curve_items(self._h, p, f, c, n)
        return [(p[k], f[k], c[k]) for k in range(n)]

    def curve(self, scalars, values) -> None:
        s = np.ascontiguousarray(scalars, dtype=np.float64)
        v = np.ascontiguousarray(values if len(values) else [0.0], dtype=np.float64)
        st = library().mpm_output_curve(self._h, _dptr(s), _dptr(v))
        if st:
            raise MpmError(st, "curve output")

    def contact(self, time: float, force) -> None:
        """A row of ContforcPlot.dat (decks with contact)."""
        f = np.ascontiguousarray(force, dtype=np.float64)
        st = library().mpm_output_contact(self._h, float(time), _dptr(f))
        if st:
            raise MpmError(st, "contact output")

    def anim(self, scalars, fields: dict) -> None:
        """fields: name (as in the view: xp, vxp, ..., icell) -> array in deck order."""
        keep = {}
        view = _ParticleView()
        for k in self.VIEW_FIELDS:
            a = fields.get(k)
            if a is not None:
                keep[k] = np.ascontiguousarray(a, dtype=np.float64).ravel()
                setattr(view, k, _dptr(keep[k]))
        s = np.ascontiguousarray(scalars, dtype=np.float64)
        st = library().mpm_output_anim(self._h, _dptr(s), ctypes.byref(view))
        if st:
            raise MpmError(st, "animation output")


class _ServeConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("chunk_steps", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_int64),
                ("max_scenes", ctypes.c_int), ("autotune", ctypes.c_int), ("policy", ctypes.c_int),
                ("max_resident_particles", ctypes.c_int64)]


SERVE_POLICY = {"fifo": 0, "shortest": 1}


SERVE_STATS = ("submitted", "finished", "queued", "resident", "chunks", "particle_steps", "busy_ms",
               "particle_block", "node_block", "peak_resident_bytes")


def serve_plan(np_, steps, bytes_, policy: str = "fifo", budget: int = 0, max_resident_particles: int = 0,
               max_scenes: int = 0, resident=(0, 0, 0)):
    """The serving runtime's admission decision for a queue (host only): returns
    (admitted queue positions in admission order, rejected positions)."""
    n = len(np_)
    cfg = _ServeConfig(-1, 0, int(budget), int(max_scenes), 0, SERVE_POLICY[policy], int(max_resident_particles))
    a_np = (ctypes.c_int64 * max(1, n))(*[int(x) for x in np_])
    a_st = (ctypes.c_int * max(1, n))(*[int(x) for x in steps])
    a_by = (ctypes.c_int64 * max(1, n))(*[int(x) for x in bytes_])
    adm = (ctypes.c_int * max(1, n))()
    rej = (ctypes.c_int * max(1, n))()
    nrej = ctypes.c_int()
    na = library().mpm_serve_plan(ctypes.byref(cfg), n, a_np, a_st, a_by, int(resident[0]), int(resident[1]),
                                  int(resident[2]), adm, rej, ctypes.byref(nrej))
    if na < 0:
        raise MpmError(-na, "mpm_serve_plan")
    return list(adm[:na]), list(rej[:nrej.value])


class Server:
    """Serving runtime: scenes submitted from any thread are admitted into one
    device-resident batch while they fit the device-memory budget, advanced in
    chunks of steps and retired when they reach their step count."""

    def __init__(self, device: int = -1, chunk_steps: int = 25, hbm_budget_bytes: int = 0,
                 max_scenes: int = 0, autotune: bool = False, policy: str = "fifo",
                 max_resident_particles: int = 0):
        lib = library()
        cfg = _ServeConfig(device, chunk_steps, hbm_budget_bytes, max_scenes, int(bool(autotune)),
                           SERVE_POLICY[policy], max_resident_particles)
        h = ctypes.c_void_p()
        st = lib.mpm_serve_create(ctypes.byref(cfg), ctypes.byref(h))
        if st:
            raise MpmError(st, "mpm_serve_create failed")
        self._h = h
        self._np = {}

    def _check(self, st: int) -> None:
        if st:
            raise MpmError(st, library().mpm_serve_last_error(self._h).decode(errors="replace"))

    def close(self) -> None:
        if self._h and self._h.value:
            library().mpm_serve_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, deck: Deck, steps: int, fields=()) -> int:
        mask = 0
        for f in fields:
            mask |= 1 << FIELDS[f]
        t = ctypes.c_int64()
        self._check(library().mpm_serve_submit(self._h, deck.handle, int(steps), mask, ctypes.byref(t)))
        self._np[t.value] = deck.nb_particle
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> bool:
        """True once the ticket finished, False on timeout; raises if it failed."""
        st = library().mpm_serve_wait(self._h, int(ticket), int(timeout_ms))
        if st == 8:
            return False
        self._check(st)
        return True

    def result(self, ticket: int) -> dict:
        sc = np.zeros(16)
        tm = np.zeros(3)
        self._check(library().mpm_serve_result(self._h, int(ticket), _dptr(sc), _dptr(tm)))
        out = dict(zip(SCALARS, sc.tolist()))
        out.update({"queue_ms": tm[0], "resident_ms": tm[1], "latency_ms": tm[2]})
        return out

    def field(self, ticket: int, name: str) -> np.ndarray:
        ncomp = COMPONENTS.get(name, 1)
        n = self._np[ticket]
        out = np.empty(ncomp * n)
        self._check(library().mpm_serve_field(self._h, int(ticket), FIELDS[name], _dptr(out)))
        return out.reshape(ncomp, n) if ncomp > 1 else out

    def release(self, ticket: int) -> None:
        self._check(library().mpm_serve_release(self._h, int(ticket)))
        self._np.pop(ticket, None)

    def stats(self) -> dict:
        o = np.zeros(10)
        self._check(library().mpm_serve_stats(self._h, _dptr(o)))
        return dict(zip(SERVE_STATS, o.tolist()))

    def launch_shape(self) -> Optional[dict]:
        """The autotuned launch shape, None before the tuner has chosen."""
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        st = library().mpm_serve_launch_shape(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        if st == 9:
            return None
        self._check(st)
        return {"particle_block": a.value, "node_block": b.value, "scatter_blocks_per_sm": c.value}

    def drain(self, timeout_ms: int = -1) -> bool:
        st = library().mpm_serve_drain(self._h, int(timeout_ms))
        if st == 8:
            return False
        self._check(st)
        return True


__all__ = ["Deck", "pinned_empty", "MpmStep", "Batch", "Server", "Output", "format_e", "serve_plan", "MpmError", "library", "FIELDS", "PHASES", "PRECISION",
           "LIB_PATH"]
