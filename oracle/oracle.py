"""Python view of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded by the test suite, the smoke check and the benchmark's CPU baseline
leg.  The product never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from hystrath_gb300 import spec as S

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libdsmc_oracle.so")
_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        vp = C.c_void_p
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [C.POINTER(S.CaseSpec), C.c_int]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_set_threads.argtypes = [vp, C.c_int]
        L.oracle_set_step.argtypes = [vp, C.c_longlong]
        L.oracle_reset_sampling.argtypes = [vp]
        for f in ("oracle_initialise",):
            getattr(L, f).argtypes = [vp]
        L.oracle_run_phases.argtypes = [vp, C.c_uint]
        L.oracle_evolve.argtypes = [vp, C.c_longlong]
        L.oracle_set_particles.argtypes = [vp, C.c_longlong, vp, vp, vp, vp, vp, vp, C.c_int]
        L.oracle_n_particles.restype = C.c_longlong
        L.oracle_n_particles.argtypes = [vp]
        L.oracle_get_particles.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp]
        L.oracle_get_cell_array.argtypes = [vp, C.c_char_p, vp]
        L.oracle_set_cell_array.argtypes = [vp, C.c_char_p, vp]
        L.oracle_get_field.argtypes = [vp, C.c_char_p, vp]
        L.oracle_get_wall.argtypes = [vp, vp]
        L.oracle_n_boundary_faces.restype = C.c_longlong
        L.oracle_n_boundary_faces.argtypes = [vp]
        L.oracle_n_accumulators.argtypes = [vp]
        L.oracle_set_face_tracking.argtypes = [vp, C.c_int]
        L.oracle_get_face_flux.argtypes = [vp, vp]
        L.oracle_info.argtypes = [vp, C.POINTER(S.Info)]
        L.oracle_philox.argtypes = [C.POINTER(C.c_uint), C.POINTER(C.c_uint), C.POINTER(C.c_uint)]
        L.oracle_u01_from.restype = C.c_double
        L.oracle_u01_from.argtypes = [C.c_uint, C.c_uint]
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_set_domain.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        L.oracle_step_begin.restype = C.c_longlong
        L.oracle_step_begin.argtypes = [vp]
        L.oracle_get_migrants.argtypes = [vp, vp, C.c_longlong]
        L.oracle_add_migrants.argtypes = [vp, vp, C.c_longlong]
        L.oracle_step_end.argtypes = [vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def philox(ctr, key):
    c = (C.c_uint * 4)(*ctr)
    k = (C.c_uint * 2)(*key)
    o = (C.c_uint * 4)()
    lib().oracle_philox(c, k, o)
    return list(o)


class OracleCloud:
    """CPU replay of one dsmcCloud on the same case spec as the GPU handle."""

    def __init__(self, spec: S.CaseSpec, threads: int = 1):
        self.spec = spec
        self.h = lib().oracle_create(C.byref(spec), threads)
        if not self.h:
            raise RuntimeError(lib().oracle_last_error().decode())
        self.n_cells = spec.n_cells[0] * spec.n_cells[1] * spec.n_cells[2]

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_destroy(self.h)
            self.h = None

    def _chk(self, rc):
        if rc != 0:
            raise RuntimeError(f"oracle status {rc}")

    def set_threads(self, threads: int):
        lib().oracle_set_threads(self.h, int(threads))

    def set_step(self, step: int):
        """The step counter that keys the random streams."""
        lib().oracle_set_step(self.h, int(step))

    def initialise(self):
        self._chk(lib().oracle_initialise(self.h))

    def reset_sampling(self):
        """Restarts the time averages (the library's dsmc_reset_sampling)."""
        lib().oracle_reset_sampling(self.h)

    def run_phases(self, phases):
        self._chk(lib().oracle_run_phases(self.h, phases))

    def evolve(self, n):
        self._chk(lib().oracle_evolve(self.h, n))

    # the spatial decomposition's two half-steps (the library's dsmc_set_domain,
    # dsmc_step_begin, dsmc_get_migrants, dsmc_add_migrants, dsmc_step_end)
    def set_domain(self, axis, lo=0, hi=0):
        self._chk(lib().oracle_set_domain(self.h, int(axis), int(lo), int(hi)))

    def step_begin(self):
        return int(lib().oracle_step_begin(self.h))

    def get_migrants(self, n):
        out = np.empty((int(n), 68), dtype=np.uint8)
        if n:
            self._chk(lib().oracle_get_migrants(self.h, out.ctypes.data_as(C.c_void_p), int(n)))
        return out

    def add_migrants(self, src, n=None):
        src = np.ascontiguousarray(src, dtype=np.uint8).reshape(-1, 68)
        self._chk(lib().oracle_add_migrants(self.h, src.ctypes.data_as(C.c_void_p), len(src)))

    def step_end(self):
        self._chk(lib().oracle_step_end(self.h))

    def set_particles(self, pos, U, erot=None, vib=None, species=None, ids=None, fresh=False):
        n = len(pos)
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        U = np.ascontiguousarray(U, dtype=np.float64)
        erot = None if erot is None else np.ascontiguousarray(erot, dtype=np.float64)
        vib = None if vib is None else np.ascontiguousarray(vib, dtype=np.int32)
        species = None if species is None else np.ascontiguousarray(species, dtype=np.int32)
        ids = np.arange(n, dtype=np.uint32) if ids is None else np.ascontiguousarray(ids, dtype=np.uint32)
        self._chk(lib().oracle_set_particles(self.h, n, _p(pos), _p(U), _p(erot), _p(vib),
                                             _p(species), _p(ids), 1 if fresh else 0))

    def particles(self):
        n = lib().oracle_n_particles(self.h)
        out = dict(pos=np.empty((n, 3)), U=np.empty((n, 3)), erot=np.empty(n),
                   vib=np.empty(n, np.int32), species=np.empty(n, np.int32),
                   id=np.empty(n, np.uint32), cell=np.empty(n, np.int32))
        self._chk(lib().oracle_get_particles(self.h, _p(out["pos"]), _p(out["U"]), _p(out["erot"]),
                                             _p(out["vib"]), _p(out["species"]), _p(out["id"]),
                                             _p(out["cell"])))
        return out

    def cell_array(self, name):
        if name in ("count", "start"):
            a = np.empty(self.n_cells, np.int32)
        elif name == "accumulators":
            a = np.empty(self.n_cells * lib().oracle_n_accumulators(self.h))
        elif name == "inflowAccumulator":
            a = np.empty(lib().oracle_n_boundary_faces(self.h) * self.spec.n_species)
        else:
            a = np.empty(self.n_cells)
        self._chk(lib().oracle_get_cell_array(self.h, name.encode(), _p(a)))
        return a

    def set_cell_array(self, name, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self._chk(lib().oracle_set_cell_array(self.h, name.encode(), _p(a)))

    def field(self, name):
        a = np.empty(self.n_cells)
        self._chk(lib().oracle_get_field(self.h, name.encode(), _p(a)))
        return a

    def wall(self):
        nf = lib().oracle_n_boundary_faces(self.h)
        a = np.empty((nf, 14))
        self._chk(lib().oracle_get_wall(self.h, _p(a)))
        return a

    def set_face_tracking(self, on: bool = True):
        self._chk(lib().oracle_set_face_tracking(self.h, 1 if on else 0))

    def face_flux(self, name: str = "parcelIdFlux", species: int = 0):
        n = list(self.spec.n_cells)
        nf = (n[0] + 1) * n[1] * n[2] + n[0] * (n[1] + 1) * n[2] + n[0] * n[1] * (n[2] + 1)
        a = np.empty((2, self.spec.n_species, nf))
        self._chk(lib().oracle_get_face_flux(self.h, _p(a)))
        return a[{"parcelIdFlux": 0, "massIdFlux": 1}[name], species].copy()

    def info(self) -> S.Info:
        i = S.Info()
        self._chk(lib().oracle_info(self.h, C.byref(i)))
        return i
