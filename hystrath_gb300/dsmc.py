"""Python face of the GB300 dsmcFoam+ hot path, over the C ABI.

``DsmcCloud`` mirrors the calls the dsmcFoam+ driver makes on a dsmcCloud
(applications/solvers/discreteMethods/dsmc/dsmcFoam+/dsmcFoam+.C:92-180):
construct from a case, ``evolve()`` once per time step, ``info()``, field
output.  Every call goes to libhystrath_gb300.so; there is no CPU path, and a
missing library or GPU raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import spec as S

# a migrant between domains: the 64-byte parcel record and the 4-byte cell
# word (DSMC_MIGRANT_BYTES of the C header)
MIGRANT_BYTES = 68

_lib = None


def _load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    from . import build as _build
    path = _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the CUDA library first (python -m hystrath_gb300.build)")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.dsmc_spec_defaults.argtypes = [C.POINTER(S.CaseSpec)]
    L.dsmc_create_from_spec.argtypes = [C.POINTER(S.CaseSpec), C.POINTER(vp)]
    L.dsmc_create.argtypes = [C.c_char_p, C.POINTER(vp)]
    L.dsmc_parse_case.argtypes = [C.c_char_p, C.POINTER(S.CaseSpec)]
    L.dsmc_initialise.argtypes = [vp]
    L.dsmc_evolve.argtypes = [vp, C.c_longlong]
    L.dsmc_run_phases.argtypes = [vp, C.c_uint]
    L.dsmc_evolve_timed.argtypes = [vp, C.c_longlong, C.POINTER(C.c_double)]
    L.dsmc_evolve_profiled.argtypes = [vp, C.c_longlong, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.dsmc_set_selection_audit.argtypes = [vp, C.c_int]
    L.dsmc_set_limits.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_longlong]
    L.dsmc_evolve_kernel_profile.argtypes = [vp, C.c_longlong, C.POINTER(C.c_double), C.c_int,
                                             C.POINTER(C.c_double)]
    L.dsmc_set_particles.argtypes = [vp, C.c_longlong, vp, vp, vp, vp, vp, vp]
    L.dsmc_get_particles.argtypes = [vp, C.c_longlong, C.POINTER(C.c_longlong), vp, vp, vp, vp, vp, vp, vp]
    L.dsmc_get_cell_array.argtypes = [vp, C.c_char_p, vp, C.c_longlong]
    L.dsmc_set_cell_array.argtypes = [vp, C.c_char_p, vp, C.c_longlong]
    L.dsmc_get_field.argtypes = [vp, C.c_char_p, vp, C.c_longlong]
    L.dsmc_get_species_field.argtypes = [vp, C.c_char_p, C.c_uint, vp, C.c_longlong]
    L.dsmc_get_wall_field.argtypes = [vp, C.c_char_p, vp, C.c_longlong]
    L.dsmc_n_boundary_faces.argtypes = [vp]
    L.dsmc_n_boundary_faces.restype = C.c_longlong
    L.dsmc_reset_sampling.argtypes = [vp]
    L.dsmc_write_fields.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_char_p]
    L.dsmc_write_parcels.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_char_p]
    L.dsmc_read_parcels.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_char_p]
    L.dsmc_parse_parcels.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_longlong),
                                     vp, vp, vp, vp, vp, vp]
    L.dsmc_parse_last_error.restype = C.c_char_p
    L.dsmc_counts.argtypes = [vp, C.POINTER(S.Counts)]
    L.dsmc_evolve_counts.argtypes = [vp, C.c_longlong, vp]
    L.dsmc_set_face_tracking.argtypes = [vp, C.c_int]
    L.dsmc_n_faces.argtypes = [vp]
    L.dsmc_n_faces.restype = C.c_longlong
    L.dsmc_get_face_flux.argtypes = [vp, C.c_char_p, C.c_int, vp, C.c_longlong]
    L.dsmc_add_flux_surface.argtypes = [vp, C.POINTER(S.FluxSurface)]
    L.dsmc_n_flux_surfaces.argtypes = [vp]
    L.dsmc_get_flux_surface.argtypes = [vp, C.c_int, C.POINTER(S.FluxSurface), vp]
    L.dsmc_write_flux_surfaces.argtypes = [vp, C.c_char_p, C.c_double]
    L.dsmc_parse_flux_surfaces.argtypes = [C.c_char_p, C.POINTER(S.FluxSurface), C.POINTER(C.c_int)]
    L.dsmc_info.argtypes = [vp, C.POINTER(S.Info)]
    L.dsmc_checkpoint.argtypes = [vp, C.c_char_p]
    L.dsmc_restore.argtypes = [vp, C.c_char_p]
    L.dsmc_phase_times.argtypes = [vp] + [C.POINTER(C.c_double)] * 5
    L.dsmc_last_error.argtypes = [vp]
    L.dsmc_last_error.restype = C.c_char_p
    L.dsmc_last_global_error.restype = C.c_char_p
    L.dsmc_destroy.argtypes = [vp]
    L.dsmc_mlp_create.argtypes = [C.POINTER(vp)]
    L.dsmc_mlp_destroy.argtypes = [vp]
    L.dsmc_mlp_destroy.restype = None
    L.dsmc_mlp_last_error.argtypes = [vp]
    L.dsmc_mlp_last_error.restype = C.c_char_p
    L.dsmc_mlp_set_params.argtypes = [vp, vp, vp]
    L.dsmc_mlp_get_params.argtypes = [vp, vp, vp]
    L.dsmc_mlp_set_data.argtypes = [vp, vp, vp, C.c_longlong]
    L.dsmc_mlp_set_loss.argtypes = [vp, C.c_float]
    L.dsmc_mlp_train.argtypes = [vp, C.c_int, C.c_int, C.c_float, C.c_ulonglong, vp]
    L.dsmc_mlp_grad.argtypes = [vp, vp, vp, C.c_int, vp, vp]
    L.dsmc_mlp_predict.argtypes = [vp, vp, C.c_longlong, vp]
    L.dsmc_set_learned.argtypes = [vp, vp, C.c_int, C.c_float]
    L.dsmc_set_learned_forget.argtypes = [vp, C.c_float]
    L.dsmc_learn_record.argtypes = [vp, C.c_longlong, vp, vp, C.POINTER(C.c_longlong)]
    L.dsmc_set_domain.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    L.dsmc_step_begin.argtypes = [vp, C.POINTER(C.c_longlong)]
    L.dsmc_get_migrants.argtypes = [vp, vp, C.c_longlong]
    L.dsmc_add_migrants.argtypes = [vp, vp, C.c_longlong]
    L.dsmc_step_end.argtypes = [vp]
    _lib = L
    return L


def lib() -> C.CDLL:
    return _load()


class DsmcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[dsmc status {code}] {msg}")
        self.code = code


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def parse_parcels(case_dir: str, time_name: str, cloud_name: str = "dsmc"):
    """The parcels of an OpenFOAM lagrangian cloud directory (no GPU needed)."""
    n = C.c_longlong(0)
    args = (case_dir.encode(), time_name.encode(), cloud_name.encode())
    rc = lib().dsmc_parse_parcels(*args, C.byref(n), None, None, None, None, None, None)
    if rc != 0:
        raise DsmcError(rc, lib().dsmc_parse_last_error().decode())
    out = {"pos": np.empty((n.value, 3)), "U": np.empty((n.value, 3)), "erot": np.empty(n.value),
           "vib": np.empty(n.value, np.int32), "species": np.empty(n.value, np.int32),
           "id": np.empty(n.value, np.uint32)}
    rc = lib().dsmc_parse_parcels(*args, C.byref(n), _p(out["pos"]), _p(out["U"]), _p(out["erot"]),
                                  _p(out["vib"]), _p(out["species"]), _p(out["id"]))
    if rc != 0:
        raise DsmcError(rc, lib().dsmc_parse_last_error().decode())
    return out


def parse_flux_surfaces(case_dir: str) -> list:
    """The dsmcFluxSurface entries of a case (fieldPropertiesDict with their
    zones from topoSetDict), as FluxSurface structs (no GPU needed)."""
    n = C.c_int(0)
    rc = lib().dsmc_parse_flux_surfaces(case_dir.encode(), None, C.byref(n))
    if rc != 0:
        raise DsmcError(rc, lib().dsmc_parse_last_error().decode())
    arr = (S.FluxSurface * max(n.value, 1))()
    rc = lib().dsmc_parse_flux_surfaces(case_dir.encode(), arr, C.byref(n))
    if rc != 0:
        raise DsmcError(rc, lib().dsmc_parse_last_error().decode())
    return [arr[i] for i in range(n.value)]


def parse_case(case_dir: str) -> S.CaseSpec:
    """Resolve an OpenFOAM dsmcFoam+ case directory into a CaseSpec."""
    s = S.CaseSpec()
    rc = lib().dsmc_parse_case(case_dir.encode(), C.byref(s))
    if rc != 0:
        raise DsmcError(rc, lib().dsmc_last_global_error().decode())
    return s


class DsmcCloud:
    """One DSMC cloud resident on the GPU (the dsmcCloud of dsmcFoam+)."""

    def __init__(self, spec: S.CaseSpec | str):
        L = lib()
        h = C.c_void_p()
        if isinstance(spec, str):
            rc = L.dsmc_create(spec.encode(), C.byref(h))
            self.spec = parse_case(spec) if rc == 0 else None
        else:
            rc = L.dsmc_create_from_spec(C.byref(spec), C.byref(h))
            self.spec = spec
        if rc != 0:
            raise DsmcError(rc, L.dsmc_last_global_error().decode())
        self.h = h
        s = self.spec
        self.n_cells = s.n_cells[0] * s.n_cells[1] * s.n_cells[2]

    def close(self):
        if getattr(self, "h", None):
            lib().dsmc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _chk(self, rc):
        if rc != 0:
            raise DsmcError(rc, lib().dsmc_last_error(self.h).decode())

    # dsmcInitialise+ / dsmcMeshFill
    def initialise(self):
        self._chk(lib().dsmc_initialise(self.h))

    # dsmcCloud::evolve, n times
    def evolve(self, n: int = 1):
        self._chk(lib().dsmc_evolve(self.h, n))

    def evolve_timed(self, n: int) -> float:
        """n graph-launched steps; returns the CUDA-event time in ms."""
        ms = C.c_double()
        self._chk(lib().dsmc_evolve_timed(self.h, n, C.byref(ms)))
        return ms.value

    def evolve_profiled(self, n: int):
        """n steps with CUDA events around every phase; returns (total ms,
        dict of summed phase ms)."""
        ph = (C.c_double * 5)()
        tot = C.c_double()
        self._chk(lib().dsmc_evolve_profiled(self.h, n, ph, C.byref(tot)))
        return tot.value, dict(zip(("inflow", "move", "sort", "collide_sample", "end"), list(ph)))

    KERNEL_GROUPS = ("zero", "inflow", "move", "move_slow", "sample", "scan", "scatter_index", "gather", "finish",
                     "learned", "select", "collide_heavy", "collide_light", "pending", "end")

    def evolve_kernel_profile(self, n: int):
        """n steps with CUDA events between the kernel groups; returns (total
        ms, dict of summed group ms in the order of KERNEL_GROUPS)."""
        k = len(self.KERNEL_GROUPS)
        g = (C.c_double * k)()
        tot = C.c_double()
        self._chk(lib().dsmc_evolve_kernel_profile(self.h, n, g, k, C.byref(tot)))
        return tot.value, dict(zip(self.KERNEL_GROUPS, list(g)))

    def set_selection_audit(self, on: bool = True):
        """Per-cell sums of sigma c_R / max and of its part above 1 over the
        candidates (cell_array("selectionAudit")): the expected collision
        shortfall of a maximum below the product."""
        self._chk(lib().dsmc_set_selection_audit(self.h, 1 if on else 0))

    def set_limits(self, max_rejection: int = 0, max_crossings: int = 0, max_cell_parcels: int = 0,
                   capacity: int = 0):
        """Lower the device loop caps, the ordered cell size and the inflow
        capacity (0: default); a cap reached is reported as a status."""
        self._chk(lib().dsmc_set_limits(self.h, int(max_rejection), int(max_crossings), int(max_cell_parcels),
                                        int(capacity)))

    def run_phases(self, phases: int):
        self._chk(lib().dsmc_run_phases(self.h, phases))

    # ------------------------------------------------ spatial decomposition
    def set_domain(self, axis: int, lo: int = 0, hi: int = 0):
        """Own only the cells lo <= index < hi along axis (-1: all cells)."""
        self._chk(lib().dsmc_set_domain(self.h, int(axis), int(lo), int(hi)))

    def step_begin(self) -> int:
        """Inflow and move of a divided cloud; returns the migrant count."""
        n = C.c_longlong(0)
        self._chk(lib().dsmc_step_begin(self.h, C.byref(n)))
        return n.value

    def get_migrants(self, n: int, dst=None):
        """The step's first n migrants: into dst (a device pointer, int) or,
        without dst, as a host array of n x MIGRANT_BYTES bytes."""
        if dst is not None:
            self._chk(lib().dsmc_get_migrants(self.h, C.c_void_p(int(dst)), int(n)))
            return None
        out = np.empty((int(n), MIGRANT_BYTES), dtype=np.uint8)
        if n:
            self._chk(lib().dsmc_get_migrants(self.h, out.ctypes.data_as(C.c_void_p), int(n)))
        return out

    def add_migrants(self, src, n: int = None):
        """Migrants from other domains: a host array of n x MIGRANT_BYTES
        bytes, or a device pointer (int) with n."""
        if isinstance(src, np.ndarray):
            src = np.ascontiguousarray(src, dtype=np.uint8).reshape(-1, MIGRANT_BYTES)
            self._chk(lib().dsmc_add_migrants(self.h, src.ctypes.data_as(C.c_void_p), len(src)))
        else:
            self._chk(lib().dsmc_add_migrants(self.h, C.c_void_p(int(src)), int(n)))

    def step_end(self):
        """Sort, collisions and sampling of a divided cloud's step."""
        self._chk(lib().dsmc_step_end(self.h))

    def phase_times(self):
        v = [C.c_double() for _ in range(5)]
        self._chk(lib().dsmc_phase_times(self.h, *[C.byref(x) for x in v]))
        return dict(zip(("inflow", "move", "sort", "collide_sample", "end"), [x.value for x in v]))

    def set_particles(self, pos, U, erot=None, vib=None, species=None, ids=None):
        n = len(pos)
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        U = np.ascontiguousarray(U, dtype=np.float64)
        erot = None if erot is None else np.ascontiguousarray(erot, dtype=np.float64)
        vib = None if vib is None else np.ascontiguousarray(vib, dtype=np.int32)
        species = None if species is None else np.ascontiguousarray(species, dtype=np.int32)
        ids = np.arange(n, dtype=np.uint32) if ids is None else np.ascontiguousarray(ids, dtype=np.uint32)
        self._chk(lib().dsmc_set_particles(self.h, n, _p(pos), _p(U), _p(erot), _p(vib), _p(species), _p(ids)))

    def n_particles(self) -> int:
        return self.info().n_particles

    def particles(self):
        n = self.n_particles()
        out = dict(pos=np.empty((n, 3)), U=np.empty((n, 3)), erot=np.empty(n),
                   vib=np.empty(n, np.int32), species=np.empty(n, np.int32),
                   id=np.empty(n, np.uint32), cell=np.empty(n, np.int32))
        nn = C.c_longlong()
        self._chk(lib().dsmc_get_particles(self.h, n, C.byref(nn), _p(out["pos"]), _p(out["U"]),
                                           _p(out["erot"]), _p(out["vib"]), _p(out["species"]),
                                           _p(out["id"]), _p(out["cell"])))
        return out

    def cell_array(self, name: str):
        if name in ("count", "start"):
            a = np.empty(self.n_cells, np.int32)
        elif name == "accumulators":
            n_acc = self.spec.n_species * 7 + 2
            a = np.empty(self.n_cells * n_acc)
        elif name == "inflowAccumulator":
            a = np.empty(lib().dsmc_n_boundary_faces(self.h) * self.spec.n_species)
        elif name == "selectionAudit":
            a = np.empty((self.n_cells, 2))
        elif name == "learnedFeatures":
            a = np.empty((self.n_cells, 4), np.float32)
        else:
            a = np.empty(self.n_cells)
        self._chk(lib().dsmc_get_cell_array(self.h, name.encode(), _p(a), a.size))
        return a

    def set_cell_array(self, name: str, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self._chk(lib().dsmc_set_cell_array(self.h, name.encode(), _p(a), a.size))

    def field(self, name: str, species=None):
        """A dsmcVolFields field over all species, or over the species
        indices in ``species`` (the entry's typeIds)."""
        a = np.empty(self.n_cells)
        if species is None:
            self._chk(lib().dsmc_get_field(self.h, name.encode(), _p(a), a.size))
        else:
            mask = 0
            for s in ([species] if isinstance(species, int) else species):
                mask |= 1 << int(s)
            self._chk(lib().dsmc_get_species_field(self.h, name.encode(), mask, _p(a), a.size))
        return a

    def wall_accumulators(self):
        nf = lib().dsmc_n_boundary_faces(self.h)
        a = np.empty((nf, 14))
        self._chk(lib().dsmc_get_wall_field(self.h, b"wallAccumulators", _p(a), a.size))
        return a

    def wall_field(self, name: str):
        nf = lib().dsmc_n_boundary_faces(self.h)
        a = np.empty(nf)
        self._chk(lib().dsmc_get_wall_field(self.h, name.encode(), _p(a), a.size))
        return a

    def reset_sampling(self):
        self._chk(lib().dsmc_reset_sampling(self.h))

    def write_parcels(self, case_dir: str, time_name: str, cloud_name: str = "dsmc"):
        """The cloud as <case_dir>/<time_name>/lagrangian/<cloud_name>/ files."""
        self._chk(lib().dsmc_write_parcels(self.h, case_dir.encode(), time_name.encode(), cloud_name.encode()))

    def read_parcels(self, case_dir: str, time_name: str, cloud_name: str = "dsmc"):
        self._chk(lib().dsmc_read_parcels(self.h, case_dir.encode(), time_name.encode(), cloud_name.encode()))

    def set_face_tracking(self, on: bool = True):
        self._chk(lib().dsmc_set_face_tracking(self.h, 1 if on else 0))

    def face_flux(self, name: str = "parcelIdFlux", species: int = 0):
        n = lib().dsmc_n_faces(self.h)
        out = np.empty(n)
        self._chk(lib().dsmc_get_face_flux(self.h, name.encode(), int(species), _p(out), n))
        return out

    def add_flux_surface(self, zone_name: str, box_min, box_max, direction, species=None,
                         field_name: str = "dsmc") -> int:
        """A dsmcFluxSurface over the faces whose centres lie in the box, for
        the species indices given (all by default); returns its index."""
        f = S.FluxSurface()
        f.zone_name = zone_name.encode()
        f.field_name = field_name.encode()
        for a in range(3):
            f.box_min[a], f.box_max[a], f.direction[a] = box_min[a], box_max[a], direction[a]
        ns = self.spec.n_species
        f.species_mask = sum(1 << m for m in (range(ns) if species is None else species))
        self._chk(lib().dsmc_add_flux_surface(self.h, C.byref(f)))
        return lib().dsmc_n_flux_surfaces(self.h) - 1

    def n_flux_surfaces(self) -> int:
        return lib().dsmc_n_flux_surfaces(self.h)

    def flux_surface(self, i: int = 0) -> dict:
        """faceParticleFlux, faceParticleFlowRate, faceMassFlux,
        faceMassFlowRate, area and averaging_time of surface i, with its
        zone_name and field_name."""
        f = S.FluxSurface()
        out = np.empty(6)
        self._chk(lib().dsmc_get_flux_surface(self.h, int(i), C.byref(f), _p(out)))
        d = dict(zip(S.FLUX_SURFACE_VALUES, out.tolist()))
        d["zone_name"] = f.zone_name.decode()
        d["field_name"] = f.field_name.decode()
        return d

    def write_flux_surfaces(self, case_dir: str, time_value: float):
        """Append this output time to case_dir/fieldMeasurements/*.xy."""
        self._chk(lib().dsmc_write_flux_surfaces(self.h, case_dir.encode(), float(time_value)))

    def write_fields(self, case_dir: str, time_name: str, field_name: str = ""):
        """The averaged fields as OpenFOAM files in case_dir/time_name."""
        self._chk(lib().dsmc_write_fields(self.h, case_dir.encode(), time_name.encode(), field_name.encode()))

    def info(self) -> S.Info:
        i = S.Info()
        self._chk(lib().dsmc_info(self.h, C.byref(i)))
        return i

    def counts(self) -> S.Counts:
        """Particle count and collision counters (no pass over the parcels)."""
        c = S.Counts()
        self._chk(lib().dsmc_counts(self.h, C.byref(c)))
        return c

    def evolve_counts(self, n: int):
        """n steps, each followed by its counters (copied to the host without a
        wait between steps); returns the n Counts."""
        arr = (S.Counts * max(int(n), 1))()
        self._chk(lib().dsmc_evolve_counts(self.h, int(n), arr))
        return [arr[i] for i in range(int(n))]

    def checkpoint(self, path: str):
        self._chk(lib().dsmc_checkpoint(self.h, path.encode()))

    def restore(self, path: str):
        self._chk(lib().dsmc_restore(self.h, path.encode()))

    # learned (sigma_T c_R)max
    def set_learned(self, model: "Mlp | None", every: int = 1, margin: float = 0.0):
        """Attach a trained model (None: the plain running maximum)."""
        self._learned = model   # keep the model alive while attached
        self._chk(lib().dsmc_set_learned(self.h, model.h if model else None, int(every), float(margin)))

    def set_learned_forget(self, forget: float):
        """Fraction of a cell's remembered excess over its predictions kept
        at each prediction (1: kept for good; 0: forgotten)."""
        self._chk(lib().dsmc_set_learned_forget(self.h, float(forget)))

    def learn_record(self, max_rows: int):
        """(features[n,3], log observed maximum[n]) of the cells that had
        candidates in the last step."""
        X = np.empty((max_rows, 3), dtype=np.float32)
        Y = np.empty(max_rows, dtype=np.float32)
        n = C.c_longlong()
        self._chk(lib().dsmc_learn_record(self.h, int(max_rows), _p(X), _p(Y), C.byref(n)))
        return X[:n.value].copy(), Y[:n.value].copy()


NPARAM = 4481


class Mlp:
    """The 3-64-64-1 BF16 perceptron of the learned (sigma_T c_R)max, on the
    GPU: training, gradients and predictions run in the library's kernels."""

    def __init__(self):
        L = lib()
        h = C.c_void_p()
        rc = L.dsmc_mlp_create(C.byref(h))
        if rc != 0:
            raise DsmcError(rc, L.dsmc_mlp_last_error(None).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().dsmc_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _chk(self, rc):
        if rc != 0:
            raise DsmcError(rc, lib().dsmc_mlp_last_error(self.h).decode())

    def set_params(self, params=None, norm=None):
        p = None if params is None else np.ascontiguousarray(params, dtype=np.float32)
        q = None if norm is None else np.ascontiguousarray(norm, dtype=np.float32)
        if p is not None and p.size != NPARAM:
            raise ValueError(f"expected {NPARAM} parameters")
        self._chk(lib().dsmc_mlp_set_params(self.h, _p(p), _p(q)))

    def params(self):
        p = np.empty(NPARAM, dtype=np.float32)
        q = np.empty(8, dtype=np.float32)
        self._chk(lib().dsmc_mlp_get_params(self.h, _p(p), _p(q)))
        return p, q

    def set_loss(self, tau: float = 0.0):
        """0: mean squared error; tau in (0, 1): pinball loss (tau-quantile)."""
        self._chk(lib().dsmc_mlp_set_loss(self.h, float(tau)))

    def set_data(self, X, Y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        self._chk(lib().dsmc_mlp_set_data(self.h, _p(X), _p(Y), len(Y)))

    def train(self, steps: int, batch: int, lr: float = 1e-3, seed: int = 1):
        loss = np.empty(max(steps, 1), dtype=np.float32)
        self._chk(lib().dsmc_mlp_train(self.h, int(steps), int(batch), float(lr), int(seed), _p(loss)))
        return loss[:steps]

    def grad(self, X, Y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        g = np.empty(NPARAM, dtype=np.float32)
        loss = np.empty(1, dtype=np.float32)
        self._chk(lib().dsmc_mlp_grad(self.h, _p(X), _p(Y), len(Y), _p(g), _p(loss)))
        return g, float(loss[0])

    def predict(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        out = np.empty(len(X), dtype=np.float32)
        self._chk(lib().dsmc_mlp_predict(self.h, _p(X), len(X), _p(out)))
        return out
