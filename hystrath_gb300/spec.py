"""ctypes mirror of ``dsmc_case_spec`` and the named workloads.

The structures here are byte-for-byte the C structs of
``include/hystrath_gb300.h``.  ``make_box_case`` builds the Cartesian cases
the path is measured on; ``dsmc_parse_case`` (C side) builds the same struct
from an OpenFOAM case directory.

Species constants follow ``moleculeProperties`` entries of the reference's
tutorials (e.g. run/hyStrath/dsmcFoam+/heatBath-5species/constant/dsmcProperties
for N2, hypersonicCorner/constant/dsmcProperties for Ar).
"""
from __future__ import annotations

import ctypes as C
import math

MAX_SPECIES = 8
MAX_PATCHES = 16
MAX_OBSTACLES = 8
NAME_LEN = 64

# status codes
OK = 0
ERR_IO, ERR_PARSE, ERR_UNKNOWN_MODEL, ERR_INVALID, ERR_CUDA, ERR_DEVICE, ERR_CAPACITY, ERR_NO_DEVICE = range(1, 9)

PATCH_WALL, PATCH_PATCH, PATCH_SYMMETRY, PATCH_CYCLIC, PATCH_EMPTY = range(5)
BC_NONE, BC_SPECULAR, BC_DIFFUSE, BC_DELETION = range(4)
COLL_VHS, COLL_LB_VHS, COLL_VSS, COLL_LB_VSS = range(4)
SEL_NTC, SEL_SBT = 0, 1

PHASE_INFLOW, PHASE_MOVE, PHASE_SORT, PHASE_COLLIDE, PHASE_SAMPLE = 1, 2, 4, 8, 16
PHASE_ALL = 31

KB = 1.3806504e-23


class Species(C.Structure):
    _fields_ = [
        ("name", C.c_char * NAME_LEN),
        ("mass", C.c_double),
        ("diameter", C.c_double),
        ("omega", C.c_double),
        ("alpha", C.c_double),
        ("rotational_dof", C.c_double),
        ("n_vib_modes", C.c_int),
        ("theta_v", C.c_double),
        ("theta_d", C.c_double),
        ("zref", C.c_double),
        ("tref_zv", C.c_double),
    ]


class Patch(C.Structure):
    _fields_ = [
        ("name", C.c_char * NAME_LEN),
        ("type", C.c_int),
        ("model", C.c_int),
        ("wall_temperature", C.c_double),
        ("wall_velocity", C.c_double * 3),
        ("inflow", C.c_int),
        ("inflow_number_density", C.c_double * MAX_SPECIES),
        ("inflow_t_tra", C.c_double),
        ("inflow_t_rot", C.c_double),
        ("inflow_t_vib", C.c_double),
        ("inflow_velocity", C.c_double * 3),
    ]


class Obstacle(C.Structure):
    _fields_ = [
        ("lo", C.c_int * 3),
        ("hi", C.c_int * 3),
        ("patch", C.c_int * 6),
    ]


class CaseSpec(C.Structure):
    _fields_ = [
        ("n_cells", C.c_int * 3),
        ("origin", C.c_double * 3),
        ("cell_size", C.c_double * 3),
        ("side_patch", C.c_int * 6),
        ("face_patch", C.POINTER(C.c_int) * 6),
        ("n_obstacles", C.c_int),
        ("obstacles", Obstacle * MAX_OBSTACLES),
        ("n_patches", C.c_int),
        ("patches", Patch * MAX_PATCHES),
        ("n_species", C.c_int),
        ("species", Species * MAX_SPECIES),
        ("n_equivalent_particles", C.c_double),
        ("binary_collision_model", C.c_int),
        ("partner_selection_model", C.c_int),
        ("tref", C.c_double),
        ("zrot", C.c_double),
        ("fixed_zv", C.c_double),
        ("inv_zv_formulation", C.c_int),
        ("delta_t", C.c_double),
        ("seed", C.c_ulonglong),
        ("measure_mean_free_path", C.c_int),
        ("mfp_tref", C.c_double),
        ("init_number_density", C.c_double * MAX_SPECIES),
        ("init_t_tra", C.c_double),
        ("init_t_rot", C.c_double),
        ("init_t_vib", C.c_double),
        ("init_velocity", C.c_double * 3),
        ("init_t_tra_xyz", C.c_double * 3),
        ("max_particles", C.c_longlong),
        ("node_coords", C.POINTER(C.c_double) * 3),
        ("write_interval_steps", C.c_longlong),
        ("reset_at_output", C.c_int),
        ("reset_at_output_until_time", C.c_double),
        ("measure_errors", C.c_int),
        ("measure_heat_flux_shear_stress", C.c_int),
    ]


class Counts(C.Structure):
    _fields_ = [
        ("n_particles", C.c_longlong),
        ("step", C.c_longlong),
        ("collisions_last_step", C.c_longlong),
        ("candidates_last_step", C.c_longlong),
        ("collisions_total", C.c_longlong),
        ("candidates_total", C.c_longlong),
    ]


class FluxSurface(C.Structure):
    """dsmc_flux_surface: a dsmcFluxSurface over the faces whose centres lie
    in [box_min, box_max] (topoSet boxToFace)."""
    _fields_ = [
        ("field_name", C.c_char * NAME_LEN),
        ("zone_name", C.c_char * NAME_LEN),
        ("box_min", C.c_double * 3),
        ("box_max", C.c_double * 3),
        ("direction", C.c_double * 3),
        ("species_mask", C.c_uint),
    ]


FLUX_SURFACE_VALUES = ("faceParticleFlux", "faceParticleFlowRate", "faceMassFlux", "faceMassFlowRate",
                       "area", "averaging_time")


class Info(C.Structure):
    _fields_ = [
        ("n_particles", C.c_longlong),
        ("step", C.c_longlong),
        ("linear_ke", C.c_double),
        ("rotational_e", C.c_double),
        ("vibrational_e", C.c_double),
        ("momentum", C.c_double * 3),
        ("collisions_last_step", C.c_longlong),
        ("candidates_last_step", C.c_longlong),
        ("collisions_total", C.c_longlong),
        ("candidates_total", C.c_longlong),
        ("wall_hits_last_step", C.c_longlong),
        ("inserted_last_step", C.c_longlong),
        ("deleted_last_step", C.c_longlong),
        ("sample_steps", C.c_longlong),
    ]


# moleculeProperties of the tutorial species used by the workloads
AR = dict(name="Ar", mass=6.63e-26, diameter=4.17e-10, omega=0.81, alpha=1.0,
          rotational_dof=0.0, n_vib_modes=0)
N2 = dict(name="N2", mass=4.65e-26, diameter=4.17e-10, omega=0.74, alpha=1.36,
          rotational_dof=2.0, n_vib_modes=1, theta_v=3371.0, theta_d=113500.0,
          zref=52560.0, tref_zv=3371.0)


def set_species(spec: CaseSpec, i: int, d: dict) -> None:
    s = spec.species[i]
    for k, v in d.items():
        if k == "name":
            s.name = v.encode()
        else:
            setattr(s, k, v)


def spec_defaults() -> CaseSpec:
    """Reference defaults: Tref 273 (VariableHardSphere.C:62), Zrot 5,
    variable Zv with formulation 2 (LarsenBorgnakkeVariableHardSphere.C:58-80),
    mfpReferenceTemperature 273 (dsmcVolFields.C:1044)."""
    s = CaseSpec()
    s.tref = 273.0
    s.zrot = 5.0
    s.fixed_zv = 0.0
    s.inv_zv_formulation = 2
    s.mfp_tref = 273.0
    s.measure_mean_free_path = 1
    s.binary_collision_model = COLL_VHS
    s.partner_selection_model = SEL_NTC
    return s


def make_box_case(n_cells, cell_size, species, fn, dt, seed=0, n_density=1e20,
                  t_tra=300.0, t_rot=0.0, t_vib=0.0, velocity=(0.0, 0.0, 0.0),
                  t_xyz=(0.0, 0.0, 0.0), side_model=BC_SPECULAR, side_type=PATCH_WALL,
                  collision=COLL_VHS, max_particles=0) -> CaseSpec:
    """A closed Cartesian box of one species with the same model on all six sides."""
    s = spec_defaults()
    for a in range(3):
        s.n_cells[a] = int(n_cells[a])
        s.origin[a] = 0.0
        s.cell_size[a] = float(cell_size if not hasattr(cell_size, "__len__") else cell_size[a])
    s.n_patches = 1
    p = s.patches[0]
    p.name = b"walls"
    p.type = side_type
    p.model = side_model
    p.wall_temperature = t_tra
    for q in range(6):
        s.side_patch[q] = 0
    s.n_species = 1
    set_species(s, 0, species)
    s.n_equivalent_particles = fn
    s.binary_collision_model = collision
    s.delta_t = dt
    s.seed = seed
    s.init_number_density[0] = n_density
    s.init_t_tra = t_tra
    s.init_t_rot = t_rot
    s.init_t_vib = t_vib
    for a in range(3):
        s.init_velocity[a] = velocity[a]
        s.init_t_tra_xyz[a] = t_xyz[a]
    s.max_particles = max_particles
    return s


def config0(seed=0, cyclic=False) -> CaseSpec:
    """Ar VHS, 10^3 cells of 1 mm, n=1e20, 20 parcels per cell (FN=5e9),
    bi-Maxwellian Tx=600 K, Ty=Tz=150 K, dt=1e-6 s, all faces specular
    (or cyclic)."""
    s = make_box_case((10, 10, 10), 1e-3, AR, fn=5e9, dt=1e-6, seed=seed, n_density=1e20,
                      t_tra=300.0, t_xyz=(600.0, 150.0, 150.0),
                      side_model=BC_SPECULAR,
                      side_type=PATCH_CYCLIC if cyclic else PATCH_WALL)
    return s


def config1(seed=0, n=64) -> CaseSpec:
    """N2 Larsen-Borgnakke heat bath: n^3 cells of 1 mm, n=1e20, 50 parcels per
    cell (FN=2e9), T_tr=10000 K, T_rot=T_vib=300 K, dt=2e-7 s, specular walls."""
    return make_box_case((n, n, n), 1e-3, N2, fn=2e9, dt=2e-7, seed=seed, n_density=1e20,
                         t_tra=10000.0, t_rot=300.0, t_vib=300.0,
                         side_model=BC_SPECULAR, collision=COLL_LB_VHS)


def mach10_speed(t=200.0, m=N2["mass"], gamma=1.4) -> float:
    return 10.0 * math.sqrt(gamma * KB * t / m)


def config2(seed=0, scale=1) -> CaseSpec:
    """Mach 10 N2 past a diffuse 300 K cube: (256,128,128)/scale cells of
    0.5 mm*scale, n=1e21, ~20 parcels per cell, freestream inflow at x=0,
    deletion at x=max, specular sides, cube of 32/scale cells at x 48-80."""
    nx, ny, nz = 256 // scale, 128 // scale, 128 // scale
    h = 5e-4 * scale
    s = spec_defaults()
    for a, nn in enumerate((nx, ny, nz)):
        s.n_cells[a] = nn
        s.origin[a] = 0.0
        s.cell_size[a] = h
    U = mach10_speed()
    s.n_patches = 4
    names = [b"inlet", b"outlet", b"sides", b"cube"]
    for i, nm in enumerate(names):
        s.patches[i].name = nm
    s.patches[0].type = PATCH_PATCH
    s.patches[0].model = BC_DELETION
    s.patches[0].inflow = 1
    s.patches[0].inflow_number_density[0] = 1e21
    s.patches[0].inflow_t_tra = 200.0
    s.patches[0].inflow_t_rot = 200.0
    s.patches[0].inflow_t_vib = 200.0
    s.patches[0].inflow_velocity[0] = U
    s.patches[1].type = PATCH_PATCH
    s.patches[1].model = BC_DELETION
    s.patches[2].type = PATCH_WALL
    s.patches[2].model = BC_SPECULAR
    s.patches[3].type = PATCH_WALL
    s.patches[3].model = BC_DIFFUSE
    s.patches[3].wall_temperature = 300.0
    s.side_patch[0] = 0
    s.side_patch[1] = 1
    for q in range(2, 6):
        s.side_patch[q] = 2
    s.n_obstacles = 1
    ob = s.obstacles[0]
    c0, c1 = 48 // scale, 80 // scale
    for a in range(3):
        ob.lo[a] = c0
        ob.hi[a] = c1
    for q in range(6):
        ob.patch[q] = 3
    s.n_species = 1
    set_species(s, 0, N2)
    s.binary_collision_model = COLL_LB_VHS
    vol = h ** 3
    s.n_equivalent_particles = 1e21 * vol / 20.0
    s.delta_t = 5e-8 * scale
    s.seed = seed
    s.init_number_density[0] = 1e21
    s.init_t_tra = 200.0
    s.init_t_rot = 200.0
    s.init_t_vib = 200.0
    s.init_velocity[0] = U
    return s
