/*
 * hystrath_gb300.h -- C ABI of the GB300-native dsmcFoam+ particle hot path.
 *
 * One handle owns one DSMC cloud on one GPU: its parcel state in HBM (one
 * 64-byte record per parcel plus a cell word), per-cell collision and sampling
 * state, the stream it runs on (and a second stream that carries the step's
 * concurrent branches -- the inflow beside the move, the heavy cells'
 * collisions beside the light cells' -- joined back into the first before
 * the step ends) and its captured step graphs.  The entry points replace the
 * calls that the dsmcFoam+ driver makes on a dsmcCloud:
 *
 *   reference (path in hystrath/hyStrath)                         this ABI
 *   dsmcCloud ctor  src/lagrangian/dsmc/clouds/dsmcCloud.C:586-691  dsmc_create / dsmc_create_from_spec
 *   dsmcMeshFill    src/lagrangian/dsmc/initialiseDsmcParcels/
 *                   derived/dsmcMeshFill/dsmcMeshFill.C:68-238      dsmc_initialise
 *   dsmcCloud::evolve  dsmcCloud.C:819-902                         dsmc_evolve
 *   dsmcCloud::info    dsmcCloud.C:935-985                         dsmc_info
 *   dsmcVolFields::calculateField (output part)
 *                   src/lagrangian/dsmc/macroscopicProperties/derived/
 *                   combined/dsmcVolFields/dsmcVolFields.C:1365-1876 dsmc_get_field
 *   lagrangian/dsmc parcel IO    src/lagrangian/dsmc/parcels/
 *                   dsmcParcelIO.C:133-450                          dsmc_get_particles / dsmc_set_particles,
 *                                                                   dsmc_read_parcels / dsmc_write_parcels
 *   sigmaTcRMax field (MUST_READ/AUTO_WRITE) dsmcCloud.C:625-636     dsmc_get_cell_array / dsmc_set_cell_array
 *   runtime selection New() of BinaryCollisionModel
 *                   (collisions/BinaryCollisionModel/.../BinaryCollisionModel.C:59-90),
 *                   collisionPartnerSelection (collisionPartnerSelection.C:64-97),
 *                   dsmcPatchBoundary (dsmcPatchBoundary.C:130-165)  the model fields of dsmc_case_spec,
 *                                                                   resolved by name in dsmc_create
 *
 * Every call returns a status (DSMC_OK == 0).  The reference aborts with
 * FatalError instead; here the message is kept per handle (dsmc_last_error) or
 * per thread when no handle exists yet (dsmc_last_global_error).  A handle is
 * not thread safe.  All pointers in this header are HOST pointers.
 */
#ifndef HYSTRATH_GB300_H
#define HYSTRATH_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define DSMC_MAX_SPECIES 8
#define DSMC_MAX_PATCHES 16
#define DSMC_MAX_OBSTACLES 8
#define DSMC_NAME_LEN 64

/* Status codes. */
enum {
    DSMC_OK = 0,
    DSMC_ERR_IO = 1,            /* a case file could not be read */
    DSMC_ERR_PARSE = 2,         /* a dictionary could not be parsed */
    DSMC_ERR_UNKNOWN_MODEL = 3, /* model name not in the runtime-selection table */
    DSMC_ERR_INVALID = 4,       /* inconsistent or unsupported case description */
    DSMC_ERR_CUDA = 5,          /* a CUDA call failed */
    DSMC_ERR_DEVICE = 6,        /* a device loop hit its iteration cap or a bound check */
    DSMC_ERR_CAPACITY = 7,      /* particle or buffer capacity exceeded */
    DSMC_ERR_NO_DEVICE = 8      /* no usable GPU */
};

/* polyPatch types of the boundary mesh. */
enum {
    DSMC_PATCH_WALL = 0,     /* wall: dispatched to a dsmcPatchBoundary model */
    DSMC_PATCH_PATCH = 1,    /* patch: dispatched to a dsmcPatchBoundary model */
    DSMC_PATCH_SYMMETRY = 2, /* symmetry / symmetryPlane: specular transform */
    DSMC_PATCH_CYCLIC = 3,   /* cyclic: periodic translation to the opposite side */
    DSMC_PATCH_EMPTY = 4     /* empty: reduced-D axis, one cell thick, both sides */
};

/* dsmcPatchBoundary models (boundariesDict dsmcPatchBoundaries). */
enum {
    DSMC_BC_NONE = 0,
    DSMC_BC_SPECULAR = 1,  /* dsmcSpecularWallPatch */
    DSMC_BC_DIFFUSE = 2,   /* dsmcDiffuseWallPatch */
    DSMC_BC_DELETION = 3   /* dsmcDeletionPatch */
};

/* BinaryCollisionModel and collisionPartnerSelectionModel selections. */
enum {
    DSMC_COLL_VHS = 0,     /* VariableHardSphere */
    DSMC_COLL_LB_VHS = 1,  /* LarsenBorgnakkeVariableHardSphere */
    DSMC_COLL_VSS = 2,     /* VariableSoftSphere */
    DSMC_COLL_LB_VSS = 3   /* LarsenBorgnakkeVariableSoftSphere */
};
enum {
    DSMC_SEL_NTC = 0,      /* noTimeCounter */
    DSMC_SEL_SBT = 1       /* simplifiedBernoulliTrials */
};

/* Step phases, for dsmc_run_phases. */
enum {
    DSMC_PHASE_INFLOW = 1,   /* dsmcFreeStreamInflowPatch::controlParcelsBeforeMove */
    DSMC_PHASE_MOVE = 2,     /* Cloud::move with patch interactions */
    DSMC_PHASE_SORT = 4,     /* buildCellOccupancy (counting sort into cells) */
    DSMC_PHASE_COLLIDE = 8,  /* noTimeCounter::collide */
    DSMC_PHASE_SAMPLE = 16,  /* dsmcVolFields::calculateField sample loop */
    DSMC_PHASE_ALL = 31
};

/* One species of moleculeProperties (dsmcParcelI.H:37-200). */
typedef struct {
    char name[DSMC_NAME_LEN];
    double mass;
    double diameter;
    double omega;
    double alpha;
    double rotational_dof;
    int n_vib_modes;      /* 0 or 1 on this path */
    double theta_v;       /* characteristicVibrationalTemperature[0] */
    double theta_d;       /* dissociationTemperature */
    double zref;          /* Zref[0] */
    double tref_zv;       /* referenceTempForZref[0] */
} dsmc_species;

/* One boundary patch with its patch model and optional freestream inflow. */
typedef struct {
    char name[DSMC_NAME_LEN];
    int type;                      /* DSMC_PATCH_* */
    int model;                     /* DSMC_BC_* (wall and patch types) */
    double wall_temperature;       /* dsmcDiffuseWallPatchProperties.temperature */
    double wall_velocity[3];       /* dsmcDiffuseWallPatchProperties.velocity */
    int inflow;                    /* 1: dsmcFreeStreamInflowPatch on this patch */
    double inflow_number_density[DSMC_MAX_SPECIES];
    double inflow_t_tra;
    double inflow_t_rot;
    double inflow_t_vib;
    double inflow_velocity[3];
} dsmc_patch;

/* An axis-aligned solid block of cells [lo, hi) excluded from the flow. */
typedef struct {
    int lo[3];
    int hi[3];
    int patch[6];   /* patch of its -x,+x,-y,+y,-z,+z faces */
} dsmc_obstacle;

/*
 * Fully resolved case: a Cartesian hexahedral mesh (uniform unless node_coords
 * gives an axis its nodes), its patches, the
 * species, the dsmcProperties models and the dsmcMeshFill initial state.
 * Side order everywhere is -x, +x, -y, +y, -z, +z.  The face grid of a side
 * is indexed (a + na*b) with (a, b) = (y, z) for x sides, (x, z) for y sides
 * and (x, y) for z sides.
 */
typedef struct {
    int n_cells[3];
    double origin[3];
    double cell_size[3];
    int side_patch[6];             /* patch of every face of a side ...          */
    const int* face_patch[6];      /* ... unless a per-face patch map is given   */
    int n_obstacles;
    dsmc_obstacle obstacles[DSMC_MAX_OBSTACLES];
    int n_patches;
    dsmc_patch patches[DSMC_MAX_PATCHES];

    int n_species;
    dsmc_species species[DSMC_MAX_SPECIES];

    double n_equivalent_particles;   /* nEquivalentParticles (FN) */
    int binary_collision_model;      /* DSMC_COLL_* */
    int partner_selection_model;     /* DSMC_SEL_* */
    double tref;                     /* <Model>Coeffs.Tref, default 273 */
    double zrot;                     /* rotationalRelaxationCollisionNumber, default 5 */
    double fixed_zv;                 /* vibrationalRelaxationCollisionNumber, 0 = variable Zv */
    int inv_zv_formulation;          /* 0 pre-2008, 1 2008, 2 default */
    double delta_t;                  /* controlDict deltaT */
    unsigned long long seed;         /* Philox key */

    int measure_mean_free_path;      /* dsmcVolFieldsProperties.measureMeanFreePath */
    double mfp_tref;                 /* mfpReferenceTemperature, default 273 */

    /* dsmcInitialiseDict dsmcMeshFill configuration */
    double init_number_density[DSMC_MAX_SPECIES];
    double init_t_tra;
    double init_t_rot;
    double init_t_vib;
    double init_velocity[3];
    double init_t_tra_xyz[3];        /* >0: per-axis translational temperatures
                                        (anisotropic start; not a reference key) */
    long long max_particles;         /* capacity; 0 = 2x the initial fill + inflow margin; at most
                                        2^31 - 1 (32-bit parcel indices), else DSMC_ERR_CAPACITY */

    /* Rectilinear grading (blockMesh simpleGrading): for a graded axis the
     * n_cells[a] + 1 node coordinates, strictly increasing (origin[a] and
     * cell_size[a] are then ignored); NULL for a uniform axis. */
    const double* node_coords[3];

    /* Output schedule of the time averages (dsmcField timeProperties,
     * dsmcField.C:113-150; controlDict writeInterval): every
     * write_interval_steps steps is an output time (0: none).  With
     * reset_at_output set, the averages restart after every output time t
     * whose previous output time t' (or the start) has t' + deltaT <=
     * reset_at_output_until_time (every output if that is 0). */
    long long write_interval_steps;
    int reset_at_output;
    double reset_at_output_until_time;
    /* dsmcVolFieldsProperties switches: measureErrors (the rhoMError,
     * UError, TError, pError fields) and measureHeatFluxShearStress (the
     * moment sums behind heatFluxVector, pressureTensor, shearStressTensor). */
    int measure_errors;
    int measure_heat_flux_shear_stress;
} dsmc_case_spec;

/* Cloud totals, as printed by dsmcCloud::info (dsmcCloud.C:935-985). */
typedef struct {
    long long n_particles;
    long long step;
    double linear_ke;        /* sum of 0.5 m |U|^2 over parcels, times FN */
    double rotational_e;     /* times FN */
    double vibrational_e;    /* times FN */
    double momentum[3];      /* times FN */
    long long collisions_last_step;
    long long candidates_last_step;
    long long collisions_total;
    long long candidates_total;
    long long wall_hits_last_step;
    long long inserted_last_step;
    long long deleted_last_step;
    long long sample_steps;
} dsmc_info_t;

/* The step counters alone (no pass over the parcels). */
typedef struct {
    long long n_particles;
    long long step;
    long long collisions_last_step;
    long long candidates_last_step;
    long long collisions_total;
    long long candidates_total;
} dsmc_counts_t;

typedef struct dsmc_handle dsmc_handle;

/* Fill *spec with the reference's defaults (Tref 273, Zrot 5, ...). */
void dsmc_spec_defaults(dsmc_case_spec* spec);

/* sizeof(dsmc_case_spec), for bindings that mirror the struct. */
long long dsmc_case_spec_size(void);

/* Build a cloud from a resolved spec (replaces dsmcCloud ctor). */
int dsmc_create_from_spec(const dsmc_case_spec* spec, dsmc_handle** out);

/* Build a cloud from an OpenFOAM case directory: constant/dsmcProperties,
 * system/{controlDict,boundariesDict,fieldPropertiesDict,dsmcInitialiseDict}
 * and an axis-aligned uniform system/blockMeshDict (or constant/polyMesh/blockMeshDict). */
int dsmc_create(const char* case_dir, dsmc_handle** out);

/* Parse a case directory into *spec without touching a GPU.  face_patch maps
 * stay owned by the library until the next call on this thread. */
int dsmc_parse_case(const char* case_dir, dsmc_case_spec* spec);

/* dsmcMeshFill: fill every cell from the spec's initial state and set
 * sigmaTcRMax to sigmaT * most probable speed. */
int dsmc_initialise(dsmc_handle* h);

/* Advance n full steps (dsmcCloud::evolve). */
int dsmc_evolve(dsmc_handle* h, long long n_steps);

/* Advance one step running only the given DSMC_PHASE_* bits (tests). */
int dsmc_run_phases(dsmc_handle* h, unsigned phases);

/* dsmc_evolve with CUDA events on the handle's stream around the whole run
 * (graph launches) and, for the profiled form, around every phase of every
 * step: phase_ms[5] receives the summed inflow, move, sort, collide+sample
 * and bookkeeping times, total_ms the first-to-last event time.  No host
 * synchronisation happens inside the run. */
int dsmc_evolve_timed(dsmc_handle* h, long long n_steps, double* total_ms);
int dsmc_evolve_profiled(dsmc_handle* h, long long n_steps, double* phase_ms, double* total_ms);

/* The same with events between the step's kernel groups: group_ms[k] (k <
 * n_groups <= DSMC_KGROUP_COUNT) receives the summed time of group k over the
 * n steps.  No counterpart in the reference (a profiling aid). */
enum {
    DSMC_KGROUP_ZERO = 0,      /* step counters reset */
    DSMC_KGROUP_INFLOW,        /* freestream inflow (count, scan, fill, commit) */
    DSMC_KGROUP_MOVE,          /* k_move (fast path) */
    DSMC_KGROUP_MOVE_SLOW,     /* k_move_slow (boundary path) */
    DSMC_KGROUP_SAMPLE,        /* sample commit of the fixed-point sums */
    DSMC_KGROUP_SCAN,          /* occupancy scan */
    DSMC_KGROUP_SCATTER,       /* k_scatter_index: a slot per parcel */
    DSMC_KGROUP_GATHER,        /* k_gather: the records into cell order */
    DSMC_KGROUP_FINISH,        /* sort bookkeeping */
    DSMC_KGROUP_LEARNED,       /* learned maximum: features and inference */
    DSMC_KGROUP_SELECT,        /* candidate counts, work list, heavy-cell ordering */
    DSMC_KGROUP_HEAVY,         /* collisions of heavy cells */
    DSMC_KGROUP_LIGHT,         /* collisions of light cells */
    DSMC_KGROUP_PENDING,       /* marks the post-collision state for sampling */
    DSMC_KGROUP_END,           /* step bookkeeping */
    DSMC_KGROUP_COUNT
};
int dsmc_evolve_kernel_profile(dsmc_handle* h, long long n_steps, double* group_ms, int n_groups,
                               double* total_ms);

/* Replace the particle set.  pos and U are n x 3 interleaved; vib may be NULL;
 * ids must be unique.  Particles are placed in their cells and sorted. */
int dsmc_set_particles(dsmc_handle* h, long long n, const double* pos, const double* U,
                       const double* erot, const int* vib, const int* species,
                       const unsigned* id);

/* Read the particle set in device order (cell order after a sort). Any output
 * pointer may be NULL.  cell receives the cell index, or -1 if deleted. */
int dsmc_get_particles(dsmc_handle* h, long long capacity, long long* n, double* pos, double* U,
                       double* erot, int* vib, int* species, unsigned* id, int* cell);

/* Per-cell arrays: "count" (int, parcels per cell after the last sort),
 * "start" (int), "sigmaTcRMax", "collisionSelectionRemainder" (double); and
 * per boundary face and species (n = dsmc_n_boundary_faces x species, face
 * major) "inflowAccumulator" (double): the fraction of a parcel that the
 * freestream inflow carries to the next step (accumulatedParcelsToInsert_,
 * dsmcFreeStreamInflowPatch.C:131-141), zero on faces without inflow; and
 * with the selection audit on, "selectionAudit" (double, n = 2 x cells,
 * cell major): the audit sums of dsmc_set_selection_audit; "learnedFeatures"
 * (float, n = 4 x cells, cell major, read only): the learned maximum's
 * inputs of the current state (log number density, log translational
 * temperature, speed ratio, 1 where valid). */
int dsmc_get_cell_array(dsmc_handle* h, const char* name, void* out, long long n);
int dsmc_set_cell_array(dsmc_handle* h, const char* name, const void* in, long long n);

/* Derived volume field by its dsmcVolFields name, e.g. "rhoN", "rhoM",
 * "Ttra", "Trot", "Tvib", "Tov", "p", "Ux", "Uy", "Uz", "dsmcNMean",
 * "nColls", "measuredCollisionRate", "meanCollisionRate", "mfp".
 * n must equal the number of cells. */
int dsmc_get_field(dsmc_handle* h, const char* name, double* out, long long n);

/* The same field over a subset of the species (bit s of species_mask selects
 * species s): a dsmcVolFields entry with its own typeIds list
 * (dsmcVolFields.C:841), e.g. Ttra_N2 of the N2/O2 Couette case. */
int dsmc_get_species_field(dsmc_handle* h, const char* name, unsigned species_mask, double* out, long long n);

/* Per-boundary-face wall fields averaged over the steps since the last
 * dsmc_reset_sampling (dsmcVolFields.C:2110-2126): "wallHeatFlux", the force
 * density "wallShearStress_x|y|z" (fD), its tangential magnitude
 * "wallShearStress", the surface pressure "p_wall" (fD . n, n the outward
 * normal of the gas) and "rhoN_wall"; n = number of boundary faces. */
int dsmc_get_wall_field(dsmc_handle* h, const char* name, double* out, long long n);
long long dsmc_n_boundary_faces(const dsmc_handle* h);

/* Restart the time averages (dsmcField resetAtOutput). */
int dsmc_reset_sampling(dsmc_handle* h);

/* dsmcVolFields::writeField (dsmcVolFields.C:1878-2380): the averaged fields
 * as OpenFOAM ASCII files in case_dir/time_name/ -- rhoN, rhoM, Ttra, Trot,
 * Tvib, Tov, p, dsmcNMean and U (each with the suffix "_" field_name, as the
 * fieldName of fieldPropertiesDict) and dsmcSigmaTcRMax.  Cells are written
 * in the order of the case's blockMeshDict when case_dir has one (block by
 * block, i fastest), else in the Cartesian order i + nx (j + ny k). */
int dsmc_write_fields(dsmc_handle* h, const char* case_dir, const char* time_name, const char* field_name);

/* dsmcParcelIO (dsmcParcelIO.C:133-450): the cloud as the lagrangian files of
 * an OpenFOAM time directory, <case_dir>/<time_name>/lagrangian/<cloud_name>/
 * (positions "(x y z) celli" with OpenFOAM's cell labels, U, ERot, typeId,
 * vibLevel, origId, newParcel, origProcId, classification), 17 significant
 * digits.  Reading takes positions, U and typeId, and ERot, vibLevel and
 * origId when present; cells follow from the positions.  Cartesian positions
 * only (the OpenFOAM v1706 format of dsmcFoam+; not the barycentric one of
 * OpenFOAM 5 and later).  dsmc_parse_parcels reads without a cloud or a GPU:
 * call it with pos == NULL for *n, then with arrays of *n entries (*n on
 * input is their capacity). */
int dsmc_write_parcels(dsmc_handle* h, const char* case_dir, const char* time_name, const char* cloud_name);
int dsmc_read_parcels(dsmc_handle* h, const char* case_dir, const char* time_name, const char* cloud_name);
int dsmc_parse_parcels(const char* case_dir, const char* time_name, const char* cloud_name, long long* n,
                       double* pos, double* U, double* erot, int* vib, int* species, unsigned* id);
const char* dsmc_parse_last_error(void);

/* dsmcFaceTracker (faceTracker/dsmcFaceTracker.C:124-190, dsmcCloud.C:425-437):
 * with tracking on, every cell face a parcel crosses in the move gets
 * sign(U . S) ("parcelIdFlux") and sign(U . S) m ("massIdFlux") for the
 * parcel's species, S the face's area vector (+axis between two cells,
 * outward on a boundary face, the velocity after a wall or symmetry
 * interaction); a cyclic crossing counts +1 on the face it leaves through
 * and an inserted parcel counts -1 on its inflow face.  Sums over the steps
 * since the last dsmc_reset_sampling (the reference clears them every step).
 * Faces: x faces i + (nx+1)(j + ny k), then y faces i + nx(j + (ny+1) k),
 * then z faces i + nx(j + ny k), n = dsmc_n_faces.  Off by default (it adds
 * a division per crossing and two atomics per face). */
int dsmc_set_face_tracking(dsmc_handle* h, int on);
long long dsmc_n_faces(const dsmc_handle* h);
int dsmc_get_face_flux(dsmc_handle* h, const char* name, int species, double* out, long long n);

/* dsmcFluxSurface (macroscopicProperties/derived/flux/dsmcFluxSurface/
 * dsmcFluxSurface.C:203-400), the fieldModel that reads the face tracker:
 * over the faces of a face zone and the species of typeIds it sums
 * parcelIdFlux FN (S/|S| . d) and massIdFlux FN (S/|S| . d), d the
 * normalised fluxDirection, and divides by the averaging time (steps since
 * the face sums were reset x deltaT) and by the zone's area (the sum of |S|).
 * The zone is the set of mesh faces whose centres lie in a box, bounds
 * included: topoSet's boxToFace, which is how a faceZone of a blockMesh case
 * is made.  A face between two solid cells is not a mesh face.
 * dsmc_add_flux_surface switches face tracking on; a surface added to a cloud
 * that already tracks faces reads the sums since their last reset. */
typedef struct {
    char field_name[DSMC_NAME_LEN];   /* fieldName */
    char zone_name[DSMC_NAME_LEN];    /* faceZoneName */
    double box_min[3];
    double box_max[3];
    double direction[3];              /* fluxDirection (any length > 0) */
    unsigned species_mask;            /* typeIds: bit m for species m */
} dsmc_flux_surface;

int dsmc_add_flux_surface(dsmc_handle* h, const dsmc_flux_surface* surface);
int dsmc_n_flux_surfaces(const dsmc_handle* h);
/* out[6]: faceParticleFlux (1/(m^2 s)), faceParticleFlowRate (1/s),
 * faceMassFlux (kg/(m^2 s)), faceMassFlowRate (kg/s), the zone's area (m^2)
 * and the averaging time (s); surface may be NULL.  DSMC_ERR_INVALID before
 * the first step after a reset (the averaging time is zero). */
int dsmc_get_flux_surface(dsmc_handle* h, int i, dsmc_flux_surface* surface, double* out);
/* dsmcFluxSurface::writeField (dsmcFluxSurface.C:455-509): appends
 * "time<TAB>value" (11 significant digits) to
 * case_dir/fieldMeasurements/face{ParticleFlux,ParticleFlowRate,MassFlux,
 * MassFlowRate}_<zone>_<field>.xy for every surface. */
int dsmc_write_flux_surfaces(dsmc_handle* h, const char* case_dir, double time_value);
/* The dsmcFluxSurface entries of system/fieldPropertiesDict with their
 * zones from system/topoSetDict (a faceSet made by one boxToFace, turned
 * into a zone by setsToZones or a faceZoneSet's setToFaceZone).  Call with
 * out == NULL for *n; then *n on input is the capacity of out.  dsmc_create
 * adds them to the cloud it makes. */
int dsmc_parse_flux_surfaces(const char* case_dir, dsmc_flux_surface* out, int* n);

int dsmc_info(dsmc_handle* h, dsmc_info_t* out);
/* Particle count and collision counters after the last step, read without
 * the energy sums of dsmc_info (a few bytes instead of a pass over the
 * parcels). */
int dsmc_counts(dsmc_handle* h, dsmc_counts_t* out);
/* n steps of dsmc_evolve with each step's counters (dsmc_counts) in out[0..n):
 * every step's counters are copied to pinned host memory on the cloud's
 * stream right after the step, and the host waits once, at the end. */
int dsmc_evolve_counts(dsmc_handle* h, long long n, dsmc_counts_t* out);

/* Binary checkpoint: particles, per-cell state, step and seed.  Together with
 * the counter-based random stream this resumes bit for bit. */
int dsmc_checkpoint(dsmc_handle* h, const char* path);
int dsmc_restore(dsmc_handle* h, const char* path);

/* Wall-clock of each phase of the last dsmc_evolve, milliseconds (CUDA events). */
int dsmc_phase_times(dsmc_handle* h, double* ms_inflow, double* ms_move, double* ms_sort,
                     double* ms_collide, double* ms_sample);

const char* dsmc_last_error(const dsmc_handle* h);
const char* dsmc_last_global_error(void);
/* Frees the cloud.  A handle from dsmc_batch_case is left alone (its
 * dsmc_last_error says so): dsmc_batch_destroy frees the batch's cases. */
void dsmc_destroy(dsmc_handle* h);

/*
 * Spatial decomposition, the reference's processor patches: Cloud::move
 * (Cloud.C:255-466) hands a parcel that reaches a processor patch to the
 * neighbouring domain, and the step's totals are summed over the processors
 * (noTimeCounter.C:312-314, dsmcCloud.C:938-958).  Here a cloud keeps the
 * whole case but owns only the parcels of the cells with lo <= index < hi
 * along axis (0 x, 1 y, 2 z; meshes below 2^24 cells): dsmc_set_domain drops
 * the others (also from later dsmc_initialise / dsmc_set_particles /
 * dsmc_restore), and a parcel whose move ends in another domain's cell
 * leaves the cloud as a migrant, its move complete.  The inflow counts every
 * inflow face, so the parcel ids are those of the undivided case, and
 * inserts into owned cells only.  Collisions and sampling are per cell and
 * keyed by the global cell: the domains of a divided case together step
 * exactly as the undivided case does.  axis = -1 undoes the division (the
 * parcels stay).  A divided cloud steps in two halves with the migrants
 * handed over between them:
 *   dsmc_step_begin   inflow and move; the migrants packed on the device
 *   dsmc_get_migrants n migrants, DSMC_MIGRANT_BYTES each (the 64-byte parcel
 *                     record and the 4-byte cell word), to host or device
 *                     memory
 *   dsmc_add_migrants migrants from other domains (host or device memory),
 *                     before the sort; one for a cell this cloud does not own
 *                     is dropped and reported by dsmc_step_end
 *   dsmc_step_end     occupancy sort, collisions, sampling
 * The whole-step calls (dsmc_evolve, dsmc_evolve_timed, dsmc_evolve_counts,
 * dsmc_run_phases, the profiles) return DSMC_ERR_INVALID on a divided cloud.
 */
#define DSMC_MIGRANT_BYTES 68
int dsmc_set_domain(dsmc_handle* h, int axis, int lo, int hi);
int dsmc_step_begin(dsmc_handle* h, long long* n_migrants);
int dsmc_get_migrants(dsmc_handle* h, void* dst, long long n);
int dsmc_add_migrants(dsmc_handle* h, const void* src, long long n);
int dsmc_step_end(dsmc_handle* h);

/*
 * Cell start offsets for callers that must not allocate device memory.  This
 * entry point has no counterpart in the reference (whose occupancy lists live
 * in host memory); it is the exclusive scan of the occupancy sort, offered to
 * code that owns its device memory in a fixed pool or may not grow its
 * footprint.  Unlike the rest of this header it takes DEVICE pointers:
 * d_counts[n_cells] parcels per cell in, d_start[n_cells + 1] out (the last
 * entry is the total), on the given cudaStream_t (NULL = legacy stream).
 * No cudaMalloc/cudaFree: the block sums live in a 16 KiB static device array
 * that every GPU loading the library holds until exit, which limits n_cells to
 * 2^24.  Every call made outside stream capture resolves that array's
 * address on the current device (the first call on a device, and the first
 * after a device reset, must come before any stream capture; captured calls
 * use the last address resolved).  Calls share the array: calls that overlap on
 * the GPU race.  Errors: DSMC_ERR_INVALID beyond 2^24 cells or for null
 * buffers, message in dsmc_noalloc_last_error().
 */
int dsmc_cell_starts_noalloc(const int* d_counts, long long n_cells, int* d_start, void* stream);
const char* dsmc_noalloc_last_error(void);

/*
 * Learned (sigma_T c_R)max.  No counterpart in the reference, which keeps only
 * the running maximum of noTimeCounter (noTimeCounter.C:243-246).  A
 * 3-64-64-1 SiLU perceptron (BF16 weights and activations, FP32 sums) maps a
 * cell's (log n, log T_tr, speed ratio) to log (sigma_T c_R)max.  It is
 * trained on the GPU with Adam on (state, observed maximum) rows recorded
 * from plain runs; attached to a cloud, it replaces the running maximum in
 * the candidate count and the acceptance test of each cell until a product
 * exceeds it, after which the cell uses the running maximum again until the
 * next prediction.
 *
 * Parameter vector (DSMC_MLP_NPARAM floats): W1[64][3], b1[64], W2[64][64]
 * (row = output), b2[64], w3[64], b3.  norm8: input means (3), input scales
 * (3), output mean, output scale: the net sees (x - mean) / scale and its
 * output y maps to ymean + yscale * y.
 */
#define DSMC_MLP_NPARAM 4481
typedef struct dsmc_mlp dsmc_mlp;
int dsmc_mlp_nparam(void);
int dsmc_mlp_create(dsmc_mlp** out);
void dsmc_mlp_destroy(dsmc_mlp* m);
const char* dsmc_mlp_last_error(const dsmc_mlp* m);
int dsmc_mlp_set_params(dsmc_mlp* m, const float* params, const float* norm8);
int dsmc_mlp_get_params(dsmc_mlp* m, float* params, float* norm8);
/* loss of dsmc_mlp_train and dsmc_mlp_grad: tau 0 (default) the mean squared
   error, tau in (0, 1) the pinball loss whose minimiser is the tau-quantile */
int dsmc_mlp_set_loss(dsmc_mlp* m, float tau);
/* training rows: X[n][3] features, Y[n] log maxima */
int dsmc_mlp_set_data(dsmc_mlp* m, const float* X, const float* Y, long long n);
/* steps Adam steps (beta 0.9/0.999) on minibatches of batch rows drawn with
   replacement from the data by a Philox stream of seed; loss_out[steps] or
   NULL receives the minibatch mean loss (normalised units) */
int dsmc_mlp_train(dsmc_mlp* m, int steps, int batch, float lr, unsigned long long seed, float* loss_out);
/* gradient of the mean loss over rows [0, n) (no update) */
int dsmc_mlp_grad(dsmc_mlp* m, const float* X, const float* Y, int n, float* grad_out, float* loss_out);
/* log-maximum predictions for n rows */
int dsmc_mlp_predict(dsmc_mlp* m, const float* X, long long n, float* out);
/* Selection audit (no counterpart in the reference): with it on, every
   noTimeCounter candidate adds, to its cell, sigma_T c_R / max (its
   acceptance probability when the maximum bounds the product) and
   max(0, sigma_T c_R / max - 1) (the part the acceptance test cannot
   honour).  Per cell, the ratio of the second sum to the first is the
   expected relative shortfall of its collision count caused by a maximum
   below the product: zero for an exact NTC, the reference's own snapshot
   shortfall for the running maximum (noTimeCounter.C:243-248), the learned
   selection's error with a prediction.  Read with dsmc_get_cell_array
   "selectionAudit"; cleared by dsmc_reset_sampling and when switched on. */
int dsmc_set_selection_audit(dsmc_handle* h, int on);
/* attach a model (NULL: plain running maximum); predictions every `every`
   steps, used as exp(prediction + margin) */
int dsmc_set_learned(dsmc_handle* h, const dsmc_mlp* model, int every, float margin);
/* A learned cell whose candidates produced a sigma_T c_R above the value it
   selected with falls back to the running maximum until the next
   prediction, and a later prediction is used only if it reaches the largest
   such product remembered for the cell.  At every prediction the memory is
   multiplied by `forget` in [0, 1]: 1 (the default) keeps it for good, 0
   forgets it at every prediction. */
int dsmc_set_learned_forget(dsmc_handle* h, float forget);
/* after a step: (features, log largest product among the step's candidates)
   of the cells that had candidates, at most max_rows of them */
int dsmc_learn_record(dsmc_handle* h, long long max_rows, float* X, float* Y, long long* n_out);

/*
 * Lower the caps of the device loops that the reference runs without bound
 * (acceptance-rejection draws: the inflow normal speed, the vibrational
 * level, dsmcFreeStreamInflowPatch.C:288-305, dsmcCloud.C:1516-1526; face
 * crossings of one move), of the cell size the collision kernels order (a
 * larger cell skips its collisions), and of the parcel capacity the inflow
 * may fill.  0 keeps the default (100000 draws, 64 crossings, 16384 parcels,
 * the allocated capacity); larger values are rejected.  A cap that is
 * reached sets a bit of the device error word instead of faulting or
 * hanging: the next call that checks it returns DSMC_ERR_DEVICE (caps) or
 * DSMC_ERR_CAPACITY with a message, the bits are cleared once reported and
 * the handle steps on.  For tests of that path; the reference's FatalError
 * sites (BinaryCollisionModel.C:72-83, dsmcCloud.C:1354-1383) abort instead.
 */
int dsmc_set_limits(dsmc_handle* h, int max_rejection, int max_crossings, int max_cell_parcels,
                    long long capacity);

/*
 * Launch shape of a cloud's step (no counterpart in the reference, which runs
 * on CPU threads): threads per CTA of the parcel-streaming kernels (move,
 * sample, sort; 128, 256 or 512) and cells per CTA of the one-lane-per-cell
 * collision kernel (32, 64 or 128).  Chosen by the autotuner of
 * hystrath_gb300/batch.py.
 */
int dsmc_set_launch(dsmc_handle* h, int cta_threads, int cells_per_cta);
int dsmc_get_launch(dsmc_handle* h, int* cta_threads, int* cells_per_cta);

/*
 * A batch of independent clouds stepped together (no counterpart in the
 * reference, which runs one case per process).  Every batched step is ONE
 * launch of a CUDA graph that holds each case's captured step as an
 * independent child graph.  The cases are created and initialised as by
 * dsmc_create_from_spec / dsmc_initialise; dsmc_batch_case gives each case's
 * handle for reads (dsmc_info, dsmc_get_field, ...), which must not step it
 * on its own.  Errors: dsmc_batch_last_error.
 */
typedef struct dsmc_batch dsmc_batch;
int dsmc_batch_create(int n, const dsmc_case_spec* specs, dsmc_batch** out);
/* The same from n OpenFOAM case directories (each as dsmc_create). */
int dsmc_batch_create_from_dirs(int n, const char* const* case_dirs, dsmc_batch** out);
void dsmc_batch_destroy(dsmc_batch* b);
const char* dsmc_batch_last_error(const dsmc_batch* b);
int dsmc_batch_size(const dsmc_batch* b);
dsmc_handle* dsmc_batch_case(dsmc_batch* b, int i);
int dsmc_batch_initialise(dsmc_batch* b);
int dsmc_batch_set_launch(dsmc_batch* b, int i, int cta_threads, int cells_per_cta);
int dsmc_batch_evolve(dsmc_batch* b, long long n_steps);
/* Persistent mode of the batch (no counterpart in the reference): every
 * batched step is seven cooperative persistent launches over all cases -- four
 * ranges of the move and sort phases, then three of the collision phases,
 * each with its own register footprint -- whose CTAs take
 * (case, tile) work items from a queue per phase and wait at a grid barrier
 * between phases, so that small and large cases share the SMs; the step of
 * each buffer parity is captured as a CUDA graph where the driver allows
 * cooperative launches in a capture, else launched directly.  Results equal
 * the cases stepped alone.  move_threads: 128, 256 or 512; collide_threads:
 * 64 or 128 (the light cells per CTA); 0, 0 returns to the graph of case
 * graphs.  Every case must be a uniform box without inflow, obstacles,
 * reduced-D axes, face tracking, learned maximum, selection audit or moment
 * sums, with noTimeCounter selection; cells above 1024 parcels skip their
 * collisions with the dense-cell error.  A grid barrier wait that runs out
 * (it cannot while the launch is cooperative) returns DSMC_ERR_DEVICE. */
int dsmc_batch_set_persistent(dsmc_batch* b, int move_threads, int collide_threads);
int dsmc_batch_get_persistent(const dsmc_batch* b, int* move_threads, int* collide_threads);
/* the same, with the device time of the n steps in *total_ms */
int dsmc_batch_evolve_timed(dsmc_batch* b, long long n_steps, double* total_ms);

#ifdef __cplusplus
}
#endif
#endif /* HYSTRATH_GB300_H */
