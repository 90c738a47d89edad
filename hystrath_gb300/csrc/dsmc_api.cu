// dsmc_api.cu -- the C ABI of include/hystrath_gb300.h: handle life cycle,
// device memory, the captured step graph and host<->device transfers.
//
// The handle plays the role of dsmcCloud (src/lagrangian/dsmc/clouds/
// dsmcCloud.C): construction resolves the runtime-selected models
// (BinaryCollisionModel::New, collisionPartnerSelection::New,
// dsmcPatchBoundary::New), dsmc_initialise is dsmcMeshFill, dsmc_evolve is
// dsmcCloud::evolve.  One step is captured once per buffer parity as a CUDA
// graph and replayed; nothing in a step waits on the host.

#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <memory>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "dsmc_kernels.h"

namespace dsmc {
bool foam_cell_order(const std::string& dir, std::vector<long long>& order, std::string& err);   // case_parser.cpp
// internalField of a volScalarField file (one value when uniform); false with
// err empty when the file is absent
bool foam_read_scalar_field(const std::string& path, std::vector<double>& out, std::string& err);
}

using namespace dsmc;

struct dsmc_handle {
    dsmc_case_spec spec{};
    std::vector<std::vector<int>> facePatch;
    std::vector<double> node[3];       // node coordinates along each axis (n + 1)
    std::vector<double> width[3];      // cell widths (cell_size on a uniform axis)
    std::vector<double> bfAreaHost;    // area of every boundary face
    CaseDev cs{};
    InflowDev inflow{};
    StepBuffers B{};
    Parcels buf[2]{};
    double* faceBuf = nullptr;   // face tracker sums, kept while tracking is off
    double2* auditBuf = nullptr; // selection audit sums, kept while the audit is off
    long long faceStep0 = 0;     // step count when the face sums were last cleared
    struct FluxSurface {
        dsmc_flux_surface d;
        int* faces;       // device: the zone's faces
        double* w;        // device: FN (S/|S| . fluxDirection) of each face
        int nF;
        double area;
    };
    std::vector<FluxSurface> surfaces;
    double* surfOut = nullptr;   // device: the two sums of k_flux_surface
    std::vector<unsigned char> solidHost;   // 1 for cells inside a solid box
    long long nFluid = 0;        // cells outside the solid boxes
    bool smaxSet = false;        // sigmaTcRMax initialised, restored or read
    unsigned* packFlags = nullptr;   // dsmc_set_particles: range flags and largest id + 1
    int cur = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    // the side branch of a captured step: the inflow beside the move of the
    // last step's parcels, and the heavy cells' collisions beside the light
    // cells' (forked from and joined back into stream within the step)
    cudaStream_t side = nullptr;
    cudaEvent_t forkEv = nullptr, joinEv = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    cudaGraph_t graphT[2] = {nullptr, nullptr};   // the captured steps (child graphs of a batch)
    unsigned long long graphGen = 0;   // bumped whenever the step graphs are dropped
    bool batchOwned = false;           // a case of a dsmc_batch: freed only by dsmc_batch_destroy
    // spatial decomposition: the two halves of a step (inflow and move to the
    // packed migrants; the sort onwards) as graphs per parity, whether a step
    // is between its halves, and its moved-parcel count as of then
    cudaGraphExec_t half1[2] = {nullptr, nullptr};
    cudaGraphExec_t half2[2] = {nullptr, nullptr};
    bool midStep = false;
    long long nMovedHost = 0;
    long long nMigHost = 0;
    unsigned char* solid = nullptr;
    double* info6 = nullptr;
    double* fieldTmp = nullptr;
    Counters* ctrHost = nullptr;   // pinned mirror
    Counters* ctrRing = nullptr;   // pinned, one per step of dsmc_evolve_counts
    long long ctrRingN = 0;
    std::vector<void*> allocs;
    std::string err;
    double phaseMs[5] = {0, 0, 0, 0, 0};
    bool hasInflow = false;
    long long expectedN = 0;
    // output schedule of the time averages (resetAtOutput): the step count
    // as of the last read of the counters, whether resets at output are
    // still on, and a reset due before the next step
    long long stepHost = 0;
    bool resetActive = true;
    bool resetPending = false;
    // learned selection
    const MlpModel* model = nullptr;
    int learnEvery = 0;
    float learnMargin = 0.f;
    float learnForget = 1.f;      // kept fraction of a cell's remembered excess at a prediction
};

namespace {

thread_local std::string g_err;

int fail(dsmc_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    g_err = msg;
    return code;
}

#define CUDA_TRY(h, call)                                                                   \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(h, DSMC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
int dalloc(dsmc_handle* h, T** p, long long count) {
    void* q = nullptr;
    const size_t bytes = (size_t)(count > 0 ? count : 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess)
        return fail(h, e == cudaErrorMemoryAllocation ? DSMC_ERR_CAPACITY : DSMC_ERR_CUDA,
                    std::string("cudaMalloc of ") + std::to_string(bytes) + " bytes: " + cudaGetErrorString(e));
    cudaMemset(q, 0, bytes);
    h->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return DSMC_OK;
}

int alloc_soa(dsmc_handle* h, Parcels* s, long long cap) {
    int rc;
    if ((rc = dalloc(h, &s->r, cap))) return rc;
    if ((rc = dalloc(h, &s->cellw, cap))) return rc;
    if ((rc = dalloc(h, &s->id, cap))) return rc;
    return DSMC_OK;
}

const char* patch_type_names[] = {"wall", "patch", "symmetry", "cyclic", "empty"};

int validate(dsmc_handle* h, const dsmc_case_spec& s) {
    for (int a = 0; a < 3; ++a) {
        if (s.n_cells[a] <= 0) return fail(h, DSMC_ERR_INVALID, "n_cells must be positive");
        if (!(s.cell_size[a] > 0)) return fail(h, DSMC_ERR_INVALID, "cell_size must be positive");
    }
    const long long C = (long long)s.n_cells[0] * s.n_cells[1] * s.n_cells[2];
    if (C > (1LL << 28)) return fail(h, DSMC_ERR_INVALID, "more than 2^28 cells");
    for (int a = 0; a < 3; ++a) {
        if (!s.node_coords[a]) continue;
        for (int i = 0; i <= s.n_cells[a]; ++i)
            if (!std::isfinite(s.node_coords[a][i]) || (i > 0 && !(s.node_coords[a][i] > s.node_coords[a][i - 1])))
                return fail(h, DSMC_ERR_INVALID, "node_coords must be finite and strictly increasing");
    }
    if (s.n_species < 1 || s.n_species > DSMC_MAX_SPECIES)
        return fail(h, DSMC_ERR_INVALID, "n_species must be 1.." + std::to_string(DSMC_MAX_SPECIES));
    for (int i = 0; i < s.n_species; ++i) {
        const dsmc_species& q = s.species[i];
        if (!(q.mass > 0) || !(q.diameter > 0))
            return fail(h, DSMC_ERR_INVALID, std::string("species ") + q.name + ": mass and diameter must be positive");
        if (q.n_vib_modes < 0 || q.n_vib_modes > 1)
            return fail(h, DSMC_ERR_INVALID, std::string("species ") + q.name +
                                                 ": nVibrationalModes > 1 is not supported on this path");
    }
    if (s.binary_collision_model < DSMC_COLL_VHS || s.binary_collision_model > DSMC_COLL_LB_VSS)
        return fail(h, DSMC_ERR_UNKNOWN_MODEL,
                    "Unknown BinaryCollisionModel type. Valid BinaryCollisionModel types are: "
                    "4(VariableHardSphere LarsenBorgnakkeVariableHardSphere VariableSoftSphere "
                    "LarsenBorgnakkeVariableSoftSphere)");
    if (s.binary_collision_model == DSMC_COLL_VSS || s.binary_collision_model == DSMC_COLL_LB_VSS)
        for (int i = 0; i < s.n_species; ++i)
            if (!(s.species[i].alpha > 0))
                return fail(h, DSMC_ERR_INVALID, std::string("species ") + s.species[i].name +
                                                     ": VariableSoftSphere needs alpha > 0");
    if (s.partner_selection_model != DSMC_SEL_NTC && s.partner_selection_model != DSMC_SEL_SBT)
        return fail(h, DSMC_ERR_UNKNOWN_MODEL,
                    "Unknown collisionPartnerSelectionModel type. Valid types are: "
                    "2(noTimeCounter simplifiedBernoulliTrials)");
    if (s.n_patches < 1 || s.n_patches > DSMC_MAX_PATCHES)
        return fail(h, DSMC_ERR_INVALID, "n_patches must be 1.." + std::to_string(DSMC_MAX_PATCHES));
    for (int p = 0; p < s.n_patches; ++p) {
        const dsmc_patch& pt = s.patches[p];
        if (pt.type < 0 || pt.type > DSMC_PATCH_EMPTY)
            return fail(h, DSMC_ERR_INVALID, std::string("patch ") + pt.name + ": bad type");
        if (pt.type == DSMC_PATCH_EMPTY && pt.inflow)
            return fail(h, DSMC_ERR_INVALID, std::string("patch ") + pt.name + ": an empty patch takes no inflow");
        if ((pt.type == DSMC_PATCH_WALL || pt.type == DSMC_PATCH_PATCH) &&
            (pt.model < DSMC_BC_SPECULAR || pt.model > DSMC_BC_DELETION))
            return fail(h, DSMC_ERR_UNKNOWN_MODEL,
                        std::string("patch ") + pt.name + " (" + patch_type_names[pt.type] +
                            ") has no dsmcPatchBoundary model. Valid models are: "
                            "3(dsmcSpecularWallPatch dsmcDiffuseWallPatch dsmcDeletionPatch)");
    }
    for (int q = 0; q < 6; ++q) {
        if (s.side_patch[q] < 0 || s.side_patch[q] >= s.n_patches)
            return fail(h, DSMC_ERR_INVALID, "side_patch out of range");
        if (s.patches[s.side_patch[q]].type == DSMC_PATCH_CYCLIC) {
            const int o = q ^ 1;
            if (s.patches[s.side_patch[o]].type != DSMC_PATCH_CYCLIC)
                return fail(h, DSMC_ERR_INVALID, "a cyclic side needs a cyclic opposite side");
        }
    }
    // an empty direction: both sides empty on every face, one cell thick
    // (OpenFOAM's emptyPolyPatch rules)
    int nEmpty = 0;
    for (int q = 0; q < 6; ++q) {
        const int a = q / 2, b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
        const long long nf = (long long)s.n_cells[b] * s.n_cells[c];
        int ne = 0;
        for (long long f = 0; f < nf; ++f) {
            const int p = s.face_patch[q] ? s.face_patch[q][f] : s.side_patch[q];
            if (p >= 0 && p < s.n_patches && s.patches[p].type == DSMC_PATCH_EMPTY) ++ne;
        }
        if (ne && ne != nf)
            return fail(h, DSMC_ERR_INVALID, "an empty patch must cover a whole side of the mesh");
        if (ne && s.n_cells[a] != 1)
            return fail(h, DSMC_ERR_INVALID, "an empty direction must be one cell thick");
        if (ne && (q & 1) == 0) {
            const int p = s.face_patch[q ^ 1] ? s.face_patch[q ^ 1][0] : s.side_patch[q ^ 1];
            if (s.patches[p].type != DSMC_PATCH_EMPTY)
                return fail(h, DSMC_ERR_INVALID, "an empty side needs an empty opposite side");
            ++nEmpty;
        }
    }
    if (nEmpty == 3) return fail(h, DSMC_ERR_INVALID, "every direction is empty");
    for (int o = 0; o < s.n_obstacles; ++o)
        for (int q = 0; q < 6; ++q)
            if (s.patches[s.obstacles[o].patch[q]].type == DSMC_PATCH_EMPTY &&
                !((q & 1) ? s.obstacles[o].hi[q / 2] == s.n_cells[q / 2] : s.obstacles[o].lo[q / 2] == 0))
                return fail(h, DSMC_ERR_INVALID, "a solid box face cannot be empty");
    if (s.n_obstacles < 0 || s.n_obstacles > DSMC_MAX_OBSTACLES)
        return fail(h, DSMC_ERR_INVALID, "too many obstacles");
    for (int o = 0; o < s.n_obstacles; ++o) {
        const dsmc_obstacle& ob = s.obstacles[o];
        for (int a = 0; a < 3; ++a)
            if (ob.lo[a] < 0 || ob.hi[a] > s.n_cells[a] || ob.lo[a] >= ob.hi[a])
                return fail(h, DSMC_ERR_INVALID, "obstacle outside the mesh");
        for (int q = 0; q < 6; ++q)
            if (ob.patch[q] < 0 || ob.patch[q] >= s.n_patches)
                return fail(h, DSMC_ERR_INVALID, "obstacle patch out of range");
    }
    if (!(s.n_equivalent_particles > 0)) return fail(h, DSMC_ERR_INVALID, "nEquivalentParticles must be positive");
    if (!(s.delta_t > 0)) return fail(h, DSMC_ERR_INVALID, "deltaT must be positive");
    return DSMC_OK;
}

// Boundary-face patch map: 6 domain sides then obstacle sides.
void build_faces(dsmc_handle* h, std::vector<int>& bfPatch, std::vector<long long>& inflowFace,
                 std::vector<int>& inflowSide, std::vector<int>& inflowCell) {
    const dsmc_case_spec& s = h->spec;
    CaseDev& cs = h->cs;
    long long off = 0;
    for (int q = 0; q < 6; ++q) {
        const int a = q / 2;
        const int b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
        cs.sideOff[q] = off;
        const long long nf = (long long)s.n_cells[b] * s.n_cells[c];
        // a side deletes when every face's patch removes what reaches it
        // (not symmetry or cyclic, no specular or diffuse model)
        cs.sideDeletes[q] = 1;
        for (long long f = 0; f < nf; ++f) {
            const int p = s.face_patch[q] ? s.face_patch[q][f] : s.side_patch[q];
            bfPatch.push_back(p);
            {
                const long long ib = f % s.n_cells[b], ic = f / s.n_cells[b];
                h->bfAreaHost.push_back(h->width[b][ib] * h->width[c][ic]);
            }
            if (p < 0 || p >= s.n_patches || s.patches[p].type == DSMC_PATCH_SYMMETRY ||
                s.patches[p].type == DSMC_PATCH_CYCLIC || s.patches[p].model == DSMC_BC_SPECULAR ||
                s.patches[p].model == DSMC_BC_DIFFUSE)
                cs.sideDeletes[q] = 0;
            if (p >= 0 && p < s.n_patches && s.patches[p].inflow) {
                inflowFace.push_back(off + f);
                inflowSide.push_back(q);
                long long cc[3];
                cc[a] = (q & 1) ? s.n_cells[a] - 1 : 0;
                cc[b] = f % s.n_cells[b];
                cc[c] = f / s.n_cells[b];
                inflowCell.push_back((int)(cc[0] + (long long)s.n_cells[0] * (cc[1] + (long long)s.n_cells[1] * cc[2])));
            }
        }
        off += nf;
    }
    cs.sideOff[6] = off;
    for (int o = 0; o < s.n_obstacles; ++o) {
        const dsmc_obstacle& ob = s.obstacles[o];
        for (int q = 0; q < 6; ++q) {
            const int a = q / 2;
            const int b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
            cs.obstOff[o][q] = off;
            const long long nf = (long long)(ob.hi[b] - ob.lo[b]) * (ob.hi[c] - ob.lo[c]);
            const int nb = ob.hi[b] - ob.lo[b];
            for (long long f = 0; f < nf; ++f) {
                bfPatch.push_back(ob.patch[q]);
                const long long ib = ob.lo[b] + f % nb, ic = ob.lo[c] + f / nb;
                h->bfAreaHost.push_back(h->width[b][ib] * h->width[c][ic]);
            }
            off += nf;
        }
    }
    cs.nBFaces = off;
}

void fill_case_dev(dsmc_handle* h) {
    const dsmc_case_spec& s = h->spec;
    CaseDev& cs = h->cs;
    for (int a = 0; a < 3; ++a) {
        cs.n[a] = s.n_cells[a];
        if (s.node_coords[a]) {
            // graded: cells are found in the half-node table; dx and inv
            // describe the mean cell only
            cs.lo[a] = h->node[a].front();
            cs.hi[a] = h->node[a].back();
            cs.dx[a] = (cs.hi[a] - cs.lo[a]) / s.n_cells[a];
            cs.inv[a] = 1.0 / cs.dx[a];
            cs.negOinv[a] = -(cs.lo[a] * cs.inv[a]);
        } else {
            cs.dx[a] = s.cell_size[a];
            cs.inv[a] = 1.0 / s.cell_size[a];
            cs.negOinv[a] = -(s.origin[a] * cs.inv[a]);
            cs.lo[a] = s.origin[a];
            cs.hi[a] = s.origin[a] + s.n_cells[a] * s.cell_size[a];
        }
        cs.invF[a] = (float)cs.inv[a];
        cs.negOinvF[a] = (float)cs.negOinv[a];
        cs.mid[a] = 0.5 * (cs.lo[a] + cs.hi[a]);
        const int p = s.face_patch[2 * a] ? s.face_patch[2 * a][0] : s.side_patch[2 * a];
        cs.emptyAx[a] = s.patches[p].type == DSMC_PATCH_EMPTY;
    }
    cs.anyEmpty = cs.emptyAx[0] | cs.emptyAx[1] | cs.emptyAx[2];
    cs.C = (long long)cs.n[0] * cs.n[1] * cs.n[2];
    cs.rcpN0 = 1.0f / (float)cs.n[0];
    cs.rcpN01 = 1.0f / (float)((long long)cs.n[0] * cs.n[1]);
    cs.V = cs.dx[0] * cs.dx[1] * cs.dx[2];
    cs.FN = s.n_equivalent_particles;
    cs.dt = s.delta_t;
    cs.selK = cs.FN * cs.dt / cs.V;
    for (int a = 0; a < 3; ++a)
        cs.invDtFa[a] = 1.0 / (cs.dt * cs.dx[a == 0 ? 1 : 0] * cs.dx[a == 2 ? 1 : 2]);
    cs.seedLo = (uint32_t)s.seed;
    cs.seedHi = (uint32_t)(s.seed >> 32);
    cs.nSpecies = s.n_species;
    cs.collModel = s.binary_collision_model;
    cs.selModel = s.partner_selection_model;
    cs.zrot = s.zrot;
    cs.invZrot = 1.0 / s.zrot;
    cs.fixedZv = s.fixed_zv;
    cs.invZvForm = s.inv_zv_formulation;
    cs.nPatches = s.n_patches;
    for (int i = 0; i < s.n_species; ++i) cs.mRel[i] = (float)(s.species[i].mass / s.species[0].mass);
    for (int i = 0; i < s.n_species; ++i) {
        const dsmc_species& q = s.species[i];
        SpeciesDev& d = cs.sp[i];
        d.m = q.mass; d.d = q.diameter; d.omega = q.omega; d.rotDof = q.rotational_dof;
        d.thetaV = q.theta_v; d.thetaD = q.theta_d; d.zref = q.zref; d.trefZv = q.tref_zv;
        d.nVib = q.n_vib_modes;
        d.kThetaV = kB * q.theta_v;
        d.invKThetaV = q.theta_v > 0 ? 1.0 / d.kThetaV : 0.0;
        d.sqrtKoverM = std::sqrt(kB / q.mass);
    }
    for (int i = 0; i < s.n_species; ++i) {
        for (int j = 0; j < s.n_species; ++j) {
            const dsmc_species& a = s.species[i];
            const dsmc_species& b = s.species[j];
            PairDev& p = cs.pair[i * DSMC_MAX_SPECIES + j];
            const double dPQ = 0.5 * (a.diameter + b.diameter);
            const double om = 0.5 * (a.omega + b.omega);
            const double mR = a.mass * b.mass / (a.mass + b.mass);
            p.omegaPQ = om;
            p.mR = mR;
            p.expo = 1.0 - om;
            p.sigmaPrefactor = PI * dPQ * dPQ * std::pow(2.0 * kB * s.tref / mR, om - 0.5) /
                               std::exp(std::lgamma(2.5 - om));
            p.mPfrac = a.mass / (a.mass + b.mass);
            p.mQfrac = b.mass / (a.mass + b.mass);
            p.invAlphaPQ = 1.0 / (0.5 * (a.alpha + b.alpha));
            p.invAlphaF = (float)p.invAlphaPQ;
            p.chiBF = (float)(2.5 - om);
            p.invChiBF = (float)(1.0 / (2.5 - om));
            p.twoOverMR = 2.0 / mR;
            p.sigmaPrefactorF = (float)p.sigmaPrefactor;
            p.expoF = (float)p.expo;
        }
    }
    for (int p = 0; p < s.n_patches; ++p) {
        const dsmc_patch& pt = s.patches[p];
        cs.patch[p].type = pt.type;
        cs.patch[p].model = pt.model;
        cs.patch[p].Twall = pt.wall_temperature;
        for (int a = 0; a < 3; ++a) cs.patch[p].Uwall[a] = pt.wall_velocity[a];
        InflowPatchDev& ip = h->inflow.p[p];
        for (int m = 0; m < DSMC_MAX_SPECIES; ++m) ip.nd[m] = pt.inflow ? pt.inflow_number_density[m] : 0.0;
        ip.Ttra = pt.inflow_t_tra;
        ip.Trot = pt.inflow_t_rot;
        ip.Tvib = pt.inflow_t_vib;
        for (int a = 0; a < 3; ++a) ip.U[a] = pt.inflow_velocity[a];
        if (pt.inflow) h->hasInflow = true;
        cs.hasWallMeasure = 1;
    }
    h->inflow.nPatches = s.n_patches;
    cs.nObst = s.n_obstacles;
    for (int o = 0; o < s.n_obstacles; ++o) {
        for (int a = 0; a < 3; ++a) {
            cs.obLoI[o][a] = s.obstacles[o].lo[a];
            cs.obHiI[o][a] = s.obstacles[o].hi[a];
            cs.obLo[o][a] = h->node[a][s.obstacles[o].lo[a]];
            cs.obHi[o][a] = h->node[a][s.obstacles[o].hi[a]];
        }
    }
    cs.nAcc = s.n_species * SACC + CACC;
    cs.maxRejection = MAX_REJECTION;
    cs.maxCrossings = MAX_CROSSINGS;
    cs.maxCellParcels = MAX_ORDERED_CELL;
    cs.capacityLimit = 1LL << 62;
    cs.domAxis = -1;
    cs.domLo = cs.domHi = 0;
}

Parcels& cur_soa(dsmc_handle* h) { return h->buf[h->cur]; }

// The output schedule as of step h->stepHost: resets at output stay on
// until the first output time t with t + deltaT > resetAtOutputUntilTime
// (dsmcField::updateBasicFieldProperties, dsmcField.C:113-150).
void schedule_sync(dsmc_handle* h) {
    const long long wi = h->spec.write_interval_steps;
    const double until = h->spec.reset_at_output_until_time;
    h->resetActive = true;
    if (wi <= 0 || until <= 0) return;
    const long long last = (h->stepHost / wi) * wi;   // the last output step so far
    if (last > 0 && (double)last * h->spec.delta_t + h->spec.delta_t > until) h->resetActive = false;
}

int check_device_error(dsmc_handle* h) {
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    CUDA_TRY(h, cudaMemcpy(h->ctrHost, h->B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost));
    h->stepHost = h->ctrHost->step;
    const unsigned e = h->ctrHost->err;
    if (e) {
        // reported once: the bits are cleared, and the handle steps on (the
        // step that set them is not undone)
        h->ctrHost->err = 0;
        CUDA_TRY(h, cudaMemcpy(&h->B.ctr->err, &h->ctrHost->err, sizeof(unsigned), cudaMemcpyHostToDevice));
        std::string m = "device error bits 0x" + std::to_string(e) + ":";
        if (e & ERRB_CROSSINGS) m += " face-crossing cap reached;";
        if (e & ERRB_REJECTION) m += " acceptance-rejection cap reached;";
        if (e & ERRB_CAPACITY) m += " particle capacity exceeded;";
        if (e & ERRB_BOUNDS) m += " index out of bounds;";
        if (e & ERRB_PATCH) m += " boundary face without a patch;";
        if (e & ERRB_DENSE)
            m += " a cell above " + std::to_string(h->cs.maxCellParcels) +
                 " parcels or 2^24 candidates (its collisions were skipped);";
        if (e & ERRB_IDS) m += " parcel id space exhausted (more than 2^32 parcels inserted since the start);";
        if (e & ERRB_MIGRANT) m += " a migrant for a cell outside this domain (dropped);";
        if (e & ERRB_MIGRANT_CAP) m += " more migrants than the migrant buffer holds (the rest dropped);";
        return fail(h, (e & (ERRB_CAPACITY | ERRB_MIGRANT_CAP)) ? DSMC_ERR_CAPACITY : DSMC_ERR_DEVICE, m);
    }
    return DSMC_OK;
}

// Restart the time averages on stream st (dsmcVolFields' reset at output,
// dsmcVolFields.C:2269-2300): the sampling sums, wall and face sums and the
// selection audit; a pending sample belongs to the window being discarded.
void enqueue_reset(dsmc_handle* h, cudaStream_t st) {
    const CaseDev& cs = h->cs;
    cudaMemsetAsync(h->B.acc, 0, sizeof(double) * cs.C * cs.nAcc, st);
    cudaMemsetAsync(h->B.sfix, 0, sizeof(long long) * cs.C * cs.nSpecies * SACC, st);
    cudaMemsetAsync(h->B.wall, 0, sizeof(double) * cs.nBFaces * W_N, st);
    if (h->B.audit) cudaMemsetAsync(h->B.audit, 0, sizeof(double2) * cs.C, st);
    if (h->B.macc) cudaMemsetAsync(h->B.macc, 0, sizeof(double) * cs.C * cs.nSpecies * MACC, st);
    if (cs.faceFlux) cudaMemsetAsync(cs.faceFlux, 0, sizeof(double) * 2 * cs.nSpecies * cs.nFacesAll, st);
    launch_reset_sample_counters(h->B, st);
}

// Before a step: a reset that an output time left due.
void schedule_pre(dsmc_handle* h, cudaStream_t st) {
    if (!h->resetPending) return;
    enqueue_reset(h, st);
    h->faceStep0 = h->stepHost;
    h->resetPending = false;
}

// After a step: at an output time, a reset is due before the next step (the
// caller reads or writes the output in between), while resets are on.
void schedule_post(dsmc_handle* h) {
    ++h->stepHost;
    const long long wi = h->spec.write_interval_steps;
    if (wi <= 0 || h->stepHost % wi) return;
    if (h->spec.reset_at_output && h->resetActive) h->resetPending = true;
    const double t = (double)h->stepHost * h->spec.delta_t;
    const double until = h->spec.reset_at_output_until_time;
    if (until > 0 && t + h->spec.delta_t > until) h->resetActive = false;
}

// Event marks of a step (enqueue_step with events): the intervals between
// consecutive marks are the kernel groups of dsmc_evolve_kernel_profile, and
// the coarse phases of dsmc_evolve_profiled are unions of them.
enum {
    MK_START = 0,
    MK_ZERO,          // k_zero_step (and the sample flush of a step without a move)
    MK_INFLOW,        // k_inflow_count/scan/fill/commit
    MK_MOVE,          // k_move
    MK_MOVE_SLOW,     // k_move_slow
    MK_SAMPLE,        // k_sample_done/finalize/flushed
    MK_SCAN,          // k_scan_reduce/top/down (k_count_dev before them without a move)
    MK_SCATTER,       // k_scatter_index
    MK_GATHER,        // k_gather
    MK_FINISH,        // k_finish_sort
    MK_LEARNED,       // k_cell_features, k_mlp_infer
    MK_SELECT,        // k_ntc_select/buckets/list, k_cell_order(_big)
    MK_HEAVY,         // k_collide_heavy (k_sbt_collide)
    MK_LIGHT,         // k_collide_light
    MK_PENDING,       // k_set_pending
    MK_END,           // k_end_step
    MK_COUNT
};

// Enqueue one step on the handle's stream (graph capture or direct launch).
// ev: NULL, or MK_COUNT events recorded at the marks above.
// part: 0 the whole step; for a divided cloud 1 the inflow, the move and the
// packed migrants, 2 the rest (received migrants are added in between).
constexpr long long HEAVY_BRANCH_MIN_CELLS = 1LL << 18;

void enqueue_step(dsmc_handle* h, int parity, unsigned phases, cudaEvent_t* ev, int part) {
    const CaseDev& cs = h->cs;
    StepBuffers& B = h->B;
    cudaStream_t st = h->stream;
    Parcels& a = h->buf[parity];
    Parcels& b = h->buf[parity ^ 1];
    auto mark = [&](int k) {
        if (ev) cudaEventRecord(ev[k], st);
    };
    // a step that moves and sorts leaves the plain moves' end points to the gather
    const bool movePending = (phases & DSMC_PHASE_MOVE) && (phases & DSMC_PHASE_SORT);
    if (part != 2) {
        mark(MK_START);
        launch_zero_step(B, st);
        // a sample pending from the previous step is taken by the move
        // kernel, or here when this step does not move
        if (!(phases & DSMC_PHASE_MOVE)) launch_sample_flush(cs, B, a, 0, st);
        mark(MK_ZERO);
        // in a captured step the inflow runs on the side branch while the
        // last step's parcels move (the inserted ones, appended after them,
        // move once it has joined); the profiled steps and divided clouds
        // keep the sequential order
        const bool inflow = (phases & DSMC_PHASE_INFLOW) && h->hasInflow;
        const bool branch = inflow && (phases & DSMC_PHASE_MOVE) && !ev && cs.domAxis < 0;
        if (branch) {
            cudaEventRecord(h->forkEv, st);
            cudaStreamWaitEvent(h->side, h->forkEv, 0);
            launch_inflow(cs, h->inflow, B, a, h->side);
            cudaEventRecord(h->joinEv, h->side);
            launch_move(cs, B, a, st, nullptr, movePending, 1);
            cudaStreamWaitEvent(st, h->joinEv, 0);
            launch_move(cs, B, a, st, nullptr, movePending, 2);
        } else {
            if (inflow) launch_inflow(cs, h->inflow, B, a, st);
            mark(MK_INFLOW);
            if (phases & DSMC_PHASE_MOVE) launch_move(cs, B, a, st, ev ? ev[MK_MOVE] : nullptr, movePending);
            else mark(MK_MOVE);
        }
        mark(MK_MOVE_SLOW);
        if (phases & DSMC_PHASE_MOVE) launch_sample_commit(cs, B, 0, st);
        if (part == 1) {
            launch_pack_migrants(cs, B, a, st);
            return;
        }
        mark(MK_SAMPLE);
    }
    if (phases & DSMC_PHASE_SORT) {
        if (!(phases & DSMC_PHASE_MOVE)) launch_count(cs, B, a, st);
        launch_scan(cs, B, st);
        mark(MK_SCAN);
        launch_scatter(cs, B, a, b, st, ev ? ev[MK_SCATTER] : nullptr, movePending);
        mark(MK_GATHER);
        launch_finish_sort(B, st);
    } else {
        if (phases & DSMC_PHASE_MOVE) cudaMemsetAsync(B.count, 0, sizeof(int) * cs.C, st);
        mark(MK_SCAN);
        mark(MK_SCATTER);
        mark(MK_GATHER);
    }
    mark(MK_FINISH);
    if (phases & DSMC_PHASE_COLLIDE) {
        const Parcels& cur = (phases & DSMC_PHASE_SORT) ? b : a;
        if (h->model) {
            launch_cell_features(cs, B, cur, h->learnEvery, 1, st, h->learnForget);
            mlp_launch_infer(h->model, B.feat, cs.C, B.pred, h->learnMargin, &B.ctr->step, h->learnEvery, st);
        }
        mark(MK_LEARNED);
        // with event marks (the profiled steps) the heavy and light kernels
        // run one after the other so that each is timed alone; the heavy
        // cells' branch only pays on large meshes: for a case of a few
        // thousand cells its fork and join cost more than the overlap gives
        // (256 small heat baths one at a time: 111 -> 118 ms per step)
        const bool heavyBranch = !ev && cs.C >= HEAVY_BRANCH_MIN_CELLS;
        if (heavyBranch) launch_collide(cs, B, cur, h->model ? 1 : 0, st, nullptr, h->side, h->forkEv, h->joinEv);
        else launch_collide(cs, B, cur, h->model ? 1 : 0, st, ev ? ev + MK_SELECT : nullptr);
    } else {
        mark(MK_LEARNED);
        mark(MK_SELECT);
        mark(MK_HEAVY);
    }
    mark(MK_LIGHT);
    // dsmcVolFields samples the state after the collisions; the sums are
    // taken when that state is next streamed (the next move, or a flush);
    // the velocity moments of measureHeatFluxShearStress are taken here
    if (phases & DSMC_PHASE_SAMPLE) {
        if (B.macc) launch_sample_moments(cs, B, (phases & DSMC_PHASE_SORT) ? b : a, st);
        launch_set_pending(B, st);
    }
    mark(MK_PENDING);
    launch_end_step(B, st);
    mark(MK_END);
}

// The coarse phases (inflow, move, sort, collide+sample, bookkeeping) as
// mark intervals [PHASE_MARKS[k], PHASE_MARKS[k + 1]).
const int PHASE_MARKS[6] = {MK_START, MK_INFLOW, MK_SAMPLE, MK_FINISH, MK_PENDING, MK_END};

// Takes a pending sample of the current state (before fields are read,
// checkpointed or reset).
void flush_sample(dsmc_handle* h) { launch_sample_flush(h->cs, h->B, h->buf[h->cur], 1, h->stream); }

int build_graphs(dsmc_handle* h) {
    for (int p = 0; p < 2; ++p) {
        if (h->graph[p]) continue;
        cudaGraph_t g;
        CUDA_TRY(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_step(h, p, DSMC_PHASE_ALL, nullptr, 0);
        CUDA_TRY(h, cudaStreamEndCapture(h->stream, &g));
        CUDA_TRY(h, cudaGraphInstantiate(&h->graph[p], g, 0));
        h->graphT[p] = g;
    }
    return DSMC_OK;
}

// The step graphs hold the launch shape and the selection mode: drop them
// when either changes (they are captured again on the next step).
void drop_graphs(dsmc_handle* h) {
    ++h->graphGen;
    for (int p = 0; p < 2; ++p) {
        if (h->graph[p]) cudaGraphExecDestroy(h->graph[p]);
        if (h->graphT[p]) cudaGraphDestroy(h->graphT[p]);
        if (h->half1[p]) cudaGraphExecDestroy(h->half1[p]);
        if (h->half2[p]) cudaGraphExecDestroy(h->half2[p]);
        h->graph[p] = nullptr;
        h->graphT[p] = nullptr;
        h->half1[p] = h->half2[p] = nullptr;
    }
}

// The two halves of a divided cloud's step, captured per parity.
int build_half_graphs(dsmc_handle* h) {
    for (int p = 0; p < 2; ++p) {
        for (int part = 1; part <= 2; ++part) {
            cudaGraphExec_t& ex = part == 1 ? h->half1[p] : h->half2[p];
            if (ex) continue;
            cudaGraph_t g;
            CUDA_TRY(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            enqueue_step(h, p, DSMC_PHASE_ALL, nullptr, part);
            CUDA_TRY(h, cudaStreamEndCapture(h->stream, &g));
            const cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            CUDA_TRY(h, e);
        }
    }
    return DSMC_OK;
}

// The whole-step entry points do not run a divided cloud (its migrants
// must be handed over between the two halves).
int refuse_divided(dsmc_handle* h, const char* fn) {
    if (h->cs.domAxis < 0) return DSMC_OK;
    return fail(h, DSMC_ERR_INVALID,
                std::string(fn) + ": the cloud is divided (dsmc_set_domain); it steps with dsmc_step_begin, "
                                  "dsmc_get_migrants / dsmc_add_migrants and dsmc_step_end");
}

int sort_current(dsmc_handle* h, long long n) {
    // particles [0,n) of the current buffer: recompute cells, count, scan, scatter
    const CaseDev& cs = h->cs;
    StepBuffers& B = h->B;
    cudaStream_t st = h->stream;
    Counters c{};
    CUDA_TRY(h, cudaMemcpy(h->ctrHost, B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost));
    c = *h->ctrHost;
    c.n = n;
    c.nMoved = n;
    c.nMig = 0;
    c.migIn = 0;
    *h->ctrHost = c;
    CUDA_TRY(h, cudaMemcpy(B.ctr, h->ctrHost, sizeof(Counters), cudaMemcpyHostToDevice));
    launch_cellw(cs, cur_soa(h), n, st);
    CUDA_TRY(h, cudaMemsetAsync(B.count, 0, sizeof(int) * cs.C, st));
    launch_count_n(cur_soa(h), n, B.count, st);
    launch_scan(cs, B, st);
    launch_scatter(cs, B, h->buf[h->cur], h->buf[h->cur ^ 1], st);
    launch_finish_sort(B, st);
    h->cur ^= 1;
    CUDA_TRY(h, cudaGetLastError());
    return check_device_error(h);
}

}  // namespace

namespace dsmc {
void set_global_error(const std::string& msg) { g_err = msg; }
}

extern "C" {

void dsmc_spec_defaults(dsmc_case_spec* s) {
    std::memset(s, 0, sizeof(*s));
    s->tref = 273.0;
    s->zrot = 5.0;
    s->fixed_zv = 0.0;
    s->inv_zv_formulation = 2;
    s->mfp_tref = 273.0;
    s->measure_mean_free_path = 1;
    s->binary_collision_model = DSMC_COLL_VHS;
    s->partner_selection_model = DSMC_SEL_NTC;
}

const char* dsmc_last_global_error(void) { return g_err.c_str(); }
const char* dsmc_last_error(const dsmc_handle* h) { return h ? h->err.c_str() : g_err.c_str(); }

int dsmc_create_from_spec(const dsmc_case_spec* spec, dsmc_handle** out) {
    *out = nullptr;
    std::unique_ptr<dsmc_handle> hp(new dsmc_handle());
    dsmc_handle* h = hp.get();
    int rc = validate(h, *spec);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(h, DSMC_ERR_NO_DEVICE, "no CUDA device: this library has no CPU path");
    CUDA_TRY(h, cudaGetDevice(&h->device));
    h->spec = *spec;
    for (int q = 0; q < 6; ++q) {
        if (spec->face_patch[q]) {
            const int a = q / 2;
            const int b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
            h->facePatch.emplace_back(spec->face_patch[q],
                                      spec->face_patch[q] + (long long)spec->n_cells[b] * spec->n_cells[c]);
            h->spec.face_patch[q] = h->facePatch.back().data();
        }
    }
    for (int a = 0; a < 3; ++a) {
        h->node[a].resize((size_t)spec->n_cells[a] + 1);
        for (int i = 0; i <= spec->n_cells[a]; ++i)
            h->node[a][i] = spec->node_coords[a] ? spec->node_coords[a][i]
                                                 : spec->origin[a] + i * spec->cell_size[a];
        h->spec.node_coords[a] = spec->node_coords[a] ? h->node[a].data() : nullptr;
        h->width[a].resize((size_t)spec->n_cells[a]);
        for (int i = 0; i < spec->n_cells[a]; ++i)
            h->width[a][i] = spec->node_coords[a] ? h->node[a][i + 1] - h->node[a][i] : spec->cell_size[a];
    }
    fill_case_dev(h);
    CaseDev& cs = h->cs;
    std::vector<int> bfPatch;
    std::vector<long long> inflowFace;
    std::vector<int> inflowSide, inflowCell;
    build_faces(h, bfPatch, inflowFace, inflowSide, inflowCell);
    for (size_t f = 0; f < bfPatch.size(); ++f)
        if (bfPatch[f] < 0 || bfPatch[f] >= spec->n_patches)
            return fail(h, DSMC_ERR_INVALID, "boundary face " + std::to_string(f) + " has no patch");

    // capacity
    std::vector<unsigned char> solid(cs.C, 0);
    long long fluid = cs.C;
    for (int o = 0; o < spec->n_obstacles; ++o) {
        const dsmc_obstacle& ob = spec->obstacles[o];
        for (int k = ob.lo[2]; k < ob.hi[2]; ++k)
            for (int j = ob.lo[1]; j < ob.hi[1]; ++j)
                for (int i = ob.lo[0]; i < ob.hi[0]; ++i) {
                    unsigned char& sv = solid[i + (long long)cs.n[0] * (j + (long long)cs.n[1] * k)];
                    if (!sv) { sv = 1; --fluid; }
                }
    }
    double ndSum = 0, fluidV = 0;
    for (int m = 0; m < spec->n_species; ++m) ndSum += spec->init_number_density[m];
    for (long long c = 0; c < cs.C; ++c)
        if (!solid[c])
            fluidV += h->width[0][c % cs.n[0]] * h->width[1][(c / cs.n[0]) % cs.n[1]] *
                      h->width[2][c / ((long long)cs.n[0] * cs.n[1])];
    h->nFluid = fluid;
    h->solidHost = solid;
    h->expectedN = (long long)(ndSum * fluidV / cs.FN);
    long long cap = spec->max_particles;
    if (cap <= 0) cap = (long long)((h->hasInflow ? 2.0 : 1.3) * h->expectedN) + 65536;
    // parcel indices are 32-bit in the sort's slots, the boundary-path and
    // migrant lists and the collision queues
    if (cap > 0x7FFFFFFFLL)
        return fail(h, DSMC_ERR_CAPACITY, "a cloud holds at most 2^31 - 1 parcels (capacity " + std::to_string(cap) +
                                              "): divide the case into domains (dsmc_set_domain)");
    h->B.capacity = cap;

    CUDA_TRY(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    CUDA_TRY(h, cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
    CUDA_TRY(h, cudaEventCreateWithFlags(&h->forkEv, cudaEventDisableTiming));
    CUDA_TRY(h, cudaEventCreateWithFlags(&h->joinEv, cudaEventDisableTiming));
    if (collide_init()) return fail(h, DSMC_ERR_CUDA, "cannot raise the shared-memory limit of the cell-order kernel");
    StepBuffers& B = h->B;
    if ((rc = alloc_soa(h, &h->buf[0], cap))) return rc;
    if ((rc = alloc_soa(h, &h->buf[1], cap))) return rc;
    if ((rc = dalloc(h, &B.count, cs.C))) return rc;
    if ((rc = dalloc(h, &B.start, cs.C + 1))) return rc;
    if ((rc = dalloc(h, &B.blockSums, scan_scratch_ints(cs.C) + 1))) return rc;
    if ((rc = dalloc(h, &B.smax, cs.C))) return rc;
    if ((rc = dalloc(h, &B.rem, cs.C))) return rc;
    if ((rc = dalloc(h, &B.acc, cs.C * cs.nAcc))) return rc;
    if ((rc = dalloc(h, &B.sfix, cs.C * cs.nSpecies * SACC))) return rc;
    if (spec->measure_heat_flux_shear_stress && (rc = dalloc(h, &B.macc, cs.C * cs.nSpecies * MACC))) return rc;
    if ((rc = dalloc(h, &B.wall, cs.nBFaces * W_N))) return rc;
    if ((rc = dalloc(h, &B.bfPatch, cs.nBFaces))) return rc;
    if ((rc = dalloc(h, &B.bigList, cs.C))) return rc;
    if ((rc = dalloc(h, &B.work, cs.C))) return rc;
    if ((rc = dalloc(h, &B.ncCell, cs.C))) return rc;
    if ((rc = dalloc(h, &B.buckets, 32))) return rc;
    if ((rc = dalloc(h, &B.perm, cap))) return rc;
    if ((rc = dalloc(h, &B.subs, cs.C))) return rc;
    if ((rc = dalloc(h, &B.obsMax, cs.C))) return rc;
    if ((rc = dalloc(h, &B.feat, cs.C))) return rc;
    if ((rc = dalloc(h, &B.pred, cs.C))) return rc;
    if ((rc = dalloc(h, &B.useR, cs.C))) return rc;
    if ((rc = dalloc(h, &B.exceed, cs.C))) return rc;
    if ((rc = dalloc(h, &B.smaxSel, cs.C))) return rc;
    if ((rc = dalloc(h, &B.slowList, cap))) return rc;
    if ((rc = dalloc(h, &B.sortSrc, cap))) return rc;
    if ((rc = dalloc(h, &B.ctr, 1))) return rc;
    if ((rc = dalloc(h, &h->solid, cs.C))) return rc;
    if ((rc = dalloc(h, &h->info6, 8))) return rc;
    if ((rc = dalloc(h, &h->fieldTmp, cs.C))) return rc;
    if ((rc = dalloc(h, &h->packFlags, 2))) return rc;
    B.nInflowFaces = (int)inflowFace.size();
    const long long ni = (long long)B.nInflowFaces * spec->n_species;
    if ((rc = dalloc(h, &B.inflowFace, B.nInflowFaces))) return rc;
    if ((rc = dalloc(h, &B.inflowSide, B.nInflowFaces))) return rc;
    if ((rc = dalloc(h, &B.inflowCell, B.nInflowFaces))) return rc;
    if ((rc = dalloc(h, &B.inflowAcc, ni))) return rc;
    if ((rc = dalloc(h, &B.inflowCount, ni))) return rc;
    if ((rc = dalloc(h, &B.inflowOff, ni + 1))) return rc;
    if ((rc = dalloc(h, &B.inflowOffLocal, ni + 1))) return rc;
    if ((rc = dalloc(h, &B.inflowTerm, ni))) return rc;
    // graded mesh: half-node tables, cell volumes and boundary-face areas
    if (spec->node_coords[0] || spec->node_coords[1] || spec->node_coords[2]) {
        for (int a = 0; a < 3; ++a) {
            if (!spec->node_coords[a]) continue;
            const int na = cs.n[a];
            std::vector<double> hv((size_t)2 * na + 1);
            for (int i = 0; i <= na; ++i) hv[2 * (size_t)i] = h->node[a][i];
            for (int i = 0; i < na; ++i) hv[2 * (size_t)i + 1] = 0.5 * (h->node[a][i] + h->node[a][i + 1]);
            double* d = nullptr;
            if ((rc = dalloc(h, &d, (long long)hv.size()))) return rc;
            CUDA_TRY(h, cudaMemcpy(d, hv.data(), sizeof(double) * hv.size(), cudaMemcpyHostToDevice));
            cs.half[a] = d;
        }
        std::vector<double> vol((size_t)cs.C);
        for (long long c = 0; c < cs.C; ++c) {
            const long long i = c % cs.n[0], j = (c / cs.n[0]) % cs.n[1], k = c / ((long long)cs.n[0] * cs.n[1]);
            vol[(size_t)c] = h->width[0][i] * h->width[1][j] * h->width[2][k];
        }
        double* dv = nullptr;
        double* da = nullptr;
        if ((rc = dalloc(h, &dv, cs.C))) return rc;
        if ((rc = dalloc(h, &da, cs.nBFaces))) return rc;
        CUDA_TRY(h, cudaMemcpy(dv, vol.data(), sizeof(double) * vol.size(), cudaMemcpyHostToDevice));
        CUDA_TRY(h, cudaMemcpy(da, h->bfAreaHost.data(), sizeof(double) * cs.nBFaces, cudaMemcpyHostToDevice));
        cs.cellV = dv;
        cs.bfArea = da;
    }
    // 1/Zv by quantised level (postCollisionVibrationalEnergyLevel, dsmcCloud.C:1420-1490)
    {
        std::vector<double> tab((size_t)DSMC_MAX_SPECIES * DSMC_MAX_SPECIES * ZV_TAB, 0.0);
        for (int p = 0; p < spec->n_species; ++p) {
            const dsmc_species& sp = spec->species[p];
            if (sp.n_vib_modes == 0) continue;
            for (int q = 0; q < spec->n_species; ++q) {
                const double omega = 0.5 * (sp.omega + spec->species[q].omega);
                double* row = &tab[(size_t)(p * DSMC_MAX_SPECIES + q) * ZV_TAB];
                for (int iMax = 1; iMax < ZV_TAB; ++iMax) {
                    const double T = iMax * sp.theta_v / (3.5 - omega);
                    const double pow1 = std::pow(sp.theta_d / T, 1. / 3.) - 1.0;
                    const double pow2 = std::pow(sp.theta_d / sp.tref_zv, 1. / 3.) - 1.0;
                    const double ZvP1 = std::pow(sp.theta_d / T, omega);
                    const double ZvP2 = std::pow(sp.zref * std::pow(sp.theta_d / sp.tref_zv, -omega), pow1 / pow2);
                    const double Zv = ZvP1 * ZvP2;
                    row[iMax] = (spec->inv_zv_formulation == 2) ? 1.0 / (5.0 * Zv) : 1.0 / Zv;
                }
            }
        }
        double* dtab = nullptr;
        if ((rc = dalloc(h, &dtab, (long long)tab.size()))) return rc;
        CUDA_TRY(h, cudaMemcpy(dtab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice));
        cs.invZvTab = dtab;
    }
    CUDA_TRY(h, cudaMemcpy(B.bfPatch, bfPatch.data(), sizeof(int) * bfPatch.size(), cudaMemcpyHostToDevice));
    CUDA_TRY(h, cudaMemcpy(h->solid, solid.data(), cs.C, cudaMemcpyHostToDevice));
    if (B.nInflowFaces) {
        CUDA_TRY(h, cudaMemcpy(B.inflowFace, inflowFace.data(), sizeof(long long) * inflowFace.size(),
                               cudaMemcpyHostToDevice));
        CUDA_TRY(h, cudaMemcpy(B.inflowSide, inflowSide.data(), sizeof(int) * inflowSide.size(),
                               cudaMemcpyHostToDevice));
        CUDA_TRY(h, cudaMemcpy(B.inflowCell, inflowCell.data(), sizeof(int) * inflowCell.size(),
                               cudaMemcpyHostToDevice));
        // the Bird eq. 4.22 number of parcels per step through each inflow
        // face (dsmcFreeStreamInflowPatch.C:96-141): constant in time, so it
        // is evaluated once, here
        std::vector<double> term((size_t)ni, 0.0);
        const double sqrtPi = std::sqrt(PI);
        for (size_t f = 0; f < inflowFace.size(); ++f) {
            const int sd = inflowSide[f];
            const int a = sd / 2;
            const int b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
            const double sgnOut = (sd & 1) ? 1.0 : -1.0;
            (void)b; (void)c;
            const double fA = h->bfAreaHost[(size_t)inflowFace[f]];
            const int pi = bfPatch[(size_t)inflowFace[f]];
            const dsmc_patch& pt = spec->patches[pi];
            for (int m = 0; m < spec->n_species; ++m) {
                const double nd = pt.inflow_number_density[m];
                if (!(nd > 0)) continue;
                const double cmp = std::sqrt(2.0 * kB * pt.inflow_t_tra / spec->species[m].mass);
                const double sCos = (pt.inflow_velocity[a] * (-sgnOut)) / cmp;
                term[f * spec->n_species + m] =
                    (fA * nd * spec->delta_t * cmp * (std::exp(-sCos * sCos) + sqrtPi * sCos * (1 + std::erf(sCos)))) /
                    (2.0 * sqrtPi * spec->n_equivalent_particles);
            }
        }
        CUDA_TRY(h, cudaMemcpy(B.inflowTerm, term.data(), sizeof(double) * term.size(), cudaMemcpyHostToDevice));
    }
    void* pinned = nullptr;
    CUDA_TRY(h, cudaMallocHost(&pinned, sizeof(Counters)));
    h->ctrHost = static_cast<Counters*>(pinned);
    std::memset(h->ctrHost, 0, sizeof(Counters));
    launch_remainder_init(cs, B.rem, h->stream);
    CUDA_TRY(h, cudaGetLastError());
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    *out = hp.release();
    return DSMC_OK;
}

void dsmc_destroy(dsmc_handle* h) {
    if (!h) return;
    if (h->batchOwned) {
        // the batch still steps this case: leave it to dsmc_batch_destroy
        h->err = "dsmc_destroy: the case belongs to a batch (dsmc_batch_destroy frees it)";
        return;
    }
    if (h->stream) cudaStreamSynchronize(h->stream);
    drop_graphs(h);
    if (h->B.migIn) cudaFree(h->B.migIn);
    for (void* q : h->allocs) cudaFree(q);
    if (h->ctrHost) cudaFreeHost(h->ctrHost);
    if (h->ctrRing) cudaFreeHost(h->ctrRing);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->side) cudaStreamDestroy(h->side);
    if (h->forkEv) cudaEventDestroy(h->forkEv);
    if (h->joinEv) cudaEventDestroy(h->joinEv);
    delete h;
}

// sigmaTcRMax = sigmaT * most probable speed of the most abundant species at
// the initial temperature (dsmcMeshFill's starting value)
int init_smax(dsmc_handle* h) {
    const dsmc_case_spec& s = h->spec;
    int most = 0;
    for (int m = 1; m < s.n_species; ++m)
        if (s.init_number_density[m] > s.init_number_density[most]) most = m;
    const dsmc_species& sp = s.species[most];
    const double T = s.init_t_tra > 0 ? s.init_t_tra : 273.0;
    const double smax = PI * sp.diameter * sp.diameter * std::sqrt(2.0 * kB * T / sp.mass);
    std::vector<double> sm(h->cs.C, smax);
    CUDA_TRY(h, cudaMemcpy(h->B.smax, sm.data(), sizeof(double) * h->cs.C, cudaMemcpyHostToDevice));
    h->smaxSet = true;
    return DSMC_OK;
}

int dsmc_initialise(dsmc_handle* h) {
    const CaseDev& cs = h->cs;
    StepBuffers& B = h->B;
    cudaStream_t st = h->stream;
    const dsmc_case_spec& s = h->spec;
    // device copy of the number densities in the info scratch
    double nd[DSMC_MAX_SPECIES] = {0};
    for (int m = 0; m < s.n_species; ++m) nd[m] = s.init_number_density[m];
    double* dnd = nullptr;
    CUDA_TRY(h, cudaMalloc(&dnd, sizeof(nd)));
    CUDA_TRY(h, cudaMemcpy(dnd, nd, sizeof(nd), cudaMemcpyHostToDevice));
    CUDA_TRY(h, cudaMemsetAsync(B.count, 0, sizeof(int) * cs.C, st));
    launch_init_count(cs, dnd, h->solid, B.count, st);
    launch_scan(cs, B, st);
    CUDA_TRY(h, cudaStreamSynchronize(st));
    int total = 0;
    CUDA_TRY(h, cudaMemcpy(&total, B.start + cs.C, sizeof(int), cudaMemcpyDeviceToHost));
    if (total > B.capacity) {
        cudaFree(dnd);
        return fail(h, DSMC_ERR_CAPACITY, "initial fill of " + std::to_string(total) +
                                              " parcels exceeds capacity " + std::to_string(B.capacity));
    }
    const double Txyz[3] = {s.init_t_tra_xyz[0], s.init_t_tra_xyz[1], s.init_t_tra_xyz[2]};
    const double U[3] = {s.init_velocity[0], s.init_velocity[1], s.init_velocity[2]};
    launch_init_fill(cs, B, cur_soa(h), dnd, h->solid, B.start, s.init_t_tra, Txyz, s.init_t_rot, s.init_t_vib,
                     U, st);
    CUDA_TRY(h, cudaGetLastError());
    CUDA_TRY(h, cudaStreamSynchronize(st));
    cudaFree(dnd);
    int rc0 = init_smax(h);
    if (rc0) return rc0;
    CUDA_TRY(h, cudaMemcpy(h->ctrHost, B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost));
    h->ctrHost->nextId = total;
    CUDA_TRY(h, cudaMemcpy(B.ctr, h->ctrHost, sizeof(Counters), cudaMemcpyHostToDevice));
    return sort_current(h, total);
}

int dsmc_evolve(dsmc_handle* h, long long n) {
    int rc = refuse_divided(h, "dsmc_evolve");
    if (rc) return rc;
    rc = build_graphs(h);
    if (rc) return rc;
    for (long long i = 0; i < n; ++i) {
        schedule_pre(h, h->stream);
        CUDA_TRY(h, cudaGraphLaunch(h->graph[h->cur], h->stream));
        h->cur ^= 1;
        schedule_post(h);
    }
    return check_device_error(h);
}

// n steps enqueued with the events of every mark; per_mark[k] receives the
// summed time of interval k (mark k to mark k + 1), total the first-to-last
// event time.
int profile_steps(dsmc_handle* h, long long n, double* per_mark, double* total_ms) {
    if (n <= 0) return fail(h, DSMC_ERR_INVALID, "n must be positive");
    if (int rc = refuse_divided(h, "the profiled steps")) return rc;
    std::vector<cudaEvent_t> ev((size_t)n * MK_COUNT);
    for (auto& e : ev) CUDA_TRY(h, cudaEventCreate(&e));
    for (long long i = 0; i < n; ++i) {
        schedule_pre(h, h->stream);
        enqueue_step(h, h->cur, DSMC_PHASE_ALL, &ev[(size_t)i * MK_COUNT], 0);
        h->cur ^= 1;
        schedule_post(h);
    }
    CUDA_TRY(h, cudaGetLastError());
    int rc = check_device_error(h);
    for (int k = 0; k + 1 < MK_COUNT; ++k) per_mark[k] = 0.0;
    for (long long i = 0; i < n; ++i) {
        for (int k = 0; k + 1 < MK_COUNT; ++k) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ev[(size_t)i * MK_COUNT + k], ev[(size_t)i * MK_COUNT + k + 1]);
            per_mark[k] += ms;
        }
    }
    float tot = 0;
    cudaEventElapsedTime(&tot, ev[0], ev[(size_t)(n - 1) * MK_COUNT + MK_END]);
    for (auto& e : ev) cudaEventDestroy(e);
    if (total_ms) *total_ms = tot;
    return rc;
}

int dsmc_evolve_profiled(dsmc_handle* h, long long n, double* phase_ms, double* total_ms) {
    double per[MK_COUNT] = {0};
    const int rc = profile_steps(h, n, per, total_ms);
    if (n <= 0) return rc;
    for (int k = 0; k < 5; ++k) {
        double sum = 0;
        for (int m = PHASE_MARKS[k]; m < PHASE_MARKS[k + 1]; ++m) sum += per[m];
        if (phase_ms) phase_ms[k] = sum;
        h->phaseMs[k] = sum / (double)n;
    }
    return rc;
}

int dsmc_evolve_kernel_profile(dsmc_handle* h, long long n, double* group_ms, int n_groups, double* total_ms) {
    if (n_groups < 0) return fail(h, DSMC_ERR_INVALID, "n_groups must not be negative");
    double per[MK_COUNT] = {0};
    const int rc = profile_steps(h, n, per, total_ms);
    for (int k = 0; k < n_groups && k + 1 < MK_COUNT; ++k) group_ms[k] = per[k];
    return rc;
}

int dsmc_evolve_timed(dsmc_handle* h, long long n, double* total_ms) {
    int rc = refuse_divided(h, "dsmc_evolve_timed");
    if (rc) return rc;
    rc = build_graphs(h);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    CUDA_TRY(h, cudaEventCreate(&e0));
    CUDA_TRY(h, cudaEventCreate(&e1));
    CUDA_TRY(h, cudaEventRecord(e0, h->stream));
    for (long long i = 0; i < n; ++i) {
        schedule_pre(h, h->stream);
        CUDA_TRY(h, cudaGraphLaunch(h->graph[h->cur], h->stream));
        h->cur ^= 1;
        schedule_post(h);
    }
    CUDA_TRY(h, cudaEventRecord(e1, h->stream));
    rc = check_device_error(h);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (total_ms) *total_ms = ms;
    return rc;
}

int dsmc_run_phases(dsmc_handle* h, unsigned phases) {
    if (int rc = refuse_divided(h, "dsmc_run_phases")) return rc;
    cudaEvent_t ev[MK_COUNT];
    for (int k = 0; k < MK_COUNT; ++k) cudaEventCreate(&ev[k]);
    if (phases == DSMC_PHASE_ALL) schedule_pre(h, h->stream);
    enqueue_step(h, h->cur, phases, ev, 0);
    if (phases == DSMC_PHASE_ALL) schedule_post(h);
    CUDA_TRY(h, cudaGetLastError());
    if (phases & DSMC_PHASE_SORT) h->cur ^= 1;
    int rc = check_device_error(h);
    for (int k = 0; k < 5; ++k) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ev[PHASE_MARKS[k]], ev[PHASE_MARKS[k + 1]]);
        h->phaseMs[k] = ms;
    }
    for (int k = 0; k < MK_COUNT; ++k) cudaEventDestroy(ev[k]);
    return rc;
}

int dsmc_phase_times(dsmc_handle* h, double* a, double* b, double* c, double* d, double* e) {
    // times of the last dsmc_run_phases call: inflow, move, sort, collide+sample, end
    if (a) *a = h->phaseMs[0];
    if (b) *b = h->phaseMs[1];
    if (c) *c = h->phaseMs[2];
    if (d) *d = h->phaseMs[3];
    if (e) *e = h->phaseMs[4];
    return DSMC_OK;
}

// Device -> host parcel reads go through chunks of packed records
// (PACK_CHUNK parcels at a time); writes are packed on the device.
constexpr long long PACK_CHUNK = 1 << 20;

int dsmc_set_particles(dsmc_handle* h, long long n, const double* pos, const double* U, const double* erot,
                       const int* vib, const int* species, const unsigned* id) {
    if (n < 0 || n > h->B.capacity) return fail(h, DSMC_ERR_CAPACITY, "particle count exceeds capacity");
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    // the arrays are copied as they are into the spare buffer (68 B per parcel
    // of room: 56 B of doubles and two int arrays in its records, the ids in
    // its cell words) and packed into records on the device
    Parcels& s = cur_soa(h);
    Parcels& spare = h->buf[h->cur ^ 1];
    char* base = reinterpret_cast<char*>(spare.r);
    const size_t N = (size_t)n;
    double* dPos = pos ? reinterpret_cast<double*>(base) : nullptr;
    double* dU = U ? reinterpret_cast<double*>(base + 24 * N) : nullptr;
    double* dE = erot ? reinterpret_cast<double*>(base + 48 * N) : nullptr;
    int* dVib = vib ? reinterpret_cast<int*>(base + 56 * N) : nullptr;
    int* dSp = species ? reinterpret_cast<int*>(base + 60 * N) : nullptr;
    unsigned* dId = id ? spare.cellw : nullptr;
    cudaStream_t st = h->stream;
    if (n > 0) {
        if (pos) CUDA_TRY(h, cudaMemcpyAsync(dPos, pos, 24 * N, cudaMemcpyHostToDevice, st));
        if (U) CUDA_TRY(h, cudaMemcpyAsync(dU, U, 24 * N, cudaMemcpyHostToDevice, st));
        if (erot) CUDA_TRY(h, cudaMemcpyAsync(dE, erot, 8 * N, cudaMemcpyHostToDevice, st));
        if (vib) CUDA_TRY(h, cudaMemcpyAsync(dVib, vib, 4 * N, cudaMemcpyHostToDevice, st));
        if (species) CUDA_TRY(h, cudaMemcpyAsync(dSp, species, 4 * N, cudaMemcpyHostToDevice, st));
        if (id) CUDA_TRY(h, cudaMemcpyAsync(dId, id, 4 * N, cudaMemcpyHostToDevice, st));
    }
    // check first: a rejected call leaves the cloud as it was
    CUDA_TRY(h, cudaMemsetAsync(h->packFlags, 0, 2 * sizeof(unsigned), st));
    launch_pack(s, n, dPos, dU, dE, dVib, dSp, dId, h->spec.n_species, h->packFlags, 0, st);
    CUDA_TRY(h, cudaGetLastError());
    unsigned flags[2] = {0, 0};
    CUDA_TRY(h, cudaMemcpyAsync(flags, h->packFlags, sizeof(flags), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(h, cudaStreamSynchronize(st));
    if (flags[0] & 1u) return fail(h, DSMC_ERR_INVALID, "species index out of range");
    if (flags[0] & 2u) return fail(h, DSMC_ERR_INVALID, "vibrational level out of range");
    launch_pack(s, n, dPos, dU, dE, dVib, dSp, dId, h->spec.n_species, h->packFlags, 1, st);
    CUDA_TRY(h, cudaGetLastError());
    CUDA_TRY(h, cudaMemcpy(h->ctrHost, h->B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost));
    h->ctrHost->nextId = flags[1];
    CUDA_TRY(h, cudaMemcpy(h->B.ctr, h->ctrHost, sizeof(Counters), cudaMemcpyHostToDevice));
    return sort_current(h, n);
}

int dsmc_get_particles(dsmc_handle* h, long long capacity, long long* n_out, double* pos, double* U, double* erot,
                       int* vib, int* species, unsigned* id, int* cell) {
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    CUDA_TRY(h, cudaMemcpy(h->ctrHost, h->B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost));
    const long long n = h->ctrHost->n;
    if (n_out) *n_out = n;
    if (capacity < n) return fail(h, DSMC_ERR_CAPACITY, "output capacity smaller than the particle count");
    Parcels& s = cur_soa(h);
    std::vector<Rec> rec((size_t)std::min(n, PACK_CHUNK));
    std::vector<uint32_t> cw((size_t)std::min(n, PACK_CHUNK));
    for (long long c0 = 0; c0 < n; c0 += PACK_CHUNK) {
        const long long m = std::min(PACK_CHUNK, n - c0);
        CUDA_TRY(h, cudaMemcpy(rec.data(), s.r + c0, sizeof(Rec) * m, cudaMemcpyDeviceToHost));
        if (cell) CUDA_TRY(h, cudaMemcpy(cw.data(), s.cellw + c0, sizeof(uint32_t) * m, cudaMemcpyDeviceToHost));
        for (long long k = 0; k < m; ++k) {
            const long long i = c0 + k;
            const Rec& r = rec[k];
            if (pos) { pos[3 * i] = r.x; pos[3 * i + 1] = r.y; pos[3 * i + 2] = r.z; }
            if (U) { U[3 * i] = r.ux; U[3 * i + 1] = r.uy; U[3 * i + 2] = r.uz; }
            if (erot) erot[i] = r.erot;
            if (vib) vib[i] = sv_vib(r.sv);
            if (species) species[i] = sv_species(r.sv);
            if (id) id[i] = r.id;
            if (cell) cell[i] = cw[k] == CELLW_DELETED ? -1 : (int)cellw_cell(cw[k]);
        }
    }
    return DSMC_OK;
}

int dsmc_get_cell_array(dsmc_handle* h, const char* name, void* out, long long n) {
    const std::string nm(name);
    const long long C = h->cs.C;
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    if (nm == "count" || nm == "start") {
        if (n != C) return fail(h, DSMC_ERR_INVALID, "n must equal the number of cells");
        std::vector<int> st(C + 1);
        CUDA_TRY(h, cudaMemcpy(st.data(), h->B.start, sizeof(int) * (C + 1), cudaMemcpyDeviceToHost));
        int* o = static_cast<int*>(out);
        for (long long c = 0; c < C; ++c) o[c] = (nm == "start") ? st[c] : st[c + 1] - st[c];
        return DSMC_OK;
    }
    if (nm == "sigmaTcRMax" || nm == "collisionSelectionRemainder") {
        if (n != C) return fail(h, DSMC_ERR_INVALID, "n must equal the number of cells");
        CUDA_TRY(h, cudaMemcpy(out, nm == "sigmaTcRMax" ? h->B.smax : h->B.rem, sizeof(double) * C,
                               cudaMemcpyDeviceToHost));
        return DSMC_OK;
    }
    if (nm == "accumulators") {
        if (n != C * h->cs.nAcc) return fail(h, DSMC_ERR_INVALID, "n must equal cells x accumulators");
        flush_sample(h);
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        CUDA_TRY(h, cudaMemcpy(out, h->B.acc, sizeof(double) * n, cudaMemcpyDeviceToHost));
        return DSMC_OK;
    }
    if (nm == "selectionAudit") {
        if (n != 2 * C) return fail(h, DSMC_ERR_INVALID, "n must equal 2 x the number of cells");
        if (!h->B.audit) return fail(h, DSMC_ERR_INVALID, "the selection audit is off (dsmc_set_selection_audit)");
        CUDA_TRY(h, cudaMemcpy(out, h->B.audit, sizeof(double2) * C, cudaMemcpyDeviceToHost));
        return DSMC_OK;
    }
    if (nm == "learnedFeatures") {
        // the learned maximum's inputs of the current state, per cell: log
        // number density, log translational temperature, speed ratio, valid
        if (n != 4 * C) return fail(h, DSMC_ERR_INVALID, "n must equal 4 x the number of cells");
        launch_cell_features(h->cs, h->B, cur_soa(h), 0, 0, h->stream);
        CUDA_TRY(h, cudaGetLastError());
        CUDA_TRY(h, cudaMemcpyAsync(out, h->B.feat, sizeof(float4) * C, cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        return DSMC_OK;
    }
    if (nm == "inflowAccumulator") {
        const int ns = h->spec.n_species;
        if (n != h->cs.nBFaces * ns) return fail(h, DSMC_ERR_INVALID, "n must equal boundary faces x species");
        std::vector<double> acc((size_t)h->B.nInflowFaces * ns);
        std::vector<long long> face((size_t)h->B.nInflowFaces);
        if (!acc.empty()) {
            CUDA_TRY(h, cudaMemcpy(acc.data(), h->B.inflowAcc, sizeof(double) * acc.size(), cudaMemcpyDeviceToHost));
            CUDA_TRY(h, cudaMemcpy(face.data(), h->B.inflowFace, sizeof(long long) * face.size(),
                                   cudaMemcpyDeviceToHost));
        }
        double* o = static_cast<double*>(out);
        std::fill(o, o + n, 0.0);
        for (size_t f = 0; f < face.size(); ++f)
            for (int m = 0; m < ns; ++m) o[face[f] * ns + m] = acc[f * ns + m];
        return DSMC_OK;
    }
    return fail(h, DSMC_ERR_INVALID, "unknown cell array " + nm +
                                         "; valid: count start sigmaTcRMax collisionSelectionRemainder accumulators "
                                         "inflowAccumulator selectionAudit learnedFeatures");
}

int dsmc_set_cell_array(dsmc_handle* h, const char* name, const void* in, long long n) {
    const std::string nm(name);
    const long long C = h->cs.C;
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    if (nm == "inflowAccumulator") {
        const int ns = h->spec.n_species;
        if (n != h->cs.nBFaces * ns) return fail(h, DSMC_ERR_INVALID, "n must equal boundary faces x species");
        std::vector<long long> face((size_t)h->B.nInflowFaces);
        if (face.empty()) return DSMC_OK;
        CUDA_TRY(h, cudaMemcpy(face.data(), h->B.inflowFace, sizeof(long long) * face.size(), cudaMemcpyDeviceToHost));
        const double* v = static_cast<const double*>(in);
        std::vector<double> acc(face.size() * ns);
        for (size_t f = 0; f < face.size(); ++f)
            for (int m = 0; m < ns; ++m) acc[f * ns + m] = v[face[f] * ns + m];
        CUDA_TRY(h, cudaMemcpy(h->B.inflowAcc, acc.data(), sizeof(double) * acc.size(), cudaMemcpyHostToDevice));
        return DSMC_OK;
    }
    if (n != C) return fail(h, DSMC_ERR_INVALID, "n must equal the number of cells");
    if (nm == "sigmaTcRMax" || nm == "collisionSelectionRemainder") {
        if (nm == "sigmaTcRMax") h->smaxSet = true;
        CUDA_TRY(h, cudaMemcpy(nm == "sigmaTcRMax" ? h->B.smax : h->B.rem, in, sizeof(double) * C,
                               cudaMemcpyHostToDevice));
        return DSMC_OK;
    }
    return fail(h, DSMC_ERR_INVALID, "unknown settable cell array " + nm);
}

int dsmc_get_species_field(dsmc_handle* h, const char* name, unsigned species_mask, double* out, long long n) {
    static const char* names[F_COUNT_FIELDS] = {"rhoN", "rhoM", "Ux", "Uy", "Uz", "Ttra", "p", "Trot", "Tvib",
                                                "Tov", "dsmcNMean", "nColls", "measuredCollisionRate",
                                                "meanCollisionRate", "mfp", "Ma", "rhoMError", "UError",
                                                "TError", "pError", "pressureTensor_xx", "pressureTensor_xy",
                                                "pressureTensor_xz", "pressureTensor_yy", "pressureTensor_yz",
                                                "pressureTensor_zz", "shearStressTensor_xx", "shearStressTensor_xy",
                                                "shearStressTensor_xz", "shearStressTensor_yy",
                                                "shearStressTensor_yz", "shearStressTensor_zz", "heatFluxVector_x",
                                                "heatFluxVector_y", "heatFluxVector_z"};
    int which = -1;
    for (int k = 0; k < F_COUNT_FIELDS; ++k)
        if (!std::strcmp(name, names[k])) which = k;
    if (which < 0) {
        std::string valid;
        for (int k = 0; k < F_COUNT_FIELDS; ++k) valid += std::string(" ") + names[k];
        return fail(h, DSMC_ERR_INVALID, std::string("unknown field ") + name + "; valid:" + valid);
    }
    if (n != h->cs.C) return fail(h, DSMC_ERR_INVALID, "n must equal the number of cells");
    if (which >= F_PXX && which <= F_QZ && !h->B.macc)
        return fail(h, DSMC_ERR_INVALID, std::string(name) + " needs measureHeatFluxShearStress in the case");
    const unsigned all = (1u << h->cs.nSpecies) - 1u;
    if (!(species_mask & all) || (species_mask & ~all))
        return fail(h, DSMC_ERR_INVALID, "species_mask must select species of the case");
    flush_sample(h);
    launch_field(h->cs, h->B, which, h->fieldTmp, h->spec.measure_mean_free_path, h->spec.mfp_tref, species_mask,
                 h->stream);
    CUDA_TRY(h, cudaGetLastError());
    CUDA_TRY(h, cudaMemcpyAsync(out, h->fieldTmp, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return DSMC_OK;
}

int dsmc_get_field(dsmc_handle* h, const char* name, double* out, long long n) {
    return dsmc_get_species_field(h, name, (1u << h->cs.nSpecies) - 1u, out, n);
}

long long dsmc_n_boundary_faces(const dsmc_handle* h) { return h->cs.nBFaces; }


long long dsmc_case_spec_size(void) { return (long long)sizeof(dsmc_case_spec); }

int dsmc_get_wall_field(dsmc_handle* h, const char* name, double* out, long long n) {
    const long long nf = h->cs.nBFaces;
    const std::string nm(name);
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    if (nm == "wallAccumulators") {
        if (n != nf * W_N) return fail(h, DSMC_ERR_INVALID, "n must equal faces x 14");
        CUDA_TRY(h, cudaMemcpy(out, h->B.wall, sizeof(double) * n, cudaMemcpyDeviceToHost));
        return DSMC_OK;
    }
    if (n != nf) return fail(h, DSMC_ERR_INVALID, "n must equal the number of boundary faces");
    // dsmcVolFields divides the boundary sums by its sample count
    // (dsmcVolFields.C:2111-2126), the steps since the last reset
    flush_sample(h);
    std::vector<double> w(nf * W_N);
    CUDA_TRY(h, cudaMemcpy(w.data(), h->B.wall, sizeof(double) * nf * W_N, cudaMemcpyDeviceToHost));
    CUDA_TRY(h, cudaMemcpy(h->ctrHost, h->B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost));
    const double nT = h->ctrHost->sampleSteps > 0 ? (double)h->ctrHost->sampleSteps : 1.0;
    const CaseDev& cs = h->cs;
    for (long long f = 0; f < nf; ++f) {
        const double* W = &w[f * W_N];
        // normal axis and outward sign of the face (obstacle faces point into the solid)
        int side = -1;
        double sgn = 1.0;
        for (int q = 0; q < 6 && side < 0; ++q)
            if (f >= cs.sideOff[q] && f < cs.sideOff[q + 1]) { side = q; sgn = (q & 1) ? 1.0 : -1.0; }
        for (int o = 0; o < cs.nObst && side < 0; ++o)
            for (int q = 0; q < 6 && side < 0; ++q) {
                const long long end = (q < 5) ? cs.obstOff[o][q + 1]
                                              : (o + 1 < cs.nObst ? cs.obstOff[o + 1][0] : cs.nBFaces);
                if (f >= cs.obstOff[o][q] && f < end) { side = q; sgn = (q & 1) ? -1.0 : 1.0; }
            }
        const int a = side / 2;
        const double fD[3] = {W[W_FDX] / nT, W[W_FDY] / nT, W[W_FDZ] / nT};
        double v;
        if (nm == "wallHeatFlux") v = W[W_Q] / nT;
        else if (nm == "wallShearStress_x") v = fD[0];
        else if (nm == "wallShearStress_y") v = fD[1];
        else if (nm == "wallShearStress_z") v = fD[2];
        else if (nm == "wallShearStress")   // |fD . t1, fD . t2|
            v = std::sqrt(fD[(a + 1) % 3] * fD[(a + 1) % 3] + fD[(a + 2) % 3] * fD[(a + 2) % 3]);
        else if (nm == "p_wall") v = fD[a] * sgn;   // fD . n
        else if (nm == "rhoN_wall") v = W[W_RHON] * cs.FN / nT;
        else return fail(h, DSMC_ERR_INVALID, "unknown wall field " + nm);
        out[f] = v;
    }
    return DSMC_OK;
}

int dsmc_reset_sampling(dsmc_handle* h) {
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    enqueue_reset(h, h->stream);
    CUDA_TRY(h, cudaGetLastError());
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    CUDA_TRY(h, cudaMemcpy(h->ctrHost, h->B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost));
    h->faceStep0 = h->ctrHost->step;
    h->resetPending = false;
    return DSMC_OK;
}

int dsmc_counts(dsmc_handle* h, dsmc_counts_t* o) {
    // the step counters only: one small read, no pass over the parcels
    CUDA_TRY(h, cudaMemcpyAsync(h->ctrHost, h->B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    const Counters& c = *h->ctrHost;
    o->n_particles = c.n;
    o->step = c.step;
    o->collisions_last_step = (long long)c.coll;
    o->candidates_last_step = (long long)c.cand;
    o->collisions_total = (long long)c.collTot;
    o->candidates_total = (long long)c.candTot;
    if (c.err) return check_device_error(h);
    return DSMC_OK;
}

int dsmc_evolve_counts(dsmc_handle* h, long long n, dsmc_counts_t* out) {
    if (n < 0) return fail(h, DSMC_ERR_INVALID, "n must not be negative");
    if (n > 0 && !out) return fail(h, DSMC_ERR_INVALID, "dsmc_evolve_counts: out is NULL");
    int rc = refuse_divided(h, "dsmc_evolve_counts");
    if (rc) return rc;
    rc = build_graphs(h);
    if (rc) return rc;
    if (n > h->ctrRingN) {
        if (h->ctrRing) cudaFreeHost(h->ctrRing);
        h->ctrRing = nullptr;
        h->ctrRingN = 0;
        void* p = nullptr;
        CUDA_TRY(h, cudaMallocHost(&p, sizeof(Counters) * (size_t)n));
        h->ctrRing = static_cast<Counters*>(p);
        h->ctrRingN = n;
    }
    // each step's counters follow it to the host on the same stream: no
    // host round trip between steps
    for (long long i = 0; i < n; ++i) {
        schedule_pre(h, h->stream);
        CUDA_TRY(h, cudaGraphLaunch(h->graph[h->cur], h->stream));
        h->cur ^= 1;
        schedule_post(h);
        CUDA_TRY(h, cudaMemcpyAsync(h->ctrRing + i, h->B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, h->stream));
    }
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    for (long long i = 0; i < n; ++i) {
        const Counters& c = h->ctrRing[i];
        dsmc_counts_t& o = out[i];
        o.n_particles = c.n;
        o.step = c.step;
        o.collisions_last_step = (long long)c.coll;
        o.candidates_last_step = (long long)c.cand;
        o.collisions_total = (long long)c.collTot;
        o.candidates_total = (long long)c.candTot;
    }
    return check_device_error(h);
}

int dsmc_info(dsmc_handle* h, dsmc_info_t* o) {
    std::memset(o, 0, sizeof(*o));
    flush_sample(h);
    launch_info(h->cs, cur_soa(h), h->B.ctr, h->info6, h->stream);
    CUDA_TRY(h, cudaGetLastError());
    double v[6];
    CUDA_TRY(h, cudaMemcpyAsync(v, h->info6, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    CUDA_TRY(h, cudaMemcpy(h->ctrHost, h->B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost));
    const Counters& c = *h->ctrHost;
    const double FN = h->cs.FN;
    o->n_particles = c.n;
    o->step = c.step;
    o->linear_ke = v[0] * FN;
    o->rotational_e = v[1] * FN;
    o->vibrational_e = v[2] * FN;
    for (int a = 0; a < 3; ++a) o->momentum[a] = v[3 + a] * FN;
    o->collisions_last_step = (long long)c.coll;
    o->candidates_last_step = (long long)c.cand;
    o->collisions_total = (long long)c.collTot;
    o->candidates_total = (long long)c.candTot;
    o->wall_hits_last_step = (long long)c.wallHits;
    o->inserted_last_step = (long long)c.inserted;
    o->deleted_last_step = (long long)c.deleted;
    o->sample_steps = c.sampleSteps;
    return DSMC_OK;
}

// Checkpoint layout: magic, version, C, nAcc, nBFaces, nInflow, counters,
// parcels (n 64-byte records, then n cell words), smax, rem, acc, wall, inflow accumulators.
int dsmc_checkpoint(dsmc_handle* h, const char* path) {
    flush_sample(h);
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    CUDA_TRY(h, cudaMemcpy(h->ctrHost, h->B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost));
    const Counters c = *h->ctrHost;
    std::ofstream f(path, std::ios::binary);
    if (!f) return fail(h, DSMC_ERR_IO, std::string("cannot write ") + path);
    const long long hdr[6] = {0x44534D4347423330LL, 2, h->cs.C, h->cs.nAcc, h->cs.nBFaces,
                              (long long)h->B.nInflowFaces * h->spec.n_species};
    f.write(reinterpret_cast<const char*>(hdr), sizeof(hdr));
    f.write(reinterpret_cast<const char*>(&c), sizeof(c));
    const long long n = c.n;
    Parcels& s = cur_soa(h);
    std::vector<char> buf;
    auto dump = [&](const void* dptr, size_t bytes) -> int {
        buf.resize(bytes);
        if (bytes) CUDA_TRY(h, cudaMemcpy(buf.data(), dptr, bytes, cudaMemcpyDeviceToHost));
        f.write(buf.data(), (std::streamsize)bytes);
        return DSMC_OK;
    };
    int rc;
    if ((rc = dump(s.r, sizeof(Rec) * n))) return rc;
    if ((rc = dump(s.cellw, sizeof(uint32_t) * n))) return rc;
    if ((rc = dump(h->B.start, sizeof(int) * (h->cs.C + 1)))) return rc;
    if ((rc = dump(h->B.smax, sizeof(double) * h->cs.C))) return rc;
    if ((rc = dump(h->B.rem, sizeof(double) * h->cs.C))) return rc;
    if ((rc = dump(h->B.acc, sizeof(double) * h->cs.C * h->cs.nAcc))) return rc;
    if ((rc = dump(h->B.wall, sizeof(double) * h->cs.nBFaces * W_N))) return rc;
    if ((rc = dump(h->B.inflowAcc, sizeof(double) * hdr[5]))) return rc;
    if (!f) return fail(h, DSMC_ERR_IO, std::string("write failed: ") + path);
    return DSMC_OK;
}

int dsmc_restore(dsmc_handle* h, const char* path) {
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(h, DSMC_ERR_IO, std::string("cannot read ") + path);
    long long hdr[6];
    f.read(reinterpret_cast<char*>(hdr), sizeof(hdr));
    if (!f || hdr[0] != 0x44534D4347423330LL || hdr[1] != 2 || hdr[2] != h->cs.C || hdr[3] != h->cs.nAcc ||
        hdr[4] != h->cs.nBFaces || hdr[5] != (long long)h->B.nInflowFaces * h->spec.n_species)
        return fail(h, DSMC_ERR_INVALID, "checkpoint does not match this case");
    Counters c;
    f.read(reinterpret_cast<char*>(&c), sizeof(c));
    const long long n = c.n;
    if (n > h->B.capacity) return fail(h, DSMC_ERR_CAPACITY, "checkpoint holds more parcels than the capacity");
    Parcels& s = cur_soa(h);
    std::vector<char> buf;
    auto load = [&](void* dptr, size_t bytes) -> int {
        buf.resize(bytes);
        f.read(buf.data(), (std::streamsize)bytes);
        if (!f) return fail(h, DSMC_ERR_IO, "truncated checkpoint");
        if (bytes) CUDA_TRY(h, cudaMemcpy(dptr, buf.data(), bytes, cudaMemcpyHostToDevice));
        return DSMC_OK;
    };
    int rc;
    if ((rc = load(s.r, sizeof(Rec) * n))) return rc;
    if ((rc = load(s.cellw, sizeof(uint32_t) * n))) return rc;
    launch_ids_from_records(s, n, h->stream);
    if ((rc = load(h->B.start, sizeof(int) * (h->cs.C + 1)))) return rc;
    if ((rc = load(h->B.smax, sizeof(double) * h->cs.C))) return rc;
    if ((rc = load(h->B.rem, sizeof(double) * h->cs.C))) return rc;
    if ((rc = load(h->B.acc, sizeof(double) * h->cs.C * h->cs.nAcc))) return rc;
    if ((rc = load(h->B.wall, sizeof(double) * h->cs.nBFaces * W_N))) return rc;
    if ((rc = load(h->B.inflowAcc, sizeof(double) * hdr[5]))) return rc;
    c.err = 0;
    *h->ctrHost = c;
    CUDA_TRY(h, cudaMemcpy(h->B.ctr, h->ctrHost, sizeof(Counters), cudaMemcpyHostToDevice));
    CUDA_TRY(h, cudaMemset(h->B.count, 0, sizeof(int) * h->cs.C));
    CUDA_TRY(h, cudaMemset(h->B.sfix, 0, sizeof(long long) * h->cs.C * h->cs.nSpecies * SACC));
    // the face sums start again from the restored step
    if (h->cs.faceFlux)
        CUDA_TRY(h, cudaMemset(h->cs.faceFlux, 0, sizeof(double) * 2 * h->cs.nSpecies * h->cs.nFacesAll));
    h->faceStep0 = c.step;
    h->stepHost = c.step;
    h->resetPending = false;
    schedule_sync(h);
    h->smaxSet = true;
    return DSMC_OK;
}

// ------------------------------------------------------- learned selection
int dsmc_set_learned(dsmc_handle* h, const dsmc_mlp* model, int every, float margin) {
    if (every < 1) return fail(h, DSMC_ERR_INVALID, "every must be at least 1");
    if (model && h->spec.partner_selection_model != DSMC_SEL_NTC)
        return fail(h, DSMC_ERR_INVALID, "the learned maximum applies to noTimeCounter selection only");
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    h->model = reinterpret_cast<const MlpModel*>(model);
    h->learnEvery = every;
    h->learnMargin = margin;
    drop_graphs(h);
    // every cell starts on the running maximum until the first prediction
    CUDA_TRY(h, cudaMemset(h->B.pred, 0, sizeof(float) * h->cs.C));
    CUDA_TRY(h, cudaMemset(h->B.useR, 1, h->cs.C));
    CUDA_TRY(h, cudaMemset(h->B.exceed, 0, sizeof(float) * h->cs.C));
    return DSMC_OK;
}

int dsmc_set_learned_forget(dsmc_handle* h, float forget) {
    if (!(forget >= 0.f && forget <= 1.f)) return fail(h, DSMC_ERR_INVALID, "forget must lie in [0, 1]");
    h->learnForget = forget;
    drop_graphs(h);
    return DSMC_OK;
}

int dsmc_learn_record(dsmc_handle* h, long long max_rows, float* X, float* Y, long long* n_out) {
    if (n_out) *n_out = 0;
    if (max_rows <= 0) return DSMC_OK;
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    float *dX = nullptr, *dY = nullptr;
    unsigned long long* dn = nullptr;
    CUDA_TRY(h, cudaMalloc(&dX, sizeof(float) * 3 * max_rows));
    CUDA_TRY(h, cudaMalloc(&dY, sizeof(float) * max_rows));
    CUDA_TRY(h, cudaMalloc(&dn, sizeof(unsigned long long)));
    launch_cell_features(h->cs, h->B, cur_soa(h), 0, 0, h->stream);
    launch_learn_compact(h->cs, h->B, max_rows, dX, dY, dn, h->stream);
    unsigned long long n = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&n, dn, sizeof(n), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    const long long m = (long long)n < max_rows ? (long long)n : max_rows;
    if (e == cudaSuccess && m > 0) e = cudaMemcpy(X, dX, sizeof(float) * 3 * m, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && m > 0) e = cudaMemcpy(Y, dY, sizeof(float) * m, cudaMemcpyDeviceToHost);
    cudaFree(dX);
    cudaFree(dY);
    cudaFree(dn);
    if (e != cudaSuccess) return fail(h, DSMC_ERR_CUDA, std::string("dsmc_learn_record: ") + cudaGetErrorString(e));
    if (n_out) *n_out = m;
    return DSMC_OK;
}

// ------------------------------------------------------- selection audit
int dsmc_set_selection_audit(dsmc_handle* h, int on) {
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    if (on && !h->auditBuf) {
        int rc = dalloc(h, &h->auditBuf, h->cs.C);
        if (rc) return rc;
    }
    if (on) CUDA_TRY(h, cudaMemset(h->auditBuf, 0, sizeof(double2) * h->cs.C));
    h->B.audit = on ? h->auditBuf : nullptr;
    drop_graphs(h);   // the collision kernels take the buffer as a parameter
    return DSMC_OK;
}

// ------------------------------------------------------- spatial decomposition
int dsmc_set_domain(dsmc_handle* h, int axis, int lo, int hi) {
    if (h->batchOwned) return fail(h, DSMC_ERR_INVALID, "dsmc_set_domain: the case belongs to a batch");
    if (h->midStep) return fail(h, DSMC_ERR_INVALID, "dsmc_set_domain: a step is between its halves");
    if (axis < -1 || axis > 2) return fail(h, DSMC_ERR_INVALID, "dsmc_set_domain: axis must be -1, 0, 1 or 2");
    if (axis >= 0 && !(0 <= lo && lo < hi && hi <= h->cs.n[axis]))
        return fail(h, DSMC_ERR_INVALID, "dsmc_set_domain: need 0 <= lo < hi <= " + std::to_string(h->cs.n[axis]) +
                                             " cells along the axis");
    if (axis >= 0 && h->cs.C >= (1LL << 24))
        return fail(h, DSMC_ERR_INVALID, "dsmc_set_domain: meshes of 2^24 cells and more are not divided");
    StepBuffers& B = h->B;
    if (axis >= 0 && !B.migList) {
        // the migrants of one step: an eighth of the capacity (a domain
        // thinner than a step's travel needs more; the overflow is reported)
        B.migCap = B.capacity / 8 + 65536;
        int rc;
        if ((rc = dalloc(h, &B.migList, B.migCap))) return rc;
        if ((rc = dalloc(h, &B.migOut, B.migCap * MIGRANT_WORDS))) return rc;
    }
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    h->cs.domAxis = axis;
    h->cs.domLo = axis >= 0 ? lo : 0;
    h->cs.domHi = axis >= 0 ? hi : 0;
    drop_graphs(h);
    // the parcels of other domains' cells leave now
    CUDA_TRY(h, cudaMemcpy(h->ctrHost, B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost));
    const long long n = h->ctrHost->n;
    if (axis >= 0 && n > 0) {
        flush_sample(h);
        return sort_current(h, n);
    }
    return DSMC_OK;
}

int dsmc_step_begin(dsmc_handle* h, long long* n_migrants) {
    if (h->cs.domAxis < 0) return fail(h, DSMC_ERR_INVALID, "dsmc_step_begin: the cloud is not divided");
    if (h->midStep) return fail(h, DSMC_ERR_INVALID, "dsmc_step_begin: the previous step has not ended");
    int rc = build_half_graphs(h);
    if (rc) return rc;
    schedule_pre(h, h->stream);
    CUDA_TRY(h, cudaGraphLaunch(h->half1[h->cur], h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->ctrHost, h->B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    h->midStep = true;
    h->nMovedHost = h->ctrHost->nMoved;
    h->nMigHost = std::min((long long)h->ctrHost->nMig, h->B.migCap);
    if (n_migrants) *n_migrants = h->nMigHost;
    return DSMC_OK;
}

int dsmc_get_migrants(dsmc_handle* h, void* dst, long long n) {
    if (!h->midStep) return fail(h, DSMC_ERR_INVALID, "dsmc_get_migrants: no step between its halves");
    if (n < 0 || n > h->nMigHost)
        return fail(h, DSMC_ERR_INVALID, "dsmc_get_migrants: n must lie in [0, " + std::to_string(h->nMigHost) + "]");
    if (n == 0) return DSMC_OK;
    if (!dst) return fail(h, DSMC_ERR_INVALID, "dsmc_get_migrants: dst is NULL");
    CUDA_TRY(h, cudaMemcpyAsync(dst, h->B.migOut, (size_t)n * MIGRANT_WORDS * 4, cudaMemcpyDefault, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return DSMC_OK;
}

int dsmc_add_migrants(dsmc_handle* h, const void* src, long long n) {
    if (!h->midStep) return fail(h, DSMC_ERR_INVALID, "dsmc_add_migrants: no step between its halves");
    if (n < 0) return fail(h, DSMC_ERR_INVALID, "dsmc_add_migrants: n must not be negative");
    if (n == 0) return DSMC_OK;
    if (!src) return fail(h, DSMC_ERR_INVALID, "dsmc_add_migrants: src is NULL");
    StepBuffers& B = h->B;
    const long long limit = std::min(B.capacity, h->cs.capacityLimit);
    if (h->nMovedHost + n > limit)
        return fail(h, DSMC_ERR_CAPACITY, "dsmc_add_migrants: " + std::to_string(n) + " migrants exceed the capacity");
    cudaPointerAttributes at{};
    const bool onDevice = cudaPointerGetAttributes(&at, src) == cudaSuccess &&
                          (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged);
    cudaGetLastError();   // a host pointer may leave an error behind on older runtimes
    const uint32_t* d = static_cast<const uint32_t*>(src);
    if (!onDevice) {
        if (n > B.migInCap) {
            if (B.migIn) cudaFree(B.migIn);
            B.migIn = nullptr;
            B.migInCap = 0;
            void* q = nullptr;
            CUDA_TRY(h, cudaMalloc(&q, (size_t)n * MIGRANT_WORDS * 4));
            B.migIn = static_cast<uint32_t*>(q);
            B.migInCap = n;
        }
        CUDA_TRY(h, cudaMemcpyAsync(B.migIn, src, (size_t)n * MIGRANT_WORDS * 4, cudaMemcpyHostToDevice, h->stream));
        d = B.migIn;
    }
    launch_unpack_migrants(h->cs, B, cur_soa(h), d, n, h->nMovedHost, h->stream);
    CUDA_TRY(h, cudaGetLastError());
    h->nMovedHost += n;
    return DSMC_OK;
}

int dsmc_step_end(dsmc_handle* h) {
    if (!h->midStep) return fail(h, DSMC_ERR_INVALID, "dsmc_step_end: no step between its halves");
    CUDA_TRY(h, cudaGraphLaunch(h->half2[h->cur], h->stream));
    h->cur ^= 1;
    h->midStep = false;
    schedule_post(h);
    return check_device_error(h);
}

// ------------------------------------------------------- loop caps
int dsmc_set_limits(dsmc_handle* h, int max_rejection, int max_crossings, int max_cell_parcels,
                    long long capacity) {
    if (max_rejection < 0 || max_crossings < 0 || max_cell_parcels < 0 || capacity < 0)
        return fail(h, DSMC_ERR_INVALID, "limits must not be negative");
    if (max_rejection > MAX_REJECTION || max_crossings > MAX_CROSSINGS || max_cell_parcels > MAX_ORDERED_CELL)
        return fail(h, DSMC_ERR_INVALID, "limits can only be lowered (at most " + std::to_string(MAX_REJECTION) +
                                             " draws, " + std::to_string(MAX_CROSSINGS) + " crossings, " +
                                             std::to_string(MAX_ORDERED_CELL) + " parcels per cell)");
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    h->cs.maxRejection = max_rejection ? max_rejection : MAX_REJECTION;
    h->cs.maxCrossings = max_crossings ? max_crossings : MAX_CROSSINGS;
    h->cs.maxCellParcels = max_cell_parcels ? max_cell_parcels : MAX_ORDERED_CELL;
    h->cs.capacityLimit = capacity ? capacity : (1LL << 62);
    drop_graphs(h);   // the step graphs hold the case constants
    return DSMC_OK;
}

// ------------------------------------------------------- launch shape
int dsmc_set_launch(dsmc_handle* h, int cta_threads, int cells_per_cta) {
    if (cta_threads != 128 && cta_threads != 256 && cta_threads != 512)
        return fail(h, DSMC_ERR_INVALID, "cta_threads must be 128, 256 or 512");
    if (cells_per_cta != 32 && cells_per_cta != 64 && cells_per_cta != 128)
        return fail(h, DSMC_ERR_INVALID, "cells_per_cta must be 32, 64 or 128");
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    h->B.cfg.streamThreads = cta_threads;
    h->B.cfg.streamCtasPerSm = 2048 / cta_threads;
    h->B.cfg.lightCells = cells_per_cta;
    drop_graphs(h);
    return DSMC_OK;
}

int dsmc_get_launch(dsmc_handle* h, int* cta_threads, int* cells_per_cta) {
    if (cta_threads) *cta_threads = h->B.cfg.streamThreads;
    if (cells_per_cta) *cells_per_cta = h->B.cfg.lightCells;
    return DSMC_OK;
}

// ------------------------------------------------------- batch of clouds
struct dsmc_batch {
    std::vector<dsmc_handle*> cases;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    // persistent mode: two cooperative launches per batched step (move and
    // sort, then collisions) over all cases; 0 threads: graph of case graphs
    int persistMove = 0, persistCollide = 0;
    BatchSlot* dSlots = nullptr;     // [2][n]: the cases as seen from each buffer parity
    BatchCtl* dCtl = nullptr;
    int pgraphState = 0;             // 0 not tried, 1 captured, -1 capture refused: direct launches
    cudaGraphExec_t pgraph[2] = {nullptr, nullptr};
    // each case's graph generation when the batch graphs were built: a case
    // whose step graphs were dropped since (learned model, face tracking,
    // launch shape, ...) makes the batch graphs stale
    std::vector<unsigned long long> gen;
    std::string err;
};

static thread_local std::string g_batch_err;

static int bfail(dsmc_batch* b, int code, const std::string& msg) {
    if (b) b->err = msg;
    g_batch_err = msg;
    return code;
}

static void drop_batch_graphs(dsmc_batch* b) {
    for (int p = 0; p < 2; ++p) {
        if (b->graph[p]) cudaGraphExecDestroy(b->graph[p]);
        b->graph[p] = nullptr;
    }
}

// One graph per parity holding every case's captured step as an independent
// child: a batched step is one launch, and the cases' kernels run side by
// side as the GPU has room.
static int build_batch_graphs(dsmc_batch* b) {
    bool stale = b->gen.size() != b->cases.size();
    for (size_t i = 0; !stale && i < b->cases.size(); ++i) stale = b->gen[i] != b->cases[i]->graphGen;
    if (stale) drop_batch_graphs(b);
    for (int p = 0; p < 2; ++p) {
        if (b->graph[p]) continue;
        for (dsmc_handle* h : b->cases) {
            int rc = build_graphs(h);
            if (rc) return bfail(b, rc, std::string("case graph: ") + h->err);
        }
        cudaGraph_t pg;
        cudaError_t e = cudaGraphCreate(&pg, 0);
        for (size_t i = 0; e == cudaSuccess && i < b->cases.size(); ++i) {
            cudaGraphNode_t node;
            e = cudaGraphAddChildGraphNode(&node, pg, nullptr, 0, b->cases[i]->graphT[p]);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph[p], pg, 0);
        cudaGraphDestroy(pg);
        if (e != cudaSuccess) return bfail(b, DSMC_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e));
    }
    b->gen.resize(b->cases.size());
    for (size_t i = 0; i < b->cases.size(); ++i) b->gen[i] = b->cases[i]->graphGen;
    return DSMC_OK;
}


int dsmc_batch_create(int n, const dsmc_case_spec* specs, dsmc_batch** out) {
    *out = nullptr;
    if (n < 1) return bfail(nullptr, DSMC_ERR_INVALID, "a batch needs at least one case");
    auto b = std::make_unique<dsmc_batch>();
    for (int i = 0; i < n; ++i) {
        dsmc_handle* h = nullptr;
        int rc = dsmc_create_from_spec(&specs[i], &h);
        if (rc) {
            const std::string m = "case " + std::to_string(i) + ": " + dsmc_last_global_error();
            for (dsmc_handle* q : b->cases) dsmc_destroy(q);
            return bfail(nullptr, rc, m);
        }
        b->cases.push_back(h);
    }
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        for (dsmc_handle* q : b->cases) dsmc_destroy(q);
        return bfail(nullptr, DSMC_ERR_CUDA, "cannot create the batch stream");
    }
    for (dsmc_handle* q : b->cases) q->batchOwned = true;
    *out = b.release();
    return DSMC_OK;
}

int dsmc_batch_create_from_dirs(int n, const char* const* case_dirs, dsmc_batch** out) {
    *out = nullptr;
    if (n < 1) return bfail(nullptr, DSMC_ERR_INVALID, "a batch needs at least one case");
    auto b = std::make_unique<dsmc_batch>();
    for (int i = 0; i < n; ++i) {
        // each case is parsed and created before the next is parsed: the
        // parser's per-face and node tables live until the next parse
        dsmc_handle* h = nullptr;
        int rc = dsmc_create(case_dirs[i], &h);
        if (rc) {
            const std::string m = std::string("case ") + case_dirs[i] + ": " + dsmc_last_global_error();
            for (dsmc_handle* q : b->cases) dsmc_destroy(q);
            return bfail(nullptr, rc, m);
        }
        b->cases.push_back(h);
    }
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        for (dsmc_handle* q : b->cases) dsmc_destroy(q);
        return bfail(nullptr, DSMC_ERR_CUDA, "cannot create the batch stream");
    }
    for (dsmc_handle* q : b->cases) q->batchOwned = true;
    *out = b.release();
    return DSMC_OK;
}

static void drop_persistent_graphs(dsmc_batch* b) {
    for (int p = 0; p < 2; ++p) {
        if (b->pgraph[p]) cudaGraphExecDestroy(b->pgraph[p]);
        b->pgraph[p] = nullptr;
    }
    b->pgraphState = 0;
}

void dsmc_batch_destroy(dsmc_batch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_batch_graphs(b);
    drop_persistent_graphs(b);
    if (b->dSlots) cudaFree(b->dSlots);
    if (b->dCtl) cudaFree(b->dCtl);
    for (dsmc_handle* h : b->cases) {
        h->batchOwned = false;
        dsmc_destroy(h);
    }
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

const char* dsmc_batch_last_error(const dsmc_batch* b) { return b ? b->err.c_str() : g_batch_err.c_str(); }

int dsmc_batch_size(const dsmc_batch* b) { return (int)b->cases.size(); }

dsmc_handle* dsmc_batch_case(dsmc_batch* b, int i) {
    if (i < 0 || i >= (int)b->cases.size()) return nullptr;
    return b->cases[i];
}

int dsmc_batch_initialise(dsmc_batch* b) {
    for (size_t i = 0; i < b->cases.size(); ++i) {
        int rc = dsmc_initialise(b->cases[i]);
        if (rc) return bfail(b, rc, "case " + std::to_string(i) + ": " + b->cases[i]->err);
    }
    drop_batch_graphs(b);
    return DSMC_OK;
}

int dsmc_batch_set_launch(dsmc_batch* b, int i, int cta_threads, int cells_per_cta) {
    if (i < 0 || i >= (int)b->cases.size()) return bfail(b, DSMC_ERR_INVALID, "case index out of range");
    int rc = dsmc_set_launch(b->cases[i], cta_threads, cells_per_cta);
    if (rc) return bfail(b, rc, b->cases[i]->err);
    drop_batch_graphs(b);
    return DSMC_OK;
}

int dsmc_batch_set_persistent(dsmc_batch* b, int move_threads, int collide_threads) {
    if (!move_threads && !collide_threads) {
        b->persistMove = b->persistCollide = 0;
        return DSMC_OK;
    }
    if (move_threads != 128 && move_threads != 256 && move_threads != 512)
        return bfail(b, DSMC_ERR_INVALID, "move_threads must be 128, 256 or 512");
    if (collide_threads != 64 && collide_threads != 128)
        return bfail(b, DSMC_ERR_INVALID, "collide_threads must be 64 or 128");
    const int n = (int)b->cases.size();
    if (n > BATCH_MAX_CASES)
        return bfail(b, DSMC_ERR_INVALID, "the persistent batch takes at most " + std::to_string(BATCH_MAX_CASES) +
                                              " cases");
    for (int i = 0; i < n; ++i) {
        const dsmc_handle* h = b->cases[i];
        const CaseDev& cs = h->cs;
        const char* why = nullptr;
        if (h->hasInflow) why = "a freestream inflow";
        else if (cs.nObst) why = "an obstacle";
        else if (cs.anyEmpty) why = "a reduced-D (empty) axis";
        else if (cs.half[0] || cs.half[1] || cs.half[2]) why = "a graded axis";
        else if (cs.faceFlux) why = "face tracking";
        else if (h->model) why = "a learned maximum";
        else if (h->B.audit) why = "the selection audit";
        else if (h->B.macc) why = "measureHeatFluxShearStress";
        else if (cs.selModel != DSMC_SEL_NTC) why = "simplifiedBernoulliTrials";
        if (why)
            return bfail(b, DSMC_ERR_INVALID, "case " + std::to_string(i) + " has " + why +
                                                  ": the persistent batch kernels take uniform boxes with "
                                                  "noTimeCounter selection only");
    }
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return bfail(b, DSMC_ERR_CUDA, "batch stream");
    if (!b->dSlots && cudaMalloc(&b->dSlots, sizeof(BatchSlot) * 2 * (size_t)n) != cudaSuccess)
        return bfail(b, DSMC_ERR_CAPACITY, "cannot allocate the batch slots");
    if (!b->dCtl) {
        if (cudaMalloc(&b->dCtl, sizeof(BatchCtl)) != cudaSuccess)
            return bfail(b, DSMC_ERR_CAPACITY, "cannot allocate the batch control block");
        cudaMemset(b->dCtl, 0, sizeof(BatchCtl));
    }
    if (batch_move_grid(move_threads) <= 0 || batch_collide_grid(collide_threads) <= 0)
        return bfail(b, DSMC_ERR_CUDA, "no occupancy for the persistent batch kernels");
    b->persistMove = move_threads;
    b->persistCollide = collide_threads;
    drop_persistent_graphs(b);
    return DSMC_OK;
}

int dsmc_batch_get_persistent(const dsmc_batch* b, int* move_threads, int* collide_threads) {
    if (move_threads) *move_threads = b->persistMove;
    if (collide_threads) *collide_threads = b->persistCollide;
    return DSMC_OK;
}

// One batched step of the persistent mode on the batch stream: the tickets
// cleared, then the move/sort launch and the collision launch.
static cudaError_t enqueue_persistent_step(dsmc_batch* b, int p) {
    const int n = (int)b->cases.size();
    void* tickets = reinterpret_cast<char*>(b->dCtl) + offsetof(BatchCtl, ticket);
    cudaError_t e = cudaMemsetAsync(tickets, 0, sizeof(unsigned long long) * BATCH_PHASES, b->stream);
    if (e == cudaSuccess) e = launch_batch_move(b->dSlots + (size_t)p * n, n, b->dCtl, b->persistMove, b->stream);
    if (e == cudaSuccess)
        e = launch_batch_collide(b->dSlots + (size_t)p * n, n, b->dCtl, b->persistCollide, b->stream);
    return e;
}

// The cases as the persistent kernels see them from each buffer parity.
static int upload_slots(dsmc_batch* b) {
    const int n = (int)b->cases.size();
    std::vector<BatchSlot> sl((size_t)2 * n);
    for (int p = 0; p < 2; ++p)
        for (int i = 0; i < n; ++i) {
            const dsmc_handle* h = b->cases[i];
            BatchSlot& s = sl[(size_t)p * n + i];
            s.cs = h->cs;
            // the collision launch orders cells by warps only: larger cells
            // are skipped with the dense-cell error
            if (s.cs.maxCellParcels > WARP_ORDERED_CELL) s.cs.maxCellParcels = WARP_ORDERED_CELL;
            s.B = h->B;
            s.src = h->buf[p];
            s.dst = h->buf[p ^ 1];
        }
    if (cudaMemcpy(b->dSlots, sl.data(), sizeof(BatchSlot) * sl.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return bfail(b, DSMC_ERR_CUDA, "cannot upload the batch slots");
    return DSMC_OK;
}

// The persistent step of each parity captured as a graph (tickets memset and
// the two cooperative launches); where the capture is refused, the steps are
// launched directly.
static void capture_persistent(dsmc_batch* b) {
    if (b->pgraphState != 0) return;
    for (int p = 0; p < 2; ++p) {
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            const cudaError_t e1 = enqueue_persistent_step(b, p);
            e = cudaStreamEndCapture(b->stream, &g);
            if (e1 != cudaSuccess) e = e1;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->pgraph[p], g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            cudaGetLastError();
            drop_persistent_graphs(b);
            b->pgraphState = -1;
            return;
        }
    }
    b->pgraphState = 1;
}

static int batch_evolve_persistent(dsmc_batch* b, long long n, double* total_ms) {
    int rc = upload_slots(b);
    if (rc) return rc;
    for (dsmc_handle* h : b->cases)
        if (cudaStreamSynchronize(h->stream) != cudaSuccess) return bfail(b, DSMC_ERR_CUDA, "case stream");
    capture_persistent(b);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (total_ms) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, b->stream);
    }
    int p = b->cases[0]->cur;
    for (long long s = 0; s < n; ++s) {
        for (dsmc_handle* h : b->cases) schedule_pre(h, b->stream);
        const cudaError_t e = b->pgraphState == 1 ? cudaGraphLaunch(b->pgraph[p], b->stream)
                                                  : enqueue_persistent_step(b, p);
        if (e != cudaSuccess)
            return bfail(b, DSMC_ERR_CUDA, std::string("persistent batch launch: ") + cudaGetErrorString(e));
        p ^= 1;
        for (dsmc_handle* h : b->cases) schedule_post(h);
    }
    if (total_ms) cudaEventRecord(e1, b->stream);
    const cudaError_t e = cudaStreamSynchronize(b->stream);
    if (total_ms) {
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        *total_ms = ms;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    if (e != cudaSuccess) return bfail(b, DSMC_ERR_CUDA, std::string("persistent batch step: ") + cudaGetErrorString(e));
    BatchCtl ctl;
    if (cudaMemcpy(&ctl, b->dCtl, sizeof(ctl), cudaMemcpyDeviceToHost) != cudaSuccess)
        return bfail(b, DSMC_ERR_CUDA, "cannot read the batch control block");
    for (size_t i = 0; i < b->cases.size(); ++i) {
        dsmc_handle* h = b->cases[i];
        if (n & 1) h->cur ^= 1;
    }
    if (ctl.err) {
        cudaMemset(b->dCtl, 0, sizeof(BatchCtl));
        return bfail(b, DSMC_ERR_DEVICE, "persistent batch: a grid barrier wait ran out (the step is incomplete)");
    }
    for (size_t i = 0; i < b->cases.size(); ++i) {
        rc = check_device_error(b->cases[i]);
        if (rc) return bfail(b, rc, "case " + std::to_string(i) + ": " + b->cases[i]->err);
    }
    return DSMC_OK;
}

int dsmc_batch_evolve_timed(dsmc_batch* b, long long n, double* total_ms) {
    // the cases are stepped together, so they share the buffer parity
    const int cur = b->cases[0]->cur;
    for (dsmc_handle* h : b->cases)
        if (h->cur != cur) return bfail(b, DSMC_ERR_INVALID, "cases of a batch must be at the same buffer parity");
    if (b->persistMove) return batch_evolve_persistent(b, n, total_ms);
    int rc = build_batch_graphs(b);
    if (rc) return rc;
    // the cases' own streams may still hold work (initialisation, reads)
    for (dsmc_handle* h : b->cases)
        if (cudaStreamSynchronize(h->stream) != cudaSuccess) return bfail(b, DSMC_ERR_CUDA, "case stream");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (total_ms) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, b->stream);
    }
    int p = cur;
    for (long long s = 0; s < n; ++s) {
        // each case's output schedule (resets at output) around the launch
        for (dsmc_handle* h : b->cases) schedule_pre(h, b->stream);
        const cudaError_t e = cudaGraphLaunch(b->graph[p], b->stream);
        if (e != cudaSuccess) return bfail(b, DSMC_ERR_CUDA, std::string("batch launch: ") + cudaGetErrorString(e));
        p ^= 1;
        for (dsmc_handle* h : b->cases) schedule_post(h);
    }
    if (total_ms) cudaEventRecord(e1, b->stream);
    const cudaError_t e = cudaStreamSynchronize(b->stream);
    if (total_ms) {
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        *total_ms = ms;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    if (e != cudaSuccess) return bfail(b, DSMC_ERR_CUDA, std::string("batch step: ") + cudaGetErrorString(e));
    for (size_t i = 0; i < b->cases.size(); ++i) {
        dsmc_handle* h = b->cases[i];
        if (n & 1) h->cur ^= 1;
        rc = check_device_error(h);
        if (rc) return bfail(b, rc, "case " + std::to_string(i) + ": " + h->err);
    }
    return DSMC_OK;
}

int dsmc_batch_evolve(dsmc_batch* b, long long n) { return dsmc_batch_evolve_timed(b, n, nullptr); }

// ------------------------------------------------------- OpenFOAM output
// volScalarField / volVectorField files as dsmcVolFields::writeField writes
// them (dsmcVolFields.C:1878-2380): ASCII, nonuniform internal field in
// OpenFOAM's cell order, constraint types on constraint patches.
namespace {

const char* FOAM_BANNER =
    "/*--------------------------------*- C++ -*----------------------------------*\\\n"
    "  written by libhystrath_gb300 (GB300 dsmcFoam+ particle step)\n"
    "\\*---------------------------------------------------------------------------*/\n";

void foam_write(const std::string& path, const std::string& cls, const std::string& object,
                const std::string& location, const char* dims, const std::vector<const double*>& comps,
                const std::vector<long long>& order, const dsmc_case_spec& spec, bool* ok, int digits = 10) {
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) { *ok = false; return; }
    const bool vec = comps.size() == 3;
    std::fprintf(f, "%sFoamFile\n{\n    version     2.0;\n    format      ascii;\n    class       %s;\n"
                    "    location    \"%s\";\n    object      %s;\n}\n\ndimensions      %s;\n\n"
                    "internalField   nonuniform List<%s> \n%lld\n(\n",
                 FOAM_BANNER, cls.c_str(), location.c_str(), object.c_str(), dims, vec ? "vector" : "scalar",
                 (long long)order.size());
    for (long long c : order) {
        if (vec) std::fprintf(f, "(%.*g %.*g %.*g)\n", digits, comps[0][c], digits, comps[1][c], digits, comps[2][c]);
        else std::fprintf(f, "%.*g\n", digits, comps[0][c]);
    }
    std::fprintf(f, ")\n;\n\nboundaryField\n{\n");
    for (int p = 0; p < spec.n_patches; ++p) {
        const dsmc_patch& pt = spec.patches[p];
        std::fprintf(f, "    %s\n    {\n", pt.name);
        if (pt.type == DSMC_PATCH_CYCLIC) std::fprintf(f, "        type            cyclic;\n");
        else if (pt.type == DSMC_PATCH_SYMMETRY) std::fprintf(f, "        type            symmetryPlane;\n");
        else if (pt.type == DSMC_PATCH_EMPTY) std::fprintf(f, "        type            empty;\n");
        else std::fprintf(f, "        type            calculated;\n        value           uniform %s;\n",
                          vec ? "(0 0 0)" : "0");
        std::fprintf(f, "    }\n");
    }
    std::fprintf(f, "}\n");
    if (std::fclose(f) != 0) *ok = false;
}

}  // namespace

// OpenFOAM's cell order of the case (blockMesh: block by block), as the
// Cartesian cell of each OpenFOAM cell; the Cartesian order itself when the
// case has no blockMeshDict.
int case_cell_order(dsmc_handle* h, const char* case_dir, std::vector<long long>& order) {
    const long long C = h->cs.C;
    std::string err;
    std::string bm = std::string(case_dir) + "/system/blockMeshDict";
    std::ifstream probe(bm);
    if (!probe) probe.open(std::string(case_dir) + "/constant/polyMesh/blockMeshDict");
    order.clear();
    if (probe) {
        if (!foam_cell_order(case_dir, order, err)) return fail(h, DSMC_ERR_PARSE, "cell order: " + err);
        if ((long long)order.size() != h->nFluid)
            return fail(h, DSMC_ERR_INVALID, "the case's blockMeshDict does not match this cloud");
        for (long long c : order)
            if (c < 0 || c >= C) return fail(h, DSMC_ERR_INVALID, "the case's blockMeshDict does not match this cloud");
    } else {
        for (long long c = 0; c < C; ++c)
            order.push_back(c);
    }
    return DSMC_OK;
}

int dsmc_write_fields(dsmc_handle* h, const char* case_dir, const char* time_name, const char* field_name) {
    const long long C = h->cs.C;
    std::vector<long long> order;
    int orc = case_cell_order(h, case_dir, order);
    if (orc) return orc;
    const std::string dir = std::string(case_dir) + "/" + time_name;
    mkdir(dir.c_str(), 0755);
    struct FieldOut {
        const char* name;   // dsmc_get_field name(s)
        const char* file;   // file prefix
        const char* dims;
        bool vec;
    };
    const FieldOut fields[] = {
        {"rhoN", "rhoN", "[0 -3 0 0 0 0 0]", false}, {"rhoM", "rhoM", "[1 -3 0 0 0 0 0]", false},
        {"Ttra", "Ttra", "[0 0 0 1 0 0 0]", false},  {"Trot", "Trot", "[0 0 0 1 0 0 0]", false},
        {"Tvib", "Tvib", "[0 0 0 1 0 0 0]", false},  {"Tov", "Tov", "[0 0 0 1 0 0 0]", false},
        {"p", "p", "[1 -1 -2 0 0 0 0]", false},       {"dsmcNMean", "dsmcNMean", "[0 0 0 0 0 0 0]", false},
        {"U", "U", "[0 1 -1 0 0 0 0]", true},
    };
    std::vector<double> a(C), b(C), c(C);
    bool ok = true;
    const std::string suffix = (field_name && *field_name) ? std::string("_") + field_name : std::string();
    for (const FieldOut& fo : fields) {
        int rc;
        std::vector<const double*> comps;
        if (fo.vec) {
            if ((rc = dsmc_get_field(h, "Ux", a.data(), C)) || (rc = dsmc_get_field(h, "Uy", b.data(), C)) ||
                (rc = dsmc_get_field(h, "Uz", c.data(), C)))
                return rc;
            comps = {a.data(), b.data(), c.data()};
        } else {
            if ((rc = dsmc_get_field(h, fo.name, a.data(), C))) return rc;
            comps = {a.data()};
        }
        foam_write(dir + "/" + fo.file + suffix, fo.vec ? "volVectorField" : "volScalarField", fo.file + suffix,
                   time_name, fo.dims, comps, order, h->spec, &ok);
    }
    int rc = dsmc_get_cell_array(h, "sigmaTcRMax", a.data(), C);
    if (rc) return rc;
    foam_write(dir + "/dsmcSigmaTcRMax", "volScalarField", "dsmcSigmaTcRMax", time_name, "[0 3 -1 0 0 0 0]",
               {a.data()}, order, h->spec, &ok);
    if (!ok) return fail(h, DSMC_ERR_IO, "cannot write fields under " + dir);
    return DSMC_OK;
}

// ------------------------------------------------------- face tracker
int dsmc_set_face_tracking(dsmc_handle* h, int on) {
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    CaseDev& cs = h->cs;
    const long long nx = cs.n[0], ny = cs.n[1], nz = cs.n[2];
    cs.faceOff[0] = 0;
    cs.faceOff[1] = (nx + 1) * ny * nz;
    cs.faceOff[2] = cs.faceOff[1] + nx * (ny + 1) * nz;
    cs.nFacesAll = cs.faceOff[2] + nx * ny * (nz + 1);
    const long long n = 2 * (long long)cs.nSpecies * cs.nFacesAll;
    if (on && !h->faceBuf) {
        int rc;
        if ((rc = dalloc(h, &h->faceBuf, n))) return rc;
    }
    if (on && !cs.faceFlux) {
        CUDA_TRY(h, cudaMemset(h->faceBuf, 0, sizeof(double) * n));
        CUDA_TRY(h, cudaMemcpy(h->ctrHost, h->B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost));
        h->faceStep0 = h->ctrHost->step;
    }
    cs.faceFlux = on ? h->faceBuf : nullptr;
    drop_graphs(h);
    return DSMC_OK;
}

long long dsmc_n_faces(const dsmc_handle* h) {
    const long long nx = h->cs.n[0], ny = h->cs.n[1], nz = h->cs.n[2];
    return (nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1);
}

int dsmc_get_face_flux(dsmc_handle* h, const char* name, int species, double* out, long long n) {
    const std::string nm(name);
    const CaseDev& cs = h->cs;
    if (!cs.faceFlux) return fail(h, DSMC_ERR_INVALID, "face tracking is off (dsmc_set_face_tracking)");
    if (n != cs.nFacesAll) return fail(h, DSMC_ERR_INVALID, "n must equal dsmc_n_faces");
    if (species < 0 || species >= cs.nSpecies) return fail(h, DSMC_ERR_INVALID, "species index out of range");
    int k;
    if (nm == "parcelIdFlux") k = 0;
    else if (nm == "massIdFlux") k = 1;
    else return fail(h, DSMC_ERR_INVALID, "unknown face flux " + nm + " (parcelIdFlux, massIdFlux)");
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    CUDA_TRY(h, cudaMemcpy(out, cs.faceFlux + ((long long)k * cs.nSpecies + species) * cs.nFacesAll,
                           sizeof(double) * n, cudaMemcpyDeviceToHost));
    return DSMC_OK;
}

// ------------------------------------------------------- flux surfaces
namespace {

// The mesh face f of the tracker numbering: its axis, centre, area and the
// sign of its area vector along the axis (+ between two fluid cells and on
// the high side of a fluid cell, - on the low side).  False when no fluid
// cell touches it (inside a solid box): then it is not a mesh face.
bool face_geometry(const dsmc_handle* h, long long f, int* axis, double* centre, double* area, double* sgn) {
    const CaseDev& cs = h->cs;
    const long long nx = cs.n[0], ny = cs.n[1];
    int a, p, c[3];
    if (f < cs.faceOff[1]) {
        a = 0;
        p = (int)(f % (nx + 1));
        c[1] = (int)((f / (nx + 1)) % ny);
        c[2] = (int)(f / ((nx + 1) * ny));
    } else if (f < cs.faceOff[2]) {
        const long long l = f - cs.faceOff[1];
        a = 1;
        c[0] = (int)(l % nx);
        p = (int)((l / nx) % (ny + 1));
        c[2] = (int)(l / (nx * (ny + 1)));
    } else {
        const long long l = f - cs.faceOff[2];
        a = 2;
        c[0] = (int)(l % nx);
        c[1] = (int)((l / nx) % ny);
        p = (int)(l / (nx * ny));
    }
    auto fluid = [&](int i) {
        if (i < 0 || i >= cs.n[a]) return false;
        int q[3] = {c[0], c[1], c[2]};
        q[a] = i;
        return !h->solidHost[q[0] + (long long)cs.n[0] * (q[1] + (long long)cs.n[1] * q[2])];
    };
    const bool lo = fluid(p - 1), hi = fluid(p);
    if (!lo && !hi) return false;
    *axis = a;
    *sgn = lo ? 1.0 : -1.0;
    *area = 1.0;
    for (int b = 0; b < 3; ++b) {
        if (b == a) {
            centre[b] = h->node[b][p];
        } else {
            centre[b] = 0.5 * (h->node[b][c[b]] + h->node[b][c[b] + 1]);
            *area *= h->width[b][c[b]];
        }
    }
    return true;
}

}  // namespace

int dsmc_add_flux_surface(dsmc_handle* h, const dsmc_flux_surface* sf) {
    const CaseDev& cs = h->cs;
    dsmc_handle::FluxSurface fs{};
    fs.d = *sf;
    fs.d.field_name[DSMC_NAME_LEN - 1] = 0;
    fs.d.zone_name[DSMC_NAME_LEN - 1] = 0;
    const double* d = sf->direction;
    const double mag = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (!(mag > 0.0) || !std::isfinite(mag))
        return fail(h, DSMC_ERR_INVALID, std::string("flux surface ") + fs.d.zone_name + ": fluxDirection is zero");
    for (int a = 0; a < 3; ++a) fs.d.direction[a] = d[a] / mag;
    if (sf->species_mask == 0 || (sf->species_mask >> cs.nSpecies) != 0)
        return fail(h, DSMC_ERR_INVALID, std::string("flux surface ") + fs.d.zone_name +
                                             ": typeIds must name species of the cloud");
    for (const auto& o : h->surfaces)
        if (!std::strcmp(o.d.zone_name, fs.d.zone_name) && !std::strcmp(o.d.field_name, fs.d.field_name))
            return fail(h, DSMC_ERR_INVALID, std::string("flux surface ") + fs.d.zone_name + " (" +
                                                 fs.d.field_name + ") exists already");
    int rc = dsmc_set_face_tracking(h, 1);
    if (rc) return rc;
    std::vector<int> faces;
    std::vector<double> w;
    const long long nAll = cs.nFacesAll;
    for (long long f = 0; f < nAll; ++f) {
        int a;
        double x[3], area, sgn;
        if (!face_geometry(h, f, &a, x, &area, &sgn)) continue;
        bool in = true;
        for (int b = 0; b < 3; ++b) in = in && x[b] >= sf->box_min[b] && x[b] <= sf->box_max[b];
        if (!in) continue;
        faces.push_back((int)f);
        w.push_back(cs.FN * sgn * fs.d.direction[a]);
        fs.area += area;
    }
    if (faces.empty())
        return fail(h, DSMC_ERR_INVALID, std::string("Cannot find region: ") + fs.d.zone_name +
                                             " (no mesh face centre in its box)");
    fs.nF = (int)faces.size();
    if ((rc = dalloc(h, &fs.faces, fs.nF))) return rc;
    if ((rc = dalloc(h, &fs.w, fs.nF))) return rc;
    if (!h->surfOut && (rc = dalloc(h, &h->surfOut, 2))) return rc;
    CUDA_TRY(h, cudaMemcpy(fs.faces, faces.data(), sizeof(int) * fs.nF, cudaMemcpyHostToDevice));
    CUDA_TRY(h, cudaMemcpy(fs.w, w.data(), sizeof(double) * fs.nF, cudaMemcpyHostToDevice));
    h->surfaces.push_back(fs);
    return DSMC_OK;
}

int dsmc_n_flux_surfaces(const dsmc_handle* h) { return (int)h->surfaces.size(); }

int dsmc_get_flux_surface(dsmc_handle* h, int i, dsmc_flux_surface* surface, double* out) {
    if (i < 0 || i >= (int)h->surfaces.size()) return fail(h, DSMC_ERR_INVALID, "flux surface index out of range");
    const auto& fs = h->surfaces[i];
    if (surface) *surface = fs.d;
    if (!h->cs.faceFlux) return fail(h, DSMC_ERR_INVALID, "face tracking is off (dsmc_set_face_tracking)");
    launch_flux_surface(h->cs, fs.faces, fs.w, fs.nF, fs.d.species_mask, h->surfOut, h->stream);
    CUDA_TRY(h, cudaGetLastError());
    double sums[2];
    CUDA_TRY(h, cudaMemcpyAsync(sums, h->surfOut, sizeof(sums), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->ctrHost, h->B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    const long long steps = h->ctrHost->step - h->faceStep0;
    if (steps <= 0) return fail(h, DSMC_ERR_INVALID, "no step since the face sums were reset");
    // dsmcFluxSurface.C:364-386
    const double T = (double)steps * h->spec.delta_t;
    out[1] = sums[0] / T;
    out[0] = out[1] / fs.area;
    out[3] = sums[1] / T;
    out[2] = out[3] / fs.area;
    out[4] = fs.area;
    out[5] = T;
    return DSMC_OK;
}

int dsmc_write_flux_surfaces(dsmc_handle* h, const char* case_dir, double time_value) {
    const std::string dir = std::string(case_dir) + "/fieldMeasurements";
    mkdir(dir.c_str(), 0755);
    static const char* names[4] = {"faceParticleFlux_", "faceParticleFlowRate_", "faceMassFlux_",
                                   "faceMassFlowRate_"};
    for (int i = 0; i < (int)h->surfaces.size(); ++i) {
        double v[6];
        int rc = dsmc_get_flux_surface(h, i, nullptr, v);
        if (rc) return rc;
        const auto& d = h->surfaces[i].d;
        for (int k = 0; k < 4; ++k) {
            const std::string path = dir + "/" + names[k] + d.zone_name + "_" + d.field_name + ".xy";
            FILE* f = std::fopen(path.c_str(), "a");
            if (!f) return fail(h, DSMC_ERR_IO, "cannot open " + path);
            std::fprintf(f, "%.11g\t%.11g\n", time_value, v[k]);
            if (std::fclose(f)) return fail(h, DSMC_ERR_IO, "cannot write " + path);
        }
    }
    return DSMC_OK;
}

// ------------------------------------------------------- lagrangian files
namespace {

// one IOField file of a lagrangian cloud directory
bool write_ioField(const std::string& path, const char* cls, const std::string& location, const char* object,
                   long long n, const std::function<void(FILE*, long long)>& item, const char* uniform) {
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    std::fprintf(f, "%sFoamFile\n{\n    version     2.0;\n    format      ascii;\n    class       %s;\n"
                    "    location    \"%s\";\n    object      %s;\n}\n\n",
                 FOAM_BANNER, cls, location.c_str(), object);
    if (uniform) {
        std::fprintf(f, "%lld{%s}\n", n, uniform);
    } else {
        std::fprintf(f, "\n%lld\n(\n", n);
        for (long long k = 0; k < n; ++k) item(f, k);
        std::fprintf(f, ")\n");
    }
    std::fprintf(f, "\n\n// ************************************************************************* //\n");
    return std::fclose(f) == 0;
}

}  // namespace

int dsmc_write_parcels(dsmc_handle* h, const char* case_dir, const char* time_name, const char* cloud_name) {
    std::vector<long long> order;
    int rc = case_cell_order(h, case_dir, order);
    if (rc) return rc;
    std::vector<long long> label((size_t)h->cs.C, -1);
    for (size_t k = 0; k < order.size(); ++k) label[(size_t)order[k]] = (long long)k;
    long long n = 0;
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    CUDA_TRY(h, cudaMemcpy(h->ctrHost, h->B.ctr, sizeof(Counters), cudaMemcpyDeviceToHost));
    const long long cap = h->ctrHost->n;
    std::vector<double> pos(3 * (size_t)cap), U(3 * (size_t)cap), erot((size_t)cap);
    std::vector<int> vib((size_t)cap), sp((size_t)cap), cell((size_t)cap);
    std::vector<unsigned> id((size_t)cap);
    if ((rc = dsmc_get_particles(h, cap, &n, pos.data(), U.data(), erot.data(), vib.data(), sp.data(), id.data(),
                                 cell.data())))
        return rc;
    std::string dir = std::string(case_dir) + "/" + time_name;
    mkdir(dir.c_str(), 0755);
    dir += "/lagrangian";
    mkdir(dir.c_str(), 0755);
    dir += std::string("/") + cloud_name;
    mkdir(dir.c_str(), 0755);
    const std::string loc = std::string(time_name) + "/lagrangian/" + cloud_name;
    const dsmc_case_spec& s = h->spec;
    bool ok = true;
    // 17 significant digits: a written cloud reads back bit for bit
    ok &= write_ioField(dir + "/positions", "Cloud<dsmcParcel>", loc, "positions", n, [&](FILE* f, long long k) {
        std::fprintf(f, "(%.17g %.17g %.17g) %lld\n", pos[3 * k], pos[3 * k + 1], pos[3 * k + 2],
                     label[(size_t)cell[k]]);
    }, nullptr);
    ok &= write_ioField(dir + "/U", "vectorField", loc, "U", n, [&](FILE* f, long long k) {
        std::fprintf(f, "(%.17g %.17g %.17g)\n", U[3 * k], U[3 * k + 1], U[3 * k + 2]);
    }, nullptr);
    ok &= write_ioField(dir + "/ERot", "scalarField", loc, "ERot", n,
                        [&](FILE* f, long long k) { std::fprintf(f, "%.17g\n", erot[k]); }, nullptr);
    ok &= write_ioField(dir + "/typeId", "labelField", loc, "typeId", n,
                        [&](FILE* f, long long k) { std::fprintf(f, "%d\n", sp[k]); }, nullptr);
    ok &= write_ioField(dir + "/vibLevel", "labelFieldField", loc, "vibLevel", n, [&](FILE* f, long long k) {
        if (s.species[sp[k]].n_vib_modes > 0) std::fprintf(f, "1(%d)\n", vib[k]);
        else std::fprintf(f, "0()\n");
    }, nullptr);
    ok &= write_ioField(dir + "/origId", "labelField", loc, "origId", n,
                        [&](FILE* f, long long k) { std::fprintf(f, "%u\n", id[k]); }, nullptr);
    ok &= write_ioField(dir + "/newParcel", "labelField", loc, "newParcel", n, nullptr, "-1");
    ok &= write_ioField(dir + "/origProcId", "labelField", loc, "origProcId", n, nullptr, "0");
    ok &= write_ioField(dir + "/classification", "labelField", loc, "classification", n, nullptr, "0");
    std::vector<double> sm((size_t)h->cs.C);
    if ((rc = dsmc_get_cell_array(h, "sigmaTcRMax", sm.data(), h->cs.C))) return rc;
    const std::string sname = std::string(cloud_name) + "SigmaTcRMax";
    foam_write(std::string(case_dir) + "/" + time_name + "/" + sname, "volScalarField", sname, time_name,
               "[0 3 -1 0 0 0 0]", {sm.data()}, order, h->spec, &ok, 17);
    if (!ok) return fail(h, DSMC_ERR_IO, "cannot write the parcel files in " + dir);
    return DSMC_OK;
}

int dsmc_read_parcels(dsmc_handle* h, const char* case_dir, const char* time_name, const char* cloud_name) {
    long long n = 0;
    int rc = dsmc_parse_parcels(case_dir, time_name, cloud_name, &n, nullptr, nullptr, nullptr, nullptr, nullptr,
                                nullptr);
    if (rc) return fail(h, rc, dsmc_parse_last_error());
    std::vector<double> pos(3 * (size_t)n), U(3 * (size_t)n), erot((size_t)n);
    std::vector<int> vib((size_t)n), sp((size_t)n);
    std::vector<unsigned> id((size_t)n);
    rc = dsmc_parse_parcels(case_dir, time_name, cloud_name, &n, pos.data(), U.data(), erot.data(), vib.data(),
                            sp.data(), id.data());
    if (rc) return fail(h, rc, dsmc_parse_last_error());
    const CaseDev& cs = h->cs;
    for (long long k = 0; k < n; ++k)
        for (int a = 0; a < 3; ++a)
            if (!(pos[3 * k + a] >= cs.lo[a] && pos[3 * k + a] <= cs.hi[a]))
                return fail(h, DSMC_ERR_INVALID, "parcel " + std::to_string(k) + " lies outside the mesh");
    // the cloud's <name>SigmaTcRMax field of the same time (MUST_READ in
    // dsmcCloud.C:625-636); without it, the starting value of the mesh fill
    const std::string sfile = std::string(case_dir) + "/" + time_name + "/" + cloud_name + "SigmaTcRMax";
    std::vector<double> sf;
    std::string err;
    if (foam_read_scalar_field(sfile, sf, err)) {
        std::vector<long long> order;
        if ((rc = case_cell_order(h, case_dir, order))) return rc;
        if (sf.size() == 1) sf.assign(order.size(), sf[0]);
        if (sf.size() != order.size()) return fail(h, DSMC_ERR_INVALID, sfile + ": wrong number of cells");
        std::vector<double> sm((size_t)cs.C, 0.0);
        for (size_t k = 0; k < order.size(); ++k) sm[(size_t)order[k]] = sf[k];
        CUDA_TRY(h, cudaMemcpy(h->B.smax, sm.data(), sizeof(double) * cs.C, cudaMemcpyHostToDevice));
        h->smaxSet = true;
    } else if (!err.empty()) {
        return fail(h, DSMC_ERR_PARSE, err);
    } else if (!h->smaxSet) {
        if ((rc = init_smax(h))) return rc;
    }
    return dsmc_set_particles(h, n, pos.data(), U.data(), erot.data(), vib.data(), sp.data(), id.data());
}

}  // extern "C"
