// dsmc_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the dsmcFoam+ per-step particle path (dsmcCloud::evolve)
// on uniform Cartesian hexahedral meshes.  It is the checker for the GPU
// library and the timed CPU baseline; nothing in the product links, loads or
// calls it.  Only the test suite, the smoke check and the benchmark's CPU
// baseline leg use it.
//
// What it follows (paths inside hystrath/hyStrath):
//   step order            src/lagrangian/dsmc/clouds/dsmcCloud.C:819-926
//   inflow                .../generalBoundaries/dsmcFreeStreamInflowPatch/dsmcFreeStreamInflowPatch.C:91-364
//   move                  src/lagrangian/dsmc/parcels/dsmcParcel.C:38-148, Cloud.C:230-234
//   patch dispatch        dsmcParcel.C:174-204
//   specular wall         .../patchBoundaries/dsmcSpecularWallPatch/dsmcSpecularWallPatch.C:47-62
//   symmetry              src/lagrangian/basic/particle/particleTemplates.C:1511-1522
//   cyclic                particleTemplates.C:1525-1570
//   diffuse wall          .../patchBoundaries/dsmcDiffuseWallPatch/dsmcDiffuseWallPatch.C:67-138
//   wall unit vectors     .../basic/dsmcPatchBoundary/dsmcPatchBoundary.C:216-260
//   wall measurements     dsmcPatchBoundary.C:263-482
//   deletion              .../patchBoundaries/dsmcDeletionPatch/dsmcDeletionPatch.C:140-172
//   occupancy             dsmcCloud.C:63-74
//   NTC                   .../collisionPartnerSelection/derived/noTimeCounter/noTimeCounter.C:81-339
//   VHS                   .../collisions/derived/VariableHardSphere/VariableHardSphere.C:80-228
//   Larsen-Borgnakke      .../LarsenBorgnakkeVariableHardSphere/LarsenBorgnakkeVariableHardSphere.C:45-279
//   samplers              dsmcCloud.C:1015-1051, 1181-1244, 1327-1531
//   sampling              .../dsmcVolFields/dsmcVolFields.C:1071-1290 (sums), 1365-1876 (fields)
//   mesh fill             .../initialiseDsmcParcels/derived/dsmcMeshFill/dsmcMeshFill.C:68-238
//   processor transfer    src/lagrangian/basic/Cloud/Cloud.C:255-466 (stepBegin / addMigrants /
//                         stepEnd: a divided case's migrants arrive with their move complete)
//
// Random numbers: the reference draws from one sequential OpenFOAM Random
// stream, which lives outside the reference and cannot be replayed.  Here
// every draw comes from Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11),
// keyed by the case seed and countered by (object, step, block, tag), so the
// same draws can be made in any order.  The GPU library implements the same
// contract independently; moves, boundary crossings, cell indices and the
// occupancy sort then agree bit for bit (tests/test_parity_move_sort.py).
// Collisions and sampling agree statistically (transcendental functions differ
// between libm and CUDA by a few ulps).
//
// Cartesian restatement of tracking: a parcel advances along U for its
// remaining time; the earliest crossing of a domain side or of an obstacle
// face is found from the plane equation, the patch model is applied at the
// hit point and the rest of the time is tracked on.  In exact arithmetic this
// gives the same boundary events as the tet walk of trackToFace.
//
// Deviations, all statistically neutral: Box-Muller normals instead of the
// polar method; single-level electronic relaxation (which consumes draws but
// never changes state in the reference) is skipped; inflow tangents are the
// face axes instead of the face diagonal; the mesh fill draws 12 equal
// sub-volume counts per cell (the 12 tets of a hex) and places the parcels
// uniformly in the cell.

#include "hystrath_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// OpenFOAM v1706 constants (physicoChemicalConstants, doubleScalar.H).
const double kB = 1.3806504e-23;
const double NAvo = 6.0221417930e+23;   // physicoChemical::NA of the same (CODATA 2006) set
const double PI = 3.14159265358979323846;
const double SMALL = 1.0e-15;
const double VSMALL = 1.0e-300;
const double ROOTVSMALL = 1.0e-150;
const double GREAT = 1.0e15;

// Loop caps: the reference loops without bound; a capped loop flags an error.
const int MAX_CROSSINGS = 64;
const int MAX_REJECTION = 100000;

// ---------------------------------------------------------------- Philox
// Philox-4x32-10: multipliers, Weyl key increments and round function as
// published by Salmon et al. (SC'11, "Parallel random numbers: as easy as
// 1, 2, 3").
struct Philox {
    static void round(uint32_t c[4], const uint32_t k[2]) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c[1] ^ k[0];
        const uint32_t n2 = hi0 ^ c[3] ^ k[1];
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    }
    static void gen(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
        uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
        uint32_t k[2] = {key[0], key[1]};
        for (int r = 0; r < 10; ++r) {
            if (r) { k[0] += 0x9E3779B9u; k[1] += 0xBB67AE85u; }
            round(c, k);
        }
        out[0] = c[0]; out[1] = c[1]; out[2] = c[2]; out[3] = c[3];
    }
};

// Stream tags (counter word 3, low byte) of the random-number contract.
enum : uint32_t {
    TAG_MOVE = 1, TAG_COLLIDE = 2, TAG_INFLOW = 3, TAG_INIT_CELL = 4,
    TAG_INIT_PARTICLE = 5, TAG_REMAINDER = 6
};

// (2k+1) * 2^-53 for the top 52 bits k of a 64-bit word: uniform in (0,1).
inline double u01_from(uint32_t lo, uint32_t hi) {
    const uint64_t k = ((((uint64_t)hi) << 32) | lo) >> 12;
    const uint64_t bits = 0x3FF0000000000000ull | k;
    double d;
    std::memcpy(&d, &bits, 8);
    return d - (1.0 - 0x1p-53);
}

struct Rng {
    uint32_t ctr[4];
    uint32_t key[2];
    uint32_t buf[4];
    int have;     // doubles left in buf (0..2)
    Rng(uint64_t seed, uint32_t obj, uint32_t step, uint32_t tag) {
        key[0] = (uint32_t)seed; key[1] = (uint32_t)(seed >> 32);
        ctr[0] = obj; ctr[1] = step; ctr[2] = 0; ctr[3] = tag;
        have = 0;
    }
    double u01() {
        if (have == 0) {
            Philox::gen(ctr, key, buf);
            ctr[2] += 1;
            have = 2;
            return u01_from(buf[0], buf[1]);
        }
        have = 0;
        return u01_from(buf[2], buf[3]);
    }
    // dsmcCloud::randomLabel (dsmcCloud.C:1015-1040), bounded redraw.
    int label(int a, int b, int* err) {
        if (a == b) return a;
        const int s = std::min(a, b), e = std::max(a, b);
        for (int it = 0; it < MAX_REJECTION; ++it) {
            const int v = s + (int)(u01() * (double)(e - s + 1));
            if (v != e + 1) return v;
        }
        *err = 1;
        return s;
    }
    // Box-Muller pair of standard normals.
    void gauss2(double* g1, double* g2) {
        const double u1 = u01();
        const double u2 = u01();
        const double r = std::sqrt(-2.0 * std::log(u1));
        *g1 = r * std::cos(2.0 * PI * u2);
        *g2 = r * std::sin(2.0 * PI * u2);
    }
};

// ---------------------------------------------------------------- state
struct Parcel {
    double x[3];
    double U[3];
    double erot;
    int vib;
    int type;
    uint32_t id;
    int cell;       // -1 once deleted
    int sub;        // sub-cell bits (x | y<<1 | z<<2)
    int fresh;      // newParcel != -1: random step fraction on its first move
};

struct Species {
    double m, d, omega, rotDof, thetaV, thetaD, zref, trefZv;
    int nVib;
    double alpha;   // VariableSoftSphere deflection exponent
};

struct WallAcc {   // per boundary face, dsmcPatchBoundary.C:263-482
    double rhoN, rhoM, linearKE, mcc, mom[3], erot, zetaRot, evib, q, fD[3];
};

enum { ACC_N = 0, ACC_M, ACC_MOMX, ACC_MOMY, ACC_MOMZ, ACC_MCC, ACC_EROT, ACC_ZETAROT,
       ACC_NCOLLS, ACC_COLLSEP, ACC_COMMON };
enum { SACC_N = 0, SACC_MCC, SACC_EVIB, SACC_PER_SPECIES };

struct Oracle {
    dsmc_case_spec spec;
    std::vector<std::vector<int>> facePatchStore;   // copies of face_patch maps
    int n[3];
    long long C;
    double lo[3], hi[3], dx[3], inv[3], negOinv[3];
    double mid[3];          // mesh bounding-box midpoint
    // rectilinear grading: nodes and widths of every axis (a uniform axis has
    // origin + i dx and dx), the 2n+1 half-node coordinates of a graded axis
    // (empty when uniform) and the cell volumes of a graded mesh
    std::vector<double> node[3], width[3], half[3], cellVol;
    int emptyAx[3];         // reduced-D: both sides of the axis are empty patches
    double V;
    std::vector<Species> sp;
    std::vector<uint8_t> solid;
    // boundary faces: 6 domain sides then obstacle sides
    long long sideOff[7];
    std::vector<long long> obstOff;   // [o*6+s]
    long long nBFaces;
    std::vector<int> bfPatch;
    std::vector<double> bfArea;
    double obLo[DSMC_MAX_OBSTACLES][3], obHi[DSMC_MAX_OBSTACLES][3];

    std::vector<Parcel> P;
    std::vector<Parcel> Pbuf;                   // the sort's destination, swapped with P
    std::vector<int> cellStart, cellCount;      // occupancy after the last sort
    std::vector<double> sigmaTcRMax, remainder;
    std::vector<double> acc;                    // [C][nAcc]
    // measureHeatFluxShearStress (dsmcVolFields.C:1186-1206): per cell
    // sum m u_i u_j (xx xy xz yy yz zz), m |U|^2 u_i, E_int u_i; empty when off
    std::vector<double> mom;                    // [C][12]
    int nAcc;
    std::vector<WallAcc> wall;
    std::vector<double> inflowAcc;              // [nBFaces][nSpecies]
    std::vector<double> faceFlux;               // [2][nSpecies][nFacesAll]; empty: tracking off
    long long faceOff[3], nFacesAll;
    long long step;
    uint32_t nextId;
    long long sampleSteps;
    long long collLast, candLast, collTot, candTot, wallHitsLast, insertedLast, deletedLast;
    // spatial decomposition (dsmc_set_domain's restatement): the parcels of
    // cells lo <= index < hi along domAxis are this domain's; -1: all
    int domAxis = -1, domLo = 0, domHi = 0;
    std::vector<uint32_t> migOut;               // the step's migrants, 17 words each
    long long migLast = 0;                      // migrants sent by the last step
    int err;
    int nThreads;
    std::string msg;

    // ------------------------------------------------------------ geometry
    // Index of the doubled cell coordinate: floor(2 t), t = x/dx - x0/dx.
    long long floor2(double x, int a) const {
        if (!half[a].empty()) {
            // graded: k with h[k] <= x < h[k+1], -1 below and 2n from h[2n] on
            const std::vector<double>& h = half[a];
            const int m = 2 * n[a];
            if (!(x >= h[0])) return -1;
            if (x >= h[m]) return m;
            int l = 0, u = m;
            while (u - l > 1) {
                const int md = (l + u) >> 1;
                if (h[md] <= x) l = md; else u = md;
            }
            return l;
        }
        const double t = std::fma(x, inv[a], negOinv[a]);
        return (long long)std::floor(2.0 * t);
    }
    double nodeX(int a, long long p) const { return half[a].empty() ? lo[a] + p * dx[a] : half[a][2 * p]; }
    double cellW(int a, long long i) const { return half[a].empty() ? dx[a] : half[a][2 * i + 2] - half[a][2 * i]; }
    double cellVolume(long long c) const { return cellVol.empty() ? V : cellVol[c]; }
    void cellOf(const double x[3], int* cell, int* sub) const {
        int ci[3];
        int sb = 0;
        for (int a = 0; a < 3; ++a) {
            long long c2 = floor2(x[a], a);
            if (c2 < 0) c2 = 0;
            if (c2 > 2LL * n[a] - 1) c2 = 2LL * n[a] - 1;
            ci[a] = (int)(c2 >> 1);
            sb |= (int)(c2 & 1) << a;
        }
        *cell = ci[0] + n[0] * (ci[1] + n[1] * ci[2]);
        *sub = sb;
    }
    // ------------------------------------------------------------ face tracker
    // dsmcFaceTracker::trackFaceTransition (dsmcFaceTracker.C:124-190):
    // sign(U . S) and sign(U . S) m on every face crossed, S = +axis inside
    // and outward on the boundary.  Faces: x faces, then y, then z.
    long long faceIndex(int a, long long p, const int* cell) const {
        const long long nx = n[0], ny = n[1];
        if (a == 0) return faceOff[0] + p + (nx + 1) * (cell[1] + ny * cell[2]);
        if (a == 1) return faceOff[1] + cell[0] + nx * (p + (ny + 1) * cell[2]);
        return faceOff[2] + cell[0] + nx * (cell[1] + ny * p);
    }
    void faceAdd(long long f, int m, double sgn) {
        double* a = &faceFlux[(size_t)m * nFacesAll + f];
        double* b = &faceFlux[((size_t)spec.n_species + m) * nFacesAll + f];
        const double dm = sgn * sp[m].m;
#pragma omp atomic
        *a += sgn;
#pragma omp atomic
        *b += dm;
    }
    // faces crossed on the straight path from x in cell sc to cell te, in the
    // order of their crossing times (ties: the lower axis first)
    void trackInternal(const double* x, const double* U, const int* sc, const int* te, int m) {
        int cur[3] = {sc[0], sc[1], sc[2]}, left[3], dir[3];
        double t[3] = {0.0, 0.0, 0.0};
        for (int a = 0; a < 3; ++a) {
            const int d = te[a] - sc[a];
            left[a] = std::abs(d);
            dir[a] = d > 0 ? 1 : -1;
            if (left[a]) t[a] = (nodeX(a, d > 0 ? sc[a] + 1 : sc[a]) - x[a]) / U[a];
        }
        while (left[0] + left[1] + left[2] > 0) {
            int a = -1;
            for (int b = 0; b < 3; ++b)
                if (left[b] && (a < 0 || t[b] < t[a])) a = b;
            faceAdd(faceIndex(a, dir[a] > 0 ? cur[a] + 1 : cur[a], cur), m, dir[a] > 0 ? 1.0 : -1.0);
            cur[a] += dir[a];
            if (--left[a]) t[a] = (nodeX(a, dir[a] > 0 ? cur[a] + 1 : cur[a]) - x[a]) / U[a];
        }
    }

    int patchOfSideFace(int s, long long f) const {
        const int* fp = spec.face_patch[s];
        return fp ? fp[f] : spec.side_patch[s];
    }
    // face index on side s of the hit point x
    long long sideFace(int s, const double x[3]) const {
        const int a = s / 2;
        const int b = (a == 0) ? 1 : 0;
        const int c = (a == 2) ? 1 : 2;
        long long ib = floor2(x[b], b) >> 1;
        long long ic = floor2(x[c], c) >> 1;
        ib = std::min<long long>(std::max<long long>(ib, 0), n[b] - 1);
        ic = std::min<long long>(std::max<long long>(ic, 0), n[c] - 1);
        return ib + (long long)n[b] * ic;
    }
    long long obstFace(int o, int s, const double x[3]) const {
        const dsmc_obstacle& ob = spec.obstacles[o];
        const int a = s / 2;
        const int b = (a == 0) ? 1 : 0;
        const int c = (a == 2) ? 1 : 2;
        long long ib = (floor2(x[b], b) >> 1) - ob.lo[b];
        long long ic = (floor2(x[c], c) >> 1) - ob.lo[c];
        const int nb = ob.hi[b] - ob.lo[b], nc = ob.hi[c] - ob.lo[c];
        ib = std::min<long long>(std::max<long long>(ib, 0), nb - 1);
        ic = std::min<long long>(std::max<long long>(ic, 0), nc - 1);
        return obstOff[o * 6 + s] + ib + (long long)nb * ic;
    }

    bool setup(const dsmc_case_spec* s) {
        spec = *s;
        for (int a = 0; a < 3; ++a) {
            n[a] = s->n_cells[a];
            if (n[a] <= 0) { msg = "invalid mesh"; return false; }
            node[a].resize((size_t)n[a] + 1);
            width[a].resize((size_t)n[a]);
            if (s->node_coords[a]) {
                for (int i = 0; i <= n[a]; ++i) node[a][i] = s->node_coords[a][i];
                for (int i = 0; i < n[a]; ++i) width[a][i] = node[a][i + 1] - node[a][i];
                half[a].resize(2 * (size_t)n[a] + 1);
                for (int i = 0; i <= n[a]; ++i) half[a][2 * (size_t)i] = node[a][i];
                for (int i = 0; i < n[a]; ++i) half[a][2 * (size_t)i + 1] = 0.5 * (node[a][i] + node[a][i + 1]);
                lo[a] = node[a].front();
                hi[a] = node[a].back();
                dx[a] = (hi[a] - lo[a]) / n[a];
                inv[a] = 1.0 / dx[a];
                negOinv[a] = -(lo[a] * inv[a]);
            } else {
                dx[a] = s->cell_size[a];
                if (!(dx[a] > 0)) { msg = "invalid mesh"; return false; }
                inv[a] = 1.0 / dx[a];
                negOinv[a] = -(s->origin[a] * inv[a]);
                lo[a] = s->origin[a];
                hi[a] = s->origin[a] + n[a] * dx[a];
                for (int i = 0; i <= n[a]; ++i) node[a][i] = s->origin[a] + i * s->cell_size[a];
                for (int i = 0; i < n[a]; ++i) width[a][i] = dx[a];
            }
            spec.node_coords[a] = nullptr;   // the copies above are used
        }
        for (int q = 0; q < 6; ++q) {
            if (s->face_patch[q]) {
                const int a = q / 2;
                const int b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
                facePatchStore.emplace_back(s->face_patch[q], s->face_patch[q] + (long long)n[b] * n[c]);
                spec.face_patch[q] = facePatchStore.back().data();
            }
        }
        for (int a = 0; a < 3; ++a) {
            mid[a] = 0.5 * (lo[a] + hi[a]);
            const int p = spec.face_patch[2 * a] ? spec.face_patch[2 * a][0] : spec.side_patch[2 * a];
            emptyAx[a] = spec.patches[p].type == DSMC_PATCH_EMPTY;
        }
        C = (long long)n[0] * n[1] * n[2];
        V = dx[0] * dx[1] * dx[2];
        if (!half[0].empty() || !half[1].empty() || !half[2].empty()) {
            cellVol.resize((size_t)C);
            for (long long c = 0; c < C; ++c)
                cellVol[c] = width[0][c % n[0]] * width[1][(c / n[0]) % n[1]] * width[2][c / ((long long)n[0] * n[1])];
        }
        sp.resize(s->n_species);
        for (int i = 0; i < s->n_species; ++i) {
            const dsmc_species& q = s->species[i];
            sp[i] = Species{q.mass, q.diameter, q.omega, q.rotational_dof, q.theta_v, q.theta_d,
                            q.zref, q.tref_zv, q.n_vib_modes, q.alpha};
        }
        solid.assign(C, 0);
        for (int o = 0; o < s->n_obstacles; ++o) {
            const dsmc_obstacle& ob = s->obstacles[o];
            for (int k = ob.lo[2]; k < ob.hi[2]; ++k)
                for (int j = ob.lo[1]; j < ob.hi[1]; ++j)
                    for (int i = ob.lo[0]; i < ob.hi[0]; ++i)
                        solid[i + (long long)n[0] * (j + (long long)n[1] * k)] = 1;
            for (int a = 0; a < 3; ++a) {
                obLo[o][a] = node[a][ob.lo[a]];
                obHi[o][a] = node[a][ob.hi[a]];
            }
        }
        long long off = 0;
        for (int q = 0; q < 6; ++q) {
            const int a = q / 2;
            const int b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
            sideOff[q] = off;
            for (long long f = 0; f < (long long)n[b] * n[c]; ++f) {
                bfPatch.push_back(patchOfSideFace(q, f));
                bfArea.push_back(width[b][f % n[b]] * width[c][f / n[b]]);
            }
            off += (long long)n[b] * n[c];
        }
        sideOff[6] = off;
        obstOff.assign(6 * DSMC_MAX_OBSTACLES, 0);
        for (int o = 0; o < s->n_obstacles; ++o) {
            const dsmc_obstacle& ob = s->obstacles[o];
            for (int q = 0; q < 6; ++q) {
                const int a = q / 2;
                const int b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
                obstOff[o * 6 + q] = off;
                const long long nf = (long long)(ob.hi[b] - ob.lo[b]) * (ob.hi[c] - ob.lo[c]);
                const int nb = ob.hi[b] - ob.lo[b];
                for (long long f = 0; f < nf; ++f) {
                    bfPatch.push_back(ob.patch[q]);
                    bfArea.push_back(width[b][ob.lo[b] + f % nb] * width[c][ob.lo[c] + f / nb]);
                }
                off += nf;
            }
        }
        nBFaces = off;
        wall.assign(nBFaces, WallAcc{});
        inflowAcc.assign(nBFaces * s->n_species, 0.0);
        nAcc = ACC_COMMON + SACC_PER_SPECIES * s->n_species;
        acc.assign(C * nAcc, 0.0);
        if (s->measure_heat_flux_shear_stress) mom.assign(C * 12, 0.0);
        sigmaTcRMax.assign(C, 0.0);
        remainder.assign(C, 0.0);
        for (long long c = 0; c < C; ++c) {
            Rng r(s->seed, (uint32_t)c, 0, TAG_REMAINDER);
            remainder[c] = r.u01();
        }
        cellStart.assign(C, 0);
        cellCount.assign(C, 0);
        step = 0; nextId = 0; sampleSteps = 0;
        collLast = candLast = collTot = candTot = wallHitsLast = insertedLast = deletedLast = 0;
        err = 0;
        return true;
    }

    // ------------------------------------------------------------ samplers
    // equipartitionRotationalEnergy, dsmcCloud.C:1181-1218
    double eqRot(Rng& r, double T, double dof, int* e) const {
        if (dof < SMALL) return 0.0;
        if (dof < 2.0 + SMALL && dof > 2.0 - SMALL) return -std::log(r.u01()) * kB * T;
        const double a = 0.5 * dof - 1;
        for (int it = 0; it < MAX_REJECTION; ++it) {
            const double ratio = 10 * r.u01();
            const double Pr = std::pow(ratio / a, a) * std::exp(a - ratio);
            if (!(Pr < r.u01())) return ratio * kB * T;
        }
        *e = 1;
        return 0.0;
    }
    // equipartitionVibrationalEnergyLevel, dsmcCloud.C:1221-1244
    int eqVib(Rng& r, double T, const Species& s) const {
        if (s.nVib == 0) return 0;
        return (int)(-std::log(r.u01()) * T / s.thetaV);
    }
    // postCollisionRotationalEnergy, dsmcCloud.C:1327-1387
    double postRot(Rng& r, double dof, double ChiB, int* e) const {
        if (dof == 2.0) return 1.0 - std::pow(r.u01(), 1.0 / ChiB);
        const double ChiA = 0.5 * dof;
        const double A1 = ChiA - 1., B1 = ChiB - 1.;
        if (A1 < SMALL && B1 < SMALL) return r.u01();
        for (int it = 0; it < MAX_REJECTION; ++it) {
            const double ratio = r.u01();
            double Pr;
            if (A1 < SMALL) Pr = std::pow(1.0 - ratio, B1);
            else if (B1 < SMALL) Pr = std::pow(1.0 - ratio, A1);
            else Pr = std::pow((A1 + B1) * ratio / A1, A1) * std::pow((A1 + B1) * (1 - ratio) / B1, B1);
            if (!(Pr < r.u01())) return ratio;
        }
        *e = 1;
        return 0.0;
    }
    // postCollisionVibrationalEnergyLevel (non-reacting branch), dsmcCloud.C:1390-1531
    int postVib(Rng& r, int vib, int iMax, const Species& s, double omega, double Ec, int* e) const {
        double invZv;
        if (spec.fixed_zv == 0) {
            // formulations 0 and 2 use the quantised collision temperature;
            // formulation 1 would use the overall macroscopic temperature.
            const double T = iMax * s.thetaV / (3.5 - omega);
            const double pow1 = std::pow(s.thetaD / T, 1. / 3.) - 1.0;
            const double pow2 = std::pow(s.thetaD / s.trefZv, 1. / 3.) - 1.0;
            const double ZvP1 = std::pow(s.thetaD / T, omega);
            const double ZvP2 = std::pow(s.zref * std::pow(s.thetaD / s.trefZv, -omega), pow1 / pow2);
            const double Zv = ZvP1 * ZvP2;
            invZv = (spec.inv_zv_formulation == 2) ? 1.0 / (5.0 * Zv) : 1.0 / Zv;
        } else {
            invZv = 1.0 / spec.fixed_zv;
        }
        if (invZv > r.u01()) {
            for (int it = 0; it < MAX_REJECTION; ++it) {
                const int iDash = r.label(0, iMax, e);
                const double EVib = iDash * kB * s.thetaV;
                const double func = std::pow(1.0 - EVib / Ec, 1.5 - omega);
                if (!(func < r.u01())) return iDash;
            }
            *e = 1;
        }
        return vib;
    }

    // ------------------------------------------------------------ wall
    void measure(const Parcel& p, long long bf, int axis, double sgn, bool after, double* preE,
                 double preMom[3]) {
        const Species& s = sp[p.type];
        const double fA = bfArea[bf];
        double nw[3] = {0, 0, 0};
        nw[axis] = sgn;
        const double Un = p.U[0] * nw[0] + p.U[1] * nw[1] + p.U[2] * nw[2];
        double Ut[3];
        for (int a = 0; a < 3; ++a) Ut[a] = p.U[a] - Un * nw[a];
        const double w = 1.0 / std::max(std::fabs(Un) * fA * spec.delta_t, SMALL);
        const double UU = p.U[0] * p.U[0] + p.U[1] * p.U[1] + p.U[2] * p.U[2];
        const double evib = (s.nVib ? p.vib * kB * s.thetaV : 0.0);
        WallAcc& W = wall[bf];
        W.rhoN += w;
        W.rhoM += s.m * w;
        W.linearKE += 0.5 * s.m * UU * w;
        W.mcc += s.m * UU * w;
        for (int a = 0; a < 3; ++a) W.mom[a] += s.m * Ut[a] * w;
        W.erot += p.erot * w;
        W.zetaRot += s.rotDof * w;
        W.evib += evib * w;
        const double E = 0.5 * s.m * UU + p.erot + evib;
        if (!after) {
            *preE = E;
            for (int a = 0; a < 3; ++a) preMom[a] = s.m * p.U[a];
        } else {
            const double nPar = spec.n_equivalent_particles;
            W.q += nPar * (*preE - E) / (spec.delta_t * fA);
            for (int a = 0; a < 3; ++a)
                W.fD[a] += nPar * (preMom[a] - s.m * p.U[a]) / (spec.delta_t * fA);
        }
    }

    // dsmcDiffuseWallPatch::performDiffuseReflection with
    // dsmcPatchBoundary::calculateWallUnitVectors, for a face of outward
    // normal sgn*e_axis.
    void diffuse(Parcel& p, Rng& r, int axis, double sgn, const dsmc_patch& pt, int* e) {
        const Species& s = sp[p.type];
        double nw[3] = {0, 0, 0};
        nw[axis] = sgn;
        double Un = p.U[0] * nw[0] + p.U[1] * nw[1] + p.U[2] * nw[2];
        double Ut[3];
        for (int a = 0; a < 3; ++a) Ut[a] = p.U[a] - Un * nw[a];
        double magUt = std::sqrt(Ut[0] * Ut[0] + Ut[1] * Ut[1] + Ut[2] * Ut[2]);
        int it = 0;
        while (magUt < SMALL) {
            if (++it > MAX_REJECTION) {
                *e = 1;
                Ut[0] = Ut[1] = Ut[2] = 0.0;
                Ut[(axis + 1) % 3] = 1.0;
                magUt = 1.0;
                break;
            }
            for (int a = 0; a < 3; ++a) p.U[a] = p.U[a] * (0.8 + 0.2 * r.u01());
            Un = p.U[0] * nw[0] + p.U[1] * nw[1] + p.U[2] * nw[2];
            for (int a = 0; a < 3; ++a) Ut[a] = p.U[a] - Un * nw[a];
            magUt = std::sqrt(Ut[0] * Ut[0] + Ut[1] * Ut[1] + Ut[2] * Ut[2]);
        }
        double t1[3], t2[3];
        for (int a = 0; a < 3; ++a) t1[a] = Ut[a] / magUt;
        t2[0] = nw[1] * t1[2] - nw[2] * t1[1];
        t2[1] = nw[2] * t1[0] - nw[0] * t1[2];
        t2[2] = nw[0] * t1[1] - nw[1] * t1[0];
        const double T = pt.wall_temperature;
        double g1, g2;
        r.gauss2(&g1, &g2);
        const double un = std::sqrt(-2.0 * std::log(std::max(1 - r.u01(), VSMALL)));
        const double sc = std::sqrt(kB * T / s.m);
        for (int a = 0; a < 3; ++a) p.U[a] = sc * (g1 * t1[a] + g2 * t2[a] - un * nw[a]);
        p.erot = eqRot(r, T, s.rotDof, e);
        p.vib = eqVib(r, T, s);
        for (int a = 0; a < 3; ++a) p.U[a] += pt.wall_velocity[a];
    }

    // Returns false when the parcel is deleted.
    bool applyPatch(Parcel& p, Rng& r, int patch, long long bf, int axis, double sgn, int* e,
                    long long* hits) {
        const dsmc_patch& pt = spec.patches[patch];
        if (pt.type == DSMC_PATCH_SYMMETRY) {
            p.U[axis] = -p.U[axis];
            return true;
        }
        if (pt.type == DSMC_PATCH_CYCLIC) {
            return true;   // translation done by the caller
        }
        switch (pt.model) {
        case DSMC_BC_SPECULAR: {
            double preE, preM[3];
            measure(p, bf, axis, sgn, false, &preE, preM);
            if (p.U[axis] * sgn > 0.0) p.U[axis] = -p.U[axis];
            measure(p, bf, axis, sgn, true, &preE, preM);
            ++*hits;
            return true;
        }
        case DSMC_BC_DIFFUSE: {
            double preE, preM[3];
            measure(p, bf, axis, sgn, false, &preE, preM);
            diffuse(p, r, axis, sgn, pt, e);
            measure(p, bf, axis, sgn, true, &preE, preM);
            ++*hits;
            return true;
        }
        case DSMC_BC_DELETION:
            return false;
        default:
            *e = 1;
            return false;
        }
    }

    // dsmcParcel::move on the Cartesian mesh.
    void moveParcel(Parcel& p, int* e, long long* hits) {
        Rng r(spec.seed, p.id, (uint32_t)step, TAG_MOVE);
        double tr = spec.delta_t;
        if (p.fresh) {
            const double sf = r.u01();
            p.fresh = 0;
            tr = (1.0 - sf) * spec.delta_t;
        }
        int startCell[3];
        {
            int c = p.cell;
            startCell[0] = c % n[0];
            startCell[1] = (c / n[0]) % n[1];
            startCell[2] = c / (n[0] * n[1]);
        }
        for (int it = 0;; ++it) {
            if (!(tr > ROOTVSMALL)) break;
            if (it >= MAX_CROSSINGS) { *e = 1; break; }
            // dsmcParcel.C:73-84: the position is held at the mesh centre and
            // the tracking velocity is zero along a reduced-D (empty) axis
            double V[3] = {p.U[0], p.U[1], p.U[2]};
            for (int a = 0; a < 3; ++a)
                if (emptyAx[a]) { p.x[a] = mid[a]; V[a] = 0.0; }
            double ex[3];
            long long c2[3];
            int ci[3];
            bool out = false;
            for (int a = 0; a < 3; ++a) {
                ex[a] = std::fma(V[a], tr, p.x[a]);
                c2[a] = floor2(ex[a], a);
                ci[a] = (int)(c2[a] >> 1);
                if (ci[a] < 0 || ci[a] >= n[a]) out = true;
            }
            bool obst = false;
            for (int o = 0; o < spec.n_obstacles && !obst; ++o) {
                const dsmc_obstacle& ob = spec.obstacles[o];
                bool ov = true;
                // the path stays in the box of cells spanned by its end cells
                for (int a = 0; a < 3; ++a) {
                    const int mn = std::min(startCell[a], ci[a]);
                    const int mx = std::max(startCell[a], ci[a]);
                    if (mx < ob.lo[a] || mn > ob.hi[a] - 1) ov = false;
                }
                obst = ov;
            }
            if (!out && !obst) {
                if (!faceFlux.empty()) trackInternal(p.x, V, startCell, ci, p.type);
                for (int a = 0; a < 3; ++a) p.x[a] = ex[a];
                int sb = 0;
                for (int a = 0; a < 3; ++a) sb |= (int)(c2[a] & 1) << a;
                p.cell = ci[0] + n[0] * (ci[1] + n[1] * ci[2]);
                p.sub = sb;
                return;
            }
            // earliest event: domain sides first, then obstacles
            double tHit = GREAT * GREAT;
            int hitKind = -1, hitSide = -1;   // kind 0: domain side, 1+o: obstacle o
            for (int a = 0; a < 3; ++a) {
                if (ci[a] < 0) {
                    double t = (lo[a] - p.x[a]) / V[a];
                    if (!(t >= 0.0)) t = 0.0;
                    if (t > tr) t = tr;
                    if (t < tHit) { tHit = t; hitKind = 0; hitSide = 2 * a; }
                } else if (ci[a] >= n[a]) {
                    double t = (hi[a] - p.x[a]) / V[a];
                    if (!(t >= 0.0)) t = 0.0;
                    if (t > tr) t = tr;
                    if (t < tHit) { tHit = t; hitKind = 0; hitSide = 2 * a + 1; }
                }
            }
            for (int o = 0; o < spec.n_obstacles; ++o) {
                double tin = -GREAT * GREAT, tout = GREAT * GREAT;
                int ax = -1;
                bool miss = false;
                for (int a = 0; a < 3; ++a) {
                    if (V[a] != 0.0) {
                        const double t1 = (obLo[o][a] - p.x[a]) / V[a];
                        const double t2 = (obHi[o][a] - p.x[a]) / V[a];
                        const double ta = std::min(t1, t2), tb = std::max(t1, t2);
                        if (ta > tin) { tin = ta; ax = a; }
                        if (tb < tout) tout = tb;
                    } else if (p.x[a] < obLo[o][a] || p.x[a] > obHi[o][a]) {
                        miss = true;
                    }
                }
                if (!miss && ax >= 0 && tin >= 0.0 && tin < tout && tin <= tr && tin < tHit) {
                    tHit = tin;
                    hitKind = 1 + o;
                    hitSide = 2 * ax + (V[ax] > 0.0 ? 0 : 1);
                }
            }
            if (hitKind < 0) {
                // obstacle candidate without an actual hit
                if (!faceFlux.empty()) trackInternal(p.x, V, startCell, ci, p.type);
                for (int a = 0; a < 3; ++a) p.x[a] = ex[a];
                int sb = 0;
                for (int a = 0; a < 3; ++a) sb |= (int)(c2[a] & 1) << a;
                p.cell = ci[0] + n[0] * (ci[1] + n[1] * ci[2]);
                p.sub = sb;
                return;
            }
            const int axis = hitSide / 2;
            double plane;
            if (hitKind == 0) plane = (hitSide & 1) ? hi[axis] : lo[axis];
            else plane = (hitSide & 1) ? obHi[hitKind - 1][axis] : obLo[hitKind - 1][axis];
            double x0[3] = {p.x[0], p.x[1], p.x[2]};
            for (int a = 0; a < 3; ++a) p.x[a] = (a == axis) ? plane : std::fma(V[a], tHit, p.x[a]);
            // the fluid cell at the hit point and the plane index of the face hit
            int hitCell[3];
            long long facePlane;
            for (int a = 0; a < 3; ++a) {
                const long long cc = floor2(p.x[a], a) >> 1;
                hitCell[a] = (int)std::min<long long>(std::max<long long>(cc, 0), n[a] - 1);
            }
            if (hitKind == 0) {
                facePlane = (hitSide & 1) ? n[axis] : 0;
                hitCell[axis] = (hitSide & 1) ? n[axis] - 1 : 0;
            } else {
                const dsmc_obstacle& ob = spec.obstacles[hitKind - 1];
                facePlane = (hitSide & 1) ? ob.hi[axis] : ob.lo[axis];
                hitCell[axis] = (int)((hitSide & 1) ? facePlane : facePlane - 1);
            }
            if (!faceFlux.empty()) trackInternal(x0, V, startCell, hitCell, p.type);
            tr = tr - tHit;
            long long bf;
            int patch;
            double sgn;
            if (hitKind == 0) {
                const long long f = sideFace(hitSide, p.x);
                bf = sideOff[hitSide] + f;
                patch = bfPatch[bf];
                sgn = (hitSide & 1) ? 1.0 : -1.0;       // outward normal of the domain side
            } else {
                bf = obstFace(hitKind - 1, hitSide, p.x);
                patch = bfPatch[bf];
                sgn = (hitSide & 1) ? -1.0 : 1.0;       // normal pointing into the solid
            }
            const bool kept = applyPatch(p, r, patch, bf, axis, sgn, e, hits);
            if (!faceFlux.empty()) {
                // after the interaction (deletion: the unchanged velocity); a
                // cyclic crossing counts +1 on the face it leaves through
                const bool cyc = spec.patches[patch].type == DSMC_PATCH_CYCLIC;
                if (!cyc || hitKind == 0)
                    faceAdd(faceIndex(axis, facePlane, hitCell), p.type,
                            cyc ? 1.0 : (p.U[axis] * sgn > 0.0 ? 1.0 : -1.0));
            }
            if (!kept) {
                p.cell = -1;
                return;
            }
            if (spec.patches[patch].type == DSMC_PATCH_CYCLIC && hitKind == 0)
                p.x[axis] = (hitSide & 1) ? lo[axis] : hi[axis];
            for (int a = 0; a < 3; ++a) {
                long long c = floor2(p.x[a], a) >> 1;
                c = std::min<long long>(std::max<long long>(c, 0), n[a] - 1);
                startCell[a] = (int)c;
            }
        }
        int cell, sb;
        cellOf(p.x, &cell, &sb);
        p.cell = cell;
        p.sub = sb;
    }

    // ------------------------------------------------------------ phases
    // dsmcFreeStreamInflowPatch::controlParcelsBeforeMove
    void inflow() {
        const double sqrtPi = std::sqrt(PI);
        std::vector<Parcel> added;
        int e = 0;
        for (int side = 0; side < 6; ++side) {
            const int a = side / 2;
            const int b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
            const double sgnOut = (side & 1) ? 1.0 : -1.0;
            for (long long f = 0; f < sideOff[side + 1] - sideOff[side]; ++f) {
                const long long bf = sideOff[side] + f;
                const dsmc_patch& pt = spec.patches[bfPatch[bf]];
                if (!pt.inflow) continue;
                const long long ib = f % n[b], ic = f / n[b];
                long long cc[3];
                cc[a] = (side & 1) ? n[a] - 1 : 0;
                cc[b] = ib;
                cc[c] = ic;
                const int cell = (int)(cc[0] + (long long)n[0] * (cc[1] + (long long)n[1] * cc[2]));
                const double fA = bfArea[bf];
                for (int m = 0; m < spec.n_species; ++m) {
                    const double nd = pt.inflow_number_density[m];
                    if (!(nd > 0)) continue;
                    const Species& s = sp[m];
                    const double cmp = std::sqrt(2.0 * kB * pt.inflow_t_tra / s.m);
                    const double sCos = (pt.inflow_velocity[a] * (-sgnOut)) / cmp;
                    double& A = inflowAcc[bf * spec.n_species + m];
                    A += (fA * nd * spec.delta_t * cmp *
                          (std::exp(-sCos * sCos) + sqrtPi * sCos * (1 + std::erf(sCos)))) /
                         (2.0 * sqrtPi * spec.n_equivalent_particles);
                    Rng r(spec.seed, (uint32_t)bf, (uint32_t)step, TAG_INFLOW | ((uint32_t)m << 8));
                    int nI = std::max((int)A, 0);
                    if ((A - nI) > r.u01()) nI++;
                    A -= nI;
                    const double coeffA = sCos + std::sqrt(sCos * sCos + 2.0);
                    const double coeffB = 0.5 * (1.0 + sCos * (sCos - std::sqrt(sCos * sCos + 2.0)));
                    double scaling = 3.0;
                    if (sCos < -3) scaling = std::fabs(sCos) + 1;
                    for (int i = 0; i < nI; ++i) {
                        // every parcel has its own stream (face, step, species, parcel)
                        Rng r(spec.seed, (uint32_t)bf, (uint32_t)step,
                              TAG_INFLOW | ((uint32_t)m << 8) | ((uint32_t)(i + 1) << 11));
                        Parcel p{};
                        p.x[a] = (side & 1) ? hi[a] : lo[a];
                        p.x[b] = std::fma(r.u01(), cellW(b, ib), nodeX(b, ib));
                        p.x[c] = std::fma(r.u01(), cellW(c, ic), nodeX(c, ic));
                        double uNormal = 0;
                        if (std::fabs(pt.inflow_velocity[a]) > VSMALL) {
                            int it = 0;
                            for (;;) {
                                const double uth = scaling * (2.0 * r.u01() - 1);
                                uNormal = uth + sCos;
                                double Pr;
                                if (uNormal < 0.0) Pr = -1;
                                else Pr = 2.0 * uNormal / coeffA * std::exp(coeffB - uth * uth);
                                if (!(Pr < r.u01())) break;
                                if (++it >= MAX_REJECTION) { e = 1; break; }
                            }
                        } else {
                            uNormal = std::sqrt(-std::log(r.u01()));
                        }
                        double g1, g2;
                        r.gauss2(&g1, &g2);
                        const double sc = std::sqrt(kB * pt.inflow_t_tra / s.m);
                        p.U[a] = cmp * uNormal * (-sgnOut);
                        p.U[b] = sc * g1 + pt.inflow_velocity[b];
                        p.U[c] = sc * g2 + pt.inflow_velocity[c];
                        p.erot = eqRot(r, pt.inflow_t_rot, s.rotDof, &e);
                        p.vib = eqVib(r, pt.inflow_t_vib, s);
                        p.type = m;
                        p.cell = cell;
                        p.fresh = 1;
                        if (!faceFlux.empty()) {
                            // dsmcCloud::addNewParcel (dsmcCloud.C:425-437)
                            const int c3[3] = {(int)cc[0], (int)cc[1], (int)cc[2]};
                            faceAdd(faceIndex(a, (side & 1) ? n[a] : 0, c3), m, -1.0);
                        }
                        added.push_back(p);
                    }
                }
            }
        }
        for (Parcel& p : added) p.id = nextId++;
        // a divided case: every domain counts every face (the face remainders
        // and the ids are those of the undivided case) and keeps its own
        if (domAxis >= 0)
            added.erase(std::remove_if(added.begin(), added.end(), [&](const Parcel& p) { return !owned(p.cell); }),
                        added.end());
        insertedLast = (long long)added.size();
        P.insert(P.end(), added.begin(), added.end());
        if (e) err = 1;
    }

    void move() {
        long long hits = 0;
        int e = 0;
        const long long N = (long long)P.size();
#pragma omp parallel for schedule(static) reduction(+ : hits) reduction(| : e) num_threads(nThreads)
        for (long long i = 0; i < N; ++i) {
            int ee = 0;
            long long h = 0;
            moveParcel(P[i], &ee, &h);
            hits += h;
            e |= ee;
        }
        wallHitsLast = hits;
        if (e) err = 1;
    }

    // buildCellOccupancy: parcels grouped by cell, ordered by id inside a cell.
    // Parallel counting sort: cell counts with atomics, a prefix over cells,
    // slots taken with atomics (in any order), then every cell's parcels
    // sorted by id, which makes the result independent of the slot order.
    void sort() {
        const long long N = (long long)P.size();
        long long del = 0;
        std::fill(cellCount.begin(), cellCount.end(), 0);
        int* cnt = cellCount.data();
#pragma omp parallel for schedule(static) reduction(+ : del) num_threads(nThreads)
        for (long long i = 0; i < N; ++i) {
            const int c = P[i].cell;
            if (c < 0) { ++del; continue; }
#pragma omp atomic
            cnt[c]++;
        }
        deletedLast = del;
        long long s = 0;
        for (long long c = 0; c < C; ++c) { cellStart[c] = (int)s; s += cellCount[c]; }
        // the other buffer keeps its capacity from step to step, with room
        // for the next steps' inflow, so neither the sort nor the inflow's
        // append reallocates (or zero-fills) the parcel array every step
        std::vector<Parcel>& out = Pbuf;
        if (out.capacity() < (size_t)s) out.reserve((size_t)s + (size_t)s / 8 + 65536);
        out.resize((size_t)s);
        std::vector<int> cur(cellStart.begin(), cellStart.end());
        int* cp = cur.data();
#pragma omp parallel for schedule(static) num_threads(nThreads)
        for (long long i = 0; i < N; ++i) {
            const int c = P[i].cell;
            if (c < 0) continue;
            int q;
#pragma omp atomic capture
            q = cp[c]++;
            out[q] = P[i];
        }
#pragma omp parallel for schedule(dynamic, 4096) num_threads(nThreads)
        for (long long c = 0; c < C; ++c) {
            std::sort(out.begin() + cellStart[c], out.begin() + cellStart[c] + cellCount[c],
                      [](const Parcel& x, const Parcel& y) { return x.id < y.id; });
        }
        P.swap(out);
    }

    // VariableHardSphere::sigmaTcR
    double sigmaTcR(const Parcel& p, const Parcel& q) const {
        const Species& a = sp[p.type];
        const Species& b = sp[q.type];
        const double dPQ = 0.5 * (a.d + b.d);
        const double omegaPQ = 0.5 * (a.omega + b.omega);
        const double dU[3] = {p.U[0] - q.U[0], p.U[1] - q.U[1], p.U[2] - q.U[2]};
        const double cR = std::sqrt(dU[0] * dU[0] + dU[1] * dU[1] + dU[2] * dU[2]);
        if (cR < VSMALL) return 0.0;
        const double mR = a.m * b.m / (a.m + b.m);
        const double sigmaT = PI * dPQ * dPQ *
                              std::pow(2.0 * kB * spec.tref / (mR * cR * cR), omegaPQ - 0.5) /
                              std::exp(std::lgamma(2.5 - omegaPQ));
        return sigmaT * cR;
    }

    // LarsenBorgnakkeVariableHardSphere::redistribute (electronic part skipped)
    void redistribute(Parcel& p, double& Et, double omegaPQ, Rng& r, int* e) {
        const Species& s = sp[p.type];
        if (s.nVib > 0) {
            const double EcP = Et + p.vib * kB * s.thetaV;
            const int iMax = (int)(EcP / (kB * s.thetaV));
            if (iMax > 0) {
                p.vib = postVib(r, p.vib, iMax, s, omegaPQ, EcP, e);
                Et = EcP - p.vib * kB * s.thetaV;
            }
        }
        if (s.rotDof > 0) {
            const double pre = p.erot;
            if (1.0 / spec.zrot > r.u01()) {
                const double EcP = Et + pre;
                const double ChiB = 2.5 - omegaPQ;
                const double ratio = postRot(r, s.rotDof, ChiB, e);
                p.erot = ratio * EcP;
                Et = EcP - p.erot;
            }
        }
    }

    // VariableHardSphere::postCollisionVelocities
    // VariableHardSphere::postCollisionVelocities (VariableHardSphere.C:191-228),
    // or for the soft-sphere models VariableSoftSphere::postCollisionVelocities
    // (VariableSoftSphere.C:191-233, Bird eq. 2.22) with the pre-collision
    // relative velocity scaled to the post-exchange speed cR.
    void scatter(Parcel& p, Parcel& q, double cR, Rng& r) {
        const double mP = sp[p.type].m, mQ = sp[q.type].m;
        double Ucm[3];
        for (int a = 0; a < 3; ++a) Ucm[a] = (mP * p.U[a] + mQ * q.U[a]) / (mP + mQ);
        double pr[3];
        const int cm = spec.binary_collision_model;
        if (cm == DSMC_COLL_VSS || cm == DSMC_COLL_LB_VSS) {
            const double alpha = 0.5 * (sp[p.type].alpha + sp[q.type].alpha);
            const double cosT = 2.0 * std::pow(r.u01(), 1.0 / alpha) - 1.0;
            const double sinT = std::sqrt(1.0 - cosT * cosT);
            const double phi = 2.0 * PI * r.u01();
            double c[3], cpre2 = 0;
            for (int a = 0; a < 3; ++a) { c[a] = p.U[a] - q.U[a]; cpre2 += c[a] * c[a]; }
            const double cpre = std::sqrt(cpre2);
            const double k = cpre > 0.0 ? cR / cpre : 0.0;
            for (int a = 0; a < 3; ++a) c[a] *= k;
            const double D = std::sqrt(c[1] * c[1] + c[2] * c[2]);
            const double sph = std::sin(phi), cph = std::cos(phi);
            if (D > 1e-12 * cR) {
                pr[0] = cosT * c[0] + sinT * sph * D;
                pr[1] = cosT * c[1] + sinT * (cR * c[2] * cph - c[0] * c[1] * sph) / D;
                pr[2] = cosT * c[2] - sinT * (cR * c[1] * cph + c[0] * c[2] * sph) / D;
            } else {
                pr[0] = cosT * c[0];
                pr[1] = cR * sinT * cph;
                pr[2] = cR * sinT * sph;
            }
        } else {
            const double cosT = 2.0 * r.u01() - 1.0;
            const double sinT = std::sqrt(1.0 - cosT * cosT);
            const double phi = 2.0 * PI * r.u01();
            pr[0] = cR * cosT;
            pr[1] = cR * sinT * std::cos(phi);
            pr[2] = cR * sinT * std::sin(phi);
        }
        for (int a = 0; a < 3; ++a) {
            p.U[a] = Ucm[a] + pr[a] * mQ / (mP + mQ);
            q.U[a] = Ucm[a] - pr[a] * mP / (mP + mQ);
        }
    }

    // noTimeCounter::collide for one cell
    void collideCell(long long c, long long* nColl, long long* nCand, int* e) {
        const int nC = cellCount[c];
        if (nC <= 1) return;
        Parcel* cp = &P[cellStart[c]];
        Rng r(spec.seed, (uint32_t)c, (uint32_t)step, TAG_COLLIDE);
        std::vector<int> subs[8];
        for (int i = 0; i < nC; ++i) subs[cp[i].sub].push_back(i);
        const double smax0 = sigmaTcRMax[c];
        const double sel = remainder[c] + 0.5 * nC * (nC - 1) * spec.n_equivalent_particles * smax0 *
                                              spec.delta_t / cellVolume(c);
        const long long nCandidates = (long long)sel;
        remainder[c] = sel - nCandidates;
        *nCand += nCandidates;
        double* A = &acc[c * nAcc];
        for (long long k = 0; k < nCandidates; ++k) {
            const int iP = r.label(0, nC - 1, e);
            int iQ = -1;
            const std::vector<int>& sl = subs[cp[iP].sub];
            const int nSC = (int)sl.size();
            int it = 0;
            if (nSC > 1) {
                do { iQ = sl[r.label(0, nSC - 1, e)]; } while (iP == iQ && ++it < MAX_REJECTION);
            } else {
                do { iQ = r.label(0, nC - 1, e); } while (iP == iQ && ++it < MAX_REJECTION);
            }
            if (it >= MAX_REJECTION) { *e = 1; continue; }
            Parcel& p = cp[iP];
            Parcel& q = cp[iQ];
            const double s = sigmaTcR(p, q);
            if (s > sigmaTcRMax[c]) sigmaTcRMax[c] = s;
            if ((s / smax0) > r.u01()) {
                const Species& a = sp[p.type];
                const Species& b = sp[q.type];
                double cR;
                if (spec.binary_collision_model == DSMC_COLL_LB_VHS ||
                    spec.binary_collision_model == DSMC_COLL_LB_VSS) {
                    const double mR = a.m * b.m / (a.m + b.m);
                    double cr2 = 0;
                    for (int d = 0; d < 3; ++d) cr2 += (p.U[d] - q.U[d]) * (p.U[d] - q.U[d]);
                    double Et = 0.5 * mR * cr2;
                    const double omegaPQ = 0.5 * (a.omega + b.omega);
                    redistribute(p, Et, omegaPQ, r, e);
                    redistribute(q, Et, omegaPQ, r, e);
                    cR = std::sqrt(2.0 * Et / mR);
                } else {
                    double cr2 = 0;
                    for (int d = 0; d < 3; ++d) cr2 += (p.U[d] - q.U[d]) * (p.U[d] - q.U[d]);
                    cR = std::sqrt(cr2);
                }
                scatter(p, q, cR, r);
                A[ACC_COLLSEP] += std::sqrt((p.x[0] - q.x[0]) * (p.x[0] - q.x[0]) +
                                            (p.x[1] - q.x[1]) * (p.x[1] - q.x[1]) +
                                            (p.x[2] - q.x[2]) * (p.x[2] - q.x[2]));
                A[ACC_NCOLLS] += 1.0;
                ++*nColl;
            }
        }
    }

    // simplifiedBernoulliTrials::collide for one cell
    // (simplifiedBernoulliTrials.C:88-190): nC - 1 trials in list order
    void bernoulliCell(long long c, long long* nColl, long long* nCand, int* e) {
        const int nC = cellCount[c];
        if (nC <= 1) return;
        Parcel* cp = &P[cellStart[c]];
        Rng r(spec.seed, (uint32_t)c, (uint32_t)step, TAG_COLLIDE);
        const double prob1 = spec.n_equivalent_particles * spec.delta_t / cellVolume(c);
        double* A = &acc[c * nAcc];
        for (int ip = 0; ip < nC - 1; ++ip) {
            const int k = nC - 1 - ip;
            const int iq = ip + r.label(1, k, e);
            Parcel& p = cp[ip];
            Parcel& q = cp[iq];
            const double s = sigmaTcR(p, q);
            ++*nCand;
            if (k * prob1 * s > r.u01()) {
                const Species& a = sp[p.type];
                const Species& b = sp[q.type];
                double cr2 = 0;
                for (int d = 0; d < 3; ++d) cr2 += (p.U[d] - q.U[d]) * (p.U[d] - q.U[d]);
                double cR;
                if (spec.binary_collision_model == DSMC_COLL_LB_VHS ||
                    spec.binary_collision_model == DSMC_COLL_LB_VSS) {
                    const double mR = a.m * b.m / (a.m + b.m);
                    double Et = 0.5 * mR * cr2;
                    const double omegaPQ = 0.5 * (a.omega + b.omega);
                    redistribute(p, Et, omegaPQ, r, e);
                    redistribute(q, Et, omegaPQ, r, e);
                    cR = std::sqrt(2.0 * Et / mR);
                } else {
                    cR = std::sqrt(cr2);
                }
                scatter(p, q, cR, r);
                A[ACC_COLLSEP] += std::sqrt((p.x[0] - q.x[0]) * (p.x[0] - q.x[0]) +
                                            (p.x[1] - q.x[1]) * (p.x[1] - q.x[1]) +
                                            (p.x[2] - q.x[2]) * (p.x[2] - q.x[2]));
                A[ACC_NCOLLS] += 1.0;
                ++*nColl;
            }
        }
    }

    void collide() {
        long long nColl = 0, nCand = 0;
        int e = 0;
        const bool sbt = spec.partner_selection_model == DSMC_SEL_SBT;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : nColl, nCand) reduction(| : e) num_threads(nThreads)
        for (long long c = 0; c < C; ++c) {
            int ee = 0;
            if (sbt) bernoulliCell(c, &nColl, &nCand, &ee);
            else collideCell(c, &nColl, &nCand, &ee);
            e |= ee;
        }
        collLast = nColl;
        candLast = nCand;
        collTot += nColl;
        candTot += nCand;
        if (e) err = 1;
    }

    // dsmcVolFields::calculateField sample loop (dsmcVolFields.C:1115-1239)
    void sample() {
        const int ns = spec.n_species;
#pragma omp parallel for schedule(dynamic, 4096) num_threads(nThreads)
        for (long long c = 0; c < C; ++c) {
            double* A = &acc[c * nAcc];
            for (int i = cellStart[c]; i < cellStart[c] + cellCount[c]; ++i) {
                const Parcel& p = P[i];
                const Species& s = sp[p.type];
                const double mp = s.m;
                const double linearKE = mp * (p.U[0] * p.U[0] + p.U[1] * p.U[1] + p.U[2] * p.U[2]);
                A[ACC_N] += 1.0;
                A[ACC_M] += mp;
                A[ACC_MOMX] += mp * p.U[0];
                A[ACC_MOMY] += mp * p.U[1];
                A[ACC_MOMZ] += mp * p.U[2];
                A[ACC_MCC] += linearKE;
                A[ACC_EROT] += p.erot;
                A[ACC_ZETAROT] += s.rotDof;
                double* S = A + ACC_COMMON + SACC_PER_SPECIES * p.type;
                S[SACC_N] += 1.0;
                S[SACC_MCC] += linearKE;
                if (s.nVib) S[SACC_EVIB] += p.vib * kB * s.thetaV;
                if (!mom.empty()) {
                    double* Mo = &mom[c * 12];
                    const double u = p.U[0], v = p.U[1], w = p.U[2];
                    const double E = p.erot + (s.nVib ? p.vib * kB * s.thetaV : 0.0);
                    Mo[0] += mp * u * u;
                    Mo[1] += mp * u * v;
                    Mo[2] += mp * u * w;
                    Mo[3] += mp * v * v;
                    Mo[4] += mp * v * w;
                    Mo[5] += mp * w * w;
                    Mo[6] += linearKE * u;
                    Mo[7] += linearKE * v;
                    Mo[8] += linearKE * w;
                    Mo[9] += E * u;
                    Mo[10] += E * v;
                    Mo[11] += E * w;
                }
            }
        }
        (void)ns;
        sampleSteps++;
    }

    // ------------------------------------------------ spatial decomposition
    bool owned(long long c) const {
        if (domAxis < 0) return true;
        const long long ix[3] = {c % n[0], (c / n[0]) % n[1], c / ((long long)n[0] * n[1])};
        return ix[domAxis] >= domLo && ix[domAxis] < domHi;
    }

    void setDomain(int axis, int lo, int hi) {
        domAxis = axis;
        domLo = lo;
        domHi = hi;
        P.erase(std::remove_if(P.begin(), P.end(), [&](const Parcel& p) { return p.cell >= 0 && !owned(p.cell); }),
                P.end());
        sort();
    }

    // inflow and move; a parcel whose move ends in another domain's cell is
    // packed as a migrant (record words, then the cell word) and leaves
    long long stepBegin() {
        inflow();
        move();
        migOut.clear();
        long long m = 0;
        for (Parcel& p : P) {
            if (p.cell < 0 || owned(p.cell)) continue;
            uint32_t w[17];
            std::memcpy(w, p.x, 24);
            std::memcpy(w + 6, p.U, 24);
            std::memcpy(w + 12, &p.erot, 8);
            w[14] = p.id;
            w[15] = (uint32_t)p.type | ((uint32_t)p.vib << 8);
            w[16] = ((uint32_t)p.cell << 3) | (uint32_t)p.sub;
            migOut.insert(migOut.end(), w, w + 17);
            p.cell = -1;
            ++m;
        }
        migLast = m;
        return m;
    }

    void addMigrants(const uint32_t* w, long long n) {
        for (long long k = 0; k < n; ++k, w += 17) {
            Parcel p{};
            std::memcpy(p.x, w, 24);
            std::memcpy(p.U, w + 6, 24);
            std::memcpy(&p.erot, w + 12, 8);
            p.id = w[14];
            p.type = (int)(w[15] & 0xFFu);
            p.vib = (int)(w[15] >> 8);
            p.cell = (int)((w[16] & 0x7FFFFFFFu) >> 3);
            p.sub = (int)(w[16] & 7u);
            p.fresh = 0;
            if (p.cell >= C || !owned(p.cell)) { err = 1; continue; }
            P.push_back(p);
        }
    }

    // sort, collisions, sampling (the migrants sent are not deletions)
    void stepEnd() {
        sort();
        deletedLast -= migLast;
        collide();
        sample();
        step++;
    }

    void runPhases(unsigned ph) {
        if (ph & DSMC_PHASE_INFLOW) inflow();
        if (ph & DSMC_PHASE_MOVE) move();
        if (ph & DSMC_PHASE_SORT) sort();
        if (ph & DSMC_PHASE_COLLIDE) collide();
        if (ph & DSMC_PHASE_SAMPLE) sample();
        step++;
    }

    // dsmcMeshFill::setInitialConfiguration
    void initialise() {
        P.clear();
        int e = 0;
        const int ns = spec.n_species;
        std::vector<int> counts(C * ns, 0);
        for (long long c = 0; c < C; ++c) {
            if (solid[c]) continue;
            Rng r(spec.seed, (uint32_t)c, 0, TAG_INIT_CELL);
            for (int tet = 0; tet < 12; ++tet) {
                for (int m = 0; m < ns; ++m) {
                    const double nd = spec.init_number_density[m];
                    if (!(nd > 0)) continue;
                    const double req = nd * (cellVolume(c) / 12.0) / spec.n_equivalent_particles;
                    int k = (int)req;
                    if ((req - k) > r.u01()) k++;
                    counts[c * ns + m] += k;
                }
            }
        }
        uint32_t id = 0;
        for (long long c = 0; c < C; ++c) {
            const long long i0 = c % n[0], j0 = (c / n[0]) % n[1], k0 = c / ((long long)n[0] * n[1]);
            const double cl[3] = {nodeX(0, i0), nodeX(1, j0), nodeX(2, k0)};
            const double cw[3] = {cellW(0, i0), cellW(1, j0), cellW(2, k0)};
            for (int m = 0; m < ns; ++m) {
                const Species& s = sp[m];
                for (int q = 0; q < counts[c * ns + m]; ++q) {
                    Parcel p{};
                    p.id = id++;
                    Rng r(spec.seed, p.id, 0, TAG_INIT_PARTICLE);
                    for (int a = 0; a < 3; ++a) p.x[a] = std::fma(r.u01(), cw[a], cl[a]);
                    double g[4];
                    r.gauss2(&g[0], &g[1]);
                    r.gauss2(&g[2], &g[3]);
                    for (int a = 0; a < 3; ++a) {
                        const double T = spec.init_t_tra_xyz[a] > 0 ? spec.init_t_tra_xyz[a] : spec.init_t_tra;
                        p.U[a] = std::sqrt(kB * T / s.m) * g[a] + spec.init_velocity[a];
                    }
                    p.erot = eqRot(r, spec.init_t_rot, s.rotDof, &e);
                    p.vib = eqVib(r, spec.init_t_vib, s);
                    p.type = m;
                    int cell, sb;
                    cellOf(p.x, &cell, &sb);
                    p.cell = cell;
                    p.sub = sb;
                    p.fresh = 0;
                    P.push_back(p);
                }
            }
        }
        nextId = id;
        int most = 0;
        for (int m = 1; m < ns; ++m)
            if (spec.init_number_density[m] > spec.init_number_density[most]) most = m;
        const double smax = PI * sp[most].d * sp[most].d *
                            std::sqrt(2.0 * kB * spec.init_t_tra / sp[most].m);
        std::fill(sigmaTcRMax.begin(), sigmaTcRMax.end(), smax);
        sort();
        if (e) err = 1;
    }

    // dsmcVolFields output-time fields (dsmcVolFields.C:1242-1290, 1365-1876)
    bool field(const std::string& name, double* out) const {
        const double nT = (double)sampleSteps;
        const double FN = spec.n_equivalent_particles;
        for (long long c = 0; c < C; ++c) {
            const double* A = &acc[c * nAcc];
            const double V = cellVolume(c);
            double v = 0.0;
            const double N = A[ACC_N];
            double rhoN = 0, rhoM = 0, Ux = 0, Uy = 0, Uz = 0, Ttra = 0;
            if (N > 1e-3 && nT > 0) {
                rhoN = N * FN / (nT * V);
                rhoM = A[ACC_M] * FN / (nT * V);
                Ux = A[ACC_MOMX] / A[ACC_M];
                Uy = A[ACC_MOMY] / A[ACC_M];
                Uz = A[ACC_MOMZ] / A[ACC_M];
                const double keMean = 0.5 * A[ACC_MCC] * FN / (V * nT);
                Ttra = 2.0 / (3.0 * kB * rhoN) * (keMean - 0.5 * rhoM * (Ux * Ux + Uy * Uy + Uz * Uz));
            }
            const double zetaRotTot = N > SMALL ? A[ACC_ZETAROT] / N : 0.0;
            const double Trot = A[ACC_ZETAROT] > SMALL ? 2.0 * A[ACC_EROT] / (kB * A[ACC_ZETAROT]) : 0.0;
            double Tvib = 0, zetaVib = 0, molRhoN = 0;
            for (int s = 0; s < spec.n_species; ++s) {
                const double* S = A + ACC_COMMON + SACC_PER_SPECIES * s;
                if (!sp[s].nVib) continue;
                double zeta = 0, Ts = 0;
                if (S[SACC_EVIB] > VSMALL && S[SACC_N] > SMALL) {
                    const double iMean = S[SACC_EVIB] / (kB * sp[s].thetaV * S[SACC_N]);
                    if (iMean > SMALL) {
                        const double lf = std::log(1.0 + 1.0 / iMean);
                        Ts = sp[s].thetaV / lf;
                        zeta = 2.0 * iMean * lf;
                    }
                }
                if (zeta > SMALL) {
                    molRhoN += S[SACC_N] * FN;
                    Tvib += S[SACC_N] * FN * Ts;
                    zetaVib += S[SACC_N] * FN * zeta;
                }
            }
            if (molRhoN > SMALL) { Tvib /= molRhoN; zetaVib /= molRhoN; }
            const double Tov = (3.0 * Ttra + zetaRotTot * Trot + zetaVib * Tvib) / (3.0 + zetaRotTot + zetaVib);
            if (name == "rhoN") v = rhoN;
            else if (name == "rhoM") v = rhoM;
            else if (name == "Ux") v = Ux;
            else if (name == "Uy") v = Uy;
            else if (name == "Uz") v = Uz;
            else if (name == "Ttra") v = Ttra;
            else if (name == "p") v = rhoN * kB * Ttra;
            else if (name == "Trot") v = Trot;
            else if (name == "Tvib") v = Tvib;
            else if (name == "Tov") v = Tov;
            else if (name == "dsmcNMean") v = (N > 1e-3 && nT > 0) ? N / nT : 0.001;
            else if (name == "nColls") v = A[ACC_NCOLLS];
            else if (name == "measuredCollisionRate")
                v = (N > SMALL && nT > 0) ? A[ACC_NCOLLS] * FN / (N * FN * spec.delta_t) : 0.0;
            else if (name.rfind("pressureTensor_", 0) == 0 || name.rfind("shearStressTensor_", 0) == 0 ||
                     name.rfind("heatFluxVector_", 0) == 0) {
                // dsmcVolFields.C:1511-1607
                if (mom.empty()) return false;
                const double* Mo = &mom[c * 12];
                double E = A[ACC_EROT];
                for (int q = 0; q < spec.n_species; ++q) E += A[ACC_COMMON + SACC_PER_SPECIES * q + SACC_EVIB];
                const double U[3] = {Ux, Uy, Uz};
                const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
                double P[6] = {0, 0, 0, 0, 0, 0};
                if (N > SMALL && nT > 0)
                    for (int k = 0; k < 6; ++k) P[k] = rhoN / N * (Mo[k] - A[ACC_M] * U[ia[k]] * U[ib[k]]);
                static const char* comp[6] = {"xx", "xy", "xz", "yy", "yz", "zz"};
                v = 0.0;
                for (int k = 0; k < 6; ++k) {
                    if (name == std::string("pressureTensor_") + comp[k]) v = P[k];
                    if (name == std::string("shearStressTensor_") + comp[k])
                        v = -P[k] + (ia[k] == ib[k] ? (P[0] + P[3] + P[5]) / 3.0 : 0.0);
                }
                const int row[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
                for (int i = 0; i < 3; ++i) {
                    if (name != std::string("heatFluxVector_") + "xyz"[i]) continue;
                    v = (N > SMALL && nT > 0)
                            ? rhoN / N * (0.5 * Mo[6 + i] - 0.5 * A[ACC_MCC] * U[i] + Mo[9 + i] - E * U[i]) -
                                  P[row[i][0]] * U[0] - P[row[i][1]] * U[1] - P[row[i][2]] * U[2]
                            : 0.0;
                }
            }
            else if (name == "Ma" || name == "rhoMError" || name == "UError" || name == "TError" ||
                     name == "pError") {
                // dsmcVolFields.C:1625-1661 and 1859-1873
                double Ma = 0, gamma = 0, particleCv = 0;
                if (N > SMALL && Ttra > SMALL) {
                    double molarCv = 0, molarCp = 0, mMol = 0;
                    for (int s = 0; s < spec.n_species; ++s) {
                        const double Xs = A[ACC_COMMON + SACC_PER_SPECIES * s + SACC_N] / N;
                        mMol += Xs * sp[s].m;
                        molarCv += Xs * (3.0 + sp[s].rotDof);
                        molarCp += Xs * (5.0 + sp[s].rotDof);
                    }
                    particleCv = molarCv / NAvo;
                    gamma = molarCp / molarCv;
                    Ma = std::sqrt(Ux * Ux + Uy * Uy + Uz * Uz) / std::sqrt(gamma * kB / mMol * Ttra);
                }
                const double nMean = (N > 1e-3 && nT > 0) ? N / nT : 0.001;
                const double deno = std::sqrt(nMean * nT);
                const bool ok = nMean > SMALL && Ma > SMALL && gamma > SMALL && particleCv > SMALL;
                if (name == "Ma") v = Ma;
                else if (!ok) v = 0.0;
                else if (name == "rhoMError") v = 1.0 / deno;
                else if (name == "UError") v = 1.0 / (deno * Ma * std::sqrt(gamma));
                else if (name == "TError") v = std::sqrt(kB / particleCv) / deno;
                else v = std::sqrt(gamma) / deno;
            }
            else if (name == "meanCollisionRate" || name == "mfp") {
                double mfp = 0, mcr = 0;
                if (Ttra > 1.0 && nT > 0) {
                    for (int s = 0; s < spec.n_species; ++s) {
                        double smfp = 0, smcr = 0;
                        for (int q = 0; q < spec.n_species; ++q) {
                            const double* Sq = A + ACC_COMMON + SACC_PER_SPECIES * q;
                            const double dPQ = 0.5 * (sp[s].d + sp[q].d);
                            const double oPQ = 0.5 * (sp[s].omega + sp[q].omega);
                            const double mr = sp[s].m / sp[q].m;
                            if (Sq[SACC_N] > SMALL) {
                                const double nQ = Sq[SACC_N] * FN / (V * nT);
                                const double red = sp[s].m * sp[q].m / (sp[s].m + sp[q].m);
                                smfp += PI * dPQ * dPQ * nQ * std::pow(spec.mfp_tref / Ttra, oPQ - 0.5) * std::sqrt(1.0 + mr);
                                smcr += 2.0 * std::sqrt(PI) * dPQ * dPQ * nQ * std::pow(Ttra / spec.mfp_tref, 1.0 - oPQ) *
                                        std::sqrt(2.0 * kB * spec.mfp_tref / red);
                            }
                        }
                        if (smfp > SMALL) smfp = 1.0 / smfp;
                        const double* Ss = A + ACC_COMMON + SACC_PER_SPECIES * s;
                        const double rhoNi = Ss[SACC_N] * FN;
                        mfp += smfp * rhoNi / (N * FN);
                        mcr += smcr * rhoNi / (N * FN);
                    }
                    if (mfp < SMALL) mfp = GREAT;
                } else {
                    mfp = GREAT;
                }
                v = (name == "mfp") ? mfp : mcr;
            } else return false;
            out[c] = v;
        }
        return true;
    }
};

thread_local std::string g_err;

}  // namespace

extern "C" {

struct oracle_handle { Oracle o; };

void oracle_philox(const unsigned ctr[4], const unsigned key[2], unsigned out[4]) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    uint32_t k[2] = {key[0], key[1]};
    uint32_t o[4];
    Philox::gen(c, k, o);
    for (int i = 0; i < 4; ++i) out[i] = o[i];
}

double oracle_u01_from(unsigned lo, unsigned hi) { return u01_from(lo, hi); }

const char* oracle_last_error(void) { return g_err.c_str(); }

oracle_handle* oracle_create(const dsmc_case_spec* spec, int n_threads) {
    oracle_handle* h = new oracle_handle();
    h->o.nThreads = n_threads > 0 ? n_threads : 1;
    if (!h->o.setup(spec)) {
        g_err = h->o.msg;
        delete h;
        return nullptr;
    }
    return h;
}

void oracle_destroy(oracle_handle* h) { delete h; }

void oracle_set_threads(oracle_handle* h, int n_threads) { h->o.nThreads = n_threads > 0 ? n_threads : 1; }

// The step counter that keys the random streams (to continue a state that
// another implementation advanced to that step).
void oracle_set_step(oracle_handle* h, long long step) { h->o.step = step; }

// Restarts the time averages (every sampling sum and the sample count), as
// the library's dsmc_reset_sampling does.
void oracle_reset_sampling(oracle_handle* h) {
    std::fill(h->o.acc.begin(), h->o.acc.end(), 0.0);
    std::fill(h->o.mom.begin(), h->o.mom.end(), 0.0);
    h->o.sampleSteps = 0;
}

int oracle_initialise(oracle_handle* h) {
    h->o.initialise();
    return h->o.err ? DSMC_ERR_DEVICE : DSMC_OK;
}

int oracle_run_phases(oracle_handle* h, unsigned phases) {
    h->o.runPhases(phases);
    return h->o.err ? DSMC_ERR_DEVICE : DSMC_OK;
}

int oracle_set_domain(oracle_handle* h, int axis, int lo, int hi) {
    if (axis < -1 || axis > 2 || (axis >= 0 && !(0 <= lo && lo < hi && hi <= h->o.n[axis]))) return DSMC_ERR_INVALID;
    h->o.setDomain(axis, lo, hi);
    return DSMC_OK;
}

long long oracle_step_begin(oracle_handle* h) { return h->o.stepBegin(); }

int oracle_get_migrants(oracle_handle* h, void* dst, long long n) {
    if (n < 0 || n * 17 > (long long)h->o.migOut.size()) return DSMC_ERR_INVALID;
    std::memcpy(dst, h->o.migOut.data(), (size_t)n * 68);
    return DSMC_OK;
}

int oracle_add_migrants(oracle_handle* h, const void* src, long long n) {
    h->o.addMigrants(static_cast<const uint32_t*>(src), n);
    return h->o.err ? DSMC_ERR_DEVICE : DSMC_OK;
}

int oracle_step_end(oracle_handle* h) {
    h->o.stepEnd();
    return h->o.err ? DSMC_ERR_DEVICE : DSMC_OK;
}

int oracle_evolve(oracle_handle* h, long long n) {
    for (long long i = 0; i < n; ++i) h->o.runPhases(DSMC_PHASE_ALL);
    return h->o.err ? DSMC_ERR_DEVICE : DSMC_OK;
}

int oracle_set_particles(oracle_handle* h, long long n, const double* pos, const double* U,
                         const double* erot, const int* vib, const int* species,
                         const unsigned* id, int fresh) {
    Oracle& o = h->o;
    o.P.resize(n);
    uint32_t mx = 0;
    for (long long i = 0; i < n; ++i) {
        Parcel& p = o.P[i];
        for (int a = 0; a < 3; ++a) { p.x[a] = pos[3 * i + a]; p.U[a] = U[3 * i + a]; }
        p.erot = erot ? erot[i] : 0.0;
        p.vib = vib ? vib[i] : 0;
        p.type = species ? species[i] : 0;
        p.id = id[i];
        p.fresh = fresh;
        mx = std::max(mx, p.id + 1);
        int cell, sb;
        o.cellOf(p.x, &cell, &sb);
        p.cell = cell;
        p.sub = sb;
    }
    o.nextId = mx;
    if (o.domAxis >= 0)
        o.P.erase(std::remove_if(o.P.begin(), o.P.end(), [&](const Parcel& p) { return !o.owned(p.cell); }),
                  o.P.end());
    o.sort();
    return DSMC_OK;
}

long long oracle_n_particles(oracle_handle* h) { return (long long)h->o.P.size(); }

int oracle_get_particles(oracle_handle* h, double* pos, double* U, double* erot, int* vib,
                         int* species, unsigned* id, int* cell) {
    const Oracle& o = h->o;
    for (size_t i = 0; i < o.P.size(); ++i) {
        const Parcel& p = o.P[i];
        for (int a = 0; a < 3; ++a) {
            if (pos) pos[3 * i + a] = p.x[a];
            if (U) U[3 * i + a] = p.U[a];
        }
        if (erot) erot[i] = p.erot;
        if (vib) vib[i] = p.vib;
        if (species) species[i] = p.type;
        if (id) id[i] = p.id;
        if (cell) cell[i] = p.cell;
    }
    return DSMC_OK;
}

int oracle_get_cell_array(oracle_handle* h, const char* name, void* out) {
    const Oracle& o = h->o;
    const std::string nm(name);
    if (nm == "count") std::memcpy(out, o.cellCount.data(), sizeof(int) * o.C);
    else if (nm == "start") std::memcpy(out, o.cellStart.data(), sizeof(int) * o.C);
    else if (nm == "sigmaTcRMax") std::memcpy(out, o.sigmaTcRMax.data(), sizeof(double) * o.C);
    else if (nm == "collisionSelectionRemainder") std::memcpy(out, o.remainder.data(), sizeof(double) * o.C);
    else if (nm == "accumulators") std::memcpy(out, o.acc.data(), sizeof(double) * o.C * o.nAcc);
    else if (nm == "inflowAccumulator") std::memcpy(out, o.inflowAcc.data(), sizeof(double) * o.inflowAcc.size());
    else return DSMC_ERR_INVALID;
    return DSMC_OK;
}

int oracle_set_cell_array(oracle_handle* h, const char* name, const void* in) {
    Oracle& o = h->o;
    const std::string nm(name);
    if (nm == "sigmaTcRMax") std::memcpy(o.sigmaTcRMax.data(), in, sizeof(double) * o.C);
    else if (nm == "collisionSelectionRemainder") std::memcpy(o.remainder.data(), in, sizeof(double) * o.C);
    else if (nm == "inflowAccumulator") std::memcpy(o.inflowAcc.data(), in, sizeof(double) * o.inflowAcc.size());
    else return DSMC_ERR_INVALID;
    return DSMC_OK;
}

int oracle_n_accumulators(oracle_handle* h) { return h->o.nAcc; }

int oracle_get_field(oracle_handle* h, const char* name, double* out) {
    return h->o.field(name, out) ? DSMC_OK : DSMC_ERR_INVALID;
}

int oracle_get_wall(oracle_handle* h, double* out) {
    const Oracle& o = h->o;
    for (long long f = 0; f < o.nBFaces; ++f) {
        const WallAcc& w = o.wall[f];
        const double v[14] = {w.rhoN, w.rhoM, w.linearKE, w.mcc, w.mom[0], w.mom[1], w.mom[2],
                              w.erot, w.zetaRot, w.evib, w.q, w.fD[0], w.fD[1], w.fD[2]};
        std::memcpy(out + 14 * f, v, sizeof(v));
    }
    return DSMC_OK;
}

long long oracle_n_boundary_faces(oracle_handle* h) { return h->o.nBFaces; }

int oracle_set_face_tracking(oracle_handle* h, int on) {
    Oracle& o = h->o;
    const long long nx = o.n[0], ny = o.n[1], nz = o.n[2];
    o.faceOff[0] = 0;
    o.faceOff[1] = (nx + 1) * ny * nz;
    o.faceOff[2] = o.faceOff[1] + nx * (ny + 1) * nz;
    o.nFacesAll = o.faceOff[2] + nx * ny * (nz + 1);
    if (on) o.faceFlux.assign(2 * (size_t)o.spec.n_species * o.nFacesAll, 0.0);
    else o.faceFlux.clear();
    return DSMC_OK;
}

// [2][nSpecies][nFaces]: parcelIdFlux then massIdFlux
int oracle_get_face_flux(oracle_handle* h, double* out) {
    const Oracle& o = h->o;
    if (o.faceFlux.empty()) return DSMC_ERR_INVALID;
    std::memcpy(out, o.faceFlux.data(), sizeof(double) * o.faceFlux.size());
    return DSMC_OK;
}

int oracle_info(oracle_handle* h, dsmc_info_t* out) {
    const Oracle& o = h->o;
    std::memset(out, 0, sizeof(*out));
    out->n_particles = (long long)o.P.size();
    out->step = o.step;
    const double FN = o.spec.n_equivalent_particles;
    for (const Parcel& p : o.P) {
        const Species& s = o.sp[p.type];
        out->linear_ke += 0.5 * s.m * (p.U[0] * p.U[0] + p.U[1] * p.U[1] + p.U[2] * p.U[2]);
        out->rotational_e += p.erot;
        out->vibrational_e += s.nVib ? p.vib * kB * s.thetaV : 0.0;
        for (int a = 0; a < 3; ++a) out->momentum[a] += s.m * p.U[a];
    }
    out->linear_ke *= FN;
    out->rotational_e *= FN;
    out->vibrational_e *= FN;
    for (int a = 0; a < 3; ++a) out->momentum[a] *= FN;
    out->collisions_last_step = o.collLast;
    out->candidates_last_step = o.candLast;
    out->collisions_total = o.collTot;
    out->candidates_total = o.candTot;
    out->wall_hits_last_step = o.wallHitsLast;
    out->inserted_last_step = o.insertedLast;
    out->deleted_last_step = o.deletedLast;
    out->sample_steps = o.sampleSteps;
    return DSMC_OK;
}

}  // extern "C"
