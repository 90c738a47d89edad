// dsmc_move.cu -- move, occupancy sort, inflow and mesh-fill kernels.
//
// move       dsmcParcel::move (src/lagrangian/dsmc/parcels/dsmcParcel.C:38-148)
//            with the patch models it dispatches to (dsmcParcel.C:174-204):
//            dsmcSpecularWallPatch.C:47-62, dsmcDiffuseWallPatch.C:67-138,
//            dsmcDeletionPatch.C:140-172, particleTemplates.C:1511-1570 and the
//            wall measurements of dsmcPatchBoundary.C:263-482.
// sort       dsmcCloud::buildCellOccupancy (dsmcCloud.C:63-74) as a counting
//            sort: the per-cell histogram is fused into the move (warp-
//            aggregated atomics), an exclusive scan gives the cell starts and
//            a scatter moves the structure-of-arrays state into cell order.
// inflow     dsmcFreeStreamInflowPatch::controlParcelsBeforeMove
//            (dsmcFreeStreamInflowPatch.C:91-364).
// mesh fill  dsmcMeshFill::setInitialConfiguration (dsmcMeshFill.C:68-238).
//
// Compiled with -fmad=false: every FP64 operation is written out as the CPU
// replay performs it, so positions, cells and crossings agree bit for bit.

#include "dsmc_kernels.h"

namespace dsmc {

namespace {

constexpr int MAX_STREAM_THREADS = 512;   // largest CTA of the parcel-streaming kernels

__device__ __forceinline__ double eq_rot(Rng& r, double T, double dof, unsigned* err) {
    if (dof < SMALL) return 0.0;
    if (dof < 2.0 + SMALL && dof > 2.0 - SMALL) return -log(r.u01()) * kB * T;
    const double a = 0.5 * dof - 1;
    for (int it = 0; it < MAX_REJECTION; ++it) {
        const double ratio = 10 * r.u01();
        const double Pr = pow(ratio / a, a) * exp(a - ratio);
        if (!(Pr < r.u01())) return ratio * kB * T;
    }
    *err |= ERRB_REJECTION;
    return 0.0;
}

__device__ __forceinline__ int eq_vib(Rng& r, double T, const SpeciesDev& s) {
    if (s.nVib == 0) return 0;
    return (int)(-log(r.u01()) * T / s.thetaV);
}

// dsmcPatchBoundary::measurePropertiesBeforeControl / AfterControl
// (dsmcPatchBoundary.C:263-482).  The before call keeps its flux terms in
// pre[] (10 sums, then energy and momentum); the after call adds before and
// after together, one atomic per sum.
constexpr int WPRE = W_EVIB + 1 + 4;
__device__ void wall_measure(const CaseDev& cs, double* wall, long long bf, int axis, double sgn,
                             const double U[3], double erot, int vib, const SpeciesDev& s,
                             bool after, double* pre) {
    const int ax1 = (axis == 0) ? 1 : 0;
    const int ax2 = (axis == 2) ? 1 : 2;
    const double fA = cs.bfArea ? cs.bfArea[bf] : cs.dx[ax1] * cs.dx[ax2];
    // 1 / (dt fA): one division per case on a uniform mesh
    const double invDtFa = cs.bfArea ? 1.0 / (cs.dt * fA) : cs.invDtFa[axis];
    const double Un = U[axis] * sgn;
    double Ut[3] = {U[0], U[1], U[2]};
    Ut[axis] = U[axis] - Un * sgn;
    double w = fabs(Un) * fA * cs.dt;
    w = 1.0 / (w < SMALL ? SMALL : w);
    const double UU = U[0] * U[0] + U[1] * U[1] + U[2] * U[2];
    const double evib = s.nVib ? vib * s.kThetaV : 0.0;
    const double t[W_EVIB + 1] = {w, s.m * w, 0.5 * s.m * UU * w, s.m * UU * w, s.m * Ut[0] * w,
                                  s.m * Ut[1] * w, s.m * Ut[2] * w, erot * w, s.rotDof * w, evib * w};
    const double E = 0.5 * s.m * UU + erot + evib;
    if (!after) {
        for (int k = 0; k <= W_EVIB; ++k) pre[k] = t[k];
        pre[W_EVIB + 1] = E;
        for (int a = 0; a < 3; ++a) pre[W_EVIB + 2 + a] = s.m * U[a];
        return;
    }
    double* W = wall + bf * W_N;
#pragma unroll
    for (int k = 0; k <= W_EVIB; ++k) atomicAdd(W + k, pre[k] + t[k]);
    atomicAdd(W + W_Q, cs.FN * (pre[W_EVIB + 1] - E) * invDtFa);
    atomicAdd(W + W_FDX, cs.FN * (pre[W_EVIB + 2] - s.m * U[0]) * invDtFa);
    atomicAdd(W + W_FDY, cs.FN * (pre[W_EVIB + 3] - s.m * U[1]) * invDtFa);
    atomicAdd(W + W_FDZ, cs.FN * (pre[W_EVIB + 4] - s.m * U[2]) * invDtFa);
}

// The after call of a specular reflection: |U.n|, the tangential velocity and
// the energies are unchanged, so every flux term equals its before term, the
// heat flux is zero and the force is along the normal only.
__device__ void wall_measure_specular(const CaseDev& cs, double* wall, long long bf, int axis, const double U[3],
                                      const SpeciesDev& s, const double* pre) {
    double* W = wall + bf * W_N;
#pragma unroll
    for (int k = 0; k <= W_EVIB; ++k) atomicAdd(W + k, pre[k] + pre[k]);
    const double invDtFa = cs.bfArea ? 1.0 / (cs.dt * cs.bfArea[bf]) : cs.invDtFa[axis];
    atomicAdd(W + W_FDX + axis, cs.FN * (pre[W_EVIB + 2 + axis] - s.m * U[axis]) * invDtFa);
}

// dsmcDiffuseWallPatch::performDiffuseReflection for a face of outward normal
// sgn * e_axis, with dsmcPatchBoundary::calculateWallUnitVectors.
__device__ void diffuse_reflect(const CaseDev& cs, Rng& r, int axis, double sgn, const PatchDev& pt,
                                const SpeciesDev& s, double U[3], double* erot, int* vib,
                                unsigned* err) {
    double nw[3] = {0.0, 0.0, 0.0};
    nw[axis] = sgn;
    double Un = U[0] * nw[0] + U[1] * nw[1] + U[2] * nw[2];
    double Ut[3];
    for (int a = 0; a < 3; ++a) Ut[a] = U[a] - Un * nw[a];
    double magUt = sqrt(Ut[0] * Ut[0] + Ut[1] * Ut[1] + Ut[2] * Ut[2]);
    int it = 0;
    while (magUt < SMALL) {
        if (++it > MAX_REJECTION) {
            *err |= ERRB_REJECTION;
            Ut[0] = Ut[1] = Ut[2] = 0.0;
            Ut[(axis + 1) % 3] = 1.0;
            magUt = 1.0;
            break;
        }
        for (int a = 0; a < 3; ++a) U[a] = U[a] * (0.8 + 0.2 * r.u01());
        Un = U[0] * nw[0] + U[1] * nw[1] + U[2] * nw[2];
        for (int a = 0; a < 3; ++a) Ut[a] = U[a] - Un * nw[a];
        magUt = sqrt(Ut[0] * Ut[0] + Ut[1] * Ut[1] + Ut[2] * Ut[2]);
    }
    double t1[3], t2[3];
    for (int a = 0; a < 3; ++a) t1[a] = Ut[a] / magUt;
    t2[0] = nw[1] * t1[2] - nw[2] * t1[1];
    t2[1] = nw[2] * t1[0] - nw[0] * t1[2];
    t2[2] = nw[0] * t1[1] - nw[1] * t1[0];
    const double T = pt.Twall;
    double g1, g2;
    r.gauss2(&g1, &g2);
    double om = 1 - r.u01();
    om = om < VSMALL ? VSMALL : om;
    const double un = sqrt(-2.0 * log(om));
    const double sc = sqrt(kB * T / s.m);
    for (int a = 0; a < 3; ++a) U[a] = sc * (g1 * t1[a] + g2 * t2[a] - un * nw[a]);
    *erot = eq_rot(r, T, s.rotDof, err);
    *vib = eq_vib(r, T, s);
    for (int a = 0; a < 3; ++a) U[a] += pt.Uwall[a];
}

// ---------------------------------------------------------------- face tracker
// dsmcFaceTracker::trackFaceTransition (dsmcFaceTracker.C:124-190): every face
// a parcel crosses gets sign(U . S) and sign(U . S) m, with S the face's
// area vector (+axis for a face between two cells, outward for a boundary
// face), and a cyclic crossing gets +1 on the face it leaves through.

// node p along axis a, and the width of cell i along it
__device__ __forceinline__ double node_x(const CaseDev& cs, int a, int p) {
    return cs.half[a] ? cs.half[a][2 * p] : cs.lo[a] + p * cs.dx[a];
}
__device__ __forceinline__ double cell_w(const CaseDev& cs, int a, int i) {
    return cs.half[a] ? cs.half[a][2 * i + 2] - cs.half[a][2 * i] : cs.dx[a];
}

// face on axis a at plane index p, the other two cell indices from cell[]
__device__ __forceinline__ long long face_index(const CaseDev& cs, int a, int p, const int* cell) {
    const long long nx = cs.n[0], ny = cs.n[1];
    if (a == 0) return cs.faceOff[0] + p + (nx + 1) * (cell[1] + ny * cell[2]);
    if (a == 1) return cs.faceOff[1] + cell[0] + nx * (p + (ny + 1) * cell[2]);
    return cs.faceOff[2] + cell[0] + nx * (cell[1] + ny * p);
}

__device__ __forceinline__ void face_add(const CaseDev& cs, long long f, int sp, double sgn) {
    atomicAdd(cs.faceFlux + (long long)sp * cs.nFacesAll + f, sgn);
    atomicAdd(cs.faceFlux + ((long long)cs.nSpecies + sp) * cs.nFacesAll + f, sgn * cs.sp[sp].m);
}

// the cell faces crossed on the straight path from x (in cell sc) to cell te,
// in the order of their crossing times (ties: lower axis first)
__device__ void track_internal(const CaseDev& cs, const double* x, const double* U, const int* sc, const int* te,
                               int sp) {
    int cur[3] = {sc[0], sc[1], sc[2]};
    int left[3], dir[3];
    double t[3] = {0.0, 0.0, 0.0};
    for (int a = 0; a < 3; ++a) {
        const int d = te[a] - sc[a];
        left[a] = d < 0 ? -d : d;
        dir[a] = d > 0 ? 1 : -1;
        if (left[a]) {
            const int p = d > 0 ? sc[a] + 1 : sc[a];
            t[a] = (node_x(cs, a, p) - x[a]) / U[a];
        }
    }
    while (left[0] + left[1] + left[2] > 0) {
        int a = -1;
        for (int b = 0; b < 3; ++b)
            if (left[b] && (a < 0 || t[b] < t[a])) a = b;
        const int p = dir[a] > 0 ? cur[a] + 1 : cur[a];
        face_add(cs, face_index(cs, a, p, cur), sp, dir[a] > 0 ? 1.0 : -1.0);
        cur[a] += dir[a];
        if (--left[a]) {
            const int pn = dir[a] > 0 ? cur[a] + 1 : cur[a];
            t[a] = (node_x(cs, a, pn) - x[a]) / U[a];
        }
    }
}

// Full Cartesian tracking of one parcel: the same steps as the CPU replay.
// Returns the new cell word (CELLW_DELETED when removed).
__device__ uint32_t move_slow(const CaseDev& cs, const Parcels& s, long long i, uint32_t step,
                              uint32_t w, const int* bfPatch, double* wall, unsigned* err,
                              unsigned long long* hits) {
    Rec p = ld_rec(s.r + i);
    double x[3] = {p.x, p.y, p.z};
    double U[3] = {p.ux, p.uy, p.uz};
    const uint32_t pid = p.id;
    const int type = sv_species(p.sv);
    const SpeciesDev& sp = cs.sp[type];
    double erot = p.erot;
    int vib = sv_vib(p.sv);
    Rng r(cs, pid, step, TAG_MOVE);
    double tr = cs.dt;
    if (w & CELLW_FRESH) {
        const double sf = r.u01();
        tr = (1.0 - sf) * cs.dt;
    }
    int sc[3];
    {
        const uint32_t c = cellw_cell(w);
        cell_coords(cs, c, &sc[0], &sc[1], &sc[2]);
    }
    uint32_t result = 0;
    bool done = false;
    for (int it = 0; !done; ++it) {
        if (!(tr > ROOTVSMALL)) break;
        if (it >= cs.maxCrossings) { *err |= ERRB_CROSSINGS; break; }
        // tracking velocity: none along an empty (reduced-D) axis, whose
        // coordinate is held at the mesh centre; U keeps all three components
        double V[3] = {U[0], U[1], U[2]};
        if (cs.anyEmpty)
            for (int a = 0; a < 3; ++a)
                if (cs.emptyAx[a]) { x[a] = cs.mid[a]; V[a] = 0.0; }
        double ex[3];
        int c2[3], ci[3];
        bool out = false;
        for (int a = 0; a < 3; ++a) {
            ex[a] = fma(V[a], tr, x[a]);
            c2[a] = floor2_coord_fast(cs, ex[a], a);
            ci[a] = c2[a] >> 1;
            if (ci[a] < 0 || ci[a] >= cs.n[a]) out = true;
        }
        bool obst = false;
        for (int o = 0; o < cs.nObst && !obst; ++o) {
            bool ov = true;
            for (int a = 0; a < 3; ++a) {
                const int mn = min(sc[a], ci[a]);
                const int mx = max(sc[a], ci[a]);
                if (mx < cs.obLoI[o][a] || mn > cs.obHiI[o][a] - 1) ov = false;
            }
            obst = ov;
        }
        if (!out && !obst) {
            if (cs.faceFlux) track_internal(cs, x, V, sc, ci, type);
            x[0] = ex[0]; x[1] = ex[1]; x[2] = ex[2];
            result = ((uint32_t)(ci[0] + cs.n[0] * (ci[1] + cs.n[1] * ci[2])) << 3) |
                     (uint32_t)((c2[0] & 1) | ((c2[1] & 1) << 1) | ((c2[2] & 1) << 2));
            done = true;
            break;
        }
        double tHit = GREAT * GREAT;
        int hitKind = -1, hitSide = -1;
        for (int a = 0; a < 3; ++a) {
            if (ci[a] < 0) {
                double t = (cs.lo[a] - x[a]) / V[a];
                if (!(t >= 0.0)) t = 0.0;
                if (t > tr) t = tr;
                if (t < tHit) { tHit = t; hitKind = 0; hitSide = 2 * a; }
            } else if (ci[a] >= cs.n[a]) {
                double t = (cs.hi[a] - x[a]) / V[a];
                if (!(t >= 0.0)) t = 0.0;
                if (t > tr) t = tr;
                if (t < tHit) { tHit = t; hitKind = 0; hitSide = 2 * a + 1; }
            }
        }
        for (int o = 0; o < cs.nObst; ++o) {
            double tin = -GREAT * GREAT, tout = GREAT * GREAT;
            int ax = -1;
            bool miss = false;
            for (int a = 0; a < 3; ++a) {
                if (V[a] != 0.0) {
                    const double t1 = (cs.obLo[o][a] - x[a]) / V[a];
                    const double t2 = (cs.obHi[o][a] - x[a]) / V[a];
                    const double ta = dmin(t1, t2), tb = dmax(t1, t2);
                    if (ta > tin) { tin = ta; ax = a; }
                    if (tb < tout) tout = tb;
                } else if (x[a] < cs.obLo[o][a] || x[a] > cs.obHi[o][a]) {
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
            if (cs.faceFlux) track_internal(cs, x, V, sc, ci, type);
            x[0] = ex[0]; x[1] = ex[1]; x[2] = ex[2];
            result = ((uint32_t)(ci[0] + cs.n[0] * (ci[1] + cs.n[1] * ci[2])) << 3) |
                     (uint32_t)((c2[0] & 1) | ((c2[1] & 1) << 1) | ((c2[2] & 1) << 2));
            done = true;
            break;
        }
        const int axis = hitSide / 2;
        double plane;
        if (hitKind == 0) plane = (hitSide & 1) ? cs.hi[axis] : cs.lo[axis];
        else plane = (hitSide & 1) ? cs.obHi[hitKind - 1][axis] : cs.obLo[hitKind - 1][axis];
        double x0[3] = {x[0], x[1], x[2]};
        for (int a = 0; a < 3; ++a) x[a] = (a == axis) ? plane : fma(V[a], tHit, x[a]);
        // the fluid cell at the hit point and the plane index of the face hit
        int hitCell[3], facePlane;
        for (int a = 0; a < 3; ++a) {
            const int cc = floor2_coord_fast(cs, x[a], a) >> 1;
            hitCell[a] = min(max(cc, 0), cs.n[a] - 1);
        }
        if (hitKind == 0) {
            facePlane = (hitSide & 1) ? cs.n[axis] : 0;
            hitCell[axis] = (hitSide & 1) ? cs.n[axis] - 1 : 0;
        } else {
            facePlane = (hitSide & 1) ? cs.obHiI[hitKind - 1][axis] : cs.obLoI[hitKind - 1][axis];
            hitCell[axis] = (hitSide & 1) ? facePlane : facePlane - 1;
        }
        if (cs.faceFlux) track_internal(cs, x0, V, sc, hitCell, type);
        tr = tr - tHit;
        const int b = (axis == 0) ? 1 : 0;
        const int c = (axis == 2) ? 1 : 2;
        long long bf;
        double sgn;
        if (hitKind == 0) {
            int ib = floor2_coord_fast(cs, x[b], b) >> 1;
            int ic = floor2_coord_fast(cs, x[c], c) >> 1;
            ib = min(max(ib, 0), cs.n[b] - 1);
            ic = min(max(ic, 0), cs.n[c] - 1);
            bf = cs.sideOff[hitSide] + ib + (long long)cs.n[b] * ic;
            sgn = (hitSide & 1) ? 1.0 : -1.0;
        } else {
            const int o = hitKind - 1;
            const int nb = cs.obHiI[o][b] - cs.obLoI[o][b];
            const int nc = cs.obHiI[o][c] - cs.obLoI[o][c];
            int ib = (floor2_coord_fast(cs, x[b], b) >> 1) - cs.obLoI[o][b];
            int ic = (floor2_coord_fast(cs, x[c], c) >> 1) - cs.obLoI[o][c];
            ib = min(max(ib, 0), nb - 1);
            ic = min(max(ic, 0), nc - 1);
            bf = cs.obstOff[o][hitSide] + ib + (long long)nb * ic;
            sgn = (hitSide & 1) ? -1.0 : 1.0;
        }
        const int patch = bfPatch[bf];
        if (patch < 0 || patch >= cs.nPatches) { *err |= ERRB_PATCH; result = CELLW_DELETED; done = true; break; }
        const PatchDev& pt = cs.patch[patch];
        if (pt.type == DSMC_PATCH_SYMMETRY) {
            U[axis] = -U[axis];
        } else if (pt.type == DSMC_PATCH_CYCLIC) {
            if (hitKind == 0) x[axis] = (hitSide & 1) ? cs.lo[axis] : cs.hi[axis];
            // hitCyclicPatch moves the parcel onto the receiving face, and
            // the tracker adds +1 to that face's coupled face: the exit face
            if (cs.faceFlux && hitKind == 0) face_add(cs, face_index(cs, axis, facePlane, hitCell), type, 1.0);
        } else if (pt.model == DSMC_BC_SPECULAR || pt.model == DSMC_BC_DIFFUSE) {
            double pre[WPRE];
            if (cs.hasWallMeasure)
                wall_measure(cs, wall, bf, axis, sgn, U, erot, vib, sp, false, pre);
            if (pt.model == DSMC_BC_SPECULAR) {
                if (U[axis] * sgn > 0.0) U[axis] = -U[axis];
            } else {
                diffuse_reflect(cs, r, axis, sgn, pt, sp, U, &erot, &vib, err);
            }
            if (cs.hasWallMeasure) {
                if (pt.model == DSMC_BC_SPECULAR) wall_measure_specular(cs, wall, bf, axis, U, sp, pre);
                else wall_measure(cs, wall, bf, axis, sgn, U, erot, vib, sp, true, pre);
            }
            atomicAdd(hits, 1ull);
        } else {
            // deletion (and any patch without a model) removes the parcel
            if (cs.faceFlux)
                face_add(cs, face_index(cs, axis, facePlane, hitCell), type, U[axis] * sgn > 0.0 ? 1.0 : -1.0);
            result = CELLW_DELETED;
            done = true;
            break;
        }
        // a reflected parcel is counted on the face with its new velocity
        if (cs.faceFlux && pt.type != DSMC_PATCH_CYCLIC)
            face_add(cs, face_index(cs, axis, facePlane, hitCell), type, U[axis] * sgn > 0.0 ? 1.0 : -1.0);
        for (int a = 0; a < 3; ++a) {
            int cc = floor2_coord_fast(cs, x[a], a) >> 1;
            sc[a] = min(max(cc, 0), cs.n[a] - 1);
        }
    }
    if (!done) {
        int ci[3], sb = 0;
        for (int a = 0; a < 3; ++a) {
            int c2 = floor2_coord_fast(cs, x[a], a);
            c2 = min(max(c2, 0), 2 * cs.n[a] - 1);
            ci[a] = c2 >> 1;
            sb |= (c2 & 1) << a;
        }
        result = ((uint32_t)(ci[0] + cs.n[0] * (ci[1] + cs.n[1] * ci[2])) << 3) | (uint32_t)sb;
    }
    if (vib < 0 || vib > SV_MAX_VIB) { *err |= ERRB_BOUNDS; vib = 0; }
    p.x = x[0]; p.y = x[1]; p.z = x[2];
    p.ux = U[0]; p.uy = U[1]; p.uz = U[2];
    p.erot = erot;
    p.sv = make_sv(type, vib);
    st_rec(s.r + i, p);
    return result;
}

// Warp-aggregated histogram increment for a key (or -1 for none).
__device__ __forceinline__ void agg_count(int* count, int key) {
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, key);
    const int leader = __ffs(peers) - 1;
    if (key >= 0 && (int)lane_id() == leader) atomicAdd(&count[key], __popc(peers));
}

// Three transposing rounds over lanes d, d/2, d/4 apart: 8 values per lane
// become 1, lane l keeping value 4 b(d) + 2 b(d/2) + b(d/4) of its partners'
// sums (b(x): whether bit x of the lane is set).
__device__ __forceinline__ void butterfly8(long long* v, unsigned lane, int d) {
    {
        const bool up = (lane & (unsigned)d) != 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const long long send = up ? v[k] : v[4 + k];
            const long long keep = up ? v[4 + k] : v[k];
            v[k] = keep + __shfl_xor_sync(0xFFFFFFFFu, send, d);
        }
    }
    {
        const int e = d >> 1;
        const bool up = (lane & (unsigned)e) != 0;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const long long send = up ? v[k] : v[2 + k];
            const long long keep = up ? v[2 + k] : v[k];
            v[k] = keep + __shfl_xor_sync(0xFFFFFFFFu, send, e);
        }
    }
    {
        const int e = d >> 2;
        const bool up = (lane & (unsigned)e) != 0;
        const long long send = up ? v[0] : v[1];
        const long long keep = up ? v[1] : v[0];
        v[0] = keep + __shfl_xor_sync(0xFFFFFFFFu, send, e);
    }
}

// One parcel's contribution to the dsmcVolFields sample sums
// (dsmcVolFields.C:1115-1239) per lane, valid when skey = cell * 8 + species
// is not negative: summed over the warp's runs of equal keys and added to the
// per-cell fixed-point sums with 64-bit integer atomics, so the result does
// not depend on the order of parcels, warps or atomics.
__device__ __forceinline__ void sample_contrib(long long* sfix, long long C, int skey, double ux, double uy,
                                               double uz, double er, int vb, unsigned* err) {
    long long f[8] = {0, 0, 0, 0, 0, 0, 0, 0};   // SACC values, then a zero pad
    if (skey >= 0) {
        f[SACC_N] = 1;
        f[SACC_UX] = fixp(ux, F_U, err);
        f[SACC_UY] = fixp(uy, F_U, err);
        f[SACC_UZ] = fixp(uz, F_U, err);
        // |U|^2 in fixed point from the fixed-point components, on the
        // integer pipe: (u 2^28)^2 >> 42 = u^2 2^14
        unsigned long long uu = 0;
#pragma unroll
        for (int a = SACC_UX; a <= SACC_UZ; ++a) {
            const unsigned long long m = (unsigned long long)(f[a] < 0 ? -f[a] : f[a]);
            const unsigned long long hi = __umul64hi(m, m);
            if (hi >> 46) *err |= ERRB_BOUNDS;
            uu += (hi << (64 - (2 * F_U - F_UU))) | ((m * m) >> (2 * F_U - F_UU));
        }
        f[SACC_UU] = (long long)uu;
        f[SACC_EROT] = fixp(er, F_E, err);
        f[SACC_VIB] = vb;
    }
    const unsigned lane = lane_id();
    const int prev = __shfl_up_sync(0xFFFFFFFFu, skey, 1);
    const unsigned hm = __ballot_sync(0xFFFFFFFFu, lane == 0 || prev != skey);
    const int nSeg = __popc(hm);
    if (nSeg == 1) {
        // One run (most warps: cells hold tens of parcels): a transposing
        // butterfly, each round sending half of a lane's vector to its
        // partner, leaves lane l with the total of value (l >> 2) & 7.
        long long v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = f[k];
        butterfly8(v, lane, 16);
        v[0] += __shfl_xor_sync(0xFFFFFFFFu, v[0], 2);
        v[0] += __shfl_xor_sync(0xFFFFFFFFu, v[0], 1);
        const int val = (int)(lane >> 2) & 7;
        if ((lane & 3u) == 0 && val < SACC && skey >= 0 && v[0])
            atomicAdd(reinterpret_cast<unsigned long long*>(sfix + (long long)((skey & 7) * SACC + val) * C +
                                                            (skey >> 3)),
                      (unsigned long long)v[0]);
        return;
    }
    if (nSeg == 2) {
        // Two runs, the second from lane b: the first round splits a
        // 16-value vector (run 0's values, then run 1's) across lanes 16
        // apart; lane l ends with value (l >> 1) & 7 of run (l >> 4) & 1.
        const int b = 31 - __clz(hm);
        const bool inB = (int)lane >= b;
        const bool up = (lane & 16u) != 0;
        long long v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            // keep my half's run, send the other run's values
            const long long mine = (up == inB) ? f[k] : 0;
            const long long other = (up == inB) ? 0 : f[k];
            v[k] = mine + __shfl_xor_sync(0xFFFFFFFFu, other, 16);
        }
        butterfly8(v, lane, 8);
        v[0] += __shfl_xor_sync(0xFFFFFFFFu, v[0], 1);
        const int val = (int)(lane >> 1) & 7;
        const int rkey = __shfl_sync(0xFFFFFFFFu, skey, up ? b : 0);
        if ((lane & 1u) == 0 && val < SACC && rkey >= 0 && v[0])
            atomicAdd(reinterpret_cast<unsigned long long*>(sfix + (long long)((rkey & 7) * SACC + val) * C +
                                                            (rkey >> 3)),
                      (unsigned long long)v[0]);
        return;
    }
    const int segStart = 31 - __clz(hm & (0xFFFFFFFFu >> (31 - (int)lane)));
    // the count is the run's length; vibrational levels sum in 32 bits
    f[SACC_N] = (long long)((int)lane - segStart + 1);
    f[SACC_VIB] = seg_sum32((int)f[SACC_VIB], segStart);
#pragma unroll
    for (int k = SACC_UX; k <= SACC_EROT; ++k) f[k] = seg_sum(f[k], segStart);
    const bool tail = lane == 31 || ((hm >> (lane + 1)) & 1u);
    if (tail && skey >= 0) {
        const long long c = skey >> 3;
        const int sp = skey & 7;
#pragma unroll
        for (int k = 0; k < SACC; ++k)
            if (f[k]) atomicAdd(reinterpret_cast<unsigned long long*>(sfix + (long long)(sp * SACC + k) * C + c),
                                (unsigned long long)f[k]);
    }
}

// Interior parcels finish here.  Parcels that are fresh or whose straight
// move leaves the domain or approaches an obstacle are appended to slowList
// and tracked by k_move_slow: on GB300 an FP64 instruction costs the whole
// warp's pipe time, so the ~100-instruction boundary path must not be run by
// the warp of every wall-adjacent cell for its one or two boundary lanes.
// When a sample is pending, the kernel also folds the pre-move state (the
// state after the previous step's collisions, which the reference samples at
// the end of that step) into the per-cell sample sums: it streams the
// velocities anyway, in cell order.
// GEN = false is the instantiation for uniform meshes without reduced-D axes,
// solid boxes or face tracking: their branches are compiled out.
// One iteration of k_move for parcel i (lanes with i >= n take part in the
// warp-collective counts, appends and sample sums without a parcel).  The
// batched persistent kernel runs the same iterations.
template <bool GEN>
__device__ __forceinline__ void move_iter(const CaseDev& cs, const Parcels& s, Counters* ctr, int* slowList,
                                          int* count, long long* sfix, long long i, long long n, uint32_t step,
                                          int doSample, int deferPos, int* migList, long long migCap,
                                          unsigned& err) {
    int key = -1;
    bool slow = false;
    bool migrant = false;
    int skey = -1;
    double sux = 0, suy = 0, suz = 0, ser = 0;
    int svb = 0;
    if (i < n) {
        const uint32_t w = s.cellw[i];
        bool fast = false;
        {
            const bool fresh = (w & CELLW_FRESH) != 0;
            double2* q = reinterpret_cast<double2*>(s.r + i);
            const double2 q0 = q[0], q1 = q[1], q2 = q[2];
            double x = q0.x, y = q0.y, z = q1.x;
            const double ux = q1.y, uy = q2.x, uz = q2.y;
            // tracking velocity (zero along an empty axis, whose coordinate
            // is held at the mesh centre: dsmcParcel.C:73-84)
            double tux = ux, tuy = uy, tuz = uz;
            if (GEN && cs.anyEmpty) {
                if (cs.emptyAx[0]) { x = cs.mid[0]; tux = 0.0; }
                if (cs.emptyAx[1]) { y = cs.mid[1]; tuy = 0.0; }
                if (cs.emptyAx[2]) { z = cs.mid[2]; tuz = 0.0; }
            }
            double tr = cs.dt;
            if (fresh) {
                // a parcel inserted this step moves for (1 - U) dt
                // (dsmcParcel.C:52-59), with the draw of the boundary path
                const uint32_t pid = (uint32_t)__double_as_longlong(q[3].y);
                Rng r(cs, pid, step, TAG_MOVE);
                tr = (1.0 - r.u01()) * cs.dt;
            } else if (doSample) {
                const double2 q3 = q[3];
                const uint32_t sv = (uint32_t)((unsigned long long)__double_as_longlong(q3.y) >> 32);
                skey = (int)(cellw_cell(w) * 8u + (uint32_t)sv_species(sv));
                sux = ux; suy = uy; suz = uz;
                ser = q3.x;
                svb = sv_vib(sv);
            }
            const double ex = fma(tux, tr, x);
            const double ey = fma(tuy, tr, y);
            const double ez = fma(tuz, tr, z);
            const int c2x = GEN ? floor2_coord_fast(cs, ex, 0) : floor2_coord_fast_uniform(cs, ex, 0);
            const int c2y = GEN ? floor2_coord_fast(cs, ey, 1) : floor2_coord_fast_uniform(cs, ey, 1);
            const int c2z = GEN ? floor2_coord_fast(cs, ez, 2) : floor2_coord_fast_uniform(cs, ez, 2);
            const int cx = c2x >> 1, cy = c2y >> 1, cz = c2z >> 1;
            const bool inX = (unsigned)cx < (unsigned)cs.n[0], inY = (unsigned)cy < (unsigned)cs.n[1],
                       inZ = (unsigned)cz < (unsigned)cs.n[2];
            bool inside = inX && inY && inZ;
            // leaving through exactly one side whose every face deletes
            // (dsmcDeletionPatch, no wall measurement): the straight path
            // stays inside the other two slabs, so that side is the one hit
            int delSide = -1;
            if (!inside && (int)inX + (int)inY + (int)inZ == 2) {
                const int a = !inX ? 0 : !inY ? 1 : 2;
                const int c2a = a == 0 ? c2x : a == 1 ? c2y : c2z;
                const int side = 2 * a + (c2a < 0 ? 0 : 1);
                if (cs.sideDeletes[side] && !(GEN && cs.faceFlux)) delSide = side;
            }
            if (GEN && (inside || delSide >= 0) && cs.nObst) {
                // the straight path stays in the box of cells spanned by its
                // end cells: one that misses an obstacle's cells on some axis
                // cannot touch it (a point on a face plane lies in the
                // obstacle's cell there)
                int sx, sy, sz;
                cell_coords(cs, cellw_cell(w), &sx, &sy, &sz);
                for (int o = 0; o < cs.nObst; ++o) {
                    if (max(sx, cx) >= cs.obLoI[o][0] && min(sx, cx) <= cs.obHiI[o][0] - 1 &&
                        max(sy, cy) >= cs.obLoI[o][1] && min(sy, cy) <= cs.obHiI[o][1] - 1 &&
                        max(sz, cz) >= cs.obLoI[o][2] && min(sz, cz) <= cs.obHiI[o][2] - 1) {
                        inside = false;
                        delSide = -1;
                    }
                }
            }
            if (delSide >= 0) {
                s.cellw[i] = CELLW_DELETED;
                fast = true;
            } else if (inside) {
                if (GEN && cs.faceFlux) {
                    int sc[3];
                    cell_coords(cs, cellw_cell(w), &sc[0], &sc[1], &sc[2]);
                    const int te[3] = {cx, cy, cz};
                    const double xs[3] = {x, y, z}, Us[3] = {tux, tuy, tuz};
                    const uint32_t sv = (uint32_t)((unsigned long long)__double_as_longlong(q[3].y) >> 32);
                    track_internal(cs, xs, Us, sc, te, sv_species(sv));
                }
                // with the sort following, the end point of a plain move
                // (x + U dt, no reduced-D axis) is left to the gather, which
                // reads the record anyway and repeats the same fma; bit 31
                // of the cell word says so
                const bool defer = deferPos && !fresh && !(GEN && cs.anyEmpty);
                if (!defer) {
                    q[0] = make_double2(ex, ey);
                    s.r[i].z = ez;
                }
                const uint32_t nw = ((uint32_t)(cx + cs.n[0] * (cy + cs.n[1] * cz)) << 3) |
                                    (uint32_t)((c2x & 1) | ((c2y & 1) << 1) | ((c2z & 1) << 2));
                s.cellw[i] = defer ? (nw | CELLW_MOVE_PENDING) : nw;
                if (GEN && cs.domAxis >= 0) {
                    // a move that ends in another domain's cell: the parcel
                    // leaves as a migrant (a processor patch, Cloud.C:255-466)
                    const int ca = cs.domAxis == 0 ? cx : cs.domAxis == 1 ? cy : cz;
                    migrant = ca < cs.domLo || ca >= cs.domHi;
                }
                key = migrant ? -1 : (int)(nw >> 3);
                fast = true;
            }
        }
        slow = !fast;
    }
    agg_count(count, key);
    // warp-aggregated append of the deferred parcels
    const unsigned m = __ballot_sync(0xFFFFFFFFu, slow);
    if (m) {
        const unsigned lane = lane_id();
        unsigned long long base0 = 0;
        if (lane == (unsigned)(__ffs(m) - 1)) base0 = atomicAdd(&ctr->nSlow, (unsigned long long)__popc(m));
        base0 = __shfl_sync(0xFFFFFFFFu, base0, __ffs(m) - 1);
        if (slow) slowList[base0 + __popc(m & ((1u << lane) - 1u))] = (int)i;
    }
    if (GEN && cs.domAxis >= 0) {
        // warp-aggregated append of the migrants
        const unsigned mm = __ballot_sync(0xFFFFFFFFu, migrant);
        if (mm) {
            const unsigned lane = lane_id();
            unsigned long long b0 = 0;
            if (lane == (unsigned)(__ffs(mm) - 1)) b0 = atomicAdd(&ctr->nMig, (unsigned long long)__popc(mm));
            b0 = __shfl_sync(0xFFFFFFFFu, b0, __ffs(mm) - 1);
            const long long q = (long long)b0 + __popc(mm & ((1u << lane) - 1u));
            if (migrant) {
                if (q < migCap) migList[q] = (int)i;
                else err |= ERRB_MIGRANT_CAP;
            }
        }
    }
    if (doSample) sample_contrib(sfix, cs.C, skey, sux, suy, suz, ser, svb, &err);
}

// range: MOVE_ALL the parcels [0, nMoved); MOVE_KEPT the parcels of the last
// step [0, n), which needs nothing of this step's inflow; MOVE_INSERTED the
// inserted ones [n, nMoved), none of which is sampled.
enum { MOVE_ALL = 0, MOVE_KEPT, MOVE_INSERTED };

template <bool GEN>
__global__ void __launch_bounds__(MAX_STREAM_THREADS)
k_move(CaseDev cs, Parcels s, Counters* ctr, int* slowList, int* count, long long* sfix, int deferPos,
       int* migList, long long migCap, int range) {
    long long lo = 0, hi = range == MOVE_KEPT ? ctr->n : ctr->nMoved;
    const uint32_t step = (uint32_t)ctr->step;
    int doSample = ctr->pendingSample;
    if (range == MOVE_INSERTED) {
        lo = ctr->n;
        doSample = 0;
    }
    unsigned err = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = lo + (long long)blockIdx.x * blockDim.x; base < hi; base += stride)
        move_iter<GEN>(cs, s, ctr, slowList, count, sfix, base + threadIdx.x, hi, step, doSample, deferPos, migList,
                       migCap, err);
    if (err) atomicOr(&ctr->err, err);
}

// A pending sample of the current state when no move follows.
__global__ void __launch_bounds__(MAX_STREAM_THREADS)
k_sample_pass(CaseDev cs, Parcels s, Counters* ctr, long long* sfix) {
    if (!ctr->pendingSample) return;
    const long long n = ctr->n;
    unsigned err = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += stride) {
        const long long i = base + threadIdx.x;
        int skey = -1;
        double ux = 0, uy = 0, uz = 0, er = 0;
        int vb = 0;
        if (i < n) {
            const uint32_t w = s.cellw[i];
            if (w != CELLW_DELETED && !(w & CELLW_FRESH)) {
                const Rec p = ldg_rec(s.r + i);
                skey = (int)(cellw_cell(w) * 8u + (uint32_t)sv_species(p.sv));
                ux = p.ux; uy = p.uy; uz = p.uz;
                er = p.erot;
                vb = sv_vib(p.sv);
            }
        }
        sample_contrib(sfix, cs.C, skey, ux, uy, uz, er, vb, &err);
    }
    if (err) atomicOr(&ctr->err, err);
}

// Adds the fixed-point sums of the samples taken so far to the FP64
// accumulators and clears them: every SAMPLES_PER_FLUSH samples and whenever
// the fields are read.  32 samples of a cell of 2^16 parcels at 8 km/s stay
// below 2^62 in every sum (2^41 per velocity component, 2^40 per |U|^2, 2^40
// per rotational energy of 1e-18 J).
constexpr int SAMPLES_PER_FLUSH = 32;

__global__ void k_sample_finalize(CaseDev cs, const Counters* ctr, long long* sfix, double* acc, int force) {
    if (ctr->unflushed == 0 || (!force && ctr->unflushed < SAMPLES_PER_FLUSH)) return;
    const long long total = (long long)cs.nSpecies * SACC * cs.C;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long v = sfix[idx];
        if (!v) continue;
        const int k = (int)((idx / cs.C) % SACC);
        const int F = (k == SACC_UU) ? F_UU : (k == SACC_EROT) ? F_E : F_U;
        acc[idx] += (k == SACC_N || k == SACC_VIB) ? (double)v : unfix(v, F);
        sfix[idx] = 0;
    }
}

__global__ void k_sample_done(Counters* ctr) {
    if (ctr->pendingSample) {
        ctr->sampleSteps += 1;
        ctr->unflushed += 1;
        ctr->pendingSample = 0;
    }
}

__global__ void k_sample_flushed(Counters* ctr, int force) {
    if (force || ctr->unflushed >= SAMPLES_PER_FLUSH) ctr->unflushed = 0;
}

__global__ void k_set_pending(Counters* ctr) { ctr->pendingSample = 1; }

// The boundary path for the parcels k_move deferred, densely packed.
__global__ void __launch_bounds__(MAX_STREAM_THREADS)
k_move_slow(CaseDev cs, Parcels s, Counters* ctr, const int* __restrict__ slowList, const int* __restrict__ bfPatch,
            double* wall, int* count, int* migList, long long migCap) {
    const long long nSlow = (long long)ctr->nSlow;
    const uint32_t step = (uint32_t)ctr->step;
    unsigned err = 0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nSlow;
         k += (long long)gridDim.x * blockDim.x) {
        const long long i = slowList[k];
        const uint32_t w = s.cellw[i];
        const uint32_t nw = move_slow(cs, s, i, step, w, bfPatch, wall, &err, &ctr->wallHits);
        s.cellw[i] = nw;
        if (nw == CELLW_DELETED) continue;
        if (cs.domAxis >= 0 && !cell_owned(cs, nw >> 3)) {
            // the boundary path ended in another domain's cell: a migrant
            const unsigned long long q = atomicAdd(&ctr->nMig, 1ull);
            if ((long long)q < migCap) migList[q] = (int)i;
            else err |= ERRB_MIGRANT_CAP;
            continue;
        }
        atomicAdd(&count[nw >> 3], 1);
    }
    if (err) atomicOr(&ctr->err, err);
}

// The step's migrants, packed for the exchange: the record with its end
// point made (a plain move's is left to the gather otherwise) and the cell
// word; each leaves this cloud (deleted from the sort's point of view).
__global__ void k_pack_migrants(Parcels s, Counters* ctr, const int* __restrict__ migList, uint32_t* out,
                                long long migCap, double dt) {
    const long long nm = min((long long)ctr->nMig, migCap);
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < nm;
         j += (long long)gridDim.x * blockDim.x) {
        const long long i = migList[j];
        Rec p = ldg_rec(s.r + i);
        uint32_t w = s.cellw[i];
        if (w & CELLW_MOVE_PENDING) {
            p.x = fma(p.ux, dt, p.x);
            p.y = fma(p.uy, dt, p.y);
            p.z = fma(p.uz, dt, p.z);
            w &= ~CELLW_MOVE_PENDING;
        }
        const uint32_t* pw = reinterpret_cast<const uint32_t*>(&p);
        uint32_t* o = out + j * MIGRANT_WORDS;
#pragma unroll
        for (int k = 0; k < 16; ++k) o[k] = pw[k];
        o[16] = w;
        s.cellw[i] = CELLW_DELETED;
    }
}

// n migrants from other domains appended at slots base.. and counted in
// their cells; one for a cell this cloud does not own is dropped (error
// bit).
__global__ void k_unpack_migrants(CaseDev cs, Parcels s, Counters* ctr, const uint32_t* __restrict__ src,
                                  long long n, long long base, int* count) {
    unsigned err = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long b0 = (long long)blockIdx.x * blockDim.x; b0 < n; b0 += stride) {
        const long long k = b0 + threadIdx.x;
        int key = -1;
        if (k < n) {
            const uint32_t* q = src + k * MIGRANT_WORDS;
            Rec p;
            uint32_t* pw = reinterpret_cast<uint32_t*>(&p);
#pragma unroll
            for (int t = 0; t < 16; ++t) pw[t] = q[t];
            const uint32_t w = q[16] & ~CELLW_MOVE_PENDING;
            const uint32_t c = cellw_cell(w);
            st_rec(s.r + base + k, p);
            if ((long long)c < cs.C && cell_owned(cs, c)) {
                s.cellw[base + k] = w;
                key = (int)c;
            } else {
                s.cellw[base + k] = CELLW_DELETED;
                err |= ERRB_MIGRANT;
            }
        }
        agg_count(count, key);
    }
    if (err) atomicOr(&ctr->err, err);
}

__global__ void k_migrants_commit(Counters* ctr, long long n) {
    ctr->nMoved += n;
    ctr->migIn += n;
}

__global__ void k_count(Parcels s, long long n, int* count) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += stride) {
        const long long i = base + threadIdx.x;
        int key = -1;
        if (i < n) {
            const uint32_t w = s.cellw[i];
            key = (w == CELLW_DELETED) ? -1 : (int)cellw_cell(w);
        }
        agg_count(count, key);
    }
}

__global__ void k_count_dev(Parcels s, const Counters* ctr, int* count) {
    const long long n = ctr->nMoved;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += stride) {
        const long long i = base + threadIdx.x;
        int key = -1;
        if (i < n) {
            const uint32_t w = s.cellw[i];
            key = (w == CELLW_DELETED) ? -1 : (int)cellw_cell(w);
        }
        agg_count(count, key);
    }
}

// ---------------------------------------------------------------- scan
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ int block_exclusive_scan(int v, int* total) {
    __shared__ int warpSums[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warpSums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int ws = (lane < (int)(blockDim.x >> 5)) ? warpSums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xFFFFFFFFu, ws, o);
            if (lane >= o) ws += y;
        }
        warpSums[lane] = ws;
    }
    __syncthreads();
    const int warpOff = wid ? warpSums[wid - 1] : 0;
    *total = warpSums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warpOff + x - v;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const int* __restrict__ count, long long C, int* blockSums) {
    const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
        if (base + k < C) s += count[base + k];
    int total;
    block_exclusive_scan(s, &total);
    if (threadIdx.x == 0) blockSums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_top(int* blockSums, int nb, int* start, long long C,
                                                           Counters* ctr) {
    int carry = 0;
    for (int b0 = 0; b0 < nb; b0 += SCAN_THREADS) {
        const int b = b0 + threadIdx.x;
        const int v = (b < nb) ? blockSums[b] : 0;
        int total;
        const int ex = block_exclusive_scan(v, &total);
        if (b < nb) blockSums[b] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) {
        start[C] = carry;
        ctr->nKept = carry;
    }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(const int* __restrict__ count, long long C,
                                                            const int* __restrict__ blockSums, int* start) {
    const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = (base + k < C) ? count[base + k] : 0;
        s += v[k];
    }
    int total;
    int ex = block_exclusive_scan(s, &total) + blockSums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < C) start[base + k] = ex;
        ex += v[k];
    }
}

// ---------------------------------------------------------------- scatter
// The counting sort runs in two passes.  k_scatter_index gives every kept
// parcel its slot in cell order (a warp-aggregated atomic per cell present in
// the warp) and writes only the parcel's source index there.  k_gather then
// walks the destination slots in order and pulls each parcel's state from its
// source: every store is coalesced, and the loads of one warp come from a few
// runs of neighbouring source cells.  Storing the 64-byte records from the
// source side instead (each parcel to start[cell] + a rank taken in the move)
// measured 16% slower on the sort and 4% on the move that keeps the ranks;
// grouping them first per block of 2048 parcels (a shared hash of the cells
// present, one slot reservation per block and cell, stores in runs) measured
// 5% slower on the 64^3 heat bath and 40% on a cooler, collision-heavy one.
// The slot of parcel i, whose cell word w is already loaded (CELLW_DELETED
// for lanes that take part in the warp-collective slot reservation without a
// parcel).
__device__ __forceinline__ void scatter_slot(uint32_t w, Counters* ctr, const int* __restrict__ start, int* count,
                                             int2* __restrict__ sortSrc, long long i) {
    const unsigned lane = lane_id();
    const int key = (w == CELLW_DELETED) ? -1 : (int)cellw_cell(w);
    int lo = 0, hi = 0;
    if (key >= 0) {
        lo = __ldg(start + key);
        hi = __ldg(start + key + 1);
    }
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, key);
    const int leader = __ffs(peers) - 1;
    int old = 0;
    if (key >= 0 && (int)lane == leader) old = atomicSub(&count[key], __popc(peers));
    old = __shfl_sync(0xFFFFFFFFu, old, leader);
    if (key >= 0) {
        const int rank = __popc(peers & ((1u << lane) - 1u));
        const long long slot = (long long)lo + old - 1 - rank;
        if (slot < lo || slot >= hi) {
            // histogram and scatter disagree: record, never write out of range
            atomicOr(&ctr->err, ERRB_BOUNDS);
            return;
        }
        sortSrc[slot] = make_int2((int)i, (int)w);
    }
}

// One iteration of the index scatter for parcel i (lanes with i >= n take
// part without a parcel): the persistent batch kernel's form.
__device__ __forceinline__ void scatter_iter(const uint32_t* __restrict__ cellw, Counters* ctr,
                                             const int* __restrict__ start, int* count, int2* __restrict__ sortSrc,
                                             long long i, long long n) {
    scatter_slot(i < n ? __ldg(cellw + i) : CELLW_DELETED, ctr, start, count, sortSrc, i);
}

// Each pass waits on its slot atomic and the start offsets (L2 round trips);
// the cell words of the thread's next two parcels are loaded two passes
// ahead, so the DRAM latency of the stream stays out of that chain (0.40 ->
// 0.32 ms per step on the 83M-parcel channel).
__global__ void __launch_bounds__(MAX_STREAM_THREADS) k_scatter_index(const uint32_t* __restrict__ cellw, Counters* ctr,
                                                       const int* __restrict__ start, int* count,
                                                       int2* __restrict__ sortSrc) {
    const long long n = ctr->nMoved;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t w1 = i0 < n ? __ldg(cellw + i0) : CELLW_DELETED;
    uint32_t w2 = i0 + stride < n ? __ldg(cellw + i0 + stride) : CELLW_DELETED;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += stride) {
        const long long i = base + threadIdx.x;
        const uint32_t w = w1;
        w1 = w2;
        w2 = i + 2 * stride < n ? __ldg(cellw + i + 2 * stride) : CELLW_DELETED;
        scatter_slot(w, ctr, start, count, sortSrc, i);
    }
}

// One destination slot j of k_gather.  dt != 0: a cell word with
// CELLW_MOVE_PENDING marks a parcel whose move ended at x + U dt without being
// stored (k_move with deferPos); the end point is made here with the same
// fma, so it is bit for bit the move's.
__device__ __forceinline__ void gather_slot(const Parcels& src, const Parcels& dst, Counters* ctr,
                                            const int2* __restrict__ sortSrc, long long j, long long nSrc,
                                            double dt) {
    const int2 sk = __ldg(sortSrc + j);
    const long long i = sk.x;
    if (i < 0 || i >= nSrc) {
        atomicOr(&ctr->err, ERRB_BOUNDS);
        return;
    }
    Rec p = ldg_rec(src.r + i);
    uint32_t w = (uint32_t)sk.y;
    if (dt != 0.0 && (w & CELLW_MOVE_PENDING)) {
        p.x = fma(p.ux, dt, p.x);
        p.y = fma(p.uy, dt, p.y);
        p.z = fma(p.uz, dt, p.z);
        w &= ~CELLW_MOVE_PENDING;
    }
    st_rec(dst.r + j, p);
    __stcs(dst.cellw + j, w);
    dst.id[j] = p.id;
}

// At most 32 registers: the gather is bound by the loads it keeps in flight,
// so it needs the full 64 warps per SM (at 39 registers, 48, it measured 4%
// slower on the 83M-parcel channel).
__global__ void __launch_bounds__(MAX_STREAM_THREADS, 2048 / MAX_STREAM_THREADS)
k_gather(Parcels src, Parcels dst, Counters* ctr, const int2* __restrict__ sortSrc, double dt) {
    const long long n = ctr->nKept;
    const long long nSrc = ctr->nMoved;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride)
        gather_slot(src, dst, ctr, sortSrc, j, nSrc, dt);
}

// Parcels handed over as arrays (positions and velocities n x 3, ERot,
// vibrational level, species, id; a null array gives zeros, and ids 0..n-1)
// packed into records.  flags[0] gets bit 0 for a species and bit 1 for a
// vibrational level out of range; flags[1] the largest id + 1.  With write
// false the arrays are only checked (the caller fails before any state
// changes).
__global__ void k_pack(Parcels dst, long long n, const double* __restrict__ pos, const double* __restrict__ U,
                       const double* __restrict__ erot, const int* __restrict__ vib,
                       const int* __restrict__ species, const unsigned* __restrict__ id, int nSpecies,
                       unsigned* flags, int write) {
    unsigned bad = 0, maxId = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        Rec r;
        r.x = pos ? pos[3 * i] : 0.0;
        r.y = pos ? pos[3 * i + 1] : 0.0;
        r.z = pos ? pos[3 * i + 2] : 0.0;
        r.ux = U ? U[3 * i] : 0.0;
        r.uy = U ? U[3 * i + 1] : 0.0;
        r.uz = U ? U[3 * i + 2] : 0.0;
        r.erot = erot ? erot[i] : 0.0;
        r.id = id ? id[i] : (uint32_t)i;
        int sp = species ? species[i] : 0;
        int vb = vib ? vib[i] : 0;
        if (sp < 0 || sp >= nSpecies) { bad |= 1u; sp = 0; }
        if (vb < 0 || vb > SV_MAX_VIB) { bad |= 2u; vb = 0; }
        r.sv = make_sv(sp, vb);
        if (r.id + 1u > maxId) maxId = r.id + 1u;
        if (!write) continue;
        st_rec(dst.r + i, r);
        dst.cellw[i] = 0;
        dst.id[i] = r.id;
    }
    if (bad) atomicOr(flags, bad);
    if (maxId) atomicMax(flags + 1, maxId);
}

__global__ void k_ids_from_records(Parcels s, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s.id[i] = s.r[i].id;
}

__global__ void k_finish_sort(Counters* ctr) {
    // parcels dropped by the sort: deleted, or sent to another domain
    ctr->deleted += (unsigned long long)(ctr->nMoved - ctr->nKept) - ctr->nMig;
    ctr->n = ctr->nKept;
    ctr->nMoved = ctr->nKept;
}

__global__ void k_reset_sample_counters(Counters* ctr) {
    ctr->sampleSteps = 0;
    ctr->pendingSample = 0;
    ctr->unflushed = 0;
}

__global__ void k_end_step(Counters* ctr) {
    ctr->collTot += ctr->coll;
    ctr->candTot += ctr->cand;
    ctr->bigCells = 0;
    ctr->step += 1;
}

// ---------------------------------------------------------------- inflow
// One thread per (inflow face, species): Bird eq. 4.22 flux accumulation and
// the integer-plus-remainder count (dsmcFreeStreamInflowPatch.C:96-141,226-236).
// A divided cloud counts every inflow face (the face remainders and the
// parcel ids stay those of the undivided case) and fills only its own.
__global__ void k_inflow_count(CaseDev cs, int nFaces, const long long* __restrict__ face,
                               const double* __restrict__ term, double* accum, int* cnt, const Counters* ctr) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int ns = cs.nSpecies;
    if (t >= nFaces * ns) return;
    int nI = 0;
    const double add = term[t];
    if (add > 0) {
        const int m = t % ns;
        double A = accum[t] + add;
        Rng r(cs, (uint32_t)face[t / ns], (uint32_t)ctr->step, TAG_INFLOW | ((uint32_t)m << 8));
        nI = (int)A;
        if (nI < 0) nI = 0;
        if ((A - nI) > r.u01()) nI++;
        A -= nI;
        accum[t] = A;
    }
    cnt[t] = nI;
}

// Offsets of the (face, species) counts over every inflow face (off: the
// parcel ids) and over the faces of owned cells (offLocal: the slots; equal
// to off for an undivided cloud).  Single block.
__global__ void k_inflow_scan(CaseDev cs, const int* cnt, int n, const int* __restrict__ cellOf, int* off,
                              int* offLocal, Counters* ctr, long long capacity) {
    const int ns = cs.nSpecies;
    int carry = 0, carryL = 0;
    for (int b0 = 0; b0 < n; b0 += blockDim.x) {
        const int b = b0 + threadIdx.x;
        const int v = (b < n) ? cnt[b] : 0;
        const int vL = (b < n && cell_owned(cs, (uint32_t)cellOf[b / ns])) ? v : 0;
        int total, totalL;
        const int ex = block_exclusive_scan(v, &total);
        const int exL = block_exclusive_scan(vL, &totalL);
        if (b < n) {
            off[b] = carry + ex;
            offLocal[b] = carryL + exL;
        }
        carry += total;
        carryL += totalL;
    }
    if (threadIdx.x == 0) {
        off[n] = carry;
        offLocal[n] = carryL;
        if (ctr->n + carryL > capacity) {
            atomicOr(&ctr->err, ERRB_CAPACITY);
            offLocal[n] = -1;
            ctr->inflowTotal = 0;
            ctr->inflowLocal = 0;
        } else {
            ctr->inflowTotal = carry;
            ctr->inflowLocal = carryL;
        }
    }
}

// One thread per inserted parcel (dsmcFreeStreamInflowPatch.C:237-364): the
// parcel's (face, species) is found by bisection of the owned faces' count
// offsets, its id from the offsets over every face, and every parcel draws
// from its own stream (face, step, species, parcel).
__global__ void k_inflow_fill(CaseDev cs, InflowDev in, int nFaces, const long long* __restrict__ face,
                              const int* __restrict__ side, const int* __restrict__ cellOf,
                              const int* __restrict__ bfPatch, const int* __restrict__ off,
                              const int* __restrict__ offLocal, Parcels s, Counters* ctr) {
    const int ns = cs.nSpecies;
    const int nt = nFaces * ns;
    const long long total = offLocal[nt];
    if (total <= 0) return;     // nothing inserted (or capacity exceeded: -1)
    unsigned err = 0;
    for (long long gl = (long long)blockIdx.x * blockDim.x + threadIdx.x; gl < total;
         gl += (long long)gridDim.x * blockDim.x) {
        // the (face, species) slot t with offLocal[t] <= gl < offLocal[t + 1]
        int lo = 0, hi = nt;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (offLocal[mid] <= gl) lo = mid; else hi = mid;
        }
        const int t = lo;
        const int q = (int)(gl - offLocal[t]);
        const long long g = (long long)off[t] + q;     // over every face: the id
        const int f = t / ns, m = t % ns;
        const long long bf = face[f];
        const int sd = side[f];
        const int a = sd / 2;
        const int b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
        const double sgnOut = (sd & 1) ? 1.0 : -1.0;
        const InflowPatchDev& pt = in.p[bfPatch[bf]];
        const SpeciesDev& sp = cs.sp[m];
        const double cmp = sqrt(2.0 * kB * pt.Ttra / sp.m);
        const double sCos = (pt.U[a] * (-sgnOut)) / cmp;
        const double coeffA = sCos + sqrt(sCos * sCos + 2.0);
        const double coeffB = 0.5 * (1.0 + sCos * (sCos - sqrt(sCos * sCos + 2.0)));
        double scaling = 3.0;
        if (sCos < -3) scaling = fabs(sCos) + 1;
        const long long fl = bf - cs.sideOff[sd];
        const long long ib = fl % cs.n[b], ic = fl / cs.n[b];
        const double lob = node_x(cs, b, ib);
        const double loc = node_x(cs, c, ic);
        const double scT = sqrt(kB * pt.Ttra / sp.m);
        Rng r(cs, (uint32_t)bf, (uint32_t)ctr->step,
              TAG_INFLOW | ((uint32_t)m << 8) | ((uint32_t)(q + 1) << 11));
        double x[3], U[3];
        x[a] = (sd & 1) ? cs.hi[a] : cs.lo[a];
        x[b] = fma(r.u01(), cell_w(cs, b, ib), lob);
        x[c] = fma(r.u01(), cell_w(cs, c, ic), loc);
        double uNormal = 0;
        if (fabs(pt.U[a]) > VSMALL) {
            int it = 0;
            for (;;) {
                const double uth = scaling * (2.0 * r.u01() - 1);
                uNormal = uth + sCos;
                double Pr;
                if (uNormal < 0.0) Pr = -1;
                else Pr = 2.0 * uNormal / coeffA * exp(coeffB - uth * uth);
                if (!(Pr < r.u01())) break;
                if (++it >= cs.maxRejection) { err |= ERRB_REJECTION; break; }
            }
        } else {
            uNormal = sqrt(-log(r.u01()));
        }
        double g1, g2;
        r.gauss2(&g1, &g2);
        U[a] = cmp * uNormal * (-sgnOut);
        U[b] = scT * g1 + pt.U[b];
        U[c] = scT * g2 + pt.U[c];
        const double erot = eq_rot(r, pt.Trot, sp.rotDof, &err);
        const int vib = eq_vib(r, pt.Tvib, sp);
        const long long slot = ctr->n + gl;
        Rec p;
        p.x = x[0]; p.y = x[1]; p.z = x[2];
        p.ux = U[0]; p.uy = U[1]; p.uz = U[2];
        p.erot = erot;
        p.id = (uint32_t)(ctr->nextId + g);
        s.id[slot] = p.id;
        p.sv = make_sv(m, vib);
        st_rec(s.r + slot, p);
        s.cellw[slot] = ((uint32_t)cellOf[f] << 3) | CELLW_FRESH;
        if (cs.faceFlux) {
            // dsmcCloud::addNewParcel counts an inserted parcel on its face
            // (dsmcCloud.C:425-437): moving inwards, against the outward normal
            const int cc = cellOf[f];
            const int cell3[3] = {(int)(cc % cs.n[0]), (int)((cc / cs.n[0]) % cs.n[1]), (int)(cc / (cs.n[0] * cs.n[1]))};
            face_add(cs, face_index(cs, a, (sd & 1) ? cs.n[a] : 0, cell3), m, -1.0);
        }
    }
    if (err) atomicOr(&ctr->err, err);
}

__global__ void k_inflow_commit(Counters* ctr) {
    const long long add = ctr->inflowTotal;
    ctr->inserted = (unsigned long long)ctr->inflowLocal;
    // parcel ids are 32-bit and must stay unique (the light-cell picks and
    // the canonical (sub-cell, id) order rely on it): flag the step whose
    // insertions run past 2^32 ids
    if ((unsigned long long)ctr->nextId + (unsigned long long)add > 0x100000000ull) ctr->err |= ERRB_IDS;
    ctr->nextId += add;
    ctr->nMoved = ctr->n + ctr->inflowLocal;
}

// ---------------------------------------------------------------- mesh fill
// Per cell: 12 equal sub-volumes (the tets of a hex) each get
// floor(n V/12 / FN) parcels plus one with the remainder probability.
__global__ void k_init_count(CaseDev cs, const double* __restrict__ nd, const unsigned char* __restrict__ solid,
                             int* cellCounts) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cs.C) return;
    int total = 0;
    if (!solid[c]) {
        Rng r(cs, (uint32_t)c, 0, TAG_INIT_CELL);
        for (int tet = 0; tet < 12; ++tet) {
            for (int m = 0; m < cs.nSpecies; ++m) {
                if (!(nd[m] > 0)) continue;
                const double req = nd[m] * (cell_volume(cs, c) / 12.0) / cs.FN;
                int k = (int)req;
                if ((req - k) > r.u01()) k++;
                total += k;
            }
        }
    }
    cellCounts[c] = total;
}

// Per-species counts again (same draws) so that parcels come out grouped by
// species inside a cell, in the replay's order.
__global__ void k_init_fill(CaseDev cs, const double* __restrict__ nd, const unsigned char* __restrict__ solid,
                            const int* __restrict__ cellOff, Parcels s, double Ttra, double Tx, double Ty, double Tz,
                            double Trot, double Tvib, double U0, double U1, double U2, Counters* ctr) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cs.C || solid[c]) return;
    int per[DSMC_MAX_SPECIES];
    for (int m = 0; m < DSMC_MAX_SPECIES; ++m) per[m] = 0;
    {
        Rng r(cs, (uint32_t)c, 0, TAG_INIT_CELL);
        for (int tet = 0; tet < 12; ++tet) {
            for (int m = 0; m < cs.nSpecies; ++m) {
                if (!(nd[m] > 0)) continue;
                const double req = nd[m] * (cell_volume(cs, c) / 12.0) / cs.FN;
                int k = (int)req;
                if ((req - k) > r.u01()) k++;
                per[m] += k;
            }
        }
    }
    const int i0 = (int)(c % cs.n[0]);
    const int j0 = (int)((c / cs.n[0]) % cs.n[1]);
    const int k0 = (int)(c / ((long long)cs.n[0] * cs.n[1]));
    const double cl[3] = {node_x(cs, 0, i0), node_x(cs, 1, j0), node_x(cs, 2, k0)};
    const double cw[3] = {cell_w(cs, 0, i0), cell_w(cs, 1, j0), cell_w(cs, 2, k0)};
    const double Ta[3] = {Tx > 0 ? Tx : Ttra, Ty > 0 ? Ty : Ttra, Tz > 0 ? Tz : Ttra};
    const double Ub[3] = {U0, U1, U2};
    long long slot = cellOff[c];
    unsigned err = 0;
    for (int m = 0; m < cs.nSpecies; ++m) {
        const SpeciesDev& sp = cs.sp[m];
        for (int q = 0; q < per[m]; ++q, ++slot) {
            const uint32_t pid = (uint32_t)slot;
            Rng r(cs, pid, 0, TAG_INIT_PARTICLE);
            double x[3];
            for (int a = 0; a < 3; ++a) x[a] = fma(r.u01(), cw[a], cl[a]);
            double g[4];
            r.gauss2(&g[0], &g[1]);
            r.gauss2(&g[2], &g[3]);
            double U[3];
            for (int a = 0; a < 3; ++a) U[a] = sqrt(kB * Ta[a] / sp.m) * g[a] + Ub[a];
            const double erot = eq_rot(r, Trot, sp.rotDof, &err);
            const int vib = eq_vib(r, Tvib, sp);
            int sb = 0, ci[3];
            for (int a = 0; a < 3; ++a) {
                int c2 = floor2_coord(cs, x[a], a);
                c2 = min(max(c2, 0), 2 * cs.n[a] - 1);
                ci[a] = c2 >> 1;
                sb |= (c2 & 1) << a;
            }
            Rec p;
            p.x = x[0]; p.y = x[1]; p.z = x[2];
            p.ux = U[0]; p.uy = U[1]; p.uz = U[2];
            p.erot = erot;
            p.id = pid;
            s.id[slot] = pid;
            p.sv = make_sv(m, vib);
            st_rec(s.r + slot, p);
            s.cellw[slot] = ((uint32_t)(ci[0] + cs.n[0] * (ci[1] + cs.n[1] * ci[2])) << 3) | (uint32_t)sb;
        }
    }
    if (err) atomicOr(&ctr->err, err);
}

__global__ void k_cellw(CaseDev cs, Parcels s, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Rec p = ldg_rec(s.r + i);
    const double x[3] = {p.x, p.y, p.z};
    int sb = 0, ci[3];
    for (int a = 0; a < 3; ++a) {
        int c2 = floor2_coord(cs, x[a], a);
        c2 = min(max(c2, 0), 2 * cs.n[a] - 1);
        ci[a] = c2 >> 1;
        sb |= (c2 & 1) << a;
    }
    const uint32_t fresh = s.cellw[i] & CELLW_FRESH;
    const uint32_t c = (uint32_t)(ci[0] + cs.n[0] * (ci[1] + cs.n[1] * ci[2]));
    // a divided cloud keeps only the parcels of its own cells
    s.cellw[i] = cell_owned(cs, c) ? ((c << 3) | (uint32_t)sb) | fresh : CELLW_DELETED;
}

__global__ void k_remainder_init(CaseDev cs, double* rem) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cs.C) return;
    Rng r(cs, (uint32_t)c, 0, TAG_REMAINDER);
    rem[c] = r.u01();
}

// ---------------------------------------------------------------- batch
// The move and sort half of a batched step for every case of a batch, in one
// persistent launch (phases separated by grid barriers, work items taken from
// per-phase tickets; see dsmc_persist.cuh).  The per-parcel work is the
// single-case kernels' own (move_iter, move_slow, scatter_iter, gather_slot),
// so a batched case steps exactly as it steps alone.  Cases on a uniform mesh
// without inflow, obstacles, reduced-D axes or face tracking only.
#include "dsmc_persist.cuh"   // (no includes of its own: it sits in this namespace)

constexpr int BM_IT = 8;    // iterations of the CTA per move, scatter and gather item

enum { BM_ZERO = 0, BM_MOVE, BM_SLOW, BM_DONE, BM_FINAL, BM_SCAN, BM_SCATTER, BM_GATHER, BM_FINISH, BM_NPHASE };
static_assert(BATCH_TICKETS_MOVE + BM_NPHASE <= BATCH_TICKETS_COLLIDE, "ticket counters of the move launch");

// Phases [P0, P1) in one launch: the step runs as four launches (zero and
// move; boundary path, sample commit and scan; index scatter; gather and
// finish), so that each is compiled and made resident with its own phases'
// registers (one launch of every phase took the boundary path's and the
// scan's 124 registers everywhere and held the move to 16 warps per SM).
template <int P0, int P1>
__global__ void __launch_bounds__(MAX_STREAM_THREADS)
k_batch_move(const BatchSlot* __restrict__ slots, int n, BatchCtl* ctl) {
    __shared__ long long pre[BATCH_MAX_CASES + 1];
    const int T = blockDim.x;
    const int tid = threadIdx.x;
#pragma unroll
    for (int ph = P0; ph < P1; ++ph) {
        long long total;
        switch (ph) {
        case BM_MOVE:
        case BM_SCATTER:
            total = persist::phase_items(n, pre, [&](int i) {
                return (slots[i].B.ctr->nMoved + (long long)T * BM_IT - 1) / ((long long)T * BM_IT);
            });
            break;
        case BM_GATHER:
            total = persist::phase_items(n, pre, [&](int i) {
                return (slots[i].B.ctr->nKept + (long long)T * BM_IT - 1) / ((long long)T * BM_IT);
            });
            break;
        case BM_SLOW:
            total = persist::phase_items(n, pre, [&](int i) {
                return ((long long)slots[i].B.ctr->nSlow + T - 1) / T;
            });
            break;
        case BM_FINAL:
            total = persist::phase_items(n, pre, [&](int i) {
                const Counters* c = slots[i].B.ctr;
                if (c->unflushed < SAMPLES_PER_FLUSH) return 0LL;
                const long long m = (long long)slots[i].cs.nSpecies * SACC * slots[i].cs.C;
                return (m + (long long)T * BM_IT - 1) / ((long long)T * BM_IT);
            });
            break;
        default:   // one item per case
            total = persist::phase_items(n, pre, [&](int) { return 1LL; });
        }
        const int tk = BATCH_TICKETS_MOVE + ph;
        for (long long q = persist::next_item(ctl, tk, total); q >= 0; q = persist::next_item(ctl, tk, total)) {
            const int ci = persist::item_case(pre, n, q);
            const long long l = q - pre[ci];
            const BatchSlot& sl = slots[ci];
            const CaseDev& cs = sl.cs;
            const StepBuffers& B = sl.B;
            Counters* ctr = B.ctr;
            unsigned err = 0;
            switch (ph) {
            case BM_ZERO:
                if (tid == 0) {
                    ctr->nMoved = ctr->n;
                    ctr->coll = ctr->cand = 0;
                    ctr->wallHits = ctr->inserted = ctr->deleted = 0;
                    ctr->bigCells = 0;
                    ctr->nSlow = 0;
                    ctr->nWork = ctr->nHeavy = 0;
                }
                break;
            case BM_MOVE: {
                const long long nm = ctr->nMoved;
                const uint32_t step = (uint32_t)ctr->step;
                const int doSample = ctr->pendingSample;
                for (int k = 0; k < BM_IT; ++k) {
                    const long long base = (l * BM_IT + k) * T;
                    if (base >= nm) break;
                    move_iter<false>(cs, sl.src, ctr, B.slowList, B.count, B.sfix, base + tid, nm, step, doSample,
                                     1, nullptr, 0, err);
                }
                break;
            }
            case BM_SLOW: {
                const long long k = l * T + tid;
                if (k < (long long)ctr->nSlow) {
                    const long long i = B.slowList[k];
                    const uint32_t w = sl.src.cellw[i];
                    const uint32_t nw = move_slow(cs, sl.src, i, (uint32_t)ctr->step, w, B.bfPatch, B.wall, &err,
                                                  &ctr->wallHits);
                    sl.src.cellw[i] = nw;
                    if (nw != CELLW_DELETED) atomicAdd(&B.count[nw >> 3], 1);
                }
                break;
            }
            case BM_DONE:
                if (tid == 0 && ctr->pendingSample) {
                    ctr->sampleSteps += 1;
                    ctr->unflushed += 1;
                    ctr->pendingSample = 0;
                }
                break;
            case BM_FINAL: {
                const long long m = (long long)cs.nSpecies * SACC * cs.C;
                for (int k = 0; k < BM_IT; ++k) {
                    const long long idx = (l * BM_IT + k) * T + tid;
                    if (idx >= m) break;
                    const long long v = B.sfix[idx];
                    if (!v) continue;
                    const int kk = (int)((idx / cs.C) % SACC);
                    const int F = (kk == SACC_UU) ? F_UU : (kk == SACC_EROT) ? F_E : F_U;
                    B.acc[idx] += (kk == SACC_N || kk == SACC_VIB) ? (double)v : unfix(v, F);
                    B.sfix[idx] = 0;
                }
                break;
            }
            case BM_SCAN: {
                // the whole occupancy scan of the case by this CTA
                if (tid == 0 && ctr->unflushed >= SAMPLES_PER_FLUSH) ctr->unflushed = 0;
                const long long C = cs.C;
                int carry = 0;
                for (long long c0 = 0; c0 < C; c0 += (long long)T * SCAN_ITEMS) {
                    const long long b0 = c0 + (long long)tid * SCAN_ITEMS;
                    int v[SCAN_ITEMS];
                    int sum = 0;
#pragma unroll
                    for (int k = 0; k < SCAN_ITEMS; ++k) {
                        v[k] = (b0 + k < C) ? B.count[b0 + k] : 0;
                        sum += v[k];
                    }
                    int tot;
                    int ex = block_exclusive_scan(sum, &tot) + carry;
#pragma unroll
                    for (int k = 0; k < SCAN_ITEMS; ++k) {
                        if (b0 + k < C) B.start[b0 + k] = ex;
                        ex += v[k];
                    }
                    carry += tot;
                }
                if (tid == 0) {
                    B.start[C] = carry;
                    ctr->nKept = carry;
                }
                break;
            }
            case BM_SCATTER: {
                const long long nm = ctr->nMoved;
                for (int k = 0; k < BM_IT; ++k) {
                    const long long base = (l * BM_IT + k) * T;
                    if (base >= nm) break;
                    scatter_iter(sl.src.cellw, ctr, B.start, B.count, B.sortSrc, base + tid, nm);
                }
                break;
            }
            case BM_GATHER: {
                const long long nk = ctr->nKept, nm = ctr->nMoved;
                for (int k = 0; k < BM_IT; ++k) {
                    const long long j = (l * BM_IT + k) * T + tid;
                    if (j < nk) gather_slot(sl.src, sl.dst, ctr, B.sortSrc, j, nm, cs.dt);
                }
                break;
            }
            case BM_FINISH:
                if (tid == 0) {
                    ctr->deleted += (unsigned long long)(ctr->nMoved - ctr->nKept);
                    ctr->n = ctr->nKept;
                    ctr->nMoved = ctr->nKept;
                }
                break;
            }
            if (err) atomicOr(&ctr->err, err);
        }
        if (ph + 1 < P1 && !persist::grid_sync(ctl)) return;
    }
}

constexpr int BM_SPLIT1 = BM_SLOW, BM_SPLIT2 = BM_SCATTER, BM_SPLIT3 = BM_GATHER;

template <int P0, int P1>
int batch_move_grid_of(int threads) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_move<P0, P1>, threads, 0) != cudaSuccess) return 0;
    return per * sms;
}

template <int P0, int P1>
cudaError_t launch_batch_move_part(const BatchSlot* slots, int n, BatchCtl* ctl, int threads, cudaStream_t st) {
    const int grid = batch_move_grid_of<P0, P1>(threads);
    if (grid <= 0) return cudaErrorInvalidConfiguration;
    void* args[] = {(void*)&slots, (void*)&n, (void*)&ctl};
    return cudaLaunchCooperativeKernel((const void*)k_batch_move<P0, P1>, dim3(grid), dim3(threads), args, 0, st);
}

int grid_for(long long n, int threads, int perSmBlocks) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long need = (n + threads - 1) / threads;
    const long long cap = (long long)sms * perSmBlocks;
    long long g = need < cap ? need : cap;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

int scan_scratch_ints(long long C) { return (int)((C + SCAN_TILE - 1) / SCAN_TILE) + 1; }

// the smallest resident grid of the four launches (0: one cannot run)
int batch_move_grid(int threads) {
    const int a = batch_move_grid_of<0, BM_SPLIT1>(threads);
    const int b = batch_move_grid_of<BM_SPLIT1, BM_SPLIT2>(threads);
    const int c = batch_move_grid_of<BM_SPLIT2, BM_SPLIT3>(threads);
    const int d = batch_move_grid_of<BM_SPLIT3, BM_NPHASE>(threads);
    return std::min(std::min(a, b), std::min(c, d));
}

cudaError_t launch_batch_move(const BatchSlot* slots, int n, BatchCtl* ctl, int threads, cudaStream_t st) {
    cudaError_t e = launch_batch_move_part<0, BM_SPLIT1>(slots, n, ctl, threads, st);
    if (e == cudaSuccess) e = launch_batch_move_part<BM_SPLIT1, BM_SPLIT2>(slots, n, ctl, threads, st);
    if (e == cudaSuccess) e = launch_batch_move_part<BM_SPLIT2, BM_SPLIT3>(slots, n, ctl, threads, st);
    if (e == cudaSuccess) e = launch_batch_move_part<BM_SPLIT3, BM_NPHASE>(slots, n, ctl, threads, st);
    return e;
}

void launch_move(const CaseDev& cs, const StepBuffers& B, const Parcels& s, cudaStream_t st, cudaEvent_t mid,
                 bool deferPos, int range) {
    const int T = B.cfg.streamThreads;
    const int grid = grid_for(B.capacity, T, B.cfg.streamCtasPerSm);
    const bool general = cs.anyEmpty || cs.nObst || cs.faceFlux || cs.half[0] || cs.half[1] || cs.half[2] ||
                         cs.domAxis >= 0;
    const int d = deferPos ? 1 : 0;
    if (general)
        k_move<true><<<grid, T, 0, st>>>(cs, s, B.ctr, B.slowList, B.count, B.sfix, d, B.migList, B.migCap, range);
    else k_move<false><<<grid, T, 0, st>>>(cs, s, B.ctr, B.slowList, B.count, B.sfix, d, nullptr, 0, range);
    if (range == MOVE_KEPT) return;   // the inserted parcels' move and the boundary path follow
    if (mid) cudaEventRecord(mid, st);
    k_move_slow<<<grid_for(B.capacity, T, 2), T, 0, st>>>(cs, s, B.ctr, B.slowList, B.bfPatch, B.wall, B.count,
                                                          B.migList, B.migCap);
}

void launch_pack_migrants(const CaseDev& cs, const StepBuffers& B, const Parcels& s, cudaStream_t st) {
    k_pack_migrants<<<grid_for(B.migCap, 256, 2), 256, 0, st>>>(s, B.ctr, B.migList, B.migOut, B.migCap, cs.dt);
}

void launch_unpack_migrants(const CaseDev& cs, const StepBuffers& B, const Parcels& s, const uint32_t* src,
                            long long n, long long base, cudaStream_t st) {
    if (n <= 0) return;
    k_unpack_migrants<<<grid_for(n, 256, 8), 256, 0, st>>>(cs, s, B.ctr, src, n, base, B.count);
    k_migrants_commit<<<1, 1, 0, st>>>(B.ctr, n);
}

void launch_count(const CaseDev& cs, const StepBuffers& B, const Parcels& s, cudaStream_t st) {
    (void)cs;
    const int grid = grid_for(B.capacity, 256, 8);
    k_count_dev<<<grid, 256, 0, st>>>(s, B.ctr, B.count);
}

void launch_scan(const CaseDev& cs, const StepBuffers& B, cudaStream_t st) {
    const int nb = (int)((cs.C + SCAN_TILE - 1) / SCAN_TILE);
    k_scan_reduce<<<nb, SCAN_THREADS, 0, st>>>(B.count, cs.C, B.blockSums);
    k_scan_top<<<1, SCAN_THREADS, 0, st>>>(B.blockSums, nb, B.start, cs.C, B.ctr);
    k_scan_down<<<nb, SCAN_THREADS, 0, st>>>(B.count, cs.C, B.blockSums, B.start);
}

void launch_scatter(const CaseDev& cs, const StepBuffers& B, const Parcels& src, const Parcels& dst,
                    cudaStream_t st, cudaEvent_t mid, bool movePending) {
    const int T = B.cfg.streamThreads;
    const int grid = grid_for(B.capacity, T, B.cfg.streamCtasPerSm);
    k_scatter_index<<<grid, T, 0, st>>>(src.cellw, B.ctr, B.start, B.count, B.sortSrc);
    if (mid) cudaEventRecord(mid, st);
    k_gather<<<grid, T, 0, st>>>(src, dst, B.ctr, B.sortSrc, movePending ? cs.dt : 0.0);
}

void launch_pack(const Parcels& dst, long long n, const double* pos, const double* U, const double* erot,
                 const int* vib, const int* species, const unsigned* id, int nSpecies, unsigned* flags,
                 int write, cudaStream_t st) {
    if (n > 0)
        k_pack<<<grid_for(n, 256, 8), 256, 0, st>>>(dst, n, pos, U, erot, vib, species, id, nSpecies, flags, write);
}

// dsmcFluxSurface::calculateField (dsmcFluxSurface.C:316-343): the sum over
// the zone's faces and the selected species of the face sums times w, where
// w = FN (S/|S| . fluxDirection) of the face; out[0] parcels, out[1] mass.
// One block with a fixed reduction order, so equal sums give equal results.
__global__ void __launch_bounds__(256) k_flux_surface(const double* __restrict__ flux, int nSpecies,
                                                      long long nFacesAll, const int* __restrict__ faces,
                                                      const double* __restrict__ w, int nF, unsigned mask,
                                                      double* out) {
    __shared__ double sh[2][256];
    double p = 0.0, m = 0.0;
    for (int i = threadIdx.x; i < nF; i += 256) {
        const long long f = faces[i];
        double fp = 0.0, fm = 0.0;
        for (int q = 0; q < nSpecies; ++q)
            if ((mask >> q) & 1u) {
                fp += flux[(long long)q * nFacesAll + f];
                fm += flux[((long long)nSpecies + q) * nFacesAll + f];
            }
        p = fma(fp, w[i], p);
        m = fma(fm, w[i], m);
    }
    sh[0][threadIdx.x] = p;
    sh[1][threadIdx.x] = m;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) {
            sh[0][threadIdx.x] += sh[0][threadIdx.x + k];
            sh[1][threadIdx.x] += sh[1][threadIdx.x + k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sh[0][0];
        out[1] = sh[1][0];
    }
}

void launch_flux_surface(const CaseDev& cs, const int* faces, const double* w, int nF, unsigned mask,
                         double* out2, cudaStream_t st) {
    k_flux_surface<<<1, 256, 0, st>>>(cs.faceFlux, cs.nSpecies, cs.nFacesAll, faces, w, nF, mask, out2);
}

void launch_ids_from_records(const Parcels& s, long long n, cudaStream_t st) {
    if (n > 0) k_ids_from_records<<<grid_for(n, 256, 8), 256, 0, st>>>(s, n);
}

void launch_finish_sort(const StepBuffers& B, cudaStream_t st) {
    k_finish_sort<<<1, 1, 0, st>>>(B.ctr);
}

void launch_sample_commit(const CaseDev& cs, const StepBuffers& B, int force, cudaStream_t st) {
    const long long total = (long long)cs.nSpecies * SACC * cs.C;
    k_sample_done<<<1, 1, 0, st>>>(B.ctr);
    k_sample_finalize<<<grid_for(total, 256, 8), 256, 0, st>>>(cs, B.ctr, B.sfix, B.acc, force);
    k_sample_flushed<<<1, 1, 0, st>>>(B.ctr, force);
}

void launch_sample_flush(const CaseDev& cs, const StepBuffers& B, const Parcels& s, int force, cudaStream_t st) {
    const int T = B.cfg.streamThreads;
    k_sample_pass<<<grid_for(B.capacity, T, B.cfg.streamCtasPerSm), T, 0, st>>>(cs, s, B.ctr, B.sfix);
    launch_sample_commit(cs, B, force, st);
}

void launch_set_pending(const StepBuffers& B, cudaStream_t st) { k_set_pending<<<1, 1, 0, st>>>(B.ctr); }

void launch_reset_sample_counters(const StepBuffers& B, cudaStream_t st) {
    k_reset_sample_counters<<<1, 1, 0, st>>>(B.ctr);
}

void launch_end_step(const StepBuffers& B, cudaStream_t st) {
    k_end_step<<<1, 1, 0, st>>>(B.ctr);
}

void launch_inflow(const CaseDev& cs, const InflowDev& in, const StepBuffers& B, const Parcels& s,
                   cudaStream_t st) {
    const int nt = B.nInflowFaces * cs.nSpecies;
    if (nt == 0) return;
    const int grid = (nt + 255) / 256;
    k_inflow_count<<<grid, 256, 0, st>>>(cs, B.nInflowFaces, B.inflowFace, B.inflowTerm, B.inflowAcc,
                                         B.inflowCount, B.ctr);
    k_inflow_scan<<<1, 1024, 0, st>>>(cs, B.inflowCount, nt, B.inflowCell, B.inflowOff, B.inflowOffLocal, B.ctr,
                                      cs.capacityLimit < B.capacity ? cs.capacityLimit : B.capacity);
    k_inflow_fill<<<grid_for(B.capacity, 256, 8), 256, 0, st>>>(cs, in, B.nInflowFaces, B.inflowFace,
                                                                B.inflowSide, B.inflowCell, B.bfPatch,
                                                                B.inflowOff, B.inflowOffLocal, s, B.ctr);
    k_inflow_commit<<<1, 1, 0, st>>>(B.ctr);
}

void launch_init_fill(const CaseDev& cs, const StepBuffers& B, const Parcels& s, const double* dnd,
                      const unsigned char* solid, const int* cellOff, double Ttra, const double* Txyz,
                      double Trot, double Tvib, const double* U, cudaStream_t st) {
    const int grid = (int)((cs.C + 127) / 128);
    k_init_fill<<<grid, 128, 0, st>>>(cs, dnd, solid, cellOff, s, Ttra, Txyz[0], Txyz[1], Txyz[2], Trot,
                                      Tvib, U[0], U[1], U[2], B.ctr);
}

void launch_init_count(const CaseDev& cs, const double* dnd, const unsigned char* solid, int* cellCounts,
                       cudaStream_t st) {
    const int grid = (int)((cs.C + 255) / 256);
    k_init_count<<<grid, 256, 0, st>>>(cs, dnd, solid, cellCounts);
}

void launch_cellw(const CaseDev& cs, const Parcels& s, long long n, cudaStream_t st) {
    if (n <= 0) return;
    k_cellw<<<(int)((n + 255) / 256), 256, 0, st>>>(cs, s, n);
}

void launch_count_n(const Parcels& s, long long n, int* count, cudaStream_t st) {
    if (n <= 0) return;
    const int grid = grid_for(n, 256, 8);
    k_count<<<grid, 256, 0, st>>>(s, n, count);
}

void launch_remainder_init(const CaseDev& cs, double* rem, cudaStream_t st) {
    k_remainder_init<<<(int)((cs.C + 255) / 256), 256, 0, st>>>(cs, rem);
}

}  // namespace dsmc
