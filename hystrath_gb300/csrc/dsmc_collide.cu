// dsmc_collide.cu -- per-cell collisions and sampling, derived fields, totals.
//
// collide   noTimeCounter::collide (src/lagrangian/dsmc/collisionPartnerSelection/
//           derived/noTimeCounter/noTimeCounter.C:81-339) with
//           VariableHardSphere::sigmaTcR/scatter/postCollisionVelocities
//           (collisions/derived/VariableHardSphere/VariableHardSphere.C:80-228),
//           LarsenBorgnakkeVariableHardSphere::collide/redistribute
//           (LarsenBorgnakkeVariableHardSphere.C:110-279) and the
//           dsmcCloud::postCollision* samplers (dsmcCloud.C:1327-1531).
// sample    dsmcVolFields::calculateField sample loop
//           (macroscopicProperties/derived/combined/dsmcVolFields/dsmcVolFields.C:1115-1239).
// fields    dsmcVolFields.C:1242-1290 and 1365-1876 (output-time fields).
// info      dsmcCloud::info (dsmcCloud.C:935-985).
//
// A warp takes a tile of 32 consecutive cells, one cell per lane.  Each lane
// puts its cell's parcels in canonical (particle id) order, runs the cell's
// candidate loop serially as the reference requires (later candidates see
// earlier collisions) and sums the cell's samples in that order, so results
// do not depend on the order the sort scatter left in memory.  GB300 issues
// an FP64 instruction over the whole warp whatever the active mask, which is
// why the serial work is spread over lanes rather than left to one lane.
// Cells with more than BIGN parcels take a warp-per-cell path.

#include "dsmc_kernels.h"

namespace dsmc {

namespace {

constexpr int CWARPS = 4;         // warps per block

struct StageView {
    uint32_t* sid;
    int* perm;
    int* scl;
    double *ux, *uy, *uz, *erot;
    int* vib;
    unsigned char* spsub;
    unsigned char* dirty;
};


__device__ __forceinline__ double post_rot(Rng& r, double dof, double ChiB, unsigned* err) {
    if (dof == 2.0) return 1.0 - pow(r.u01(), 1.0 / ChiB);
    const double ChiA = 0.5 * dof;
    const double A1 = ChiA - 1., B1 = ChiB - 1.;
    if (A1 < SMALL && B1 < SMALL) return r.u01();
    for (int it = 0; it < MAX_REJECTION; ++it) {
        const double ratio = r.u01();
        double Pr;
        if (A1 < SMALL) Pr = pow(1.0 - ratio, B1);
        else if (B1 < SMALL) Pr = pow(1.0 - ratio, A1);
        else Pr = pow((A1 + B1) * ratio / A1, A1) * pow((A1 + B1) * (1 - ratio) / B1, B1);
        if (!(Pr < r.u01())) return ratio;
    }
    *err |= ERRB_REJECTION;
    return 0.0;
}

// postCollisionVibrationalEnergyLevel, non-reacting branch.  1/Zv comes from
// the per-pair table when iMax is tabulated.  The level acceptance
// probability (Bird eq. 5.61) is only compared with a uniform deviate, so it
// is evaluated in FP32.
__device__ __forceinline__ int post_vib(const CaseDev& cs, Rng& r, int vib, int iMax, const SpeciesDev& s,
                                        double omega, double Ec, const double* tab, unsigned* err) {
    double invZv;
    if (cs.fixedZv == 0) {
        if (tab && iMax < ZV_TAB) {
            invZv = tab[iMax];
        } else {
            const double T = iMax * s.thetaV / (3.5 - omega);
            const double pow1 = pow(s.thetaD / T, 1. / 3.) - 1.0;
            const double pow2 = pow(s.thetaD / s.trefZv, 1. / 3.) - 1.0;
            const double ZvP1 = pow(s.thetaD / T, omega);
            const double ZvP2 = pow(s.zref * pow(s.thetaD / s.trefZv, -omega), pow1 / pow2);
            const double Zv = ZvP1 * ZvP2;
            invZv = (cs.invZvForm == 2) ? 1.0 / (5.0 * Zv) : 1.0 / Zv;
        }
    } else {
        invZv = 1.0 / cs.fixedZv;
    }
    if (invZv > r.u01()) {
        const float ex = (float)(1.5 - omega);
        for (int it = 0; it < MAX_REJECTION; ++it) {
            const int iDash = r.label(0, iMax, err);
            const float base = (float)(1.0 - (iDash * s.kThetaV) / Ec);
            const float func = powf(base > 0.0f ? base : 0.0f, ex);
            if (!((double)func < r.u01())) return iDash;
        }
        *err |= ERRB_REJECTION;
    }
    return vib;
}

__device__ __forceinline__ void redistribute(const CaseDev& cs, const SpeciesDev& s, double* erot, int* vib,
                                             double& Et, double omegaPQ, Rng& r, const double* tab,
                                             unsigned* err) {
    if (s.nVib > 0) {
        const double EcP = Et + *vib * s.kThetaV;
        const int iMax = (int)(EcP / s.kThetaV);
        if (iMax > 0) {
            *vib = post_vib(cs, r, *vib, iMax, s, omegaPQ, EcP, tab, err);
            Et = EcP - *vib * s.kThetaV;
        }
    }
    if (s.rotDof > 0) {
        const double pre = *erot;
        if (1.0 / cs.zrot > r.u01()) {
            const double EcP = Et + pre;
            const double ChiB = 2.5 - omegaPQ;
            const double ratio = post_rot(r, s.rotDof, ChiB, err);
            *erot = ratio * EcP;
            Et = EcP - *erot;
        }
    }
}

__device__ __forceinline__ const double* zv_row(const CaseDev& cs, int p, int q) {
    return cs.invZvTab ? cs.invZvTab + (size_t)(p * DSMC_MAX_SPECIES + q) * ZV_TAB : nullptr;
}

// sigma_T c_R of VariableHardSphere::sigmaTcR.  It feeds only the acceptance
// test and the running maximum, so it is evaluated in FP32.
__device__ __forceinline__ double sigma_cr(const PairDev& pr, double cr2) {
    if (sqrt(cr2) < VSMALL) return 0.0;
    return (double)(pr.sigmaPrefactorF * powf((float)cr2, pr.expoF));
}

// Serial NTC over the candidates of one cell (lane 0 only).
__device__ void ntc_cell(const CaseDev& cs, const Soa& s, long long c, int off, int n, const StageView& v,
                         const int* subStart, double* smax, double* rem, double* acc, uint32_t step,
                         long long nCand, double smax0, unsigned* err, unsigned long long* nColl) {
    Rng r(cs, (uint32_t)c, step, TAG_COLLIDE);
    double smaxRun = smax[c];
    unsigned long long coll = 0;
    double collSep = 0.0;
    for (long long k = 0; k < nCand; ++k) {
        const int iP = r.label(0, n - 1, err);
        const int jP0 = v.perm[iP];
        const int sub = v.spsub[jP0] & 7;
        const int s0 = subStart[sub], nSC = subStart[sub + 1] - s0;
        int iQ = -1, it = 0;
        if (nSC > 1) {
            do { iQ = v.scl[s0 + r.label(0, nSC - 1, err)]; } while (iP == iQ && ++it < MAX_REJECTION);
        } else {
            do { iQ = r.label(0, n - 1, err); } while (iP == iQ && ++it < MAX_REJECTION);
        }
        if (it >= MAX_REJECTION) { *err |= ERRB_REJECTION; continue; }
        const int jP = jP0, jQ = v.perm[iQ];
        const int tP = v.spsub[jP] >> 3, tQ = v.spsub[jQ] >> 3;
        const PairDev& pr = cs.pair[tP * DSMC_MAX_SPECIES + tQ];
        double UP[3] = {v.ux[jP], v.uy[jP], v.uz[jP]};
        double UQ[3] = {v.ux[jQ], v.uy[jQ], v.uz[jQ]};
        const double d0 = UP[0] - UQ[0], d1 = UP[1] - UQ[1], d2 = UP[2] - UQ[2];
        const double cr2 = d0 * d0 + d1 * d1 + d2 * d2;
        const double sigma = sigma_cr(pr, cr2);
        if (sigma > smaxRun) smaxRun = sigma;
        if (sigma > r.u01() * smax0) {      // (sigma/smax0) > U with smax0 > 0
            double cR;
            if (cs.collModel == DSMC_COLL_LB_VHS) {
                double Et = 0.5 * pr.mR * cr2;
                double eP = v.erot[jP], eQ = v.erot[jQ];
                int vP = v.vib[jP], vQ = v.vib[jQ];
                redistribute(cs, cs.sp[tP], &eP, &vP, Et, pr.omegaPQ, r, zv_row(cs, tP, tQ), err);
                redistribute(cs, cs.sp[tQ], &eQ, &vQ, Et, pr.omegaPQ, r, zv_row(cs, tQ, tP), err);
                v.erot[jP] = eP; v.erot[jQ] = eQ;
                v.vib[jP] = vP; v.vib[jQ] = vQ;
                cR = sqrt(2.0 * Et / pr.mR);
            } else {
                cR = sqrt(cr2);
            }
            double Ucm[3];
            for (int a = 0; a < 3; ++a) Ucm[a] = pr.mPfrac * UP[a] + pr.mQfrac * UQ[a];
            const double cosT = 2.0 * r.u01() - 1.0;
            const double sinT = sqrt(1.0 - cosT * cosT);
            const double phi = 2.0 * PI * r.u01();
            double sph, cph;
            sincos(phi, &sph, &cph);
            const double prel[3] = {cR * cosT, cR * sinT * cph, cR * sinT * sph};
            for (int a = 0; a < 3; ++a) {
                UP[a] = Ucm[a] + prel[a] * pr.mQfrac;
                UQ[a] = Ucm[a] - prel[a] * pr.mPfrac;
            }
            v.ux[jP] = UP[0]; v.uy[jP] = UP[1]; v.uz[jP] = UP[2];
            v.ux[jQ] = UQ[0]; v.uy[jQ] = UQ[1]; v.uz[jQ] = UQ[2];
            v.dirty[jP] = 1;
            v.dirty[jQ] = 1;
            const double dx = s.x[off + jP] - s.x[off + jQ];
            const double dy = s.y[off + jP] - s.y[off + jQ];
            const double dz = s.z[off + jP] - s.z[off + jQ];
            collSep += sqrt(dx * dx + dy * dy + dz * dz);
            ++coll;
        }
    }
    smax[c] = smaxRun;
    if (coll) {
        acc[(cs.nSpecies * SACC + CACC_NCOLLS) * cs.C + c] += (double)coll;
        acc[(cs.nSpecies * SACC + CACC_COLLSEP) * cs.C + c] += collSep;
    }
    *nColl += coll;
}

__device__ void process_cell(const CaseDev& cs, const Soa& s, long long c, int off, int n, const StageView& v,
                             int* subStart, double* smax, double* rem, double* acc, uint32_t step,
                             int doCollide, int doSample, unsigned* err, unsigned long long* nColl,
                             unsigned long long* nCandTot) {
    const unsigned lane = lane_id();
    for (int j = lane; j < n; j += 32) {
        const long long g = (long long)off + j;
        v.sid[j] = s.id[g];
        v.spsub[j] = (unsigned char)((s.spc[g] << 3) | (s.cellw[g] & 7u));
        v.ux[j] = s.ux[g];
        v.uy[j] = s.uy[g];
        v.uz[j] = s.uz[g];
        v.erot[j] = s.erot[g];
        v.vib[j] = s.vib[g];
        v.dirty[j] = 0;
    }
    __syncwarp();
    // canonical order: rank by particle id
    for (int j = lane; j < n; j += 32) {
        const uint32_t my = v.sid[j];
        int rk = 0;
        for (int k = 0; k < n; ++k) {
            const uint32_t o = v.sid[k];
            rk += (o < my || (o == my && k < j)) ? 1 : 0;
        }
        v.perm[rk] = j;
    }
    __syncwarp();
    if (doCollide && n > 1) {
        long long nCand = 0;
        double smax0 = 0.0;
        if (lane == 0) {
            smax0 = smax[c];
            const double sel = rem[c] + 0.5 * n * (n - 1) * cs.FN * smax0 * cs.dt / cs.V;
            nCand = (long long)sel;
            rem[c] = sel - (double)nCand;
        }
        nCand = __shfl_sync(0xFFFFFFFFu, nCand, 0);
        smax0 = __shfl_sync(0xFFFFFFFFu, smax0, 0);
        if (nCand > 0) {
            // sub-cell member lists in canonical order
            int cnt[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) cnt[q] = 0;
            for (int k0 = 0; k0 < n; k0 += 32) {
                const int k = k0 + lane;
                const int sb = (k < n) ? (v.spsub[v.perm[k]] & 7) : 8;
#pragma unroll
                for (int q = 0; q < 8; ++q) cnt[q] += __popc(__ballot_sync(0xFFFFFFFFu, sb == q));
            }
            if (lane == 0) {
                int acc0 = 0;
                for (int q = 0; q < 8; ++q) { subStart[q] = acc0; acc0 += cnt[q]; }
                subStart[8] = acc0;
            }
            __syncwarp();
            int fill[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) fill[q] = subStart[q];
            for (int k0 = 0; k0 < n; k0 += 32) {
                const int k = k0 + lane;
                const int sb = (k < n) ? (v.spsub[v.perm[k]] & 7) : 8;
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const unsigned m = __ballot_sync(0xFFFFFFFFu, sb == q);
                    if (sb == q) v.scl[fill[q] + __popc(m & ((1u << lane) - 1u))] = k;
                    fill[q] += __popc(m);
                }
            }
            __syncwarp();
            if (lane == 0) {
                ntc_cell(cs, s, c, off, n, v, subStart, smax, rem, acc, step, nCand, smax0, err, nColl);
                *nCandTot += (unsigned long long)nCand;
            }
            __syncwarp();
            for (int j = lane; j < n; j += 32) {
                if (v.dirty[j]) {
                    const long long g = (long long)off + j;
                    s.ux[g] = v.ux[j];
                    s.uy[g] = v.uy[j];
                    s.uz[g] = v.uz[j];
                    s.erot[g] = v.erot[j];
                    s.vib[g] = v.vib[j];
                }
            }
        }
    }
    if (doSample) {
        for (int sp = 0; sp < cs.nSpecies; ++sp) {
            double a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0, a5 = 0, a6 = 0;
            for (int k = lane; k < n; k += 32) {
                const int j = v.perm[k];
                if ((v.spsub[j] >> 3) != sp) continue;
                const double ux = v.ux[j], uy = v.uy[j], uz = v.uz[j];
                a0 += 1.0;
                a1 += ux;
                a2 += uy;
                a3 += uz;
                a4 += ux * ux + uy * uy + uz * uz;
                a5 += v.erot[j];
                a6 += (double)v.vib[j];
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                a0 += __shfl_xor_sync(0xFFFFFFFFu, a0, o);
                a1 += __shfl_xor_sync(0xFFFFFFFFu, a1, o);
                a2 += __shfl_xor_sync(0xFFFFFFFFu, a2, o);
                a3 += __shfl_xor_sync(0xFFFFFFFFu, a3, o);
                a4 += __shfl_xor_sync(0xFFFFFFFFu, a4, o);
                a5 += __shfl_xor_sync(0xFFFFFFFFu, a5, o);
                a6 += __shfl_xor_sync(0xFFFFFFFFu, a6, o);
            }
            if (lane < SACC && a0 > 0.0) {
                const double val = lane == 0 ? a0 : lane == 1 ? a1 : lane == 2 ? a2 : lane == 3 ? a3
                                 : lane == 4 ? a4 : lane == 5 ? a5 : a6;
                acc[(sp * SACC + lane) * cs.C + c] += val;
            }
        }
    }
    __syncwarp();
}

// Cells above BIGN parcels (or tiles beyond the shared-memory capacity): one
// warp per cell with its staging arrays in a slot-indexed global scratch.
__global__ void __launch_bounds__(CWARPS * 32)
k_collide_big(CaseDev cs, Soa s, const int* __restrict__ start, double* smax, double* rem, double* acc,
              Counters* ctr, const int* __restrict__ bigList, Soa stageSoa, int* permS, int* sclS,
              unsigned char* dirtyS, int doCollide, int doSample) {
    __shared__ int subStartS[CWARPS][9];
    const int w = threadIdx.x >> 5;
    const uint32_t step = (uint32_t)ctr->step;
    const int nBig = ctr->bigCells;
    unsigned err = 0;
    unsigned long long nColl = 0, nCand = 0;
    const long long nWarps = (long long)gridDim.x * CWARPS;
    for (long long q = (long long)blockIdx.x * CWARPS + w; q < nBig; q += nWarps) {
        const long long c = bigList[q];
        const int off = start[c];
        const int n = start[c + 1] - off;
        // spsub shares the byte array of the cell word scratch
        StageView v{stageSoa.id + off, permS + off, sclS + off, stageSoa.ux + off, stageSoa.uy + off,
                    stageSoa.uz + off, stageSoa.erot + off, stageSoa.vib + off,
                    reinterpret_cast<unsigned char*>(stageSoa.cellw) + off, dirtyS + off};
        process_cell(cs, s, c, off, n, v, subStartS[w], smax, rem, acc, step, doCollide, doSample, &err,
                     &nColl, &nCand);
    }
    if (lane_id() == 0) {
        if (nColl) atomicAdd(&ctr->coll, nColl);
        if (nCand) atomicAdd(&ctr->cand, nCand);
        if (err) atomicOr(&ctr->err, err);
    }
}

// ---------------------------------------------------------------- tiles
// A warp takes 32 consecutive cells (one per lane).  Their parcels are one
// contiguous slot range; ids and sub-cell/species bytes are staged in shared
// memory with coalesced loads, then every lane orders its own cell by id,
// runs its cell's serial NTC loop and sums its cell's samples.  Serial work
// is spread across lanes, so FP64 instructions run 32 lanes wide.
constexpr int TCAP = 2048;     // staged parcels per warp tile
constexpr int TWARPS = 4;      // warps per block
constexpr int BIGN = 192;      // cells above this go to the warp-per-cell path

struct TileStage {
    uint32_t id[TCAP];
    unsigned char perm[TCAP];   // within-cell canonical order (n <= BIGN < 256)
    unsigned char spsub[TCAP];  // species << 3 | sub-cell
};

// r-th parcel (canonical order) of sub-cell sb
__device__ __forceinline__ int nth_in_sub(const unsigned char* perm, const unsigned char* spsub, int n, int sb,
                                          int r) {
    for (int k = 0; k < n; ++k) {
        if ((spsub[perm[k]] & 7) == sb) {
            if (r == 0) return k;
            --r;
        }
    }
    return 0;
}

// noTimeCounter::collide for one cell, run by one lane on global state.
__device__ void ntc_lane(const CaseDev& cs, const Soa& s, long long c, long long off, int n,
                         const unsigned char* perm, const unsigned char* spsub, const int subCnt[8],
                         double* smax, double* acc, uint32_t step, long long nCand, double smax0, unsigned* err,
                         unsigned long long* nColl) {
    Rng r(cs, (uint32_t)c, step, TAG_COLLIDE);
    double smaxRun = smax0;
    unsigned long long coll = 0;
    double collSep = 0.0;
    for (long long k = 0; k < nCand; ++k) {
        const int iP = r.label(0, n - 1, err);
        const int jP = perm[iP];
        const int sub = spsub[jP] & 7;
        const int nSC = subCnt[sub];
        int iQ = -1, it = 0;
        if (nSC > 1) {
            do { iQ = nth_in_sub(perm, spsub, n, sub, r.label(0, nSC - 1, err)); }
            while (iP == iQ && ++it < MAX_REJECTION);
        } else {
            do { iQ = r.label(0, n - 1, err); } while (iP == iQ && ++it < MAX_REJECTION);
        }
        if (it >= MAX_REJECTION) { *err |= ERRB_REJECTION; continue; }
        const int jQ = perm[iQ];
        const long long gP = off + jP, gQ = off + jQ;
        const int tP = spsub[jP] >> 3, tQ = spsub[jQ] >> 3;
        const PairDev& pr = cs.pair[tP * DSMC_MAX_SPECIES + tQ];
        double UP[3] = {s.ux[gP], s.uy[gP], s.uz[gP]};
        double UQ[3] = {s.ux[gQ], s.uy[gQ], s.uz[gQ]};
        const double d0 = UP[0] - UQ[0], d1 = UP[1] - UQ[1], d2 = UP[2] - UQ[2];
        const double cr2 = d0 * d0 + d1 * d1 + d2 * d2;
        const double sigma = sigma_cr(pr, cr2);
        if (sigma > smaxRun) smaxRun = sigma;
        if (sigma > r.u01() * smax0) {      // (sigma/smax0) > U with smax0 > 0
            double cR;
            if (cs.collModel == DSMC_COLL_LB_VHS) {
                double Et = 0.5 * pr.mR * cr2;
                double eP = s.erot[gP], eQ = s.erot[gQ];
                int vP = s.vib[gP], vQ = s.vib[gQ];
                redistribute(cs, cs.sp[tP], &eP, &vP, Et, pr.omegaPQ, r, zv_row(cs, tP, tQ), err);
                redistribute(cs, cs.sp[tQ], &eQ, &vQ, Et, pr.omegaPQ, r, zv_row(cs, tQ, tP), err);
                s.erot[gP] = eP; s.erot[gQ] = eQ;
                s.vib[gP] = vP; s.vib[gQ] = vQ;
                cR = sqrt(2.0 * Et / pr.mR);
            } else {
                cR = sqrt(cr2);
            }
            double Ucm[3];
            for (int a = 0; a < 3; ++a) Ucm[a] = pr.mPfrac * UP[a] + pr.mQfrac * UQ[a];
            const double cosT = 2.0 * r.u01() - 1.0;
            const double sinT = sqrt(1.0 - cosT * cosT);
            const double phi = 2.0 * PI * r.u01();
            double sph, cph;
            sincos(phi, &sph, &cph);
            const double prel[3] = {cR * cosT, cR * sinT * cph, cR * sinT * sph};
            s.ux[gP] = Ucm[0] + prel[0] * pr.mQfrac;
            s.uy[gP] = Ucm[1] + prel[1] * pr.mQfrac;
            s.uz[gP] = Ucm[2] + prel[2] * pr.mQfrac;
            s.ux[gQ] = Ucm[0] - prel[0] * pr.mPfrac;
            s.uy[gQ] = Ucm[1] - prel[1] * pr.mPfrac;
            s.uz[gQ] = Ucm[2] - prel[2] * pr.mPfrac;
            const double dx = s.x[gP] - s.x[gQ];
            const double dy = s.y[gP] - s.y[gQ];
            const double dz = s.z[gP] - s.z[gQ];
            collSep += sqrt(dx * dx + dy * dy + dz * dz);
            ++coll;
        }
    }
    smax[c] = smaxRun;
    if (coll) {
        acc[(cs.nSpecies * SACC + CACC_NCOLLS) * cs.C + c] += (double)coll;
        acc[(cs.nSpecies * SACC + CACC_COLLSEP) * cs.C + c] += collSep;
    }
    *nColl += coll;
}

__global__ void __launch_bounds__(TWARPS * 32)
k_collide_tile(CaseDev cs, Soa s, const int* __restrict__ start, double* smax, double* rem, double* acc,
               Counters* ctr, int* bigList, int doCollide, int doSample) {
    extern __shared__ unsigned char smraw[];
    TileStage& st = reinterpret_cast<TileStage*>(smraw)[threadIdx.x >> 5];
    const unsigned lane = lane_id();
    const uint32_t step = (uint32_t)ctr->step;
    unsigned err = 0;
    unsigned long long nColl = 0, nCand = 0;
    const long long nTiles = (cs.C + 31) / 32;
    const long long nWarps = (long long)gridDim.x * TWARPS;
    for (long long t = (long long)blockIdx.x * TWARPS + (threadIdx.x >> 5); t < nTiles; t += nWarps) {
        const long long c0 = t * 32;
        const long long cEnd = (c0 + 32 < cs.C) ? c0 + 32 : cs.C;
        const long long c = c0 + lane;
        const bool valid = c < cEnd;
        const int P0 = start[c0];
        const int P1 = start[cEnd];
        const int myStart = valid ? start[c] : P1;
        const int n = valid ? start[c + 1] - myStart : 0;
        const bool fits = (P1 - P0) <= TCAP;
        const bool big = n > BIGN || (!fits && n > 0);
        if (big) {
            const int idx = atomicAdd(&ctr->bigCells, 1);
            bigList[idx] = (int)c;
        }
        if (fits) {
            for (int p = lane; p < P1 - P0; p += 32) {
                const long long g = (long long)P0 + p;
                st.id[p] = s.id[g];
                st.spsub[p] = (unsigned char)((s.spc[g] << 3) | (s.cellw[g] & 7u));
            }
        }
        __syncwarp();
        if (fits && !big && n > 0) {
            const int b = myStart - P0;
            uint32_t* id = st.id + b;
            unsigned char* perm = st.perm + b;
            const unsigned char* spsub = st.spsub + b;
            // insertion sort of the cell's local indices by particle id
            perm[0] = 0;
            for (int k = 1; k < n; ++k) {
                const uint32_t key = id[k];
                int m = k - 1;
                while (m >= 0 && id[perm[m]] > key) {
                    perm[m + 1] = perm[m];
                    --m;
                }
                perm[m + 1] = (unsigned char)k;
            }
            if (doCollide && n > 1) {
                const double smax0 = smax[c];
                const double sel = rem[c] + 0.5 * n * (n - 1) * cs.FN * smax0 * cs.dt / cs.V;
                const long long nc = (long long)sel;
                rem[c] = sel - (double)nc;
                if (nc > 0) {
                    int subCnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                    for (int j = 0; j < n; ++j) subCnt[spsub[j] & 7]++;
                    ntc_lane(cs, s, c, myStart, n, perm, spsub, subCnt, smax, acc, step, nc, smax0, &err, &nColl);
                    nCand += (unsigned long long)nc;
                }
            }
            if (doSample) {
                // counts and vibrational levels are integers: summed on the
                // integer pipe; 7 FP64 operations per parcel remain
                for (int sp = 0; sp < cs.nSpecies; ++sp) {
                    double a1 = 0, a2 = 0, a3 = 0, a4 = 0, a5 = 0;
                    int a0 = 0, a6 = 0;
                    for (int k = 0; k < n; ++k) {
                        const int j = perm[k];
                        if ((spsub[j] >> 3) != sp) continue;
                        const long long g = (long long)myStart + j;
                        const double ux = s.ux[g], uy = s.uy[g], uz = s.uz[g];
                        a0 += 1;
                        a1 += ux;
                        a2 += uy;
                        a3 += uz;
                        a4 = fma(ux, ux, fma(uy, uy, fma(uz, uz, a4)));
                        a5 += s.erot[g];
                        a6 += s.vib[g];
                    }
                    if (a0 > 0) {
                        const long long C = cs.C;
                        double* A = acc + (long long)sp * SACC * C + c;
                        A[SACC_N * C] += (double)a0;
                        A[SACC_UX * C] += a1;
                        A[SACC_UY * C] += a2;
                        A[SACC_UZ * C] += a3;
                        A[SACC_UU * C] += a4;
                        A[SACC_EROT * C] += a5;
                        A[SACC_VIB * C] += (double)a6;
                    }
                }
            }
        }
        __syncwarp();
    }
    if (nColl) atomicAdd(&ctr->coll, nColl);
    if (nCand) atomicAdd(&ctr->cand, nCand);
    if (err) atomicOr(&ctr->err, err);
}

__global__ void k_zero_step(Counters* ctr) {
    ctr->nMoved = ctr->n;
    ctr->coll = 0;
    ctr->cand = 0;
    ctr->wallHits = 0;
    ctr->inserted = 0;
    ctr->deleted = 0;
    ctr->bigCells = 0;
    ctr->nSlow = 0;
}

// ---------------------------------------------------------------- fields
__global__ void k_field(CaseDev cs, const double* __restrict__ acc, const Counters* ctr, int which, double* out,
                        int measureMfp, double mfpTref) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cs.C) return;
    const double nT = (double)ctr->sampleSteps;
    const double FN = cs.FN, V = cs.V;
    const long long C = cs.C;
    // accumulator k of cell c lives at acc[k * C + c]
    auto A = [&](int k) { return acc[(long long)k * C + c]; };
    double N = 0, M = 0, mom[3] = {0, 0, 0}, mcc = 0, Er = 0, zr = 0;
    for (int s = 0; s < cs.nSpecies; ++s) {
        const double S[SACC] = {A(s * SACC + 0), A(s * SACC + 1), A(s * SACC + 2), A(s * SACC + 3),
                                A(s * SACC + 4), A(s * SACC + 5), A(s * SACC + 6)};
        const double m = cs.sp[s].m;
        N += S[SACC_N];
        M += m * S[SACC_N];
        mom[0] += m * S[SACC_UX];
        mom[1] += m * S[SACC_UY];
        mom[2] += m * S[SACC_UZ];
        mcc += m * S[SACC_UU];
        Er += S[SACC_EROT];
        zr += cs.sp[s].rotDof * S[SACC_N];
    }
    double rhoN = 0, rhoM = 0, Ux = 0, Uy = 0, Uz = 0, Ttra = 0;
    if (N > 1e-3 && nT > 0) {
        rhoN = N * FN / (nT * V);
        rhoM = M * FN / (nT * V);
        Ux = mom[0] / M;
        Uy = mom[1] / M;
        Uz = mom[2] / M;
        const double keMean = 0.5 * mcc * FN / (V * nT);
        Ttra = 2.0 / (3.0 * kB * rhoN) * (keMean - 0.5 * rhoM * (Ux * Ux + Uy * Uy + Uz * Uz));
    }
    const double zetaRotTot = N > SMALL ? zr / N : 0.0;
    const double Trot = zr > SMALL ? 2.0 * Er / (kB * zr) : 0.0;
    double Tvib = 0, zetaVib = 0, molRhoN = 0;
    for (int s = 0; s < cs.nSpecies; ++s) {
        const double S[SACC] = {A(s * SACC + 0), A(s * SACC + 1), A(s * SACC + 2), A(s * SACC + 3),
                                A(s * SACC + 4), A(s * SACC + 5), A(s * SACC + 6)};
        const SpeciesDev& sp = cs.sp[s];
        if (!sp.nVib) continue;
        const double Ev = sp.kThetaV * S[SACC_VIB];
        double zeta = 0, Ts = 0;
        if (Ev > VSMALL && S[SACC_N] > SMALL) {
            const double iMean = Ev / (sp.kThetaV * S[SACC_N]);
            if (iMean > SMALL) {
                const double lf = log(1.0 + 1.0 / iMean);
                Ts = sp.thetaV / lf;
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
    const double CA[CACC] = {A(cs.nSpecies * SACC + CACC_NCOLLS), A(cs.nSpecies * SACC + CACC_COLLSEP)};
    double v = 0;
    switch (which) {
    case F_RHON: v = rhoN; break;
    case F_RHOM: v = rhoM; break;
    case F_UX: v = Ux; break;
    case F_UY: v = Uy; break;
    case F_UZ: v = Uz; break;
    case F_TTRA: v = Ttra; break;
    case F_P: v = rhoN * kB * Ttra; break;
    case F_TROT: v = Trot; break;
    case F_TVIB: v = Tvib; break;
    case F_TOV: v = Tov; break;
    case F_NMEAN: v = (N > 1e-3 && nT > 0) ? N / nT : 0.001; break;
    case F_NCOLLS: v = CA[CACC_NCOLLS]; break;
    case F_MEASCR: v = (N > SMALL && nT > 0) ? CA[CACC_NCOLLS] * FN / (N * FN * cs.dt) : 0.0; break;
    case F_MEANCR:
    case F_MFP: {
        double mfp = 0, mcr = 0;
        if (Ttra > 1.0 && nT > 0) {
            for (int s = 0; s < cs.nSpecies; ++s) {
                double smfp = 0, smcr = 0;
                for (int q = 0; q < cs.nSpecies; ++q) {
                    const double Sq[1] = {A(q * SACC + SACC_N)};
                    const double dPQ = 0.5 * (cs.sp[s].d + cs.sp[q].d);
                    const double oPQ = 0.5 * (cs.sp[s].omega + cs.sp[q].omega);
                    const double mr = cs.sp[s].m / cs.sp[q].m;
                    if (Sq[SACC_N] > SMALL) {
                        const double nQ = Sq[SACC_N] * FN / (V * nT);
                        const double red = cs.sp[s].m * cs.sp[q].m / (cs.sp[s].m + cs.sp[q].m);
                        smfp += PI * dPQ * dPQ * nQ * pow(mfpTref / Ttra, oPQ - 0.5) * sqrt(1.0 + mr);
                        smcr += 2.0 * sqrt(PI) * dPQ * dPQ * nQ * pow(Ttra / mfpTref, 1.0 - oPQ) *
                                sqrt(2.0 * kB * mfpTref / red);
                    }
                }
                if (smfp > SMALL) smfp = 1.0 / smfp;
                const double rhoNi = A(s * SACC + SACC_N) * FN;
                mfp += smfp * rhoNi / (N * FN);
                mcr += smcr * rhoNi / (N * FN);
            }
            if (mfp < SMALL) mfp = GREAT;
        } else {
            mfp = GREAT;
        }
        v = (which == F_MFP) ? mfp : mcr;
        break;
    }
    default: v = 0.0;
    }
    (void)measureMfp;
    out[c] = v;
}

// Totals for dsmcCloud::info: KE, Erot, Evib, momentum (times FN on the host).
__global__ void k_info(CaseDev cs, Soa s, const Counters* ctr, double* out) {
    const long long n = ctr->n;
    double v[6] = {0, 0, 0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const SpeciesDev& sp = cs.sp[s.spc[i]];
        const double ux = s.ux[i], uy = s.uy[i], uz = s.uz[i];
        v[0] += 0.5 * sp.m * (ux * ux + uy * uy + uz * uz);
        v[1] += s.erot[i];
        v[2] += sp.nVib ? s.vib[i] * sp.kThetaV : 0.0;
        v[3] += sp.m * ux;
        v[4] += sp.m * uy;
        v[5] += sp.m * uz;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xFFFFFFFFu, v[k], o);
    }
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 6; ++k) atomicAdd(out + k, v[k]);
    }
}

int sm_count() {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

}  // namespace

void launch_collide_sample(const CaseDev& cs, const StepBuffers& B, const Soa& s, int doCollide, int doSample,
                           cudaStream_t st) {
    static bool attrSet = false;
    const int smem = (int)sizeof(TileStage) * TWARPS;
    if (!attrSet) {
        cudaFuncSetAttribute(k_collide_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attrSet = true;
    }
    const long long tiles = (cs.C + 31) / 32;
    long long blocks = (tiles + TWARPS - 1) / TWARPS;
    const long long cap = (long long)sm_count() * 4;
    if (blocks > cap) blocks = cap;
    k_collide_tile<<<(int)blocks, TWARPS * 32, smem, st>>>(cs, s, B.start, B.smax, B.rem, B.acc, B.ctr, B.bigList,
                                                          doCollide, doSample);
    k_collide_big<<<sm_count() * 2, CWARPS * 32, 0, st>>>(cs, s, B.start, B.smax, B.rem, B.acc, B.ctr,
                                                          B.bigList, B.stage, B.perm, B.scl, B.dirty,
                                                          doCollide, doSample);
}

void launch_zero_step(const StepBuffers& B, cudaStream_t st) { k_zero_step<<<1, 1, 0, st>>>(B.ctr); }

void launch_field(const CaseDev& cs, const StepBuffers& B, int which, double* out, int measureMfp,
                  double mfpTref, cudaStream_t st) {
    k_field<<<(int)((cs.C + 255) / 256), 256, 0, st>>>(cs, B.acc, B.ctr, which, out, measureMfp, mfpTref);
}

void launch_info(const CaseDev& cs, const Soa& s, const Counters* ctr, double* out6, cudaStream_t st) {
    cudaMemsetAsync(out6, 0, sizeof(double) * 6, st);
    k_info<<<sm_count() * 4, 256, 0, st>>>(cs, s, ctr, out6);
}

}  // namespace dsmc
