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
// The collision kernels themselves are in dsmc_tile.cuh; this file holds the
// Larsen-Borgnakke samplers they use, the output-time fields and the cloud
// totals.

#include "dsmc_kernels.h"

namespace dsmc {

namespace {




// postCollisionRotationalEnergy (dsmcCloud.C:1327-1387): the fraction of
// the collision energy that goes to rotation.  Energy is conserved by the
// caller (the translational part is the remainder), so the fraction only
// needs its distribution: it is drawn in FP32 (an FP64 pow costs tens of
// FP64 instructions, which on this part issue over the whole warp).
__device__ __forceinline__ double post_rot(Rng& r, double dof, const PairDev& pr, unsigned* err) {
    if (dof == 2.0) return 1.0 - (double)powf((float)r.u01(), pr.invChiBF);
    const float ChiA = (float)(0.5 * dof);
    const float A1 = ChiA - 1.f, B1 = pr.chiBF - 1.f;
    if (A1 < (float)SMALL && B1 < (float)SMALL) return r.u01();
    for (int it = 0; it < MAX_REJECTION; ++it) {
        const double ratio = r.u01();
        const float rf = (float)ratio;
        float Pr;
        if (A1 < (float)SMALL) Pr = powf(1.f - rf, B1);
        else if (B1 < (float)SMALL) Pr = powf(1.f - rf, A1);
        else Pr = powf((A1 + B1) * rf / A1, A1) * powf((A1 + B1) * (1.f - rf) / B1, B1);
        if (!((double)Pr < r.u01())) return ratio;
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
        for (int it = 0; it < cs.maxRejection; ++it) {
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
                                             double& Et, const PairDev& pr, Rng& r, const double* tab,
                                             unsigned* err) {
    const double omegaPQ = pr.omegaPQ;
    if (s.nVib > 0) {
        const double EcP = Et + *vib * s.kThetaV;
        const int iMax = (int)(EcP * s.invKThetaV);
        if (iMax > 0) {
            *vib = post_vib(cs, r, *vib, iMax, s, omegaPQ, EcP, tab, err);
            Et = EcP - *vib * s.kThetaV;
        }
    }
    if (s.rotDof > 0) {
        const double pre = *erot;
        if (cs.invZrot > r.u01()) {
            const double EcP = Et + pre;
            const double ratio = post_rot(r, s.rotDof, pr, err);
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
    if (!(cr2 > 0.0)) return 0.0;      // sqrt(cr2) < VSMALL only for cr2 == 0
    return (double)(pr.sigmaPrefactorF * powf((float)cr2, pr.expoF));
}

#include "dsmc_tile.cuh"

__global__ void k_zero_step(Counters* ctr) {
    ctr->nMoved = ctr->n;
    ctr->coll = 0;
    ctr->cand = 0;
    ctr->wallHits = 0;
    ctr->inserted = 0;
    ctr->deleted = 0;
    ctr->bigCells = 0;
    ctr->nSlow = 0;
    ctr->nWork = 0;
    ctr->nHeavy = 0;
    ctr->nMig = 0;
    ctr->migIn = 0;
    ctr->inflowLocal = 0;
}

// ---------------------------------------------------------------- moments
// One thread per cell: the cell's parcels (contiguous after the sort) summed
// species by species as exact fixed-point integers, so the step's sums do not
// depend on the parcels' order in the cell, then added to the FP64
// accumulators in step order (reproducible bit for bit).
constexpr int F_MUU = 14;   // u_i u_j: resolution 6.1e-5 m^2/s^2
constexpr int F_MCCU = 4;   // |U|^2 u_i: resolution 0.0625 m^3/s^3
constexpr int F_MEU = 90;   // E_int u_i: resolution 8.1e-28 J m/s

__global__ void k_sample_moments(CaseDev cs, Parcels s, const int* __restrict__ start, double* macc,
                                 Counters* ctr) {
    const long long C = cs.C;
    unsigned err = 0;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < C;
         c += (long long)gridDim.x * blockDim.x) {
        const int j0 = start[c], j1 = start[c + 1];
        if (j1 <= j0) continue;
        for (int sp = 0; sp < cs.nSpecies; ++sp) {
            long long m[MACC];
#pragma unroll
            for (int k = 0; k < MACC; ++k) m[k] = 0;
            int any = 0;
            for (int j = j0; j < j1; ++j) {
                const Rec p = ldg_rec(s.r + j);
                if (sv_species(p.sv) != sp) continue;
                any = 1;
                const double u = p.ux, v = p.uy, w = p.uz;
                const double cc = u * u + v * v + w * w;
                const double E = p.erot + (double)sv_vib(p.sv) * cs.sp[sp].kThetaV;
                m[MACC_UU] += fixp(u * u, F_MUU, &err);
                m[MACC_UV] += fixp(u * v, F_MUU, &err);
                m[MACC_UW] += fixp(u * w, F_MUU, &err);
                m[MACC_VV] += fixp(v * v, F_MUU, &err);
                m[MACC_VW] += fixp(v * w, F_MUU, &err);
                m[MACC_WW] += fixp(w * w, F_MUU, &err);
                m[MACC_CCU] += fixp(cc * u, F_MCCU, &err);
                m[MACC_CCV] += fixp(cc * v, F_MCCU, &err);
                m[MACC_CCW] += fixp(cc * w, F_MCCU, &err);
                m[MACC_EU] += fixp(E * u, F_MEU, &err);
                m[MACC_EV] += fixp(E * v, F_MEU, &err);
                m[MACC_EW] += fixp(E * w, F_MEU, &err);
            }
            if (!any) continue;
#pragma unroll
            for (int k = 0; k < MACC; ++k) {
                const int F = k < MACC_CCU ? F_MUU : k < MACC_EU ? F_MCCU : F_MEU;
                macc[(long long)(sp * MACC + k) * C + c] += ldexp((double)m[k], -F);
            }
        }
    }
    if (err) atomicOr(&ctr->err, err);
}

// ---------------------------------------------------------------- fields
// Species outside mask are left out of every sum (a dsmcVolFields typeIds
// subset, dsmcVolFields.C:841).
__global__ void k_field(CaseDev cs, const double* __restrict__ acc, const double* __restrict__ macc,
                        const Counters* ctr, int which, double* out, int measureMfp, double mfpTref, unsigned mask) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cs.C) return;
    const double nT = (double)ctr->sampleSteps;
    const double FN = cs.FN, V = cell_volume(cs, c);
    const long long C = cs.C;
    // accumulator k of cell c lives at acc[k * C + c]
    auto A = [&](int k) { return acc[(long long)k * C + c]; };
    double N = 0, M = 0, mom[3] = {0, 0, 0}, mcc = 0, Er = 0, zr = 0;
    for (int s = 0; s < cs.nSpecies; ++s) {
        if (!((mask >> s) & 1u)) continue;
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
        if (!sp.nVib || !((mask >> s) & 1u)) continue;
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
                if (!((mask >> s) & 1u)) continue;
                double smfp = 0, smcr = 0;
                for (int q = 0; q < cs.nSpecies; ++q) {
                    if (!((mask >> q) & 1u)) continue;
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
    case F_MA:
    case F_RHOM_ERR:
    case F_U_ERR:
    case F_T_ERR:
    case F_P_ERR: {
        // dsmcVolFields.C:1625-1661 (Mach number from the trans-rotational
        // gamma of the mixture) and :1859-1873 (statistical error estimates)
        double Ma = 0.0, gamma = 0.0, particleCv = 0.0;
        if (N > SMALL && Ttra > SMALL) {
            double molarCv = 0.0, molarCp = 0.0, mMol = 0.0;
            for (int s = 0; s < cs.nSpecies; ++s) {
                if (!((mask >> s) & 1u)) continue;
                const double Xs = A(s * SACC + SACC_N) / N;
                mMol += Xs * cs.sp[s].m;
                molarCv += Xs * (3.0 + cs.sp[s].rotDof);
                molarCp += Xs * (5.0 + cs.sp[s].rotDof);
            }
            particleCv = molarCv / NAVO;
            gamma = molarCp / molarCv;
            Ma = sqrt(Ux * Ux + Uy * Uy + Uz * Uz) / sqrt(gamma * kB / mMol * Ttra);
        }
        if (which == F_MA) {
            v = Ma;
            break;
        }
        const double nMean = (N > 1e-3 && nT > 0) ? N / nT : 0.001;
        v = 0.0;
        if (nMean > SMALL && Ma > SMALL && gamma > SMALL && particleCv > SMALL) {
            const double deno = sqrt(nMean * nT);
            if (which == F_RHOM_ERR) v = 1.0 / deno;
            else if (which == F_U_ERR) v = 1.0 / (deno * Ma * sqrt(gamma));
            else if (which == F_T_ERR) v = sqrt(kB / particleCv) / deno;
            else v = sqrt(gamma) / deno;
        }
        break;
    }
    default:
        if (which >= F_PXX && which <= F_QZ && macc && N > SMALL && nT > 0) {
            // dsmcVolFields.C:1511-1607: pressure tensor, shear stress tensor
            // (pressure tensor minus its trace part, negated) and heat flux
            double Muu[6] = {0, 0, 0, 0, 0, 0}, Mccu[3] = {0, 0, 0}, Eu[3] = {0, 0, 0}, E = Er;
            for (int s = 0; s < cs.nSpecies; ++s) {
                if (!((mask >> s) & 1u)) continue;
                const double m = cs.sp[s].m;
                auto Q = [&](int k) { return macc[(long long)(s * MACC + k) * C + c]; };
                for (int k = 0; k < 6; ++k) Muu[k] += m * Q(MACC_UU + k);
                for (int k = 0; k < 3; ++k) {
                    Mccu[k] += m * Q(MACC_CCU + k);
                    Eu[k] += Q(MACC_EU + k);
                }
                E += cs.sp[s].kThetaV * A(s * SACC + SACC_VIB);
            }
            const double U[3] = {Ux, Uy, Uz};
            const double f = rhoN / N;
            // symmetric tensor in xx xy xz yy yz zz order
            const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
            double P[6];
            for (int k = 0; k < 6; ++k) P[k] = f * (Muu[k] - M * U[ia[k]] * U[ib[k]]);
            if (which <= F_PZZ) {
                v = P[which - F_PXX];
            } else if (which <= F_SZZ) {
                const int k = which - F_SXX;
                const double sp = (P[0] + P[3] + P[5]) / 3.0;
                v = -P[k] + (ia[k] == ib[k] ? sp : 0.0);
            } else {
                const int i = which - F_QX;
                // row i of the (symmetric) pressure tensor
                const int row[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
                v = f * (0.5 * Mccu[i] - 0.5 * mcc * U[i] + Eu[i] - E * U[i]) - P[row[i][0]] * U[0] -
                    P[row[i][1]] * U[1] - P[row[i][2]] * U[2];
            }
        } else {
            v = 0.0;
        }
    }
    (void)measureMfp;
    out[c] = v;
}

// Totals for dsmcCloud::info: KE, Erot, Evib, momentum (times FN on the host).
__global__ void k_info(CaseDev cs, Parcels s, const Counters* ctr, double* out) {
    const long long n = ctr->n;
    double v[6] = {0, 0, 0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const Rec p = ldg_rec(s.r + i);
        const SpeciesDev& sp = cs.sp[sv_species(p.sv)];
        const double ux = p.ux, uy = p.uy, uz = p.uz;
        v[0] += 0.5 * sp.m * (ux * ux + uy * uy + uz * uz);
        v[1] += p.erot;
        v[2] += sp.nVib ? sv_vib(p.sv) * sp.kThetaV : 0.0;
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

// ------------------------------------------------------- learned maximum
// Features of the learned maximum: log number density, log translational
// temperature and speed ratio |U| / sqrt(2 k T / m) (m the mean parcel mass)
// of each cell's parcels.  A CTA takes a tile of FEAT_TILE consecutive cells,
// whose parcels are contiguous after the sort, and streams them warp by warp
// with coalesced loads; each parcel's exact fixed-point values (mass weight:
// the species mass over species 0's in units of 1/256; velocities in units
// of 1/16 m/s) are summed over the warp's runs of equal cells and added to
// the cell's sums in shared memory by the run's last lane, so the sums do
// not depend on the parcels' order.  (Every parcel adding to shared memory
// itself measured 1.44 ms for the 13.1M-parcel heat bath: twenty-odd lanes
// of a warp contend for one cell's 64-bit sums.)  Then one thread per cell
// makes the features.
constexpr int FEAT_TILE = 256;

__global__ void __launch_bounds__(FEAT_TILE)
k_cell_features(CaseDev cs, Parcels s, const int* __restrict__ start, const Counters* ctr, int every, float4* feat,
                unsigned char* useR, float* exceed, float forget) {
    if (every > 0 && (ctr->step % every) != 0) return;
    __shared__ int sN[FEAT_TILE];
    __shared__ unsigned long long sW[FEAT_TILE], sWU[3][FEAT_TILE], sWUU[FEAT_TILE];
    const float kOverM0 = (float)(kB / cs.sp[0].m);
    const float ndScaleU = (float)(cs.FN / cs.V);
    int mw[DSMC_MAX_SPECIES];
#pragma unroll
    for (int q = 0; q < DSMC_MAX_SPECIES; ++q) mw[q] = q < cs.nSpecies ? __float2int_rn(cs.mRel[q] * 256.f) : 0;
    const long long nTiles = (cs.C + FEAT_TILE - 1) / FEAT_TILE;
    for (long long tile = blockIdx.x; tile < nTiles; tile += gridDim.x) {
        const long long c0 = tile * FEAT_TILE;
        const long long c1 = c0 + FEAT_TILE < cs.C ? c0 + FEAT_TILE : cs.C;
        const int t = threadIdx.x;
        sN[t] = 0;
        sW[t] = 0ull;
        sWU[0][t] = sWU[1][t] = sWU[2][t] = 0ull;
        sWUU[t] = 0ull;
        __syncthreads();
        const long long j0 = start[c0], j1 = start[c1];
        const int lane = t & 31;
        for (long long jb = j0 + (t & ~31); jb < j1; jb += FEAT_TILE) {
            const long long j = jb + lane;
            int lc = -1;
            long long v[5] = {0, 0, 0, 0, 0};
            if (j < j1) {
                lc = (int)((long long)cellw_cell(__ldg(s.cellw + j)) - c0);
                if ((unsigned)lc >= (unsigned)FEAT_TILE) lc = -1;   // never: the tile's parcels are its cells'
            }
            if (lc >= 0) {
                const double2* q = reinterpret_cast<const double2*>(s.r + j);
                const double2 b = __ldg(q + 1), d = __ldg(q + 2), e = __ldg(q + 3);
                const uint32_t sv = (uint32_t)((unsigned long long)__double_as_longlong(e.y) >> 32);
                const long long w = mw[sv_species(sv) & (DSMC_MAX_SPECIES - 1)];
                const long long ux = __double2ll_rn(b.y * 16.0), uy = __double2ll_rn(d.x * 16.0),
                                uz = __double2ll_rn(d.y * 16.0);
                v[0] = w;
                v[1] = w * ux;
                v[2] = w * uy;
                v[3] = w * uz;
                v[4] = w * (ux * ux + uy * uy + uz * uz);
            }
            // the warp's runs of equal cells (the parcels are sorted by cell)
            const int prev = __shfl_up_sync(0xFFFFFFFFu, lc, 1);
            const unsigned hm = __ballot_sync(0xFFFFFFFFu, lane == 0 || prev != lc);
            const int segStart = 31 - __clz(hm & (0xFFFFFFFFu >> (31 - lane)));
#pragma unroll
            for (int k = 0; k < 5; ++k) v[k] = seg_sum(v[k], segStart);
            const bool tail = lane == 31 || ((hm >> (lane + 1)) & 1u);
            if (tail && lc >= 0) {
                atomicAdd(&sN[lc], lane - segStart + 1);
                atomicAdd(&sW[lc], (unsigned long long)v[0]);
                atomicAdd(&sWU[0][lc], (unsigned long long)v[1]);
                atomicAdd(&sWU[1][lc], (unsigned long long)v[2]);
                atomicAdd(&sWU[2][lc], (unsigned long long)v[3]);
                atomicAdd(&sWUU[lc], (unsigned long long)v[4]);
            }
        }
        __syncthreads();
        const long long c = c0 + t;
        if (c < c1) {
            const int n = sN[t];
            float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
            if (n >= 2) {
                const float M = (float)(long long)sW[t] * (1.f / 256.f);
                const float Mu0 = (float)(long long)sWU[0][t] * (1.f / 4096.f);
                const float Mu1 = (float)(long long)sWU[1][t] * (1.f / 4096.f);
                const float Mu2 = (float)(long long)sWU[2][t] * (1.f / 4096.f);
                const float Muu = (float)(long long)sWUU[t] * (1.f / 65536.f);
                const float U2 = (Mu0 * Mu0 + Mu1 * Mu1 + Mu2 * Mu2) / (M * M);
                // T = m0 (sum m_rel u^2 - M U^2) / (3 k n)
                const float T = (Muu - M * U2) / (3.0f * kOverM0 * (float)n);
                if (T > 0.f) {
                    const float ndScale = cs.cellV ? (float)(cs.FN / cs.cellV[c]) : ndScaleU;
                    const float cmp = sqrtf(2.0f * kOverM0 * T / (M / (float)n));
                    f = make_float4(logf(ndScale * (float)n), logf(T), sqrtf(U2) / cmp, 1.f);
                }
            }
            feat[c] = f;
            if (useR) useR[c] = 0;
            if (exceed) exceed[c] *= forget;
        }
        __syncthreads();
    }
}

// (features, log observed maximum) of the cells that had candidates in the
// last step, compacted in any order
__global__ void k_learn_compact(CaseDev cs, const int* __restrict__ ncCell, const float4* __restrict__ feat,
                                const float* __restrict__ obsMax, long long maxRows, float* X, float* Y,
                                unsigned long long* nOut) {
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < cs.C;
         c += (long long)gridDim.x * blockDim.x) {
        const float4 f = feat[c];
        const float o = obsMax[c];
        if (ncCell[c] <= 0 || f.w == 0.f || !(o > 0.f)) continue;
        const unsigned long long q = atomicAdd(nOut, 1ull);
        if ((long long)q >= maxRows) continue;
        X[3 * q] = f.x;
        X[3 * q + 1] = f.y;
        X[3 * q + 2] = f.z;
        Y[q] = logf(o);
    }
}

// ---------------------------------------------------------------- batch
// The collision half of a batched step for every case of a batch, in one
// persistent launch (phases separated by grid barriers, work items taken from
// per-phase tickets; see dsmc_persist.cuh).  The per-cell work is the
// single-case kernels' own (select_cell, list_iter, order_item, heavy_item,
// light_group), so a batched case collides exactly as it does alone.  Plain
// noTimeCounter selection only (no learned maximum, no selection audit); a
// cell above ORDER_WARP_N parcels is skipped with the dense-cell error (the
// slot's maxCellParcels is lowered to it).
#include "dsmc_persist.cuh"   // (no includes of its own: it sits in this namespace)

enum { BC_SELECT = 0, BC_BUCKETS, BC_LIST, BC_ORDER, BC_HEAVY, BC_LIGHT, BC_END, BC_NPHASE };
static_assert(BATCH_TICKETS_COLLIDE + BC_NPHASE <= BATCH_PHASES, "ticket counters of the collision launch");

constexpr int BC_MAX_THREADS = 128;

// dynamic shared memory: per warp its ordering keys and its light picks
__host__ __device__ constexpr size_t batch_collide_smem(int threads) {
    return (size_t)(threads / 32) * (tile::ORDER_WARP_N * sizeof(unsigned long long) + sizeof(tile::LightPicks));
}

// Phases [P0, P1) in one launch: selection, list and ordering; the heavy
// cells; the light cells and the end of the step, as three launches with
// their own phases' registers (the heavy cells' up to 170: at 128 they
// spill).
template <int P0, int P1>
__global__ void __launch_bounds__(BC_MAX_THREADS, P0 == BC_HEAVY ? 3 : 4)
k_batch_collide(const BatchSlot* __restrict__ slots, int n, BatchCtl* ctl) {
    extern __shared__ __align__(16) unsigned char bcSmem[];
    __shared__ long long pre[BATCH_MAX_CASES + 1];
    __shared__ unsigned hist[2 * tile::NBUCKET];
    const int T = blockDim.x;
    const int W = T >> 5;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    unsigned long long* keys =
        reinterpret_cast<unsigned long long*>(bcSmem) + (size_t)warp * tile::ORDER_WARP_N;
    tile::LightPicks& pk =
        reinterpret_cast<tile::LightPicks*>(bcSmem + (size_t)W * tile::ORDER_WARP_N * sizeof(unsigned long long))[warp];
#pragma unroll
    for (int ph = P0; ph < P1; ++ph) {
        long long total;
        switch (ph) {
        case BC_SELECT:
        case BC_LIST:
            total = persist::phase_items(n, pre, [&](int i) { return (slots[i].cs.C + T - 1) / T; });
            break;
        case BC_ORDER:
        case BC_HEAVY:
            total = persist::phase_items(n, pre, [&](int i) {
                return ((long long)slots[i].B.ctr->nHeavy + W - 1) / W;
            });
            break;
        case BC_LIGHT:
            total = persist::phase_items(n, pre, [&](int i) {
                const Counters* c = slots[i].B.ctr;
                return ((long long)(c->nWork - c->nHeavy) + T - 1) / T;
            });
            break;
        default:   // one item per case
            total = persist::phase_items(n, pre, [&](int) { return 1LL; });
        }
        const int tk = BATCH_TICKETS_COLLIDE + ph;
        for (long long q = persist::next_item(ctl, tk, total); q >= 0; q = persist::next_item(ctl, tk, total)) {
            const int ci = persist::item_case(pre, n, q);
            const long long l = q - pre[ci];
            const BatchSlot& sl = slots[ci];
            const CaseDev& cs = sl.cs;
            const StepBuffers& B = sl.B;
            const Parcels& s = sl.dst;      // the sorted buffer
            Counters* ctr = B.ctr;
            unsigned* slotCount = B.buckets;
            unsigned* slotCursor = B.buckets + 2 * tile::NBUCKET;
            unsigned err = 0;
            switch (ph) {
            case BC_SELECT: {
                if (tid < 2 * tile::NBUCKET) hist[tid] = 0;
                __syncthreads();
                const long long c = l * T + tid;
                if (c < cs.C) {
                    int nn;
                    const int nc = tile::select_cell(cs, B.start, B.smax, B.rem, 0, nullptr, nullptr, nullptr,
                                                     nullptr, c, &nn, err);
                    B.ncCell[c] = nc;
                    if (nc > 0) atomicAdd(&hist[tile::slot_of(nn, nc)], 1u);
                }
                __syncthreads();
                if (tid < 2 * tile::NBUCKET && hist[tid]) atomicAdd(&slotCount[tid], hist[tid]);
                break;
            }
            case BC_BUCKETS:
                if (tid == 0) {
                    unsigned off = 0;
                    for (int b = 2 * tile::NBUCKET - 1; b >= 0; --b) {
                        slotCursor[b] = off;
                        off += slotCount[b];
                        slotCount[b] = 0;
                        if (b == tile::NBUCKET) ctr->nHeavy = off;
                    }
                    ctr->nWork = off;
                }
                break;
            case BC_LIST:
                tile::list_iter(cs.C, B.start, B.ncCell, slotCursor, B.work, B.bigList, ctr, 0, l * T + tid);
                break;
            case BC_ORDER: {
                const long long qh = l * W + warp;
                if (qh < (long long)ctr->nHeavy) tile::order_item(s, B.start, B.work, B.perm, B.subs, qh, keys);
                break;
            }
            case BC_HEAVY: {
                const long long qh = l * W + warp;
                unsigned long long nColl = 0, nCand = 0;
                if (qh < (long long)ctr->nHeavy)
                    tile::heavy_item(cs, s, B.start, B.smax, B.acc, B.work, B.perm, B.subs, 0, nullptr, nullptr,
                                     nullptr, B.obsMax, nullptr, qh, (uint32_t)ctr->step, err, nColl, nCand);
                if (lane == 0) {
                    if (nColl) atomicAdd(&ctr->coll, nColl);
                    if (nCand) atomicAdd(&ctr->cand, nCand);
                }
                break;
            }
            case BC_LIGHT: {
                const long long nWork = (long long)ctr->nWork;
                const long long qb = (long long)ctr->nHeavy + l * T + warp * 32;
                unsigned long long nColl = 0, nCand = 0;
                if (qb < nWork)
                    tile::light_group(cs, s, B.start, B.smax, B.acc, B.work, 0, nullptr, nullptr, nullptr, B.obsMax,
                                      nullptr, qb, nWork, (uint32_t)ctr->step, pk, err, nColl, nCand);
                if (nColl) atomicAdd(&ctr->coll, nColl);
                if (nCand) atomicAdd(&ctr->cand, nCand);
                break;
            }
            case BC_END:
                if (tid == 0) {
                    ctr->pendingSample = 1;
                    ctr->collTot += ctr->coll;
                    ctr->candTot += ctr->cand;
                    ctr->bigCells = 0;
                    ctr->step += 1;
                }
                break;
            }
            if (err) atomicOr(&ctr->err, err);
        }
        if (ph + 1 < P1 && !persist::grid_sync(ctl)) return;
    }
}

template <int P0, int P1>
int batch_collide_grid_of(int threads) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_collide<P0, P1>, threads,
                                                      batch_collide_smem(threads)) != cudaSuccess)
        return 0;
    return per * sms;
}

template <int P0, int P1>
cudaError_t launch_batch_collide_part(const BatchSlot* slots, int n, BatchCtl* ctl, int threads, cudaStream_t st) {
    const int grid = batch_collide_grid_of<P0, P1>(threads);
    if (grid <= 0) return cudaErrorInvalidConfiguration;
    void* args[] = {(void*)&slots, (void*)&n, (void*)&ctl};
    return cudaLaunchCooperativeKernel((const void*)k_batch_collide<P0, P1>, dim3(grid), dim3(threads), args,
                                       batch_collide_smem(threads), st);
}

int sm_count() {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

}  // namespace

int collide_init() {
    const cudaError_t e = cudaFuncSetAttribute(tile::k_cell_order_big, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)(tile::ORDER_MAX_N * sizeof(unsigned long long)));
    return e == cudaSuccess ? 0 : (int)e;
}

// the smallest resident grid of the three launches (0: one cannot run)
int batch_collide_grid(int threads) {
    const int a = batch_collide_grid_of<BC_SELECT, BC_HEAVY>(threads);
    const int b = batch_collide_grid_of<BC_HEAVY, BC_LIGHT>(threads);
    const int c = batch_collide_grid_of<BC_LIGHT, BC_NPHASE>(threads);
    return std::min(a, std::min(b, c));
}

cudaError_t launch_batch_collide(const BatchSlot* slots, int n, BatchCtl* ctl, int threads, cudaStream_t st) {
    if (threads > BC_MAX_THREADS || threads < 32 || threads % 32) return cudaErrorInvalidConfiguration;
    cudaError_t e = launch_batch_collide_part<BC_SELECT, BC_HEAVY>(slots, n, ctl, threads, st);
    if (e == cudaSuccess) e = launch_batch_collide_part<BC_HEAVY, BC_LIGHT>(slots, n, ctl, threads, st);
    if (e == cudaSuccess) e = launch_batch_collide_part<BC_LIGHT, BC_NPHASE>(slots, n, ctl, threads, st);
    return e;
}

void launch_collide(const CaseDev& cs, const StepBuffers& B, const Parcels& s, int learned, cudaStream_t st,
                    cudaEvent_t* marks, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join) {
    const int sms = sm_count();
    long long selBlocks = (cs.C + 255) / 256;
    if (selBlocks > (long long)sms * 8) selBlocks = (long long)sms * 8;
    unsigned* slotCount = B.buckets;
    unsigned* slotCursor = B.buckets + 2 * tile::NBUCKET;
    const bool sbt = cs.selModel == DSMC_SEL_SBT;
    if (sbt)
        tile::k_sbt_select<<<(int)selBlocks, 256, 0, st>>>(cs, B.start, B.ctr, B.ncCell, slotCount);
    else
        tile::k_ntc_select<<<(int)selBlocks, 256, 0, st>>>(cs, B.start, B.smax, B.rem, B.ctr, B.ncCell, slotCount,
                                                            learned, B.pred, B.useR, B.exceed, B.smaxSel);
    tile::k_ntc_buckets<<<1, 1, 0, st>>>(B.ctr, slotCount, slotCursor);
    tile::k_ntc_list<<<(int)selBlocks, 256, 0, st>>>(cs.C, B.start, B.ncCell, slotCursor, B.work, B.bigList, B.ctr,
                                                      sbt ? 1 : 0);
    tile::k_cell_order<<<sms * 8, tile::WARPS * 32, 0, st>>>(s, B.start, B.ctr, B.work, B.perm, B.subs);
    tile::k_cell_order_big<<<sms, tile::ORDER_BLOCK, tile::ORDER_MAX_N * sizeof(unsigned long long), st>>>(
        s, B.start, B.ctr, B.work, B.bigList, B.perm, B.subs);
    if (marks) cudaEventRecord(marks[0], st);
    if (sbt) {
        tile::k_sbt_collide<<<sms * 4, tile::WARPS * 32, 0, st>>>(cs, s, B.start, B.acc, B.ctr, B.work, B.perm);
        if (marks) cudaEventRecord(marks[1], st);
        return;
    }
    // the heavy cells (their long tail: a few dense cells' warps) beside the
    // light cells when a side stream is given
    const bool branch = side && fork && join && !marks;
    cudaStream_t hs = st;
    if (branch) {
        cudaEventRecord(fork, st);
        cudaStreamWaitEvent(side, fork, 0);
        hs = side;
    }
    tile::k_collide_heavy<<<sms * 4, tile::WARPS * 32, 0, hs>>>(cs, s, B.start, B.smax, B.acc, B.ctr, B.work,
                                                                B.perm, B.subs, learned, B.smaxSel, B.useR,
                                                                B.exceed, B.obsMax, B.audit);
    if (branch) cudaEventRecord(join, side);
    if (marks) cudaEventRecord(marks[1], st);
    const int L = B.cfg.lightCells;
    tile::k_collide_light<<<sms * 4 * (128 / L), L, (L / 32) * (sizeof(tile::LightPicks) + sizeof(tile::LightDefer)),
                            st>>>(
        cs, s, B.start, B.smax, B.acc, B.ctr, B.work, learned, B.smaxSel, B.useR, B.exceed, B.obsMax, B.audit);
    if (branch) cudaStreamWaitEvent(st, join, 0);
}

void launch_cell_features(const CaseDev& cs, const StepBuffers& B, const Parcels& s, int every, int resetFallback,
                          cudaStream_t st, float forget) {
    long long blocks = (cs.C + FEAT_TILE - 1) / FEAT_TILE;
    if (blocks > (long long)sm_count() * 8) blocks = (long long)sm_count() * 8;
    k_cell_features<<<(int)blocks, FEAT_TILE, 0, st>>>(cs, s, B.start, B.ctr, every, B.feat,
                                                       resetFallback ? B.useR : nullptr,
                                                       resetFallback && forget < 1.f ? B.exceed : nullptr, forget);
}

void launch_learn_compact(const CaseDev& cs, const StepBuffers& B, long long maxRows, float* X, float* Y,
                          unsigned long long* nOut, cudaStream_t st) {
    long long blocks = (cs.C + 255) / 256;
    if (blocks > (long long)sm_count() * 16) blocks = (long long)sm_count() * 16;
    cudaMemsetAsync(nOut, 0, sizeof(unsigned long long), st);
    k_learn_compact<<<(int)blocks, 256, 0, st>>>(cs, B.ncCell, B.feat, B.obsMax, maxRows, X, Y, nOut);
}

void launch_zero_step(const StepBuffers& B, cudaStream_t st) { k_zero_step<<<1, 1, 0, st>>>(B.ctr); }

void launch_field(const CaseDev& cs, const StepBuffers& B, int which, double* out, int measureMfp,
                  double mfpTref, unsigned mask, cudaStream_t st) {
    k_field<<<(int)((cs.C + 255) / 256), 256, 0, st>>>(cs, B.acc, B.macc, B.ctr, which, out, measureMfp, mfpTref,
                                                       mask);
}

void launch_sample_moments(const CaseDev& cs, const StepBuffers& B, const Parcels& s, cudaStream_t st) {
    long long blocks = (cs.C + 255) / 256;
    if (blocks > (long long)sm_count() * 16) blocks = (long long)sm_count() * 16;
    k_sample_moments<<<(int)blocks, 256, 0, st>>>(cs, s, B.start, B.macc, B.ctr);
}

void launch_info(const CaseDev& cs, const Parcels& s, const Counters* ctr, double* out6, cudaStream_t st) {
    cudaMemsetAsync(out6, 0, sizeof(double) * 6, st);
    k_info<<<sm_count() * 4, 256, 0, st>>>(cs, s, ctr, out6);
}

}  // namespace dsmc
