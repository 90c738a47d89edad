// dsmc_device.cuh -- device-side constants, case description, Philox stream,
// integer-pipe floor and warp helpers shared by the dsmcFoam+ kernels.
//
// GB300 runs FP64 at roughly 1/57 of its FP32 rate (about 0.6 T DFMA/s
// against 34 T FFMA/s, measured), so the per-particle kernels keep FP64
// instructions to the state updates and do index arithmetic, comparisons and
// random-number work on the integer pipe.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "hystrath_gb300.h"

namespace dsmc {

// OpenFOAM v1706 constants (physicoChemicalConstants, doubleScalar.H)
constexpr double kB = 1.3806504e-23;
constexpr double NAVO = 6.0221417930e+23;   // Avogadro constant of the same (CODATA 2006) set
constexpr double PI = 3.14159265358979323846;
constexpr double SMALL = 1.0e-15;
constexpr double VSMALL = 1.0e-300;
constexpr double ROOTVSMALL = 1.0e-150;
constexpr double GREAT = 1.0e15;

// Bounds on the loops that the reference runs without limit.  Hitting one
// sets an error bit that the host turns into DSMC_ERR_DEVICE.
constexpr int MAX_CROSSINGS = 64;
constexpr int MAX_REJECTION = 100000;
constexpr int MAX_ORDERED_CELL = 16384;   // parcels of the largest cell the collision kernels order
constexpr int WARP_ORDERED_CELL = 1024;   // cells up to this size are ordered by one warp
constexpr int ZV_TAB = 512;     // iMax values tabulated for 1/Zv

// Error bits of the device error word.
enum : unsigned {
    ERRB_CROSSINGS = 1u, ERRB_REJECTION = 2u, ERRB_CAPACITY = 4u, ERRB_BOUNDS = 8u,
    ERRB_PATCH = 16u, ERRB_DENSE = 32u, ERRB_IDS = 64u, ERRB_MIGRANT = 128u, ERRB_MIGRANT_CAP = 256u
};

// Random-stream tags (counter word 3) shared with the CPU replay.
enum : uint32_t {
    TAG_MOVE = 1, TAG_COLLIDE = 2, TAG_INFLOW = 3, TAG_INIT_CELL = 4,
    TAG_INIT_PARTICLE = 5, TAG_REMAINDER = 6
};

// Cell word layout: bits 0-2 sub-cell (x | y<<1 | z<<2), bits 3-30 cell,
// bit 31 "fresh" before the move (inserted this step: random step fraction
// on first move) and "move pending" between the move and the gather (the end
// point x + U dt is not stored yet).
constexpr uint32_t CELLW_DELETED = 0xFFFFFFFFu;
constexpr uint32_t CELLW_FRESH = 0x80000000u;
constexpr uint32_t CELLW_MOVE_PENDING = 0x80000000u;
__host__ __device__ inline uint32_t cellw_cell(uint32_t w) { return (w & 0x7FFFFFFFu) >> 3; }
__host__ __device__ inline uint32_t cellw_sub(uint32_t w) { return w & 7u; }

struct SpeciesDev {
    double m, d, omega, rotDof, thetaV, thetaD, zref, trefZv;
    double kThetaV;     // kB * thetaV
    double invKThetaV;  // 1 / (kB * thetaV), 0 without vibration
    double sqrtKoverM;  // sqrt(kB / m)
    int nVib;
    int pad;
};

struct PairDev {
    double sigmaPrefactor;  // pi dPQ^2 (2 kB Tref / mR)^(omegaPQ - 1/2) / Gamma(5/2 - omegaPQ)
    double expo;            // 1 - omegaPQ: sigma_T cR = prefactor * (cR^2)^expo
    float sigmaPrefactorF;  // FP32 copies for the acceptance test
    float expoF;
    double omegaPQ;
    double mR;
    double mPfrac;          // mP / (mP + mQ)
    double mQfrac;          // mQ / (mP + mQ)
    double invAlphaPQ;      // 1 / alphaPQ, alphaPQ = (alphaP + alphaQ) / 2 (VariableSoftSphere)
    float invAlphaF;        // FP32 copies for the energy-ratio and deflection draws
    float invChiBF;         // 1 / (5/2 - omegaPQ)
    float chiBF;            // 5/2 - omegaPQ
    double twoOverMR;       // 2 / mR
};

struct PatchDev {
    int type;
    int model;
    double Twall;
    double Uwall[3];
};

// Everything a kernel needs about the case, passed by value (constant bank).
struct CaseDev {
    int n[3];
    int nObst;
    long long C;
    double lo[3], hi[3], dx[3], inv[3], negOinv[3];
    float invF[3], negOinvF[3];   // FP32 roundings of inv and negOinv (cell index screen)
    int sideDeletes[6];           // every face of the domain side deletes (dsmcDeletionPatch)
    // reduced-D: an axis whose two sides are empty is tracked at the mesh
    // centre with no velocity along it (dsmcParcel.C:73-84)
    int emptyAx[3];
    int anyEmpty;
    double mid[3];                // mesh bounding-box midpoint
    // rectilinear grading: per graded axis the 2n+1 half-node coordinates
    // (nodes at even, cell midpoints at odd indices), null for a uniform
    // axis; per-cell volumes and per-boundary-face areas, null when uniform
    const double* half[3];
    const double* cellV;
    const double* bfArea;
    // dsmcFaceTracker: per face and species the signed parcel count and mass
    // through every cell face (x faces, then y faces, then z faces), or null
    double* faceFlux;             // [2][nSpecies][nFacesAll]
    long long faceOff[3];
    long long nFacesAll;
    double V;
    double FN, dt;
    double selK;         // FN dt / V: the selection factor of a uniform mesh's cells
    double invDtFa[3];   // 1 / (dt * area of a face normal to each axis)
    uint32_t seedLo, seedHi;
    int nSpecies;
    int collModel;
    int selModel;       // DSMC_SEL_*
    double zrot, fixedZv;
    double invZrot;     // 1 / Zrot
    int invZvForm;
    int nPatches;
    SpeciesDev sp[DSMC_MAX_SPECIES];
    float mRel[DSMC_MAX_SPECIES];   // species mass / mass of species 0 (FP32 feature sums)
    PairDev pair[DSMC_MAX_SPECIES * DSMC_MAX_SPECIES];
    PatchDev patch[DSMC_MAX_PATCHES];
    int obLoI[DSMC_MAX_OBSTACLES][3], obHiI[DSMC_MAX_OBSTACLES][3];
    double obLo[DSMC_MAX_OBSTACLES][3], obHi[DSMC_MAX_OBSTACLES][3];
    long long sideOff[7];
    long long obstOff[DSMC_MAX_OBSTACLES][6];
    long long nBFaces;
    int nAcc;           // doubles per cell of sampling accumulators
    int hasWallMeasure;
    // FP32 reciprocals of n[0] and n[0] n[1] for cell_coords
    float rcpN0, rcpN01;
    // caps of the loops the reference runs without bound and of the cell size
    // the collision kernels order (MAX_REJECTION, MAX_CROSSINGS, ORDER_MAX_N
    // unless lowered by dsmc_set_limits), and the parcel capacity the inflow
    // may fill (the allocation unless lowered)
    int maxRejection;
    int maxCrossings;
    int maxCellParcels;
    long long capacityLimit;
    // 1/Zv of the variable-Zv model by quantised collision level iMax
    // (dsmcCloud.C:1420-1490 depends on iMax, species and pair omega only):
    // invZvTab[((p * DSMC_MAX_SPECIES + q) * ZV_TAB) + iMax]
    const double* invZvTab;
    // spatial decomposition (dsmc_set_domain): the cloud owns the parcels of
    // the cells with domLo <= index < domHi along axis domAxis; -1: all cells
    int domAxis;
    int domLo, domHi;
    int pad2;
};

// Sampling accumulators: per cell, per species s at s*SACC + k.
enum { SACC_N = 0, SACC_UX, SACC_UY, SACC_UZ, SACC_UU, SACC_EROT, SACC_VIB, SACC };
// per-cell collision counters after the species blocks
enum { CACC_NCOLLS = 0, CACC_COLLSEP, CACC };
// wall accumulators per boundary face
enum { W_RHON = 0, W_RHOM, W_LINKE, W_MCC, W_MOMX, W_MOMY, W_MOMZ, W_EROT, W_ZETAROT, W_EVIB,
       W_Q, W_FDX, W_FDY, W_FDZ, W_N };

// Parcel state: one 64-byte record per parcel, aligned so that it is two
// whole sectors, plus the cell word in its own array (the sort key).  A parcel
// that changes cell is moved by the sort as two sectors instead of one sector
// per field, and the collision kernels reach a parcel's velocity, energy and
// species in one record.
struct __align__(16) Rec {
    double x, y, z;
    double ux, uy, uz;
    double erot;
    uint32_t id;
    uint32_t sv;     // species index (bits 0-7) | vibrational level << 8
};
static_assert(sizeof(Rec) == 64, "parcel record must be 64 bytes");

constexpr int SV_MAX_VIB = (1 << 24) - 1;
__host__ __device__ inline int sv_species(uint32_t sv) { return (int)(sv & 0xFFu); }
__host__ __device__ inline int sv_vib(uint32_t sv) { return (int)(sv >> 8); }
__host__ __device__ inline uint32_t make_sv(int species, int vib) { return (uint32_t)species | ((uint32_t)vib << 8); }

struct Parcels {
    Rec* r;            // [capacity]
    uint32_t* cellw;   // [capacity]
    uint32_t* id;      // [capacity] copy of r[i].id, written wherever records take new slots: the
                       // collision kernels stage a cell's ids from here (8 per sector)
};

// Whole-record access with four 16-byte loads or stores.
__device__ __forceinline__ Rec rec_from(double2 a, double2 b, double2 c, double2 d) {
    Rec v;
    v.x = a.x; v.y = a.y; v.z = b.x;
    v.ux = b.y; v.uy = c.x; v.uz = c.y;
    v.erot = d.x;
    const unsigned long long t = (unsigned long long)__double_as_longlong(d.y);
    v.id = (uint32_t)t;
    v.sv = (uint32_t)(t >> 32);
    return v;
}
__device__ __forceinline__ double tail_word(const Rec& v) {
    return __longlong_as_double((long long)(((unsigned long long)v.sv << 32) | v.id));
}
__device__ __forceinline__ Rec ld_rec(const Rec* p) {
    const double2* q = reinterpret_cast<const double2*>(p);
    return rec_from(q[0], q[1], q[2], q[3]);
}
// read-only path: for kernels that do not write the record
__device__ __forceinline__ Rec ldg_rec(const Rec* p) {
    const double2* q = reinterpret_cast<const double2*>(p);
    return rec_from(__ldg(q), __ldg(q + 1), __ldg(q + 2), __ldg(q + 3));
}
__device__ __forceinline__ void st_rec(Rec* p, const Rec& v) {
    double2* q = reinterpret_cast<double2*>(p);
    q[0] = make_double2(v.x, v.y);
    q[1] = make_double2(v.z, v.ux);
    q[2] = make_double2(v.uy, v.uz);
    q[3] = make_double2(v.erot, tail_word(v));
}
// streaming store (the record is not read again soon)
__device__ __forceinline__ void st_rec_cs(Rec* p, const Rec& v) {
    double2* q = reinterpret_cast<double2*>(p);
    __stcs(q, make_double2(v.x, v.y));
    __stcs(q + 1, make_double2(v.z, v.ux));
    __stcs(q + 2, make_double2(v.uy, v.uz));
    __stcs(q + 3, make_double2(v.erot, tail_word(v)));
}

// ------------------------------------------------------------------ Philox
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): two 32x32->64
// multiplies per round with the published multipliers and Weyl key steps.
__device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                              uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint32_t lo0 = 0xD2511F53u * c0;
        const uint32_t hi0 = __umulhi(0xD2511F53u, c0);
        const uint32_t lo1 = 0xCD9E8D57u * c2;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2);
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// (2k+1) 2^-53 for the top 52 bits k of (hi:lo); one FP64 add.
__device__ __forceinline__ double u01_from(uint32_t lo, uint32_t hi) {
    const unsigned long long k = ((((unsigned long long)hi) << 32) | lo) >> 12;
    const double d = __longlong_as_double((long long)(0x3FF0000000000000ull | k));
    return __dsub_rn(d, 1.0 - 0x1p-53);
}

struct Rng {
    uint32_t c0, c1, blk, tag, k0, k1;
    uint32_t b2, b3;
    int have;
    __device__ __forceinline__ Rng(const CaseDev& cs, uint32_t obj, uint32_t step, uint32_t t)
        : c0(obj), c1(step), blk(0), tag(t), k0(cs.seedLo), k1(cs.seedHi), b2(0), b3(0), have(0) {}
    __device__ __forceinline__ double u01() {
        if (have == 0) {
            uint32_t o[4];
            philox4x32_10(c0, c1, blk, tag, k0, k1, o);
            ++blk;
            b2 = o[2]; b3 = o[3];
            have = 1;
            return u01_from(o[0], o[1]);
        }
        have = 0;
        return u01_from(b2, b3);
    }
    // dsmcCloud::randomLabel (dsmcCloud.C:1015-1040), bounded redraw
    __device__ __forceinline__ int label(int a, int b, unsigned* err) {
        if (a == b) return a;
        const int s = a < b ? a : b, e = a < b ? b : a;
        for (int it = 0; it < MAX_REJECTION; ++it) {
            const int v = s + (int)(u01() * (double)(e - s + 1));
            if (v != e + 1) return v;
        }
        *err |= ERRB_REJECTION;
        return s;
    }
    __device__ __forceinline__ void gauss2(double* g1, double* g2) {
        const double u1 = u01();
        const double u2 = u01();
        const double r = sqrt(-2.0 * log(u1));
        double s, c;
        sincos(2.0 * PI * u2, &s, &c);
        *g1 = r * c;
        *g2 = r * s;
    }
};

// floor(2 t) computed from the bits of t on the integer pipe.  Exact for
// |2t| < 2^30; larger magnitudes saturate to +-2^30 (treated as outside).
__device__ __forceinline__ int floor2_bits(double t) {
    const long long b = __double_as_longlong(t);
    const int e = (int)((b >> 52) & 0x7FF) - 1022;   // exponent of 2t
    if (e < 0) return (b < 0 && (b << 1) != 0) ? -1 : 0;
    if (e > 29) return b < 0 ? -(1 << 30) : (1 << 30);
    const unsigned long long m = ((unsigned long long)b & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
    const int sh = 52 - e;
    const int ip = (int)(m >> sh);
    const int frac = (m << (64 - sh)) != 0ull;
    return b < 0 ? -(ip + frac) : ip;
}

// float(v) truncated, from the bits of v on the integer pipe (normal range;
// values below FLT_MIN become 0)
__device__ __forceinline__ float d2f_bits(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
    if (e <= 0) return 0.0f;
    const unsigned sign = (unsigned)(b >> 63) << 31;
    if (e >= 255) return __uint_as_float(sign | 0x7F800000u);
    return __uint_as_float(sign | ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7FFFFFu));
}

// Doubled cell coordinate on a graded axis: k with h[k] <= x < h[k+1] for the
// half-node coordinates h[0..m], -1 below h[0] and m from h[m] on.
__device__ __forceinline__ int floor2_graded(const double* __restrict__ h, int m, double x) {
    if (!(x >= h[0])) return -1;
    if (x >= h[m]) return m;
    int lo = 0, hi = m;
    while (hi - lo > 1) {
        const int md = (lo + hi) >> 1;
        if (h[md] <= x) lo = md; else hi = md;
    }
    return lo;
}

__device__ __forceinline__ int floor2_coord(const CaseDev& cs, double x, int a) {
    if (cs.half[a]) return floor2_graded(cs.half[a], 2 * cs.n[a], x);
    return floor2_bits(fma(x, cs.inv[a], cs.negOinv[a]));
}

// cell volume and the nodes and widths of the cells along an axis
__device__ __forceinline__ double cell_volume(const CaseDev& cs, long long c) {
    return cs.cellV ? cs.cellV[c] : cs.V;
}

// floor2_coord with the FP64 multiply-add replaced, where it cannot change
// the result, by an FP32 one.  t32 = fmaf(float(x), float(inv), float(negOinv))
// differs from the FP64 coordinate t by at most 2^-21 (|x inv| + |negOinv| +
// |t|) (truncation of x: 2^-23, roundings of the constants and of the fmaf:
// 2^-24 each), so when 2 t32 lies farther than twice that bound from an
// integer both floors agree; otherwise (about one coordinate in 10^4, and
// every exact integer) the FP64 path decides.  The result is bit for bit that
// of floor2_coord.
__device__ __forceinline__ int floor2_coord_fast_uniform(const CaseDev& cs, double x, int a) {
    const float xf = d2f_bits(x);
    const float p = xf * cs.invF[a];
    const float t = fmaf(xf, cs.invF[a], cs.negOinvF[a]);
    const float u = 2.0f * t;
    const float f = floorf(u);
    const float margin = 1.9073486e-6f * (fabsf(p) + fabsf(cs.negOinvF[a]) + fabsf(t));   // 2 x 2^-20 x (...)
    if (fabsf(u) < 4194304.0f && u - f > margin && (f + 1.0f) - u > margin) return (int)f;
    return floor2_bits(fma(x, cs.inv[a], cs.negOinv[a]));
}

__device__ __forceinline__ int floor2_coord_fast(const CaseDev& cs, double x, int a) {
    if (cs.half[a]) return floor2_graded(cs.half[a], 2 * cs.n[a], x);
    return floor2_coord_fast_uniform(cs, x, a);
}

// ------------------------------------------------------- cell coordinates
// q = c / d for c < 2^24 (exact in FP32) from the FP32 reciprocal of d: the
// rounded product is within one of the quotient, and one remainder test
// corrects it (a few instructions instead of a 32-bit integer division).
__device__ __forceinline__ uint32_t udiv24(uint32_t c, uint32_t d, float rcp) {
    uint32_t q = __float2uint_rz((float)c * rcp);
    const int r = (int)(c - q * d);
    if (r < 0) --q;
    else if (r >= (int)d) ++q;
    return q;
}

// (i, j, k) of linear cell c = i + n0 (j + n1 k)
__device__ __forceinline__ void cell_coords(const CaseDev& cs, uint32_t c, int* i, int* j, int* k) {
    const uint32_t n0 = (uint32_t)cs.n[0], n01 = (uint32_t)cs.n[0] * (uint32_t)cs.n[1];
    if (cs.C < (1LL << 24)) {
        const uint32_t kk = udiv24(c, n01, cs.rcpN01);
        const uint32_t r = c - kk * n01;
        const uint32_t jj = udiv24(r, n0, cs.rcpN0);
        *i = (int)(r - jj * n0);
        *j = (int)jj;
        *k = (int)kk;
    } else {
        *i = (int)(c % n0);
        *j = (int)((c / n0) % (uint32_t)cs.n[1]);
        *k = (int)(c / n01);
    }
}

// Whether linear cell c belongs to this cloud's domain (dsmc_set_domain).
__device__ __forceinline__ bool cell_owned(const CaseDev& cs, uint32_t c) {
    if (cs.domAxis < 0) return true;
    int i, j, k;
    cell_coords(cs, c, &i, &j, &k);
    const int v = cs.domAxis == 0 ? i : cs.domAxis == 1 ? j : k;
    return v >= cs.domLo && v < cs.domHi;
}

// ------------------------------------------------------- velocity moments
// Per species and cell (measureHeatFluxShearStress, dsmcVolFields.C:
// 1186-1206): sums of u_i u_j (6), |U|^2 u_i (3) and E_int u_i (3), E_int the
// rotational plus vibrational energy; the mass is applied when fields are
// made.
enum { MACC_UU = 0, MACC_UV, MACC_UW, MACC_VV, MACC_VW, MACC_WW, MACC_CCU, MACC_CCV, MACC_CCW,
       MACC_EU, MACC_EV, MACC_EW, MACC };

// ------------------------------------------------------- sampling sums
// The per-step sums of the dsmcVolFields sample loop are exact integer
// fixed-point sums (value * 2^F), so they come out the same for any parcel
// order and any grouping of partial sums; they are added to the FP64
// accumulators once per cell.
constexpr int F_U = 28;        // velocity: resolution 3.7e-9 m/s
constexpr int F_UU = 14;       // |U|^2: resolution 6.1e-5 m^2/s^2
constexpr int F_E = 100;       // rotational energy: resolution 7.9e-31 J

// round(v 2^F), halves away from zero, from the bits on the integer pipe;
// |v 2^F| must stay below 2^62 (saturates and flags otherwise)
// round(v 2^F) as a 64-bit integer: the exponent field takes the scaling
// (exact) and one round-to-nearest conversion the rest; zero and subnormal
// inputs give 0, magnitudes of 2^(62-F) and more set the bounds flag.
__device__ __forceinline__ long long fixp(double v, int F, unsigned* err) {
    const long long b = __double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7FF);
    if (e - 1075 + F > 9) *err |= ERRB_BOUNDS;
    const long long r = __double2ll_rn(__longlong_as_double(b + ((long long)F << 52)));
    return e == 0 ? 0 : r;
}

__device__ __forceinline__ double unfix(long long s, int F) { return ldexp((double)s, -F); }

// Sum of v over this lane's run of the warp (the run starts at lane
// segStart).  The run's last lane holds the total.
__device__ __forceinline__ long long seg_sum(long long v, int segStart) {
    const int lane = (int)(threadIdx.x & 31u);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane - o >= segStart) v += y;
    }
    return v;
}

__device__ __forceinline__ int seg_sum32(int v, int segStart) {
    const int lane = (int)(threadIdx.x & 31u);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane - o >= segStart) v += y;
    }
    return v;
}

__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

}  // namespace dsmc
