// dsmc_tile.cuh -- the per-cell collision kernels (noTimeCounter::collide,
// noTimeCounter.C:81-339).
//
// Order of work in one step:
//   k_ntc_select    one thread per cell: the number of candidate pairs
//                   (selectedPairs, noTimeCounter.C:146-153) and the
//                   remainder update; counts cells per work class.
//   k_ntc_buckets   offsets of the work classes.
//   k_ntc_list      the cells with candidates, grouped by class: heavy cells
//                   (many parcels or candidates) first, then light cells,
//                   each class heaviest first.
//   k_cell_order    one warp per heavy cell (one block above ORDER_WARP_N
//                   parcels): the cell's members sorted by (sub-cell, parcel
//                   id).  This is the cell's canonical list: sub-cells are
//                   contiguous in it and it does not depend on the order in
//                   which the sort scatter left the parcels in memory.
//   k_collide_heavy one warp per heavy cell.
//   k_collide_light one lane per light cell.
//
// Every candidate k of cell c draws its acceptance test and post-collision
// deviates from its own counter-based stream (cell, step, k).
//
// Heavy cells pick the pair as the reference does (randomLabel draws over
// the cell's list, with the redraw while Q == P, noTimeCounter.C:164-198) over
// the canonical list.  A candidate then depends only on the state of its own
// two parcels when it runs, so the warp runs up to 32 candidates of the cell
// at once: each round runs every candidate that shares no parcel with an
// earlier candidate still waiting, which gives exactly the result of running
// them one after the other (disjoint candidates commute).
//
// Light cells (at most LIGHT_N parcels, fewer than LIGHT_CAND candidates)
// run their candidates one after the other in one lane and pick without a
// list: P is the member whose id has the smallest keyed 32-bit hash, Q the
// member of P's sub-cell (or of the cell when P is alone there) other than P
// with the smallest hash under a second key.  For a given key the hash is a
// bijection of the id, so every member is equally likely and picks under
// different keys are independent: the same distribution as the list draws,
// without a sort.  The picks do not depend on earlier candidates' outcomes,
// so a warp makes all picks of its 32 light cells first, cell by cell (one
// coalesced load of the cell's ids, a warp minimum per pick), and each lane
// then tests and collides its own cell's candidates.
//
// Both paths give results that do not depend on the parcels' order in
// memory, so a run is reproducible.  Serial work is spread across lanes
// because GB300 issues an FP64 instruction over the whole warp whatever the
// active mask.
#pragma once

namespace tile {

constexpr int WARPS = 4;             // warps per block
constexpr int LIGHT_N = 64;          // light cells: at most this many parcels
constexpr int LIGHT_CAND = 16;       //   and fewer candidates than this
constexpr int ORDER_WARP_N = WARP_ORDERED_CELL;   // cells up to this size are ordered by one warp
constexpr int ORDER_MAX_N = MAX_ORDERED_CELL;   // cells up to this size are ordered by one block
constexpr int ORDER_BLOCK = 512;     // threads of the block that orders a large cell
constexpr int NBUCKET = 8;           // candidate-count buckets per class
constexpr int MAX_CAND = 1 << 24;    // candidates of one cell in one step

// bucket b holds candidate counts in [2^b, 2^(b+1)); heavier buckets come
// first in the work list so that they start first
__device__ __forceinline__ int bucket_of(int nc) {
    const int b = 31 - __clz(nc);
    return b < NBUCKET - 1 ? b : NBUCKET - 1;
}

__device__ __forceinline__ bool is_heavy(int n, int nc) { return n > LIGHT_N || nc >= LIGHT_CAND; }

__device__ __forceinline__ int slot_of(int n, int nc) { return (is_heavy(n, nc) ? NBUCKET : 0) + bucket_of(nc); }

// the 16-bit field s (0..7) of a packed sub-cell start table
__device__ __forceinline__ int get16(const uint4& w, int s) {
    const unsigned x = s < 2 ? w.x : s < 4 ? w.y : s < 6 ? w.z : w.w;
    return (int)((x >> ((s & 1) << 4)) & 0xFFFFu);
}

// ------------------------------------------------------------ selection
// selectedPairs and the remainder, one thread per cell; the candidate count
// of each cell is kept for k_ntc_list and counted per slot
// learned: the maximum is the prediction unless the cell has fallen back to
// the running maximum, has no prediction, or saw a product above an earlier
// prediction that this one does not cover (the fallback is kept until a
// prediction covers the largest such product); it is kept in smaxSel for the
// acceptance tests of this step
// The candidate count of cell c (0 for a cell with fewer than two parcels
// or one skipped as too dense, with the error bit set).
__device__ __forceinline__ int select_cell(const CaseDev& cs, const int* __restrict__ start,
                                           const double* __restrict__ smax, double* rem, int learned,
                                           const float* __restrict__ pred, const unsigned char* __restrict__ useR,
                                           const float* __restrict__ exceed, double* smaxSel, long long c, int* n_out,
                                           unsigned& err) {
    int nc = 0;
    const int n = start[c + 1] - start[c];
    *n_out = n;
    if (n > 1) {
        double sm = smax[c];
        if (learned) {
            const float pv = pred[c];
            if (!useR[c] && pv > 0.f && pv < 3.0e38f && pv >= exceed[c]) sm = (double)pv;
            smaxSel[c] = sm;
        }
        // rem + 0.5 n (n - 1) FN sm dt / V: on a uniform mesh FN dt / V is
        // one factor of the case, which leaves no FP64 division per cell (on
        // GB300 the division's dozen FP64 instructions dominated this pass)
        const double pairs = (double)((n * (n - 1)) >> 1);
        const double k = cs.cellV ? cs.FN * cs.dt / cs.cellV[c] : cs.selK;
        const double sel = fma(pairs, sm * k, rem[c]);
        const double whole = floor(sel);
        rem[c] = sel - whole;
        if (n > cs.maxCellParcels || whole >= (double)MAX_CAND) err |= ERRB_DENSE;
        else nc = (int)whole;
    }
    return nc;
}

__global__ void k_ntc_select(CaseDev cs, const int* __restrict__ start, const double* __restrict__ smax, double* rem,
                             Counters* ctr, int* ncCell, unsigned* slotCount, int learned,
                             const float* __restrict__ pred, const unsigned char* __restrict__ useR,
                             const float* __restrict__ exceed, double* smaxSel) {
    __shared__ unsigned hist[2 * NBUCKET];
    if (threadIdx.x < 2 * NBUCKET) hist[threadIdx.x] = 0;
    __syncthreads();
    const long long C = cs.C;
    unsigned err = 0;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < C;
         c += (long long)gridDim.x * blockDim.x) {
        int n;
        const int nc = select_cell(cs, start, smax, rem, learned, pred, useR, exceed, smaxSel, c, &n, err);
        ncCell[c] = nc;
        if (nc > 0) atomicAdd(&hist[slot_of(n, nc)], 1u);
    }
    __syncthreads();
    if (threadIdx.x < 2 * NBUCKET && hist[threadIdx.x]) atomicAdd(&slotCount[threadIdx.x], hist[threadIdx.x]);
    if (err) atomicOr(&ctr->err, err);
}

// slot offsets: heavy slots first, heaviest first; resets the counts
__global__ void k_ntc_buckets(Counters* ctr, unsigned* slotCount, unsigned* slotCursor) {
    unsigned off = 0;
    for (int b = 2 * NBUCKET - 1; b >= 0; --b) {
        slotCursor[b] = off;
        off += slotCount[b];
        slotCount[b] = 0;
        if (b == NBUCKET) ctr->nHeavy = off;
    }
    ctr->nWork = off;
}

// work list of the cells with candidates; cells too large for one warp to
// order are also listed (by work index) for k_cell_order_big
// allHeavy: every listed cell is ordered and takes a heavy slot (the
// Bernoulli-trial selection walks the canonical list of every cell)
// One warp-wide iteration of k_ntc_list over cells c (lanes past C take part
// without a cell).
__device__ __forceinline__ void list_iter(long long C, const int* __restrict__ start, const int* __restrict__ ncCell,
                                          unsigned* slotCursor, int2* work, int* bigList, Counters* ctr, int allHeavy,
                                          long long c) {
    const unsigned lane = threadIdx.x & 31u;
    int nc = 0, n = 0;
    if (c < C) {
        nc = ncCell[c];
        if (nc > 0) n = start[c + 1] - start[c];
    }
    if (!__ballot_sync(0xFFFFFFFFu, nc > 0)) return;
    const int slot = nc > 0 ? (allHeavy ? NBUCKET + bucket_of(nc) : slot_of(n, nc)) : -1;
    // one atomic per slot present in the warp
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, slot);
    const int leader = __ffs(peers) - 1;
    unsigned q0 = 0;
    if (nc > 0 && (int)lane == leader) q0 = atomicAdd(&slotCursor[slot], (unsigned)__popc(peers));
    q0 = __shfl_sync(0xFFFFFFFFu, q0, leader);
    if (nc > 0) {
        const unsigned q = q0 + __popc(peers & ((1u << lane) - 1u));
        work[q] = make_int2((int)c, nc);
        if (n > ORDER_WARP_N) bigList[atomicAdd(&ctr->bigCells, 1)] = (int)q;
    }
}

// work list of the cells with candidates; cells too large for one warp to
// order are also listed (by work index) for k_cell_order_big
// allHeavy: every listed cell is ordered and takes a heavy slot (the
// Bernoulli-trial selection walks the canonical list of every cell)
// The 16 slot cursors are shared by every cell of the mesh, so the block
// reserves its cells' places in shared memory first and takes them from the
// cursors with one atomic per slot present (a reservation per warp queued
// every warp of the grid on the light slots' cursor).  The order inside a
// slot does not matter: cells are independent.
__global__ void k_ntc_list(long long C, const int* __restrict__ start, const int* __restrict__ ncCell,
                           unsigned* slotCursor, int2* work, int* bigList, Counters* ctr, int allHeavy) {
    __shared__ unsigned blkCnt[2 * NBUCKET], blkBase[2 * NBUCKET];
    const unsigned lane = threadIdx.x & 31u;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < C; base += (long long)gridDim.x * blockDim.x) {
        if (threadIdx.x < 2 * NBUCKET) blkCnt[threadIdx.x] = 0;
        __syncthreads();
        const long long c = base + threadIdx.x;
        int nc = 0, n = 0;
        if (c < C) {
            nc = ncCell[c];
            if (nc > 0) n = start[c + 1] - start[c];
        }
        const int slot = nc > 0 ? (allHeavy ? NBUCKET + bucket_of(nc) : slot_of(n, nc)) : -1;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, slot);
        const int leader = __ffs(peers) - 1;
        unsigned off = 0;
        if (nc > 0 && (int)lane == leader) off = atomicAdd(&blkCnt[slot], (unsigned)__popc(peers));
        off = __shfl_sync(0xFFFFFFFFu, off, leader);
        __syncthreads();
        if (threadIdx.x < 2 * NBUCKET && blkCnt[threadIdx.x])
            blkBase[threadIdx.x] = atomicAdd(&slotCursor[threadIdx.x], blkCnt[threadIdx.x]);
        __syncthreads();
        if (nc > 0) {
            const unsigned q = blkBase[slot] + off + __popc(peers & ((1u << lane) - 1u));
            work[q] = make_int2((int)c, nc);
            if (n > ORDER_WARP_N) bigList[atomicAdd(&ctr->bigCells, 1)] = (int)q;
        }
        __syncthreads();   // blkCnt and blkBase are reused by the next pass
    }
}

// ------------------------------------------------------------ ordering
// Key of member j: (sub-cell, parcel id, j).  Ids are unique, so the order is
// total and j rides in the low bits.
__device__ __forceinline__ unsigned long long order_key(uint32_t cellw, uint32_t id, int j) {
    return ((unsigned long long)(cellw & 7u) << 48) | ((unsigned long long)id << 16) | (unsigned long long)j;
}

// bitonic sort of keys[0, N) (N a power of two) by the nt threads of a group
// (thread t) that all call it; bar() synchronises the group
template <class Bar>
__device__ __forceinline__ void bitonic(unsigned long long* keys, int N, int t, int nt, Bar bar) {
    for (int k = 2; k <= N; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = t; i < (N >> 1); i += nt) {
                const int lo = ((i & ~(j - 1)) << 1) | (i & (j - 1));
                const int hi = lo + j;
                const unsigned long long a = keys[lo], b = keys[hi];
                const bool up = (lo & k) == 0;
                if ((a > b) == up) { keys[lo] = b; keys[hi] = a; }
            }
            bar();
        }
    }
}

__device__ __forceinline__ uint4 pack_starts(const int* cnt) {
    int so[8];
    int acc = 0;
#pragma unroll
    for (int b = 0; b < 8; ++b) { so[b] = acc; acc += cnt[b]; }
    return make_uint4((unsigned)so[0] | ((unsigned)so[1] << 16), (unsigned)so[2] | ((unsigned)so[3] << 16),
                      (unsigned)so[4] | ((unsigned)so[5] << 16), (unsigned)so[6] | ((unsigned)so[7] << 16));
}

struct WarpBar {
    __device__ __forceinline__ void operator()() const { __syncwarp(); }
};
struct BlockBar {
    __device__ __forceinline__ void operator()() const { __syncthreads(); }
};

// one warp per heavy cell of at most ORDER_WARP_N parcels: perm[off + r] is
// the local index of the r-th member in canonical order, subs[q] the start
// of each sub-cell in it
// One warp orders heavy work item q (keys: ORDER_WARP_N words of the warp's
// shared memory).
__device__ __forceinline__ void order_item(const Parcels& s, const int* __restrict__ start,
                                           const int2* __restrict__ work, uint16_t* perm, uint4* subs, long long q,
                                           unsigned long long* keys) {
    const int lane = (int)(threadIdx.x & 31u);
    const int c = work[q].x;
    const long long off = start[c];
    const int n = start[c + 1] - (int)off;
    if (n > ORDER_WARP_N) return;
    int N = 32;
    while (N < n) N <<= 1;
    int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int j0 = 0; j0 < N; j0 += 32) {
        const int j = j0 + lane;
        unsigned long long key = ~0ull;
        int sb = 8;
        if (j < n) {
            const uint32_t w = s.cellw[off + j];
            sb = (int)(w & 7u);
            key = order_key(w, __ldg(s.id + off + j), j);
        }
        keys[j] = key;
#pragma unroll
        for (int b = 0; b < 8; ++b) cnt[b] += __popc(__ballot_sync(0xFFFFFFFFu, sb == b));
    }
    __syncwarp();
    bitonic(keys, N, lane, 32, WarpBar());
    for (int r = lane; r < n; r += 32) perm[off + r] = (uint16_t)(keys[r] & 0xFFFFu);
    if (lane == 0) subs[q] = pack_starts(cnt);
    __syncwarp();
}

__global__ void __launch_bounds__(WARPS * 32)
k_cell_order(Parcels s, const int* __restrict__ start, const Counters* ctr, const int2* __restrict__ work,
             uint16_t* perm, uint4* subs) {
    __shared__ unsigned long long keysAll[WARPS][ORDER_WARP_N];
    unsigned long long* keys = keysAll[threadIdx.x >> 5];
    const long long nHeavy = (long long)ctr->nHeavy;
    const long long nWarps = (long long)gridDim.x * WARPS;
    for (long long q = (long long)blockIdx.x * WARPS + (threadIdx.x >> 5); q < nHeavy; q += nWarps)
        order_item(s, start, work, perm, subs, q, keys);
}

// one block per listed cell above ORDER_WARP_N parcels (dynamic shared
// memory of ORDER_MAX_N keys)
__global__ void __launch_bounds__(ORDER_BLOCK)
k_cell_order_big(Parcels s, const int* __restrict__ start, const Counters* ctr, const int2* __restrict__ work,
                 const int* __restrict__ bigList, uint16_t* perm, uint4* subs) {
    extern __shared__ unsigned long long keysBig[];
    __shared__ int cnt[8];
    const int nBig = ctr->bigCells;
    for (int b = blockIdx.x; b < nBig; b += gridDim.x) {
        const int q = bigList[b];
        const int c = work[q].x;
        const long long off = start[c];
        const int n = start[c + 1] - (int)off;
        int N = 32;
        while (N < n) N <<= 1;
        if (threadIdx.x < 8) cnt[threadIdx.x] = 0;
        __syncthreads();
        for (int j = threadIdx.x; j < N; j += blockDim.x) {
            unsigned long long key = ~0ull;
            if (j < n) {
                const uint32_t w = s.cellw[off + j];
                atomicAdd(&cnt[w & 7u], 1);
                key = order_key(w, __ldg(s.id + off + j), j);
            }
            keysBig[j] = key;
        }
        __syncthreads();
        bitonic(keysBig, N, (int)threadIdx.x, (int)blockDim.x, BlockBar());
        for (int r = threadIdx.x; r < n; r += blockDim.x) perm[off + r] = (uint16_t)(keysBig[r] & 0xFFFFu);
        if (threadIdx.x == 0) {
            int c8[8];
            for (int k = 0; k < 8; ++k) c8[k] = cnt[k];
            subs[q] = pack_starts(c8);
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------ candidates
// One accepted collision: Larsen-Borgnakke redistribution (or plain VHS) and
// the isotropic centre-of-mass scatter (VariableHardSphere.C:191-228).
struct Post {
    double UP[3], UQ[3];
    double eP, eQ;
    int vP, vQ;
};

// A uniform azimuth phi = 2 pi U as (sin, cos): the angle in FP32
// (sincospif), the pair then scaled to unit length in FP64 so that the
// scattered relative speed, and with it the energy, stays exact to FP64.
__device__ __forceinline__ void azimuth(Rng& r, double* s, double* c) {
    float sf, cf;
    sincospif(2.0f * (float)r.u01(), &sf, &cf);
    const double sd = sf, cd = cf;
    const double inv = rsqrt(sd * sd + cd * cd);
    *s = sd * inv;
    *c = cd * inv;
}

__device__ __forceinline__ void collide_pair(const CaseDev& cs, Rng& r, const PairDev& pr, int tP, int tQ,
                                             double cr2, Post& o, unsigned* err) {
    double cR;
    if (cs.collModel == DSMC_COLL_LB_VHS || cs.collModel == DSMC_COLL_LB_VSS) {
        double Et = 0.5 * pr.mR * cr2;
        redistribute(cs, cs.sp[tP], &o.eP, &o.vP, Et, pr, r, zv_row(cs, tP, tQ), err);
        redistribute(cs, cs.sp[tQ], &o.eQ, &o.vQ, Et, pr, r, zv_row(cs, tQ, tP), err);
        cR = sqrt(Et * pr.twoOverMR);
    } else {
        cR = sqrt(cr2);
    }
    double Ucm[3];
    for (int a = 0; a < 3; ++a) Ucm[a] = pr.mPfrac * o.UP[a] + pr.mQfrac * o.UQ[a];
    double prel[3];
    if (cs.collModel == DSMC_COLL_VSS || cs.collModel == DSMC_COLL_LB_VSS) {
        // VariableSoftSphere::postCollisionVelocities (VariableSoftSphere.C:191-233):
        // deflection cos(chi) = 2 U^(1/alpha) - 1 about the pre-collision
        // relative velocity, Bird eq. 2.22.  Its components are first scaled
        // to the post-exchange speed cR (equal for plain VSS), so the
        // Larsen-Borgnakke variant keeps the energy it computed.
        const double cosT = 2.0 * (double)powf((float)r.u01(), pr.invAlphaF) - 1.0;
        const double sinT = sqrt(1.0 - cosT * cosT);
        double sph, cph;
        azimuth(r, &sph, &cph);
        const double cpre = sqrt(cr2);
        const double k = cpre > 0.0 ? cR / cpre : 0.0;
        const double c0 = k * (o.UP[0] - o.UQ[0]), c1 = k * (o.UP[1] - o.UQ[1]), c2 = k * (o.UP[2] - o.UQ[2]);
        const double D = sqrt(c1 * c1 + c2 * c2);
        if (D > 1e-12 * cR) {
            prel[0] = cosT * c0 + sinT * sph * D;
            prel[1] = cosT * c1 + sinT * (cR * c2 * cph - c0 * c1 * sph) / D;
            prel[2] = cosT * c2 - sinT * (cR * c1 * cph + c0 * c2 * sph) / D;
        } else {   // relative velocity along x
            prel[0] = cosT * c0;
            prel[1] = cR * sinT * cph;
            prel[2] = cR * sinT * sph;
        }
    } else {
        const double cosT = 2.0 * r.u01() - 1.0;
        const double sinT = sqrt(1.0 - cosT * cosT);
        double sph, cph;
        azimuth(r, &sph, &cph);
        prel[0] = cR * cosT;
        prel[1] = cR * sinT * cph;
        prel[2] = cR * sinT * sph;
    }
    for (int a = 0; a < 3; ++a) {
        o.UP[a] = Ucm[a] + prel[a] * pr.mQfrac;
        o.UQ[a] = Ucm[a] - prel[a] * pr.mPfrac;
    }
}

// Positions (in the canonical list of n members with sub-cell starts so) of
// candidate pair P, Q: P uniform over the cell, Q uniform over P's sub-cell
// when it holds another member, else over the cell; Q != P.
__device__ __forceinline__ void draw_pair(Rng& r, int n, const uint4& so, int* pP, int* pQ, unsigned* err) {
    const int p = r.label(0, n - 1, err);
    int sub = 0;
#pragma unroll
    for (int b = 1; b < 8; ++b) sub += (get16(so, b) <= p) ? 1 : 0;
    const int lo = get16(so, sub);
    const int hi = sub < 7 ? get16(so, sub + 1) : n;
    int q = p;
    if (hi - lo > 1) {
        for (int it = 0; it < MAX_REJECTION && q == p; ++it) q = lo + r.label(0, hi - lo - 1, err);
    } else {
        for (int it = 0; it < MAX_REJECTION && q == p; ++it) q = r.label(0, n - 1, err);
    }
    if (q == p) {
        *err |= ERRB_REJECTION;
        q = p == 0 ? 1 : 0;
    }
    *pP = p;
    *pQ = q;
}

// Candidate (gP, gQ): sigma_T c_R, the running maximum, the acceptance test
// against the maximum the candidate count was based on, and the collision.
// run_candidate in two parts: the acceptance test (loads the pair, keeps
// the step's largest product) and the collision of an accepted pair.
// audit (selection audit on): the candidate's expected acceptance
// sigma/max and the part of it above 1, which the test cannot honour
__device__ __forceinline__ void audit_add(float2* au, double sigma, double smax0) {
    const float a = (float)(sigma / smax0);
    au->x += a;
    au->y += fmaxf(a - 1.0f, 0.0f);
}

// The part of a record a collision reads and writes: the velocity, the
// rotational energy and the tail word (id, species and vibrational level).
// Positions stay in memory (the separation reads them on its own), so they
// are not held across the exchange, and a collision stores 40 of the 64
// bytes.
struct CollRec {
    double ux, uy, uz, erot;
    uint32_t id, sv;
};

__device__ __forceinline__ CollRec ld_coll(const Rec* p) {
    const double2* q = reinterpret_cast<const double2*>(p);
    const double2 b = q[1], c = q[2], d = q[3];
    CollRec v;
    v.ux = b.y; v.uy = c.x; v.uz = c.y;
    v.erot = d.x;
    const unsigned long long t = (unsigned long long)__double_as_longlong(d.y);
    v.id = (uint32_t)t;
    v.sv = (uint32_t)(t >> 32);
    return v;
}

__device__ __forceinline__ void st_coll(Rec* p, const CollRec& v) {
    double2* q = reinterpret_cast<double2*>(p);
    reinterpret_cast<double*>(p)[3] = v.ux;
    q[2] = make_double2(v.uy, v.uz);
    q[3] = make_double2(v.erot, __longlong_as_double((long long)(((unsigned long long)v.sv << 32) | v.id)));
}

// the separation only feeds the mean collision separation field: FP32
// after the FP64 differences
__device__ __forceinline__ float coll_separation(const Rec* a, const Rec* b) {
    const double2* qa = reinterpret_cast<const double2*>(a);
    const double2* qb = reinterpret_cast<const double2*>(b);
    const double2 a0 = qa[0], b0 = qb[0];
    const double az = qa[1].x, bz = qb[1].x;
    const float dx = (float)(a0.x - b0.x);
    const float dy = (float)(a0.y - b0.y);
    const float dz = (float)(az - bz);
    return sqrtf(dx * dx + dy * dy + dz * dz);
}

__device__ __forceinline__ bool test_candidate(const CaseDev& cs, const Parcels& s, Rng& r, long long gP,
                                               long long gQ, double smax0, double* stepMax, CollRec* P,
                                               CollRec* Q, double* cr2, float2* au) {
    *P = ld_coll(s.r + gP);
    *Q = ld_coll(s.r + gQ);
    const int tP = sv_species(P->sv), tQ = sv_species(Q->sv);
    const PairDev& pr = cs.pair[tP * DSMC_MAX_SPECIES + tQ];
    const double d0 = P->ux - Q->ux, d1 = P->uy - Q->uy, d2 = P->uz - Q->uz;
    *cr2 = d0 * d0 + d1 * d1 + d2 * d2;
    const double sigma = sigma_cr(pr, *cr2);
    if (sigma > *stepMax) *stepMax = sigma;
    if (au) audit_add(au, sigma, smax0);
    return sigma > r.u01() * smax0;
}

// The exchange of an accepted pair and the stores of its two parcels.
__device__ __forceinline__ void exchange_pair(const CaseDev& cs, const Parcels& s, Rng& r, long long gP, long long gQ,
                                              CollRec P, CollRec Q, double cr2, unsigned* err) {
    const int tP = sv_species(P.sv), tQ = sv_species(Q.sv);
    const PairDev& pr = cs.pair[tP * DSMC_MAX_SPECIES + tQ];
    Post o;
    o.UP[0] = P.ux; o.UP[1] = P.uy; o.UP[2] = P.uz;
    o.UQ[0] = Q.ux; o.UQ[1] = Q.uy; o.UQ[2] = Q.uz;
    o.eP = P.erot; o.eQ = Q.erot;
    o.vP = sv_vib(P.sv); o.vQ = sv_vib(Q.sv);
    collide_pair(cs, r, pr, tP, tQ, cr2, o, err);
    if (o.vP > SV_MAX_VIB || o.vQ > SV_MAX_VIB) *err |= ERRB_BOUNDS;
    P.ux = o.UP[0]; P.uy = o.UP[1]; P.uz = o.UP[2];
    Q.ux = o.UQ[0]; Q.uy = o.UQ[1]; Q.uz = o.UQ[2];
    P.erot = o.eP; Q.erot = o.eQ;
    P.sv = make_sv(tP, o.vP); Q.sv = make_sv(tQ, o.vQ);
    st_coll(s.r + gP, P);
    st_coll(s.r + gQ, Q);
}

__device__ __forceinline__ void collide_candidate(const CaseDev& cs, const Parcels& s, Rng& r, long long gP,
                                                  long long gQ, const CollRec& P, const CollRec& Q, double cr2,
                                                  double* collSep, unsigned* err) {
    *collSep += (double)coll_separation(s.r + gP, s.r + gQ);
    exchange_pair(cs, s, r, gP, gQ, P, Q, cr2, err);
}

__device__ __forceinline__ bool run_candidate(const CaseDev& cs, const Parcels& s, Rng& r, long long gP,
                                              long long gQ, double smax0, double* stepMax, double* collSep,
                                              unsigned* err, float2* au = nullptr) {
    CollRec P, Q;
    double cr2;
    if (!test_candidate(cs, s, r, gP, gQ, smax0, stepMax, &P, &Q, &cr2, au)) return false;
    collide_candidate(cs, s, r, gP, gQ, P, Q, cr2, collSep, err);
    return true;
}

// After a cell's candidates: the running maximum takes the largest product
// seen (noTimeCounter.C:243-246), the step's largest product is kept for
// training, and a learned cell whose prediction was exceeded falls back to
// the running maximum until the next prediction.
__device__ __forceinline__ void cell_epilogue(double* smax, long long c, double R, double smax0, double stepMax,
                                              int learned, unsigned char* useR, float* exceed, float* obsMax,
                                              double2* audit, float2 au) {
    if (stepMax > R) smax[c] = stepMax;
    obsMax[c] = (float)stepMax;
    if (learned && stepMax > smax0) {
        useR[c] = 1;
        if ((float)stepMax > exceed[c]) exceed[c] = (float)stepMax;
    }
    if (audit) {
        double2 v = audit[c];
        v.x += (double)au.x;
        v.y += (double)au.y;
        audit[c] = v;
    }
}

__device__ __forceinline__ uint32_t cand_tag(int k) { return (uint32_t)TAG_COLLIDE | ((uint32_t)k << 8); }

// One warp runs the candidates of heavy work item q, up to 32 at a time; the
// cell's collision and candidate counts go to nColl and nCandTot of lane 0.
__device__ __forceinline__ void heavy_item(const CaseDev& cs, const Parcels& s, const int* __restrict__ start,
                                           double* smax, double* acc, const int2* __restrict__ work,
                                           const uint16_t* __restrict__ perm, const uint4* __restrict__ subs,
                                           int learned, const double* __restrict__ smaxSel, unsigned char* useR,
                                           float* exceed, float* obsMax, double2* audit, long long q, uint32_t step,
                                           unsigned& err, unsigned long long& nColl,
                                           unsigned long long& nCandTot) {
    const unsigned lane = lane_id();
    const long long C = cs.C;
    const int2 it = work[q];
    const long long c = it.x;
    const int nCand = it.y;
    const long long off = start[c];
    const int n = start[c + 1] - (int)off;
    const uint4 so = subs[q];
    const double R = smax[c];
    const double smax0 = learned ? smaxSel[c] : R;
    double stepMax = 0.0, collSep = 0.0;
    unsigned coll = 0;
    float2 au = make_float2(0.f, 0.f);
    for (int base = 0; base < nCand; base += 32) {
        const int k = base + (int)lane;
        Rng r(cs, (uint32_t)c, step, cand_tag(k));
        long long gP = 0, gQ = 0;
        int pP = -1, pQ = -1;
        if (k < nCand) {
            draw_pair(r, n, so, &pP, &pQ, &err);
            gP = off + perm[off + pP];
            gQ = off + perm[off + pQ];
        }
        unsigned pend = __ballot_sync(0xFFFFFFFFu, k < nCand);
        while (pend) {
            // ready: no earlier waiting candidate shares a parcel
            bool ready = (pend >> lane) & 1u;
            unsigned m = pend;
            while (m) {
                const int j = __ffs(m) - 1;
                m &= m - 1u;
                const int a = __shfl_sync(0xFFFFFFFFu, pP, j);
                const int b = __shfl_sync(0xFFFFFFFFu, pQ, j);
                if (j < (int)lane && (a == pP || a == pQ || b == pP || b == pQ)) ready = false;
            }
            if (ready && run_candidate(cs, s, r, gP, gQ, smax0, &stepMax, &collSep, &err,
                                       audit ? &au : nullptr)) ++coll;
            __syncwarp();
            pend &= ~__ballot_sync(0xFFFFFFFFu, ready);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        collSep += __shfl_xor_sync(0xFFFFFFFFu, collSep, o);
        stepMax = fmax(stepMax, __shfl_xor_sync(0xFFFFFFFFu, stepMax, o));
        coll += __shfl_xor_sync(0xFFFFFFFFu, coll, o);
        if (audit) {
            au.x += __shfl_xor_sync(0xFFFFFFFFu, au.x, o);
            au.y += __shfl_xor_sync(0xFFFFFFFFu, au.y, o);
        }
    }
    if (lane == 0) {
        cell_epilogue(smax, c, R, smax0, stepMax, learned, useR, exceed, obsMax, audit, au);
        if (coll) {
            acc[(cs.nSpecies * SACC + CACC_NCOLLS) * C + c] += (double)coll;
            acc[(cs.nSpecies * SACC + CACC_COLLSEP) * C + c] += collSep;
        }
        nColl += coll;
        nCandTot += (unsigned long long)nCand;
    }
}

// one warp per heavy cell, up to 32 candidates at a time
__global__ void __launch_bounds__(WARPS * 32)
k_collide_heavy(CaseDev cs, Parcels s, const int* __restrict__ start, double* smax, double* acc, Counters* ctr,
                const int2* __restrict__ work, const uint16_t* __restrict__ perm, const uint4* __restrict__ subs,
                int learned, const double* __restrict__ smaxSel, unsigned char* useR, float* exceed, float* obsMax,
                double2* audit) {
    const unsigned lane = lane_id();
    const uint32_t step = (uint32_t)ctr->step;
    const long long nHeavy = (long long)ctr->nHeavy;
    unsigned err = 0;
    unsigned long long nColl = 0, nCandTot = 0;
    const long long nWarps = (long long)gridDim.x * WARPS;
    for (long long q = (long long)blockIdx.x * WARPS + (threadIdx.x >> 5); q < nHeavy; q += nWarps)
        heavy_item(cs, s, start, smax, acc, work, perm, subs, learned, smaxSel, useR, exceed, obsMax, audit, q, step,
                   err, nColl, nCandTot);
    if (lane == 0) {
        if (nColl) atomicAdd(&ctr->coll, nColl);
        if (nCandTot) atomicAdd(&ctr->cand, nCandTot);
    }
    if (err) atomicOr(&ctr->err, err);
}

// MurmurHash3's 32-bit finaliser (Appleby): a bijection with full avalanche.
__device__ __forceinline__ uint32_t fmix32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

// pick_key in two parts: the cell's and step's base, then one draw of it
__device__ __forceinline__ uint32_t pick_base(const CaseDev& cs, uint32_t cell, uint32_t step) {
    uint32_t h = fmix32(cs.seedHi ^ 0x51ED270Bu);
    h = fmix32(h ^ cell);
    return fmix32(h ^ step);
}
__device__ __forceinline__ uint32_t pick_draw(const CaseDev& cs, uint32_t base, uint32_t draw) {
    return fmix32(base ^ draw) ^ cs.seedLo;
}
__device__ __forceinline__ uint32_t pick_key(const CaseDev& cs, uint32_t cell, uint32_t step, uint32_t draw) {
    return pick_draw(cs, pick_base(cs, cell, step), draw);
}

// The picks of a light cell's candidates, made by the whole warp: member j
// hashes to fmix32(key ^ id_j); P is the member with the smallest hash, Q the
// smallest among the others of P's sub-cell when it holds two or more
// parcels, else among all others (no two members share a hash: ids are
// distinct and fmix32 is a bijection).
struct LightPicks {
    uint8_t pq[LIGHT_CAND][2][32];   // [candidate][P, Q][lane of the cell]
};

// index j (lane, or lane + 32) of the valid member with the smallest hash
__device__ __forceinline__ int warp_argmin(uint32_t hA, bool vA, uint32_t hB, bool vB) {
    const uint32_t m = min(vA ? hA : 0xFFFFFFFFu, vB ? hB : 0xFFFFFFFFu);
    const uint32_t w = __reduce_min_sync(0xFFFFFFFFu, m);
    const unsigned a = __ballot_sync(0xFFFFFFFFu, vA && hA == w);
    const unsigned b = __ballot_sync(0xFFFFFFFFu, vB && hB == w);
    return a ? __ffs(a) - 1 : (b ? 31 + __ffs(b) : -1);
}

// Accepted candidates of single-candidate light cells whose exchange is
// deferred: a warp collects them (parcel indices and cell) until 32 are
// waiting and then runs 32 exchanges with every lane busy.  On this part an
// FP64 instruction occupies the pipe for the whole warp whatever its active
// lanes, and on the channel 93% of the light cells have one candidate, of
// which 57% are accepted: run where they were tested, the exchanges kept
// half the FP64 pipe's lanes idle.  The exchange repeats the test's one
// draw and reloads the pair, so the result is bit for bit the immediate
// one (no other candidate touches the pair's parcels in this step).
struct LightDefer {
    int4 e[64];      // (gP, gQ, cell, -)
    int count;
};

__device__ __forceinline__ void exchange_deferred(const CaseDev& cs, const Parcels& s, const int4& e, uint32_t step,
                                                  unsigned* err) {
    const long long gP = e.x, gQ = e.y;
    const CollRec P = ld_coll(s.r + gP), Q = ld_coll(s.r + gQ);
    Rng r(cs, (uint32_t)e.z, step, cand_tag(0));
    (void)r.u01();   // the acceptance test's draw
    const double d0 = P.ux - Q.ux, d1 = P.uy - Q.uy, d2 = P.uz - Q.uz;
    const double cr2 = d0 * d0 + d1 * d1 + d2 * d2;
    exchange_pair(cs, s, r, gP, gQ, P, Q, cr2, err);
}

// One warp's group of 32 light work items from qb (lanes past nWork take part
// in the warp-made picks without a cell); pk: the warp's picks in shared
// memory.  Collision and candidate counts accumulate in nColl and nCandTot.
__device__ __forceinline__ void light_group(const CaseDev& cs, const Parcels& s, const int* __restrict__ start,
                                            double* smax, double* acc, const int2* __restrict__ work, int learned,
                                            const double* __restrict__ smaxSel, unsigned char* useR, float* exceed,
                                            float* obsMax, double2* audit, long long qb, long long nWork,
                                            uint32_t step, LightPicks& pk, unsigned& err, unsigned long long& nColl,
                                            unsigned long long& nCandTot, LightDefer* dq = nullptr) {
    const int lane = (int)(threadIdx.x & 31u);
    const long long C = cs.C;
    const long long q = qb + lane;
    int2 it = make_int2(0, 0);
    long long off = 0;
    int n = 0;
    if (q < nWork) {
        it = work[q];
        off = start[it.x];
        n = start[it.x + 1] - (int)off;
    }
    const long long c = it.x;
    int nCand = it.y;   // 0 past the end of the list
    if (nCand >= LIGHT_CAND || n > LIGHT_N) {
        // the list put a heavy cell here: record, never index past the picks
        err |= ERRB_BOUNDS;
        nCand = 0;
    }
    // every lane's picks, one cell at a time: coalesced loads of the
    // cell's ids and cell words (the next cell's issued before this
    // cell's picks), a warp minimum per pick
    const uint32_t myBase = pick_base(cs, (uint32_t)c, step);
    int ncN = __shfl_sync(0xFFFFFFFFu, nCand, 0);
    int nN = __shfl_sync(0xFFFFFFFFu, n, 0);
    long long offN = __shfl_sync(0xFFFFFFFFu, off, 0);
    uint32_t idAN = 0, idBN = 0, sAN = 0, sBN = 0;
    if (ncN) {
        if (lane < nN) {
            idAN = __ldg(s.id + offN + lane);
            sAN = __ldg(s.cellw + offN + lane);
        }
        if (lane + 32 < nN) {
            idBN = __ldg(s.id + offN + lane + 32);
            sBN = __ldg(s.cellw + offN + lane + 32);
        }
    }
    for (int L = 0; L < 32; ++L) {
        const int nc = min(ncN, LIGHT_CAND - 1), nL = nN;
        const uint32_t idA = idAN, idB = idBN, sA = sAN & 7u, sB = sBN & 7u;
        const uint32_t baseL = __shfl_sync(0xFFFFFFFFu, myBase, L);
        if (L + 1 < 32) {
            ncN = __shfl_sync(0xFFFFFFFFu, nCand, L + 1);
            nN = __shfl_sync(0xFFFFFFFFu, n, L + 1);
            offN = __shfl_sync(0xFFFFFFFFu, off, L + 1);
            idAN = idBN = sAN = sBN = 0;
            if (ncN) {
                if (lane < nN) {
                    idAN = __ldg(s.id + offN + lane);
                    sAN = __ldg(s.cellw + offN + lane);
                }
                if (lane + 32 < nN) {
                    idBN = __ldg(s.id + offN + lane + 32);
                    sBN = __ldg(s.cellw + offN + lane + 32);
                }
            }
        }
        if (nc == 0) continue;
        const bool vA = lane < nL, vB = lane + 32 < nL;
        // sub-cell occupancy, 8 bits per sub-cell (nL <= LIGHT_N < 256)
        uint32_t cnt0 = 0, cnt1 = 0;
        if (vA) (sA < 4 ? cnt0 : cnt1) += 1u << (8u * (sA & 3u));
        if (vB) (sB < 4 ? cnt0 : cnt1) += 1u << (8u * (sB & 3u));
        cnt0 = __reduce_add_sync(0xFFFFFFFFu, cnt0);
        cnt1 = __reduce_add_sync(0xFFFFFFFFu, cnt1);
        for (int k = 0; k < nc; ++k) {
            const uint32_t kP = pick_draw(cs, baseL, 2u * k);
            const int jP = warp_argmin(fmix32(kP ^ idA), vA, fmix32(kP ^ idB), vB);
            const uint32_t sub = __shfl_sync(0xFFFFFFFFu, jP < 32 ? sA : sB, jP & 31);
            const bool inSub = (((sub < 4 ? cnt0 : cnt1) >> (8u * (sub & 3u))) & 0xFFu) > 1;
            const uint32_t kQ = pick_draw(cs, baseL, 2u * k + 1u);
            const bool qA = vA && lane != jP && (!inSub || sA == sub);
            const bool qB = vB && lane + 32 != jP && (!inSub || sB == sub);
            const int jQ = warp_argmin(fmix32(kQ ^ idA), qA, fmix32(kQ ^ idB), qB);
            if (lane == L) {
                pk.pq[k][0][L] = (uint8_t)(jP < 0 ? 255 : jP);
                pk.pq[k][1][L] = (uint8_t)(jQ < 0 ? 255 : jQ);
            }
        }
    }
    __syncwarp();
    bool defer = false;
    long long dP = 0, dQ = 0;
    if (q < nWork) {
        const double R = smax[c];
        const double smax0 = learned ? smaxSel[c] : R;
        double stepMax = 0.0, collSep = 0.0;
        unsigned coll = 0;
        float2 au = make_float2(0.f, 0.f);
        // The lane tests candidates until one is accepted, then collides
        // it: lanes that reach an accepted candidate in the same pass run
        // the FP64 exchange together, whatever the rejections before it.
        // A single candidate is only tested here when its exchange can be
        // deferred to the warp's queue.
        int k = 0;
        if (dq && nCand == 1) {
            const int jP = pk.pq[0][0][lane], jQ = pk.pq[0][1][lane];
            k = 1;
            if (jP >= n || jQ >= n) {
                err |= ERRB_BOUNDS;
            } else {
                dP = off + jP;
                dQ = off + jQ;
                Rng r(cs, (uint32_t)c, step, cand_tag(0));
                CollRec P, Q;
                double cr2;
                if (test_candidate(cs, s, r, dP, dQ, smax0, &stepMax, &P, &Q, &cr2, audit ? &au : nullptr)) {
                    defer = true;
                    collSep += (double)coll_separation(s.r + dP, s.r + dQ);
                    ++coll;
                }
            }
        }
        while (k < nCand) {
            bool accepted = false;
            long long gP = 0, gQ = 0;
            Rng r(cs, (uint32_t)c, step, cand_tag(k));
            double cr2 = 0.0;
            CollRec P, Q;
            while (k < nCand) {
                const int jP = pk.pq[k][0][lane], jQ = pk.pq[k][1][lane];
                r = Rng(cs, (uint32_t)c, step, cand_tag(k));
                ++k;
                if (jP >= n || jQ >= n) {
                    err |= ERRB_BOUNDS;
                    continue;
                }
                gP = off + jP;
                gQ = off + jQ;
                if (test_candidate(cs, s, r, gP, gQ, smax0, &stepMax, &P, &Q, &cr2, audit ? &au : nullptr)) {
                    accepted = true;
                    break;
                }
            }
            if (accepted) {
                collide_candidate(cs, s, r, gP, gQ, P, Q, cr2, &collSep, &err);
                ++coll;
            }
        }
        cell_epilogue(smax, c, R, smax0, stepMax, learned, useR, exceed, obsMax, audit, au);
        if (coll) {
            acc[(cs.nSpecies * SACC + CACC_NCOLLS) * C + c] += (double)coll;
            acc[(cs.nSpecies * SACC + CACC_COLLSEP) * C + c] += collSep;
        }
        nColl += coll;
        nCandTot += (unsigned long long)nCand;
    }
    if (dq) {
        // queue the deferred exchanges; run 32 once 32 are waiting
        const unsigned m = __ballot_sync(0xFFFFFFFFu, defer);
        int cnt = dq->count;
        if (defer) dq->e[cnt + __popc(m & ((1u << lane) - 1u))] = make_int4((int)dP, (int)dQ, (int)c, 0);
        cnt += __popc(m);
        __syncwarp();
        if (cnt >= 32) {
            exchange_deferred(cs, s, dq->e[lane], step, &err);
            __syncwarp();
            if (lane < cnt - 32) dq->e[lane] = dq->e[32 + lane];
            cnt -= 32;
        }
        __syncwarp();
        if (lane == 0) dq->count = cnt;
    }
    __syncwarp();   // the picks are read before the next cells overwrite them
}

// one lane per light cell, its candidates one after the other; blockDim.x
// (the cells per CTA) is 32, 64 or 128, with one LightPicks and one
// LightDefer per warp in dynamic shared memory
__global__ void __launch_bounds__(128, 4)
k_collide_light(CaseDev cs, Parcels s, const int* __restrict__ start, double* smax, double* acc, Counters* ctr,
                const int2* __restrict__ work, int learned, const double* __restrict__ smaxSel, unsigned char* useR,
                float* exceed, float* obsMax, double2* audit) {
    extern __shared__ __align__(16) unsigned char lightSmem[];
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    LightPicks& pk = reinterpret_cast<LightPicks*>(lightSmem)[w];
    LightDefer* dq = reinterpret_cast<LightDefer*>(lightSmem + nw * sizeof(LightPicks)) + w;
    const unsigned lane = lane_id();
    if (lane == 0) dq->count = 0;
    __syncwarp();
    const uint32_t step = (uint32_t)ctr->step;
    const long long nWork = (long long)ctr->nWork;
    const long long nHeavy = (long long)ctr->nHeavy;
    unsigned err = 0;
    unsigned long long nColl = 0, nCandTot = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long qb = nHeavy + (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); qb < nWork;
         qb += stride)
        light_group(cs, s, start, smax, acc, work, learned, smaxSel, useR, exceed, obsMax, audit, qb, nWork, step,
                    pk, err, nColl, nCandTot, dq);
    // the exchanges still waiting
    if ((int)lane < dq->count) exchange_deferred(cs, s, dq->e[lane], step, &err);
    if (nColl) atomicAdd(&ctr->coll, nColl);
    if (nCandTot) atomicAdd(&ctr->cand, nCandTot);
    if (err) atomicOr(&ctr->err, err);
}

// ------------------------------------------------------------ Bernoulli trials
// simplifiedBernoulliTrials::collide (simplifiedBernoulliTrials.C:88-190):
// every cell with two or more parcels has nC - 1 trials; trial p pairs the
// p-th member of the cell's list with one of the k = nC - 1 - p members after
// it (randomLabel(1, k)) and collides them with probability
// k FN dt / V sigma_T c_R.  There is no maximum and no sub-cell.
__global__ void k_sbt_select(CaseDev cs, const int* __restrict__ start, Counters* ctr, int* ncCell,
                             unsigned* slotCount) {
    __shared__ unsigned hist[2 * NBUCKET];
    if (threadIdx.x < 2 * NBUCKET) hist[threadIdx.x] = 0;
    __syncthreads();
    unsigned err = 0;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < cs.C;
         c += (long long)gridDim.x * blockDim.x) {
        const int n = start[c + 1] - start[c];
        int nt = 0;
        if (n > 1) {
            if (n > cs.maxCellParcels) err |= ERRB_DENSE;
            else nt = n - 1;
        }
        ncCell[c] = nt;
        if (nt > 0) atomicAdd(&hist[NBUCKET + bucket_of(nt)], 1u);
    }
    __syncthreads();
    if (threadIdx.x < 2 * NBUCKET && hist[threadIdx.x]) atomicAdd(&slotCount[threadIdx.x], hist[threadIdx.x]);
    if (err) atomicOr(&ctr->err, err);
}

// one lane per listed cell, its trials one after the other in list order
__global__ void __launch_bounds__(WARPS * 32, 4)
k_sbt_collide(CaseDev cs, Parcels s, const int* __restrict__ start, double* acc, Counters* ctr,
              const int2* __restrict__ work, const uint16_t* __restrict__ perm) {
    const uint32_t step = (uint32_t)ctr->step;
    const long long nWork = (long long)ctr->nWork;
    const long long C = cs.C;
    const double prob1u = cs.FN * cs.dt / cs.V;
    unsigned err = 0;
    unsigned long long nColl = 0, nTrials = 0;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nWork;
         q += (long long)gridDim.x * blockDim.x) {
        const int c = work[q].x;
        const long long off = start[c];
        const int n = start[c + 1] - (int)off;
        const double prob1 = cs.cellV ? cs.FN * cs.dt / cs.cellV[c] : prob1u;
        double stepMax = 0.0, collSep = 0.0;
        unsigned coll = 0;
        for (int p = 0; p < n - 1; ++p) {
            Rng r(cs, (uint32_t)c, step, cand_tag(p));
            const int k = n - 1 - p;
            const int qq = p + r.label(1, k, &err);
            const long long gP = off + perm[off + p];
            const long long gQ = off + perm[off + qq];
            // accept when k prob1 sigma > U, i.e. sigma > U / (k prob1)
            if (run_candidate(cs, s, r, gP, gQ, 1.0 / (k * prob1), &stepMax, &collSep, &err)) ++coll;
        }
        if (coll) {
            acc[(cs.nSpecies * SACC + CACC_NCOLLS) * C + c] += (double)coll;
            acc[(cs.nSpecies * SACC + CACC_COLLSEP) * C + c] += collSep;
        }
        nColl += coll;
        nTrials += (unsigned long long)(n - 1);
    }
    if (nColl) atomicAdd(&ctr->coll, nColl);
    if (nTrials) atomicAdd(&ctr->cand, nTrials);
    if (err) atomicOr(&ctr->err, err);
}

}  // namespace tile
