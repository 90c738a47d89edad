// dsmc_kernels.h -- host-side launchers of the dsmcFoam+ step kernels.
#pragma once

#include <cuda_runtime.h>

#include "dsmc_device.cuh"

namespace dsmc {

// Device-resident counters of one cloud (one cache line each).
struct Counters {
    long long n;            // parcels in the current sorted buffer
    long long nMoved;       // parcels in [0, nMoved) taken by move/scatter (n + inserted)
    long long nKept;        // parcels after the last sort
    long long step;
    unsigned long long coll, cand;          // last step
    unsigned long long collTot, candTot;
    unsigned long long wallHits, inserted, deleted;
    long long nextId;
    long long sampleSteps;
    unsigned err;
    int bigCells;           // listed cells too large for one warp to order
    long long inflowTotal;
    unsigned long long nSlow;   // parcels deferred to the boundary-path kernel this step
    int pendingSample;          // the state after the last collide is still to be sampled
    int unflushed;              // samples held in the fixed-point sums
    unsigned long long nWork;   // cells with candidates this step
    unsigned long long nHeavy;  // of which one warp each (the first nHeavy of the work list)
    // spatial decomposition: parcels that left for another domain this step
    // (their indices in migList) and parcels received from other domains;
    // the inflow's insertions into owned cells (inflowTotal counts every
    // inflow face: the parcel ids of the undivided case)
    unsigned long long nMig;
    long long migIn;
    long long inflowLocal;
};

// Launch shape of one cloud's step, chosen by the autotuner: threads per CTA
// of the parcel-streaming kernels (move, sample, sort) and their CTAs per
// SM, and cells per CTA of the one-lane-per-cell collision kernel.
struct LaunchCfg {
    int streamThreads = 256;     // 128, 256 or 512
    int streamCtasPerSm = 8;
    int lightCells = 128;        // 32, 64 or 128 (one warp per 32 cells)
};

struct StepBuffers {
    LaunchCfg cfg;
    Parcels a, b;                 // current / other particle buffers
    int* count;               // [C]
    int* start;               // [C+1]
    int* blockSums;           // scan scratch
    double* smax;             // sigmaTcRMax [C]
    double* rem;              // collisionSelectionRemainder [C]
    double* acc;              // sampling accumulators, accumulator-major [nAcc][C]
    long long* sfix;          // one sample's fixed-point sums [nSpecies*SACC][C]
    // measureHeatFluxShearStress (null when off): per species the velocity
    // moments of the samples, [nSpecies*MACC][C] (MACC_* order)
    double* macc;
    double* wall;             // [nBFaces][W_N]
    int* bfPatch;             // [nBFaces]
    int2* work;               // [C] cells with candidates: (cell, candidates)
    int* bigList;             // [C] work indices of cells ordered by one block
    int* ncCell;              // [C] candidates of each cell this step
    unsigned* buckets;        // [32] work-slot counts and cursors
    uint16_t* perm;           // [capacity] canonical member order of the cells with candidates
    uint4* subs;              // [C] sub-cell starts in that order, per work item
    float* obsMax;            // [C] largest sigma_T c_R among this step's candidates of the cell
    // learned selection (used when a model is attached)
    float4* feat;             // [C] log n, log T_tr, speed ratio, valid
    float* pred;              // [C] predicted (sigma_T c_R)max
    unsigned char* useR;      // [C] 1: the cell has fallen back to the running maximum
    float* exceed;            // [C] largest product seen above a prediction (0: none)
    double* smaxSel;          // [C] the maximum this step's selection used
    // selection audit (null when off): per cell, summed over candidates,
    // x = sigma_T c_R / max (the expected acceptances) and
    // y = max(0, sigma_T c_R / max - 1) (the expected collisions lost
    // because the maximum used was below the product)
    double2* audit;
    int* slowList;            // [capacity] parcels that take the boundary path this step
    // spatial decomposition (allocated by dsmc_set_domain): indices of the
    // step's migrants, their packed records (MIGRANT_WORDS words each) and a
    // staging buffer for migrants handed over in host memory
    int* migList;             // [migCap]
    uint32_t* migOut;         // [migCap * MIGRANT_WORDS]
    uint32_t* migIn;          // [migInCap * MIGRANT_WORDS]
    long long migCap;
    long long migInCap;
    int* inflowOffLocal;      // [nInflowFaces * nSpecies + 1] inflow offsets of the owned faces
    int2* sortSrc;            // [capacity] (source index, cell word) of each destination slot of the sort
    // inflow
    int nInflowFaces;
    long long* inflowFace;    // boundary face ids with inflow [nInflowFaces]
    int* inflowSide;          // side of each inflow face
    int* inflowCell;          // owner cell
    double* inflowAcc;        // [nInflowFaces * nSpecies]
    double* inflowTerm;       // [nInflowFaces * nSpecies] parcels per step (Bird eq. 4.22)
    int* inflowCount;         // [nInflowFaces * nSpecies]
    int* inflowOff;           // [nInflowFaces * nSpecies + 1]
    double inflowND[DSMC_MAX_PATCHES][DSMC_MAX_SPECIES];
    long long capacity;
    Counters* ctr;
};

struct InflowPatchDev {
    double nd[DSMC_MAX_SPECIES];
    double Ttra, Trot, Tvib;
    double U[3];
};

struct InflowDev {
    int nPatches;
    int pad;
    InflowPatchDev p[DSMC_MAX_PATCHES];
};

int scan_scratch_ints(long long C);

void launch_count(const CaseDev& cs, const StepBuffers& B, const Parcels& s, cudaStream_t st);
// mid (optional): an event recorded between the fast path and the boundary path
// A migrant between domains: the 64-byte parcel record and its cell word.
constexpr int MIGRANT_WORDS = 17;

// deferPos: the sort follows in the same step, and the end points of plain
// moves are left to its gather (launch_scatter with movePending)
// range: 0 every parcel [0, nMoved), then the boundary path; 1 the last
// step's parcels [0, n) only (needs nothing of this step's inflow); 2 the
// inserted parcels [n, nMoved), then the boundary path
void launch_move(const CaseDev& cs, const StepBuffers& B, const Parcels& s, cudaStream_t st,
                 cudaEvent_t mid = nullptr, bool deferPos = false, int range = 0);
void launch_scan(const CaseDev& cs, const StepBuffers& B, cudaStream_t st);
// mid (optional): an event recorded between the index scatter and the gather
void launch_scatter(const CaseDev& cs, const StepBuffers& B, const Parcels& src, const Parcels& dst,
                    cudaStream_t st, cudaEvent_t mid = nullptr, bool movePending = false);
void launch_finish_sort(const StepBuffers& B, cudaStream_t st);
// spatial decomposition: the step's migrants packed into B.migOut (their end
// points made) and dropped from the cloud; n migrants at src (device
// memory, MIGRANT_WORDS words each) appended at slot base and counted
void launch_pack_migrants(const CaseDev& cs, const StepBuffers& B, const Parcels& s, cudaStream_t st);
void launch_unpack_migrants(const CaseDev& cs, const StepBuffers& B, const Parcels& s, const uint32_t* src,
                            long long n, long long base, cudaStream_t st);
// sample count, pending sample and unflushed samples back to zero (a reset
// of the time averages)
void launch_reset_sample_counters(const StepBuffers& B, cudaStream_t st);
// learned != 0: the selection uses the prediction (or the running maximum of
// cells that fell back to it) instead of the running maximum alone
// marks (optional): two events, recorded after the selection, list and
// ordering kernels and after the heavy-cell kernel
// side (optional, without marks): the heavy cells' kernel runs on it, forked
// from st by the event fork and joined back by join, beside the light
// cells' kernel on st (disjoint cells: the state is the same either way)
void launch_collide(const CaseDev& cs, const StepBuffers& B, const Parcels& s, int learned, cudaStream_t st,
                    cudaEvent_t* marks = nullptr, cudaStream_t side = nullptr, cudaEvent_t fork = nullptr,
                    cudaEvent_t join = nullptr);
// per-cell features of the learned maximum; every > 0: only on steps that are
// multiples of every, every == 0: always; resetFallback: the cells go back to
// the prediction
// resetFallback: a prediction follows (the cells' fallback flags are cleared
// and their remembered excess multiplied by forget)
void launch_cell_features(const CaseDev& cs, const StepBuffers& B, const Parcels& s, int every, int resetFallback,
                          cudaStream_t st, float forget = 1.f);
// compacts (features, log observed maximum) of the cells with candidates in
// the last step; returns the count in *nOut (device)
void launch_learn_compact(const CaseDev& cs, const StepBuffers& B, long long maxRows, float* X, float* Y,
                          unsigned long long* nOut, cudaStream_t st);

struct MlpModel;
// prediction for n rows of features: out = exp(net + margin); with step !=
// nullptr and every > 0 only when *step is a multiple of every
void mlp_launch_infer(const MlpModel* m, const float4* X, long long n, float* out, float margin,
                      const long long* step, int every, cudaStream_t st);
// one-time kernel attributes (large dynamic shared memory); call before the
// first capture
int collide_init();
// Sampling: the move kernel folds a pending sample of the pre-move state into
// per-cell fixed-point sums; launch_sample_flush takes a pending sample of the
// current state when no move follows.  Both then add the sums to the FP64
// accumulators and count the sample.
// force: add the fixed-point sums to the FP64 accumulators now (otherwise
// every 32 samples).
void launch_sample_commit(const CaseDev& cs, const StepBuffers& B, int force, cudaStream_t st);
void launch_sample_flush(const CaseDev& cs, const StepBuffers& B, const Parcels& s, int force, cudaStream_t st);
void launch_set_pending(const StepBuffers& B, cudaStream_t st);
void launch_end_step(const StepBuffers& B, cudaStream_t st);
void launch_inflow(const CaseDev& cs, const InflowDev& in, const StepBuffers& B, const Parcels& s,
                   cudaStream_t st);
void launch_init_count(const CaseDev& cs, const double* dnd, const unsigned char* solid, int* cellCounts,
                       cudaStream_t st);
void launch_init_fill(const CaseDev& cs, const StepBuffers& B, const Parcels& s, const double* dnd,
                      const unsigned char* solid, const int* cellOff, double Ttra, const double* Txyz,
                      double Trot, double Tvib, const double* U, cudaStream_t st);
void launch_count_n(const Parcels& s, long long n, int* count, cudaStream_t st);
void launch_ids_from_records(const Parcels& s, long long n, cudaStream_t st);
// dsmcFluxSurface: out2 = {sum of parcel sums x w, sum of mass sums x w} over
// the nF faces (device arrays) and the species of mask
void launch_flux_surface(const CaseDev& cs, const int* faces, const double* w, int nF, unsigned mask,
                         double* out2, cudaStream_t st);
void launch_pack(const Parcels& dst, long long n, const double* pos, const double* U, const double* erot,
                 const int* vib, const int* species, const unsigned* id, int nSpecies, unsigned* flags,
                 int write, cudaStream_t st);
void launch_zero_step(const StepBuffers& B, cudaStream_t st);
void launch_cellw(const CaseDev& cs, const Parcels& s, long long n, cudaStream_t st);
void launch_remainder_init(const CaseDev& cs, double* rem, cudaStream_t st);
// velocity moments of the current (cell-sorted) state, added to B.macc
void launch_sample_moments(const CaseDev& cs, const StepBuffers& B, const Parcels& s, cudaStream_t st);
void launch_field(const CaseDev& cs, const StepBuffers& B, int which, double* out,
                  int measureMfp, double mfpTref, unsigned speciesMask, cudaStream_t st);
void launch_info(const CaseDev& cs, const Parcels& s, const Counters* ctr, double* out7,
                 cudaStream_t st);

// ------------------------------------------------------------ batch
// One case of a batch as the persistent batch kernels see it: its constants,
// its buffers, and the parcel buffer the step starts in (src) and the one the
// sort fills (dst).
struct BatchSlot {
    CaseDev cs;
    StepBuffers B;
    Parcels src, dst;
};

// Control block of the persistent batch kernels: the grid barrier (arrival
// count and generation), an error word (a barrier wait that ran out), and one
// work-queue ticket per phase (zeroed before every launch).
constexpr int BATCH_PHASES = 16;
constexpr int BATCH_TICKETS_MOVE = 0;      // tickets 0..8: the phases of the move/sort launch
constexpr int BATCH_TICKETS_COLLIDE = 9;   // tickets 9..15: the phases of the collision launch
constexpr int BATCH_MAX_CASES = 1024;
struct BatchCtl {
    unsigned barCount;
    unsigned barGen;
    unsigned err;
    unsigned pad;
    unsigned long long ticket[BATCH_PHASES];
};
constexpr unsigned BATCH_ERR_BARRIER = 1u;

// The two persistent launches of one batched step over n cases (slots in
// device memory): the move and sort phases, then the collision phases.  Both
// are cooperative launches sized to the occupancy of their thread count.
int batch_move_grid(int threads);
int batch_collide_grid(int threads);
cudaError_t launch_batch_move(const BatchSlot* slots, int n, BatchCtl* ctl, int threads, cudaStream_t st);
cudaError_t launch_batch_collide(const BatchSlot* slots, int n, BatchCtl* ctl, int threads, cudaStream_t st);

// field selectors of launch_field
enum {
    F_RHON = 0, F_RHOM, F_UX, F_UY, F_UZ, F_TTRA, F_P, F_TROT, F_TVIB, F_TOV, F_NMEAN, F_NCOLLS,
    F_MEASCR, F_MEANCR, F_MFP, F_MA, F_RHOM_ERR, F_U_ERR, F_T_ERR, F_P_ERR,
    // measureHeatFluxShearStress: pressure tensor xx xy xz yy yz zz, shear
    // stress tensor in the same order, heat flux vector x y z
    F_PXX, F_PXY, F_PXZ, F_PYY, F_PYZ, F_PZZ, F_SXX, F_SXY, F_SXZ, F_SYY, F_SYZ, F_SZZ, F_QX, F_QY, F_QZ,
    F_COUNT_FIELDS
};

}  // namespace dsmc
