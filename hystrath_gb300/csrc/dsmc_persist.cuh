// dsmc_persist.cuh -- the machinery of the persistent batch kernels, shared by
// the move/sort launch (dsmc_move.cu) and the collision launch
// (dsmc_collide.cu).
//
// A persistent launch runs every phase of its half of a step for all cases
// of a batch.  Its CTAs are co-resident (a cooperative launch), wait for one
// another at a grid barrier between phases, and within a phase take work
// items -- (case, tile) pairs -- from one atomic ticket counter per phase, so
// that the tiles of small and large cases share the SMs.  Every barrier wait
// is bounded: a wait that runs out sets an error bit in the control block,
// and every CTA leaves the kernel at the next barrier.
#pragma once

namespace persist {

constexpr unsigned long long BAR_SPIN_LIMIT = 1ull << 24;   // waits of >= 64 ns: > 1 s

// Grid barrier: the last CTA to arrive resets the count and advances the
// generation; the others wait (bounded) for the generation to change.
// Returns false when the kernel must stop (a wait ran out here or earlier).
__device__ __forceinline__ bool grid_sync(BatchCtl* ctl) {
    __syncthreads();
    __shared__ int stop;
    if (threadIdx.x == 0) {
        volatile unsigned* gen = &ctl->barGen;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(&ctl->barCount, 1u) == gridDim.x - 1) {
            ctl->barCount = 0;
            __threadfence();
            atomicAdd(&ctl->barGen, 1u);
        } else {
            unsigned long long it = 0;
            while (*gen == g) {
                if (++it > BAR_SPIN_LIMIT) {
                    atomicOr(&ctl->err, BATCH_ERR_BARRIER);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        stop = (*(volatile unsigned*)&ctl->err) != 0;
    }
    __syncthreads();
    return !stop;
}

// Prefix sums of the phase's work items per case into pre[0..n] (shared
// memory of the CTA); count(i) gives case i's items.  Returns the total.
template <class Count>
__device__ __forceinline__ long long phase_items(int n, long long* pre, Count count) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) pre[i + 1] = count(i);
    __syncthreads();
    if (threadIdx.x < 32) {
        // warp 0: each lane sums a contiguous chunk, a shuffle scan of the
        // chunk totals, then each lane writes its chunk's running sums
        const int lane = threadIdx.x;
        const int per = (n + 31) / 32;
        const int a = lane * per, b = min(a + per, n);
        long long t = 0;
        for (int i = a; i < b; ++i) t += pre[i + 1];
        long long x = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += y;
        }
        long long run = x - t;
        for (int i = a; i < b; ++i) {
            run += pre[i + 1];
            pre[i + 1] = run;
        }
        if (lane == 0) pre[0] = 0;
    }
    __syncthreads();
    return pre[n];
}

// The next work item of the phase for this CTA (all threads get it), or -1.
__device__ __forceinline__ long long next_item(BatchCtl* ctl, int phase, long long total) {
    __shared__ long long item;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned long long t = atomicAdd(&ctl->ticket[phase], 1ull);
        item = (long long)t < total ? (long long)t : -1;
    }
    __syncthreads();
    return item;
}

// The case of global item q: the last i with pre[i] <= q.
__device__ __forceinline__ int item_case(const long long* pre, int n, long long q) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= q) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

}  // namespace persist
