// Device building blocks of the persistent Krylov kernels: bounded grid
// barriers, fixed-order reductions, the scalar state of a solve and the
// SELL row product.
#pragma once
#include "tf_internal.cuh"

namespace tf {

constexpr int kKryThreads = 256;

// Loads of vectors that the same persistent launch writes (basis vectors,
// search directions, iterates) and reads again after a grid barrier.  They go
// through L1 (ld.global.ca): neighbouring rows gather largely the same
// entries, and an 8-byte gather that misses L1 costs a whole 32-byte L2
// sector.  Every such read happens after the barrier of the step that wrote
// the data, i.e. after thread 0's fence following the release it observed and
// the block's bar.sync, which orders it after the writes in the memory model.
template <class T>
__device__ __forceinline__ T kld(const T* p) { return __ldca(p); }

// ---------------------------------------------------------------------------
// grid barrier with a bounded wait
// ---------------------------------------------------------------------------
struct GridSync {
    unsigned* count;
    unsigned* gen;
    int* status;
};
constexpr long long kSpinLimit = 20000000;  // ~1-2 s with the backoff below

__device__ __forceinline__ bool grid_barrier(const GridSync& g) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = g.gen;
        const unsigned my = *vgen;
        __threadfence();
        if (atomicAdd(g.count, 1u) == gridDim.x - 1) {
            *g.count = 0;
            __threadfence();
            atomicAdd(g.gen, 1u);
        } else {
            long long spins = 0;
            while (*vgen == my) {
                if (++spins > kSpinLimit) {
                    atomicCAS(g.status, 0, TF_ERR_WATCHDOG);
                    break;
                }
                if (spins > 256) __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
    __shared__ int st;
    if (threadIdx.x == 0) st = *((volatile int*)g.status);
    __syncthreads();
    return st == 0;
}

// ---------------------------------------------------------------------------
// reductions: warp xor-trees (every lane ends with the same sum), one FP64
// partial per block, and a fixed-order sum of all partials in every block
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T warp_sum(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Eight sums over the warp at once (a transposing butterfly): round 16 swaps
// half of the values between the half-warps, round 8 and 4 likewise, then two
// plain xor rounds; 9 shuffles instead of 40, in independent chains.  Lane l
// returns the total of value warp_sum8_index(l); the tree is fixed, so the
// result does not depend on timing.
__device__ __forceinline__ int warp_sum8_index(int lane) {
    return ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
}
template <class T>
__device__ __forceinline__ T warp_sum8(const T (&v)[8], int lane) {
    const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
    T a4[4], a2[2];
#pragma unroll
    for (int q = 0; q < 4; ++q)
        a4[q] = (b4 ? v[q + 4] : v[q]) + __shfl_xor_sync(0xffffffffu, b4 ? v[q] : v[q + 4], 16);
#pragma unroll
    for (int q = 0; q < 2; ++q)
        a2[q] = (b3 ? a4[q + 2] : a4[q]) + __shfl_xor_sync(0xffffffffu, b3 ? a4[q] : a4[q + 2], 8);
    T a1 = (b2 ? a2[1] : a2[0]) + __shfl_xor_sync(0xffffffffu, b2 ? a2[0] : a2[1], 4);
    a1 += __shfl_xor_sync(0xffffffffu, a1, 2);
    a1 += __shfl_xor_sync(0xffffffffu, a1, 1);
    return a1;
}

template <int NV, class T>
__device__ void block_partials(T (&v)[NV], double* part /* [nblocks][NV] */) {
    __shared__ double red[NV][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < NV; ++k) {
        const T x = warp_sum(v[k]);
        if (lane == 0) red[k][w] = (double)x;
    }
    __syncthreads();
    if (w == 0)
        for (int k = 0; k < NV; ++k) {
            double x = lane < nw ? red[k][lane] : 0.;
            x = warp_sum(x);
            if (lane == 0) part[(size_t)blockIdx.x * NV + k] = x;
        }
    __syncthreads();
}

template <int NV>
__device__ void grid_reduce(const double* part, double (&out)[NV]) {
    __shared__ double red[NV][32];
    __shared__ double res[NV];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < NV; ++k) {
        double x = 0.;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) x += __ldcg(part + (size_t)b * NV + k);
        x = warp_sum(x);
        if (lane == 0) red[k][w] = x;
    }
    __syncthreads();
    if (w == 0)
        for (int k = 0; k < NV; ++k) {
            double x = lane < nw ? red[k][lane] : 0.;
            x = warp_sum(x);
            if (lane == 0) res[k] = x;
        }
    __syncthreads();
    for (int k = 0; k < NV; ++k) out[k] = res[k];
    __syncthreads();
}

// Barrier and reduction in one: every block has written its NV partials; the
// last block to arrive sums all of them in a fixed order (so the result does
// not depend on which block is last), publishes the NV sums, and releases the
// others.  Cost: one reduction of nblocks values instead of one per block.
template <int NV>
__device__ bool grid_sync_reduce(const GridSync& g, const double* part, double* result, double (&out)[NV]) {
    __shared__ int last;
    __shared__ double red[NV][32];
    __shared__ int st;
    __syncthreads();
    unsigned my = 0;
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = g.gen;
        my = *vgen;
        __threadfence();
        last = atomicAdd(g.count, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last) {
        __threadfence();
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int k = 0; k < NV; ++k) {
            double x = 0.;
            for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) x += __ldcg(part + (size_t)b * NV + k);
            x = warp_sum(x);
            if (lane == 0) red[k][w] = x;
        }
        __syncthreads();
        if (w == 0)
            for (int k = 0; k < NV; ++k) {
                double x = lane < nw ? red[k][lane] : 0.;
                x = warp_sum(x);
                if (lane == 0) result[k] = x;
            }
        __syncthreads();
        if (threadIdx.x == 0) {
            *g.count = 0;
            __threadfence();
            atomicAdd(g.gen, 1u);
        }
    } else if (threadIdx.x == 0) {
        volatile unsigned* vgen = g.gen;
        long long spins = 0;
        while (*vgen == my) {
            if (++spins > kSpinLimit) {
                atomicCAS(g.status, 0, TF_ERR_WATCHDOG);
                break;
            }
            if (spins > 256) __nanosleep(32);
        }
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) st = *((volatile int*)g.status);
    __syncthreads();
    if (st != 0) return false;
    for (int k = 0; k < NV; ++k) out[k] = __ldcg(result + k);
    return true;
}

// Scalar state of a persistent Krylov solve in global memory.  Only thread 0
// of the block that completes a grid step (the last to arrive) writes it, and
// only between its reduction and the barrier release; every block copies it
// into shared memory after the release.  FP64 arithmetic issues at a small
// fraction of the FP32 rate on GB300, so the scalar recurrences (divisions,
// square roots, convergence tests) run once per step instead of once per
// thread.  8-byte fields, copied as words.
struct KryScal {
    double rho, r_last, normb, resid, alpha, beta;
    long long it, done, converged, true_res, updates, pad;
};
constexpr int kScalWords = (int)(sizeof(KryScal) / 8);

// grid_sync_reduce with a scalar update: the last block sums the partials in a
// fixed order and thread 0 runs f(sums, state) on the global state.
template <int NV, class F>
__device__ bool grid_step(const GridSync& g, const double* part, KryScal* gsc, KryScal& ssc, F f) {
    __shared__ int last;
    __shared__ double red[NV][32];
    __shared__ int st;
    __syncthreads();
    unsigned my = 0;
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = g.gen;
        my = *vgen;
        __threadfence();
        last = atomicAdd(g.count, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last) {
        __threadfence();
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int k = 0; k < NV; ++k) {
            double x = 0.;
            for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) x += __ldcg(part + (size_t)b * NV + k);
            x = warp_sum(x);
            if (lane == 0) red[k][w] = x;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double sums[NV];
            for (int k = 0; k < NV; ++k) {
                double x = 0.;
                for (int ww = 0; ww < nw; ++ww) x += red[k][ww];
                sums[k] = x;
            }
            f(sums, *gsc);
            __threadfence();
            *g.count = 0;
            __threadfence();
            atomicAdd(g.gen, 1u);
        }
    } else if (threadIdx.x == 0) {
        volatile unsigned* vgen = g.gen;
        long long spins = 0;
        while (*vgen == my) {
            if (++spins > kSpinLimit) {
                atomicCAS(g.status, 0, TF_ERR_WATCHDOG);
                break;
            }
            if (spins > 256) __nanosleep(32);
        }
        __threadfence();
    }
    if (threadIdx.x == 0) {
        st = *((volatile int*)g.status);
        const unsigned long long* src = reinterpret_cast<const unsigned long long*>(gsc);
        unsigned long long* dst = reinterpret_cast<unsigned long long*>(&ssc);
        for (int k = 0; k < kScalWords; ++k) dst[k] = __ldcg(src + k);
    }
    __syncthreads();
    return st == 0;
}

// ---------------------------------------------------------------------------
// barrier + all-reduce on one monotone arrival counter
//
// Every block publishes NV partial sums, arrives on a 64-bit counter that is
// never reset inside a launch and waits until the counter reaches
// (epoch + 1) * gridDim.x.  Arrival is a release of the whole block's writes:
// bar.sync, then thread 0's fence (cumulative over the writes the barrier
// ordered before it), then the atomic; the wait ends with an acquire (the
// polling load and a fence) before the block's bar.sync.  Then
// every block sums all partials itself, warp k taking value k over the blocks
// in one fixed order, so all blocks hold bitwise the same sums and derive the
// same scalars: the critical path is the arrival, one poll round trip and one
// load of the partials, with no last-arriver reduction and no published
// result to read back.  Partials alternate between two buffers by epoch
// parity; a block cannot be more than one barrier ahead of a reader.
// ---------------------------------------------------------------------------
constexpr int kArMax = 8;  // values per all-reduce (<= warps per block)

struct GridAR {
    unsigned long long* count;  // arrivals since launch (zeroed by the host)
    float* partf;               // [2][nblocks][kArMax]
    double* partd;              // [2][nblocks][kArMax]
    int* status;
};

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_release_add_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void fence_acquire_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// Arrive and wait for all blocks of this epoch; false after a watchdog
// timeout.  Arrival is one release reduction by thread 0 after the block's
// bar.sync (cumulative: it releases every write the barrier ordered before
// it); the wait spins on relaxed loads and ends with one acquire fence, which
// the closing bar.sync extends to the whole block.  No sequentially
// consistent fence is needed on either side.
__device__ __forceinline__ bool ar_arrive_wait(const GridAR& g, unsigned long long epoch, int* st_sh) {
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned long long target = (epoch + 1) * (unsigned long long)gridDim.x;
        red_release_add_u64(g.count, 1ull);
        long long spins = 0;
        while (ld_relaxed_u64(g.count) < target) {
            if (++spins > kSpinLimit) {
                atomicCAS(g.status, 0, TF_ERR_WATCHDOG);
                break;
            }
            if (spins > 256) __nanosleep(32);
        }
        fence_acquire_gpu();
        *st_sh = *((volatile int*)g.status);
    }
    __syncthreads();
    return *st_sh == 0;
}

template <class T>
__device__ __forceinline__ T* ar_part(const GridAR& g);
template <>
__device__ __forceinline__ float* ar_part<float>(const GridAR& g) { return g.partf; }
template <>
__device__ __forceinline__ double* ar_part<double>(const GridAR& g) { return g.partd; }

// the kArMax values of one block's record (L2 only: written by other SMs)
__device__ __forceinline__ void ar_load_record(const float* p, float (&r)[8]) {
    const float4 a = __ldcg(reinterpret_cast<const float4*>(p)), b = __ldcg(reinterpret_cast<const float4*>(p) + 1);
    r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w;
    r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
}
__device__ __forceinline__ void ar_load_record(const double* p, double (&r)[8]) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const double2 a = __ldcg(reinterpret_cast<const double2*>(p) + q);
        r[2 * q] = a.x;
        r[2 * q + 1] = a.y;
    }
}
static_assert(kArMax == 8, "records of eight values");

// Sums v[k] over every thread of the grid into out[k] (identical in all
// threads).  Call from all threads of every block, in uniform control flow.
template <class T, int NV>
__device__ bool grid_allreduce(const GridAR& g, unsigned long long& epoch, const T (&v)[NV], T (&out)[NV]) {
    static_assert(NV >= 1 && NV <= kArMax, "all-reduce width");
    constexpr int kReadWarps = 8;  // warps that load block records
    __shared__ T red[kArMax][32];
    __shared__ T tot_w[kArMax][kReadWarps];
    __shared__ T res[kArMax];
    __shared__ int st;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T* part = ar_part<T>(g) + (size_t)(epoch & 1) * gridDim.x * kArMax;
    // all NV sums of a warp at once (transposing butterfly, 9 shuffles)
    const int idx = warp_sum8_index(lane);
    {
        T v8[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v8[k] = k < NV ? v[k] : T(0);
        const T tot = warp_sum8(v8, lane);
        if ((lane & 3) == 0 && idx < NV) red[idx][w] = tot;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        T x = T(0);
        for (int ww = 0; ww < nw; ++ww) x += red[threadIdx.x][ww];
        part[(size_t)blockIdx.x * kArMax + threadIdx.x] = x;
    }
    if (!ar_arrive_wait(g, epoch, &st)) return false;
    ++epoch;
    // the block records (kArMax values: 32 or 64 bytes, 16-byte loads, one
    // L2 sector request per record) are spread over up to kReadWarps warps,
    // one record per lane, so that they are in flight at once; each warp sums
    // its records (in the order of the chunks it took, then the fixed shuffle
    // tree), and NV lanes of warp 0 add the warp totals in warp order, so
    // every block derives the same bits.  Only the NV used values are added:
    // FP64 adds issue at a small fraction of the FP32 rate.
    // FP64 records (the FP64 solvers, up to 3 blocks per SM) stay on one warp:
    // the warp-sum trees of eight warps cost more FP64 issue than the
    // sequential loads save
    const int nchunks = (int)((gridDim.x + 31) / 32);
    const int nread = sizeof(T) == 8 ? 1 : nw < kReadWarps ? nw : kReadWarps;
    if (w < nread) {
        T acc[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) acc[k] = T(0);
        for (int ch = w; ch < nchunks; ch += nread) {
            const unsigned b = (unsigned)ch * 32u + (unsigned)lane;
            if (b < gridDim.x) {
                T rec[8];
                ar_load_record(part + (size_t)b * kArMax, rec);
#pragma unroll
                for (int k = 0; k < NV; ++k) acc[k] += rec[k];
            }
        }
        const T tot = warp_sum8(acc, lane);
        if ((lane & 3) == 0 && idx < NV) tot_w[idx][w] = tot;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        const int nused = nchunks < nread ? nchunks : nread;
        T x = tot_w[threadIdx.x][0];
        for (int ww = 1; ww < nused; ++ww) x += tot_w[threadIdx.x][ww];
        res[threadIdx.x] = x;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = res[k];
    return true;
}

// plain barrier on the same counter
__device__ __forceinline__ bool grid_sync_ar(const GridAR& g, unsigned long long& epoch) {
    __shared__ int st;
    if (!ar_arrive_wait(g, epoch, &st)) return false;
    ++epoch;
    return true;
}

// Shared-memory copy of a contiguous run of SELL slots: slots [base, base +
// cap) of the column and value arrays, laid out as in global memory.  A slice
// whose slots all lie in the run is read from shared memory.
template <class T>
struct SellCache {
    const int32_t* col = nullptr;  // shared memory
    const T* val = nullptr;
    int32_t base = 0, cap = 0;
};

// n columns of a slot row from cp / vp (already at slot lane of the first
// column, 32 slots per column): in blocks of eight, the loads of the next
// block issued while the gathers of the current block are in flight, so a
// lane keeps up to 16 independent loads outstanding and n columns cost
// ceil(n/8) gather latencies.  SH: cp / vp point to shared memory.  Loads past
// n are masked and the multiply-adds past n are skipped (n is warp-uniform,
// so no FP64 pipe time goes to padding).  Terms are summed in CSR order.
template <bool SH, class T, class XL>
__device__ __forceinline__ T sell_row_walk(const int32_t* __restrict__ cp, const T* __restrict__ vp, int32_t n,
                                           XL xload) {
    constexpr int U = 8;
    auto ldc = [](const int32_t* p) { return SH ? *p : __ldg(p); };
    auto ldv = [](const T* p) { return SH ? *p : __ldg(p); };
    T acc = T(0);
    int32_t cn[U];
    T vn[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const bool in = u < n;
        cn[u] = in ? ldc(cp + 32 * u) : -1;
        vn[u] = in ? ldv(vp + 32 * u) : T(0);
    }
    for (int32_t k = 0; k < n; k += U) {
        T xv[U], vv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            xv[u] = cn[u] >= 0 ? xload(cn[u]) : T(0);
            vv[u] = vn[u];
        }
        const int32_t kn = k + U;
        if (kn < n) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const bool in = kn + u < n;
                cn[u] = in ? ldc(cp + 32 * (kn + u)) : -1;
                vn[u] = in ? ldv(vp + 32 * (kn + u)) : T(0);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (k + u < n) acc += vv[u] * xv[u];
    }
    return acc;
}

// Slot row of a SELL matrix times the vector given by xload(col), over the
// slice columns [c0, c0 + n), accumulated in T; from the shared-memory copy
// when the cache holds the whole slice.
template <class T, class XL>
__device__ __forceinline__ T sell_row_range(const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                                            const T* __restrict__ val, int64_t s, int lane, int32_t c0, int32_t n,
                                            XL xload, const SellCache<T>& cache = SellCache<T>()) {
    const int32_t ps = __ldg(ptr + s), p0 = ps + 32 * c0;
    if (cache.cap > 0 && ps >= cache.base && __ldg(ptr + s + 1) - cache.base <= cache.cap)
        return sell_row_walk<true, T>(cache.col + (p0 - cache.base) + lane, cache.val + (p0 - cache.base) + lane, n,
                                      xload);
    return sell_row_walk<false, T>(col + p0 + lane, val + p0 + lane, n, xload);
}

// the whole slot row (all columns of slice s)
template <class T, class XL>
__device__ __forceinline__ T sell_row(const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                                      const T* __restrict__ val, int64_t s, int lane, XL xload) {
    const int32_t w = (__ldg(ptr + s + 1) - __ldg(ptr + s)) >> 5;
    return sell_row_range<T>(ptr, col, val, s, lane, 0, w, xload);
}

// ---------------------------------------------------------------------------
// Balanced SELL product of one block.  The block takes the slices [s0, s1)
// (at most kBalMaxSlices) and splits their total column count T evenly over
// its NW warps: warp j walks the column positions [jT/NW, (j+1)T/NW) of the
// concatenated slices, so a wide slice is shared by several warps and every
// warp walks about T/NW columns (the gather chain of the slowest warp no
// longer follows the widest slice).  A slice that lies wholly inside one warp's
// range is emitted by that warp; a split slice's partial sums go to shared
// memory and the warp holding its last column adds them in column order
// (deterministic).  emit(slice, value) is called by all 32 lanes of a warp;
// zero-width slices (empty rows) are emitted too.  All threads of the block
// must call this, in uniform control flow; it ends with a block barrier, so
// what emit wrote to shared memory can be read right after.
// ---------------------------------------------------------------------------
constexpr int kBalMaxSlices = 64;

// First slice of part b of nparts when the slices [0, nslices) are split at
// equal work, work(s) = columns(s) + kBalRowCost per slice (the per-row
// updates that follow the product), using the SELL offsets ptr (32 x columns,
// a prefix sum): the largest s with work before s <= b W / nparts.
constexpr int kBalRowCost = 4;
__device__ __forceinline__ int64_t balanced_part_start(const int32_t* __restrict__ ptr, int64_t nslices, int64_t b,
                                                       int64_t nparts) {
    if (b <= 0) return 0;
    if (b >= nparts) return nslices;
    const int64_t total = (int64_t)(__ldg(ptr + nslices) >> 5) + kBalRowCost * nslices;
    const int64_t target = total * b / nparts;
    int64_t lo = 0, hi = nslices;  // work(lo) <= target < work(hi + 1)
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if ((int64_t)(__ldg(ptr + mid) >> 5) + kBalRowCost * mid <= target) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int NW, class T>
struct BalShared {
    int32_t P[kBalMaxSlices + 1];
    T tail[NW][32];
};

// The column prefix of the slices [s0, s0 + S) into sh.P (one block
// barrier); a block that walks the same slices repeatedly plans once.
template <int NW, class T>
__device__ __forceinline__ void sell_block_plan(BalShared<NW, T>& sh, const int32_t* __restrict__ ptr, int64_t s0,
                                                int S) {
    const int lane = threadIdx.x & 31, j = threadIdx.x >> 5;
    if (j == 0) {
        int carry = 0;
        for (int b = 0; b < S; b += 32) {
            const int i = b + lane;
            int w = i < S ? (__ldg(ptr + s0 + i + 1) - __ldg(ptr + s0 + i)) >> 5 : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += t;
            }
            if (i < S) sh.P[i + 1] = carry + w;
            carry += __shfl_sync(0xffffffffu, w, 31);
        }
        if (lane == 0) sh.P[0] = 0;
    }
    __syncthreads();
}

// The product over planned slices (sh.P holds the prefix of [s0, s0 + S)):
// row(slice, c0, n) returns one lane's partial sum over the slice columns
// [c0, c0 + n); T needs T(0) and +.
template <int NW, class T, class ROW, class EMIT>
__device__ __forceinline__ void sell_block_walk_fn(BalShared<NW, T>& sh, int64_t s0, int S, ROW row, EMIT emit) {
    const int lane = threadIdx.x & 31, j = threadIdx.x >> 5;
    const int32_t Tot = sh.P[S];
    const int32_t g0 = (int32_t)((int64_t)j * Tot / NW), g1 = (int32_t)((int64_t)(j + 1) * Tot / NW);
    // first slice that overlaps [g0, ..) or starts at g0 (zero width included)
    int lo = 0, hi = S;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (sh.P[mid + 1] > g0 || sh.P[mid] >= g0) hi = mid;
        else lo = mid + 1;
    }
    T head = T(0);
    int hslice = -1;
    for (int i = lo; i < S; ++i) {
        const int32_t pa = sh.P[i], pb = sh.P[i + 1];
        if (!(pa < g1 || (j == NW - 1 && pa == Tot))) break;
        const int32_t c0 = g0 > pa ? g0 - pa : 0;
        const int32_t c1 = (g1 < pb ? g1 : pb) - pa;
        const T acc = row(s0 + i, c0, c1 > c0 ? c1 - c0 : 0);
        const bool starts = pa >= g0, ends = pb <= g1;
        if (starts && ends) {
            emit(s0 + i, acc);
        } else if (ends) {
            head = acc;
            hslice = i;
        } else {
            sh.tail[j][lane] = acc;
        }
    }
    __syncthreads();
    if (hslice >= 0) {
        // warps from the one holding the slice's first column up to this one
        const int32_t pa = sh.P[hslice];
        int ja = j - 1;
        while (ja > 0 && (int32_t)((int64_t)ja * Tot / NW) > pa) --ja;
        T sum = T(0);
        for (int jj = ja; jj < j; ++jj) {
            const int32_t a0 = (int32_t)((int64_t)jj * Tot / NW), a1 = (int32_t)((int64_t)(jj + 1) * Tot / NW);
            if (a1 > a0) sum = sum + sh.tail[jj][lane];
        }
        emit(s0 + hslice, sum + head);
    }
    __syncthreads();  // emits visible to the block; sh.tail free for the next call
}

template <int NW, class T, class XL, class EMIT>
__device__ __forceinline__ void sell_block_walk(BalShared<NW, T>& sh, const int32_t* __restrict__ ptr,
                                                const int32_t* __restrict__ col, const T* __restrict__ val,
                                                int64_t s0, int S, XL xload, EMIT emit,
                                                const SellCache<T>& cache = SellCache<T>()) {
    const int lane = threadIdx.x & 31;
    sell_block_walk_fn<NW, T>(
        sh, s0, S,
        [&](int64_t s, int32_t c0, int32_t n) { return sell_row_range<T>(ptr, col, val, s, lane, c0, n, xload, cache); },
        emit);
}

template <int NW, class T, class XL, class EMIT>
__device__ __forceinline__ void sell_block_balanced(BalShared<NW, T>& sh, const int32_t* __restrict__ ptr,
                                                    const int32_t* __restrict__ col, const T* __restrict__ val,
                                                    int64_t s0, int S, XL xload, EMIT emit,
                                                    const SellCache<T>& cache = SellCache<T>()) {
    sell_block_plan<NW, T>(sh, ptr, s0, S);
    sell_block_walk<NW, T>(sh, ptr, col, val, s0, S, xload, emit, cache);
}

#define TF_SLICE_LOOP(nslices, s)                                                    \
    const int64_t warp__ = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;   \
    const int64_t nwarp__ = ((int64_t)gridDim.x * blockDim.x) >> 5;                  \
    for (int64_t s = warp__; s < (nslices); s += nwarp__)

// Slice order of the persistent kernels, where every warp walks several
// slices between two grid barriers and the barrier waits for the slowest
// warp.  The SELL rows are sorted by length inside windows of
// kSellWinSlices slices (512 rows), so slice rank k of every window has about
// the same width and rank 0 is the widest: taking slices in storage order
// hands the widest slice of every window to the same warp index.  Here
// position p runs rank-major (p = k * nwin + win, slice win * 16 + k: widest
// ranks first), and warp w of n takes positions w, 2n-1-w, 2n+w, ...: the
// passes alternate direction, so each warp pairs wide slices with narrow ones.
// A bijection on [0, nslices) for nslices a multiple of kSellWinSlices;
// warp-uniform control flow.
constexpr int kSellWinSlices = 16;
__device__ __forceinline__ int64_t slice_at_rank(int64_t pos, int64_t nwin) {
    return (pos % nwin) * kSellWinSlices + pos / nwin;
}
#define TF_SLICE_LOOP_BAL(nslices, s)                                                                     \
    const int64_t bw__ = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;                          \
    const int64_t bn__ = ((int64_t)gridDim.x * blockDim.x) >> 5;                                          \
    const int64_t bwin__ = (nslices) / kSellWinSlices;                                                    \
    for (int64_t bi__ = 0; bi__ * bn__ < (nslices); ++bi__)                                               \
        for (int64_t bp__ = bi__ * bn__ + ((bi__ & 1) ? bn__ - 1 - bw__ : bw__),                          \
                     s = bp__ < (nslices) ? slice_at_rank(bp__, bwin__) : -1;                             \
             s >= 0; s = -1)

}  // namespace tf
