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

// Slot row of a SELL matrix times the vector given by xload(col), accumulated
// in T.  The row is walked in blocks of eight, the last block masked (the
// slice width is the same for all 32 lanes, so the mask is warp-uniform): the
// column indices and values of the next block are loaded while the gathers of
// the current block are in flight, so a lane keeps up to 16 independent loads
// outstanding and a row of w entries costs ceil(w/8) gather latencies.  Terms
// are summed in CSR order; masked terms add +0.
template <class T, class XL>
__device__ __forceinline__ T sell_row(const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                                      const T* __restrict__ val, int64_t s, int lane, XL xload) {
    constexpr int U = 8;
    const int32_t p0 = __ldg(ptr + s);
    const int32_t w = (__ldg(ptr + s + 1) - p0) >> 5;
    const int32_t* cp = col + p0 + lane;
    const T* vp = val + p0 + lane;
    T acc = T(0);
    int32_t cn[U];
    T vn[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const bool in = u < w;
        cn[u] = in ? __ldg(cp + 32 * u) : -1;
        vn[u] = in ? __ldg(vp + 32 * u) : T(0);
    }
    for (int32_t k = 0; k < w; k += U) {
        T xv[U], vv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            xv[u] = cn[u] >= 0 ? xload(cn[u]) : T(0);
            vv[u] = vn[u];
        }
        const int32_t kn = k + U;
        if (kn < w) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const bool in = kn + u < w;
                cn[u] = in ? __ldg(cp + 32 * (kn + u)) : -1;
                vn[u] = in ? __ldg(vp + 32 * (kn + u)) : T(0);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) acc += vv[u] * xv[u];
    }
    return acc;
}

#define TF_SLICE_LOOP(nslices, s)                                                    \
    const int64_t warp__ = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;   \
    const int64_t nwarp__ = ((int64_t)gridDim.x * blockDim.x) >> 5;                  \
    for (int64_t s = warp__; s < (nslices); s += nwarp__)

}  // namespace tf
