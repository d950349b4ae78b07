// Jacobi-PCG for callers that cannot allocate device memory.
//
// tf_pcg_jacobi (krylov.cu) keeps its work vectors in memory owned by a
// tf_context, which allocates with cudaMalloc.  Some callers cannot allow
// that: applications that own all device memory through their own pool and
// forbid third-party allocations, and code that must not trigger the
// implicit device synchronisation of cudaMalloc/cudaFree inside a real-time
// loop.
// tf_pcg_jacobi_noalloc serves them: the caller passes the CSR matrix, the
// right-hand side and the solution in device memory; every other buffer the
// solve needs lives in one file-scope device array of fixed size
// (g_noalloc_scratch), which every GPU that loads the library holds until the
// process exits.  The call allocates nothing.
//
// The array is shared by all calls: calls that overlap on the GPU (two
// streams, two host threads) race on it and must be serialised by the caller.
// Each call clears the words that must start at zero (barrier counters, status)
// and writes every work vector before reading it.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/tracefem.h"

namespace {

// work vectors r, z, p0, p1, q, diag (6 per row), per-block partials, control words
constexpr int kThreads = 256;
constexpr int kMaxBlocksPerSm = 8;
constexpr int kMaxSms = 256;
constexpr int64_t kCtrlDoubles = 64;
constexpr int64_t kPartDoubles = (int64_t)kMaxSms * kMaxBlocksPerSm * 3 * 2;
constexpr int64_t kScratchDoubles = kCtrlDoubles + kPartDoubles + 6 * (int64_t)TF_NOALLOC_MAX_ROWS;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

// per-device address of g_noalloc_scratch (host code may not name the array
// itself: its host-side name is only a stand-in for the symbol)
double* g_scratch_ptr[64] = {};
std::mutex g_setup_mutex;

int scratch_for_current_device(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return TF_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return TF_ERR_CUDA;
        g_scratch_ptr[dev] = (double*)p;
    }
    *out = g_scratch_ptr[dev];
    return TF_OK;
}

// ---- warp sums and a bounded grid barrier -----------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct Ctrl {
    unsigned count, gen;
    int status, iters;
    double resid;
    int converged;
};

// block 0 publishes the outcome of the solve (every exit path calls this)
__device__ void finish(Ctrl* ctl, int iters, double resid, bool converged) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->iters = iters;
        ctl->resid = resid;
        ctl->converged = converged ? 1 : 0;
    }
}

__device__ bool barrier(Ctrl* ctl) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = &ctl->gen;
        const unsigned my = *vgen;
        __threadfence();
        if (atomicAdd(&ctl->count, 1u) == gridDim.x - 1) {
            ctl->count = 0;
            __threadfence();
            atomicAdd(&ctl->gen, 1u);
        } else {
            long long spins = 0;
            while (*vgen == my) {
                if (++spins > 20000000LL) {
                    atomicCAS(&ctl->status, 0, TF_ERR_WATCHDOG);
                    break;
                }
                if (spins > 64) __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *((volatile int*)&ctl->status) == 0;
}

template <int NV>
__device__ void partials(double (&v)[NV], double* part) {
    __shared__ double red[NV][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < NV; ++k) {
        const double x = warp_sum(v[k]);
        if (lane == 0) red[k][w] = x;
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

// every block sums all partials in the same fixed order
template <int NV>
__device__ void reduce_all(const double* part, double (&out)[NV]) {
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

// ---- persistent PCG on CSR, G lanes per row ---------------------------------------
struct Args {
    int64_t m;
    const int32_t* rowptr;
    const int32_t* colind;
    const double* vals;
    const double* b;
    double* x;
    double* scratch;
    int max_iter;
    double tol;
    int rel;
};

template <int G>
__global__ void __launch_bounds__(kThreads) k_pcg_noalloc(Args a) {
    const int64_t m = a.m;
    Ctrl* ctl = reinterpret_cast<Ctrl*>(a.scratch);
    // Partials alternate between two buffers, one per reduction in turn (set-up: B;
    // each iteration: A then B).  A block may only rewrite a buffer after every
    // block has passed the barrier that follows its last read of that buffer.
    double* partA = a.scratch + kCtrlDoubles;
    double* partB = partA + (size_t)gridDim.x * 3;
    double* r = a.scratch + kCtrlDoubles + kPartDoubles;
    double* z = r + m;
    double* p0 = z + m;
    double* p1 = p0 + m;
    double* q = p1 + m;
    double* d = q + m;
    const int lane = threadIdx.x & 31, sub = lane & (G - 1);
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;

    // diagonal (row scan, SolveGSstep<PB_JAC0>), r = b - A x, z = r/d, p0 = z
    {
        double v[3] = {0., 0., 0.};
        for (int64_t base = warp * (32 / G); base < m; base += nwarp * (32 / G)) {
            const int64_t row = base + lane / G;
            int32_t s = 0, e = 0;
            if (row < m) {
                s = a.rowptr[row];
                e = a.rowptr[row + 1];
            }
            double acc = 0., dg = 0.;
            for (int32_t k = s + sub; k < e; k += G) {
                const int32_t c = a.colind[k];
                acc += a.vals[k] * __ldcg(a.x + c);
                if (c == row) dg = a.vals[k];
            }
            for (int o = G / 2; o > 0; o >>= 1) {
                acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
                dg += __shfl_xor_sync(0xffffffffu, dg, o, G);
            }
            if (sub == 0 && row < m) {
                const double ri = a.b[row] - acc, zi = ri / dg;
                d[row] = dg;
                r[row] = ri;
                z[row] = zi;
                p0[row] = zi;
                v[0] += ri * ri;
                v[1] += a.b[row] * a.b[row];
                v[2] += zi * ri;
            }
        }
        partials<3>(v, partB);
    }
    if (!barrier(ctl)) return;
    double s0[3];
    reduce_all<3>(partB, s0);
    double normb = sqrt(s0[1]);
    if (normb == 0.0 || !a.rel) normb = 1.0;
    double resid = sqrt(s0[0]) / normb, rho = s0[2], beta = 0.;
    if (resid <= a.tol || a.max_iter == 0) {
        finish(ctl, 0, resid, resid <= a.tol);
        return;
    }
    double* pc = p0;
    double* pn = p1;
    for (int it = 1; it <= a.max_iter; ++it) {
        {
            double v[1] = {0.};
            for (int64_t base = warp * (32 / G); base < m; base += nwarp * (32 / G)) {
                const int64_t row = base + lane / G;
                int32_t s = 0, e = 0;
                if (row < m) {
                    s = a.rowptr[row];
                    e = a.rowptr[row + 1];
                }
                double acc = 0.;
                for (int32_t k = s + sub; k < e; k += G) {
                    const int32_t c = a.colind[k];
                    acc += a.vals[k] * (__ldcg(z + c) + beta * __ldcg(pc + c));
                }
                for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
                if (sub == 0 && row < m) {
                    const double pi = __ldcg(z + row) + beta * __ldcg(pc + row);
                    pn[row] = pi;
                    q[row] = acc;
                    v[0] += acc * pi;
                }
            }
            partials<1>(v, partA);
        }
        if (!barrier(ctl)) return;
        double lam[1];
        reduce_all<1>(partA, lam);
        const double alpha = rho / lam[0];
        {
            double v[2] = {0., 0.};
            for (int64_t i = tid; i < m; i += nth) {
                a.x[i] += alpha * __ldcg(pn + i);
                const double ri = r[i] + (-alpha) * __ldcg(q + i);
                const double zi = ri / __ldcg(d + i);
                r[i] = ri;
                z[i] = zi;
                v[0] += ri * ri;
                v[1] += zi * ri;
            }
            partials<2>(v, partB);
        }
        if (!barrier(ctl)) return;
        double s2[2];
        reduce_all<2>(partB, s2);
        resid = sqrt(s2[0]) / normb;
        if (resid <= a.tol || it == a.max_iter) {
            finish(ctl, it, resid, resid <= a.tol);
            return;
        }
        const double rho1 = rho;
        rho = s2[1];
        beta = rho / rho1;
        double* t = pc;
        pc = pn;
        pn = t;
    }
}

}  // namespace

extern "C" int tf_pcg_jacobi_noalloc(int64_t m, const int32_t* rowptr, const int32_t* colind, const double* vals,
                                     const double* b, double* x, int* max_iter, double* tol, int rel, void* stream) {
    if (m <= 0 || !rowptr || !colind || !vals || !b || !x || !max_iter || !tol || *max_iter < 0) return TF_ERR_BAD_INPUT;
    if (m > TF_NOALLOC_MAX_ROWS) return TF_ERR_CAPACITY;
    double* scratch = nullptr;
    int st = scratch_for_current_device(&scratch);
    if (st != TF_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return TF_ERR_CUDA;
    // average row length picks the lanes per row; the matrix's row pointers are on the device
    int32_t nnz = 0;
    if (cudaMemcpyAsync(&nnz, rowptr + m, sizeof(int32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return TF_ERR_CUDA;
    const double avg = (double)nnz / (double)m;
    const int G = avg <= 6 ? 4 : avg <= 12 ? 8 : avg <= 24 ? 16 : 32;
    const void* fn = G == 4 ? (const void*)k_pcg_noalloc<4> : G == 8 ? (const void*)k_pcg_noalloc<8>
                   : G == 16 ? (const void*)k_pcg_noalloc<16> : (const void*)k_pcg_noalloc<32>;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, 0) != cudaSuccess || per_sm < 1)
        return TF_ERR_CUDA;
    if (per_sm > kMaxBlocksPerSm) per_sm = kMaxBlocksPerSm;
    if (sms > kMaxSms) sms = kMaxSms;
    int64_t want = (m * G + kThreads - 1) / kThreads;
    int blocks = (int)(want < (int64_t)per_sm * sms ? want : (int64_t)per_sm * sms);
    if (blocks < 1) blocks = 1;
    // the control words must start at zero; everything else is written before it is read
    if (cudaMemsetAsync(scratch, 0, sizeof(double) * kCtrlDoubles, s) != cudaSuccess) return TF_ERR_CUDA;
    Args a{m, rowptr, colind, vals, b, x, scratch, *max_iter, *tol, rel};
    void* args[] = {&a};
    if (cudaLaunchCooperativeKernel(fn, blocks, kThreads, args, 0, s) != cudaSuccess) return TF_ERR_CUDA;
    Ctrl ctl;
    if (cudaMemcpyAsync(&ctl, scratch, sizeof(Ctrl), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return TF_ERR_CUDA;
    if (ctl.status != 0) return ctl.status;
    *max_iter = ctl.iters;
    *tol = ctl.resid;
    return ctl.converged ? TF_OK : TF_ERR_NOT_CONVERGED;
}
