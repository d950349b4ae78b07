// Sparse linear algebra and Krylov solvers: SpMV, linear combinations, the
// Cahn-Hilliard block matrix, persistent Jacobi-PCG (FP64 and FP32), mixed-
// precision iterative refinement and restarted GMRES.
//
// The PCG of num/krylovsolver.h:107-189 runs as ONE cooperative kernel: every
// block owns a slice of rows, a grid barrier separates the two phases of an
// iteration (q = A p with <q,p>;  x,r,z updates with <r,r>,<z,r>), and the
// search-direction update p = z + beta p is fused into the next SpMV (double
// buffered).  Dot products are compensated (TwoSum) and reduced over blocks in
// a fixed order, so every block computes bit-identical scalars and all blocks
// take the same convergence decision.  Every barrier wait is bounded: a block
// that waits too long raises TF_ERR_WATCHDOG and the kernel returns.
#include <cooperative_groups.h>

#include <cmath>

#include "tf_internal.cuh"

namespace tf {

// ---------------------------------------------------------------------------
// compensated summation
// ---------------------------------------------------------------------------
struct DD {
    double s, c;
};
__device__ __forceinline__ void two_sum_add(DD& a, double b) {
    const double s = a.s + b;
    const double bp = s - a.s;
    const double err = (a.s - (s - bp)) + (b - bp);
    a.s = s;
    a.c += err;
}
__device__ __forceinline__ DD dd_add(DD a, DD b) {
    DD r = a;
    two_sum_add(r, b.s);
    r.c += b.c;
    return r;
}
__device__ __forceinline__ DD warp_dd_sum(DD v) {
    for (int o = 16; o > 0; o >>= 1) {
        DD w;
        w.s = __shfl_xor_sync(0xffffffffu, v.s, o);
        w.c = __shfl_xor_sync(0xffffffffu, v.c, o);
        // order-independent pairing: combine the lower lane's value first
        const int lane = threadIdx.x & 31;
        v = (lane & o) ? dd_add(w, v) : dd_add(v, w);
    }
    return v;
}

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
    __threadfence();
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
                if (spins > 64) __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *((volatile int*)g.status) == 0;
}

// ---------------------------------------------------------------------------
// block-level reductions into per-block partials, and their global reduction
// ---------------------------------------------------------------------------
template <int NV>
__device__ void block_partials(DD (&v)[NV], double* part /* [nblocks][NV][2] */) {
    __shared__ DD red[NV][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < NV; ++k) {
        DD x = warp_dd_sum(v[k]);
        if (lane == 0) red[k][w] = x;
    }
    __syncthreads();
    if (w == 0) {
        for (int k = 0; k < NV; ++k) {
            DD x = lane < nw ? red[k][lane] : DD{0., 0.};
            x = warp_dd_sum(x);
            if (lane == 0) {
                part[((size_t)blockIdx.x * NV + k) * 2] = x.s;
                part[((size_t)blockIdx.x * NV + k) * 2 + 1] = x.c;
            }
        }
    }
    __syncthreads();
}

// every block reduces all partials in the same fixed order
template <int NV>
__device__ void grid_reduce(const double* part, double (&out)[NV]) {
    __shared__ DD red[NV][32];
    __shared__ double res[NV];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < NV; ++k) {
        DD x{0., 0.};
        for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
            DD y{__ldcg(part + ((size_t)b * NV + k) * 2), __ldcg(part + ((size_t)b * NV + k) * 2 + 1)};
            x = dd_add(x, y);
        }
        x = warp_dd_sum(x);
        if (lane == 0) red[k][w] = x;
    }
    __syncthreads();
    if (w == 0) {
        for (int k = 0; k < NV; ++k) {
            DD x = lane < nw ? red[k][lane] : DD{0., 0.};
            x = warp_dd_sum(x);
            if (lane == 0) res[k] = x.s + x.c;
        }
    }
    __syncthreads();
    for (int k = 0; k < NV; ++k) out[k] = res[k];
    __syncthreads();
}

// ---------------------------------------------------------------------------
// SpMV (y_Ax, num/spmat.h:1684-1709): G lanes per row
// ---------------------------------------------------------------------------
// Rows are handed out per warp (32/G rows at a time) so that every lane of a
// warp runs the same number of iterations and reaches every shuffle.
template <class T, int G>
__device__ __forceinline__ double row_dot(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                                          const T* __restrict__ vals, const T* x, int64_t row, int64_t m, int sub) {
    int32_t s = 0, e = 0;
    if (row < m) {
        s = __ldg(rowptr + row);
        e = __ldg(rowptr + row + 1);
    }
    double acc = 0.;
    for (int32_t k = s + sub; k < e; k += G) acc += (double)__ldg(vals + k) * (double)__ldcg(x + __ldg(colind + k));
    for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
    return acc;
}

#define TF_ROW_LOOP(G, m, row, sub)                                                         \
    const int sub = threadIdx.x & ((G)-1);                                                  \
    const int64_t warp__ = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;          \
    const int64_t nwarp__ = ((int64_t)gridDim.x * blockDim.x) >> 5;                         \
    for (int64_t base__ = warp__ * (32 / (G)); base__ < (m); base__ += nwarp__ * (32 / (G))) \
        for (int64_t row = base__ + (threadIdx.x & 31) / (G), once__ = 0; once__ < 1; ++once__)

template <class T, int G>
__global__ void k_spmv(int64_t m, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                       const T* __restrict__ vals, const T* __restrict__ x, T* __restrict__ y) {
    TF_ROW_LOOP(G, m, row, sub) {
        const double a = row_dot<T, G>(rowptr, colind, vals, x, row, m, sub);
        if (sub == 0 && row < m) y[row] = (T)a;
    }
}

static int pick_group(int64_t m, int64_t nnz) {
    const double avg = m > 0 ? (double)nnz / (double)m : 1.0;
    return avg <= 6 ? 4 : avg <= 12 ? 8 : avg <= 24 ? 16 : 32;
}

template <class T>
static void launch_spmv(Context* c, const CSR& A, const T* vals, const T* x, T* y) {
    const int G = pick_group(A.m, A.nnz);
    const int blocks = grid_for(c, (A.m * G + kBlock - 1) / kBlock * kBlock, kBlock, 8);
    switch (G) {
        case 4: k_spmv<T, 4><<<blocks, kBlock, 0, c->stream>>>(A.m, A.rowptr, A.colind, vals, x, y); break;
        case 8: k_spmv<T, 8><<<blocks, kBlock, 0, c->stream>>>(A.m, A.rowptr, A.colind, vals, x, y); break;
        case 16: k_spmv<T, 16><<<blocks, kBlock, 0, c->stream>>>(A.m, A.rowptr, A.colind, vals, x, y); break;
        default: k_spmv<T, 32><<<blocks, kBlock, 0, c->stream>>>(A.m, A.rowptr, A.colind, vals, x, y); break;
    }
    ++c->launches;
}

int spmv(Context* c, const CSR& A, const double* x, double* y) {
    TimedLaunch tl(c, TF_K_SPMV);
    launch_spmv<double>(c, A, A.vals, x, y);
    TF_CUDA(c, cudaGetLastError());
    return TF_OK;
}

// ---------------------------------------------------------------------------
// diagonal (found by a row scan as in SolveGSstep<PB_JAC0>) and FP32 copies
// ---------------------------------------------------------------------------
__global__ void k_diag(int64_t m, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                       const double* __restrict__ vals, double* __restrict__ d) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
        int32_t k = rowptr[r];
        const int32_t e = rowptr[r + 1];
        while (k < e && colind[k] != r) ++k;
        d[r] = k < e ? vals[k] : 0.;
    }
}
__global__ void k_to_f32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

static int mat_index(Context* c, const CSR& A) {
    for (int i = 0; i < TF_NUM_MATS; ++i)
        if (&c->mats[i] == &A) return i;
    return 0;
}

int ensure_diag(Context* c, CSR& A) {
    if (A.diag_version == A.version && A.diag) return TF_OK;
    const int id = mat_index(c, A);
    TF_TRY(ensure(c, c->mat_diag[id], (size_t)(A.m > 0 ? A.m : 1)));
    A.diag = c->mat_diag[id].p;
    k_diag<<<grid_for(c, A.m), kBlock, 0, c->stream>>>(A.m, A.rowptr, A.colind, A.vals, A.diag);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    A.diag_version = A.version;
    return TF_OK;
}

int ensure_vals32(Context* c, CSR& A) {
    if (A.vals32_version == A.version && A.vals32) return TF_OK;
    const int id = mat_index(c, A);
    TF_TRY(ensure(c, c->mat_vals32[id], (size_t)(A.nnz > 0 ? A.nnz : 1)));
    A.vals32 = c->mat_vals32[id].p;
    k_to_f32<<<grid_for(c, A.nnz), kBlock, 0, c->stream>>>(A.nnz, A.vals, A.vals32);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    A.vals32_version = A.version;
    return TF_OK;
}

// ---------------------------------------------------------------------------
// linear combination on the shared pattern, CH block matrix
// ---------------------------------------------------------------------------
__global__ void k_lincomb(int64_t nnz, int nterms, const double* const* __restrict__ src, const double* __restrict__ co,
                          double* __restrict__ dst) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
        double a = co[0] * src[0][k];
        for (int t = 1; t < nterms; ++t) a += co[t] * src[t][k];
        dst[k] = a;
    }
}

struct LincombArgs {
    const double* src[8];
    double co[8];
};
__global__ void k_lincomb2(int64_t nnz, int nterms, LincombArgs a, double* __restrict__ dst) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
        double s = a.co[0] * a.src[0][k];
        for (int t = 1; t < nterms; ++t) s += a.co[t] * a.src[t][k];
        dst[k] = s;
    }
}

int lincomb(Context* c, int nterms, const int* forms, const double* coeffs) {
    if (nterms < 1 || nterms > 8 || !forms || !coeffs) return set_err(c, TF_ERR_BAD_INPUT, "lincomb: 1..8 terms");
    LincombArgs a{};
    for (int t = 0; t < nterms; ++t) {
        if (forms[t] < 0 || forms[t] >= TF_NUM_FORMS || !c->mats[forms[t]].vals)
            return set_err(c, TF_ERR_BAD_INPUT, "lincomb: form not assembled");
        a.src[t] = c->mats[forms[t]].vals;
        a.co[t] = coeffs[t];
    }
    CSR& S = c->mats[TF_MAT_SYS];
    const CSR& F = c->mats[forms[0]];
    TF_TRY(ensure(c, c->mat_vals[TF_MAT_SYS], (size_t)(F.nnz > 0 ? F.nnz : 1)));
    S.m = F.m;
    S.nnz = F.nnz;
    S.rowptr = F.rowptr;
    S.colind = F.colind;
    S.vals = c->mat_vals[TF_MAT_SYS].p;
    k_lincomb2<<<grid_for(c, S.nnz), kBlock, 0, c->stream>>>(S.nnz, nterms, a, S.vals);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    ++S.version;
    return TF_OK;
}

__global__ void k_block_rowptr(int64_t m, const int32_t* __restrict__ rp, int32_t* __restrict__ brp) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r <= 2 * m; r += (int64_t)gridDim.x * blockDim.x) {
        if (r <= m) brp[r] = 2 * rp[r];
        else brp[r] = 2 * rp[m] + 2 * rp[r - m];
    }
}
__global__ void k_block_fill(int64_t m, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                             const double* __restrict__ M, const double* __restrict__ A, const double* __restrict__ C,
                             double alpha, double mob, double rho, double eps2, double beta,
                             const int32_t* __restrict__ brp, int32_t* __restrict__ bci, double* __restrict__ bv) {
    for (int64_t R = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; R < 2 * m; R += (int64_t)gridDim.x * blockDim.x) {
        const int half = R >= m;
        const int64_t r = half ? R - m : R;
        int32_t w = brp[R];
        for (int blk = 0; blk < 2; ++blk)
            for (int32_t k = rp[r]; k < rp[r + 1]; ++k) {
                double v;
                if (!half) v = blk == 0 ? alpha * M[k] : mob * A[k] + rho * C[k];
                else v = blk == 0 ? (eps2 * A[k] + beta * M[k]) + (eps2 * rho) * C[k] : -1. * M[k];
                bci[w] = ci[k] + (int32_t)(blk * m);
                bv[w] = v;
                ++w;
            }
    }
}

int ch_block(Context* c, double alpha, double mob, double rho, double eps2, double beta, int use_lapm) {
    const CSR& M = c->mats[TF_FORM_M];
    const CSR& A = c->mats[use_lapm ? TF_FORM_LAPM : TF_FORM_A];
    const CSR& C = c->mats[TF_FORM_CN];
    if (!M.vals || !A.vals || !C.vals) return set_err(c, TF_ERR_BAD_INPUT, "ch_block: assemble M, A (or LaplaceM) and C_n first");
    const int64_t m = M.m, nnz = M.nnz;
    if (4 * nnz >= INT32_MAX) return set_err(c, TF_ERR_CAPACITY, "ch_block: too many non-zeros");
    CSR& B = c->mats[TF_MAT_BLOCK];
    TF_TRY(ensure(c, c->block_rowptr, (size_t)(2 * m + 1)));
    TF_TRY(ensure(c, c->block_colind, (size_t)(4 * nnz > 0 ? 4 * nnz : 1)));
    TF_TRY(ensure(c, c->mat_vals[TF_MAT_BLOCK], (size_t)(4 * nnz > 0 ? 4 * nnz : 1)));
    B.m = 2 * m;
    B.nnz = 4 * nnz;
    B.rowptr = c->block_rowptr.p;
    B.colind = c->block_colind.p;
    B.vals = c->mat_vals[TF_MAT_BLOCK].p;
    k_block_rowptr<<<grid_for(c, 2 * m + 1), kBlock, 0, c->stream>>>(m, M.rowptr, B.rowptr);
    k_block_fill<<<grid_for(c, 2 * m), kBlock, 0, c->stream>>>(m, M.rowptr, M.colind, M.vals, A.vals, C.vals, alpha, mob,
                                                               rho, eps2, beta, B.rowptr, B.colind, B.vals);
    c->launches += 2;
    TF_CUDA(c, cudaGetLastError());
    ++B.version;
    return TF_OK;
}

// ---------------------------------------------------------------------------
// persistent Jacobi-PCG
// ---------------------------------------------------------------------------
template <class T>
struct PcgArgs {
    int64_t m;
    const int32_t* rowptr;
    const int32_t* colind;
    const T* vals;
    const T* diag;
    const T* b;
    T* x;
    T* r;
    T* z;
    T* p0;
    T* p1;
    T* q;
    double* part;  // [2][nblocks][3][2]
    GridSync gs;
    int max_iter;
    double tol;
    int rel;
    int* out_iter;
    double* out_resid;
};

template <class T, int G>
__global__ void __launch_bounds__(256) k_pcg(PcgArgs<T> a) {
    double* partA = a.part;
    double* partB = a.part + (size_t)gridDim.x * 3 * 2;

    // r = b - A x ; z = r / d ; p0 = z ; partials <r,r>, <b,b>, <z,r>
    {
        DD v[3] = {{0, 0}, {0, 0}, {0, 0}};
        TF_ROW_LOOP(G, a.m, row, sub) {
            const double ax = row_dot<T, G>(a.rowptr, a.colind, a.vals, a.x, row, a.m, sub);
            if (sub == 0 && row < a.m) {
                const double bi = (double)a.b[row];
                const T ri = (T)(bi - ax);
                const T zi = (T)((double)ri / (double)a.diag[row]);
                a.r[row] = ri;
                a.z[row] = zi;
                a.p0[row] = zi;
                two_sum_add(v[0], (double)ri * (double)ri);
                two_sum_add(v[1], bi * bi);
                two_sum_add(v[2], (double)zi * (double)ri);
            }
        }
        block_partials<3>(v, partA);
    }
    if (!grid_barrier(a.gs)) return;
    double s0[3];
    grid_reduce<3>(partA, s0);
    double normb = sqrt(s0[1]);
    if (normb == 0.0 || !a.rel) normb = 1.0;
    double resid = sqrt(s0[0]) / normb;
    double rho = s0[2];
    if (resid <= a.tol) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            *a.out_iter = 0;
            *a.out_resid = resid;
        }
        return;
    }
    double beta = 0.;
    T* pc = a.p0;  // current direction (previous one when beta != 0)
    T* pn = a.p1;
    for (int it = 1; it <= a.max_iter; ++it) {
        // phase A: p_new = z + beta p_cur ; q = A p_new ; <q, p_new>
        {
            DD v[1] = {{0, 0}};
            const T* z = a.z;
            TF_ROW_LOOP(G, a.m, row, sub) {
                int32_t s = 0, e = 0;
                if (row < a.m) {
                    s = __ldg(a.rowptr + row);
                    e = __ldg(a.rowptr + row + 1);
                }
                double acc = 0.;
                for (int32_t k = s + sub; k < e; k += G) {
                    const int32_t j = __ldg(a.colind + k);
                    const double pj = (double)__ldcg(z + j) + beta * (double)__ldcg(pc + j);
                    acc += (double)__ldg(a.vals + k) * (double)(T)pj;
                }
                for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
                if (sub == 0 && row < a.m) {
                    const T pi = (T)((double)__ldcg(z + row) + beta * (double)__ldcg(pc + row));
                    const T qi = (T)acc;
                    pn[row] = pi;
                    a.q[row] = qi;
                    two_sum_add(v[0], (double)qi * (double)pi);
                }
            }
            block_partials<1>(v, partA);
        }
        if (!grid_barrier(a.gs)) return;
        double lam[1];
        grid_reduce<1>(partA, lam);
        const double alpha = rho / lam[0];
        // phase B: x += alpha p ; r -= alpha q ; z = r / d ; <r,r>, <z,r>
        {
            DD v[2] = {{0, 0}, {0, 0}};
            for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.m; i += (int64_t)gridDim.x * blockDim.x) {
                const double pi = (double)__ldcg(pn + i);
                a.x[i] = (T)((double)a.x[i] + alpha * pi);
                const T ri = (T)((double)a.r[i] + (-alpha) * (double)__ldcg(a.q + i));
                const T zi = (T)((double)ri / (double)a.diag[i]);
                a.r[i] = ri;
                a.z[i] = zi;
                two_sum_add(v[0], (double)ri * (double)ri);
                two_sum_add(v[1], (double)zi * (double)ri);
            }
            block_partials<2>(v, partB);
        }
        if (!grid_barrier(a.gs)) return;
        double s2[2];
        grid_reduce<2>(partB, s2);
        resid = sqrt(s2[0]) / normb;
        if (resid <= a.tol || it == a.max_iter) {
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                *a.out_iter = resid <= a.tol ? it : -it;
                *a.out_resid = resid;
            }
            return;
        }
        const double rho1 = rho;
        rho = s2[1];
        beta = rho / rho1;
        T* tmp = pc;
        pc = pn;
        pn = tmp;
    }
}

void release_solver_workspace(Context* c) {
    release(c->kry64);
    release(c->kry32);
    release(c->kry_part);
    release(c->kry_resid);
    release(c->kry_bar);
    release(c->kry_iters);
}

template <class T>
static int run_pcg_kernel(Context* c, const CSR& A, const T* vals, const T* diag, const T* b, T* x, T* work, int max_iter,
                          double tol, int rel, int* iters_out, double* resid_out) {
    const int G = pick_group(A.m, A.nnz);
    int dev_blocks_per_sm = 0;
    cudaError_t e;
    void* fn;
    switch (G) {
        case 4: fn = (void*)k_pcg<T, 4>; break;
        case 8: fn = (void*)k_pcg<T, 8>; break;
        case 16: fn = (void*)k_pcg<T, 16>; break;
        default: fn = (void*)k_pcg<T, 32>; break;
    }
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&dev_blocks_per_sm, fn, 256, 0);
    if (e != cudaSuccess || dev_blocks_per_sm < 1) return set_err(c, TF_ERR_CUDA, "pcg: occupancy query failed");
    int64_t want = (A.m * G + 255) / 256;
    int blocks = (int)std::min<int64_t>(want, (int64_t)dev_blocks_per_sm * c->num_sms);
    if (blocks < 1) blocks = 1;
    TF_TRY(ensure(c, c->kry_part, (size_t)blocks * 3 * 2 * 2));
    TF_TRY(ensure(c, c->kry_bar, 2));
    TF_TRY(ensure(c, c->kry_iters, 1));
    TF_TRY(ensure(c, c->kry_resid, 1));
    TF_CUDA(c, cudaMemsetAsync(c->kry_bar.p, 0, 2 * sizeof(unsigned), c->stream));
    TF_CUDA(c, cudaMemsetAsync(c->status.p, 0, 4 * sizeof(int), c->stream));
    PcgArgs<T> a;
    a.m = A.m;
    a.rowptr = A.rowptr;
    a.colind = A.colind;
    a.vals = vals;
    a.diag = diag;
    a.b = b;
    a.x = x;
    a.r = work;
    a.z = work + A.m;
    a.p0 = work + 2 * A.m;
    a.p1 = work + 3 * A.m;
    a.q = work + 4 * A.m;
    a.part = c->kry_part.p;
    a.gs = GridSync{c->kry_bar.p, c->kry_bar.p + 1, c->status.p};
    a.max_iter = max_iter;
    a.tol = tol;
    a.rel = rel;
    a.out_iter = c->kry_iters.p;
    a.out_resid = c->kry_resid.p;
    void* args[] = {&a};
    TF_CUDA(c, cudaLaunchCooperativeKernel(fn, blocks, 256, args, 0, c->stream));
    ++c->launches;
    int it = 0;
    double res = 0;
    TF_CUDA(c, cudaMemcpyAsync(&it, c->kry_iters.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaMemcpyAsync(&res, c->kry_resid.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    int st = 0;
    TF_TRY(sync_status(c, &st));
    if (st) return set_err(c, st, "pcg: grid barrier watchdog fired");
    *iters_out = it;
    *resid_out = res;
    return TF_OK;
}

// residual r = b - A x (FP64) with <r,r> partials, then norms on the host
__global__ void k_residual(int64_t m, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                           const double* __restrict__ vals, const double* __restrict__ b, const double* __restrict__ x,
                           double* __restrict__ r, double* __restrict__ part) {
    constexpr int G = 8;
    DD v[2] = {{0, 0}, {0, 0}};
    TF_ROW_LOOP(G, m, row, sub) {
        const double ax = row_dot<double, G>(rowptr, colind, vals, x, row, m, sub);
        if (sub == 0 && row < m) {
            const double ri = b[row] - ax;
            r[row] = ri;
            two_sum_add(v[0], ri * ri);
            two_sum_add(v[1], b[row] * b[row]);
        }
    }
    block_partials<2>(v, part);
}
__global__ void k_reduce_partials(int nblocks, const double* __restrict__ part, double* __restrict__ out) {
    // one block; same fixed order as grid_reduce
    __shared__ DD red[2][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < 2; ++k) {
        DD x{0., 0.};
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) x = dd_add(x, DD{part[(b * 2 + k) * 2], part[(b * 2 + k) * 2 + 1]});
        x = warp_dd_sum(x);
        if (lane == 0) red[k][w] = x;
    }
    __syncthreads();
    if (w == 0)
        for (int k = 0; k < 2; ++k) {
            DD x = lane < nw ? red[k][lane] : DD{0., 0.};
            x = warp_dd_sum(x);
            if (lane == 0) out[k] = x.s + x.c;
        }
}
__global__ void k_scale_to_f32(int64_t n, const double* __restrict__ a, double s, float* __restrict__ b, float* __restrict__ x0) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        b[i] = (float)(a[i] * s);
        x0[i] = 0.f;
    }
}
__global__ void k_axpy_f32(int64_t n, double s, const float* __restrict__ d, double* __restrict__ x) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] += s * (double)d[i];
}

int pcg_jacobi(Context* c, CSR& A, const double* b, double* x, int precision, int* max_iter, double* tol, int rel) {
    if (!A.vals || A.m <= 0) return set_err(c, TF_ERR_BAD_INPUT, "pcg: empty matrix");
    TF_TRY(ensure_diag(c, A));
    const int64_t m = A.m;
    TimedLaunch tl(c, TF_K_PCG);
    if (precision == TF_PREC_FP64) {
        TF_TRY(ensure(c, c->kry64, (size_t)(5 * m)));
        int it = 0;
        double res = 0.;
        TF_TRY(run_pcg_kernel<double>(c, A, A.vals, A.diag, b, x, c->kry64.p, *max_iter, *tol, rel, &it, &res));
        const bool ok = it >= 0;
        *max_iter = ok ? it : -it;
        *tol = res;
        return ok ? TF_OK : set_err(c, TF_ERR_NOT_CONVERGED, "pcg: no convergence within max_iter");
    }
    // mixed precision: FP32 PCG sweeps inside FP64 iterative refinement
    TF_TRY(ensure_vals32(c, A));
    TF_TRY(ensure(c, c->kry32, (size_t)(8 * m)));
    TF_TRY(ensure(c, c->kry64, (size_t)(5 * m)));
    float* d32 = c->kry32.p;  // diag, rhs, x, work(5m)
    float* b32 = d32 + m;
    float* x32 = b32 + m;
    float* w32 = x32 + m;
    k_to_f32<<<grid_for(c, m), kBlock, 0, c->stream>>>(m, A.diag, d32);
    ++c->launches;
    double* r64 = c->kry64.p;
    double* part = c->kry64.p + m;  // needs <= 4 m doubles of room
    const int rblocks = (int)std::min<int64_t>((m * 8 + kBlock - 1) / kBlock, (int64_t)c->num_sms * 8);
    if ((int64_t)rblocks * 4 + 2 > 4 * m) return set_err(c, TF_ERR_CAPACITY, "pcg: matrix too small for mixed precision");
    double* sums = part + (size_t)rblocks * 4;
    int total_inner = 0;
    double res = 0.;
    const int max_outer = 60;
    for (int outer = 0; outer <= max_outer; ++outer) {
        k_residual<<<rblocks, kBlock, 0, c->stream>>>(m, A.rowptr, A.colind, A.vals, b, x, r64, part);
        k_reduce_partials<<<1, 256, 0, c->stream>>>(rblocks, part, sums);
        c->launches += 2;
        double h[2];
        TF_CUDA(c, cudaMemcpyAsync(h, sums, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        TF_CUDA(c, cudaStreamSynchronize(c->stream));
        double normb = std::sqrt(h[1]);
        if (normb == 0.0 || !rel) normb = 1.0;
        const double rn = std::sqrt(h[0]);
        res = rn / normb;
        if (res <= *tol) {
            *max_iter = total_inner;
            *tol = res;
            return TF_OK;
        }
        if (total_inner >= *max_iter || outer == max_outer) break;
        // inner FP32 PCG on A d = r / |r|
        k_scale_to_f32<<<grid_for(c, m), kBlock, 0, c->stream>>>(m, r64, 1.0 / rn, b32, x32);
        ++c->launches;
        double inner_tol = 0.25 * (*tol) / res;
        if (inner_tol < 2e-6) inner_tol = 2e-6;
        if (inner_tol > 0.1) inner_tol = 0.1;
        int it = 0;
        double ires = 0.;
        TF_TRY(run_pcg_kernel<float>(c, A, A.vals32, d32, b32, x32, w32, *max_iter - total_inner, inner_tol, 1, &it,
                                     &ires));
        total_inner += it >= 0 ? it : -it;
        k_axpy_f32<<<grid_for(c, m), kBlock, 0, c->stream>>>(m, rn, x32, x);
        ++c->launches;
        TF_CUDA(c, cudaGetLastError());
    }
    *max_iter = total_inner;
    *tol = res;
    return set_err(c, TF_ERR_NOT_CONVERGED, "pcg (mixed): no convergence within max_iter");
}

int gmres_jacobi(Context* c, CSR& A, const double* b, double* x, int restart, int method, int precision, int* max_iter,
                 double* tol, int rel) {
    (void)A; (void)b; (void)x; (void)restart; (void)method; (void)precision; (void)max_iter; (void)tol; (void)rel;
    return set_err(c, TF_ERR_BAD_INPUT, "gmres: not available in this build");
}

}  // namespace tf
