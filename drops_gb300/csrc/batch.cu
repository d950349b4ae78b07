// Batches of independent surface problems.
//
// A batch is a concatenation of bricks (tf_mesh_brick_batch).  Classification,
// numbering, assembly and the CSR pattern run over the whole concatenation
// with the single-mesh kernels: vertex and edge ids of different instances
// are disjoint and tets are ordered instance after instance, so the
// first-touch numbering of IdxDescCL::DistributeDOFs (misc/problem.cpp:283-336)
// over the concatenation numbers every instance exactly as it would be
// numbered alone, shifted by the DOFs of the instances before it, and the
// assembled matrices are block diagonal.
//
// The solve is one persistent launch: every CTA takes instances from a work
// queue, largest first, and runs Jacobi-PCG (num/krylovsolver.h:107-189) on
// its own rows with block-wide barriers only -- no grid synchronisation, no
// cooperative launch.  Rows are processed by groups of G lanes (32/G rows per
// warp); G and the CTA size are picked by a timing autotuner on the batch
// itself.  The launch sequence (queue reset, solve, statistics copy) is
// captured once as a CUDA graph and replayed by later solves.
#include <algorithm>
#include <numeric>

#include "tf_internal.cuh"

namespace tf {

// ---------------------------------------------------------------------------
// per-instance ranges
// ---------------------------------------------------------------------------
// cut[i]: first active-tet rank of instance i; rows[i]: first DOF of instance
// i.  The first active tet of an instance touches its vertex 0 before any
// other DOF of that instance, so that DOF is the instance's first.
__global__ void k_batch_ranges(int count, const int64_t* __restrict__ tstart, const int32_t* __restrict__ active,
                               int64_t n_active, int nl, const int32_t* __restrict__ loc2glo, int64_t n_dofs,
                               int64_t* __restrict__ cut, int64_t* __restrict__ rows) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > count) return;
    const int64_t key = tstart[i];
    int64_t lo = 0, hi = n_active;  // first rank with active[rank] >= key
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if ((int64_t)active[mid] < key) lo = mid + 1; else hi = mid;
    }
    cut[i] = lo;
    rows[i] = lo < n_active ? (int64_t)loc2glo[lo * nl] : n_dofs;
}

int batch_ranges(Context* c) {
    if (c->batch_count < 1) return set_err(c, TF_ERR_BAD_INPUT, "not a batch mesh (tf_mesh_brick_batch)");
    if (!c->fe || c->legacy_numbering) return set_err(c, TF_ERR_BAD_INPUT, "batch: tf_distribute_dofs first");
    if (c->batch_dof_version == c->dof_version) return TF_OK;
    const int n = c->batch_count;
    TF_TRY(ensure(c, c->batch_rows, (size_t)2 * (n + 1)));
    const int nl = c->fe == TF_P2IF ? 10 : 4;
    k_batch_ranges<<<(n + 1 + 127) / 128, 128, 0, c->stream>>>(n, c->mesh.tstart, c->active.p, c->n_active, nl,
                                                               c->loc2glo.p, c->n_dofs, c->batch_rows.p + (n + 1),
                                                               c->batch_rows.p);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    c->h_batch_rows.assign(n + 1, 0);
    c->h_batch_cut.assign(n + 1, 0);
    TF_CUDA(c, cudaMemcpyAsync(c->h_batch_rows.data(), c->batch_rows.p, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost,
                               c->stream));
    TF_CUDA(c, cudaMemcpyAsync(c->h_batch_cut.data(), c->batch_rows.p + (n + 1), sizeof(int64_t) * (n + 1),
                               cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    c->batch_dof_version = c->dof_version;
    return TF_OK;
}

// ---------------------------------------------------------------------------
// per-instance linear combination of assembled forms
// ---------------------------------------------------------------------------
struct BatchLincombArgs {
    const double* src[8];
    int nterms, count;
    const int64_t* rows;   // count+1
    const double* coef;    // count x nterms
};

__global__ void k_batch_lincomb(int64_t m, BatchLincombArgs a, const int32_t* __restrict__ rowptr,
                                double* __restrict__ dst) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
        const double* co = a.coef + (size_t)batch_find(a.rows, a.count, r) * a.nterms;
        for (int32_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
            double s = co[0] * a.src[0][k];
            for (int t = 1; t < a.nterms; ++t) s += co[t] * a.src[t][k];
            dst[k] = s;
        }
    }
}

int batch_lincomb(Context* c, int nterms, const int* forms, const double* coeffs) {
    if (nterms < 1 || nterms > 8 || !forms || !coeffs) return set_err(c, TF_ERR_BAD_INPUT, "batch_lincomb: 1..8 terms");
    TF_TRY(batch_ranges(c));
    BatchLincombArgs a{};
    for (int t = 0; t < nterms; ++t) {
        if (!is_form_handle(forms[t]) || !c->mats[forms[t]].vals)
            return set_err(c, TF_ERR_BAD_INPUT, "batch_lincomb: form not assembled");
        if (c->mats[forms[t]].pattern_gen != c->mats[forms[0]].pattern_gen)
            return set_err(c, TF_ERR_BAD_INPUT, "batch_lincomb: forms of different patterns");
        a.src[t] = c->mats[forms[t]].vals;
    }
    const CSR& F = c->mats[forms[0]];
    if (F.m != c->n_dofs) return set_err(c, TF_ERR_BAD_INPUT, "batch_lincomb: forms do not match the numbering");
    const int n = c->batch_count;
    TF_TRY(ensure(c, c->batch_coef, (size_t)n * nterms));
    TF_CUDA(c, cudaMemcpyAsync(c->batch_coef.p, coeffs, sizeof(double) * n * nterms, cudaMemcpyHostToDevice, c->stream));
    a.nterms = nterms;
    a.count = n;
    a.rows = c->batch_rows.p;
    a.coef = c->batch_coef.p;
    CSR& S = c->mats[TF_MAT_SYS];
    TF_TRY(ensure(c, c->mat_vals[TF_MAT_SYS], (size_t)(F.nnz > 0 ? F.nnz : 1)));
    S.m = F.m;
    S.nnz = F.nnz;
    S.rowptr = F.rowptr;
    S.colind = F.colind;
    S.pattern_gen = F.pattern_gen;
    S.vals = c->mat_vals[TF_MAT_SYS].p;
    k_batch_lincomb<<<grid_for(c, S.m), kBlock, 0, c->stream>>>(S.m, a, S.rowptr, S.vals);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    TF_CUDA(c, cudaStreamSynchronize(c->stream));  // coefficients are a caller buffer
    ++S.version;
    return TF_OK;
}

// ---------------------------------------------------------------------------
// block-local building blocks
// ---------------------------------------------------------------------------
constexpr int kMaxBatchThreads = 1024;

// Sum NV values over the CTA in a fixed order (warp tree, then warp 0 over the
// warp partials in FP64) and hand the sums to f, which thread 0 alone runs:
// FP64 arithmetic issues at a small fraction of the FP32 rate on GB300, so
// the scalar recurrences of the solver run once per CTA, not once per thread,
// and reach the other threads through shared memory.  sh holds 32*4 doubles.
template <int NV, class V, class F>
__device__ __forceinline__ void cta_sum(const V (&v)[NV], double* sh, F f) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        V s = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) sh[k * 32 + warp] = (double)s;
    }
    __syncthreads();
    if (warp == 0) {
        double out[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = lane < nw ? sh[k * 32 + lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            out[k] = s;
        }
        if (lane == 0) f(out);
    }
    __syncthreads();
}

// <row of A, x> by a group of G lanes (aligned inside the warp); every lane of
// the group receives the sum.  All 32 lanes of the warp must call it.
template <int G, class V, class F>
__device__ __forceinline__ V group_row_dot(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                           const V* __restrict__ val, int64_t row, bool valid, int sub, F xval) {
    V acc = V(0);
    if (valid) {
        const int32_t b = __ldg(rowptr + row), e = __ldg(rowptr + row + 1);
        for (int32_t k = b + sub; k < e; k += G) acc += __ldg(val + k) * xval(__ldg(col + k));
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

// Two rows at once, row0 and row1, by the same group of G lanes: both rows'
// row pointers, then rounds of U entries of each row whose column and value
// loads are issued together, then their x gathers.  A pass over the rows thus
// waits for one chain of dependent loads for two rows.  Each row's products
// are added in k order, as group_row_dot adds them; every lane of the group
// receives both sums, and all 32 lanes of the warp must call it.  (The FP32
// iterations use it; in FP64 it was slower than one row at a time.)
template <int G, class V, class F>
__device__ __forceinline__ void group_row_dot2(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                               const V* __restrict__ val, int64_t row0, bool ok0, int64_t row1,
                                               bool ok1, int sub, F xval, V& s0, V& s1) {
    constexpr int U = G >= 8 ? 1 : 8 / G;
    V acc[2] = {V(0), V(0)};
    int32_t k[2] = {0, 0}, e[2] = {0, 0};
    if (ok0) {
        k[0] = __ldg(rowptr + row0) + sub;
        e[0] = __ldg(rowptr + row0 + 1);
    }
    if (ok1) {
        k[1] = __ldg(rowptr + row1) + sub;
        e[1] = __ldg(rowptr + row1 + 1);
    }
    while (k[0] < e[0] || k[1] < e[1]) {
        int32_t c[2][U];
        V v[2][U], xv[2][U];
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const bool in = k[r] + u * G < e[r];
                c[r][u] = in ? __ldg(col + k[r] + u * G) : -1;
                v[r][u] = in ? __ldg(val + k[r] + u * G) : V(0);
            }
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int u = 0; u < U; ++u) xv[r][u] = c[r][u] >= 0 ? xval(c[r][u]) : V(0);
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (c[r][u] >= 0) acc[r] += v[r][u] * xv[r][u];
        k[0] += U * G;
        k[1] += U * G;
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        acc[0] += __shfl_xor_sync(0xffffffffu, acc[0], o);
        acc[1] += __shfl_xor_sync(0xffffffffu, acc[1], o);
    }
    s0 = acc[0];
    s1 = acc[1];
}

struct BatchPcgArgs {
    int count;
    const int32_t* order;   // instances, most non-zeros first
    const int64_t* rows;    // count+1 row starts
    const int32_t* rowptr;
    const int32_t* col;
    const double* val64;
    const float* val32;
    const double* b;
    double* x;
    void* work;             // 6 m values of the work type: r, z, p0, p1, q, d
    int64_t m;
    int* queue;
    int* out_iter;          // per instance: iterations k, or -1-k when not converged
    double* out_resid;      // per instance: reached residual
    int max_iter;
    double tol;
    int rel;
    double rel_update;      // mixed: FP64 residual replacement when the FP32 one dropped by this factor
};

// scalar state of one instance's solve, owned by thread 0, read by all
struct BatchScalars {
    double rho, r_last, normb, resid, alpha;
    float alpha32, beta_f;
    double beta_d;
    int done, converged, true_res;
};

// One instance, rows [r0, r1), solved by the whole CTA.
//   V = double: PCG with Jacobi in FP64, stopping on the recursive residual
//               like the reference;
//   V = float:  FP32 iterations; x accumulates in FP64 and the FP64 true
//               residual replaces the FP32 one whenever the latter dropped by
//               a.rel_update or claims convergence (reliable updates).
template <int G, class V>
__device__ void batch_pcg_instance(const BatchPcgArgs& a, int inst, double* sh, BatchScalars& sc) {
    constexpr bool kMixed = sizeof(V) == 4;
    const int64_t r0 = a.rows[inst], r1 = a.rows[inst + 1];
    const int64_t m = a.m;
    V* r = (V*)a.work;
    V* z = r + m;
    V* pa = r + 2 * m;
    V* pb = r + 3 * m;
    V* q = r + 4 * m;
    V* d = r + 5 * m;
    const V* val = kMixed ? (const V*)a.val32 : (const V*)a.val64;
    const int nt = blockDim.x;
    const int slot = threadIdx.x / G, sub = threadIdx.x % G;
    const int per_pass = nt / G;
    const double tol = a.tol;
    const int max_iter = a.max_iter;

    // Jacobi diagonal (SolveGSstep<PB_JAC0> locates it by a row scan)
    for (int64_t i = r0 + threadIdx.x; i < r1; i += nt) {
        double di = 0.;
        for (int32_t k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k)
            if (a.col[k] == (int32_t)i) di = a.val64[k];
        d[i] = (V)di;
    }
    __syncthreads();

    // r = b - A x (FP64), z = r / d (p = z the first time); sums <r,r>, <b,b>, <z,r>
    auto true_residual = [&](bool first) {
        double v[3] = {0., 0., 0.};
        for (int64_t base = r0; base < r1; base += per_pass) {
            const int64_t row = base + slot;
            const bool valid = row < r1;
            const double ax = group_row_dot<G, double>(a.rowptr, a.col, a.val64, row, valid, sub,
                                                       [&](int32_t j) { return a.x[j]; });
            if (valid && sub == 0) {
                const double bi = a.b[row];
                const double ri = bi - ax;
                const V rv = (V)ri;
                const V zv = rv / d[row];
                r[row] = rv;
                z[row] = zv;
                if (first) pa[row] = zv;
                v[0] += ri * ri;
                v[1] += bi * bi;
                v[2] += (double)(zv * rv);
            }
        }
        if (first) {
            cta_sum<3, double>(v, sh, [&](const double* s) {
                double nb = sqrt(s[1]);
                if (nb == 0.0 || !a.rel) nb = 1.0;
                sc.normb = nb;
                sc.r_last = sqrt(s[0]);
                sc.resid = sc.r_last / nb;
                sc.rho = s[2];
                sc.converged = sc.resid <= tol;
                sc.done = sc.converged || max_iter <= 0;
                sc.beta_f = 0.f;
                sc.beta_d = 0.;
            });
        } else {  // reliable update: the FP64 residual replaces the FP32 one
            cta_sum<3, double>(v, sh, [&](const double* s) {
                sc.r_last = sqrt(s[0]);
                sc.resid = sc.r_last / sc.normb;
                sc.converged = sc.resid <= tol;
                const double rho_new = s[2];
                sc.beta_d = rho_new / sc.rho;
                sc.beta_f = (float)sc.beta_d;
                sc.rho = rho_new;
            });
        }
    };

    true_residual(true);
    V* pc = pa;
    V* pn = pb;
    int it = 0;
    // first iteration uses p = z: with beta = 0, p_new = z + 0 * p_old = z
    while (!sc.done) {
        ++it;
        const V beta = kMixed ? (V)sc.beta_f : (V)sc.beta_d;
        // phase A: p_new = z + beta p_old (on the fly), q = A p_new, <q, p_new>
        {
            V v[1] = {V(0)};
            if constexpr (!kMixed) {
                for (int64_t base = r0; base < r1; base += per_pass) {
                    const int64_t row = base + slot;
                    const bool valid = row < r1;
                    const V acc = group_row_dot<G, V>(a.rowptr, a.col, val, row, valid, sub,
                                                      [&](int32_t j) { return z[j] + beta * pc[j]; });
                    if (valid && sub == 0) {
                        const V pi = z[row] + beta * pc[row];
                        pn[row] = pi;
                        q[row] = acc;
                        v[0] += acc * pi;
                    }
                }
            } else {
                // rows base + slot and base + per_pass + slot, in that order
                for (int64_t base = r0; base < r1; base += 2 * per_pass) {
                    const int64_t rows[2] = {base + slot, base + per_pass + slot};
                    V acc[2];
                    group_row_dot2<G, V>(a.rowptr, a.col, val, rows[0], rows[0] < r1, rows[1], rows[1] < r1, sub,
                                         [&](int32_t j) { return z[j] + beta * pc[j]; }, acc[0], acc[1]);
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int64_t row = rows[h];
                        if (row < r1 && sub == 0) {
                            const V pi = z[row] + beta * pc[row];
                            pn[row] = pi;
                            q[row] = acc[h];
                            v[0] += acc[h] * pi;
                        }
                    }
                }
            }
            cta_sum<1, V>(v, sh, [&](const double* s) {
                sc.alpha = sc.rho / s[0];
                sc.alpha32 = (float)sc.alpha;
            });
        }
        // phase B: x += alpha p, r -= alpha q, z = r / d; <r,r>, <z,r>
        {
            const double alpha = sc.alpha;
            const V alphav = kMixed ? (V)sc.alpha32 : (V)alpha;
            V v[2] = {V(0), V(0)};
            for (int64_t i = r0 + threadIdx.x; i < r1; i += nt) {
                const V pi = pn[i];
                a.x[i] += alpha * (double)pi;
                const V ri = r[i] - alphav * q[i];
                const V zi = ri / d[i];
                r[i] = ri;
                z[i] = zi;
                v[0] += ri * ri;
                v[1] += zi * ri;
            }
            cta_sum<2, V>(v, sh, [&](const double* s) {
                const double rn = sqrt(s[0]);
                if (kMixed) {
                    sc.true_res = rn <= a.rel_update * sc.r_last || rn / sc.normb <= tol || it == max_iter;
                    if (!sc.true_res) {
                        sc.beta_d = s[1] / sc.rho;
                        sc.beta_f = (float)sc.beta_d;
                        sc.rho = s[1];
                    }
                } else {
                    sc.true_res = 0;
                    sc.resid = rn / sc.normb;
                    sc.converged = sc.resid <= tol;
                    sc.beta_d = s[1] / sc.rho;
                    sc.rho = s[1];
                    sc.done = sc.converged || it == max_iter;
                }
            });
        }
        if (kMixed && sc.true_res) {
            true_residual(false);
            if (threadIdx.x == 0) sc.done = sc.converged || it == max_iter;
            __syncthreads();
        }
        V* tmp = pc;
        pc = pn;
        pn = tmp;
    }
    if (threadIdx.x == 0) {
        a.out_iter[inst] = sc.converged ? it : -1 - it;
        a.out_resid[inst] = sc.resid;
    }
    __syncthreads();  // the next instance reuses sh and sc
}

template <int G, class V>
__global__ void __launch_bounds__(kMaxBatchThreads) k_batch_pcg(BatchPcgArgs a) {
    __shared__ double sh[128];
    __shared__ BatchScalars sc;
    __shared__ int next;
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(a.queue, 1);
        __syncthreads();
        const int k = next;
        __syncthreads();
        if (k >= a.count) return;
        batch_pcg_instance<G, V>(a, a.order[k], sh, sc);
    }
}

// ---------------------------------------------------------------------------
// host side: configuration, autotuner, graph
// ---------------------------------------------------------------------------
static const void* batch_kernel(int G, bool mixed) {
    if (mixed) {
        switch (G) {
            case 2: return (const void*)k_batch_pcg<2, float>;
            case 4: return (const void*)k_batch_pcg<4, float>;
            case 8: return (const void*)k_batch_pcg<8, float>;
            case 16: return (const void*)k_batch_pcg<16, float>;
        }
    } else {
        switch (G) {
            case 2: return (const void*)k_batch_pcg<2, double>;
            case 4: return (const void*)k_batch_pcg<4, double>;
            case 8: return (const void*)k_batch_pcg<8, double>;
            case 16: return (const void*)k_batch_pcg<16, double>;
        }
    }
    return nullptr;
}

static bool valid_batch_config(int G, int threads) {
    return (G == 2 || G == 4 || G == 8 || G == 16) && threads >= 64 && threads <= kMaxBatchThreads && threads % 32 == 0;
}

// everything a launch needs except the output/x pointers
struct BatchSetup {
    BatchPcgArgs a;
    const void* fn;
    int grid, threads;
};

static int batch_prepare(Context* c, CSR& A, bool mixed, int G, int threads, BatchSetup* s) {
    const int n = c->batch_count;
    const void* fn = batch_kernel(G, mixed);
    if (!fn || !valid_batch_config(G, threads)) return set_err(c, TF_ERR_BAD_INPUT, "batch: bad lanes/threads");
    int per_sm = 0;
    TF_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0));
    if (per_sm < 1) return set_err(c, TF_ERR_CAPACITY, "batch: kernel does not fit the SM at this CTA size");
    if (!A.rowptr || !A.colind || !A.vals || (mixed && !A.vals32) || !c->batch_order.p || !c->batch_rows.p)
        return set_err(c, TF_ERR_BAD_INPUT, "batch: matrix or workspace missing");
    s->fn = fn;
    s->threads = threads;
    s->grid = std::min<int64_t>(n, (int64_t)per_sm * c->num_sms);
    BatchPcgArgs& a = s->a;
    a = BatchPcgArgs{};
    a.count = n;
    a.order = c->batch_order.p;
    a.rows = c->batch_rows.p;
    a.rowptr = A.rowptr;
    a.col = A.colind;
    a.val64 = A.vals;
    a.val32 = mixed ? A.vals32 : nullptr;
    a.m = A.m;
    a.queue = c->batch_queue.p;
    a.out_iter = c->batch_iters.p;
    a.out_resid = c->batch_resid.p;
    a.work = mixed ? (void*)c->kry32.p : (void*)c->kry64.p;
    return TF_OK;
}

__global__ void k_csr_to_f32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

// FP32 copy of the CSR values (the batched kernel reads CSR, not SELL)
static int ensure_csr_f32(Context* c, CSR& A) {
    const int64_t idx = &A - c->mats;
    if (idx < 0 || idx >= TF_NUM_MATS) return set_err(c, TF_ERR_BAD_INPUT, "batch: matrix is not a context matrix");
    if (A.vals32 && A.vals32_version == A.version) return TF_OK;
    TF_TRY(ensure(c, c->mat_vals32[idx], (size_t)(A.nnz > 0 ? A.nnz : 1)));
    k_csr_to_f32<<<grid_for(c, A.nnz), kBlock, 0, c->stream>>>(A.nnz, A.vals, c->mat_vals32[idx].p);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    A.vals32 = c->mat_vals32[idx].p;
    A.vals32_version = A.version;
    return TF_OK;
}

__global__ void k_batch_nnz(int count, const int64_t* __restrict__ rows, const int32_t* __restrict__ rowptr,
                            int64_t* __restrict__ nnz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) nnz[i] = (int64_t)rowptr[rows[i + 1]] - rowptr[rows[i]];
}

// Structure of the batch for caching the queue order and the tuned launch
// shape: rebuilding the same problems gives the same key.
static std::vector<int64_t> batch_key(Context* c, const std::vector<int64_t>& nnz, bool mixed) {
    std::vector<int64_t> k(c->h_batch_rows);
    k.insert(k.end(), nnz.begin(), nnz.end());
    k.push_back(mixed);
    return k;
}

static int batch_workspace(Context* c, CSR& A, bool mixed) {
    const int n = c->batch_count;
    TF_TRY(ensure(c, c->batch_queue, 1));
    TF_TRY(ensure(c, c->batch_iters, (size_t)n));
    TF_TRY(ensure(c, c->batch_resid, (size_t)n));
    TF_TRY(ensure(c, c->batch_order, (size_t)n));
    if (mixed) {
        TF_TRY(ensure_csr_f32(c, A));
        TF_TRY(ensure(c, c->kry32, (size_t)6 * A.m + 1));
    } else {
        TF_TRY(ensure(c, c->kry64, (size_t)6 * A.m + 1));
    }
    TF_TRY(ensure(c, c->batch_xtmp, (size_t)A.m + 1));
    if (!c->h_batch_out) {
        TF_CUDA(c, cudaMallocHost((void**)&c->h_batch_out, sizeof(double) * 2 * kMaxBatchInstances));
    }
    // largest instances first (longest-processing-time order for the queue)
    if (c->batch_order_gen != A.pattern_gen) {
        TF_TRY(ensure(c, c->batch_nnz, (size_t)n));
        k_batch_nnz<<<(n + 127) / 128, 128, 0, c->stream>>>(n, c->batch_rows.p, A.rowptr, c->batch_nnz.p);
        ++c->launches;
        TF_CUDA(c, cudaGetLastError());
        std::vector<int64_t> nnz(n);
        TF_CUDA(c, cudaMemcpyAsync(nnz.data(), c->batch_nnz.p, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, c->stream));
        TF_CUDA(c, cudaStreamSynchronize(c->stream));
        if (nnz != c->h_batch_nnz) {
            std::vector<int32_t> ord(n);
            std::iota(ord.begin(), ord.end(), 0);
            std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return nnz[x] > nnz[y]; });
            TF_CUDA(c, cudaMemcpyAsync(c->batch_order.p, ord.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice,
                                       c->stream));
            TF_CUDA(c, cudaStreamSynchronize(c->stream));
            c->h_batch_nnz = nnz;
        }
        c->batch_order_gen = A.pattern_gen;
    }
    return TF_OK;
}

static int batch_launch(Context* c, const BatchSetup& s, const double* b, double* x, int max_iter, double tol, int rel) {
    BatchPcgArgs a = s.a;
    a.b = b;
    a.x = x;
    a.max_iter = max_iter;
    a.tol = tol;
    a.rel_update = c->batch_rel_update;
    a.rel = rel;
    TF_CUDA(c, cudaMemsetAsync(a.queue, 0, sizeof(int), c->stream));
    void* args[] = {&a};
    TF_CUDA(c, cudaLaunchKernel(s.fn, s.grid, s.threads, args, 0, c->stream));
    ++c->launches;
    return TF_OK;
}

// Times every (lanes per row, CTA size) candidate on this batch for a fixed
// number of iterations (tolerance 0, scratch iterate) and keeps the fastest.
int batch_tune(Context* c, CSR& A, const double* b, bool mixed, int* lanes_out, int* threads_out) {
    TF_TRY(batch_ranges(c));
    TF_TRY(batch_workspace(c, A, mixed));
    static const int kLanes[] = {2, 4, 8, 16};
    static const int kThreads[] = {128, 256, 512, 1024};
    constexpr int kTuneIters = 12;
    cudaEvent_t e0, e1;
    TF_CUDA(c, cudaEventCreate(&e0));
    TF_CUDA(c, cudaEventCreate(&e1));
    float best = 1e30f;
    int bl = 4, bt = 256;
    int st = TF_OK;
    for (int G : kLanes) {
        for (int T : kThreads) {
            BatchSetup s;
            if (batch_prepare(c, A, mixed, G, T, &s) != TF_OK) {  // does not fit: skip the candidate
                c->err.clear();
                continue;
            }
            float ms_min = 1e30f;
            for (int rep = 0; rep < 3; ++rep) {
                if (cudaMemsetAsync(c->batch_xtmp.p, 0, sizeof(double) * A.m, c->stream) != cudaSuccess) {
                    st = set_err(c, TF_ERR_CUDA, "batch_tune: memset failed");
                    break;
                }
                cudaEventRecord(e0, c->stream);
                st = batch_launch(c, s, b, c->batch_xtmp.p, kTuneIters, 0.0, 1);
                cudaEventRecord(e1, c->stream);
                if (st != TF_OK) break;
                if (cudaEventSynchronize(e1) != cudaSuccess) {
                    st = set_err(c, TF_ERR_CUDA, "batch_tune: kernel failed");
                    break;
                }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep > 0) ms_min = std::min(ms_min, ms);  // the first run warms caches
            }
            if (st != TF_OK) break;
            if (ms_min < best) {
                best = ms_min;
                bl = G;
                bt = T;
            }
        }
        if (st != TF_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    TF_TRY(st);
    c->batch_lanes = bl;
    c->batch_threads = bt;
    c->batch_tuned_key = batch_key(c, c->h_batch_nnz, mixed);
    if (lanes_out) *lanes_out = bl;
    if (threads_out) *threads_out = bt;
    return TF_OK;
}

static void drop_batch_graph(Context* c) {
    if (c->batch_exec) cudaGraphExecDestroy(c->batch_exec);
    c->batch_exec = nullptr;
    c->batch_graph_key.clear();
}

int batch_pcg(Context* c, CSR& A, const double* b, double* x, int precision, int max_iter, double tol, int rel,
              int* iters, double* resids) {
    const bool mixed = precision == TF_PREC_MIXED;
    if (precision != TF_PREC_FP64 && !mixed) return set_err(c, TF_ERR_BAD_INPUT, "batch_pcg: precision");
    if (max_iter < 0 || !(tol >= 0.)) return set_err(c, TF_ERR_BAD_INPUT, "batch_pcg: max_iter >= 0 and tol >= 0");
    TF_TRY(batch_ranges(c));
    if (A.m != c->n_dofs) return set_err(c, TF_ERR_BAD_INPUT, "batch_pcg: matrix does not match the numbering");
    const int n = c->batch_count;
    if (n > kMaxBatchInstances) return set_err(c, TF_ERR_CAPACITY, "batch_pcg: too many instances");
    TF_TRY(batch_workspace(c, A, mixed));
    if (c->batch_fixed_lanes == 0 && (c->batch_lanes == 0 || c->batch_tuned_key != batch_key(c, c->h_batch_nnz, mixed)))
        TF_TRY(batch_tune(c, A, b, mixed, nullptr, nullptr));
    const int G = c->batch_fixed_lanes ? c->batch_fixed_lanes : c->batch_lanes;
    const int T = c->batch_fixed_lanes ? c->batch_fixed_threads : c->batch_threads;
    BatchSetup s;
    TF_TRY(batch_prepare(c, A, mixed, G, T, &s));
    TimedLaunch tl(c, TF_K_BATCH);
    if (!c->batch_use_graph) {
        drop_batch_graph(c);
        TF_TRY(batch_launch(c, s, b, x, max_iter, tol, rel));
        TF_CUDA(c, cudaMemcpyAsync(c->h_batch_out, c->batch_iters.p, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
        TF_CUDA(c, cudaMemcpyAsync(c->h_batch_out + kMaxBatchInstances, c->batch_resid.p, sizeof(double) * n,
                                   cudaMemcpyDeviceToHost, c->stream));
    } else {
        union { double d; int64_t i; } tb;
        tb.d = tol;
        const std::vector<int64_t> key = {(int64_t)(intptr_t)b, (int64_t)(intptr_t)x, (int64_t)(intptr_t)A.vals,
                                          A.pattern_gen, mixed, max_iter, tb.i, rel, G, T, s.grid,
                                          (int64_t)(intptr_t)s.a.work, (int64_t)(intptr_t)s.a.val32};
        if (!c->batch_exec || key != c->batch_graph_key) {
            drop_batch_graph(c);
            cudaGraph_t g = nullptr;
            TF_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            int st = batch_launch(c, s, b, x, max_iter, tol, rel);
            if (st == TF_OK &&
                cudaMemcpyAsync(c->h_batch_out, c->batch_iters.p, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream) !=
                    cudaSuccess)
                st = set_err(c, TF_ERR_CUDA, "batch graph: capture of the statistics copy failed");
            if (st == TF_OK && cudaMemcpyAsync(c->h_batch_out + kMaxBatchInstances, c->batch_resid.p,
                                               sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess)
                st = set_err(c, TF_ERR_CUDA, "batch graph: capture of the statistics copy failed");
            const cudaError_t ec = cudaStreamEndCapture(c->stream, &g);
            TF_TRY(st);
            if (ec != cudaSuccess) return set_err(c, TF_ERR_CUDA, std::string("batch graph capture: ") + cudaGetErrorString(ec));
            const cudaError_t ei = cudaGraphInstantiate(&c->batch_exec, g, 0);
            cudaGraphDestroy(g);
            if (ei != cudaSuccess) {
                c->batch_exec = nullptr;
                return set_err(c, TF_ERR_CUDA, std::string("batch graph instantiate: ") + cudaGetErrorString(ei));
            }
            c->batch_graph_key = key;
        } else {
            ++c->launches;  // the replayed graph holds one kernel launch
        }
        TF_CUDA(c, cudaGraphLaunch(c->batch_exec, c->stream));
    }
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    const int* hi = (const int*)c->h_batch_out;
    const double* hr = c->h_batch_out + kMaxBatchInstances;
    int st = TF_OK;
    for (int i = 0; i < n; ++i) {
        if (iters) iters[i] = hi[i] < 0 ? -1 - hi[i] : hi[i];
        if (resids) resids[i] = hr[i];
        if (hi[i] < 0) st = TF_ERR_NOT_CONVERGED;
    }
    if (st != TF_OK) return set_err(c, st, "batch_pcg: some instances did not reach the tolerance");
    return TF_OK;
}

int batch_config(Context* c, int lanes, int threads, int use_graph) {
    if (lanes != 0 && !valid_batch_config(lanes, threads))
        return set_err(c, TF_ERR_BAD_INPUT, "batch_config: lanes in {2,4,8,16}, threads a multiple of 32 in [64,1024]");
    c->batch_fixed_lanes = lanes;
    c->batch_fixed_threads = lanes ? threads : 0;
    if (!lanes) {  // re-tune on the next solve
        c->batch_lanes = 0;
        c->batch_tuned_key.clear();
    }
    c->batch_use_graph = use_graph != 0;
    drop_batch_graph(c);
    return TF_OK;
}

void release_batch(Context* c) {
    drop_batch_graph(c);
    if (c->h_batch_out) cudaFreeHost(c->h_batch_out);
    c->h_batch_out = nullptr;
}

}  // namespace tf
