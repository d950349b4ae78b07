// Autotuned launch shapes of the single-system Krylov kernels.
//
// The reference has no counterpart (its kernels are OpenMP loops).  The best
// shape of the balanced SELL SpMV (threads per block x blocks per SM) and the
// best single-barrier mixed PCG (shared-memory resident, or k_pcg_cg1 with
// 512 or 256 threads per block) depend on the matrix: its rows, stored
// entries and padding, the width of its slices and how much of a block's
// share fits the shared memory.  The first call on a matrix structure --
// keyed by rows, stored entries and SELL slots, so a pattern that is rebuilt
// identically (a new time step, a new benchmark step) keeps its choice --
// times every candidate on that matrix and keeps the fastest for the
// context.  The timing runs on internal scratch vectors: the caller's x and y
// are not touched.  tf_autotune(ctx, 0) or TF_AUTOTUNE=0 keeps the fixed
// defaults; the shape switches of the environment (TF_SPMV_THREADS,
// TF_KRY_THREADS, TF_PCG_RESIDENT, ...) fix the shape they name.
#include <algorithm>

#include "tf_internal.cuh"

namespace tf {

namespace {

TuneEntry& entry_for(Context* c, const CSR& A) {
    for (auto& e : c->tuned)
        if (e.m == A.m && e.nnz == A.nnz && e.npad == A.sell.npad) return e;
    TuneEntry e;
    e.m = A.m;
    e.nnz = A.nnz;
    e.npad = A.sell.npad;
    c->tuned.push_back(e);
    return c->tuned.back();
}

__global__ void k_tune_fill(int64_t n, double* __restrict__ x, double v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = v;
}

// milliseconds between two events recorded around f() on the context stream
template <class F>
int timed(Context* c, F f, float* ms) {
    for (auto& ev : c->tune_ev)
        if (!ev) TF_CUDA(c, cudaEventCreate(&ev));
    TF_CUDA(c, cudaEventRecord(c->tune_ev[0], c->stream));
    TF_TRY(f());
    TF_CUDA(c, cudaEventRecord(c->tune_ev[1], c->stream));
    TF_CUDA(c, cudaEventSynchronize(c->tune_ev[1]));
    TF_CUDA(c, cudaEventElapsedTime(ms, c->tune_ev[0], c->tune_ev[1]));
    return TF_OK;
}

}  // namespace

int tuned_spmv_shape(Context* c, CSR& A, int* threads, int* per_sm) {
    TuneEntry& e = entry_for(c, A);
    if (e.spmv_threads == 0) {
        const int64_t m = A.m;
        TF_TRY(ensure(c, c->tune_buf, (size_t)(2 * m)));
        double* x = c->tune_buf.p;
        double* y = c->tune_buf.p + m;
        k_tune_fill<<<grid_for(c, m), kBlock, 0, c->stream>>>(m, x, 1.0);
        ++c->launches;
        static const int cand[4][2] = {{512, 1}, {512, 2}, {256, 2}, {256, 4}};
        float best = 1e30f;
        for (int k = 0; k < 4; ++k) {
            for (int w = 0; w < 2; ++w) launch_spmv_shape(c, A, x, y, cand[k][0], cand[k][1]);
            float ms = 0.f;
            TF_TRY(timed(
                c,
                [&]() {
                    for (int r = 0; r < 8; ++r) launch_spmv_shape(c, A, x, y, cand[k][0], cand[k][1]);
                    return TF_OK;
                },
                &ms));
            TF_CUDA(c, cudaGetLastError());
            e.spmv_us[k] = 1e3f * ms / 8.f;
            if (e.spmv_us[k] < best) {
                best = e.spmv_us[k];
                e.spmv_threads = cand[k][0];
                e.spmv_per_sm = cand[k][1];
            }
        }
    }
    *threads = e.spmv_threads;
    *per_sm = e.spmv_per_sm;
    return TF_OK;
}

int tuned_pcg_kind(Context* c, CSR& A, const double* b, int* kind) {
    TuneEntry& e = entry_for(c, A);
    if (e.pcg_kind < 0) {
        const int64_t m = A.m;
        TF_TRY(ensure(c, c->tune_buf, (size_t)(2 * m)));
        double* x = c->tune_buf.p;
        float best = 1e30f;
        // per-iteration time as the slope between a short and a long run, so that the launch and
        // the kernels' one-time set-up (the resident kernel loads its run into shared memory) do
        // not count: a solve runs hundreds to thousands of iterations per launch
        constexpr int kShort = 40, kLong = 160;
        const std::string keep_err = c->err;
        for (int k = kPcgResident; k <= kPcgCg1_256; ++k) {
            float ms_run[3] = {0.f, 0.f, 0.f};
            for (int pass = 0; pass < 3; ++pass) {  // warm-up (first use), short, long; from x = 0
                k_tune_fill<<<grid_for(c, m), kBlock, 0, c->stream>>>(m, x, 0.0);
                ++c->launches;
                int it = pass == 0 ? 4 : pass == 1 ? kShort : kLong;
                double tol = 1e-300;  // never reached: every run takes exactly `it` iterations
                const int st = timed(
                    c,
                    [&]() {
                        const int r = pcg_mixed_kind(c, A, b, x, k, &it, &tol, 1);
                        return r == TF_ERR_NOT_CONVERGED ? TF_OK : r;
                    },
                    &ms_run[pass]);
                if (st != TF_OK) return st;
            }
            e.pcg_us[k] = 1e3f * std::max(ms_run[2] - ms_run[1], 1e-6f) / (float)(kLong - kShort);
            if (e.pcg_us[k] < best) {
                best = e.pcg_us[k];
                e.pcg_kind = k;
            }
        }
        c->err = keep_err;  // the cut-off runs report "no convergence"; that is not the caller's error
    }
    *kind = e.pcg_kind;
    return TF_OK;
}

}  // namespace tf
