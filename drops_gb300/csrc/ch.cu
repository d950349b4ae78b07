// Surface Cahn-Hilliard time stepping on the interface space (BDF1 branch of
// surfphasesep/surfphasesep.cpp:397-440, constant mobility, no wind):
//   F_chi   = f + (1/dt) M chi
//   F_omega = beta_s M chi - M f0'(chi),  f0'(c) = xi * 2 c (1 - c) (1 - 2 c)
//   [[M/dt, mob A + rho C], [eps^2 A + beta_s M + eps^2 rho C, -M]] [chi; omega] = [F_chi; F_omega]
// solved by GMRES(restart) with nodal 2x2 block-Jacobi from the right.  State:
// TF_VEC_X = [chi; omega] (previous step = warm start), TF_VEC_CHI = chi.
#include "tf_internal.cuh"

namespace tf {

int ensure_sell(Context* c, CSR& A, bool fp32);

// one pass over the rows of M (SELL-32): M chi and M f0'(chi) together
__global__ void k_ch_rhs(int64_t m, int64_t nslices, const int32_t* __restrict__ perm, const int32_t* __restrict__ ptr,
                         const int32_t* __restrict__ col,
                         const double* __restrict__ val, const double* __restrict__ x, const double* __restrict__ f,
                         double alpha, double beta, double xi, double* __restrict__ rhs, double* __restrict__ chi_out) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t s = warp; s < nslices; s += nwarp) {
        const int32_t p0 = ptr[s], w = (ptr[s + 1] - p0) >> 5;
        double mc = 0., mf = 0.;
        for (int32_t k = 0; k < w; ++k) {
            const int32_t j = col[p0 + 32 * k + lane];
            const double v = val[p0 + 32 * k + lane];
            const double cj = x[j];
            mc += v * cj;
            mf += v * (xi * 2. * cj * (1. - cj) * (1. - 2. * cj));
        }
        const int32_t row = perm[s * 32 + lane];
        if (row >= 0) {
            rhs[row] = (f ? f[row] : 0.) + alpha * mc;
            rhs[row + m] = beta * mc - mf;
            chi_out[row] = x[row];
        }
    }
}

// right-hand side of one step from the state X = [chi; omega] into TF_VEC_B, chi into TF_VEC_CHI
int ch_rhs(Context* c, const double* X, double dt, double beta_s, double xi) {
    CSR& M = c->mats[TF_FORM_M];
    const int64_t m = M.m;
    const double* f = (int64_t)c->vecs[TF_VEC_RHS].n == m ? c->vecs[TF_VEC_RHS].p : nullptr;
    TF_TRY(ensure_sell(c, M, false));
    TF_TRY(ensure(c, c->vecs[TF_VEC_B], (size_t)(2 * m)));
    TF_TRY(ensure(c, c->vecs[TF_VEC_CHI], (size_t)m));
    k_ch_rhs<<<grid_for(c, M.sell.nslices * 32), kBlock, 0, c->stream>>>(
        m, M.sell.nslices, M.sell.perm, M.sell.ptr, M.sell.col, M.sell.v64, X, f, 1.0 / dt, beta_s, xi,
        c->vecs[TF_VEC_B].p, c->vecs[TF_VEC_CHI].p);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    return TF_OK;
}

int ch_steps(Context* c, int nsteps, double dt, double mob, double eps, double beta_s, double xi, double rho_vol,
             int restart, double tol, int max_iter, int warm, int* iters, double* resids) {
    CSR& M = c->mats[TF_FORM_M];
    if (!M.vals || !c->mats[TF_FORM_A].vals || !c->mats[TF_FORM_CN].vals)
        return set_err(c, TF_ERR_BAD_INPUT, "ch_steps: assemble M, A and C_n first");
    if (dt <= 0. || nsteps < 0) return set_err(c, TF_ERR_BAD_INPUT, "ch_steps: dt > 0, nsteps >= 0");
    const int64_t m = M.m;
    if ((int64_t)c->vecs[TF_VEC_X].n != 2 * m) return set_err(c, TF_ERR_BAD_INPUT, "ch_steps: TF_VEC_X must hold [chi; omega] (2m)");
    TF_TRY(ch_block(c, 1.0 / dt, mob, rho_vol, eps * eps, beta_s, 0));
    for (int step = 0; step < nsteps; ++step) {
        double* X = c->vecs[TF_VEC_X].p;
        TF_TRY(ch_rhs(c, X, dt, beta_s, xi));
        if (!warm) TF_CUDA(c, cudaMemsetAsync(X, 0, sizeof(double) * 2 * m, c->stream));
        int it = max_iter;
        double res = tol;
        const int st = gmres_jacobi(c, c->mats[TF_MAT_BLOCK], c->vecs[TF_VEC_B].p, X, restart, 0, TF_PREC_FP64, &it,
                                    &res, 1);
        if (iters) iters[step] = it;
        if (resids) resids[step] = res;
        if (st != TF_OK) return st;
    }
    // chi of the final state
    TF_TRY(ensure(c, c->vecs[TF_VEC_CHI], (size_t)m));
    TF_CUDA(c, cudaMemcpyAsync(c->vecs[TF_VEC_CHI].p, c->vecs[TF_VEC_X].p, sizeof(double) * m, cudaMemcpyDeviceToDevice,
                               c->stream));
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    return TF_OK;
}

// ---------------------------------------------------------------------------
// per-step statistics of surfphasesep/surfphasesep.cpp:324-345 (exportStats):
// with 1 the ones vector and f0(c) = xi (c (1 - c))^2 (:135-139),
//   area = 1'M1, raft fraction = 1'M chi / area, perimeter = eps chi'A chi,
//   Lyapunov energy = (M1)'f0(chi) + eps^2/2 chi'A chi, max / min of chi.
// Row per thread over the shared CSR pattern of M and A; FP64 partial sums
// per block in a fixed tree, then one block sums the block partials in order.
// ---------------------------------------------------------------------------
constexpr int kStatThreads = 256;

__global__ void __launch_bounds__(kStatThreads) k_ch_stats(int64_t m, const int32_t* __restrict__ rowptr,
                                                           const int32_t* __restrict__ colind,
                                                           const double* __restrict__ mv, const double* __restrict__ av,
                                                           const double* __restrict__ chi, double xi,
                                                           double* __restrict__ part /* [grid][6] */) {
    double s[4] = {0., 0., 0., 0.};
    double mx = -INFINITY, mn = INFINITY;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
        double m1 = 0., mc = 0., ac = 0.;
        for (int32_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
            const double cj = chi[colind[k]];
            m1 += mv[k];
            mc += mv[k] * cj;
            ac += av[k] * cj;
        }
        const double cr = chi[r], q = cr * (1. - cr);
        s[0] += m1;
        s[1] += mc;
        s[2] += cr * ac;
        s[3] += m1 * (xi * (q * q));
        mx = fmax(mx, cr);
        mn = fmin(mn, cr);
    }
    __shared__ double red[6][kStatThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        for (int k = 0; k < 4; ++k) s[k] += __shfl_xor_sync(0xffffffffu, s[k], o);
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    }
    if (lane == 0) {
        for (int k = 0; k < 4; ++k) red[k][w] = s[k];
        red[4][w] = mx;
        red[5][w] = mn;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        double a = red[k][0];
        for (int ww = 1; ww < kStatThreads / 32; ++ww)
            a = k < 4 ? a + red[k][ww] : (k == 4 ? fmax(a, red[k][ww]) : fmin(a, red[k][ww]));
        part[(size_t)blockIdx.x * 6 + k] = a;
    }
}

__global__ void k_ch_stats_final(int nblocks, const double* __restrict__ part, double* __restrict__ out) {
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        double a = part[k];
        for (int b = 1; b < nblocks; ++b) {
            const double v = part[(size_t)b * 6 + k];
            a = k < 4 ? a + v : (k == 4 ? fmax(a, v) : fmin(a, v));
        }
        out[k] = a;
    }
}

int ch_stats(Context* c, double eps, double xi, double* out) {
    const CSR& M = c->mats[TF_FORM_M];
    const CSR& A = c->mats[TF_FORM_A];
    if (!M.vals || !A.vals || M.pattern_gen != A.pattern_gen)
        return set_err(c, TF_ERR_BAD_INPUT, "ch_stats: assemble M and A (one pattern) first");
    const int64_t m = M.m;
    if (m <= 0 || (int64_t)c->vecs[TF_VEC_CHI].n != m)
        return set_err(c, TF_ERR_BAD_INPUT, "ch_stats: TF_VEC_CHI must hold m values");
    const int grid = grid_for(c, m, kStatThreads, 4);
    TF_TRY(ensure(c, c->scratch, sizeof(double) * (6 * (size_t)grid + 8)));
    double* part = reinterpret_cast<double*>(c->scratch.p);
    k_ch_stats<<<grid, kStatThreads, 0, c->stream>>>(m, M.rowptr, M.colind, M.vals, A.vals, c->vecs[TF_VEC_CHI].p,
                                                     xi, part);
    k_ch_stats_final<<<1, 32, 0, c->stream>>>(grid, part, part + 6 * (size_t)grid);
    c->launches += 2;
    TF_CUDA(c, cudaGetLastError());
    double r[6];
    TF_CUDA(c, cudaMemcpyAsync(r, part + 6 * (size_t)grid, sizeof r, cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    out[0] = r[0];                              // Integral.SurfacaAreaP1
    out[1] = r[1] / r[0];                       // Integral.FESolution.RaftFraction
    out[2] = eps * r[2];                        // Integral.FESolution.PerimeterEstimate
    out[3] = r[3] + 0.5 * eps * eps * r[2];     // Integral.FESolution.LyapunovEnergy
    out[4] = r[4];                              // c_h.Max
    out[5] = r[5];                              // c_h.Min
    return TF_OK;
}

}  // namespace tf
