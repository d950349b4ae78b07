// Surface Cahn-Hilliard time stepping on the interface space (BDF1 branch of
// surfphasesep/surfphasesep.cpp:397-440, constant mobility, no wind):
//   F_chi   = f + (1/dt) M chi
//   F_omega = beta_s M chi - M f0'(chi),  f0'(c) = xi * 2 c (1 - c) (1 - 2 c)
//   [[M/dt, mob A + rho C], [eps^2 A + beta_s M + eps^2 rho C, -M]] [chi; omega] = [F_chi; F_omega]
// solved by GMRES(restart) with nodal 2x2 block-Jacobi from the right.  State:
// TF_VEC_X = [chi; omega] (previous step = warm start), TF_VEC_CHI = chi.
#include <cmath>

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

// Mobility and wind of the time loops (tf_ch_options).  Degenerate mobility:
// LaplaceM_P1P1 assembled again from the chi in TF_VEC_CHI before each solve
// (surfphasesep.cpp:414-418, 452-455), then the block matrix; wind: N_P1P1 of
// the uploaded (time-independent) wind, assembled once per loop (:417-420).
int ch_loop_begin(Context* c) {
    if (c->ch_flags & TF_CH_WIND) TF_TRY(setup_fe_system(c, 1u << TF_FORM_N, TF_RHS_NONE, nullptr, 0));
    return TF_OK;
}
int ch_step_block(Context* c, double alpha, double mob, double rho, double eps2, double beta) {
    if (c->ch_flags & TF_CH_DEGENERATE_MOBILITY)
        TF_TRY(setup_fe_system(c, 1u << TF_FORM_LAPM, TF_RHS_NONE, nullptr, 0));
    return ch_block(c, alpha, mob, rho, eps2, beta, c->ch_flags);
}

__global__ void k_ch_extrap(int64_t m, const double* __restrict__ chi, const double* __restrict__ prev, double r,
                            double* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (1. + r) * chi[i] - r * prev[i];
}

int ch_steps(Context* c, int nsteps, double dt, double mob, double eps, double beta_s, double xi, double rho_vol,
             int restart, double tol, int max_iter, int warm, int* iters, double* resids) {
    CSR& M = c->mats[TF_FORM_M];
    if (!M.vals || !c->mats[TF_FORM_A].vals || !c->mats[TF_FORM_CN].vals)
        return set_err(c, TF_ERR_BAD_INPUT, "ch_steps: assemble M, A and C_n first");
    if (dt <= 0. || nsteps < 0) return set_err(c, TF_ERR_BAD_INPUT, "ch_steps: dt > 0, nsteps >= 0");
    const int64_t m = M.m;
    if ((int64_t)c->vecs[TF_VEC_X].n != 2 * m) return set_err(c, TF_ERR_BAD_INPUT, "ch_steps: TF_VEC_X must hold [chi; omega] (2m)");
    TF_TRY(ch_loop_begin(c));
    const bool per_step = c->ch_flags & TF_CH_DEGENERATE_MOBILITY;
    if (!per_step) TF_TRY(ch_block(c, 1.0 / dt, mob, rho_vol, eps * eps, beta_s, c->ch_flags));
    for (int step = 0; step < nsteps; ++step) {
        double* X = c->vecs[TF_VEC_X].p;
        TF_TRY(ch_rhs(c, X, dt, beta_s, xi));  // also TF_VEC_CHI = chi_n
        if (per_step) TF_TRY(ch_step_block(c, 1.0 / dt, mob, rho_vol, eps * eps, beta_s));
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
// adaptive BDF1/BDF2 stepping (surfphasesep/surfphasesep.cpp:397-483)
// ---------------------------------------------------------------------------
// BDF2 right-hand side (:456-460) in one pass over M (SELL-32), chi_ext on the fly
__global__ void k_ch_rhs2(int64_t m, int64_t nslices, const int32_t* __restrict__ perm,
                          const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                          const double* __restrict__ val, const double* __restrict__ chi,
                          const double* __restrict__ chi_prev, const double* __restrict__ f, double r, double dt,
                          double beta, double xi, double* __restrict__ rhs) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t s = warp; s < nslices; s += nwarp) {
        const int32_t p0 = ptr[s], w = (ptr[s + 1] - p0) >> 5;
        double mc = 0., mp = 0., me = 0., mf = 0.;
        for (int32_t k = 0; k < w; ++k) {
            const int32_t j = col[p0 + 32 * k + lane];
            const double v = val[p0 + 32 * k + lane];
            const double cj = chi[j], pj = chi_prev[j];
            const double ce = (1. + r) * cj - r * pj;
            mc += v * cj;
            mp += v * pj;
            me += v * ce;
            mf += v * (xi * 2. * ce * (1. - ce) * (1. - 2. * ce));
        }
        const int32_t row = perm[s * 32 + lane];
        if (row >= 0) {
            rhs[row] = (f ? f[row] : 0.) + ((1. + r) / dt) * mc - (r * r / (1. + r) / dt) * mp;
            rhs[row + m] = beta * me - mf;
        }
    }
}

// d'M d and x2'M x2 for d = x2 - x1 (chi parts), per block, then in order
__global__ void __launch_bounds__(256) k_ch_err(int64_t m, const int32_t* __restrict__ rowptr,
                                                const int32_t* __restrict__ colind, const double* __restrict__ mv,
                                                const double* __restrict__ x1, const double* __restrict__ x2,
                                                double* __restrict__ part) {
    double s0 = 0., s1 = 0.;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
        double md = 0., m2 = 0.;
        for (int32_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
            const int32_t j = colind[k];
            md += mv[k] * (x2[j] - x1[j]);
            m2 += mv[k] * x2[j];
        }
        s0 += (x2[r] - x1[r]) * md;
        s1 += x2[r] * m2;
    }
    __shared__ double red[2][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    if (lane == 0) {
        red[0][w] = s0;
        red[1][w] = s1;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        double a = 0.;
        for (int ww = 0; ww < 8; ++ww) a += red[threadIdx.x][ww];
        part[2 * (size_t)blockIdx.x + threadIdx.x] = a;
    }
}

__global__ void k_ch_err_final(int nblocks, const double* __restrict__ part, double* __restrict__ out) {
    if (threadIdx.x < 2) {
        double a = 0.;
        for (int b = 0; b < nblocks; ++b) a += part[2 * (size_t)b + threadIdx.x];
        out[threadIdx.x] = a;
    }
}

static int ch_rel_error(Context* c, const double* x1, const double* x2, double* e) {
    const CSR& M = c->mats[TF_FORM_M];
    const int grid = grid_for(c, M.m, 256, 4);
    TF_TRY(ensure(c, c->scratch, sizeof(double) * (2 * (size_t)grid + 4)));
    double* part = reinterpret_cast<double*>(c->scratch.p);
    k_ch_err<<<grid, 256, 0, c->stream>>>(M.m, M.rowptr, M.colind, M.vals, x1, x2, part);
    k_ch_err_final<<<1, 32, 0, c->stream>>>(grid, part, part + 2 * (size_t)grid);
    c->launches += 2;
    TF_CUDA(c, cudaGetLastError());
    double r[2];
    TF_CUDA(c, cudaMemcpyAsync(r, part + 2 * (size_t)grid, sizeof r, cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    *e = r[1] > 0. ? std::sqrt(r[0] / r[1]) : 0.;
    return TF_OK;
}

// the step-size rule F of surfphasesep.cpp:117-123
static double ch_next_dt(const tf_ch_adapt_params& P, double e, double dt) {
    if (e == 0.) return P.dt0;
    const double f = P.F_rho * std::sqrt(P.F_tol / e) * dt;
    if (f > P.F_max) return P.F_max;
    if (f < P.F_min) return P.F_min;
    return f;
}

int ch_steps_adaptive(Context* c, const tf_ch_adapt_params& P, int* nsteps, double* t_end, double* dts, double* errs,
                      int* tries, int* iters) {
    CSR& M = c->mats[TF_FORM_M];
    if (!M.vals || !c->mats[TF_FORM_A].vals || !c->mats[TF_FORM_CN].vals)
        return set_err(c, TF_ERR_BAD_INPUT, "ch_steps_adaptive: assemble M, A and C_n first");
    if (!(P.dt0 > 0.) || P.max_steps < 0 || (P.adaptive && !(P.F_min > 0. && P.F_min <= P.F_max && P.F_tol > 0.)))
        return set_err(c, TF_ERR_BAD_INPUT, "ch_steps_adaptive: dt0 > 0, 0 < F_min <= F_max, F_tol > 0");
    const int64_t m = M.m;
    if ((int64_t)c->vecs[TF_VEC_X].n != 2 * m)
        return set_err(c, TF_ERR_BAD_INPUT, "ch_steps_adaptive: TF_VEC_X must hold [chi; omega] (2m)");
    TF_TRY(ensure_sell(c, M, false));
    TF_TRY(ensure(c, c->ch_prev, (size_t)m));
    TF_TRY(ensure(c, c->ch_x1, (size_t)(2 * m)));
    TF_TRY(ensure(c, c->ch_x2, (size_t)(2 * m)));
    TF_TRY(ensure(c, c->vecs[TF_VEC_B], (size_t)(2 * m)));
    const double* f = (int64_t)c->vecs[TF_VEC_RHS].n == m ? c->vecs[TF_VEC_RHS].p : nullptr;
    const size_t bytes2 = sizeof(double) * 2 * (size_t)m;
    TF_TRY(ch_loop_begin(c));
    double t = P.t0, dt = P.dt0, e = 0.;
    int i = 0;
    constexpr int kMaxTries = 64;
    while (t < P.t_final && i < P.max_steps) {
        ++i;
        const double t_prev = t, dt_prev = dt;
        int ntry = 0, its = 0;
        double* X = c->vecs[TF_VEC_X].p;
        do {
            ++ntry;
            if (i == 1 || P.adaptive) dt = ch_next_dt(P, e, dt);
            t = t_prev + dt;
            // BDF1 (surfphasesep.cpp:412-440)
            TF_TRY(ch_rhs(c, X, dt, P.beta_s, P.xi));  // also TF_VEC_CHI = chi (mobility of the BDF1 solve)
            TF_TRY(ch_step_block(c, 1.0 / dt, P.mobility, P.rho_vol, P.eps * P.eps, P.beta_s));
            TF_CUDA(c, cudaMemcpyAsync(c->ch_x1.p, X, bytes2, cudaMemcpyDeviceToDevice, c->stream));
            int it = P.max_iter;
            double res = P.tol;
            int st = gmres_jacobi(c, c->mats[TF_MAT_BLOCK], c->vecs[TF_VEC_B].p, c->ch_x1.p, P.restart, 0,
                                  TF_PREC_FP64, &it, &res, 1);
            if (st != TF_OK) return st;
            its += it;
            if (i == 1) {  // BDF2 solution = BDF1 solution (:447-451)
                TF_CUDA(c, cudaMemcpyAsync(c->ch_x2.p, c->ch_x1.p, bytes2, cudaMemcpyDeviceToDevice, c->stream));
                break;
            }
            // BDF2 (:452-476)
            const double r = dt / dt_prev;
            k_ch_rhs2<<<grid_for(c, M.sell.nslices * 32), kBlock, 0, c->stream>>>(
                m, M.sell.nslices, M.sell.perm, M.sell.ptr, M.sell.col, M.sell.v64, X, c->ch_prev.p, f, r, dt,
                P.beta_s, P.xi, c->vecs[TF_VEC_B].p);
            ++c->launches;
            TF_CUDA(c, cudaGetLastError());
            if (c->ch_flags & TF_CH_DEGENERATE_MOBILITY) {  // mobility of the BDF2 solve from chi_ext
                k_ch_extrap<<<grid_for(c, m), kBlock, 0, c->stream>>>(m, X, c->ch_prev.p, r, c->vecs[TF_VEC_CHI].p);
                ++c->launches;
            }
            TF_TRY(ch_step_block(c, (1. + 2. * r) / (1. + r) / dt, P.mobility, P.rho_vol, P.eps * P.eps, P.beta_s));
            TF_CUDA(c, cudaMemcpyAsync(c->ch_x2.p, c->ch_x1.p, bytes2, cudaMemcpyDeviceToDevice, c->stream));
            it = P.max_iter;
            res = P.tol;
            st = gmres_jacobi(c, c->mats[TF_MAT_BLOCK], c->vecs[TF_VEC_B].p, c->ch_x2.p, P.restart, 0, TF_PREC_FP64,
                              &it, &res, 1);
            if (st != TF_OK) return st;
            its += it;
            TF_TRY(ch_rel_error(c, c->ch_x1.p, c->ch_x2.p, &e));
        } while (P.adaptive && e > P.F_tol && P.F_min < dt && dt < P.F_max && ntry < kMaxTries);
        // chi_prev = chi; [chi; omega] = BDF2 solution (:481-485)
        TF_CUDA(c, cudaMemcpyAsync(c->ch_prev.p, X, sizeof(double) * m, cudaMemcpyDeviceToDevice, c->stream));
        TF_CUDA(c, cudaMemcpyAsync(X, c->ch_x2.p, bytes2, cudaMemcpyDeviceToDevice, c->stream));
        if (dts) dts[i - 1] = dt;
        if (errs) errs[i - 1] = e;
        if (tries) tries[i - 1] = ntry;
        if (iters) iters[i - 1] = its;
    }
    TF_TRY(ensure(c, c->vecs[TF_VEC_CHI], (size_t)m));
    TF_CUDA(c, cudaMemcpyAsync(c->vecs[TF_VEC_CHI].p, c->vecs[TF_VEC_X].p, sizeof(double) * m,
                               cudaMemcpyDeviceToDevice, c->stream));
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    if (nsteps) *nsteps = i;
    if (t_end) *t_end = t;
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
