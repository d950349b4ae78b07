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

}  // namespace tf
