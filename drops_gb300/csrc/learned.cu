// Learned warm start of the Cahn-Hilliard steps.
//
// The reference starts every GMRES solve of surfphasesep.cpp:397-440 from the
// previous step's state (UsePreviousFrameAsInitialGuess).  Here a per-DOF MLP
// (mlp.cu) predicts the increment of [chi; omega] over the next step from the
// last two states around the DOF; the guess is state + predicted increment.
// The network is trained online on the increments the solver itself
// produces during the first `train_steps` steps.
//
// Inputs of DOF i (80, BF16): for slot s = 0..15 -- the DOF itself, then its
// first 15 neighbours in the row of the mass matrix (the 1-ring), zeros when
// the row is shorter --
//     2 (chi_n - 1/2),  (chi_n - chi_{n-1}) / s_chi,  omega_n / S_omega,
//     (omega_n - omega_{n-1}) / s_omega
// at that DOF; then the DOF's coordinates, the unit normal of the level set
// in the tet that first touched the DOF, the constant 1 (bias), zeros.
// s_chi, s_omega are the RMS increments of the last step and S_omega the RMS
// of omega_n.  The network corrects linear extrapolation: its targets are
// ((chi_{n+1} - chi_n) - (chi_n - chi_{n-1})) / s_chi and the same for omega,
// and the guess is x_n + (x_n - x_{n-1}) + s * prediction, so an untrained
// network (prediction ~ 0) already gives the extrapolated state.
//
// Minimal-residual projection.  A restarted GMRES(50) solve to 1e-10 gains
// only a little from a better start, and a correction of linear
// extrapolation gains nothing unless it is very accurate.  The guess of
// learned = 1 is therefore the combination of the recent states and the
// network's correction that minimises the FP64 residual: with the backward
// differences D_0 = x_n, D_1 = x_n - x_{n-1}, ... of the last kProjStates
// states and the correction vector s * prediction as basis V, it solves
// min_c ||b - A V c|| (the Gram matrix of A V in FP64, scaled by its
// diagonal and solved by a truncated eigen-decomposition on the host) and
// starts from V c.  learned = 3 is the same projection without the network,
// so the network's own contribution is the difference between the two.
// Both contain x_n and the extrapolated state in their span, so neither
// starts from a larger residual than the previous state or extrapolation.
//
// Guard: the learned guess is used only when its FP64 residual is smaller
// than the previous-step guess's, and after a step whose learned solve took
// more than 5/4 of the GMRES iterations of the last plain solve the next step
// falls back to the previous-step guess.
//
// Compiled without contraction (like the mesh code), so features equal a host
// restatement in IEEE double bit for bit.
#include <algorithm>
#include <cmath>

#include "tf_internal.cuh"

namespace tf {

constexpr int kFeat = 80, kSlots = 16;

// coordinates and level-set normal of every DOF (P1 numbering of DistributeDOFs)
__global__ void k_dof_geometry(MeshView M, const int32_t* __restrict__ dof_vert, const int32_t* __restrict__ keys_v,
                               const int32_t* __restrict__ active, const double* __restrict__ lsv,
                               float* __restrict__ xyz, float* __restrict__ nrm) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < M.nv; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t d = dof_vert[v];
        if (d < 0) continue;
        double x[3];
        mesh_coord(M, (int32_t)v, x);
        const int32_t tet = active[keys_v[v] / 4];
        int32_t tv[4];
        mesh_tet(M, tet, tv, nullptr);
        double p[4][3], f[4];
        for (int k = 0; k < 4; ++k) {
            mesh_coord(M, tv[k], p[k]);
            f[k] = lsv[tv[k]];
        }
        double e[3][3];
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) e[k][c] = p[k + 1][c] - p[0][c];
        // gradient of the linear interpolant: sum_k (f_k - f_0) (e_{k+1} x e_{k+2}) / det
        double g[3] = {0., 0., 0.};
        for (int k = 0; k < 3; ++k) {
            const double* a = e[(k + 1) % 3];
            const double* b = e[(k + 2) % 3];
            const double cr[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
            for (int c = 0; c < 3; ++c) g[c] += (f[k + 1] - f[0]) * cr[c];
        }
        const double nn = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        const double inv = nn > 0. ? 1.0 / nn : 0.;
        for (int c = 0; c < 3; ++c) {
            xyz[3 * (int64_t)d + c] = (float)x[c];
            nrm[3 * (int64_t)d + c] = (float)(g[c] * inv);
        }
    }
}

// out[0..2] = RMS(chi_n - chi_{n-1}), RMS(omega_n - omega_{n-1}), RMS(omega_n); one block, fixed order
__global__ void k_ch_scales(int64_t m, const double* __restrict__ xn, const double* __restrict__ xp,
                            double* __restrict__ out) {
    __shared__ double sh[3][32];
    double s[3] = {0., 0., 0.};
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
        const double dc = xn[i] - xp[i], dw = xn[m + i] - xp[m + i], w = xn[m + i];
        s[0] += dc * dc;
        s[1] += dw * dw;
        s[2] += w * w;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < 3; ++k) {
        double v = s[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sh[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double v = 0.;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += sh[threadIdx.x][w];
        const double r = sqrt(v / (double)(m > 0 ? m : 1));
        out[threadIdx.x] = r > 1e-300 ? r : 1e-300;
    }
}

// inputs of every DOF from (x_n, x_{n-1}); targets from x_{n+1} when given
__global__ void k_ch_features(int64_t m, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                              const double* __restrict__ xn, const double* __restrict__ xp,
                              const double* __restrict__ xnext, const double* __restrict__ sc,
                              const float* __restrict__ xyz, const float* __restrict__ nrm, __nv_bfloat16* __restrict__ X,
                              float* __restrict__ Y) {
    const double s_c = sc[0], s_w = sc[1], S_w = sc[2];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        __align__(16) __nv_bfloat16 f[kFeat];
        int32_t slot[kSlots];
        int ns = 0;
        slot[ns++] = (int32_t)i;
        for (int32_t k = rowptr[i]; k < rowptr[i + 1] && ns < kSlots; ++k)
            if (colind[k] != (int32_t)i) slot[ns++] = colind[k];
        for (int s = 0; s < kSlots; ++s) {
            double v[4] = {0., 0., 0., 0.};
            if (s < ns) {
                const int32_t j = slot[s];
                v[0] = 2.0 * (xn[j] - 0.5);
                v[1] = (xn[j] - xp[j]) / s_c;
                v[2] = xn[m + j] / S_w;
                v[3] = (xn[m + j] - xp[m + j]) / s_w;
            }
            for (int q = 0; q < 4; ++q) f[4 * s + q] = __float2bfloat16_rn((float)v[q]);
        }
        for (int c = 0; c < 3; ++c) {
            f[64 + c] = __float2bfloat16_rn(xyz[3 * i + c]);
            f[67 + c] = __float2bfloat16_rn(nrm[3 * i + c]);
        }
        f[70] = __float2bfloat16_rn(1.f);
        for (int q = 71; q < kFeat; ++q) f[q] = __float2bfloat16_rn(0.f);
        uint4* dst = reinterpret_cast<uint4*>(X + i * kFeat);
        const uint4* src = reinterpret_cast<const uint4*>(f);
        for (int q = 0; q < kFeat / 8; ++q) dst[q] = src[q];
        if (Y && xnext) {
            Y[2 * i] = (float)(((xnext[i] - xn[i]) - (xn[i] - xp[i])) / s_c);
            Y[2 * i + 1] = (float)(((xnext[m + i] - xn[m + i]) - (xn[m + i] - xp[m + i])) / s_w);
        }
    }
}

// guess = x_n + (x_n - x_{n-1}) + (s_chi, s_omega) * prediction (pred == nullptr: extrapolation only)
__global__ void k_ch_apply(int64_t m, const double* __restrict__ xn, const double* __restrict__ xp,
                           const float* __restrict__ pred, const double* __restrict__ sc, double* __restrict__ guess) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 2 * m; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t d = i < m ? i : i - m;
        const double corr = pred ? sc[i < m ? 0 : 1] * (double)pred[2 * d + (i < m ? 0 : 1)] : 0.;
        guess[i] = (xn[i] + (xn[i] - xp[i])) + corr;
    }
}

constexpr int kProjStates = 6;  // states of the projection basis (backward differences)
constexpr int kProjMax = kProjStates + 1;

// backward differences of the ring of states (newest first): D_j = sum_k (-1)^k C(j,k) s_k
struct RingPtrs {
    const double* s[kProjStates];
    double* d[kProjStates];
};
__global__ void k_ch_diffs(int64_t n, int ns, RingPtrs R) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double t[kProjStates];
        for (int k = 0; k < ns; ++k) t[k] = R.s[k][i];
        // difference table: after level j, t[0] holds D_j
        for (int j = 0; j < ns; ++j) {
            R.d[j][i] = t[0];
            for (int k = 0; k + 1 < ns - j; ++k) t[k] = t[k] - t[k + 1];
        }
    }
}

// all products <y_j, y_k> (j <= k) and <y_j, b> of nv vectors, per block (blockIdx.y = product)
struct DotPtrs {
    const double* a[kProjMax * (kProjMax + 1) / 2 + kProjMax];
    const double* b[kProjMax * (kProjMax + 1) / 2 + kProjMax];
};
__global__ void k_ch_dots(int64_t n, DotPtrs P, double* __restrict__ part) {
    __shared__ double sh[32];
    const double* __restrict__ a = P.a[blockIdx.y];
    const double* __restrict__ b = P.b[blockIdx.y];
    double s = 0.;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += a[i] * b[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += sh[w];
        part[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = v;
    }
}

// guess = sum_j c_j V_j
struct CombPtrs {
    const double* v[kProjMax];
    double c[kProjMax];
};
__global__ void k_ch_combine(int64_t n, int nv, CombPtrs C, double* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double g = 0.;
        for (int j = 0; j < nv; ++j) g += C.c[j] * C.v[j][i];
        out[i] = g;
    }
}

// correction vector of the network: (s_chi, s_omega) * prediction
__global__ void k_ch_corr(int64_t m, const float* __restrict__ pred, const double* __restrict__ sc,
                          double* __restrict__ corr) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 2 * m; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t d = i < m ? i : i - m;
        corr[i] = sc[i < m ? 0 : 1] * (double)pred[2 * d + (i < m ? 0 : 1)];
    }
}

// ||b - A x||^2 into out (one value), fixed order: rows in chunks, one block
__global__ void k_resid_sq(int64_t m, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                           const double* __restrict__ val, const double* __restrict__ b, const double* __restrict__ x,
                           double* __restrict__ part) {
    __shared__ double sh[32];
    double s = 0.;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
        double ax = 0.;
        for (int32_t k = rp[r]; k < rp[r + 1]; ++k) ax += val[k] * x[ci[k]];
        const double d = b[r] - ax;
        s += d * d;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += sh[w];
        part[blockIdx.x] = v;
    }
}

static int resid_norm(Context* c, const CSR& A, const double* b, const double* x, double* out) {
    const int blocks = 2 * c->num_sms;
    TF_TRY(ensure(c, c->ch_part, (size_t)blocks));
    k_resid_sq<<<blocks, 256, 0, c->stream>>>(A.m, A.rowptr, A.colind, A.vals, b, x, c->ch_part.p);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    std::vector<double> h(blocks);
    TF_CUDA(c, cudaMemcpyAsync(h.data(), c->ch_part.p, sizeof(double) * blocks, cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    double s = 0.;
    for (double v : h) s += v;
    *out = std::sqrt(s);
    return TF_OK;
}

// Symmetric eigen-decomposition of a small n x n matrix (cyclic Jacobi
// rotations); a is overwritten, eigenvalues in w, eigenvectors in the columns of v.
static void sym_eig(int n, double a[kProjMax][kProjMax], double w[kProjMax], double v[kProjMax][kProjMax]) {
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) v[i][j] = i == j ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) off += a[p][q] * a[p][q];
        if (off < 1e-300) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                if (a[p][q] == 0.) continue;
                const double th = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
                const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
                const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
                for (int k = 0; k < n; ++k) {
                    const double akp = a[k][p], akq = a[k][q];
                    a[k][p] = cs * akp - sn * akq;
                    a[k][q] = sn * akp + cs * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = cs * apk - sn * aqk;
                    a[q][k] = sn * apk + cs * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = cs * vkp - sn * vkq;
                    v[k][q] = sn * vkp + cs * vkq;
                }
            }
    }
    for (int i = 0; i < n; ++i) w[i] = a[i][i];
}

// guess = V c with c = argmin ||b - A V c|| over the nv basis vectors V (device);
// scratch ch_av holds A V
static int ch_project(Context* c, CSR& B, const double* b, const double* const* V, int nv, double* guess) {
    const int64_t n = B.m;
    TF_TRY(ensure(c, c->ch_av, (size_t)(kProjMax * n)));
    for (int j = 0; j < nv; ++j) TF_TRY(spmv(c, B, V[j], c->ch_av.p + (size_t)j * n));
    DotPtrs P{};
    int np = 0;
    int pj[kProjMax * (kProjMax + 1) / 2 + kProjMax], pk[kProjMax * (kProjMax + 1) / 2 + kProjMax];
    for (int j = 0; j < nv; ++j)
        for (int k = j; k <= nv; ++k) {  // k == nv: the right-hand side
            P.a[np] = c->ch_av.p + (size_t)j * n;
            P.b[np] = k < nv ? c->ch_av.p + (size_t)k * n : b;
            pj[np] = j;
            pk[np] = k;
            ++np;
        }
    const int gx = c->num_sms;
    TF_TRY(ensure(c, c->ch_part, (size_t)(gx * np)));
    k_ch_dots<<<dim3(gx, np), 256, 0, c->stream>>>(n, P, c->ch_part.p);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    std::vector<double> h((size_t)gx * np);
    TF_CUDA(c, cudaMemcpyAsync(h.data(), c->ch_part.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    double G[kProjMax][kProjMax] = {}, r[kProjMax] = {};
    for (int q = 0; q < np; ++q) {
        double sum = 0.;
        for (int x = 0; x < gx; ++x) sum += h[(size_t)q * gx + x];
        if (pk[q] == nv) r[pj[q]] = sum;
        else G[pj[q]][pk[q]] = G[pk[q]][pj[q]] = sum;
    }
    // scale by the diagonal, truncated eigen-solve (directions below 1e-12 of the largest are dropped)
    double sc[kProjMax], Gs[kProjMax][kProjMax], w[kProjMax], U[kProjMax][kProjMax], cf[kProjMax] = {};
    for (int j = 0; j < nv; ++j) sc[j] = G[j][j] > 0. ? 1.0 / std::sqrt(G[j][j]) : 0.;
    for (int j = 0; j < nv; ++j)
        for (int k = 0; k < nv; ++k) Gs[j][k] = sc[j] * G[j][k] * sc[k];
    sym_eig(nv, Gs, w, U);
    double wmax = 0.;
    for (int j = 0; j < nv; ++j) wmax = std::max(wmax, w[j]);
    for (int e = 0; e < nv; ++e) {
        if (!(w[e] > 1e-12 * wmax)) continue;
        double t = 0.;
        for (int j = 0; j < nv; ++j) t += U[j][e] * sc[j] * r[j];
        t /= w[e];
        for (int j = 0; j < nv; ++j) cf[j] += U[j][e] * t;
    }
    CombPtrs Cp{};
    for (int j = 0; j < nv; ++j) {
        Cp.v[j] = V[j];
        Cp.c[j] = cf[j] * sc[j];
    }
    k_ch_combine<<<grid_for(c, n), kBlock, 0, c->stream>>>(n, nv, Cp, guess);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    return TF_OK;
}

int ch_geometry(Context* c) {
    if (c->fe != TF_P1IF || c->legacy_numbering)
        return set_err(c, TF_ERR_BAD_INPUT, "learned warm start: P1 DistributeDOFs numbering required");
    if (c->ch_geom_version == c->dof_version) return TF_OK;
    const int64_t m = c->n_dofs;
    TF_TRY(ensure(c, c->ch_xyz, (size_t)(3 * m)));
    TF_TRY(ensure(c, c->ch_nrm, (size_t)(3 * m)));
    k_dof_geometry<<<grid_for(c, c->mesh.nv), kBlock, 0, c->stream>>>(c->mesh, c->dof_vert.p, c->keys_v.p, c->active.p,
                                                                      c->ls_vert.p, c->ch_xyz.p, c->ch_nrm.p);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    c->ch_geom_version = c->dof_version;
    return TF_OK;
}

// features (and targets when xnext != nullptr) of all DOFs into ch_X / ch_Y
int ch_features_dev(Context* c, const double* xn, const double* xp, const double* xnext) {
    const CSR& M = c->mats[TF_FORM_M];
    const int64_t m = M.m;
    TF_TRY(ch_geometry(c));
    TF_TRY(ensure(c, c->ch_X, (size_t)(kFeat * m)));
    TF_TRY(ensure(c, c->ch_Y, (size_t)(2 * m)));
    TF_TRY(ensure(c, c->ch_scales, 4));
    k_ch_scales<<<1, 1024, 0, c->stream>>>(m, xn, xp, c->ch_scales.p);
    k_ch_features<<<grid_for(c, m), kBlock, 0, c->stream>>>(m, M.rowptr, M.colind, xn, xp, xnext, c->ch_scales.p,
                                                            c->ch_xyz.p, c->ch_nrm.p, c->ch_X.p, c->ch_Y.p);
    c->launches += 2;
    TF_CUDA(c, cudaGetLastError());
    return TF_OK;
}

int ch_targets_dev(Context* c, const double* xn, const double* xp, const double* xnext) {
    return ch_features_dev(c, xn, xp, xnext);
}

int ch_steps_learned(Context* c, const ChLearnParams& P, int* iters, double* resids, int* used) {
    CSR& M = c->mats[TF_FORM_M];
    if (!M.vals || !c->mats[TF_FORM_A].vals || !c->mats[TF_FORM_CN].vals)
        return set_err(c, TF_ERR_BAD_INPUT, "ch_steps_learned: assemble M, A and C_n first");
    if (P.dt <= 0. || P.nsteps < 0) return set_err(c, TF_ERR_BAD_INPUT, "ch_steps_learned: dt > 0, nsteps >= 0");
    const int64_t m = M.m;
    if ((int64_t)c->vecs[TF_VEC_X].n != 2 * m)
        return set_err(c, TF_ERR_BAD_INPUT, "ch_steps_learned: TF_VEC_X must hold [chi; omega] (2m)");
    TF_TRY(ch_geometry(c));
    TF_TRY(ch_loop_begin(c));
    const bool per_step = c->ch_flags & TF_CH_DEGENERATE_MOBILITY;
    if (!per_step) TF_TRY(ch_block(c, 1.0 / P.dt, P.mob, P.rho_vol, P.eps * P.eps, P.beta_s, c->ch_flags));
    CSR& B = c->mats[TF_MAT_BLOCK];
    TF_TRY(ensure(c, c->ch_hist, (size_t)(6 * m)));  // x_old, guess
    TF_TRY(ensure(c, c->ch_pred, (size_t)(2 * m)));
    double* x_old = c->ch_hist.p;
    double* guess = c->ch_hist.p + 2 * m;
    double* x_prev = c->ch_hist.p + 4 * m;  // x_n kept for the targets
    TF_CUDA(c, cudaMemcpyAsync(x_old, c->vecs[TF_VEC_X].p, sizeof(double) * 2 * m, cudaMemcpyDeviceToDevice, c->stream));
    // projection: ring of the last kProjStates states (slot of state n: n % kProjStates), their
    // differences and the network's correction vector
    const bool project = P.learned == 1 || P.learned == 3;
    int ring_n = 0, ring_head = -1;
    if (project) {
        TF_TRY(ensure(c, c->ch_ring, (size_t)(2 * kProjStates + 1) * 2 * m));
        ring_head = 0;
        ring_n = 1;
        TF_CUDA(c, cudaMemcpyAsync(c->ch_ring.p, c->vecs[TF_VEC_X].p, sizeof(double) * 2 * m, cudaMemcpyDeviceToDevice,
                                   c->stream));
    }
    auto ring_state = [&](int k) { return c->ch_ring.p + (size_t)((ring_head - k + kProjStates) % kProjStates) * 2 * m; };
    double* diffs = project ? c->ch_ring.p + (size_t)kProjStates * 2 * m : nullptr;
    double* corr = project ? c->ch_ring.p + (size_t)(2 * kProjStates) * 2 * m : nullptr;
    int trained = 0, plain_ref = -1;
    bool fallback_next = false;
    c->ch_train_loss = 0.;
    for (int step = 0; step < P.nsteps; ++step) {
        double* X = c->vecs[TF_VEC_X].p;  // x_n (previous state)
        TF_TRY(ch_rhs(c, X, P.dt, P.beta_s, P.xi));
        if (per_step) TF_TRY(ch_step_block(c, 1.0 / P.dt, P.mob, P.rho_vol, P.eps * P.eps, P.beta_s));
        const bool have_hist = step > 0;
        bool use = false;
        if (have_hist) TF_TRY(ch_features_dev(c, X, x_old, nullptr));
        const bool mlp_ready = P.learned == 1 && trained >= P.min_trained;
        if (have_hist && !fallback_next && (P.learned == 2 || project)) {
            if (project) {
                // basis: differences of the ring (newest first), then the network's correction
                RingPtrs R{};
                const double* V[kProjMax];
                for (int k = 0; k < ring_n; ++k) {
                    R.s[k] = ring_state(k);
                    R.d[k] = diffs + (size_t)k * 2 * m;
                    V[k] = R.d[k];
                }
                k_ch_diffs<<<grid_for(c, 2 * m), kBlock, 0, c->stream>>>(2 * m, ring_n, R);
                ++c->launches;
                int nv = ring_n;
                if (mlp_ready) {
                    TF_TRY(mlp_forward_dev(c, c->ch_X.p, m, c->ch_pred.p));
                    k_ch_corr<<<grid_for(c, 2 * m), kBlock, 0, c->stream>>>(m, c->ch_pred.p, c->ch_scales.p, corr);
                    ++c->launches;
                    V[nv++] = corr;
                }
                TF_CUDA(c, cudaGetLastError());
                TF_TRY(ch_project(c, B, c->vecs[TF_VEC_B].p, V, nv, guess));
            } else {
                k_ch_apply<<<grid_for(c, 2 * m), kBlock, 0, c->stream>>>(m, X, x_old, nullptr, c->ch_scales.p, guess);
                ++c->launches;
                TF_CUDA(c, cudaGetLastError());
            }
            double r_plain = 0., r_learn = 0.;
            TF_TRY(resid_norm(c, B, c->vecs[TF_VEC_B].p, X, &r_plain));
            TF_TRY(resid_norm(c, B, c->vecs[TF_VEC_B].p, guess, &r_learn));
            use = r_learn < r_plain;
        }
        fallback_next = false;
        TF_CUDA(c, cudaMemcpyAsync(x_prev, X, sizeof(double) * 2 * m, cudaMemcpyDeviceToDevice, c->stream));
        if (use) TF_CUDA(c, cudaMemcpyAsync(X, guess, sizeof(double) * 2 * m, cudaMemcpyDeviceToDevice, c->stream));
        int it = P.max_iter;
        double res = P.tol;
        const int st = gmres_jacobi(c, B, c->vecs[TF_VEC_B].p, X, P.restart, 0, P.precision, &it, &res, 1);
        if (iters) iters[step] = it;
        if (resids) resids[step] = res;
        if (used) used[step] = use ? 1 : 0;
        if (st != TF_OK) return st;
        if (use) {
            if (plain_ref >= 0 && 4 * it > 5 * plain_ref) fallback_next = true;
        } else {
            plain_ref = it;
        }
        if (project) {  // the new state enters the ring
            ring_head = (ring_head + 1) % kProjStates;
            ring_n = std::min(ring_n + 1, kProjStates);
            TF_CUDA(c, cudaMemcpyAsync(ring_state(0), X, sizeof(double) * 2 * m, cudaMemcpyDeviceToDevice, c->stream));
        }
        // online training on this step's increment
        if (have_hist && P.learned == 1 && step < P.train_steps) {
            TF_TRY(ch_features_dev(c, x_prev, x_old, X));
            double loss = 0.;
            for (int e = 0; e < P.epochs; ++e)
                TF_TRY(mlp_epoch_dev(c, c->ch_X.p, c->ch_Y.p, m, P.mb_tiles, P.lr, nullptr, e + 1 == P.epochs ? &loss : nullptr));
            c->ch_train_loss = loss;
            ++trained;
        }
        TF_CUDA(c, cudaMemcpyAsync(x_old, x_prev, sizeof(double) * 2 * m, cudaMemcpyDeviceToDevice, c->stream));
    }
    TF_CUDA(c, cudaMemcpyAsync(c->vecs[TF_VEC_CHI].p, c->vecs[TF_VEC_X].p, sizeof(double) * m, cudaMemcpyDeviceToDevice,
                               c->stream));
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    return TF_OK;
}

}  // namespace tf
