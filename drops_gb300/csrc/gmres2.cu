// Restarted GMRES with classical Gram-Schmidt and one reorthogonalisation
// (CGS2), right preconditioning, as one persistent cooperative kernel; the
// Arnoldi cycles run in V = float (mixed precision: every restart is one step
// of FP64 iterative refinement, the true residual b - A x and the update of x
// being FP64) or in V = double.
//
// Compared with the modified Gram-Schmidt solver of num/krylovsolver.h:320-463
// (k_gmres, one grid barrier per projection, about restart/2 barriers per
// Arnoldi step), CGS2 projects against all basis vectors at once: an Arnoldi
// step costs three grid barriers, (1) w = B v_i fused with the first
// projection dots, (2) first update fused with the second dots and |w1|^2
// (|w2|^2 = |w1|^2 - |h'|^2 on the orthonormal basis), (3) second update and a
// plain grid barrier.  The preconditioned operator B = A P^{-1} (P point
// or nodal 2x2 block Jacobi) is formed once per matrix in SELL order, so the
// Arnoldi loop is a plain SpMV; x += P^{-1} V y at the end of a cycle.  The
// Hessenberg matrix, Givens rotations and the small triangular solve are
// computed by thread 0 of the block that completes a grid step, in V, and
// published through global memory.
#include <cmath>

#include "krylov_dev.cuh"

namespace tf {

constexpr int kGm2MaxR = 64;
constexpr int kGm2Stride = kGm2MaxR + 2;  // partials per block
constexpr int kGm2Warps = kKryThreads / 32;
constexpr int kGm2Chunks = 10;                   // 32-block chunks the master reads per value
constexpr int kGm2MaxBlocks = 32 * kGm2Chunks;   // blocks of the launch (two per SM on 152 SMs: 304)
constexpr int kGm2Group = 4;                     // values a master warp reads at once

struct Gm2Scal {
    double normb, resid, beta;
    long long it, done, converged, cycle_end, cycles, i, pad;
};

template <class V>
struct Gm2Args {
    int64_t m, nslices;
    const int32_t* perm;
    const int32_t* ptr;
    const int32_t* col;
    const V* bval;        // SELL values of B = A P^{-1}
    const double* aval;   // SELL values of A (FP64), true residual
    const double* b;
    double* x;
    const double* diag;   // point Jacobi (nullptr with binv)
    const double* binv;   // nodal 2x2 inverses [m/2][4]
    V* basis;             // (R+1) x m, unnormalised; v_k = scl[k] * basis_k
    double* part;         // [nblocks][kGm2Stride]
    Gm2Scal* sc;
    V* small;             // H (R+1) x R column-major, cs[R], sn[R], s[R+1], y[R], scl[R+1], coef[R+1]
    GridSync gs;
    unsigned* mcount;  // grid-step arrivals (monotone)
    int R, max_iter, rel;
    double tol, inner_floor;
    int* out_iter;
    double* out_resid;
    int* out_cycles;
};

// Grid step with a fixed master block.  Every block has written n partial
// sums (type S) for this step; block 0 waits until all others have arrived,
// sums the partials in a fixed order, and its thread 0 runs f(sums, state) on
// block 0's shared-memory copy of the state (the Hessenberg matrix and the
// Givens rotations live in block 0's shared memory too, so the serial scalar
// work never waits on global-memory latency), publishes the state, and
// releases the others, which copy it.  The Arnoldi dots of the FP32 cycles
// reduce in FP32 all the way (S = float): FP64 instructions tie up the FP64
// pipe whatever the number of active lanes, and the basis itself is FP32.
// Grid-step synchronisation words: arrivals of the non-master blocks on a
// monotone counter (one release reduction each), the master's release of the
// step on the generation word (also bumped by grid_barrier, so monotone too).
// Every block keeps the generation and the step count it expects, so no word
// is read before arriving.
struct Gm2Sync {
    unsigned gen = 0;    // generation word value after the last grid step or barrier
    unsigned steps = 0;  // grid steps so far
};
__device__ __forceinline__ void gm2_red_release_add(unsigned* p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned gm2_ld_relaxed(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

template <class S, class F>
__device__ bool gm2_step(const GridSync& g, unsigned* mcount, Gm2Sync& sy, const S* part, int n, Gm2Scal* gsc,
                         Gm2Scal& ssc, F f) {
    __shared__ int st;
    __shared__ S sums[kGm2Stride];
    const unsigned target_gen = sy.gen + 1;
    __syncthreads();
    if (blockIdx.x != 0) {
        if (threadIdx.x == 0) {
            gm2_red_release_add(mcount, 1u);  // releases the block's partials (ordered by the barrier above)
            long long spins = 0;
            while ((int)(gm2_ld_relaxed(g.gen) - target_gen) < 0) {
                if (++spins > kSpinLimit) {
                    atomicCAS(g.status, 0, TF_ERR_WATCHDOG);
                    break;
                }
                if (spins > 256) __nanosleep(32);
            }
            __threadfence();
            // the published state and the status in one round of loads
            const unsigned long long* src = reinterpret_cast<const unsigned long long*>(gsc);
            unsigned long long* dst = reinterpret_cast<unsigned long long*>(&ssc);
            const int stv = __ldcg(g.status);
#pragma unroll
            for (int k = 0; k < (int)(sizeof(Gm2Scal) / 8); ++k) dst[k] = __ldcg(src + k);
            st = stv;
        }
        __syncthreads();
        sy.gen = target_gen;
        ++sy.steps;
        return st == 0;
    }
    if (threadIdx.x == 0) {
        const unsigned target = (sy.steps + 1) * (gridDim.x - 1);
        long long spins = 0;
        while ((int)(gm2_ld_relaxed(mcount) - target) < 0) {
            if (++spins > kSpinLimit) {
                atomicCAS(g.status, 0, TF_ERR_WATCHDOG);
                break;
            }
            if (spins > 256) __nanosleep(32);
        }
        __threadfence();
        st = __ldcg(g.status);
    }
    __syncthreads();
    if (st != 0) return false;
    // The partials are value-major (part[k][block]).  Warp w sums the values
    // k = w, w + 8, ..., kGm2Group of them at a time: its lanes load the
    // blocks lane, lane + 32, ... of each, all kGm2Group x kGm2Chunks loads
    // independent and coalesced (one round trip), then add them in chunk
    // order and close with a fixed warp tree, so the sum does not depend on
    // timing.  (Block-major partials read block after block took about ten
    // dependent round trips per grid step.)
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const int nb = (int)gridDim.x;
        for (int k0 = warp; k0 < n; k0 += kGm2Warps * kGm2Group) {
            S v[kGm2Group][kGm2Chunks];
#pragma unroll
            for (int g = 0; g < kGm2Group; ++g) {
                const int k = k0 + g * kGm2Warps;
#pragma unroll
                for (int j = 0; j < kGm2Chunks; ++j) {
                    const int b = lane + 32 * j;
                    v[g][j] = k < n && b < nb ? __ldcg(part + (size_t)k * nb + b) : S(0);
                }
            }
#pragma unroll
            for (int g = 0; g < kGm2Group; ++g) {
                S acc = S(0);
#pragma unroll
                for (int j = 0; j < kGm2Chunks; ++j) acc += v[g][j];
                acc = warp_sum(acc);
                const int k = k0 + g * kGm2Warps;
                if (lane == 0 && k < n) sums[k] = acc;
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        f(sums, ssc);
        const unsigned long long* src = reinterpret_cast<const unsigned long long*>(&ssc);
        unsigned long long* dst = reinterpret_cast<unsigned long long*>(gsc);
        for (int k = 0; k < (int)(sizeof(Gm2Scal) / 8); ++k) dst[k] = src[k];
        gm2_red_release_add(g.gen, 1u);  // releases the state and what f published
    }
    __syncthreads();
    sy.gen = target_gen;
    ++sy.steps;
    return true;
}

// warp partials (wred[k][warp]) -> block partials part[k][block] (value-major)
template <class S>
__device__ __forceinline__ void gm2_block_partials(S (*wred)[kGm2Warps], int n, S* part) {
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        S x = S(0);
        for (int w = 0; w < kGm2Warps; ++w) x += wred[k][w];
        part[(size_t)k * gridDim.x + blockIdx.x] = x;
    }
}

template <class V>
__global__ void __launch_bounds__(kKryThreads, 2) k_gmres2(Gm2Args<V> a) {
    __shared__ Gm2Scal sc;
    __shared__ V wred[kGm2Stride][kGm2Warps];   // Arnoldi dots, in V
    // least-squares state, used by block 0 (the master of every grid step)
    __shared__ V H[(kGm2MaxR + 1) * kGm2MaxR];  // H[k][i] at H[i * (R + 1) + k]
    __shared__ V cs[kGm2MaxR], sn[kGm2MaxR], s[kGm2MaxR + 1], ys[kGm2MaxR];
    __shared__ double wres[2][kGm2Warps];       // FP64 true residual
    double* const part64 = a.part;
    V* const partV = reinterpret_cast<V*>(a.part);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t m = a.m;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
    const int R = a.R;
    // published by the master for every block: solution of the least-squares
    // problem, basis scales, projection coefficients
    V* const y = a.small;
    V* const scl = y + R;
    V* const coef = scl + R + 1;
    const double tol = a.tol, inner_floor = a.inner_floor;
    const int max_iter = a.max_iter, rel = a.rel;
    bool first = true;
    Gm2Sync sy;

    for (;;) {
        // ---- cycle start: r = b - A x (FP64) into basis_0; |r|^2, |b|^2 ----
        {
            double v[2] = {0., 0.};
            const double* x = a.x;
            TF_SLICE_LOOP_BAL(a.nslices, sl) {
                const double ax = sell_row<double>(a.ptr, a.col, a.aval, sl, lane, [&](int32_t j) { return kld(x + j); });
                const int32_t row = __ldg(a.perm + sl * 32 + lane);
                if (row >= 0) {
                    const double bi = a.b[row];
                    const double r = bi - ax;
                    a.basis[row] = (V)r;
                    v[0] += r * r;
                    v[1] += bi * bi;
                }
            }
            for (int k = 0; k < 2; ++k) {
                const double t = warp_sum(v[k]);
                if (lane == 0) wres[k][warp] = t;
            }
            gm2_block_partials<double>(wres, 2, part64);
            const bool init = first;
            if (!gm2_step<double>(a.gs, a.mcount, sy, part64, 2, a.sc, sc, [&](const double* t, Gm2Scal& g) {
                    if (init) {
                        double nb = sqrt(t[1]);
                        if (nb == 0.0 || !rel) nb = 1.0;
                        g.normb = nb;
                        g.it = 0;
                        g.cycles = 0;
                    }
                    g.beta = sqrt(t[0]);
                    g.resid = g.beta / g.normb;
                    g.converged = g.resid <= tol;
                    g.done = g.converged || g.it >= max_iter;
                    g.cycle_end = 0;
                    g.i = 0;
                    if (!g.done) {
                        ++g.cycles;
                        scl[0] = (V)(1.0 / g.beta);
                        s[0] = (V)g.beta;
                        for (int k = 1; k <= R; ++k) s[k] = V(0);
                    }
                }))
                return;
            first = false;
            if (sc.done) break;
        }
        // ---- Arnoldi steps ----
        while (!sc.cycle_end) {
            const int i = (int)sc.i;
            V* const Vi = a.basis + (size_t)i * m;
            V* const W = a.basis + (size_t)(i + 1) * m;
            const V sci = scl[i];
            // (1) w = B v_i and the first projection dots <v_k, w>, k <= i
            for (int k = threadIdx.x; k <= i; k += blockDim.x)
                for (int w = 0; w < kGm2Warps; ++w) wred[k][w] = V(0);
            __syncthreads();
            TF_SLICE_LOOP_BAL(a.nslices, sl) {
                const V acc = sell_row<V>(a.ptr, a.col, a.bval, sl, lane, [&](int32_t j) { return sci * kld(Vi + j); });
                const int32_t row = __ldg(a.perm + sl * 32 + lane);
                if (row >= 0) W[row] = acc;
                // eight dots per transposing warp butterfly (9 shuffles instead of 40)
                for (int k0 = 0; k0 <= i; k0 += 8) {
                    V t8[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const int k = k0 + q;
                        t8[q] = row >= 0 && k <= i ? scl[k] * kld(a.basis + (size_t)k * m + row) * acc : V(0);
                    }
                    const V tot = warp_sum8(t8, lane);
                    const int k = k0 + warp_sum8_index(lane);
                    if ((lane & 3) == 0 && k <= i) wred[k][warp] += tot;
                }
            }
            gm2_block_partials<V>(wred, i + 1, partV);
            if (!gm2_step<V>(a.gs, a.mcount, sy, partV, i + 1, a.sc, sc, [&](const V* t, Gm2Scal& g) {
                    for (int k = 0; k <= i; ++k) {
                        coef[k] = (V)t[k];
                        H[(size_t)i * (R + 1) + k] = (V)t[k];
                    }
                }))
                return;
            // (2) w1 = w - sum_k h_k v_k with the second dots h'_k = <v_k, w1> and |w1|^2 (one grid
            // step: the master forms |w2|^2 = |w1|^2 - sum_k h'_k^2, the basis being orthonormal, and
            // with it the rotation and the stopping test); (3) w2 = w1 - sum_k h'_k v_k, then a grid
            // barrier, as the next product gathers w2 across blocks
            for (int pass = 0; pass < 2; ++pass) {
                for (int k = threadIdx.x; k <= i + 1; k += blockDim.x)
                    for (int w = 0; w < kGm2Warps; ++w) wred[k][w] = V(0);
                __syncthreads();
                // warp-uniform trip count (the warp's first row decides), so every
                // lane reaches the warp reductions; rows past m are masked
                for (int64_t e0 = tid; e0 - lane < m; e0 += 4 * nth) {
                    V wv[4];
                    bool in[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int64_t e = e0 + q * nth;
                        in[q] = e < m;
                        V w = in[q] ? kld(W + e) : V(0);
                        if (in[q])
                            for (int k = 0; k <= i; ++k) w -= coef[k] * (scl[k] * kld(a.basis + (size_t)k * m + e));
                        wv[q] = w;
                        if (in[q]) W[e] = w;
                    }
                    if (pass == 0) {
                        // values 0..i: <v_k, w1>; value i + 1: |w1|^2
                        for (int k0 = 0; k0 <= i + 1; k0 += 8) {
                            V t8[8];
#pragma unroll
                            for (int g = 0; g < 8; ++g) {
                                const int k = k0 + g;
                                V t = V(0);
                                if (k <= i) {
                                    const V* Vk = a.basis + (size_t)k * m;
#pragma unroll
                                    for (int q = 0; q < 4; ++q)
                                        if (in[q]) t += scl[k] * kld(Vk + e0 + q * nth) * wv[q];
                                } else if (k == i + 1) {
#pragma unroll
                                    for (int q = 0; q < 4; ++q) t += wv[q] * wv[q];
                                }
                                t8[g] = t;
                            }
                            const V tot = warp_sum8(t8, lane);
                            const int k = k0 + warp_sum8_index(lane);
                            if ((lane & 3) == 0 && k <= i + 1) wred[k][warp] += tot;
                        }
                    }
                }
                if (pass == 1) {
                    if (!grid_barrier(a.gs)) return;
                    ++sy.gen;  // the barrier's last arrival bumped the generation word
                    continue;
                }
                gm2_block_partials<V>(wred, i + 2, partV);
                if (!gm2_step<V>(a.gs, a.mcount, sy, partV, i + 2, a.sc, sc, [&](const V* t, Gm2Scal& g) {
                        V* hc = H + (size_t)i * (R + 1);
                        V h2sq = V(0);
                        for (int k = 0; k <= i; ++k) {
                            coef[k] = (V)t[k];
                            hc[k] += (V)t[k];
                            h2sq += (V)t[k] * (V)t[k];
                        }
                        const V n2 = (V)t[i + 1] - h2sq;
                        const V hn = n2 > V(0) ? (V)sqrt(n2) : V(0);
                        hc[i + 1] = hn;
                        scl[i + 1] = hn != V(0) ? V(1) / hn : V(0);
                        // previous rotations on column i, then the new one
                        for (int k = 0; k < i; ++k) {
                            const V t0 = cs[k] * hc[k] + sn[k] * hc[k + 1];
                            hc[k + 1] = -sn[k] * hc[k] + cs[k] * hc[k + 1];
                            hc[k] = t0;
                        }
                        const V dx = hc[i], dy = hc[i + 1];
                        if (dy == V(0)) {
                            cs[i] = V(1);
                            sn[i] = V(0);
                        } else {
                            const V r = sqrt(dx * dx + dy * dy);
                            cs[i] = dx / r;
                            sn[i] = dy / r;
                        }
                        hc[i] = cs[i] * dx + sn[i] * dy;
                        hc[i + 1] = V(0);
                        const V si = s[i];
                        s[i] = cs[i] * si;
                        s[i + 1] = -sn[i] * si;
                        g.it += 1;
                        const double est = fabs((double)s[i + 1]);
                        const bool stop = est <= fmax(inner_floor * g.beta, 0.5 * tol * g.normb) || i + 1 == R ||
                                          g.it >= max_iter || hn == V(0);
                        if (stop) {
                            // y = H^{-1} s on the leading (i+1) x (i+1) triangle
                            for (int q = i; q >= 0; --q) {
                                V acc = s[q];
                                for (int p2 = q + 1; p2 <= i; ++p2) acc -= H[(size_t)p2 * (R + 1) + q] * ys[p2];
                                ys[q] = acc / H[(size_t)q * (R + 1) + q];
                            }
                            for (int q = 0; q <= i; ++q) y[q] = ys[q];
                            g.cycle_end = 1;
                        }
                        g.i = i + 1;
                    }))
                    return;
            }
        }
        // ---- x += P^{-1} sum_k y_k v_k (FP64 update) ----
        {
            const int kk = (int)sc.i - 1;
            if (a.binv) {
                const int64_t half = m / 2;
                for (int64_t e = tid; e < half; e += nth) {
                    V za = V(0), zb = V(0);
                    for (int q = 0; q <= kk; ++q) {
                        const V c = y[q] * scl[q];
                        za += c * kld(a.basis + (size_t)q * m + e);
                        zb += c * kld(a.basis + (size_t)q * m + e + half);
                    }
                    const double* q4 = a.binv + 4 * e;
                    a.x[e] += q4[0] * (double)za + q4[1] * (double)zb;
                    a.x[e + half] += q4[2] * (double)za + q4[3] * (double)zb;
                }
            } else {
                for (int64_t e = tid; e < m; e += nth) {
                    V z = V(0);
                    for (int q = 0; q <= kk; ++q) z += (y[q] * scl[q]) * kld(a.basis + (size_t)q * m + e);
                    a.x[e] += (double)z / a.diag[e];
                }
            }
            if (!grid_barrier(a.gs)) return;
            ++sy.gen;  // the barrier's last arrival bumped the generation word
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *a.out_iter = sc.converged ? (int)sc.it : -1 - (int)sc.it;
        *a.out_resid = sc.resid;
        *a.out_cycles = (int)sc.cycles;
    }
}

// B = A P^{-1} in SELL order (warp per slice).  Block Jacobi: rows of the
// 2x2 block matrix hold the columns of both halves in the same order, so the
// partner of CSR entry k of row r (column j +- m/2) is entry k +- n_r/2.
template <class V>
__global__ void k_gm2_bvals(int64_t nslices, int64_t half, const int32_t* __restrict__ perm,
                            const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                            const int32_t* __restrict__ src, const int32_t* __restrict__ rowptr,
                            const double* __restrict__ aval, const double* __restrict__ diag,
                            const double* __restrict__ binv, V* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    TF_SLICE_LOOP(nslices, sl) {
        const int32_t p0 = ptr[sl], w = (ptr[sl + 1] - p0) >> 5;
        const int32_t row = perm[sl * 32 + lane];
        for (int32_t k = 0; k < w; ++k) {
            const int64_t q = p0 + 32 * k + lane;
            const int32_t c = src[q];
            double v = 0.;
            if (c >= 0 && row >= 0) {
                const int32_t j = col[q];
                if (!binv) {
                    v = aval[c] / diag[j];
                } else {
                    const int32_t r0 = rowptr[row], nr = rowptr[row + 1] - r0;
                    const int32_t pc = (c - r0 < nr / 2) ? c + nr / 2 : c - nr / 2;
                    const int64_t node = j < half ? j : j - half;
                    const double* q4 = binv + 4 * node;
                    // (A P^{-1})[r][e] = A[r][e] q0 + A[r][e+h] q2 ; [r][e+h] = A[r][e] q1 + A[r][e+h] q3
                    const double ae = j < half ? aval[c] : aval[pc];
                    const double ah = j < half ? aval[pc] : aval[c];
                    v = j < half ? ae * q4[0] + ah * q4[2] : ae * q4[1] + ah * q4[3];
                }
            }
            out[q] = (V)v;
        }
    }
}

__global__ void k_gm2_block_inv(int64_t half, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                                const double* __restrict__ vals, double* __restrict__ inv) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < half; i += (int64_t)gridDim.x * blockDim.x) {
        double a11 = 0, a12 = 0, a21 = 0, a22 = 0;
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            if (colind[k] == i) a11 = vals[k];
            if (colind[k] == i + half) a12 = vals[k];
        }
        for (int32_t k = rowptr[i + half]; k < rowptr[i + half + 1]; ++k) {
            if (colind[k] == i) a21 = vals[k];
            if (colind[k] == i + half) a22 = vals[k];
        }
        const double det = a11 * a22 - a12 * a21;
        inv[4 * i] = a22 / det;
        inv[4 * i + 1] = -a12 / det;
        inv[4 * i + 2] = -a21 / det;
        inv[4 * i + 3] = a11 / det;
    }
}

template <class V>
static int run_gmres2(Context* c, CSR& A, const double* b, double* x, int R, int* max_iter, double* tol, int rel) {
    const int64_t m = A.m;
    const bool block = &A == &c->mats[TF_MAT_BLOCK];
    DBuf<V>& bv = *reinterpret_cast<DBuf<V>*>(sizeof(V) == 4 ? (void*)&c->gm2_b32 : (void*)&c->gm2_b64);
    // preconditioner and B = A P^{-1}, once per matrix version
    if (block) TF_TRY(ensure(c, c->gm2_binv, (size_t)(2 * m)));
    if (c->gm2_src_version[sizeof(V) == 4] != A.version || c->gm2_src_gen[sizeof(V) == 4] != A.pattern_gen) {
        if (block) {
            k_gm2_block_inv<<<grid_for(c, m / 2), kBlock, 0, c->stream>>>(m / 2, A.rowptr, A.colind, A.vals, c->gm2_binv.p);
            ++c->launches;
        }
        TF_TRY(ensure(c, bv, (size_t)A.sell.npad));
        k_gm2_bvals<V><<<grid_for(c, A.sell.nslices * 32), kBlock, 0, c->stream>>>(
            A.sell.nslices, m / 2, A.sell.perm, A.sell.ptr, A.sell.col, A.sell.src, A.rowptr, A.vals,
            block ? nullptr : A.diag, block ? c->gm2_binv.p : nullptr, bv.p);
        ++c->launches;
        TF_CUDA(c, cudaGetLastError());
        c->gm2_src_version[sizeof(V) == 4] = A.version;
        c->gm2_src_gen[sizeof(V) == 4] = A.pattern_gen;
    }
    const void* fn = (const void*)k_gmres2<V>;
    int blocks = 0;
    TF_TRY(coop_blocks(c, fn, A.sell.nslices, &blocks, kKryThreads));
    blocks = std::min(blocks, kGm2MaxBlocks);  // the master's partial reads cover kGm2MaxBlocks blocks
    // H (R+1) x R, cs R, sn R, s R+1, y R, scl R+1, coef R+1
    const size_t small = (size_t)(R + 1) * R + 6 * (size_t)R + 3;
    DBuf<V>& basis = *reinterpret_cast<DBuf<V>*>(sizeof(V) == 4 ? (void*)&c->gm2_v32 : (void*)&c->gm2_v64);
    TF_TRY(ensure(c, basis, (size_t)(R + 1) * m + small));
    TF_TRY(ensure(c, c->kry_part, (size_t)blocks * kGm2Stride + 16 + sizeof(Gm2Scal) / 8));
    TF_TRY(ensure(c, c->kry_bar, 4));
    TF_TRY(ensure(c, c->kry_iters, 2));
    TF_TRY(ensure(c, c->kry_resid, 1));
    TF_CUDA(c, cudaMemsetAsync(c->kry_bar.p, 0, 4 * sizeof(unsigned), c->stream));
    TF_CUDA(c, cudaMemsetAsync(c->status.p, 0, 4 * sizeof(int), c->stream));
    Gm2Args<V> g{};
    g.m = m;
    g.nslices = A.sell.nslices;
    g.perm = A.sell.perm;
    g.ptr = A.sell.ptr;
    g.col = A.sell.col;
    g.bval = bv.p;
    g.aval = A.sell.v64;
    g.b = b;
    g.x = x;
    g.diag = block ? nullptr : A.diag;
    g.binv = block ? c->gm2_binv.p : nullptr;
    g.basis = basis.p;
    g.small = basis.p + (size_t)(R + 1) * m;
    g.part = c->kry_part.p;
    g.sc = reinterpret_cast<Gm2Scal*>(c->kry_part.p + (size_t)blocks * kGm2Stride + 16);
    g.gs = GridSync{c->kry_bar.p, c->kry_bar.p + 1, c->status.p};
    g.mcount = c->kry_bar.p + 2;
    g.R = R;
    g.max_iter = *max_iter;
    g.rel = rel;
    g.tol = *tol;
    g.inner_floor = sizeof(V) == 4 ? 1e-5 : 0.0;
    g.out_iter = c->kry_iters.p;
    g.out_resid = c->kry_resid.p;
    g.out_cycles = c->kry_iters.p + 1;
    void* args[] = {&g};
    TF_CUDA(c, cudaLaunchCooperativeKernel(fn, blocks, kKryThreads, args, 0, c->stream));
    ++c->launches;
    int it[2] = {0, 0};
    double res = 0.;
    TF_CUDA(c, cudaMemcpyAsync(it, c->kry_iters.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaMemcpyAsync(&res, c->kry_resid.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    int st = 0;
    TF_TRY(sync_status(c, &st));
    if (st) return set_err(c, st, "gmres (CGS2): grid barrier watchdog fired");
    c->last_refinements = it[1];
    *max_iter = it[0] >= 0 ? it[0] : -1 - it[0];
    *tol = res;
    return it[0] >= 0 ? TF_OK : set_err(c, TF_ERR_NOT_CONVERGED, "gmres (CGS2): no convergence within max_iter");
}

int gmres2(Context* c, CSR& A, const double* b, double* x, int restart, bool mixed, int* max_iter, double* tol, int rel) {
    if (!A.vals || A.m <= 0) return set_err(c, TF_ERR_BAD_INPUT, "gmres: empty matrix");
    if (restart < 2 || restart > kGm2MaxR) return set_err(c, TF_ERR_CAPACITY, "gmres (CGS2): restart in [2, 64]");
    TF_TRY(ensure_diag(c, A));
    TF_TRY(ensure_sell(c, A, false));
    TimedLaunch tl(c, TF_K_GMRES);
    return mixed ? run_gmres2<float>(c, A, b, x, restart, max_iter, tol, rel)
                 : run_gmres2<double>(c, A, b, x, restart, max_iter, tol, rel);
}

}  // namespace tf
