// Sparse linear algebra and Krylov solvers: SpMV, linear combinations, the
// Cahn-Hilliard block matrix, persistent Jacobi-PCG (FP64 and FP32), mixed-
// precision iterative refinement and restarted GMRES.
//
// GB300 note: FP64 arithmetic runs at a small fraction of the FP32 rate, so
// these kernels spend FP64 operations only where the result needs them (the
// FP64 SpMV of the FP64 solvers, their vector updates and reductions).  The
// FP32 inner solver of the mixed-precision path does all of its arithmetic in
// FP32; only per-warp partial sums are widened to FP64.
//
// The PCG of num/krylovsolver.h:107-189 runs as ONE cooperative kernel: every
// block owns a slice of rows, a grid barrier separates the two phases of an
// iteration (q = A p with <q,p>;  x,r,z updates with <r,r>,<z,r>), and the
// search-direction update p = z + beta p is fused into the next SpMV (double
// buffered).  Dot products are reduced over warps, blocks and then over all
// blocks in one fixed order, so every block computes bit-identical scalars and
// all blocks take the same convergence decision.  Every barrier wait is
// bounded: a block that waits too long raises TF_ERR_WATCHDOG and the kernel
// returns.
#include <cmath>

#include "krylov_dev.cuh"

namespace tf {

// ---------------------------------------------------------------------------
// SELL-32-sigma layout and SpMV (y_Ax, num/spmat.h:1684-1709)
// ---------------------------------------------------------------------------
constexpr int kSigma = 512;  // rows sorted by length inside windows of 512
static_assert(kSigma / 32 == kSellWinSlices, "slice order of the persistent kernels assumes 16 slices per window");

// one block of kSigma threads per window: bitonic sort of (descending length,
// row); window w holds rows order[w kSigma ..] (order == nullptr: the rows in
// numbering order)
__global__ void __launch_bounds__(kSigma) k_sell_sort(int64_t m, const int32_t* __restrict__ rowptr,
                                                      const int32_t* __restrict__ order, int32_t* __restrict__ perm) {
    __shared__ uint64_t key[kSigma];
    const int t = threadIdx.x;
    const int64_t idx = (int64_t)blockIdx.x * kSigma + t;
    const int64_t row = idx < m && order ? order[idx] : idx;
    if (idx < m) {
        const uint32_t len = (uint32_t)(rowptr[row + 1] - rowptr[row]);
        key[t] = ((uint64_t)(0x7fffffffu - len) << 32) | (uint64_t)(uint32_t)row;
    } else {
        key[t] = ~0ull;
    }
    __syncthreads();
    for (int size = 2; size <= kSigma; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            const int partner = t ^ stride;
            if (partner > t) {
                const bool up = (t & size) == 0;
                const uint64_t a = key[t], b = key[partner];
                if ((a > b) == up) {
                    key[t] = b;
                    key[partner] = a;
                }
            }
            __syncthreads();
        }
    perm[(int64_t)blockIdx.x * kSigma + t] = key[t] == ~0ull ? -1 : (int32_t)(key[t] & 0xffffffffu);
}

__global__ void k_sell_width(int64_t nslices, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ perm,
                             int32_t* __restrict__ w) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t s = warp; s < nslices; s += nwarp) {
        const int32_t row = perm[s * 32 + lane];
        int len = row >= 0 ? rowptr[row + 1] - rowptr[row] : 0;
        len = __reduce_max_sync(0xffffffffu, len);
        if (lane == 0) w[s] = 32 * len;
    }
}

__global__ void k_sell_fill(int64_t nslices, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
                            const int32_t* __restrict__ perm, const int32_t* __restrict__ ptr,
                            int32_t* __restrict__ col, int32_t* __restrict__ src) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t s = warp; s < nslices; s += nwarp) {
        const int32_t row = perm[s * 32 + lane];
        const int32_t p0 = ptr[s], w = (ptr[s + 1] - p0) >> 5;
        int32_t rs = 0, len = 0;
        if (row >= 0) {
            rs = rowptr[row];
            len = rowptr[row + 1] - rs;
        }
        const int32_t pad_col = row >= 0 ? row : 0;
        for (int32_t k = 0; k < w; ++k) {
            const int32_t pos = p0 + k * 32 + lane;
            if (k < len) {
                col[pos] = colind[rs + k];
                src[pos] = rs + k;
            } else {
                col[pos] = pad_col;
                src[pos] = -1;
            }
        }
    }
}

template <class T>
__global__ void k_sell_vals(int64_t npad, const int32_t* __restrict__ src, const double* __restrict__ vals,
                            T* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npad; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t k = src[i];
        out[i] = k >= 0 ? (T)vals[k] : (T)0;
    }
}

static int mat_index(Context* c, const CSR& A) {
    for (int i = 0; i < TF_NUM_MATS; ++i)
        if (&c->mats[i] == &A) return i;
    return 0;
}

int ensure_sell(Context* c, CSR& A, bool fp32) {
    const int id = mat_index(c, A);
    Sell& S = A.sell;
    if (S.pattern_gen != A.pattern_gen || !S.ptr) {
        const int64_t nwin = (A.m + kSigma - 1) / kSigma;
        const int64_t ns = nwin * (kSigma / 32);
        TF_TRY(ensure(c, c->sell_perm[id], (size_t)(ns * 32)));
        TF_TRY(ensure(c, c->sell_ptr[id], (size_t)ns + 1));
        TF_TRY(ensure(c, c->scratch, sizeof(int32_t) * (size_t)(ns + 1)));
        int32_t* w = (int32_t*)c->scratch.p;
        // a matrix on the current DistributeDOFs pattern takes its windows in the locality order of the DOFs
        const int32_t* order = nullptr;
        if (c->locality_order && A.rowptr == c->rowptr.p && A.m == c->n_dofs &&
            c->pattern_dof_version == c->dof_version)
            TF_TRY(dof_locality_order(c, &order));
        k_sell_sort<<<(unsigned)nwin, kSigma, 0, c->stream>>>(A.m, A.rowptr, order, c->sell_perm[id].p);
        k_sell_width<<<grid_for(c, ns * 32), kBlock, 0, c->stream>>>(ns, A.rowptr, c->sell_perm[id].p, w);
        c->launches += 2;
        int64_t npad = 0;
        TF_TRY(exclusive_scan_i32_to_i32(c, w, c->sell_ptr[id].p, ns, &npad));
        TF_TRY(ensure(c, c->sell_col[id], (size_t)(npad > 0 ? npad : 1)));
        TF_TRY(ensure(c, c->sell_src[id], (size_t)(npad > 0 ? npad : 1)));
        k_sell_fill<<<grid_for(c, ns * 32), kBlock, 0, c->stream>>>(ns, A.rowptr, A.colind, c->sell_perm[id].p,
                                                                     c->sell_ptr[id].p, c->sell_col[id].p,
                                                                     c->sell_src[id].p);
        ++c->launches;
        TF_CUDA(c, cudaGetLastError());
        S.nslices = ns;
        S.npad = npad;
        S.perm = c->sell_perm[id].p;
        S.ptr = c->sell_ptr[id].p;
        S.col = c->sell_col[id].p;
        S.src = c->sell_src[id].p;
        S.pattern_gen = A.pattern_gen;
        S.v64_version = S.v32_version = S.v2f_version = -1;
    }
    if (fp32) {
        if (S.v32_version != A.version || !S.v32) {
            TF_TRY(ensure(c, c->sell_v32[id], (size_t)(S.npad > 0 ? S.npad : 1)));
            S.v32 = c->sell_v32[id].p;
            k_sell_vals<float><<<grid_for(c, S.npad), kBlock, 0, c->stream>>>(S.npad, S.src, A.vals, S.v32);
            ++c->launches;
            S.v32_version = A.version;
        }
    } else if (S.v64_version != A.version || !S.v64) {
        TF_TRY(ensure(c, c->sell_v64[id], (size_t)(S.npad > 0 ? S.npad : 1)));
        S.v64 = c->sell_v64[id].p;
        k_sell_vals<double><<<grid_for(c, S.npad), kBlock, 0, c->stream>>>(S.npad, S.src, A.vals, S.v64);
        ++c->launches;
        S.v64_version = A.version;
    }
    TF_CUDA(c, cudaGetLastError());
    return TF_OK;
}


template <class T>
__global__ void k_spmv(int64_t nslices, const int32_t* __restrict__ perm, const int32_t* __restrict__ ptr,
                       const int32_t* __restrict__ col, const T* __restrict__ val, const T* __restrict__ x,
                       T* __restrict__ y) {
    const int lane = threadIdx.x & 31;
    TF_SLICE_LOOP(nslices, s) {
        const T a = sell_row<T>(ptr, col, val, s, lane, [&](int32_t j) { return __ldg(x + j); });
        const int32_t row = perm[s * 32 + lane];
        if (row >= 0) y[row] = a;
    }
}

// ---------------------------------------------------------------------------
// Balanced SELL SpMV (the standalone y_Ax).  Block b of B (a multiple of the
// SM count) takes a contiguous run of n/B slices and its warps split the
// run's column work evenly (sell_block_balanced, in chunks of at most
// kBalMaxSlices slices): about 3 gather rounds per warp for the P2 matrices
// instead of the 8 of a 62-wide slice walked by one warp.  FP64
// multiply-adds only on stored entries (one warp instruction per 32 products;
// GB300 issues FP64 at ~1/64 of the FP32 rate, so the FP64 pipe and HBM bound
// this kernel about equally).  Bytes: 12 per stored entry + perm, ptr, x
// gathered, y written.
// ---------------------------------------------------------------------------
template <int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) k_spmv_bal(int64_t nslices, const int32_t* __restrict__ perm,
                                                 const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                                                 const double* __restrict__ val, const double* __restrict__ x,
                                                 double* __restrict__ y) {
    __shared__ BalShared<NT / 32, double> sh;
    const int lane = threadIdx.x & 31;
    // equal slice counts: a work-balanced split (balanced_part_start) costs
    // two binary searches of dependent loads, too much for one short launch
    const int64_t s0 = (int64_t)blockIdx.x * nslices / gridDim.x;
    const int64_t s1 = (int64_t)(blockIdx.x + 1) * nslices / gridDim.x;
    for (int64_t c0 = s0; c0 < s1; c0 += kBalMaxSlices)
        sell_block_balanced<NT / 32, double>(
            sh, ptr, col, val, c0, (int)(s1 - c0 < kBalMaxSlices ? s1 - c0 : kBalMaxSlices),
            [&](int32_t j) { return __ldg(x + j); },
            [&](int64_t s, double v) {
                const int32_t row = __ldg(perm + s * 32 + lane);
                if (row >= 0) y[row] = v;
            });
}

void launch_spmv_shape(Context* c, const CSR& A, const double* x, double* y, int threads, int per_sm) {
    const int64_t ns = A.sell.nslices;
    int64_t nb = (int64_t)c->num_sms * per_sm;
    if (nb > ns) nb = ns;
    if (nb < 1) nb = 1;
    if (threads == 256)
        k_spmv_bal<256><<<(unsigned)nb, 256, 0, c->stream>>>(ns, A.sell.perm, A.sell.ptr, A.sell.col, A.sell.v64, x, y);
    else
        k_spmv_bal<512><<<(unsigned)nb, 512, 0, c->stream>>>(ns, A.sell.perm, A.sell.ptr, A.sell.col, A.sell.v64, x, y);
    ++c->launches;
}

// ---------------------------------------------------------------------------
// FP64-accurate SpMV on FP32 pairs
//
// GB300 issues FP64 at 1/64 of the FP32 rate: one FP64 FMA per non-zero keeps
// the FP64 pipe about as busy as HBM.  Instead every row is scaled by a power
// of two 2^-e (its largest |a| lands in [0.5, 1)) and each scaled value is
// stored as an unevaluated FP32 pair hi + lo (8 bytes, like the FP64 value);
// x is split the same way (without scaling) once per call.  Products and the
// row sum are formed in pair arithmetic (exact product error by FMA, two-sum
// for the running sum): about 12 FP32 operations per non-zero and 4 FP64
// operations per row.  Each product carries ~2^-48 relative error, so
// |y - A x| <= ~2^-44 sum_j |a_ij x_j| + 2^-140 max|a_i.| max|x|, far inside
// the 1e-12 parity bound.  x entries outside {0} U [2^-100, 2^100] (or not
// finite) raise a flag that switches the same launch to FP64 FMAs.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 split_pair(double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - (double)h));
}

__device__ __forceinline__ double pow2(int e) {  // 2^e, |e| <= 1022
    return __longlong_as_double((long long)(e + 1023) << 52);
}

// warp per slice: row exponent, then the scaled pairs; *bad set on a
// non-finite value
__global__ void k_sell_vals_pair(int64_t nslices, const int32_t* __restrict__ ptr, const int32_t* __restrict__ src,
                                 const double* __restrict__ vals, float2* __restrict__ out, int32_t* __restrict__ rexp,
                                 int* bad) {
    const int lane = threadIdx.x & 31;
    TF_SLICE_LOOP(nslices, s) {
        const int32_t p0 = ptr[s], w = (ptr[s + 1] - p0) >> 5;
        double mx = 0.;
        for (int32_t k = 0; k < w; ++k) {
            const int32_t q = src[p0 + 32 * k + lane];
            if (q >= 0) {
                const double v = vals[q];
                if (!isfinite(v)) atomicOr(bad, 1);
                mx = fmax(mx, fabs(v));
            }
        }
        int e = 0;
        if (mx > 0. && isfinite(mx)) frexp(mx, &e);
        e = max(-1000, min(1000, e));
        rexp[s * 32 + lane] = e;
        const double sc = pow2(-e);
        for (int32_t k = 0; k < w; ++k) {
            const int32_t q = src[p0 + 32 * k + lane];
            out[p0 + 32 * k + lane] = split_pair(q >= 0 ? vals[q] * sc : 0.);
        }
    }
}

// (sh, sl) += a * x in pair arithmetic; a = (0, 0) leaves the sum unchanged
__device__ __forceinline__ void pair_fma(float& sh, float& sl, float2 a, float2 x) {
    const float p = __fmul_rn(a.x, x.x);
    const float pe = __fmaf_rn(a.x, x.x, -p);
    const float t = __fmaf_rn(a.x, x.y, __fmaf_rn(a.y, x.x, pe));
    const float s = __fadd_rn(sh, p);
    const float bb = __fsub_rn(s, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    sl = __fadd_rn(sl, __fadd_rn(err, t));
    sh = s;
}

// x -> pairs with integer operations only (no conversions, which GB300 runs
// on its narrow FP64 pipe): hi = the top 24 bits of the significand
// (truncated), lo = the remaining 29 bits normalised and truncated to 24, so
// |x - hi - lo| <= 2^-47 |x|.  Valid for |x| in [2^-74, 2^100], where lo is a
// normal float; other non-zero x (and non-finite x) set *flag, which sends the
// launch to FP64 FMAs.
__global__ void k_split_x_int(int64_t n, const double* __restrict__ x, float2* __restrict__ out, int* flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(x[i]);
        float2 r = make_float2(0.f, 0.f);
        if ((b << 1) != 0ull) {
            const unsigned e = (unsigned)(b >> 52) & 0x7ffu, sgn = (unsigned)(b >> 63) << 31;
            if (e < 949u || e > 1123u) {
                atomicOr(flag, 1);
            } else {
                const unsigned long long mant = b & 0xfffffffffffffull;
                const unsigned hb = sgn | ((e - 896u) << 23) | (unsigned)(mant >> 29);
                const unsigned rem = (unsigned)(mant & 0x1fffffffu);
                unsigned lb = 0u;
                if (rem) {
                    const int lz = __clz((int)rem);          // >= 3
                    const unsigned p = 31u - (unsigned)lz;   // leading bit of rem
                    const unsigned m23 = (unsigned)((((unsigned long long)rem << (lz + 1)) & 0xffffffffull) >> 9);
                    lb = sgn | ((p + e - 948u) << 23) | m23;  // rem * 2^(e - 1075)
                }
                r = make_float2(__int_as_float((int)hb), __int_as_float((int)lb));
            }
        }
        out[i] = r;
    }
}

// n columns of a slot row in pair arithmetic (loads staged like sell_row_walk)
struct Pair2 {
    float h, l;
    __device__ Pair2(float a = 0.f, float b = 0.f) : h(a), l(b) {}
};
__device__ __forceinline__ Pair2 operator+(Pair2 a, Pair2 b) {  // two-sum of the highs, lows added
    const float s = __fadd_rn(a.h, b.h);
    const float bb = __fsub_rn(s, a.h);
    const float err = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
    return Pair2(s, __fadd_rn(__fadd_rn(a.l, b.l), err));
}

__device__ __forceinline__ Pair2 pair_row_walk(const int32_t* __restrict__ cp, const float2* __restrict__ vp, int32_t n,
                                               const float2* __restrict__ x) {
    constexpr int U = 4;  // 8 spills at 64 registers
    float sh = 0.f, sl = 0.f;
    int32_t cn[U];
    float2 vn[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const bool in = u < n;
        cn[u] = in ? __ldg(cp + 32 * u) : -1;
        vn[u] = in ? __ldg(vp + 32 * u) : make_float2(0.f, 0.f);
    }
    for (int32_t k = 0; k < n; k += U) {
        float2 xv[U], vv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            xv[u] = cn[u] >= 0 ? __ldg(x + cn[u]) : make_float2(0.f, 0.f);
            vv[u] = vn[u];
        }
        const int32_t kn = k + U;
        if (kn < n) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const bool in = kn + u < n;
                cn[u] = in ? __ldg(cp + 32 * (kn + u)) : -1;
                vn[u] = in ? __ldg(vp + 32 * (kn + u)) : make_float2(0.f, 0.f);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (k + u < n) pair_fma(sh, sl, vv[u], xv[u]);
    }
    return Pair2(sh, sl);
}

// Balanced SpMV in pair arithmetic: the block split of k_spmv_bal, FP32
// operations per non-zero, 4 FP64 operations per row (the epilogue
// ((double)hi + (double)lo) 2^e).  *flag (x out of the pair range) switches
// the whole launch to FP64 FMAs.
template <int NT>
__global__ void __launch_bounds__(NT, 1024 / NT)
    k_spmv_pair_bal(int64_t nslices, const int32_t* __restrict__ perm, const int32_t* __restrict__ ptr,
                    const int32_t* __restrict__ col, const float2* __restrict__ v2, const int32_t* __restrict__ rexp,
                    const double* __restrict__ v64, const float2* __restrict__ x2, const double* __restrict__ x,
                    const int* __restrict__ flag, double* __restrict__ y) {
    constexpr int NW = NT / 32;
    constexpr size_t kRaw = sizeof(BalShared<NW, double>) > sizeof(BalShared<NW, Pair2>) ? sizeof(BalShared<NW, double>)
                                                                                           : sizeof(BalShared<NW, Pair2>);
    __shared__ __align__(16) unsigned char raw[kRaw];
    const int lane = threadIdx.x & 31;
    const bool native = *flag != 0;
    const int64_t s0 = (int64_t)blockIdx.x * nslices / gridDim.x;
    const int64_t s1 = (int64_t)(blockIdx.x + 1) * nslices / gridDim.x;
    for (int64_t c0 = s0; c0 < s1; c0 += kBalMaxSlices) {
        const int S = (int)(s1 - c0 < kBalMaxSlices ? s1 - c0 : kBalMaxSlices);
        if (native) {
            auto& sh = *reinterpret_cast<BalShared<NW, double>*>(raw);
            sell_block_balanced<NW, double>(
                sh, ptr, col, v64, c0, S, [&](int32_t j) { return __ldg(x + j); },
                [&](int64_t s, double v) {
                    const int32_t row = __ldg(perm + s * 32 + lane);
                    if (row >= 0) y[row] = v;
                });
        } else {
            auto& sh = *reinterpret_cast<BalShared<NW, Pair2>*>(raw);
            sell_block_plan<NW, Pair2>(sh, ptr, c0, S);
            sell_block_walk_fn<NW, Pair2>(
                sh, c0, S,
                [&](int64_t s, int32_t cc, int32_t n) {
                    const int32_t p0 = __ldg(ptr + s) + 32 * cc;
                    return pair_row_walk(col + p0 + lane, v2 + p0 + lane, n, x2);
                },
                [&](int64_t s, Pair2 q) {
                    const int32_t row = __ldg(perm + s * 32 + lane);
                    if (row >= 0) y[row] = ((double)q.h + (double)q.l) * pow2(__ldg(rexp + s * 32 + lane));
                });
        }
    }
}

static int ensure_sell_pair(Context* c, CSR& A) {
    Sell& S = A.sell;
    if (S.v2f_version == A.version && S.v2f) return TF_OK;
    const int id = mat_index(c, A);
    TF_TRY(ensure(c, c->sell_v2f[id], (size_t)(S.npad > 0 ? S.npad : 1)));
    TF_TRY(ensure(c, c->sell_rexp[id], (size_t)(S.nslices > 0 ? S.nslices * 32 : 1)));
    S.v2f = c->sell_v2f[id].p;
    S.rexp = c->sell_rexp[id].p;
    TF_CUDA(c, cudaMemsetAsync(c->status.p + 3, 0, sizeof(int), c->stream));
    k_sell_vals_pair<<<grid_for(c, S.nslices * 32), kBlock, 0, c->stream>>>(S.nslices, S.ptr, S.src, A.vals, S.v2f,
                                                                            S.rexp, c->status.p + 3);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    int bad = 0;
    TF_CUDA(c, cudaMemcpyAsync(&bad, c->status.p + 3, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    S.v2f_ok = bad == 0;
    S.v2f_version = A.version;
    return TF_OK;
}

int spmv(Context* c, const CSR& Ac, const double* x, double* y) {
    CSR& A = const_cast<CSR&>(Ac);
    TF_TRY(ensure_sell(c, A, false));
    if (c->spmv_sell) {  // one warp per slice (kept for comparisons)
        TimedLaunch tl(c, TF_K_SPMV);
        k_spmv<double><<<grid_for(c, A.sell.nslices * 32), kBlock, 0, c->stream>>>(
            A.sell.nslices, A.sell.perm, A.sell.ptr, A.sell.col, A.sell.v64, x, y);
        ++c->launches;
        TF_CUDA(c, cudaGetLastError());
        return TF_OK;
    }
    const bool pair = c->spmv_pair;
    if (pair) TF_TRY(ensure_sell_pair(c, A));
    int threads = c->spmv_threads == 256 ? 256 : 512, per_sm = c->spmv_blocks_per_sm > 0 ? c->spmv_blocks_per_sm : 2;
    if (!pair && c->autotune && !c->spmv_shape_fixed) TF_TRY(tuned_spmv_shape(c, A, &threads, &per_sm));
    TimedLaunch tl(c, TF_K_SPMV);
    if (!pair || !A.sell.v2f_ok) {
        launch_spmv_shape(c, A, x, y, threads, per_sm);
    } else {
        TF_TRY(ensure(c, c->x_pairs, (size_t)(A.m > 0 ? A.m : 1)));
        TF_CUDA(c, cudaMemsetAsync(c->status.p + 2, 0, sizeof(int), c->stream));
        k_split_x_int<<<grid_for(c, A.m), kBlock, 0, c->stream>>>(A.m, x, c->x_pairs.p, c->status.p + 2);
        const int64_t ns = A.sell.nslices;
        int64_t nb = (int64_t)c->num_sms * 2;
        if (nb > ns) nb = ns;
        if (nb < 1) nb = 1;
        k_spmv_pair_bal<512><<<(unsigned)nb, 512, 0, c->stream>>>(ns, A.sell.perm, A.sell.ptr, A.sell.col, A.sell.v2f,
                                                                 A.sell.rexp, A.sell.v64, c->x_pairs.p, x,
                                                                 c->status.p + 2, y);
        c->launches += 2;
    }
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

int ensure_vals32(Context* c, CSR& A) { return ensure_sell(c, A, true); }

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
        if (!is_form_handle(forms[t]) || !c->mats[forms[t]].vals)
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
    S.pattern_gen = F.pattern_gen;
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
// rows of [[alpha M (+ N), mob Amob + rho C], [eps2 A + beta M + eps2 rho C, -M]]
// (surfphasesep/surfphasesep.cpp:431-434): Amob is A_deg (LaplaceM) or A_one,
// the lower-left block always takes A_one; N (wind convection) may be null
__global__ void k_block_fill(int64_t m, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                             const double* __restrict__ M, const double* __restrict__ A, const double* __restrict__ C,
                             const double* __restrict__ Amob, const double* __restrict__ N, double alpha, double mob,
                             double rho, double eps2, double beta, const int32_t* __restrict__ brp,
                             int32_t* __restrict__ bci, double* __restrict__ bv) {
    for (int64_t R = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; R < 2 * m; R += (int64_t)gridDim.x * blockDim.x) {
        const int half = R >= m;
        const int64_t r = half ? R - m : R;
        int32_t w = brp[R];
        for (int blk = 0; blk < 2; ++blk)
            for (int32_t k = rp[r]; k < rp[r + 1]; ++k) {
                double v;
                if (!half) v = blk == 0 ? (N ? alpha * M[k] + N[k] : alpha * M[k]) : mob * Amob[k] + rho * C[k];
                else v = blk == 0 ? (eps2 * A[k] + beta * M[k]) + (eps2 * rho) * C[k] : -1. * M[k];
                bci[w] = ci[k] + (int32_t)(blk * m);
                bv[w] = v;
                ++w;
            }
    }
}

int ch_block(Context* c, double alpha, double mob, double rho, double eps2, double beta, int flags) {
    const CSR& M = c->mats[TF_FORM_M];
    const CSR& A = c->mats[TF_FORM_A];
    const CSR& Amob = c->mats[(flags & TF_CH_DEGENERATE_MOBILITY) ? TF_FORM_LAPM : TF_FORM_A];
    const CSR& C = c->mats[TF_FORM_CN];
    const CSR& N = c->mats[TF_FORM_N];
    if (!M.vals || !A.vals || !Amob.vals || !C.vals || ((flags & TF_CH_WIND) && !N.vals))
        return set_err(c, TF_ERR_BAD_INPUT, "ch_block: assemble M, A, C_n (and LaplaceM / N when asked) first");
    const int64_t m = M.m, nnz = M.nnz;
    if (4 * nnz >= INT32_MAX) return set_err(c, TF_ERR_CAPACITY, "ch_block: too many non-zeros");
    CSR& B = c->mats[TF_MAT_BLOCK];
    TF_TRY(ensure(c, c->block_rowptr, (size_t)(2 * m + 1)));
    TF_TRY(ensure(c, c->block_colind, (size_t)(4 * nnz > 0 ? 4 * nnz : 1)));
    TF_TRY(ensure(c, c->mat_vals[TF_MAT_BLOCK], (size_t)(4 * nnz > 0 ? 4 * nnz : 1)));
    if (c->block_src_gen != M.pattern_gen || B.m != 2 * m) {
        B.pattern_gen = ++c->pattern_counter;
        c->block_src_gen = M.pattern_gen;
    }
    B.m = 2 * m;
    B.nnz = 4 * nnz;
    B.rowptr = c->block_rowptr.p;
    B.colind = c->block_colind.p;
    B.vals = c->mat_vals[TF_MAT_BLOCK].p;
    k_block_rowptr<<<grid_for(c, 2 * m + 1), kBlock, 0, c->stream>>>(m, M.rowptr, B.rowptr);
    k_block_fill<<<grid_for(c, 2 * m), kBlock, 0, c->stream>>>(
        m, M.rowptr, M.colind, M.vals, A.vals, C.vals, Amob.vals, (flags & TF_CH_WIND) ? N.vals : nullptr, alpha, mob,
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
    int64_t m, nslices;
    const int32_t* perm;
    const int32_t* ptr;
    const int32_t* col;
    const T* val;
    const T* diag;
    const T* b;
    T* x;
    T* r;
    T* z;
    T* p0;
    T* p1;
    T* q;
    GridAR g;
    int max_iter;
    double tol;
    int rel;
    int* out_iter;
    double* out_resid;
};

// Standard PCG (PCGSolverCL<JACPcCL>::Solve's recurrences): two all-reduce
// barriers per iteration, <p, A p> and then <r, r>, <z, r>.  The scalar
// recurrences (square roots, divisions) run on thread 0 of every block on
// bitwise identical sums and are broadcast through shared memory.
template <class T>
__global__ void __launch_bounds__(kKryThreads, sizeof(T) == 4 ? 4 : 3) k_pcg(PcgArgs<T> a) {
    __shared__ double sh[6];
    const int lane = threadIdx.x & 31;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
    const double tol = a.tol;
    const int max_iter = a.max_iter, rel = a.rel;
    unsigned long long epoch = 0;
    double rho = 0., normb = 1., resid = 0.;
    int it = 0;
    bool converged = false, done = false;

    // r = b - A x ; z = r / d ; p0 = z ; sums <r,r>, <b,b>, <z,r>
    {
        double v[3] = {0., 0., 0.};
        const T* x = a.x;
        TF_SLICE_LOOP_BAL(a.nslices, s) {
            const T ax = sell_row<T>(a.ptr, a.col, a.val, s, lane, [&](int32_t j) { return kld(x + j); });
            const int32_t row = __ldg(a.perm + s * 32 + lane);
            if (row >= 0) {
                const T bi = a.b[row];
                const T ri = bi - ax;
                const T zi = ri / a.diag[row];
                a.r[row] = ri;
                a.z[row] = zi;
                a.p0[row] = zi;
                v[0] += ri * ri;
                v[1] += bi * bi;
                v[2] += zi * ri;
            }
        }
        double o[3];
        if (!grid_allreduce<double, 3>(a.g, epoch, v, o)) return;
        if (threadIdx.x == 0) {
            double nb = sqrt(o[1]);
            if (nb == 0.0 || !rel) nb = 1.0;
            sh[0] = nb;
            sh[1] = sqrt(o[0]) / nb;
        }
        __syncthreads();
        normb = sh[0];
        resid = sh[1];
        rho = o[2];
        converged = resid <= tol;
        done = converged || max_iter <= 0;
    }
    T* pc = a.p0;  // previous direction (beta = 0 in the first iteration)
    T* pn = a.p1;
    T beta = T(0);
    while (!done) {
        // phase A: p_new = z + beta p_old ; q = A p_new ; <q, p_new>
        {
            double v[1] = {0.};
            const T* z = a.z;
            const T* po = pc;
            T acc1 = T(0);
            TF_SLICE_LOOP_BAL(a.nslices, s) {
                const T acc = sell_row<T>(a.ptr, a.col, a.val, s, lane,
                                          [&](int32_t j) { return kld(z + j) + beta * kld(po + j); });
                const int32_t row = __ldg(a.perm + s * 32 + lane);
                if (row >= 0) {
                    const T pi = kld(z + row) + beta * kld(po + row);
                    pn[row] = pi;
                    a.q[row] = acc;
                    acc1 += acc * pi;
                }
            }
            v[0] = acc1;
            double o[1];
            if (!grid_allreduce<double, 1>(a.g, epoch, v, o)) return;
            if (threadIdx.x == 0) sh[2] = rho / o[0];
            __syncthreads();
        }
        const T alpha = (T)sh[2];
        // phase B: x += alpha p ; r -= alpha q ; z = r / d ; <r,r>, <z,r>
        {
            T v2[2] = {T(0), T(0)};
            for (int64_t i = tid; i < a.m; i += nth) {
                a.x[i] += alpha * kld(pn + i);
                const T ri = a.r[i] - alpha * kld(a.q + i);
                const T zi = ri / a.diag[i];
                a.r[i] = ri;
                a.z[i] = zi;
                v2[0] += ri * ri;
                v2[1] += zi * ri;
            }
            double v[2] = {(double)v2[0], (double)v2[1]};
            double o[2];
            if (!grid_allreduce<double, 2>(a.g, epoch, v, o)) return;
            if (threadIdx.x == 0) {
                sh[3] = sqrt(o[0]) / normb;
                sh[4] = o[1] / rho;
            }
            __syncthreads();
            ++it;
            resid = sh[3];
            converged = resid <= tol;
            done = converged || it >= max_iter;
            beta = (T)sh[4];
            rho = o[1];
        }
        T* tmp = pc;
        pc = pn;
        pn = tmp;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *a.out_iter = converged ? it : -1 - it;
        *a.out_resid = resid;
    }
}

// ---------------------------------------------------------------------------
// mixed-precision PCG: FP32 iterations with FP64 reliable updates
//
// The search directions, the recursive residual and every SpMV of the
// iteration are FP32 (A in FP32, 8 bytes per non-zero instead of 12, FP32
// arithmetic); the iterate x is accumulated in FP64.  Whenever the FP32
// residual has dropped by a factor kRelUpdate since the last refinement, or
// claims convergence, the true residual b - A x is recomputed in FP64 (FP64
// SpMV) and replaces the FP32 one: one step of FP64 iterative refinement that
// keeps the Krylov recurrence instead of restarting it, so the iteration count
// stays close to the FP64 solver's.  Convergence is decided on the FP64
// residual only.
// ---------------------------------------------------------------------------
constexpr double kRelUpdate = 0.1;

struct PcgMixedArgs {
    KryScal* sc;
    int64_t m, nslices;
    const int32_t* perm;
    const int32_t* ptr;
    const int32_t* col;
    const float* val32;
    const double* val64;
    const float* diag;
    const double* b;
    double* x;
    float* r;
    float* z;
    float* p0;
    float* p1;
    float* q;
    double* part;  // [3][nblocks][3]
    GridSync gs;
    int max_iter;
    double tol;
    int rel;
    int* out_iter;
    double* out_resid;
    int* out_updates;
};

template <int NT>
__global__ void __launch_bounds__(NT, NT == 256 ? 3 : 1) k_pcg_mixed(PcgMixedArgs a) {
    __shared__ KryScal sc;
    const int lane = threadIdx.x & 31;
    double* partA = a.part;
    double* partB = a.part + (size_t)gridDim.x * 3;
    double* partC = a.part + (size_t)gridDim.x * 6;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
    const double tol = a.tol;
    const int max_iter = a.max_iter, rel = a.rel;

    // r = b - A x in FP64, then FP32 copies: r, z = r / d; <r,r>, <b,b>, <z,r> in FP64
    auto true_residual = [&](bool first) {
        double v[3] = {0., 0., 0.};
        const double* x = a.x;
        TF_SLICE_LOOP_BAL(a.nslices, s) {
            const double ax = sell_row<double>(a.ptr, a.col, a.val64, s, lane, [&](int32_t j) { return kld(x + j); });
            const int32_t row = __ldg(a.perm + s * 32 + lane);
            if (row >= 0) {
                const double bi = a.b[row];
                const double ri = bi - ax;
                const float r32 = (float)ri;
                const float z32 = r32 / a.diag[row];
                a.r[row] = r32;
                a.z[row] = z32;
                if (first) a.p0[row] = z32;
                v[0] += ri * ri;
                if (first) v[1] += bi * bi;
                v[2] += (double)(z32 * r32);
            }
        }
        block_partials<3>(v, partC);
    };

    true_residual(true);
    if (!grid_step<3>(a.gs, partC, a.sc, sc, [&](const double* s, KryScal& g) {
            double nb = sqrt(s[1]);
            if (nb == 0.0 || !rel) nb = 1.0;
            g.normb = nb;
            g.r_last = sqrt(s[0]);
            g.resid = g.r_last / nb;
            g.rho = s[2];
            g.beta = 0.;
            g.it = 0;
            g.updates = 1;
            g.true_res = 0;
            g.converged = g.resid <= tol;
            g.done = g.converged || max_iter <= 0;
        }))
        return;
    float* pc = a.p0;
    float* pn = a.p1;
    while (!sc.done) {
        const float beta = (float)sc.beta;
        // phase A (FP32): p_new = z + beta p_old ; q = A p_new ; <q, p_new>
        {
            float v[1] = {0.f};
            const float* z = a.z;
            const float* po = pc;
            TF_SLICE_LOOP_BAL(a.nslices, s) {
                const float acc = sell_row<float>(a.ptr, a.col, a.val32, s, lane,
                                                  [&](int32_t j) { return kld(z + j) + beta * kld(po + j); });
                const int32_t row = __ldg(a.perm + s * 32 + lane);
                if (row >= 0) {
                    const float pi = kld(z + row) + beta * kld(po + row);
                    pn[row] = pi;
                    a.q[row] = acc;
                    v[0] += acc * pi;
                }
            }
            block_partials<1>(v, partA);
        }
        if (!grid_step<1>(a.gs, partA, a.sc, sc, [&](const double* s, KryScal& g) { g.alpha = g.rho / s[0]; })) return;
        const double alpha = sc.alpha;
        const float alpha32 = (float)alpha;
        // phase B: x += alpha p (FP64) ; r -= alpha q ; z = r / d (FP32) ; <r,r>, <z,r>
        {
            float v[2] = {0.f, 0.f};
            for (int64_t i = tid; i < a.m; i += nth) {
                const float pi = kld(pn + i);
                a.x[i] += alpha * (double)pi;
                const float ri = a.r[i] - alpha32 * kld(a.q + i);
                const float zi = ri / a.diag[i];
                a.r[i] = ri;
                a.z[i] = zi;
                v[0] += ri * ri;
                v[1] += zi * ri;
            }
            block_partials<2>(v, partB);
        }
        if (!grid_step<2>(a.gs, partB, a.sc, sc, [&](const double* s, KryScal& g) {
                g.it += 1;
                const double rn = sqrt(s[0]);
                g.true_res = rn <= kRelUpdate * g.r_last || rn / g.normb <= tol || g.it >= max_iter;
                if (!g.true_res) {
                    g.beta = s[1] / g.rho;
                    g.rho = s[1];
                }
            }))
            return;
        if (sc.true_res) {
            // reliable update: the FP64 residual replaces the FP32 one
            true_residual(false);
            if (!grid_step<3>(a.gs, partC, a.sc, sc, [&](const double* s, KryScal& g) {
                    g.updates += 1;
                    g.r_last = sqrt(s[0]);
                    g.resid = g.r_last / g.normb;
                    g.converged = g.resid <= tol;
                    g.done = g.converged || g.it >= max_iter;
                    g.beta = s[2] / g.rho;
                    g.rho = s[2];
                }))
                return;
        }
        float* tmp = pc;
        pc = pn;
        pn = tmp;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *a.out_iter = sc.converged ? (int)sc.it : -1 - (int)sc.it;
        *a.out_resid = sc.resid;
        *a.out_updates = (int)sc.updates;
    }
}

// ---------------------------------------------------------------------------
// mixed-precision PCG with one grid barrier per iteration
//
// Chronopoulos-Gear form of preconditioned CG (s = A p carried by recurrence,
// w = A u computed): per iteration one SpMV w_{i+1} = A u_{i+1} and one
// all-reduce of six FP32 dots
//   gamma = (r,u), (u,w), (u,s), (p,w), (p,s), (r,r)
// from which every block derives beta = gamma / gamma_old and
// alpha = gamma / (p_new, s_new), (p_new, s_new) expanded exactly as
// (u,w) + beta ((u,s) + (p,w)) + beta^2 (p,s).  No second barrier for the
// vector updates: the SpMV gathers the per-row state V = {r_i, w_i, s_{i-1},
// 1/d} (one 16-byte load) and forms u_{i+1}[j] = (r_i - alpha (w_i + beta
// s_{i-1})) / d on the fly with the same rounding as the row's owner, which
// writes the next state into the other buffer.  The inner loop carries no
// FP64 arithmetic: the correction dx = sum alpha p is FP32 and is added to the
// FP64 iterate at each refinement.  Refinement (as in the two-barrier kernel:
// when the FP32 residual has dropped by kRelUpdate, claims convergence or
// max_iter is reached): fold x += dx; r = b - A x in FP64 (the convergence
// test); w = A (r / d) and s = A p in FP32 with p kept, continuing the
// recurrence with both carried vectors exact again.
// ---------------------------------------------------------------------------
struct PcgCg1Args {
    int64_t m, nslices;
    const int32_t* perm;
    const int32_t* ptr;
    const int32_t* col;
    const float* val32;
    const double* val64;
    const float* diag;
    const double* b;
    double* x;
    float4* V0;
    float4* V1;
    float* P;
    float* dx;
    GridAR g;
    int max_iter;
    double tol;
    int rel;
    int* out_iter;
    double* out_resid;
    int* out_updates;
    int32_t cache_cap;  // slots of the block's FP32 SELL run kept in shared memory (blocked pass)
};

// u_{i+1} of one row from its state {r_i, w_i, s_{i-1}, 1/d}; the owner and
// every gatherer evaluate exactly this sequence
__device__ __forceinline__ float cg1_s(float4 v, float beta) { return __fmaf_rn(beta, v.z, v.y); }
__device__ __forceinline__ float cg1_r(float4 v, float s, float alpha) { return __fmaf_rn(-alpha, s, v.x); }
__device__ __forceinline__ float cg1_u(float4 v, float alpha, float beta) {
    return __fmul_rn(cg1_r(v, cg1_s(v, beta), alpha), v.w);
}

template <int NT, bool BLK>
__global__ void __launch_bounds__(NT, NT == 256 ? 3 : 1) k_pcg_cg1(PcgCg1Args a) {
    const int lane = threadIdx.x & 31;
    unsigned long long epoch = 0;
    float4* Vc = a.V0;
    float4* Vn = a.V1;
    const int max_iter = a.max_iter;
    const double tol = a.tol;
    double normb = 1.0, r_last = 0.0, resid = 0.0;
    int it = 0, updates = 0;
    bool converged = false;
    float gam = 0.f, alpha = 0.f, beta = 0.f, thr_rel = 0.f, thr_tol = 0.f;

    // r = b - A x in FP64 into V.r (first: V = {r, 0, 0, 1/d}, p = 0);
    // returns false on a watchdog timeout, sets done/converged
    auto true_residual = [&](bool first, bool& done) -> bool {
        double v[2] = {0., 0.};
        const double* x = a.x;
        TF_SLICE_LOOP_BAL(a.nslices, s) {
            const double ax = sell_row<double>(a.ptr, a.col, a.val64, s, lane, [&](int32_t j) { return kld(x + j); });
            const int32_t row = __ldg(a.perm + s * 32 + lane);
            if (row >= 0) {
                const double bi = a.b[row];
                const double ri = bi - ax;
                float4 vc;
                if (first) {
                    vc = make_float4((float)ri, 0.f, 0.f, 1.0f / a.diag[row]);
                    a.P[row] = 0.f;
                } else {
                    vc = Vc[row];
                    vc.x = (float)ri;
                }
                Vc[row] = vc;
                v[0] += ri * ri;
                if (first) v[1] += bi * bi;
            }
        }
        double o[2];
        if (!grid_allreduce<double, 2>(a.g, epoch, v, o)) return false;
        // FP64 square roots and division on one thread (FP64 issues at a
        // small fraction of the FP32 rate), broadcast through shared memory
        __shared__ double sh[4];
        if (threadIdx.x == 0) {
            double nb = normb;
            if (first) {
                nb = sqrt(o[1]);
                if (nb == 0.0 || !a.rel) nb = 1.0;
            }
            const double rl = sqrt(o[0]);
            sh[0] = nb;
            sh[1] = rl;
            sh[2] = rl / nb;
        }
        __syncthreads();
        normb = sh[0];
        r_last = sh[1];
        resid = sh[2];
        __syncthreads();
        ++updates;
        converged = resid <= tol;
        done = converged || it >= max_iter;
        thr_rel = (float)(kRelUpdate * r_last);
        thr_tol = (float)(tol * normb);
        return true;
    };

    // one SpMV pass; refresh: w = A (r / d) and s = A p with r, p kept (after
    // a true residual), else the CG step with (alpha, beta)
    // row update of slot (s, lane) from its products wn = (A u)_row and, on
    // a refresh, sx = (A p)_row
    // pp / pdx: where the row's p and dx live (shared memory for a planned
    // block, which owns its rows for the whole solve; else global memory)
    auto row_update = [&](int64_t s, float wn, float sx, bool refresh, float al, float be, const float4* V,
                          float (&v)[6], int32_t row, float* pp, float* pdx) {
            if (row >= 0) {
                const float4 vc = V[row];
                float sn, rn, pn;
                if (refresh) {
                    sn = sx;
                    rn = vc.x;
                    pn = *pp;
                } else {
                    sn = cg1_s(vc, be);
                    rn = cg1_r(vc, sn, al);
                    pn = __fmaf_rn(be, *pp, __fmul_rn(vc.x, vc.w));
                    *pp = pn;
                    *pdx = __fmaf_rn(al, pn, *pdx);
                }
                const float un = __fmul_rn(rn, vc.w);
                Vn[row] = make_float4(rn, wn, sn, vc.w);
                v[0] += rn * un;
                v[1] += un * wn;
                v[2] += un * sn;
                v[3] += pn * wn;
                v[4] += pn * sn;
                v[5] += rn * rn;
            }
    };

    // Blocked pass: block b owns the contiguous slices [b n/G, (b+1) n/G)
    // (neighbouring rows, so the state gathers of an SM share its L1), splits
    // their column work evenly over its warps (sell_block_balanced), keeps the
    // row products in shared memory and then updates its rows.  The other form
    // walks whole slices per warp in the balanced global order.
    __shared__ BalShared<NT / 32, float> bsh;
    __shared__ float wsm[BLK ? kBalMaxSlices : 1][32], ssm[BLK ? kBalMaxSlices : 1][32];
    // this block's slices: equal shares of column work plus row updates
    const int64_t sb0 = BLK ? balanced_part_start(a.ptr, a.nslices, blockIdx.x, gridDim.x) : 0;
    const int64_t sb1 = BLK ? balanced_part_start(a.ptr, a.nslices, blockIdx.x + 1, gridDim.x) : 0;
    // The FP32 matrix does not change during the solve: the leading slots of
    // the block's run (as many as the dynamic shared memory holds) are copied
    // once and every pass reads them from shared memory, so only the state
    // gathers go to L1/L2.
    extern __shared__ __align__(16) unsigned char cg1_dyn[];
    SellCache<float> cache;
    if constexpr (BLK) {
        if (a.cache_cap > 0) {
            const int32_t pb = __ldg(a.ptr + sb0), pe = __ldg(a.ptr + sb1);
            const int32_t ns = pe - pb < a.cache_cap ? pe - pb : a.cache_cap;
            int32_t* ccol = reinterpret_cast<int32_t*>(cg1_dyn);
            float* cval = reinterpret_cast<float*>(cg1_dyn + sizeof(int32_t) * (size_t)a.cache_cap);
            for (int32_t k = threadIdx.x; k < ns; k += NT) {
                ccol[k] = __ldg(a.col + pb + k);
                cval[k] = __ldg(a.val32 + pb + k);
            }
            __syncthreads();
            cache.col = ccol;
            cache.val = cval;
            cache.base = pb;
            cache.cap = ns;
        }
    }
    // a block whose run fits one chunk plans its column split once and keeps
    // the rows of its slots (perm) in shared memory
    // (and its rows' p and dx: only the owner reads or writes them between two
    // refinements; the fold publishes p for the refresh pass, which gathers it)
    const bool planned = BLK && sb1 - sb0 <= kBalMaxSlices;
    __shared__ int32_t sperm[BLK ? kBalMaxSlices : 1][32];
    __shared__ float sP[BLK ? kBalMaxSlices : 1][32], sdx[BLK ? kBalMaxSlices : 1][32];
    if (planned) {
        for (int k = threadIdx.x; k < (int)(sb1 - sb0) * 32; k += NT) {
            sperm[k >> 5][k & 31] = __ldg(a.perm + sb0 * 32 + k);
            sP[k >> 5][k & 31] = 0.f;
            sdx[k >> 5][k & 31] = 0.f;
        }
        sell_block_plan<NT / 32, float>(bsh, a.ptr, sb0, (int)(sb1 - sb0));
    }
    auto pass = [&](bool refresh, float (&o)[6]) -> bool {
        float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const float al = refresh ? 0.f : alpha, be = refresh ? 0.f : beta;
        const float4* V = Vc;
        if constexpr (BLK) {
            for (int64_t c0 = sb0; c0 < sb1; c0 += kBalMaxSlices) {
                const int S = (int)(sb1 - c0 < kBalMaxSlices ? sb1 - c0 : kBalMaxSlices);
                if (!planned) sell_block_plan<NT / 32, float>(bsh, a.ptr, c0, S);
                sell_block_walk<NT / 32, float>(
                    bsh, a.ptr, a.col, a.val32, c0, S, [&](int32_t j) { return cg1_u(kld(V + j), al, be); },
                    [&](int64_t s, float val) { wsm[s - c0][lane] = val; }, cache);
                // refresh: s = A p recomputed, ending the drift of its recurrence
                if (refresh)
                    sell_block_walk<NT / 32, float>(
                        bsh, a.ptr, a.col, a.val32, c0, S, [&](int32_t j) { return kld(a.P + j); },
                        [&](int64_t s, float val) { ssm[s - c0][lane] = val; }, cache);
                // (the next chunk overwrites wsm only after the first block
                // barrier inside sell_block_balanced, i.e. after this loop)
                for (int i = threadIdx.x >> 5; i < S; i += NT / 32) {
                    const int32_t row = planned ? sperm[i][lane] : __ldg(a.perm + (c0 + i) * 32 + lane);
                    row_update(c0 + i, wsm[i][lane], refresh ? ssm[i][lane] : 0.f, refresh, al, be, V, v, row,
                               planned ? &sP[i][lane] : a.P + (row >= 0 ? row : 0),
                               planned ? &sdx[i][lane] : a.dx + (row >= 0 ? row : 0));
                }
            }
        } else {
            TF_SLICE_LOOP_BAL(a.nslices, s) {
                const float wn = sell_row<float>(a.ptr, a.col, a.val32, s, lane,
                                                 [&](int32_t j) { return cg1_u(kld(V + j), al, be); });
                const float sx = refresh ? sell_row<float>(a.ptr, a.col, a.val32, s, lane,
                                                           [&](int32_t j) { return kld(a.P + j); })
                                         : 0.f;
                const int32_t row = __ldg(a.perm + s * 32 + lane);
                row_update(s, wn, sx, refresh, al, be, V, v, row, a.P + (row >= 0 ? row : 0),
                           a.dx + (row >= 0 ? row : 0));
            }
        }
        if (!grid_allreduce<float, 6>(a.g, epoch, v, o)) return false;
        float4* t = Vc;
        Vc = Vn;
        Vn = t;
        return true;
    };

    // FP64 fold of the FP32 correction (own rows; a planned block also
    // publishes its p), then a barrier
    auto fold = [&]() -> bool {
        if (planned) {
            for (int i = threadIdx.x >> 5; i < (int)(sb1 - sb0); i += NT / 32) {
                const int32_t row = sperm[i][lane];
                if (row >= 0) {
                    a.x[row] += (double)sdx[i][lane];
                    sdx[i][lane] = 0.f;
                    a.P[row] = sP[i][lane];
                }
            }
        } else if (BLK) {
            for (int64_t s = sb0 + (threadIdx.x >> 5); s < sb1; s += NT / 32) {
                const int32_t row = __ldg(a.perm + s * 32 + lane);
                if (row >= 0) {
                    a.x[row] += (double)a.dx[row];
                    a.dx[row] = 0.f;
                }
            }
        } else {
            TF_SLICE_LOOP_BAL(a.nslices, s) {
                const int32_t row = __ldg(a.perm + s * 32 + lane);
                if (row >= 0) {
                    a.x[row] += (double)a.dx[row];
                    a.dx[row] = 0.f;
                }
            }
        }
        return grid_sync_ar(a.g, epoch);
    };

    bool done = false;
    if (!true_residual(true, done)) return;
    bool first = true;
    while (!done) {
        float o[6];
        if (!pass(true, o)) return;
        // continue the recurrence: beta against the gamma that built p
        beta = first ? 0.f : o[0] / gam;
        first = false;
        gam = o[0];
        alpha = gam / (o[1] + beta * (o[2] + o[3]) + beta * beta * o[4]);
        bool refine = false;
        while (!refine) {
            if (!pass(false, o)) return;
            ++it;
            const float rn = sqrtf(o[5]);
            refine = rn <= thr_rel || rn <= thr_tol || it >= max_iter;
            if (!refine) {
                beta = o[0] / gam;
                gam = o[0];
                alpha = gam / (o[1] + beta * (o[2] + o[3]) + beta * beta * o[4]);
            }
        }
        if (!fold()) return;
        if (!true_residual(false, done)) return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *a.out_iter = converged ? it : -1 - it;
        *a.out_resid = resid;
        *a.out_updates = updates;
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

// blocks of a cooperative launch: all co-resident, at most one row slice per warp
int coop_blocks(Context* c, const void* fn, int64_t nslices, int* out, int threads, size_t dyn_smem) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, dyn_smem) != cudaSuccess || per_sm < 1)
        return set_err(c, TF_ERR_CUDA, "occupancy query failed");
    if (c->kry_blocks_per_sm > 0 && c->kry_blocks_per_sm < per_sm) per_sm = c->kry_blocks_per_sm;
    const int64_t want = (nslices * 32 + threads - 1) / threads;
    int64_t b = std::min<int64_t>(want, (int64_t)per_sm * c->num_sms);
    *out = (int)(b < 1 ? 1 : b);
    return TF_OK;
}

template <class T>
static int run_pcg_kernel(Context* c, const CSR& A, const T* val, const T* diag, const T* b, T* x, T* work, int max_iter,
                          double tol, int rel, int* iters_out, double* resid_out) {
    const void* fn = (const void*)k_pcg<T>;
    int blocks = 0;
    TF_TRY(coop_blocks(c, fn, A.sell.nslices, &blocks, kKryThreads));
    const size_t part_d = (size_t)2 * blocks * kArMax;
    TF_TRY(ensure(c, c->kry_part, part_d + (part_d + 1) / 2 + 16));
    TF_TRY(ensure(c, c->kry_bar, 2));
    TF_TRY(ensure(c, c->kry_iters, 1));
    TF_TRY(ensure(c, c->kry_resid, 1));
    TF_CUDA(c, cudaMemsetAsync(c->kry_bar.p, 0, 2 * sizeof(unsigned), c->stream));
    TF_CUDA(c, cudaMemsetAsync(c->status.p, 0, 4 * sizeof(int), c->stream));
    PcgArgs<T> a;
    a.m = A.m;
    a.nslices = A.sell.nslices;
    a.perm = A.sell.perm;
    a.ptr = A.sell.ptr;
    a.col = A.sell.col;
    a.val = val;
    a.diag = diag;
    a.b = b;
    a.x = x;
    a.r = work;
    a.z = work + A.m;
    a.p0 = work + 2 * A.m;
    a.p1 = work + 3 * A.m;
    a.q = work + 4 * A.m;
    a.g.count = reinterpret_cast<unsigned long long*>(c->kry_bar.p);
    a.g.partd = c->kry_part.p;
    a.g.partf = reinterpret_cast<float*>(c->kry_part.p + part_d);
    a.g.status = c->status.p;
    a.max_iter = max_iter;
    a.tol = tol;
    a.rel = rel;
    a.out_iter = c->kry_iters.p;
    a.out_resid = c->kry_resid.p;
    void* args[] = {&a};
    TF_CUDA(c, cudaLaunchCooperativeKernel(fn, blocks, kKryThreads, args, 0, c->stream));
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

// single-barrier mixed PCG (k_pcg_cg1); workspace in floats: V0, V1 (4m each,
// 16-byte aligned), p, dx, FP32 diagonal
static int run_pcg_cg1(Context* c, const CSR& A, const double* b, double* x, int* max_iter, double* tol, int rel,
                       int nt) {
    const int64_t m = A.m;
    TF_TRY(ensure(c, c->kry32, (size_t)(11 * m)));
    float* base = c->kry32.p;
    float* d32 = base + 10 * m;
    k_to_f32<<<grid_for(c, m), kBlock, 0, c->stream>>>(m, A.diag, d32);
    ++c->launches;
    const void* fn = c->pcg_blocked ? (nt == 512 ? (const void*)k_pcg_cg1<512, true> : (const void*)k_pcg_cg1<256, true>)
                                    : (nt == 512 ? (const void*)k_pcg_cg1<512, false> : (const void*)k_pcg_cg1<256, false>);
    // dynamic shared memory for the matrix cache: what the opt-in limit leaves
    // after the static shared memory (one block per SM at 512 threads)
    size_t dyn = 0;
    int32_t cap = 0;
    if (c->pcg_blocked && nt == 512 && c->pcg_smem_cache_kb > 0) {
        cudaFuncAttributes fa{};
        int optin = 0;
        TF_CUDA(c, cudaFuncGetAttributes(&fa, fn));
        TF_CUDA(c, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
        const int64_t room = std::min<int64_t>((int64_t)optin - (int64_t)fa.sharedSizeBytes - 1024,
                                               (int64_t)c->pcg_smem_cache_kb * 1024);
        if (room > 4096) {
            cap = (int32_t)((room / 8) & ~(int64_t)3);
            dyn = (size_t)cap * 8;
            TF_CUDA(c, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
        }
    }
    int blocks = 0;
    TF_TRY(coop_blocks(c, fn, A.sell.nslices, &blocks, nt, dyn));
    const size_t part_d = (size_t)2 * blocks * kArMax;
    TF_TRY(ensure(c, c->kry_part, part_d + (part_d + 1) / 2 + 16));
    TF_TRY(ensure(c, c->kry_bar, 2));
    TF_TRY(ensure(c, c->kry_iters, 2));
    TF_TRY(ensure(c, c->kry_resid, 1));
    TF_CUDA(c, cudaMemsetAsync(c->kry_bar.p, 0, 2 * sizeof(unsigned), c->stream));
    TF_CUDA(c, cudaMemsetAsync(c->status.p, 0, 4 * sizeof(int), c->stream));
    TF_CUDA(c, cudaMemsetAsync(base + 9 * m, 0, sizeof(float) * (size_t)m, c->stream));
    PcgCg1Args g;
    g.m = m;
    g.nslices = A.sell.nslices;
    g.perm = A.sell.perm;
    g.ptr = A.sell.ptr;
    g.col = A.sell.col;
    g.val32 = A.sell.v32;
    g.val64 = A.sell.v64;
    g.diag = d32;
    g.b = b;
    g.x = x;
    g.V0 = reinterpret_cast<float4*>(base);
    g.V1 = reinterpret_cast<float4*>(base + 4 * m);
    g.P = base + 8 * m;
    g.dx = base + 9 * m;
    g.g.count = reinterpret_cast<unsigned long long*>(c->kry_bar.p);
    g.g.partd = c->kry_part.p;
    g.g.partf = reinterpret_cast<float*>(c->kry_part.p + part_d);
    g.g.status = c->status.p;
    g.max_iter = *max_iter;
    g.tol = *tol;
    g.rel = rel;
    g.out_iter = c->kry_iters.p;
    g.out_resid = c->kry_resid.p;
    g.out_updates = c->kry_iters.p + 1;
    g.cache_cap = cap;
    void* args[] = {&g};
    TF_CUDA(c, cudaLaunchCooperativeKernel(fn, blocks, nt, args, dyn, c->stream));
    ++c->launches;
    int it[2] = {0, 0};
    double res = 0;
    TF_CUDA(c, cudaMemcpyAsync(it, c->kry_iters.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaMemcpyAsync(&res, c->kry_resid.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    int st = 0;
    TF_TRY(sync_status(c, &st));
    if (st) return set_err(c, st, "pcg (mixed): grid barrier watchdog fired");
    c->last_refinements = it[1];
    *max_iter = it[0] >= 0 ? it[0] : -1 - it[0];
    *tol = res;
    return it[0] >= 0 ? TF_OK : set_err(c, TF_ERR_NOT_CONVERGED, "pcg (mixed): no convergence within max_iter");
}

// the single-barrier mixed solver of the given kind (the resident kernel falls
// back to the 512-thread k_pcg_cg1 where the block runs do not fit)
int pcg_mixed_kind(Context* c, CSR& A, const double* b, double* x, int kind, int* max_iter, double* tol, int rel) {
    if (kind == kPcgResident) {
        bool applied = false;
        const int st = pcg_resident<float>(c, A, b, x, max_iter, tol, rel, &applied);
        if (applied || st != TF_OK) return st;
    }
    return run_pcg_cg1(c, A, b, x, max_iter, tol, rel, kind == kPcgCg1_256 ? 256 : 512);
}

int pcg_jacobi(Context* c, CSR& A, const double* b, double* x, int precision, int* max_iter, double* tol, int rel) {
    if (!A.vals || A.m <= 0) return set_err(c, TF_ERR_BAD_INPUT, "pcg: empty matrix");
    TF_TRY(ensure_diag(c, A));
    TF_TRY(ensure_sell(c, A, precision == TF_PREC_MIXED));
    const int64_t m = A.m;
    TimedLaunch tl(c, TF_K_PCG);
    if (precision == TF_PREC_FP64) {
        if (c->pcg_fp64_kernel == TF_PCG_FP64_CG1) {
            bool applied = false;
            const int st = pcg_resident<double>(c, A, b, x, max_iter, tol, rel, &applied);
            if (applied || st != TF_OK) return st;
        }
        TF_TRY(ensure(c, c->kry64, (size_t)(5 * m)));
        int it = 0;
        double res = 0.;
        TF_TRY(run_pcg_kernel<double>(c, A, A.sell.v64, A.diag, b, x, c->kry64.p, *max_iter, *tol, rel, &it, &res));
        const bool ok = it >= 0;
        *max_iter = ok ? it : -1 - it;
        *tol = res;
        return ok ? TF_OK : set_err(c, TF_ERR_NOT_CONVERGED, "pcg: no convergence within max_iter");
    }
    // mixed precision: FP32 iterations, FP64 iterate and reliable updates
    TF_TRY(ensure_sell(c, A, false));  // FP64 copy for the refinement residuals
    if (!c->pcg_two_barrier) {
        int kind = c->pcg_resident ? kPcgResident : c->kry_threads == 256 ? kPcgCg1_256 : kPcgCg1_512;
        if (c->autotune && !c->pcg_shape_fixed) TF_TRY(tuned_pcg_kind(c, A, b, &kind));
        return pcg_mixed_kind(c, A, b, x, kind, max_iter, tol, rel);
    }
    TF_TRY(ensure(c, c->kry32, (size_t)(6 * m)));
    float* d32 = c->kry32.p;
    k_to_f32<<<grid_for(c, m), kBlock, 0, c->stream>>>(m, A.diag, d32);
    ++c->launches;
    // 512-thread blocks (one per SM): half the blocks arrive at each grid barrier
    const int nt = c->kry_threads == 512 ? 512 : 256;
    const void* fn = nt == 512 ? (const void*)k_pcg_mixed<512> : (const void*)k_pcg_mixed<256>;
    int blocks = 0;
    TF_TRY(coop_blocks(c, fn, A.sell.nslices, &blocks, nt));
    TF_TRY(ensure(c, c->kry_part, (size_t)blocks * 3 * 3 + 16 + kScalWords));
    TF_TRY(ensure(c, c->kry_bar, 2));
    TF_TRY(ensure(c, c->kry_iters, 2));
    TF_TRY(ensure(c, c->kry_resid, 1));
    TF_CUDA(c, cudaMemsetAsync(c->kry_bar.p, 0, 2 * sizeof(unsigned), c->stream));
    TF_CUDA(c, cudaMemsetAsync(c->status.p, 0, 4 * sizeof(int), c->stream));
    PcgMixedArgs g;
    g.m = m;
    g.nslices = A.sell.nslices;
    g.perm = A.sell.perm;
    g.ptr = A.sell.ptr;
    g.col = A.sell.col;
    g.val32 = A.sell.v32;
    g.val64 = A.sell.v64;
    g.diag = d32;
    g.b = b;
    g.x = x;
    g.r = d32 + m;
    g.z = d32 + 2 * m;
    g.p0 = d32 + 3 * m;
    g.p1 = d32 + 4 * m;
    g.q = d32 + 5 * m;
    g.part = c->kry_part.p;
    g.sc = reinterpret_cast<KryScal*>(c->kry_part.p + (size_t)blocks * 3 * 3 + 16);
    g.gs = GridSync{c->kry_bar.p, c->kry_bar.p + 1, c->status.p};
    g.max_iter = *max_iter;
    g.tol = *tol;
    g.rel = rel;
    g.out_iter = c->kry_iters.p;
    g.out_resid = c->kry_resid.p;
    g.out_updates = c->kry_iters.p + 1;
    void* args[] = {&g};
    TF_CUDA(c, cudaLaunchCooperativeKernel(fn, blocks, nt, args, 0, c->stream));
    ++c->launches;
    int it[2] = {0, 0};
    double res = 0;
    TF_CUDA(c, cudaMemcpyAsync(it, c->kry_iters.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaMemcpyAsync(&res, c->kry_resid.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    int st = 0;
    TF_TRY(sync_status(c, &st));
    if (st) return set_err(c, st, "pcg (mixed): grid barrier watchdog fired");
    c->last_refinements = it[1];
    *max_iter = it[0] >= 0 ? it[0] : -1 - it[0];
    *tol = res;
    return it[0] >= 0 ? TF_OK : set_err(c, TF_ERR_NOT_CONVERGED, "pcg (mixed): no convergence within max_iter");
}

// ---------------------------------------------------------------------------
// persistent restarted GMRES (num/krylovsolver.h:320-463)
//
// One cooperative kernel runs the whole solve.  Basis vectors are stored
// unnormalised with a scale factor (v_k = sc_k * V_k), so v_{i+1} = w / h_{i+1,i}
// needs no extra pass.  Modified Gram-Schmidt keeps the reference's order:
// one grid barrier per projection.  The Hessenberg matrix, the Givens
// rotations and the right-hand side s live in shared memory of every block and
// are updated redundantly (bit-identical in all blocks).
// ---------------------------------------------------------------------------
constexpr int kMaxRestart = 64;

struct GmresArgs {
    double* result;
    int64_t m, nslices;
    const int32_t* perm;
    const int32_t* ptr;
    const int32_t* col;
    const double* val;
    const double* diag;
    const double* b;
    double* x;
    double* V;     // [R][m] unnormalised basis
    double* part;  // [2][nblocks][2]
    GridSync gs;
    int R;         // restart
    int left;      // 1: left preconditioning, 0: right
    const double* binv;  // nodal 2x2 block-Jacobi inverses [m/2][4] (NULL: point Jacobi)
    double* Z;           // work vector for the block preconditioner
    int max_iter;
    double tol;
    int rel;
    int* out_iter;
    double* out_resid;
};

__global__ void __launch_bounds__(kKryThreads, 2) k_gmres(GmresArgs a) {
    const int lane = threadIdx.x & 31;
    __shared__ double H[kMaxRestart][kMaxRestart];
    __shared__ double cs[kMaxRestart], sn[kMaxRestart], s[kMaxRestart + 1], y[kMaxRestart], sc[kMaxRestart];
    const int64_t m = a.m;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
    double* partA = a.part;
    double* partB = a.part + (size_t)gridDim.x * 2;
    int flip = 0;
    auto P = [&]() { flip ^= 1; return flip ? partB : partA; };

    // r0 = b - A x (right) or M^{-1}(b - A x) (left) into V_0; <r,r>, |b| or |M^{-1} b|
    {
        double* pp = P();
        double v[2] = {0., 0.};
        const double* x0 = a.x;
        TF_SLICE_LOOP_BAL(a.nslices, sl) {
            const double ax = sell_row<double>(a.ptr, a.col, a.val, sl, lane, [&](int32_t j) { return kld(x0 + j); });
            const int32_t row = __ldg(a.perm + sl * 32 + lane);
            if (row >= 0) {
                double r = a.b[row] - ax, bb = a.b[row];
                if (a.left) {
                    r = r / a.diag[row];
                    bb = bb / a.diag[row];
                }
                a.V[row] = r;
                v[0] += r * r;
                v[1] += bb * bb;
            }
        }
        block_partials<2>(v, pp);
        double t[2];
        if (!grid_sync_reduce<2>(a.gs, pp, a.result, t)) return;
        double beta = sqrt(t[0]);
        double normb = sqrt(t[1]);
        if (normb == 0.0 || !a.rel) normb = 1.0;
        double resid = beta / normb;
        if (resid <= a.tol) {
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                *a.out_iter = 0;
                *a.out_resid = resid;
            }
            return;
        }
        int j = 1;
        while (j <= a.max_iter) {
            if (threadIdx.x == 0) {
                sc[0] = 1.0 / beta;
                s[0] = beta;
                for (int k = 1; k <= a.R; ++k) s[k] = 0.;
            }
            __syncthreads();
            int i;
            bool done = false;
            for (i = 0; i < a.R - 1 && j <= a.max_iter; ++i, ++j) {
                const double* Vi = a.V + (size_t)i * m;
                double* W = a.V + (size_t)(i + 1) * m;
                const double sci = sc[i], sc0 = sc[0];
                // block Jacobi (right): Z = P^{-1} v_i node by node, then w = A Z
                if (a.binv) {
                    const int64_t half = m / 2;
                    for (int64_t e = tid; e < half; e += nth) {
                        const double va = sci * kld(Vi + e), vb = sci * kld(Vi + e + half);
                        const double* q4 = a.binv + 4 * e;
                        a.Z[e] = q4[0] * va + q4[1] * vb;
                        a.Z[e + half] = q4[2] * va + q4[3] * vb;
                    }
                    if (!grid_barrier(a.gs)) return;
                }
                // w = A M^{-1} v_i (right) or M^{-1} A v_i (left); <w, v_0>
                {
                    double* pq = P();
                    double v1[1] = {0.};
                    const bool left = a.left;
                    const double* dg = a.diag;
                    const double* Zp = a.binv ? a.Z : nullptr;
                    TF_SLICE_LOOP_BAL(a.nslices, s2) {
                        double acc = sell_row<double>(a.ptr, a.col, a.val, s2, lane, [&](int32_t j) {
                            if (Zp) return kld(Zp + j);
                            const double vj = sci * kld(Vi + j);
                            return left ? vj : vj / __ldg(dg + j);
                        });
                        const int32_t row = __ldg(a.perm + s2 * 32 + lane);
                        if (row >= 0) {
                            if (a.left) acc = acc / a.diag[row];
                            W[row] = acc;
                            v1[0] += acc * (sc0 * kld(a.V + row));
                        }
                    }
                    block_partials<1>(v1, pq);
                    double h[1];
                    if (!grid_sync_reduce<1>(a.gs, pq, a.result + 2 + flip, h)) return;
                    if (threadIdx.x == 0) H[0][i] = h[0];
                    __syncthreads();
                }
                // modified Gram-Schmidt: w -= h_k v_k, then <w, v_{k+1}> (or <w,w>)
                for (int k = 0; k <= i; ++k) {
                    double* pq = P();
                    const double hk = H[k][i] * sc[k];
                    const double* Vk = a.V + (size_t)k * m;
                    const double* Vn = k < i ? a.V + (size_t)(k + 1) * m : nullptr;
                    const double scn = k < i ? sc[k + 1] : 0.;
                    double v1[1] = {0.};
                    for (int64_t e = tid; e < m; e += nth) {
                        const double w = kld(W + e) - hk * kld(Vk + e);
                        W[e] = w;
                        v1[0] += k < i ? w * (scn * kld(Vn + e)) : w * w;
                    }
                    block_partials<1>(v1, pq);
                    double h[1];
                    if (!grid_sync_reduce<1>(a.gs, pq, a.result + 2 + flip, h)) return;
                    if (threadIdx.x == 0) {
                        if (k < i) H[k + 1][i] = h[0];
                        else H[i + 1][i] = sqrt(h[0]);
                    }
                    __syncthreads();
                }
                if (threadIdx.x == 0) {
                    sc[i + 1] = 1.0 / H[i + 1][i];
                    for (int k = 0; k < i; ++k) {
                        const double t0 = cs[k] * H[k][i] + sn[k] * H[k + 1][i];
                        H[k + 1][i] = -sn[k] * H[k][i] + cs[k] * H[k + 1][i];
                        H[k][i] = t0;
                    }
                    const double dx = H[i][i], dy = H[i + 1][i];
                    if (dy == 0.0) {
                        cs[i] = 1.0;
                        sn[i] = 0.0;
                    } else {
                        const double r = sqrt(dx * dx + dy * dy);
                        cs[i] = dx / r;
                        sn[i] = dy / r;
                    }
                    double t0 = cs[i] * H[i][i] + sn[i] * H[i + 1][i];
                    H[i + 1][i] = -sn[i] * H[i][i] + cs[i] * H[i + 1][i];
                    H[i][i] = t0;
                    t0 = cs[i] * s[i] + sn[i] * s[i + 1];
                    s[i + 1] = -sn[i] * s[i] + cs[i] * s[i + 1];
                    s[i] = t0;
                }
                __syncthreads();
                resid = fabs(s[i + 1]) / normb;
                if (resid <= a.tol) {
                    done = true;
                    break;
                }
            }
            // x += V y (left) or x += M^{-1} V y (right) with k = i (converged) or i - 1
            const int kk = done ? i : i - 1;
            if (threadIdx.x == 0) {
                for (int q = 0; q <= kk; ++q) y[q] = s[q];
                for (int q = kk; q >= 0; --q) {
                    y[q] /= H[q][q];
                    for (int p = q - 1; p >= 0; --p) y[p] -= H[p][q] * y[q];
                }
            }
            __syncthreads();
            if (a.binv) {
                const int64_t half = m / 2;
                for (int64_t e = tid; e < half; e += nth) {
                    double za = 0., zb = 0.;
                    for (int q = 0; q <= kk; ++q) {
                        za += y[q] * (sc[q] * kld(a.V + (size_t)q * m + e));
                        zb += y[q] * (sc[q] * kld(a.V + (size_t)q * m + e + half));
                    }
                    const double* q4 = a.binv + 4 * e;
                    a.x[e] = a.x[e] + (q4[0] * za + q4[1] * zb);
                    a.x[e + half] = a.x[e + half] + (q4[2] * za + q4[3] * zb);
                }
            } else {
                for (int64_t e = tid; e < m; e += nth) {
                    double z = 0.;
                    for (int q = 0; q <= kk; ++q) z += y[q] * (sc[q] * kld(a.V + (size_t)q * m + e));
                    if (!a.left) z = z / a.diag[e];
                    a.x[e] = a.x[e] + z;
                }
            }
            if (done) {
                if (blockIdx.x == 0 && threadIdx.x == 0) {
                    *a.out_iter = j;
                    *a.out_resid = resid;
                }
                return;
            }
            if (!grid_barrier(a.gs)) return;
            // new residual into V_0
            {
                double* pq = P();
                double v1[1] = {0.};
                const double* x1 = a.x;
                TF_SLICE_LOOP_BAL(a.nslices, s3) {
                    const double ax = sell_row<double>(a.ptr, a.col, a.val, s3, lane, [&](int32_t j) { return kld(x1 + j); });
                    const int32_t row = __ldg(a.perm + s3 * 32 + lane);
                    if (row >= 0) {
                        double r = a.b[row] - ax;
                        if (a.left) r = r / a.diag[row];
                        a.V[row] = r;
                        v1[0] += r * r;
                    }
                }
                block_partials<1>(v1, pq);
                double t1[1];
                if (!grid_sync_reduce<1>(a.gs, pq, a.result + 2 + flip, t1)) return;
                beta = sqrt(t1[0]);
                resid = beta / normb;
                if (resid <= a.tol) {
                    if (blockIdx.x == 0 && threadIdx.x == 0) {
                        *a.out_iter = j;
                        *a.out_resid = resid;
                    }
                    return;
                }
            }
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            *a.out_iter = -(j - 1);
            *a.out_resid = resid;
        }
    }
}

// nodal 2x2 block-Jacobi inverses of a 2x2 block system (rows i and i + m/2)
__global__ void k_block_inv(int64_t half, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ colind,
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

int gmres_jacobi(Context* c, CSR& A, const double* b, double* x, int restart, int method, int precision, int* max_iter,
                 double* tol, int rel) {
    if (!A.vals || A.m <= 0) return set_err(c, TF_ERR_BAD_INPUT, "gmres: empty matrix");
    const bool block = &A == &c->mats[TF_MAT_BLOCK];
    if (block && method == 1)
        return set_err(c, TF_ERR_BAD_INPUT, "gmres: the block-Jacobi preconditioner is applied from the right (method 0)");
    if (precision == TF_PREC_MIXED || (precision == TF_PREC_FP64 && c->gmres_orth == TF_ORTH_CGS2)) {
        if (method != 0) return set_err(c, TF_ERR_BAD_INPUT, "gmres (CGS2 / mixed): right preconditioning only");
        return gmres2(c, A, b, x, restart, precision == TF_PREC_MIXED, max_iter, tol, rel);
    }
    if (restart > kMaxRestart) return set_err(c, TF_ERR_CAPACITY, "gmres: restart > 64");
    if (precision != TF_PREC_FP64) return set_err(c, TF_ERR_BAD_INPUT, "gmres: precision");
    TF_TRY(ensure_diag(c, A));
    TF_TRY(ensure_sell(c, A, false));
    const int64_t m = A.m;
    const int R = restart <= *max_iter ? restart : (*max_iter > 1 ? *max_iter : 2);
    TimedLaunch tl(c, TF_K_GMRES);
    TF_TRY(ensure(c, c->kry64, (size_t)(R + 1) * m + (block ? 2 * m : 0)));
    double* binv = nullptr;
    if (block) {
        binv = c->kry64.p + (size_t)(R + 1) * m;
        k_block_inv<<<grid_for(c, m / 2), kBlock, 0, c->stream>>>(m / 2, A.rowptr, A.colind, A.vals, binv);
        ++c->launches;
        TF_CUDA(c, cudaGetLastError());
    }
    const void* fn = (const void*)k_gmres;
    int blocks = 0;
    TF_TRY(coop_blocks(c, fn, A.sell.nslices, &blocks, kKryThreads));
    TF_TRY(ensure(c, c->kry_part, (size_t)blocks * 2 * 2 + 8));
    TF_TRY(ensure(c, c->kry_bar, 2));
    TF_TRY(ensure(c, c->kry_iters, 1));
    TF_TRY(ensure(c, c->kry_resid, 1));
    TF_CUDA(c, cudaMemsetAsync(c->kry_bar.p, 0, 2 * sizeof(unsigned), c->stream));
    TF_CUDA(c, cudaMemsetAsync(c->status.p, 0, 4 * sizeof(int), c->stream));
    GmresArgs g;
    g.m = m;
    g.nslices = A.sell.nslices;
    g.perm = A.sell.perm;
    g.ptr = A.sell.ptr;
    g.col = A.sell.col;
    g.val = A.sell.v64;
    g.diag = A.diag;
    g.b = b;
    g.x = x;
    g.V = c->kry64.p;
    g.part = c->kry_part.p;
    g.result = c->kry_part.p + (size_t)blocks * 2 * 2;
    g.gs = GridSync{c->kry_bar.p, c->kry_bar.p + 1, c->status.p};
    g.R = R;
    g.left = method == 1;
    g.binv = binv;
    g.Z = c->kry64.p + (size_t)R * m;
    g.max_iter = *max_iter;
    g.tol = *tol;
    g.rel = rel;
    g.out_iter = c->kry_iters.p;
    g.out_resid = c->kry_resid.p;
    void* args[] = {&g};
    TF_CUDA(c, cudaLaunchCooperativeKernel(fn, blocks, kKryThreads, args, 0, c->stream));
    ++c->launches;
    int it = 0;
    double res = 0;
    TF_CUDA(c, cudaMemcpyAsync(&it, c->kry_iters.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaMemcpyAsync(&res, c->kry_resid.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    int st = 0;
    TF_TRY(sync_status(c, &st));
    if (st) return set_err(c, st, "gmres: grid barrier watchdog fired");
    *max_iter = it >= 0 ? it : -it;
    *tol = res;
    return it >= 0 ? TF_OK : set_err(c, TF_ERR_NOT_CONVERGED, "gmres: no convergence within max_iter");
}

}  // namespace tf
