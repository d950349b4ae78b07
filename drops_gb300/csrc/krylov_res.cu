// Single-barrier Jacobi-PCG with each block's share of the system resident in
// shared memory (PCG of num/krylovsolver.h:107-189 in the Chronopoulos-Gear
// form of k_pcg_cg1, krylov.cu).
//
// k_pcg_cg1 waits on memory in every column step of its SELL walk: the
// column's 16-byte state {r, w, s, 1/d} is gathered through L1, and a warp's
// step lasts as long as its slowest lane, which often misses to L2.  Here
// block b owns the contiguous slot run [sb0, sb1) of the SELL matrix (equal
// column work, as in the blocked pass of k_pcg_cg1) for the whole solve, and
// a preprocessing kernel (once per pattern) lists the block's halo -- the
// rows of other blocks that its columns reference -- and translates each
// column of the run to a 16-bit index into the block's vector: its own slots
// first, then its halo rows.  Shared memory holds the translated columns, the
// run's values (as many as fit), the state, p and the correction dx of the
// block's rows.  Every pass then
//   1. forms u = (r - alpha (w + beta s)) / d for the block's rows and, from
//      the state gathered once from global memory, for its halo rows, into one
//      array (the halo loads are issued first, in one round);
//   2. walks its SELL run entirely in shared memory (column, value, u);
//   3. updates its rows, publishes their new state to the global double
//      buffer for the other blocks' halos, and joins the grid all-reduce.
// The owner and every halo reader evaluate u with the same operations, so all
// blocks use bitwise the same vector.
//
// T = float: the mixed-precision solver (FP32 iterations, the FP32 correction
// folded into the FP64 iterate at each refinement, refinement when the FP32
// residual has dropped by a factor 0.2 (TF_PCG_REL_UPDATE), claims
// convergence or max_iter is reached;
// convergence is decided on the FP64 residual b - A x).
// T = double: the FP64 solver on the same structure (32-byte state, FP64
// dots); it refines only when the recursive residual claims convergence or at
// max_iter, and then confirms convergence on the true residual b - A x.  The
// precomputed u keeps it at one FP64 multiply-add per stored entry (the
// on-the-fly u of k_pcg_cg1 would cost three more on GB300's narrow FP64 pipe).
//
// Applicability is decided on the host: every block's run (slot rows, halo,
// translated columns) must fit the shared memory and its vector 16-bit
// indices; otherwise the caller uses k_pcg_cg1 / the two-barrier FP64 kernel.
#include "krylov_dev.cuh"

namespace tf {

namespace {

constexpr int kResThreads = 512;
constexpr int kHaloMax = 4096;    // halo rows per block
constexpr int kHashSlots = 8192;  // open-addressing table of the halo preprocessing

struct alignas(32) Dstate {
    double x, y, z, w;
};
template <class T>
struct ResState;
template <>
struct ResState<float> {
    using V = float4;
};
template <>
struct ResState<double> {
    using V = Dstate;
};

__device__ __forceinline__ float4 st_ld(const float4* p) { return __ldca(p); }
__device__ __forceinline__ Dstate st_ld(const Dstate* p) {
    const double2 a = __ldca(reinterpret_cast<const double2*>(p)), b = __ldca(reinterpret_cast<const double2*>(p) + 1);
    return Dstate{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ void st_st(float4* p, float4 v) { *p = v; }
__device__ __forceinline__ void st_st(Dstate* p, Dstate v) {
    reinterpret_cast<double2*>(p)[0] = make_double2(v.x, v.y);
    reinterpret_cast<double2*>(p)[1] = make_double2(v.z, v.w);
}
__device__ __forceinline__ float4 mk_state(float r, float w, float s, float id) { return make_float4(r, w, s, id); }
__device__ __forceinline__ Dstate mk_state(double r, double w, double s, double id) { return Dstate{r, w, s, id}; }

__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// u_{i+1} of a row from its state {r_i, w_i, s_{i-1}, 1/d}; the owner's row
// update evaluates exactly this sequence
template <class T, class V>
__device__ __forceinline__ T res_u(const V& v, T al, T be) {
    const T s = fma_rn(be, v.z, v.y);
    const T r = fma_rn(-al, s, v.x);
    return mul_rn(r, v.w);
}

// n columns of one slot row: translated columns cp[32 k] (shared memory),
// values vp[32 k] (shared memory when vsh, else global), vector xs (shared
// memory).  Terms are summed in column order.
template <class T>
__device__ __forceinline__ T res_row(const uint16_t* __restrict__ cp, const T* __restrict__ vp, bool vsh, int32_t n,
                                     const T* __restrict__ xs) {
    constexpr int U = 8;
    T acc = T(0);
    for (int32_t k = 0; k < n; k += U) {
        T xv[U], vv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (k + u < n) {
                vv[u] = vsh ? vp[32 * (k + u)] : __ldg(vp + 32 * (k + u));
                xv[u] = xs[cp[32 * (k + u)]];
            } else {
                vv[u] = T(0);
                xv[u] = T(0);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (k + u < n) acc += vv[u] * xv[u];
    }
    return acc;
}

template <class T>
struct PcgResArgs {
    using V = typename ResState<T>::V;
    int64_t m, nslices;
    const int32_t* perm;
    const int32_t* ptr;
    const int32_t* col;
    const uint16_t* col_tr;    // SELL columns translated to the owning block's vector
    const int32_t* halo_rows;  // [block][kHaloMax]
    const int32_t* halo_n;     // [block]
    const T* val;              // SELL values in T
    const double* val64;       // SELL values in FP64 (true residual)
    const T* diag;
    const double* b;
    double* x;
    V* V0;
    V* V1;
    T* P;
    GridAR g;
    int max_iter;
    double tol;
    int rel;
    double rel_update;  // refine when the recursive residual dropped by this factor (0: never)
    int* out_iter;
    double* out_resid;
    int* out_updates;
    int smax;      // slices of the largest run: sizes the per-slot arrays
    int hmax;      // halo rows of the largest halo (a multiple of 8)
    int32_t ccap;  // translated column slots (>= the largest run, a multiple of 16)
    int32_t vcap;  // value slots kept in shared memory
};

// dynamic shared memory of one block, in this order (every part a multiple of 32 bytes):
// Vs[slots] state, Us[slots + hmax] u, Ps[slots + hmax] p, sdx[slots], wsm[slots], ssm[slots],
// sperm[slots], hrow[hmax], ccol[ccap] (16-bit), cval[vcap]
template <class T>
inline size_t res_fixed_bytes(int smax, int hmax, int32_t ccap) {
    using V = typename ResState<T>::V;
    const size_t slots = (size_t)smax * 32;
    return slots * (sizeof(V) + 5 * sizeof(T) + sizeof(int32_t)) + (size_t)hmax * (2 * sizeof(T) + sizeof(int32_t)) +
           (((size_t)ccap * 2 + 31) & ~(size_t)31);
}

template <class T>
__global__ void __launch_bounds__(kResThreads, 1) k_pcg_res(PcgResArgs<T> a) {
    using V = typename ResState<T>::V;
    constexpr int NW = kResThreads / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    extern __shared__ __align__(32) unsigned char res_dyn[];
    const size_t slots = (size_t)a.smax * 32;
    V* Vs = reinterpret_cast<V*>(res_dyn);
    T* Us = reinterpret_cast<T*>(Vs + slots);
    T* Ps = Us + slots + a.hmax;  // own slots: p; halo part: p of the halo rows (refresh)
    T* sdx = Ps + slots + a.hmax;
    T* wsm = sdx + slots;  // products A u; with ssm also the FP64 residual products
    T* ssm = wsm + slots;  // products A p (refresh)
    double* rres = reinterpret_cast<double*>(wsm);
    int32_t* sperm = reinterpret_cast<int32_t*>(ssm + slots);
    int32_t* hrow = sperm + slots;
    uint16_t* ccol = reinterpret_cast<uint16_t*>(hrow + a.hmax);
    T* cval = reinterpret_cast<T*>(reinterpret_cast<unsigned char*>(ccol) + (((size_t)a.ccap * 2 + 31) & ~(size_t)31));
    __shared__ BalShared<NW, T> bsh;
    __shared__ BalShared<NW, double> bshd;
    __shared__ double sh[4];

    unsigned long long epoch = 0;
    V* Vc = a.V0;
    V* Vn = a.V1;
    const int64_t sb0 = balanced_part_start(a.ptr, a.nslices, blockIdx.x, gridDim.x);
    const int64_t sb1 = balanced_part_start(a.ptr, a.nslices, blockIdx.x + 1, gridDim.x);
    const int S = (int)(sb1 - sb0);
    const int NS = S * 32;  // own slots; halo entries follow at NS + h
    const int32_t pb = __ldg(a.ptr + sb0), pe = __ldg(a.ptr + sb1);
    const int32_t nslot = pe - pb;
    const int nh = __ldg(a.halo_n + blockIdx.x);
    // the run: slot rows, halo rows, translated columns, leading values; p = dx = 0
    for (int k = threadIdx.x; k < NS; k += kResThreads) {
        sperm[k] = __ldg(a.perm + sb0 * 32 + k);
        Ps[k] = T(0);
        sdx[k] = T(0);
    }
    for (int h = threadIdx.x; h < nh; h += kResThreads) hrow[h] = __ldg(a.halo_rows + (size_t)blockIdx.x * kHaloMax + h);
    for (int32_t k = threadIdx.x; k < nslot; k += kResThreads) {
        ccol[k] = __ldg(a.col_tr + pb + k);
        if (k < a.vcap) cval[k] = __ldg(a.val + pb + k);
    }
    sell_block_plan<NW, T>(bsh, a.ptr, sb0, S);
    sell_block_plan<NW, double>(bshd, a.ptr, sb0, S);  // ends with a block barrier

    const int max_iter = a.max_iter;
    const double tol = a.tol;
    double normb = 1.0;
    int it = 0, updates = 0;
    bool converged = false;
    T gam = T(0), alpha = T(0), beta = T(0), thr_rel = T(0), thr_tol = T(0);

    // r = b - A x in FP64 over the block's rows (first: state {r, 0, 0, 1/d}, p = 0)
    auto true_residual = [&](bool first, bool& done) -> bool {
        const double* x = a.x;
        sell_block_walk<NW, double>(bshd, a.ptr, a.col, a.val64, sb0, S, [&](int32_t j) { return kld(x + j); },
                                    [&](int64_t s, double v) { rres[(s - sb0) * 32 + lane] = v; });
        double v[2] = {0., 0.};
        for (int i = wid; i < S; i += NW) {
            const int ls = i * 32 + lane;
            const int32_t row = sperm[ls];
            if (row >= 0) {
                const double bi = a.b[row];
                const double ri = bi - rres[ls];
                V vc;
                if (first) {
                    vc = mk_state((T)ri, T(0), T(0), T(1) / a.diag[row]);
                    a.P[row] = T(0);
                } else {
                    vc = Vs[ls];
                    vc.x = (T)ri;
                }
                Vs[ls] = vc;
                st_st(Vc + row, vc);
                v[0] += ri * ri;
                if (first) v[1] += bi * bi;
            }
        }
        double o[2];
        if (!grid_allreduce<double, 2>(a.g, epoch, v, o)) return false;
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
        const double r_last = sh[1], resid = sh[2];
        __syncthreads();
        ++updates;
        converged = resid <= tol;
        done = converged || it >= max_iter;
        thr_rel = (T)(a.rel_update * r_last);
        thr_tol = (T)(tol * normb);
        if (blockIdx.x == 0 && threadIdx.x == 0) *a.out_resid = resid;
        return true;
    };

    // one SpMV pass over the block's run; refresh: w = A (r / d) and s = A p
    // with r, p kept (after a true residual), else the CG step with (alpha, beta)
    auto pass = [&](bool refresh, T (&o)[6]) -> bool {
        T v[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
        const T al = refresh ? T(0) : alpha, be = refresh ? T(0) : beta;
        // u of the block's rows and of its halo, p of the halo on a refresh: the
        // halo states (global memory) are loaded first, kHaloRegs per thread at
        // once, and the block's own rows (shared memory) are done while they
        // are in flight (fewer at once for the 32-byte FP64 state: registers)
        constexpr int kHaloRegs = sizeof(T) == 4 ? 4 : 2;
        V hv[kHaloRegs];
        T hp[kHaloRegs];
#pragma unroll
        for (int q = 0; q < kHaloRegs; ++q) {
            const int h = threadIdx.x + q * kResThreads;
            if (h < nh) {
                const int32_t r = hrow[h];
                hv[q] = st_ld(Vc + r);
                if (refresh) hp[q] = kld(a.P + r);
            }
        }
        for (int t = threadIdx.x; t < NS; t += kResThreads) Us[t] = sperm[t] >= 0 ? res_u<T>(Vs[t], al, be) : T(0);
#pragma unroll
        for (int q = 0; q < kHaloRegs; ++q) {
            const int h = threadIdx.x + q * kResThreads;
            if (h < nh) {
                Us[NS + h] = res_u<T>(hv[q], al, be);
                if (refresh) Ps[NS + h] = hp[q];
            }
        }
        for (int h = threadIdx.x + kHaloRegs * kResThreads; h < nh; h += kResThreads) {
            const int32_t r = hrow[h];
            Us[NS + h] = res_u<T>(st_ld(Vc + r), al, be);
            if (refresh) Ps[NS + h] = kld(a.P + r);
        }
        __syncthreads();
        // the slice offsets of the run come from the plan in shared memory:
        // ptr[sb0 + i] - pb = 32 * bsh.P[i]
        auto walk = [&](const T* xs, T* out) {
            sell_block_walk_fn<NW, T>(
                bsh, sb0, S,
                [&](int64_t s, int32_t c0, int32_t n) {
                    const int i = (int)(s - sb0);
                    const int32_t p0 = 32 * (bsh.P[i] + c0) + lane;
                    const bool vsh = 32 * bsh.P[i + 1] <= a.vcap;
                    return res_row<T>(ccol + p0, vsh ? cval + p0 : a.val + pb + p0, vsh, n, xs);
                },
                [&](int64_t s, T val) { out[(s - sb0) * 32 + lane] = val; });
        };
        walk(Us, wsm);
        if (refresh) walk(Ps, ssm);  // s = A p recomputed, ending the drift of its recurrence
        for (int i = wid; i < S; i += NW) {
            const int ls = i * 32 + lane;
            const int32_t row = sperm[ls];
            if (row >= 0) {
                const V vc = Vs[ls];
                T sn, rn, pn;
                if (refresh) {
                    sn = ssm[ls];
                    rn = vc.x;
                    pn = Ps[ls];
                } else {
                    sn = fma_rn(be, vc.z, vc.y);
                    rn = fma_rn(-al, sn, vc.x);
                    pn = fma_rn(be, Ps[ls], mul_rn(vc.x, vc.w));
                    Ps[ls] = pn;
                    sdx[ls] = fma_rn(al, pn, sdx[ls]);
                }
                const T un = mul_rn(rn, vc.w), wn = wsm[ls];
                const V nv = mk_state(rn, wn, sn, vc.w);
                Vs[ls] = nv;
                st_st(Vn + row, nv);
                v[0] += rn * un;
                v[1] += un * wn;
                v[2] += un * sn;
                v[3] += pn * wn;
                v[4] += pn * sn;
                v[5] += rn * rn;
            }
        }
        if (!grid_allreduce<T, 6>(a.g, epoch, v, o)) return false;
        V* t = Vc;
        Vc = Vn;
        Vn = t;
        return true;
    };

    // FP64 fold of the correction into x, p published for the refresh pass
    auto fold = [&]() -> bool {
        for (int i = wid; i < S; i += NW) {
            const int ls = i * 32 + lane;
            const int32_t row = sperm[ls];
            if (row >= 0) {
                a.x[row] += (double)sdx[ls];
                sdx[ls] = T(0);
                a.P[row] = Ps[ls];
            }
        }
        return grid_sync_ar(a.g, epoch);
    };

    bool done = false;
    if (!true_residual(true, done)) return;
    bool first = true;
    while (!done) {
        T o[6];
        if (!pass(true, o)) return;
        beta = first ? T(0) : o[0] / gam;
        first = false;
        gam = o[0];
        alpha = gam / (o[1] + beta * (o[2] + o[3]) + beta * beta * o[4]);
        bool refine = false;
        while (!refine) {
            if (!pass(false, o)) return;
            ++it;
            const T rn = sqrt(o[5]);
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
        *a.out_updates = updates;
    }
}

__global__ void k_res_diag32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

__global__ void k_sell_iperm(int64_t nslots, const int32_t* __restrict__ perm, int32_t* __restrict__ iperm) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nslots; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = perm[i];
        if (r >= 0) iperm[r] = (int32_t)i;
    }
}

// Per part b of the balanced partition (one block each): the halo rows (the
// distinct columns of the run whose slots lie outside it, numbered in the
// order of an open-addressing table of kHashSlots entries -- deterministic:
// the table's content does not depend on insertion order, and the numbering
// is a scan over its slots) and the run's columns translated to the block's
// vector (own slot, or NS + halo number).  info[0]: set when a table or a
// halo overflows or an index needs more than 16 bits; info[1]: largest run
// in slices, info[2]: largest run in slots, info[3]: largest halo.
__device__ __forceinline__ uint32_t halo_hash(int32_t c) { return ((uint32_t)c * 2654435761u) >> 19; }  // 13 bits
static_assert(kHashSlots == 1 << 13, "hash width");

__global__ void __launch_bounds__(512) k_res_halo(const int32_t* __restrict__ ptr, int64_t nslices,
                                                  const int32_t* __restrict__ col, const int32_t* __restrict__ iperm,
                                                  uint16_t* __restrict__ col_tr, int32_t* __restrict__ halo_rows,
                                                  int32_t* __restrict__ halo_n, int* __restrict__ info) {
    extern __shared__ int32_t hsh[];  // keys[kHashSlots], ids[kHashSlots]
    int32_t* keys = hsh;
    int32_t* ids = hsh + kHashSlots;
    __shared__ int32_t wsum[16];
    __shared__ int bad;
    const int64_t sb0 = balanced_part_start(ptr, nslices, blockIdx.x, gridDim.x);
    const int64_t sb1 = balanced_part_start(ptr, nslices, blockIdx.x + 1, gridDim.x);
    const int NS = (int)(sb1 - sb0) * 32;
    const int32_t lo = (int32_t)(sb0 * 32), hi = (int32_t)(sb1 * 32);
    const int32_t pb = ptr[sb0], pe = ptr[sb1];
    for (int i = threadIdx.x; i < kHashSlots; i += blockDim.x) keys[i] = -1;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int32_t k = pb + threadIdx.x; k < pe; k += blockDim.x) {
        const int32_t c = col[k];
        const int32_t sl = iperm[c];
        if (sl >= lo && sl < hi) continue;
        uint32_t h = halo_hash(c);
        int probe = 0;
        for (; probe < kHashSlots; ++probe) {
            const int32_t old = atomicCAS(&keys[h], -1, c);
            if (old == -1 || old == c) break;
            h = (h + 1) & (kHashSlots - 1);
        }
        if (probe == kHashSlots) bad = 1;
    }
    __syncthreads();
    // number the occupied table entries in slot order (block scan, 16 entries per thread)
    constexpr int kPer = kHashSlots / 512;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    int cnt = 0;
    for (int q = 0; q < kPer; ++q) cnt += keys[t * kPer + q] >= 0;
    int inc = cnt;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    int base = 0;
    for (int q = 0; q < w; ++q) base += wsum[q];
    int id = base + inc - cnt;
    for (int q = 0; q < kPer; ++q) {
        const int i = t * kPer + q;
        if (keys[i] >= 0) {
            ids[i] = id;
            if (id < kHaloMax) halo_rows[(size_t)blockIdx.x * kHaloMax + id] = keys[i];
            ++id;
        }
    }
    __syncthreads();
    int nh = 0;
    for (int q = 0; q < 16; ++q) nh += wsum[q];
    if (nh > kHaloMax || NS + nh > 65535) bad = 1;
    __syncthreads();
    if (!bad) {
        for (int32_t k = pb + threadIdx.x; k < pe; k += blockDim.x) {
            const int32_t c = col[k];
            const int32_t sl = iperm[c];
            int32_t tr;
            if (sl >= lo && sl < hi) {
                tr = sl - lo;
            } else {
                uint32_t h = halo_hash(c);
                while (keys[h] != c) h = (h + 1) & (kHashSlots - 1);  // present: inserted above
                tr = NS + ids[h];
            }
            col_tr[k] = (uint16_t)tr;
        }
    }
    if (threadIdx.x == 0) {
        halo_n[blockIdx.x] = nh;
        if (bad) atomicOr(info, 1);
        atomicMax(info + 1, (int)(sb1 - sb0));
        atomicMax(info + 2, pe - pb);
        atomicMax(info + 3, nh);
    }
}

int mat_slot(Context* c, const CSR& A) {
    for (int i = 0; i < TF_NUM_MATS; ++i)
        if (&c->mats[i] == &A) return i;
    return 0;
}

// row -> slot map, halo lists and translated columns, once per pattern and grid
int ensure_res_plan(Context* c, CSR& A, int blocks) {
    Sell& S = A.sell;
    const int id = mat_slot(c, A);
    if (S.iperm_gen != S.pattern_gen || !S.iperm) {
        TF_TRY(ensure(c, c->sell_iperm[id], (size_t)(A.m > 0 ? A.m : 1)));
        S.iperm = c->sell_iperm[id].p;
        k_sell_iperm<<<grid_for(c, S.nslices * 32), kBlock, 0, c->stream>>>(S.nslices * 32, S.perm, S.iperm);
        ++c->launches;
        TF_CUDA(c, cudaGetLastError());
        S.iperm_gen = S.pattern_gen;
        S.res_blocks = 0;
    }
    if (S.res_blocks != blocks) {
        TF_TRY(ensure(c, c->sell_coltr[id], (size_t)(S.npad > 0 ? S.npad : 1)));
        TF_TRY(ensure(c, c->sell_halo[id], (size_t)blocks * kHaloMax + blocks));
        S.col_tr = c->sell_coltr[id].p;
        S.halo_rows = c->sell_halo[id].p;
        S.halo_n = c->sell_halo[id].p + (size_t)blocks * kHaloMax;
        TF_TRY(ensure(c, c->kry_iters, 4));
        TF_CUDA(c, cudaMemsetAsync(c->kry_iters.p, 0, 4 * sizeof(int), c->stream));
        const size_t hsm = 2 * sizeof(int32_t) * kHashSlots;
        TF_CUDA(c, cudaFuncSetAttribute((const void*)k_res_halo, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hsm));
        k_res_halo<<<blocks, 512, hsm, c->stream>>>(S.ptr, S.nslices, S.col, S.iperm, S.col_tr, S.halo_rows, S.halo_n,
                                                    c->kry_iters.p);
        ++c->launches;
        TF_CUDA(c, cudaGetLastError());
        int h[4] = {0, 0, 0, 0};
        TF_CUDA(c, cudaMemcpyAsync(h, c->kry_iters.p, 4 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        TF_CUDA(c, cudaStreamSynchronize(c->stream));
        S.res_ok = h[0] == 0;
        S.res_smax = h[1];
        S.res_maxslots = h[2];
        S.res_hmax = (h[3] + 7) & ~7;
        S.res_blocks = blocks;
    }
    return TF_OK;
}

}  // namespace

// Resident single-barrier PCG; *applied = false (nothing launched) when a
// block's run does not fit the shared memory.
template <class T>
int pcg_resident(Context* c, CSR& A, const double* b, double* x, int* max_iter, double* tol, int rel, bool* applied) {
    using V = typename ResState<T>::V;
    *applied = false;
    const int64_t m = A.m;
    const void* fn = (const void*)k_pcg_res<T>;
    const int blocks = c->num_sms;  // one 512-thread block per SM
    TF_TRY(ensure_res_plan(c, A, blocks));
    const Sell& S = A.sell;
    if (!S.res_ok || S.res_smax <= 0 || S.res_smax > kBalMaxSlices) return TF_OK;
    cudaFuncAttributes fa{};
    int optin = 0;
    TF_CUDA(c, cudaFuncGetAttributes(&fa, fn));
    TF_CUDA(c, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    const int64_t room = (int64_t)optin - (int64_t)fa.sharedSizeBytes - 1024;
    const int32_t ccap = (S.res_maxslots + 15) & ~15;
    const int64_t fixed = (int64_t)res_fixed_bytes<T>(S.res_smax, S.res_hmax, ccap);
    if (fixed > room) return TF_OK;
    int32_t vcap = (int32_t)std::min<int64_t>((room - fixed) / (int64_t)sizeof(T), (int64_t)ccap) & ~7;
    if (c->pcg_res_vcap_kb >= 0)
        vcap = std::min<int32_t>(vcap, (int32_t)(((int64_t)c->pcg_res_vcap_kb * 1024 / (int64_t)sizeof(T)) & ~7));
    const size_t dyn = (size_t)fixed + (size_t)vcap * sizeof(T);
    TF_CUDA(c, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    int per_sm = 0;
    TF_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kResThreads, dyn));
    if (per_sm < 1) return TF_OK;

    // workspace: V0, V1 (m states each), p (m), T diagonal (m)
    const T* diag = nullptr;
    V* V0 = nullptr;
    T* P = nullptr;
    if constexpr (sizeof(T) == 4) {
        TF_TRY(ensure(c, c->kry32, (size_t)(10 * m)));
        float* base = c->kry32.p;
        k_res_diag32<<<grid_for(c, m), kBlock, 0, c->stream>>>(m, A.diag, base + 9 * m);
        ++c->launches;
        V0 = reinterpret_cast<V*>(base);
        P = base + 8 * m;
        diag = base + 9 * m;
    } else {
        TF_TRY(ensure(c, c->kry64, (size_t)(9 * m)));
        double* base = c->kry64.p;
        V0 = reinterpret_cast<V*>(base);
        P = base + 8 * m;
        diag = A.diag;
    }
    const size_t part_d = (size_t)2 * blocks * kArMax;
    TF_TRY(ensure(c, c->kry_part, part_d + (part_d + 1) / 2 + 16));
    TF_TRY(ensure(c, c->kry_bar, 2));
    TF_TRY(ensure(c, c->kry_iters, 4));
    TF_TRY(ensure(c, c->kry_resid, 1));
    TF_CUDA(c, cudaMemsetAsync(c->kry_bar.p, 0, 2 * sizeof(unsigned), c->stream));
    TF_CUDA(c, cudaMemsetAsync(c->status.p, 0, 4 * sizeof(int), c->stream));
    PcgResArgs<T> g;
    g.m = m;
    g.nslices = S.nslices;
    g.perm = S.perm;
    g.ptr = S.ptr;
    g.col = S.col;
    g.col_tr = S.col_tr;
    g.halo_rows = S.halo_rows;
    g.halo_n = S.halo_n;
    if constexpr (sizeof(T) == 4) g.val = S.v32;
    else g.val = S.v64;
    g.val64 = S.v64;
    g.diag = diag;
    g.b = b;
    g.x = x;
    g.V0 = V0;
    g.V1 = V0 + m;
    g.P = P;
    g.g.count = reinterpret_cast<unsigned long long*>(c->kry_bar.p);
    g.g.partd = c->kry_part.p;
    g.g.partf = reinterpret_cast<float*>(c->kry_part.p + part_d);
    g.g.status = c->status.p;
    g.max_iter = *max_iter;
    g.tol = *tol;
    g.rel = rel;
    g.rel_update = sizeof(T) == 4 ? c->pcg_rel_update : 0.0;
    g.out_iter = c->kry_iters.p;
    g.out_resid = c->kry_resid.p;
    g.out_updates = c->kry_iters.p + 1;
    g.smax = S.res_smax;
    g.hmax = S.res_hmax;
    g.ccap = ccap;
    g.vcap = vcap;
    void* args[] = {&g};
    TF_CUDA(c, cudaLaunchCooperativeKernel(fn, blocks, kResThreads, args, dyn, c->stream));
    ++c->launches;
    *applied = true;
    int it[2] = {0, 0};
    double res = 0;
    TF_CUDA(c, cudaMemcpyAsync(it, c->kry_iters.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaMemcpyAsync(&res, c->kry_resid.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    int st = 0;
    TF_TRY(sync_status(c, &st));
    if (st) return set_err(c, st, "pcg (resident): grid barrier watchdog fired");
    c->last_refinements = it[1];
    *max_iter = it[0] >= 0 ? it[0] : -1 - it[0];
    *tol = res;
    return it[0] >= 0 ? TF_OK : set_err(c, TF_ERR_NOT_CONVERGED, "pcg: no convergence within max_iter");
}

template int pcg_resident<float>(Context*, CSR&, const double*, double*, int*, double*, int, bool*);
template int pcg_resident<double>(Context*, CSR&, const double*, double*, int*, double*, int, bool*);

}  // namespace tf
