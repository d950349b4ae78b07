// Narrow-band refinement on the device: the algorithm of refine.cu (DROPS's
// MakeInitialTriang over MultiGridCL::Refine) as level-synchronous data-
// parallel passes, with the same results bit for bit.
//
// Every step of MultiGridCL::Refine that walks a level's tet list in order
// has per-tet effects that do not depend on that order, except where new
// objects are created:
//   - marks (DistMarkingStrategyCL::visit), RestrictMark and Close write the
//     tet's own mark or its children's; commits add to edge counters
//     (atomics; RestrictMark reads only counters of the next level, which
//     commits of this level do not touch);
//   - UnrefineGrid's removal marks and rescues only clear flags;
//   - RefineGrid creates midvertices and sub-edges (one creator per split
//     edge: a pass over the flagged edges), inner edges shared by the two tets
//     of a face (a two-phase hash: keys inserted by the tets, ids assigned by a
//     pass over the table, then looked up), and children, which are appended
//     to the next level's list in parent order and rule order: an exclusive
//     scan of the new-children counts in list order gives every child its
//     place.
// Removed tets leave the list by a stable compaction.  Vertex and edge ids
// are allocation order (atomics) and carry no meaning: the output is
// renumbered by scans, and the DOF numbering downstream is first touch in tet
// order.
//
// Each kernel body is a __host__ __device__ lambda run by par_for, either as
// a grid-stride kernel on the context's stream or as a plain loop on the host
// (the host form checks the same code against the reference's fixtures
// without a device).  Every table probe and every allocation is bounded and
// reports overflow through an error counter instead of writing past a buffer.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <numeric>
#include <vector>

#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>

#include "tf_internal.cuh"

extern "C" int tf_refine_rules(int32_t* nch, int32_t* children);

namespace tf {
namespace rpar {

constexpr uint8_t kNoRef = 0, kRegRef = 63, kGreen = 127, kRemove = 64;
constexpr uint64_t kEmpty = ~0ull;

struct DRule {
    int nch;
    uint8_t ch[8][4];
    int nin;            // inner edges: pairs of local points that are neither edges of the parent nor halves of one
    uint8_t in[32][2];  // oriented by the point order 0,4,1,5,6,2,7,8,9,3
};

__host__ __device__ inline int rank_of(int p) {
    const int r[10] = {0, 2, 5, 9, 1, 3, 4, 6, 7, 8};
    return r[p];
}
__host__ __device__ inline int edge_of(int a, int b) {
    if (a > b) {
        const int t = a;
        a = b;
        b = t;
    }
    for (int e = 0; e < 6; ++e)
        if (ev0(e) == a && ev1(e) == b) return e;
    return -1;
}

// ---- host/device primitives ------------------------------------------------
__host__ __device__ inline int32_t atom_add(int32_t* p, int32_t v) {
#ifdef __CUDA_ARCH__
    return atomicAdd(p, v);
#else
    const int32_t o = *p;
    *p += v;
    return o;
#endif
}
__host__ __device__ inline uint64_t atom_cas(uint64_t* p, uint64_t cmp, uint64_t val) {
#ifdef __CUDA_ARCH__
    return (uint64_t)atomicCAS((unsigned long long*)p, (unsigned long long)cmp, (unsigned long long)val);
#else
    const uint64_t o = *p;
    if (o == cmp) *p = val;
    return o;
#endif
}
__host__ __device__ inline void atom_min(int64_t* p, int64_t v) {
#ifdef __CUDA_ARCH__
    atomicMin((long long*)p, (long long)v);
#else
    if (v < *p) *p = v;
#endif
}
__host__ __device__ inline uint32_t hmix(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return (uint32_t)k;
}
__host__ __device__ inline uint64_t ekey(int32_t a, int32_t b) { return (uint64_t)(uint32_t)a << 32 | (uint32_t)b; }

template <class F>
__global__ void k_for(int64_t n, F f) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        f(i);
}

struct Exec {
    bool dev = false;
    cudaStream_t s = nullptr;
    cudaMemPool_t pool = nullptr;  // stream-ordered device allocations, when set
    int nsm = 1;
    int err = 0;  // host-side CUDA error
    template <class F>
    void par_for(int64_t n, F f) {
        if (n <= 0) return;
        if (dev) {
            int64_t g = (n + 255) / 256;
            g = std::min<int64_t>(g, (int64_t)nsm * 8);
            k_for<<<(int)std::max<int64_t>(g, 1), 256, 0, s>>>(n, f);
            if (cudaGetLastError() != cudaSuccess) err = 1;
        } else {
            for (int64_t i = 0; i < n; ++i) f(i);
        }
    }
};

// Device buffers come from the executor's memory pool when it has one: the
// allocation and the free are ordered on the stream (no synchronisation), and
// the pool keeps freed memory for the next allocation and the next call.
template <class T>
struct Buf {
    T* p = nullptr;
    int64_t cap = 0;
    bool dev = false;
    bool pooled = false;  // p came from X->pool
    Exec* X = nullptr;
    // grows to at least n elements, keeping the first keep
    bool grow(int64_t n, int64_t keep) {
        if (n <= cap) return true;
        int64_t nc = std::max<int64_t>(n, cap + cap / 2 + 1024);
        T* q = nullptr;
        if (dev) {
            const bool from_pool = X->pool != nullptr;
            if (from_pool) {
                if (cudaMallocFromPoolAsync((void**)&q, sizeof(T) * nc, X->pool, X->s) != cudaSuccess) return false;
            } else if (cudaMalloc((void**)&q, sizeof(T) * nc) != cudaSuccess) {
                return false;
            }
            if (keep > 0 && cudaMemcpyAsync(q, p, sizeof(T) * keep, cudaMemcpyDeviceToDevice, X->s) != cudaSuccess) {
                if (from_pool)
                    cudaFreeAsync(q, X->s);
                else
                    cudaFree(q);
                return false;
            }
            free_dev();
            pooled = from_pool;
        } else {
            q = (T*)std::malloc(sizeof(T) * nc);
            if (!q) return false;
            if (keep > 0) std::memcpy(q, p, sizeof(T) * keep);
            std::free(p);
        }
        p = q;
        cap = nc;
        return true;
    }
    void free_dev() {
        if (!p) return;
        if (pooled) {
            cudaFreeAsync(p, X->s);
        } else {
            cudaStreamSynchronize(X->s);
            cudaFree(p);
        }
    }
    void release() {
        if (p) {
            if (dev)
                free_dev();
            else
                std::free(p);
        }
        p = nullptr;
        cap = 0;
        pooled = false;
    }
    void fill(int64_t n, T v) {
        T* q = p;
        X->par_for(n, [=] __host__ __device__(int64_t i) { q[i] = v; });
    }
};

// ---- distance functions (the device level sets' expressions) -------------
struct DistPar {
    int kind;
    double p[16];
};
__host__ __device__ inline double dist(const DistPar& D, const double x[3]) {
    if (D.kind == TF_LS_SPHERE) {
        const double a = x[0] - D.p[0], b = x[1] - D.p[1], c = x[2] - D.p[2];
        return sqrt(a * a + b * b + c * c) - D.p[3];
    }
    if (D.kind == TF_LS_TORUS) {
        const int ax = (int)D.p[2];
        const int a0 = (ax + 1) % 3, a1 = (ax + 2) % 3;
        const double rho = sqrt(x[a0] * x[a0] + x[a1] * x[a1]) - D.p[0];
        return sqrt(rho * rho + x[ax] * x[ax]) - D.p[1];
    }
    return ((D.p[0] * x[0] + D.p[1] * x[1]) + D.p[2] * x[2]) - D.p[3];
}

// raw view of the multigrid
struct View {
    int32_t *tv, *te, *tlev, *tpar, *tch;
    int8_t* tnch;
    uint8_t *trule, *tmark, *tchg;
    int32_t *ev, *elev, *emfr, *emid, *esub;
    uint8_t *erm, *ealive, *esplit;
    double* vx;
    int32_t* vlev;
    uint8_t *vrm, *valive;
    uint64_t* hkey;
    int32_t* hval;
    uint32_t hmask;
    int32_t* cnt;  // 0 vertices, 1 edges, 2 error, 3 modified
    const DRule* rules;
    int64_t capv, cape;
};

__host__ __device__ inline void seterr(const View& V, int code) { V.cnt[2] = code; }

// insert (key, val); val < 0 inserts the key only.  Returns the slot or -1.
__host__ __device__ inline int64_t h_insert(const View& V, uint64_t key, int32_t val) {
    uint32_t i = hmix(key) & V.hmask;
    for (uint32_t probe = 0; probe <= V.hmask; ++probe, i = (i + 1) & V.hmask) {
        const uint64_t prev = atom_cas(&V.hkey[i], kEmpty, key);
        if (prev == kEmpty || prev == key) {
            if (val >= 0) V.hval[i] = val;
            return i;
        }
    }
    seterr(V, 3);
    return -1;
}
__host__ __device__ inline int32_t h_find(const View& V, uint64_t key) {
    uint32_t i = hmix(key) & V.hmask;
    for (uint32_t probe = 0; probe <= V.hmask; ++probe, i = (i + 1) & V.hmask) {
        const uint64_t k = V.hkey[i];
        if (k == key) return V.hval[i];
        if (k == kEmpty) return -1;
    }
    return -1;
}
__host__ __device__ inline bool is_regular(const View& V, int32_t t) {
    return V.tlev[t] == 0 || V.trule[V.tpar[t]] == kRegRef;
}
__host__ __device__ inline int32_t vert_mid(const View& V, int32_t t, int p) {
    return p < 4 ? V.tv[4 * (int64_t)t + p] : V.emid[V.te[6 * (int64_t)t + p - 4]];
}

// ---- the engine --------------------------------------------------------------
struct Engine {
    Exec X;
    Buf<int32_t> tv, te, tlev, tpar, tch, ev, elev, emfr, emid, esub, vlev, cnt, tmp32, hval, sel_n;
    Buf<int64_t> tmp64;
    Buf<int8_t> tnch;
    Buf<uint8_t> trule, tmark, tchg, erm, ealive, esplit, vrm, valive, flag8;
    Buf<double> vx;
    Buf<uint64_t> hkey;
    Buf<DRule> rules;
    Buf<unsigned char> cub_tmp;
    std::vector<Buf<int32_t>> tl;  // per-level tet lists
    std::vector<int64_t> tln;      // their lengths
    int64_t nv = 0, ne = 0, nt = 0, tcap = 0;
    uint32_t hcap = 0;
    bool ok = true;

    template <class T>
    void setup(Buf<T>& b) {
        b.dev = X.dev;
        b.X = &X;
    }
    Engine(bool dev, cudaStream_t s, int nsm, cudaMemPool_t pool = nullptr) {
        X.dev = dev;
        X.s = s;
        X.pool = dev ? pool : nullptr;
        X.nsm = nsm;
        if (dev && cudaMallocHost(&pin, kPinBytes) != cudaSuccess) {
            pin = nullptr;  // unstaged copies still work
            cudaGetLastError();
        }
        setup(tv), setup(te), setup(tlev), setup(tpar), setup(tch), setup(ev), setup(elev), setup(emfr), setup(emid);
        setup(esub), setup(vlev), setup(cnt), setup(tmp32), setup(hval), setup(tmp64), setup(tnch), setup(trule);
        setup(sel_n);
        setup(tmark), setup(tchg), setup(erm), setup(ealive), setup(esplit), setup(vrm), setup(valive);
        setup(flag8), setup(vx), setup(hkey), setup(rules), setup(cub_tmp);
    }
    ~Engine() {
        if (pin) cudaFreeHost(pin);
        tv.release(), te.release(), tlev.release(), tpar.release(), tch.release(), ev.release(), elev.release();
        emfr.release(), emid.release(), esub.release(), vlev.release(), cnt.release(), tmp32.release();
        sel_n.release();
        hval.release(), tmp64.release(), tnch.release(), trule.release(), tmark.release(), tchg.release();
        erm.release(), ealive.release(), esplit.release(), vrm.release(), valive.release(), flag8.release();
        vx.release(), hkey.release(), rules.release(), cub_tmp.release();
        for (auto& l : tl) l.release();
    }
    View view() {
        View V;
        V.tv = tv.p, V.te = te.p, V.tlev = tlev.p, V.tpar = tpar.p, V.tch = tch.p, V.tnch = tnch.p;
        V.trule = trule.p, V.tmark = tmark.p, V.tchg = tchg.p;
        V.ev = ev.p, V.elev = elev.p, V.emfr = emfr.p, V.emid = emid.p, V.esub = esub.p;
        V.erm = erm.p, V.ealive = ealive.p, V.esplit = esplit.p;
        V.vx = vx.p, V.vlev = vlev.p, V.vrm = vrm.p, V.valive = valive.p;
        V.hkey = hkey.p, V.hval = hval.p, V.hmask = hcap ? hcap - 1 : 0;
        V.cnt = cnt.p, V.rules = rules.p;
        V.capv = std::min({vx.cap / 3, vlev.cap, vrm.cap, valive.cap});
        V.cape = std::min({ev.cap / 2, elev.cap, emfr.cap, emid.cap, esub.cap / 2, erm.cap, ealive.cap, esplit.cap});
        return V;
    }
    // Host copies of device values, synchronous.  Small ones (the counts read
    // before each creating pass) go through a pinned staging buffer: a copy
    // from or to pageable memory would pass through the driver's own staging.
    static constexpr size_t kPinBytes = 256;
    void* pin = nullptr;
    void get(void* dst, const void* src, size_t bytes) {
        if (X.dev) {
            const bool staged = pin && bytes <= kPinBytes;
            if (cudaMemcpyAsync(staged ? pin : dst, src, bytes, cudaMemcpyDeviceToHost, X.s) != cudaSuccess ||
                cudaStreamSynchronize(X.s) != cudaSuccess)
                ok = false;
            else if (staged)
                std::memcpy(dst, pin, bytes);
        } else {
            std::memcpy(dst, src, bytes);
        }
    }
    void put(void* dst, const void* src, size_t bytes) {
        if (X.dev) {
            const bool staged = pin && bytes <= kPinBytes;
            if (staged) std::memcpy(pin, src, bytes);
            if (cudaMemcpyAsync(dst, staged ? pin : src, bytes, cudaMemcpyHostToDevice, X.s) != cudaSuccess ||
                cudaStreamSynchronize(X.s) != cudaSuccess)
                ok = false;
        } else {
            std::memcpy(dst, src, bytes);
        }
    }
    int32_t counter(int i) {
        int32_t v = 0;
        get(&v, cnt.p + i, sizeof v);
        return v;
    }
    void set_counter(int i, int32_t v) { put(cnt.p + i, &v, sizeof v); }

    bool grow_tets(int64_t n) {
        if (n <= tcap) return true;
        const int64_t k = nt;
        bool r = tv.grow(4 * n, 4 * k) && te.grow(6 * n, 6 * k) && tlev.grow(n, k) && tpar.grow(n, k) &&
                 tch.grow(8 * n, 8 * k) && tnch.grow(n, k) && trule.grow(n, k) && tmark.grow(n, k) && tchg.grow(n, k);
        tcap = std::min({tv.cap / 4, te.cap / 6, tlev.cap, tpar.cap, tch.cap / 8, tnch.cap, trule.cap, tmark.cap,
                         tchg.cap});
        return r;
    }
    bool grow_edges(int64_t n) {
        const int64_t k = ne;
        return ev.grow(2 * n, 2 * k) && elev.grow(n, k) && emfr.grow(n, k) && emid.grow(n, k) &&
               esub.grow(2 * n, 2 * k) && erm.grow(n, k) && ealive.grow(n, k) && esplit.grow(n, k);
    }
    bool grow_verts(int64_t n) {
        const int64_t k = nv;
        return vx.grow(3 * n, 3 * k) && vlev.grow(n, k) && vrm.grow(n, k) && valive.grow(n, k);
    }
    void sync_counts_to_dev() {
        int32_t c[2] = {(int32_t)nv, (int32_t)ne};
        put(cnt.p, c, sizeof c);
    }
    void sync_counts_from_dev() {
        int32_t c[2];
        get(c, cnt.p, sizeof c);
        nv = c[0], ne = c[1];
    }
    int last() const { return (int)tl.size() - 1; }
    void append_level() {
        tl.emplace_back();
        setup(tl.back());
        tln.push_back(0);
    }

    // exclusive scan of n int32 counts into tmp64 (n + 1 entries); in must hold
    // n + 1 entries (the last is overwritten with 0).  Returns the total.
    int64_t scan(int32_t* in, int64_t n) {
        if (!tmp64.grow(n + 1, 0)) {
            ok = false;
            return 0;
        }
        int64_t total = 0;
        if (X.dev) {
            if (cudaMemsetAsync(in + n, 0, sizeof(int32_t), X.s) != cudaSuccess) ok = false;
            size_t bytes = 0;
            cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, tmp64.p, (int)(n + 1), X.s);
            if (!cub_tmp.grow((int64_t)bytes + 1, 0)) {
                ok = false;
                return 0;
            }
            if (cub::DeviceScan::ExclusiveSum(cub_tmp.p, bytes, in, tmp64.p, (int)(n + 1), X.s) != cudaSuccess)
                ok = false;
            get(&total, tmp64.p + n, sizeof total);
        } else {
            for (int64_t i = 0; i < n; ++i) {
                tmp64.p[i] = total;
                total += in[i];
            }
            tmp64.p[n] = total;
        }
        return total;
    }
    // stable selection of src[i] with flag8[i] != 0 into dst; returns the count
    int64_t select(const int32_t* src, int64_t n, int32_t* dst) {
        if (X.dev) {
            if (!sel_n.grow(1, 0)) {
                ok = false;
                return 0;
            }
            size_t bytes = 0;
            cub::DeviceSelect::Flagged(nullptr, bytes, src, flag8.p, dst, sel_n.p, (int)n, X.s);
            if (!cub_tmp.grow((int64_t)bytes + 1, 0)) {
                ok = false;
                return 0;
            }
            if (cub::DeviceSelect::Flagged(cub_tmp.p, bytes, src, flag8.p, dst, sel_n.p, (int)n, X.s) != cudaSuccess)
                ok = false;
            int32_t k = 0;
            get(&k, sel_n.p, sizeof k);
            return k;
        }
        int64_t k = 0;
        for (int64_t i = 0; i < n; ++i)
            if (flag8.p[i]) dst[k++] = src[i];
        return k;
    }

    // ---- level 0 -------------------------------------------------------------
    // tets (nt0 x 4 vertices) and their edge ids (nt0 x 6) of one mesh, ne0 edges
    bool init(int64_t nv0, const double* coords, int64_t nt0, const int32_t* tv0, const int32_t* te0, int64_t ne0,
              const std::vector<DRule>& R) {
        if (!grow_verts(nv0) || !grow_edges(ne0) || !grow_tets(nt0) || !cnt.grow(8, 0) || !rules.grow(64, 0))
            return false;
        put(rules.p, R.data(), sizeof(DRule) * 64);
        put(vx.p, coords, sizeof(double) * 3 * nv0);
        put(tv.p, tv0, sizeof(int32_t) * 4 * nt0);
        put(te.p, te0, sizeof(int32_t) * 6 * nt0);
        nv = nv0, ne = ne0, nt = nt0;
        int32_t c[8] = {(int32_t)nv, (int32_t)ne, 0, 0, 0, 0, 0, 0};
        put(cnt.p, c, sizeof c);
        View V = view();
        X.par_for(nv, [=] __host__ __device__(int64_t v) {
            V.vlev[v] = 0;
            V.vrm[v] = 0;
            V.valive[v] = 1;
        });
        X.par_for(ne, [=] __host__ __device__(int64_t e) {
            V.ev[2 * e] = -1;
            V.elev[e] = 0;
            V.emfr[e] = 0;
            V.emid[e] = -1;
            V.esub[2 * e] = V.esub[2 * e + 1] = -1;
            V.erm[e] = 0;
            V.ealive[e] = 1;
            V.esplit[e] = 0;
        });
        X.par_for(nt, [=] __host__ __device__(int64_t t) {
            V.tlev[t] = 0;
            V.tpar[t] = -1;
            V.tnch[t] = 0;
            V.trule[t] = kNoRef;
            V.tmark[t] = kNoRef;
            V.tchg[t] = 0;
            for (int j = 0; j < 6; ++j) {
                const int32_t e = V.te[6 * t + j];
                V.ev[2 * (int64_t)e] = V.tv[4 * t + ev0(j)];  // every tet writes the same pair when oriented
                V.ev[2 * (int64_t)e + 1] = V.tv[4 * t + ev1(j)];
            }
        });
        // orientation check: every tet must see each of its edges in the edge's direction
        X.par_for(nt, [=] __host__ __device__(int64_t t) {
            for (int j = 0; j < 6; ++j) {
                const int32_t e = V.te[6 * t + j];
                if (V.ev[2 * (int64_t)e] != V.tv[4 * t + ev0(j)] || V.ev[2 * (int64_t)e + 1] != V.tv[4 * t + ev1(j)])
                    seterr(V, 4);
            }
        });
        append_level();
        if (!tl[0].grow(nt, 0)) return false;
        int32_t* l0 = tl[0].p;
        X.par_for(nt, [=] __host__ __device__(int64_t t) { l0[t] = (int32_t)t; });
        tln[0] = nt;
        return ok && !X.err && counter(2) == 0;
    }

    // ---- DistMarkingStrategyCL::visit over the triangulation ------------------
    bool mark(const DistPar& D, double width, int clevel, int flevel) {
        set_counter(3, 0);
        View V = view();
        const int L = last();
        for (int l = 0; l <= L; ++l) {
            const int32_t* lst = tl[l].p;
            const bool lastl = l == L;
            X.par_for(tln[l], [=] __host__ __device__(int64_t i) {
                const int32_t t = lst[i];
                if (!lastl && V.trule[t] != kNoRef) return;
                double d = 1.7976931348623157e308;
                int npos = 0;
                double xv[4][3];
                for (int j = 0; j < 4; ++j)
                    for (int k = 0; k < 3; ++k) xv[j][k] = V.vx[3 * (int64_t)V.tv[4 * (int64_t)t + j] + k];
                for (int j = 0; j < 4; ++j) {
                    const double v = dist(D, xv[j]);
                    if (v >= 0) ++npos;
                    d = fmin(d, fabs(v));
                }
                for (int j = 0; j < 6; ++j) {
                    double x[3];
                    for (int k = 0; k < 3; ++k) x[k] = (xv[ev0(j)][k] + xv[ev1(j)][k]) * 0.5;
                    const double v = dist(D, x);
                    if (v >= 0) ++npos;
                    d = fmin(d, fabs(v));
                }
                double b[3];
                for (int k = 0; k < 3; ++k) b[k] = 0.25 * (((xv[0][k] + xv[1][k]) + xv[2][k]) + xv[3][k]);
                d = fmin(d, fabs(dist(D, b)));
                const bool change = npos != 0 && npos != 10;
                const int lv = V.tlev[t];
                const int want = (d <= width || change) ? flevel : clevel;
                if (lv < want || (lv == want && !is_regular(V, t))) {
                    V.tmark[t] = kRegRef;
                    V.cnt[3] = 1;
                } else if (lv > want) {
                    V.tmark[t] = kRemove;
                    V.cnt[3] = 1;
                }
            });
        }
        return counter(3) != 0;
    }

    // ---- MultiGridCL::Refine ----------------------------------------------------
    void restrict_marks(int L) {
        View V = view();
        const int32_t* lst = tl[L].p;
        X.par_for(tln[L], [=] __host__ __device__(int64_t i) {
            const int32_t t = lst[i];
            const uint8_t rule = V.trule[t];
            if (rule == kNoRef) {
                if (V.tmark[t] == kRegRef && is_regular(V, t))
                    for (int j = 0; j < 6; ++j) atom_add(&V.emfr[V.te[6 * (int64_t)t + j]], 1);
                if (V.tlev[t] == 0 && V.tmark[t] == kRemove) V.tmark[t] = kNoRef;
            } else if (rule == kRegRef) {
                bool keep = false;
                for (int c = 0; c < V.tnch[t]; ++c) {
                    const int32_t ch = V.tch[8 * (int64_t)t + c];
                    if (V.tmark[ch] == kRemove)
                        V.tmark[ch] = kNoRef;
                    else
                        keep = true;
                }
                if (!keep) {
                    V.tmark[t] = kNoRef;
                    for (int j = 0; j < 6; ++j) atom_add(&V.emfr[V.te[6 * (int64_t)t + j]], -1);
                }
            } else {
                bool reg = false;
                const int lv = V.tlev[t];
                for (int c = 0; c < V.tnch[t]; ++c) {
                    const int32_t ch = V.tch[8 * (int64_t)t + c];
                    if (!reg) {
                        const uint8_t m = V.tmark[ch];
                        if (m != kNoRef && m != kRemove) {
                            reg = true;
                        } else {
                            for (int j = 0; j < 6; ++j) {
                                const int32_t e = V.te[6 * (int64_t)ch + j];
                                if (V.emfr[e] && V.elev[e] != lv) {
                                    reg = true;
                                    break;
                                }
                            }
                        }
                    }
                    V.tmark[ch] = kNoRef;
                }
                if (reg) {
                    V.tmark[t] = kRegRef;
                    for (int j = 0; j < 6; ++j) atom_add(&V.emfr[V.te[6 * (int64_t)t + j]], 1);
                } else {
                    V.tmark[t] = kNoRef;
                }
            }
        });
    }
    void close_grid(int L) {
        View V = view();
        const int32_t* lst = tl[L].p;
        X.par_for(tln[L], [=] __host__ __device__(int64_t i) {
            const int32_t t = lst[i];
            if (!is_regular(V, t) || V.tmark[t] == kRegRef) return;
            unsigned m = 0;
            for (int j = 0; j < 6; ++j)
                if (V.emfr[V.te[6 * (int64_t)t + j]]) m |= 1u << j;
            if (m == kRegRef)
                V.tmark[t] = kGreen;
            else if (m == kNoRef) {
                if (V.tmark[t] != kRemove) V.tmark[t] = kNoRef;
            } else {
                V.tmark[t] = (uint8_t)m;
            }
        });
    }
    void unrefine_grid(int L) {
        View V = view();
        const int nl = L + 1;
        X.par_for(nv, [=] __host__ __device__(int64_t v) {
            if (V.valive[v] && V.vlev[v] == nl) V.vrm[v] = 1;
        });
        X.par_for(ne, [=] __host__ __device__(int64_t e) {
            if (V.ealive[e] && V.elev[e] == nl) V.erm[e] = 1;
        });
        const int32_t* lst = tl[L].p;
        X.par_for(tln[L], [=] __host__ __device__(int64_t i) {
            const int32_t t = lst[i];
            const uint8_t rule = V.trule[t], mark = V.tmark[t];
            if (rule == kNoRef) return;
            const int nch = V.tnch[t];
            if (mark == rule) {
                for (int c = 0; c < nch; ++c) {
                    const int32_t ch = V.tch[8 * (int64_t)t + c];
                    for (int k = 0; k < 4; ++k) V.vrm[V.tv[4 * (int64_t)ch + k]] = 0;
                    for (int j = 0; j < 6; ++j) V.erm[V.te[6 * (int64_t)ch + j]] = 0;
                }
                return;
            }
            for (int c = 0; c < nch; ++c) V.tmark[V.tch[8 * (int64_t)t + c]] = kRemove;
            if (mark == kNoRef) return;
            // RecycleReusables: edges and children the old and new rules share
            const DRule& my = V.rules[rule & 63];
            const DRule& nw = V.rules[mark & 63];
            for (int c = 0; c < my.nch && c < nch; ++c) {
                const int32_t ch = V.tch[8 * (int64_t)t + c];
                for (int j = 0; j < 6; ++j) {
                    const int a = my.ch[c][ev0(j)], b = my.ch[c][ev1(j)];
                    if (a < 4 && b < 4) continue;
                    bool common = false;
                    for (int d = 0; d < nw.nch && !common; ++d)
                        for (int jj = 0; jj < 6 && !common; ++jj) {
                            const int x = nw.ch[d][ev0(jj)], y = nw.ch[d][ev1(jj)];
                            common = (x == a && y == b) || (x == b && y == a);
                        }
                    if (common) {
                        V.vrm[V.tv[4 * (int64_t)ch + ev0(j)]] = 0;
                        V.vrm[V.tv[4 * (int64_t)ch + ev1(j)]] = 0;
                        V.erm[V.te[6 * (int64_t)ch + j]] = 0;
                    }
                }
            }
            for (int c = 0; c < my.nch && c < nch; ++c) {
                bool in_new = false;
                for (int d = 0; d < nw.nch && !in_new; ++d)
                    in_new = my.ch[c][0] == nw.ch[d][0] && my.ch[c][1] == nw.ch[d][1] && my.ch[c][2] == nw.ch[d][2] &&
                             my.ch[c][3] == nw.ch[d][3];
                if (in_new) V.tmark[V.tch[8 * (int64_t)t + c]] = kNoRef;
            }
        });
        // DestroyMarkedTetras: a stable compaction of the next level's list
        const int64_t n1 = tln[nl];
        if (!flag8.grow(std::max<int64_t>(n1, 1), 0) || !tmp32.grow(std::max<int64_t>(n1, 1), 0)) {
            ok = false;
            return;
        }
        uint8_t* fl = flag8.p;
        const int32_t* l1 = tl[nl].p;
        X.par_for(n1, [=] __host__ __device__(int64_t i) { fl[i] = V.tmark[l1[i]] != kRemove; });
        int32_t* t32 = tmp32.p;
        const int64_t k = select(l1, n1, t32);
        if (X.dev)
            cudaMemcpyAsync(tl[nl].p, t32, sizeof(int32_t) * k, cudaMemcpyDeviceToDevice, X.s);
        else
            std::memcpy(tl[nl].p, t32, sizeof(int32_t) * k);
        tln[nl] = k;
        // midvertices marked for removal leave their edges; then the marked vertices and edges go
        X.par_for(ne, [=] __host__ __device__(int64_t e) {
            if (V.ealive[e] && V.elev[e] == L && V.emid[e] >= 0 && V.vrm[V.emid[e]]) {
                V.emid[e] = -1;
                V.esub[2 * e] = V.esub[2 * e + 1] = -1;
            }
        });
        X.par_for(nv, [=] __host__ __device__(int64_t v) {
            if (V.valive[v] && V.vlev[v] == nl && V.vrm[v]) V.valive[v] = 0;
        });
        X.par_for(ne, [=] __host__ __device__(int64_t e) {
            if (V.ealive[e] && V.elev[e] == nl && V.erm[e]) V.ealive[e] = 0;
        });
    }
    void rebuild_hash(int64_t need) {
        uint32_t cap = 1024;
        while ((int64_t)cap < 2 * need && cap < (1u << 31)) cap <<= 1;
        if (cap > hcap) {
            hkey.release();
            hval.release();
            if (!hkey.grow(cap, 0) || !hval.grow(cap, 0)) {
                ok = false;
                return;
            }
            hcap = cap;
        }
        hkey.fill(hcap, kEmpty);
        hval.fill(hcap, -1);
        View V = view();
        X.par_for(ne, [=] __host__ __device__(int64_t e) {
            if (V.ealive[e]) h_insert(V, ekey(V.ev[2 * e], V.ev[2 * e + 1]), (int32_t)e);
        });
    }
    void refine_grid(int L) {
        if (L == last()) append_level();
        const int nl = L + 1;
        const int64_t n = tln[L];
        const int32_t* lst = tl[L].p;
        {
            View V = view();
            X.par_for(n, [=] __host__ __device__(int64_t i) {
                const int32_t t = lst[i];
                const uint8_t mark = V.tmark[t];
                const bool chg = mark != V.trule[t];
                V.tchg[t] = chg;
                if (!chg) return;
                if (mark == kRemove) {
                    seterr(V, 5);
                    return;
                }
                if (mark == kNoRef) return;
                for (int j = 0; j < 6; ++j) {
                    const int32_t e = V.te[6 * (int64_t)t + j];
                    if (V.emfr[e] > 0 && V.emid[e] < 0) V.esplit[e] = 1;
                }
            });
        }
        // counts for the capacities: split edges, inner-edge attempts
        if (!tmp32.grow(std::max(ne, n) + 1, 0)) {
            ok = false;
            return;
        }
        int32_t* t32 = tmp32.p;
        {
            View V = view();
            X.par_for(ne, [=] __host__ __device__(int64_t e) { t32[e] = V.esplit[e]; });
        }
        const int64_t nsplit = scan(t32, ne);
        {
            View V = view();
            X.par_for(n, [=] __host__ __device__(int64_t i) {
                const int32_t t = lst[i];
                t32[i] = V.tchg[t] && V.tmark[t] != kNoRef ? V.rules[V.tmark[t] & 63].nin : 0;
            });
        }
        const int64_t ninner = scan(t32, n);
        if (!ok || !grow_verts(nv + nsplit) || !grow_edges(ne + 2 * nsplit + ninner)) {
            ok = false;
            return;
        }
        rebuild_hash(ne + 2 * nsplit + ninner);
        if (!ok) return;
        sync_counts_to_dev();
        // midvertices and sub-edges, one creator per split edge
        {
            View V = view();
            const int64_t ne0 = ne;
            X.par_for(ne0, [=] __host__ __device__(int64_t e) {
                if (!V.esplit[e]) return;
                V.esplit[e] = 0;
                const int32_t mv = atom_add(&V.cnt[0], 1);
                const int32_t s0 = atom_add(&V.cnt[1], 2);
                if (mv >= V.capv || s0 + 1 >= V.cape) {
                    seterr(V, 6);
                    return;
                }
                const int32_t a = V.ev[2 * e], b = V.ev[2 * e + 1];
                for (int k = 0; k < 3; ++k) V.vx[3 * (int64_t)mv + k] = 0.5 * (V.vx[3 * (int64_t)a + k] + V.vx[3 * (int64_t)b + k]);
                const int lv = V.elev[e] + 1;
                V.vlev[mv] = lv;
                V.vrm[mv] = 0;
                V.valive[mv] = 1;
                const int32_t ends[2][2] = {{a, mv}, {mv, b}};
                for (int s = 0; s < 2; ++s) {
                    const int32_t id = s0 + s;
                    V.ev[2 * (int64_t)id] = ends[s][0];
                    V.ev[2 * (int64_t)id + 1] = ends[s][1];
                    V.elev[id] = lv;
                    V.emfr[id] = 0;
                    V.emid[id] = -1;
                    V.esub[2 * (int64_t)id] = V.esub[2 * (int64_t)id + 1] = -1;
                    V.erm[id] = 0;
                    V.ealive[id] = 1;
                    V.esplit[id] = 0;
                    h_insert(V, ekey(ends[s][0], ends[s][1]), id);
                }
                V.emid[e] = mv;
                V.esub[2 * e] = s0;
                V.esub[2 * e + 1] = s0 + 1;
            });
        }
        // inner edges: keys first, then ids
        {
            View V = view();
            X.par_for(n, [=] __host__ __device__(int64_t i) {
                const int32_t t = lst[i];
                if (!V.tchg[t] || V.tmark[t] == kNoRef) return;
                const DRule& R = V.rules[V.tmark[t] & 63];
                for (int k = 0; k < R.nin; ++k) {
                    const int32_t p = vert_mid(V, t, R.in[k][0]), q = vert_mid(V, t, R.in[k][1]);
                    if (p < 0 || q < 0) {
                        seterr(V, 7);
                        return;
                    }
                    h_insert(V, ekey(p, q), -1);
                }
            });
            const int lv = nl;
            X.par_for(hcap, [=] __host__ __device__(int64_t s) {
                if (V.hkey[s] == kEmpty || V.hval[s] >= 0) return;
                const int32_t id = atom_add(&V.cnt[1], 1);
                if (id >= V.cape) {
                    seterr(V, 6);
                    return;
                }
                V.ev[2 * (int64_t)id] = (int32_t)(V.hkey[s] >> 32);
                V.ev[2 * (int64_t)id + 1] = (int32_t)(V.hkey[s] & 0xffffffffu);
                V.elev[id] = lv;
                V.emfr[id] = 0;
                V.emid[id] = -1;
                V.esub[2 * (int64_t)id] = V.esub[2 * (int64_t)id + 1] = -1;
                V.erm[id] = 0;
                V.ealive[id] = 1;
                V.esplit[id] = 0;
                V.hval[s] = id;
            });
        }
        sync_counts_from_dev();
        // children: new ones counted, placed by a scan in list order
        {
            View V = view();
            X.par_for(n, [=] __host__ __device__(int64_t i) {
                const int32_t t = lst[i];
                int cntn = 0;
                if (V.tchg[t] && V.tmark[t] != kNoRef) {
                    const DRule& R = V.rules[V.tmark[t] & 63];
                    for (int c = 0; c < R.nch; ++c) {
                        int32_t cv[4];
                        for (int k = 0; k < 4; ++k) {
                            cv[k] = vert_mid(V, t, R.ch[c][k]);
                            if (cv[k] < 0) seterr(V, 9);
                        }
                        bool found = false;
                        for (int o = 0; o < V.tnch[t] && !found; ++o) {
                            const int32_t och = V.tch[8 * (int64_t)t + o];
                            found = V.tmark[och] != kRemove && V.tv[4 * (int64_t)och] == cv[0] &&
                                    V.tv[4 * (int64_t)och + 1] == cv[1] && V.tv[4 * (int64_t)och + 2] == cv[2] &&
                                    V.tv[4 * (int64_t)och + 3] == cv[3];
                        }
                        cntn += !found;
                    }
                }
                t32[i] = cntn;
            });
        }
        const int64_t nnew = scan(t32, n);
        if (!ok || !grow_tets(nt + nnew) || !tl[nl].grow(tln[nl] + nnew, tln[nl])) {
            ok = false;
            return;
        }
        {
            View V = view();
            const int64_t* off = tmp64.p;
            const int32_t base = (int32_t)nt;
            int32_t* l1 = tl[nl].p;
            const int64_t lbase = tln[nl];
            X.par_for(n, [=] __host__ __device__(int64_t i) {
                const int32_t t = lst[i];
                if (!V.tchg[t]) return;
                const uint8_t mark = V.tmark[t];
                V.trule[t] = mark;
                if (mark == kNoRef) {
                    V.tnch[t] = 0;
                    return;
                }
                const DRule& R = V.rules[mark & 63];
                int32_t old[8];
                const int nold = V.tnch[t];
                for (int o = 0; o < nold && o < 8; ++o) old[o] = V.tch[8 * (int64_t)t + o];
                int64_t k = off[i];
                for (int c = 0; c < R.nch; ++c) {
                    int32_t cv[4];
                    for (int q = 0; q < 4; ++q) {
                        cv[q] = vert_mid(V, t, R.ch[c][q]);
                        if (cv[q] < 0) {  // inconsistent (reported by the count pass): a valid id keeps later passes in bounds
                            seterr(V, 9);
                            cv[q] = 0;
                        }
                    }
                    int32_t ch = -1;
                    for (int o = 0; o < nold && o < 8 && ch < 0; ++o) {
                        const int32_t och = old[o];
                        if (V.tmark[och] != kRemove && V.tv[4 * (int64_t)och] == cv[0] &&
                            V.tv[4 * (int64_t)och + 1] == cv[1] && V.tv[4 * (int64_t)och + 2] == cv[2] &&
                            V.tv[4 * (int64_t)och + 3] == cv[3])
                            ch = och;
                    }
                    if (ch < 0) {
                        ch = base + (int32_t)k;
                        l1[lbase + k] = ch;
                        ++k;
                        for (int q = 0; q < 4; ++q) V.tv[4 * (int64_t)ch + q] = cv[q];
                        V.tlev[ch] = V.tlev[t] + 1;
                        V.tpar[ch] = t;
                        V.tnch[ch] = 0;
                        V.trule[ch] = kNoRef;
                        V.tmark[ch] = kNoRef;
                        V.tchg[ch] = 0;
                    }
                    V.tch[8 * (int64_t)t + c] = ch;
                    // the child's edges: parent edges, halves of split ones, inner edges
                    for (int j = 0; j < 6; ++j) {
                        const int a = R.ch[c][ev0(j)], b = R.ch[c][ev1(j)];
                        int32_t e = -1;
                        if (a < 4 && b < 4) {
                            e = V.te[6 * (int64_t)t + edge_of(a, b)];
                        } else {
                            const int corner = a < 4 ? a : (b < 4 ? b : -1);
                            const int midp = a < 4 ? b : a;
                            const int pe = midp - 4;
                            if (corner >= 0 && (ev0(pe) == corner || ev1(pe) == corner)) {
                                const int32_t ee = V.te[6 * (int64_t)t + pe];
                                e = V.ev[2 * (int64_t)ee] == V.tv[4 * (int64_t)t + corner] ? V.esub[2 * (int64_t)ee]
                                                                                           : V.esub[2 * (int64_t)ee + 1];
                            } else {
                                int p = a, q = b;
                                if (rank_of(p) > rank_of(q)) {
                                    const int tt = p;
                                    p = q;
                                    q = tt;
                                }
                                e = h_find(V, ekey(vert_mid(V, t, p), vert_mid(V, t, q)));
                            }
                        }
                        if (e < 0) seterr(V, 8);
                        V.te[6 * (int64_t)ch + j] = e < 0 ? 0 : e;
                    }
                }
                V.tnch[t] = (int8_t)R.nch;
            });
        }
        nt += nnew;
        tln[nl] += nnew;
    }
    bool refine() {
        const int top = last();
        for (int L = top; L >= 0; --L) {
            restrict_marks(L);
            close_grid(L);
        }
        for (int L = 0; L <= top && ok; ++L) {
            if (tln[L] == 0) continue;
            if (L) close_grid(L);
            if (L != top) unrefine_grid(L);
            refine_grid(L);
            if (counter(2) != 0 || X.err) ok = false;
        }
        while (tl.size() > 1 && tln.back() == 0) {
            tl.back().release();
            tl.pop_back();
            tln.pop_back();
        }
        return ok;
    }

    // ---- the last triangulation level, renumbered ------------------------------
    // out arrays sized by the caller from the returned counts (two calls)
    bool triang(Buf<int32_t>& tri, int64_t& ntri) {
        const int L = last();
        ntri = 0;
        for (int l = 0; l <= L; ++l) ntri += tln[l];
        if (!tri.grow(std::max<int64_t>(ntri, 1), 0) || !flag8.grow(std::max<int64_t>(ntri, 1), 0)) return false;
        int64_t k = 0;
        View V = view();
        for (int l = 0; l <= L; ++l) {
            const int32_t* lst = tl[l].p;
            uint8_t* fl = flag8.p;
            const bool lastl = l == L;
            X.par_for(tln[l], [=] __host__ __device__(int64_t i) { fl[i] = lastl || V.trule[lst[i]] == kNoRef; });
            k += select(lst, tln[l], tri.p + k);
        }
        ntri = k;
        return ok;
    }
};

std::vector<DRule> make_rules() {
    std::vector<DRule> R(64);
    std::vector<int32_t> nch(64), ch(64 * 8 * 4);
    if (tf_refine_rules(nch.data(), ch.data()) != TF_OK) return {};
    for (int p = 0; p < 64; ++p) {
        DRule& r = R[p];
        std::memset(&r, 0, sizeof r);
        r.nch = nch[p];
        bool seen[10][10] = {};
        for (int c = 0; c < r.nch; ++c) {
            for (int k = 0; k < 4; ++k) r.ch[c][k] = (uint8_t)ch[(p * 8 + c) * 4 + k];
            for (int j = 0; j < 6; ++j) {
                int a = r.ch[c][ev0(j)], b = r.ch[c][ev1(j)];
                if (a < 4 && b < 4) continue;
                const int corner = a < 4 ? a : (b < 4 ? b : -1);
                const int midp = a < 4 ? b : a;
                if (corner >= 0 && (ev0(midp - 4) == corner || ev1(midp - 4) == corner)) continue;
                if (rank_of(a) > rank_of(b)) std::swap(a, b);
                if (seen[a][b]) continue;
                seen[a][b] = true;
                r.in[r.nin][0] = (uint8_t)a;
                r.in[r.nin][1] = (uint8_t)b;
                ++r.nin;
            }
        }
    }
    return R;
}

// Runs MakeInitialTriang; on success the engine holds the multigrid.
int run(Engine& G, int64_t nv, const double* coords, int64_t nt, const int32_t* tv, const int32_t* te, int64_t ne,
        int kind, const double* par, int npar, double width, int clevel, int flevel, int& steps) {
    const int need = kind == TF_LS_SPHERE ? 4 : kind == TF_LS_TORUS ? 3 : kind == TF_LS_PLANE ? 4 : -1;
    if (need < 0 || npar < need || !par || clevel < 0 || flevel < clevel || flevel > 30 || !(width >= 0))
        return TF_ERR_BAD_INPUT;
    if (kind == TF_LS_TORUS && (par[2] < 0 || par[2] > 2)) return TF_ERR_BAD_INPUT;
    const std::vector<DRule> R = make_rules();
    if (R.empty()) return TF_ERR_INTERNAL;
    if (!G.init(nv, coords, nt, tv, te, ne, R)) return G.counter(2) == 4 ? TF_ERR_BAD_INPUT : TF_ERR_CUDA;
    DistPar D;
    D.kind = kind;
    for (int i = 0; i < 16; ++i) D.p[i] = i < npar ? par[i] : 0.0;
    bool modified = true;
    steps = 0;
    for (int i = 0; i < 2 * flevel && modified; ++i) {
        modified = G.mark(D, width, clevel, flevel);
        if (!G.refine()) return G.X.err ? TF_ERR_CUDA : TF_ERR_INTERNAL;
        ++steps;
    }
    return G.ok ? TF_OK : TF_ERR_INTERNAL;
}

}  // namespace rpar

// The data-parallel engine run on the host (the same kernel bodies as plain
// loops): the refined mesh with vertices and edges numbered by first touch.
int refine_band_parallel_host(int64_t nv, const double* coords, int64_t nt, const int32_t* tet_v, int kind,
                              const double* par, int npar, double width, int clevel, int flevel, RefinedMesh& out) {
    using namespace rpar;
    if (nv <= 0 || nt <= 0 || !coords || !tet_v) return TF_ERR_BAD_INPUT;
    for (int64_t i = 0; i < 4 * nt; ++i)
        if (tet_v[i] < 0 || tet_v[i] >= nv) return TF_ERR_BAD_INPUT;
    // level-0 edge ids by vertex pair (either direction; the engine checks the orientation)
    std::vector<int32_t> te((size_t)(6 * nt));
    std::map<std::pair<int32_t, int32_t>, int32_t> ids;
    for (int64_t t = 0; t < nt; ++t)
        for (int j = 0; j < 6; ++j) {
            int32_t a = tet_v[4 * t + ev0(j)], b = tet_v[4 * t + ev1(j)];
            if (a == b) return TF_ERR_BAD_INPUT;
            auto key = std::make_pair(std::min(a, b), std::max(a, b));
            auto it = ids.find(key);
            if (it == ids.end()) it = ids.emplace(key, (int32_t)ids.size()).first;
            te[6 * t + j] = it->second;
        }
    Engine G(false, nullptr, 1);
    int steps = 0;
    const int st = run(G, nv, coords, nt, tet_v, te.data(), (int64_t)ids.size(), kind, par, npar, width, clevel,
                       flevel, steps);
    if (st != TF_OK) return st;
    Buf<int32_t> tri;
    tri.dev = false;
    tri.X = &G.X;
    int64_t ntri = 0;
    if (!G.triang(tri, ntri)) {
        tri.release();
        return TF_ERR_INTERNAL;
    }
    out = RefinedMesh{};
    out.last_level = G.last();
    out.steps = steps;
    for (int64_t n : G.tln) out.per_level.push_back(n);
    std::vector<int32_t> vid((size_t)G.nv, -1), eid((size_t)G.ne, -1);
    for (int64_t i = 0; i < ntri; ++i) {
        const int32_t t = tri.p[i];
        for (int k = 0; k < 4; ++k) {
            const int32_t v = G.tv.p[4 * (int64_t)t + k];
            if (vid[v] < 0) {
                vid[v] = (int32_t)(out.coords.size() / 3);
                for (int q = 0; q < 3; ++q) out.coords.push_back(G.vx.p[3 * (int64_t)v + q]);
            }
            out.tet_v.push_back(vid[v]);
        }
        for (int j = 0; j < 6; ++j) {
            const int32_t e = G.te.p[6 * (int64_t)t + j];
            if (eid[e] < 0) {
                eid[e] = (int32_t)(out.edge_v.size() / 2);
                out.edge_v.push_back(vid[G.ev.p[2 * (int64_t)e]]);
                out.edge_v.push_back(vid[G.ev.p[2 * (int64_t)e + 1]]);
            }
            out.tet_e.push_back(eid[e]);
        }
        out.tet_level.push_back(G.tlev.p[t]);
    }
    tri.release();
    return TF_OK;
}

// The device path: the context's (brick or uploaded) mesh refined on the
// device and installed as an uploaded mesh; vertices and edges numbered by
// first touch in the triangulation's order, as the sequential form numbers
// them.
int refine_band_device(Context* c, int kind, const double* par, int npar, double width, int clevel, int flevel,
                       int* last_level, int* steps_out) {
    using namespace rpar;
    const MeshView M0 = c->mesh;
    const int64_t nv0 = M0.nv, ne0 = M0.ne, nt0 = M0.nt;
    DBuf<double> dc;
    DBuf<int32_t> dv, de;
    TF_TRY(ensure(c, dc, (size_t)(3 * nv0)));
    TF_TRY(ensure(c, dv, (size_t)(4 * nt0)));
    TF_TRY(ensure(c, de, (size_t)(6 * nt0)));
    int st = mesh_materialise(c, dc.p, dv.p, de.p, nullptr);
    // the bounding box (the refined vertices lie in the hull of the level-0 ones)
    std::vector<double> hc((size_t)(3 * nv0));
    if (st == TF_OK && cudaMemcpyAsync(hc.data(), dc.p, sizeof(double) * 3 * nv0, cudaMemcpyDeviceToHost, c->stream) !=
                           cudaSuccess)
        st = set_err(c, TF_ERR_CUDA, "refine: coordinates");
    if (st == TF_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) st = set_err(c, TF_ERR_CUDA, "refine: sync");
    int steps = 0;
    // the context's pool for the engine's buffers: kept between calls, so a
    // repeated refinement allocates nothing new (tf_destroy releases it)
    if (!c->refine_pool) {
        int pools = 0;
        if (cudaDeviceGetAttribute(&pools, cudaDevAttrMemoryPoolsSupported, c->device) == cudaSuccess && pools) {
            cudaMemPoolProps pp{};
            pp.allocType = cudaMemAllocationTypePinned;
            pp.location.type = cudaMemLocationTypeDevice;
            pp.location.id = c->device;
            if (cudaMemPoolCreate(&c->refine_pool, &pp) == cudaSuccess) {
                uint64_t keep = UINT64_MAX;
                cudaMemPoolSetAttribute(c->refine_pool, cudaMemPoolAttrReleaseThreshold, &keep);
            } else {
                c->refine_pool = nullptr;
                cudaGetLastError();
            }
        }
    }
    Engine G(true, c->stream, c->num_sms, c->refine_pool);
    if (st == TF_OK) {
        std::vector<int32_t> htv((size_t)(4 * nt0)), hte((size_t)(6 * nt0));
        cudaMemcpyAsync(htv.data(), dv.p, sizeof(int32_t) * 4 * nt0, cudaMemcpyDeviceToHost, c->stream);
        cudaMemcpyAsync(hte.data(), de.p, sizeof(int32_t) * 6 * nt0, cudaMemcpyDeviceToHost, c->stream);
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) st = set_err(c, TF_ERR_CUDA, "refine: sync");
        if (st == TF_OK) {
            const int r = run(G, nv0, hc.data(), nt0, htv.data(), hte.data(), ne0, kind, par, npar, width, clevel,
                              flevel, steps);
            if (r != TF_OK) st = set_err(c, r, "mesh_refine_band: bad parameters, an unoriented mesh or a failed pass");
        }
    }
    release(dc);
    release(dv);
    release(de);
    if (st != TF_OK) return st;
    // the last triangulation level, in list order
    Buf<int32_t> tri;
    tri.dev = true;
    tri.X = &G.X;
    int64_t ntri = 0;
    if (!G.triang(tri, ntri)) {
        tri.release();
        return set_err(c, TF_ERR_CUDA, "refine: triangulation");
    }
    // Vertices and edges numbered by first touch in the triangulation's order
    // (tet by tet, local vertex / edge order, as the sequential form): the key
    // of a vertex is the smallest slot 4 i + k of the triangulation holding it
    // (6 i + j for an edge), its id the rank of that key, by a scan over the
    // slots.  The engine's own ids come from atomic counters and are not used.
    constexpr int64_t kNone = INT64_MAX;
    if (6 * ntri >= (int64_t)INT32_MAX) {
        tri.release();
        return set_err(c, TF_ERR_CAPACITY, "refine: mesh too large for 32-bit ids");
    }
    Buf<int64_t> vkey, ekey, voff;
    Buf<int32_t> vslot, eslot;
    vkey.dev = ekey.dev = voff.dev = vslot.dev = eslot.dev = true;
    vkey.X = ekey.X = voff.X = vslot.X = eslot.X = &G.X;
    auto release_all = [&]() {
        tri.release(), vkey.release(), ekey.release(), voff.release(), vslot.release(), eslot.release();
    };
    bool okb = vkey.grow(G.nv, 0) && ekey.grow(G.ne, 0) && vslot.grow(4 * ntri + 1, 0) &&
               eslot.grow(6 * ntri + 1, 0) && voff.grow(4 * ntri + 1, 0);
    if (!okb) {
        release_all();
        return set_err(c, TF_ERR_CUDA, "refine: alloc");
    }
    vkey.fill(G.nv, kNone);
    ekey.fill(G.ne, kNone);
    vslot.fill(4 * ntri, 0);
    eslot.fill(6 * ntri, 0);
    {
        View V = G.view();
        const int32_t* tp = tri.p;
        int64_t* vk = vkey.p;
        int64_t* ek = ekey.p;
        int32_t* vs = vslot.p;
        int32_t* es = eslot.p;
        const int64_t nv = G.nv, ne = G.ne;
        G.X.par_for(ntri, [=] __host__ __device__(int64_t i) {
            const int32_t t = tp[i];
            for (int k = 0; k < 4; ++k) atom_min(&vk[V.tv[4 * (int64_t)t + k]], 4 * i + k);
            for (int j = 0; j < 6; ++j) atom_min(&ek[V.te[6 * (int64_t)t + j]], 6 * i + j);
        });
        G.X.par_for(nv, [=] __host__ __device__(int64_t v) {
            if (vk[v] != kNone) vs[vk[v]] = 1;
        });
        G.X.par_for(ne, [=] __host__ __device__(int64_t e) {
            if (ek[e] != kNone) es[ek[e]] = 1;
        });
    }
    const int64_t nvo = G.scan(vslot.p, 4 * ntri);
    if (G.ok && cudaMemcpyAsync(voff.p, G.tmp64.p, sizeof(int64_t) * (4 * ntri + 1), cudaMemcpyDeviceToDevice,
                                c->stream) != cudaSuccess)
        okb = false;
    const int64_t neo = G.scan(eslot.p, 6 * ntri);
    if (!okb || !G.ok || nvo > INT32_MAX || neo > INT32_MAX) {
        release_all();
        return set_err(c, TF_ERR_CAPACITY, "refine: mesh too large for 32-bit ids");
    }
    TF_TRY(ensure(c, c->coords, (size_t)(3 * nvo)));
    TF_TRY(ensure(c, c->tet_v, (size_t)(4 * ntri)));
    TF_TRY(ensure(c, c->tet_e, (size_t)(6 * ntri)));
    TF_TRY(ensure(c, c->edge_v, (size_t)(2 * neo)));
    {
        View V = G.view();
        const int64_t* vo = voff.p;
        const int64_t* eo = G.tmp64.p;
        const int64_t* vk = vkey.p;
        const int64_t* ek = ekey.p;
        double* oc = c->coords.p;
        int32_t *otv = c->tet_v.p, *ote = c->tet_e.p, *oev = c->edge_v.p;
        const int32_t* tp = tri.p;
        G.X.par_for(G.nv, [=] __host__ __device__(int64_t v) {
            if (vk[v] == kNone) return;
            const int64_t id = vo[vk[v]];
            for (int k = 0; k < 3; ++k) oc[3 * id + k] = V.vx[3 * v + k];
        });
        G.X.par_for(G.ne, [=] __host__ __device__(int64_t e) {
            if (ek[e] == kNone) return;
            const int64_t id = eo[ek[e]];
            // the ends of a triangulation edge are triangulation vertices
            const int64_t ka = vk[V.ev[2 * e]], kb = vk[V.ev[2 * e + 1]];
            oev[2 * id] = ka != kNone ? (int32_t)vo[ka] : -1;
            oev[2 * id + 1] = kb != kNone ? (int32_t)vo[kb] : -1;
        });
        G.X.par_for(ntri, [=] __host__ __device__(int64_t i) {
            const int32_t t = tp[i];
            for (int k = 0; k < 4; ++k) otv[4 * i + k] = (int32_t)vo[vk[V.tv[4 * (int64_t)t + k]]];
            for (int j = 0; j < 6; ++j) ote[6 * i + j] = (int32_t)eo[ek[V.te[6 * (int64_t)t + j]]];
        });
    }
    const cudaError_t ce = cudaStreamSynchronize(c->stream);
    release_all();
    if (ce != cudaSuccess || G.X.err) return set_err(c, TF_ERR_CUDA, "refine: output");
    MeshView& M = c->mesh;
    M = MeshView{};
    M.explicit_mesh = 1;
    c->batch_count = 0;
    M.nv = nvo;
    M.ne = neo;
    M.nt = ntri;
    M.coords = c->coords.p;
    M.tet_v = c->tet_v.p;
    M.tet_e = c->tet_e.p;
    M.edge_v = c->edge_v.p;
    for (int k = 0; k < 3; ++k) {
        double lo = hc[k], hi = hc[k];
        for (int64_t v = 1; v < nv0; ++v) {
            lo = std::min(lo, hc[3 * v + k]);
            hi = std::max(hi, hc[3 * v + k]);
        }
        M.bb_lo[k] = lo;
        M.bb_scale[k] = hi > lo ? 1048576.0 / (hi - lo) : 0.0;
    }
    c->has_mesh = true;
    c->has_ls = false;
    c->has_wind = false;
    c->fe = 0;
    if (last_level) *last_level = G.last();
    if (steps_out) *steps_out = steps;
    return TF_OK;
}

}  // namespace tf
