// Internal declarations shared by the CUDA translation units of libtracefem.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>
#include <vector>

#include "../../include/tracefem.h"

namespace tf {

// ---------------------------------------------------------------------------
// tet-local topology (geom/topo.cpp VertOfEdgeAr, first 6 rows)
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int ev0(int e) { return e < 3 ? (e < 2 ? 0 : 1) : (e == 3 ? 0 : (e == 4 ? 1 : 2)); }
__host__ __device__ constexpr int ev1(int e) { return e == 0 ? 1 : (e == 1 || e == 2 ? 2 : 3); }

// ---------------------------------------------------------------------------
// Mesh view: implicit Kuhn brick or explicit arrays.
// Brick edge numbering: 7 direction classes (d3,d2,d1) in the order
// 001,010,100,011,101,110,111; inside a class edges are numbered by the
// brick index of their lower vertex.
// ---------------------------------------------------------------------------
// One Kuhn brick: n1 x n2 x n3 cubes of 6 tets (geom/builder.cpp:99-180).
struct Brick {
    int n1, n2, n3;
    double orig[3], o1[3], o2[3], o3[3];
    int64_t eoff[8];  // first edge of each direction class; eoff[7] = edges
};

// Row of the instance table of a batch: the brick and where its vertices,
// edges and tets start in the concatenated numbering.
struct BatchBrick {
    Brick b;
    int64_t v0, e0, t0;
};

// Doubled brick-grid position of a node: 2 (i1, i2, i3) for a vertex, the sum
// of its two end vertices' positions for an edge (node = vertex id, or nv +
// edge id).  Edge classes run over the seven directions (d3 d2 d1) of the
// Kuhn cube's edges (class -> bits 1, 2, 4, 3, 5, 6, 7), each numbered by its
// lower vertex over the grid shortened by one in the set directions.
__device__ inline void brick_node_grid2(const Brick& B, int64_t node, int64_t nv, int g[3]) {
    int64_t v = node;
    int d3 = 0, d2 = 0, d1 = 0;
    if (node >= nv) {
        const int64_t id = node - nv;
        int cls = 0;
        while (cls < 6 && id >= B.eoff[cls + 1]) ++cls;
        const int code = (int)((0x7653421 >> (4 * cls)) & 0xf);
        d3 = (code >> 2) & 1;
        d2 = (code >> 1) & 1;
        d1 = code & 1;
        const int64_t r = id - B.eoff[cls];
        const int64_t w1 = B.n1 + 1 - d1, w2 = B.n2 + 1 - d2;
        const int64_t a1 = r % w1, q = r / w1, a2 = q % w2, a3 = q / w2;
        v = (a3 * (B.n2 + 1) + a2) * (B.n1 + 1) + a1;
    }
    const int64_t i1 = v % (B.n1 + 1), q = v / (B.n1 + 1), i2 = q % (B.n2 + 1), i3 = q / (B.n2 + 1);
    g[0] = (int)(2 * i1 + d1);
    g[1] = (int)(2 * i2 + d2);
    g[2] = (int)(2 * i3 + d3);
}

struct MeshView {
    int explicit_mesh;
    int nbatch;  // > 0: concatenation of nbatch bricks, instance after instance
    int64_t nv, ne, nt;
    Brick b;     // the brick when nbatch == 0
    // batch tables (device): instances, and nbatch+1 start offsets for the searches
    const BatchBrick* batch;
    const int64_t* tstart;
    const int64_t* vstart;
    const int64_t* estart;
    // explicit arrays (device)
    const double* coords;
    const int32_t* tet_v;
    const int32_t* tet_e;
    const int32_t* edge_v;
    // explicit meshes: the bounding box's low corner and 2^20 / extent per
    // axis (grid positions for the locality order)
    double bb_lo[3], bb_scale[3];
};

// instance owning index x: the largest i with start[i] <= x (start[0] = 0)
__host__ __device__ inline int batch_find(const int64_t* start, int n, int64_t x) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= x) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__host__ __device__ inline int edir_class(int d3, int d2, int d1) {
    // offsets (d3,d2,d1) -> class index
    const int code = d3 * 4 + d2 * 2 + d1;  // 1,2,4,3,5,6,7
    switch (code) {
        case 1: return 0;
        case 2: return 1;
        case 4: return 2;
        case 3: return 3;
        case 5: return 4;
        case 6: return 5;
        default: return 6;
    }
}

// Kuhn split (geom/builder.cpp:151-176): vertex offsets (i3,i2,i1) per tet type
__host__ __device__ inline void kuhn_offset(int l, int k, int& d3, int& d2, int& d1) {
    // k = 0: (0,0,0); k = 3: (1,1,1)
    if (k == 0) { d3 = d2 = d1 = 0; return; }
    if (k == 3) { d3 = d2 = d1 = 1; return; }
    // first step axis and second step axis per tet type, (i3,i2,i1) = axis 0,1,2
    // l=0: +i1, +i2   l=1: +i1, +i3   l=2: +i2, +i1   l=3: +i2, +i3   l=4: +i3, +i1   l=5: +i3, +i2
    // first = {2,2,1,1,0,0}, second = {1,0,2,0,2,1}, one nibble per type
    // (packed constants rather than small arrays that a dynamic index would
    // put in local memory)
    const int f = (0x001122 >> (4 * l)) & 0xf, s = (0x120201 >> (4 * l)) & 0xf;
    const bool two = k == 2;
    d3 = (f == 0) | (two & (s == 0));
    d2 = (f == 1) | (two & (s == 1));
    d1 = (f == 2) | (two & (s == 2));
}

__host__ __device__ inline void brick_tet(const Brick& B, int64_t t, int64_t v0, int64_t e0, int32_t v[4], int32_t e[6]) {
    // 32-bit divisions (cube < 2^32 for any mesh with 32-bit vertex ids; a
    // 64-bit division by a runtime divisor is a long emulated sequence)
    const uint32_t cube = (uint32_t)(t / 6);
    const int l = (int)(t - (int64_t)cube * 6);
    const uint32_t n1 = (uint32_t)B.n1, n2 = (uint32_t)B.n2;
    const uint32_t r = cube / n1;
    const int i1 = (int)(cube - r * n1);
    const uint32_t r2 = r / n2;
    const int i2 = (int)(r - r2 * n2);
    const int i3 = (int)r2;
    int p[4][3];
    for (int k = 0; k < 4; ++k) {
        int d3, d2, d1;
        kuhn_offset(l, k, d3, d2, d1);
        p[k][0] = i3 + d3; p[k][1] = i2 + d2; p[k][2] = i1 + d1;
        v[k] = (int32_t)(v0 + ((int64_t)p[k][0] * (B.n2 + 1) + p[k][1]) * (B.n1 + 1) + p[k][2]);
    }
    if (e) {
        for (int k = 0; k < 6; ++k) {
            const int* a = p[ev0(k)];
            const int* b = p[ev1(k)];
            const int d3 = b[0] - a[0], d2 = b[1] - a[1], d1 = b[2] - a[2];
            const int c = edir_class(d3, d2, d1);
            e[k] = (int32_t)(e0 + B.eoff[c] + ((int64_t)a[0] * (B.n2 + 1 - d2) + a[1]) * (B.n1 + 1 - d1) + a[2]);
        }
    }
}

__device__ inline void mesh_tet(const MeshView& M, int64_t t, int32_t v[4], int32_t e[6]) {
    if (M.explicit_mesh) {
        for (int k = 0; k < 4; ++k) v[k] = M.tet_v[4 * t + k];
        if (e)
            for (int k = 0; k < 6; ++k) e[k] = M.tet_e[6 * t + k];
        return;
    }
    if (M.nbatch) {
        const BatchBrick& I = M.batch[batch_find(M.tstart, M.nbatch, t)];
        brick_tet(I.b, t - I.t0, I.v0, I.e0, v, e);
        return;
    }
    brick_tet(M.b, t, 0, 0, v, e);
}

// Vertex coordinates; for a brick, ((orig + i1*o1) + i2*o2) + i3*o3 per
// component with round-to-nearest products and sums (no contraction), as in
// BrickBuilderCL::build_ser_impl.
__device__ inline void brick_coord(const Brick& B, int64_t v, double x[3]) {
    const uint32_t u = (uint32_t)v, m1 = (uint32_t)B.n1 + 1u, m2 = (uint32_t)B.n2 + 1u;
    const uint32_t r = u / m1;
    const int i1 = (int)(u - r * m1);
    const uint32_t r2 = r / m2;
    const int i2 = (int)(r - r2 * m2);
    const int i3 = (int)r2;
    for (int c = 0; c < 3; ++c)
        x[c] = __dadd_rn(__dadd_rn(__dadd_rn(B.orig[c], __dmul_rn((double)i1, B.o1[c])), __dmul_rn((double)i2, B.o2[c])),
                         __dmul_rn((double)i3, B.o3[c]));
}

__device__ inline void mesh_coord(const MeshView& M, int32_t v, double x[3]) {
    if (M.explicit_mesh) {
        x[0] = M.coords[3 * (int64_t)v];
        x[1] = M.coords[3 * (int64_t)v + 1];
        x[2] = M.coords[3 * (int64_t)v + 2];
        return;
    }
    if (M.nbatch) {
        const BatchBrick& I = M.batch[batch_find(M.vstart, M.nbatch, v)];
        brick_coord(I.b, v - I.v0, x);
        return;
    }
    brick_coord(M.b, v, x);
}

// ---------------------------------------------------------------------------
// device buffers
// ---------------------------------------------------------------------------
template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;    // elements
    size_t cap = 0;  // capacity
};

// Sliced ELLPACK (SELL-32-sigma) copy of a CSR matrix for the Krylov kernels:
// rows are sorted by length inside windows of 512 rows, cut into slices of 32,
// each slice padded to its longest row and stored column-major, so that lane l
// of a warp streams row perm[32s+l] with coalesced loads and little padding.
struct Sell {
    int64_t nslices = 0, npad = 0;
    int32_t* perm = nullptr; // nslices*32: row of each slot (-1: none)
    int32_t* ptr = nullptr;  // nslices+1 offsets (elements)
    int32_t* col = nullptr;  // npad
    int32_t* src = nullptr;  // npad: CSR index or -1 for padding
    double* v64 = nullptr;
    float* v32 = nullptr;
    float2* v2f = nullptr;   // npad: row-scaled FP64 values as FP32 pairs hi + lo
    int32_t* rexp = nullptr; // nslices*32: row scale exponent (value = (hi + lo) * 2^rexp)
    int64_t pattern_gen = -1, v64_version = -1, v32_version = -1, v2f_version = -1;
    bool v2f_ok = false;     // every value finite (else the pair form is not used)
    // resident PCG (krylov_res.cu): row -> slot map, columns translated to the
    // owning block's vector, per-block halo lists, sizes of the largest run
    int32_t* iperm = nullptr;
    int64_t iperm_gen = -1;
    uint16_t* col_tr = nullptr;
    int32_t* halo_rows = nullptr;  // [block][halo capacity]
    int32_t* halo_n = nullptr;     // [block]
    int res_blocks = 0, res_smax = 0, res_hmax = 0;
    int32_t res_maxslots = 0;
    bool res_ok = false;
};

// measured choices for one matrix structure (rows, stored entries, SELL slots)
struct TuneEntry {
    int64_t m = 0, nnz = 0, npad = 0;
    int spmv_threads = 0, spmv_per_sm = 0;  // 0: not tuned yet
    int pcg_kind = -1;                      // -1: not tuned yet
    float spmv_us[4] = {}, pcg_us[3] = {};  // measured times of the candidates
};

struct CSR {
    int64_t m = 0, nnz = 0;
    int64_t pattern_gen = 0;    // bumps whenever the pattern changes
    Sell sell;
    int32_t* rowptr = nullptr;  // m+1 (device)
    int32_t* colind = nullptr;  // nnz
    double* vals = nullptr;     // nnz
    float* vals32 = nullptr;    // nnz (mixed precision copy, on demand)
    double* diag = nullptr;     // m (Jacobi)
    bool own_pattern = false;
    int64_t version = 0;        // bumps whenever values change
    int64_t vals32_version = -1, diag_version = -1;
};

struct KernelTimer {
    double total_ms = 0;
    int64_t launches = 0;
};

struct Context {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int num_sms = 0;
    // mesh
    MeshView mesh{};
    bool has_mesh = false;
    DBuf<double> coords;
    DBuf<int32_t> tet_v, tet_e, edge_v;
    // level set
    DBuf<double> ls_vert, ls_edge;
    bool has_ls = false;
    int64_t ls_version = 0;
    // DOFs
    int fe = 0;  // TF_P1IF / TF_P2IF, 0 = none
    int64_t n_active = 0, n_dofs = 0;
    int64_t dof_version = 0;
    bool legacy_numbering = false;
    int64_t legacy_n_active = 0;  // active tets as CreateNumbOnInterfaceVertex counts them
    DBuf<int32_t> dof_vert, dof_edge, active, loc2glo;
    // rows of the DistributeDOFs numbering in Morton order of their nodes on the
    // brick (the SELL windows of the solvers follow it), for dof_order_version
    DBuf<int32_t> dof_order;
    DBuf<unsigned long long> order_keys;
    DBuf<unsigned char> order_tmp;
    int64_t dof_order_version = -1;
    DBuf<uint8_t> flags;
    DBuf<int32_t> keys_v, keys_e, owner;
    // pattern
    int64_t pattern_dof_version = -1;
    DBuf<int32_t> rowptr, colind, seg_start, row_cursor, diag_slot;
    DBuf<uint64_t> contrib;  // sorted (col << 32 | contribution) per row
    DBuf<double> elem;       // packed element matrices [form][tet][nsym]
    DBuf<double> elem_rhs;   // [tet][nl]
    DBuf<uint8_t> legacy_mask;  // legacy forms: tet has a non-empty patch
    CSR mats[TF_NUM_MATS];
    DBuf<double> mat_vals[TF_NUM_MATS];
    DBuf<int32_t> block_rowptr, block_colind, user_rowptr, user_colind;
    DBuf<float> mat_vals32[TF_NUM_MATS];
    DBuf<double> mat_diag[TF_NUM_MATS];
    DBuf<double> vecs[TF_NUM_VECS];
    // Krylov workspaces
    DBuf<double> kry64, kry_part, kry_resid;
    DBuf<float> kry32;
    DBuf<unsigned> kry_bar;
    DBuf<int> kry_iters;
    // scratch
    DBuf<unsigned char> scratch;
    DBuf<int64_t> scan_tmp;
    DBuf<int> status;  // device status word(s)
    int* h_status = nullptr;  // pinned
    // timing
    bool timing = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t markers[8] = {};
    DBuf<double> wind_v, wind_e;  // N_P1P1 wind, xyz per vertex / edge
    bool has_wind = false;
    int ch_flags = 0;             // TF_CH_DEGENERATE_MOBILITY | TF_CH_WIND for the time loops
    DBuf<double> elem_n;          // N_P1P1 element matrices [n_active][16] (full, row i col j)
    DBuf<unsigned char> flush_buf;
    DBuf<uint4> stream_buf;  // tf_stream_read_timed
    KernelTimer timers[TF_NUM_KERNELS];
    int64_t launches = 0;
    int last_refinements = 0;  // FP64 residual replacements of the last mixed solve
    int kry_blocks_per_sm = 0; // cap on resident Krylov blocks per SM (0: occupancy limit)
    int kry_threads = 512;     // block size of the mixed-precision PCG (256 or 512)
    bool pcg_two_barrier = false;  // mixed PCG: classic two-barrier kernel instead of the single-barrier one
    bool gmres2_master = false;    // CGS2 GMRES: master-block grid steps instead of the all-reduce ones
    int64_t pattern_counter = 0, block_src_gen = -1;
    DBuf<int32_t> sell_ptr[TF_NUM_MATS], sell_col[TF_NUM_MATS], sell_src[TF_NUM_MATS], sell_perm[TF_NUM_MATS];
    DBuf<double> sell_v64[TF_NUM_MATS];
    DBuf<float> sell_v32[TF_NUM_MATS];
    DBuf<float2> sell_v2f[TF_NUM_MATS];
    DBuf<int32_t> sell_rexp[TF_NUM_MATS];
    DBuf<int32_t> sell_iperm[TF_NUM_MATS], sell_halo[TF_NUM_MATS];
    DBuf<uint16_t> sell_coltr[TF_NUM_MATS];
    bool pcg_resident = true;   // PCG: block share of the system resident in shared memory where it fits
    bool autotune = true;       // measured launch shapes per matrix structure (tune.cu)
    bool spmv_shape_fixed = false, pcg_shape_fixed = false;  // set by the environment switches
    std::vector<TuneEntry> tuned;
    DBuf<double> tune_buf;
    cudaEvent_t tune_ev[2] = {};
    int pcg_fp64_kernel = 0;    // TF_PCG_FP64_CLASSIC or TF_PCG_FP64_CG1
    int pcg_res_vcap_kb = -1;   // resident PCG: cap on the KB of matrix values kept in shared memory (-1: none)
    cudaMemPool_t refine_pool = nullptr;  // device memory of the refinement engine, kept between calls
    double pcg_rel_update = 0.2;  // mixed resident PCG: FP64 refinement when the FP32 residual dropped by this
    double batch_rel_update = 0.2;  // mixed batched PCG: the same factor
    DBuf<float2> x_pairs;       // SpMV operand split into FP32 pairs
    bool spmv_pair = false;     // tf_spmv: FP32-pair kernel instead of the FP64-FMA one
    bool asm_fp64 = false;      // P2 forms: the FP64 kernel instead of the FP32-pair one
    bool locality_order = true; // SELL windows of the DOF pattern in the Morton order of the DOFs' nodes
    bool spmv_sell = false;     // tf_spmv: one warp per slice instead of the balanced kernel
    bool pcg_blocked = true;    // mixed PCG: contiguous slices per block, balanced within the block
    int pcg_smem_cache_kb = 0;  // mixed PCG: KB of the block's FP32 matrix slots kept in shared memory (0: off)
    int spmv_blocks_per_sm = 0; // balanced SpMV launch shape (0: default)
    int spmv_threads = 512;
    // batch of bricks (tf_mesh_brick_batch); 0 = single mesh
    int batch_count = 0;
    DBuf<BatchBrick> batch_tab;
    DBuf<int64_t> batch_start;        // tet, vertex, edge starts (3 x (count+1))
    DBuf<unsigned char> batch_ls;     // per-instance level-set parameters
    std::vector<int64_t> h_batch_tstart, h_batch_vstart, h_batch_estart;
    // per-instance ranges after numbering: cut tets and rows (count+1 each)
    int64_t batch_dof_version = -1;
    std::vector<int64_t> h_batch_cut, h_batch_rows;
    DBuf<int64_t> batch_rows;         // device: row starts, then cut-tet starts (2 x (count+1))
    // batched PCG
    DBuf<double> batch_coef, batch_resid, batch_xtmp;
    DBuf<int> batch_queue, batch_iters;
    DBuf<int32_t> batch_order;
    std::vector<int64_t> h_batch_nnz;
    int64_t batch_order_gen = -1;
    std::vector<int64_t> batch_tuned_key;              // batch structure the tuned shape belongs to
    DBuf<int64_t> batch_nnz;
    bool batch_use_graph = true;
    int batch_lanes = 0, batch_threads = 0;             // autotuned
    int batch_fixed_lanes = 0, batch_fixed_threads = 0; // set by tf_batch_config (0: autotune)
    double* h_batch_out = nullptr;                      // pinned: iterations, then residuals
    cudaGraphExec_t batch_exec = nullptr;
    std::vector<int64_t> batch_graph_key;
    // learned warm start (per-DOF MLP)
    DBuf<float> mlp_w, mlp_m1, mlp_m2, mlp_grad, mlp_lossacc;
    DBuf<__nv_bfloat16> mlp_w16, mlp_xio;
    DBuf<float> mlp_yio, mlp_pio;
    int64_t mlp_step = 0;
    // learned Cahn-Hilliard warm start
    DBuf<double> ch_part, ch_scales, ch_hist;
    DBuf<double> ch_ring, ch_av;
    DBuf<double> qq_grad;  // isoparametric P2: recovered level-set gradient per interface DOF
    DBuf<double> qq_base;   // isoparametric P2: per cut tet its data, per quadrature point the base point and the point data
    DBuf<int32_t> qq_idx;   // isoparametric P2: points per tet, their offsets, each point's tet
    DBuf<uint32_t> prep_key;      // pair forms: sort keys of the prep threads (2 x chunk)
    DBuf<int32_t> prep_idx;       // and their tets (2 x chunk)
    DBuf<unsigned char> prep_tmp;
    bool prep_sort = true;        // prep threads ordered by the tets' sign patterns
    DBuf<unsigned char> prep1;  // P1 pair forms: per-tet records of one chunk of active tets
    DBuf<double> ch_prev, ch_x1, ch_x2;  // adaptive BDF1/BDF2: chi_prev, BDF1 and BDF2 states
    DBuf<float> ch_xyz, ch_nrm, ch_Y, ch_pred;
    DBuf<__nv_bfloat16> ch_X;
    int64_t ch_geom_version = -1;
    double ch_train_loss = 0.;
    // CGS2 GMRES: B = A P^{-1} in SELL order, block inverses, bases
    DBuf<float> gm2_b32, gm2_v32;
    DBuf<double> gm2_b64, gm2_v64, gm2_binv;
    int64_t gm2_src_version[2] = {-1, -1}, gm2_src_gen[2] = {-1, -1};
    int gmres_orth = TF_ORTH_MGS;
};

struct ChLearnParams {
    int nsteps = 0;
    double dt = 0., mob = 1., eps = 0., beta_s = 0., xi = 0., rho_vol = 0.;
    int restart = 50;
    double tol = 1e-10;
    int max_iter = 100000;
    int precision = TF_PREC_FP64;  // TF_PREC_MIXED: FP32 Arnoldi cycles in FP64 refinement
    int learned = 1;        // 0: previous-step guess (the reference's warm start), 1: projection with the MLP's
                            // correction, 2: linear extrapolation, 3: projection without the MLP
    int train_steps = 100;  // online training during the first steps
    int epochs = 2;
    int mb_tiles = 16;      // tiles of 128 DOFs per mini-batch
    float lr = 1e-3f;
    int min_trained = 3;    // training steps before the first learned guess
};

constexpr int kMaxBatchInstances = 65536;

// ---------------------------------------------------------------------------
// error handling helpers (host)
// ---------------------------------------------------------------------------
int set_err(Context* c, int code, const std::string& msg);
#define TF_CUDA(ctx, call)                                                                          \
    do {                                                                                            \
        cudaError_t e__ = (call);                                                                   \
        if (e__ != cudaSuccess)                                                                     \
            return ::tf::set_err((ctx), TF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e__)); \
    } while (0)
#define TF_TRY(expr)             \
    do {                         \
        int s__ = (expr);        \
        if (s__ != TF_OK) return s__; \
    } while (0)

template <class T>
int ensure(Context* c, DBuf<T>& b, size_t n) {
    if (b.cap < n) {
        if (b.p) cudaFree(b.p);
        b.p = nullptr;
        b.cap = 0;
        size_t bytes = (n > 0 ? n : 1) * sizeof(T);
        cudaError_t e = cudaMalloc((void**)&b.p, bytes);
        if (e != cudaSuccess) return set_err(c, TF_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        b.cap = n > 0 ? n : 1;
    }
    b.n = n;
    return TF_OK;
}
template <class T>
void release(DBuf<T>& b) {
    if (b.p) cudaFree(b.p);
    b = DBuf<T>();
}

// kernel timing around one launch (events on the context stream)
struct TimedLaunch {
    Context* c;
    int k;
    TimedLaunch(Context* ctx, int kernel);
    ~TimedLaunch();
};

// device-wide exclusive scan of int32 counts -> int64 offsets (out[n] = total)
int exclusive_scan_i32(Context* c, const int32_t* in, int64_t* out, int64_t n);
int exclusive_scan_i32_to_i32(Context* c, const int32_t* in, int32_t* out, int64_t n, int64_t* total);
// *order: the rows of the current DistributeDOFs numbering in Morton order of
// their nodes, or nullptr where there is none (explicit or batch meshes)
int dof_locality_order(Context* c, const int32_t** order);
int sync_status(Context* c, int* status_out);
int fill_f64(Context* c, double* p, int64_t n, double v);

// sub-module entry points (host)
int mesh_materialise(Context* c, double* coords, int32_t* tet_v, int32_t* tet_e, int32_t* edge_v);

// narrow-band refinement (refine.cu): the last triangulation level of
// MakeInitialTriang on a level-0 mesh, vertices and edges by first touch
struct RefinedMesh {
    std::vector<double> coords;
    std::vector<int32_t> tet_v, tet_e, edge_v, tet_level;
    std::vector<int64_t> per_level;
    int last_level = 0;
    int steps = 0;
};
int refine_band(int64_t nv, const double* coords, int64_t nt, const int32_t* tet_v, int kind, const double* par,
                int npar, double width, int clevel, int flevel, RefinedMesh& out);
// the data-parallel form of the same refinement (refine_par.cu): on the host
// (its kernel bodies as loops), and on the device for a context's mesh
int refine_band_parallel_host(int64_t nv, const double* coords, int64_t nt, const int32_t* tet_v, int kind,
                              const double* par, int npar, double width, int clevel, int flevel, RefinedMesh& out);
int refine_band_device(Context* c, int kind, const double* par, int npar, double width, int clevel, int flevel,
                       int* last_level, int* steps);
int ensure_tables(Context* c);
int patch_dump(Context* c, const int32_t* tets, int64_t count, int32_t* nf, int32_t* facets, int32_t* bnd,
               int32_t* nverts, double* verts);
int mesh_set_brick(Context* c, const double orig[3], const double e1[3], const double e2[3], const double e3[3],
                   int n1, int n2, int n3);
int levelset_analytic(Context* c, int kind, const double* par, int npar, int p2, int count);
int mesh_set_brick_batch(Context* c, int count, const int32_t* n, const double* orig, const double* axes);
int levelset_p1_edges(Context* c);
int distribute_dofs(Context* c, int fe, double dist);
int numb_on_interface_p1(Context* c, double omit_bound);
int setup_fe_system(Context* c, unsigned forms, int rhs_kind, const double* rhs_par, int npar);
int setup_legacy_p1(Context* c, double alpha, double D, const double* fpar, int64_t* nnz);
int lincomb(Context* c, int nterms, const int* forms, const double* coeffs);
int ch_block(Context* c, double alpha, double mob, double rho, double eps2, double beta, int flags);
int ch_loop_begin(Context* c);
int ch_step_block(Context* c, double alpha, double mob, double rho, double eps2, double beta);
int spmv(Context* c, const CSR& A, const double* x, double* y);
int pcg_jacobi(Context* c, CSR& A, const double* b, double* x, int precision, int* max_iter, double* tol, int rel);
template <class T>
int pcg_resident(Context* c, CSR& A, const double* b, double* x, int* max_iter, double* tol, int rel, bool* applied);
// kinds of the single-barrier mixed PCG (autotuned per matrix structure, tune.cu)
constexpr int kPcgResident = 0, kPcgCg1_512 = 1, kPcgCg1_256 = 2;
int pcg_mixed_kind(Context* c, CSR& A, const double* b, double* x, int kind, int* max_iter, double* tol, int rel);
void launch_spmv_shape(Context* c, const CSR& A, const double* x, double* y, int threads, int per_sm);
int tuned_spmv_shape(Context* c, CSR& A, int* threads, int* per_sm);
int tuned_pcg_kind(Context* c, CSR& A, const double* b, int* kind);
int gmres_jacobi(Context* c, CSR& A, const double* b, double* x, int restart, int method, int precision,
                 int* max_iter, double* tol, int rel);
int ensure_diag(Context* c, CSR& A);
int coop_blocks(Context* c, const void* fn, int64_t nslices, int* out, int threads, size_t dyn_smem = 0);
int gmres2(Context* c, CSR& A, const double* b, double* x, int restart, bool mixed, int* max_iter, double* tol, int rel);
int ch_steps(Context* c, int nsteps, double dt, double mob, double eps, double beta_s, double xi, double rho_vol,
             int restart, double tol, int max_iter, int warm, int* iters, double* resids);
void release_solver_workspace(Context* c);
int batch_ranges(Context* c);
int batch_lincomb(Context* c, int nterms, const int* forms, const double* coeffs);
int batch_tune(Context* c, CSR& A, const double* b, bool mixed, int* lanes_out, int* threads_out);
int batch_pcg(Context* c, CSR& A, const double* b, double* x, int precision, int max_iter, double tol, int rel,
              int* iters, double* resids);
int batch_config(Context* c, int lanes, int threads, int use_graph);
void release_batch(Context* c);
int mlp_init(Context* c, uint64_t seed);
int mlp_set_weights(Context* c, const float* w);
int mlp_get_weights(Context* c, float* w);
int mlp_forward_dev(Context* c, const __nv_bfloat16* X, int64_t n, float* pred);
int ch_rhs(Context* c, const double* X, double dt, double beta_s, double xi);
int ch_stats(Context* c, double eps, double xi, double* out);
int ch_steps_adaptive(Context* c, const tf_ch_adapt_params& P, int* nsteps, double* t_end, double* dts, double* errs,
                      int* tries, int* iters);
int ch_geometry(Context* c);
int ch_features_dev(Context* c, const double* xn, const double* xp, const double* xnext);
int ch_steps_learned(Context* c, const ChLearnParams& P, int* iters, double* resids, int* used);
int mlp_epoch_dev(Context* c, const __nv_bfloat16* X, const float* Y, int64_t n, int mb_tiles, float lr, float* gsum,
                  double* loss);
int ensure_vals32(Context* c, CSR& A);
int quaqua_elements(Context* c, double rhs_c, double tol, int maxiter, int* newton_max);
int setup_quaqua_p2(Context* c, double rhs_c, double tol, int maxiter, int* newton_max);
int ensure_sell(Context* c, CSR& A, bool fp32);

// matrix handles that hold an assembled form
inline bool is_form_handle(int f) { return (f >= 0 && f < TF_NUM_FORMS) || f == TF_FORM_N; }

constexpr int kBlock = 256;
inline int grid_for(Context* c, int64_t n, int block = kBlock, int per_sm = 8) {
    int64_t g = (n + block - 1) / block;
    int64_t cap = (int64_t)c->num_sms * per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace tf
