// Locality order of the interface DOFs for the solvers' SELL layout.
//
// The first-touch numbering of DistributeDOFs follows the tets in brick order,
// so 512 consecutive rows (one SELL window) form a thin slab of the surface,
// and a solver block that owns a contiguous run of windows references about
// twice its own rows in other blocks (2,006 against 955 on the P2 sphere at
// 96^3).  Ordering the rows by the Morton code of their nodes on the brick
// grid makes every run a compact patch: 1,091 halo rows.  The order only
// decides which rows share a window; the numbering, the matrices and every
// result vector keep the DistributeDOFs numbering.
#include <algorithm>

#include <cub/device/device_radix_sort.cuh>

#include "tf_internal.cuh"

namespace tf {

namespace {

// 21 bits of x spread to every third bit
__device__ __forceinline__ unsigned long long spread3(unsigned x) {
    unsigned long long v = x & 0x1fffffu;
    v = (v | v << 32) & 0x1f00000000ffffull;
    v = (v | v << 16) & 0x1f0000ff0000ffull;
    v = (v | v << 8) & 0x100f00f00f00f00full;
    v = (v | v << 4) & 0x10c30c30c30c30c3ull;
    v = (v | v << 2) & 0x1249249249249249ull;
    return v;
}

// every row first: the largest key (rows no node claims sort last), the row itself
__global__ void k_order_init(int64_t m, unsigned long long* __restrict__ keys, int32_t* __restrict__ rows) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        keys[i] = ~0ull;
        rows[i] = (int32_t)i;
    }
}

// the Morton key of each numbered node's doubled grid position (a brick), or
// of its position on a 2^20 grid over the bounding box (an uploaded mesh: the
// vertex, or the edge's midpoint); edge nodes only for a P2 numbering (a P1
// numbering leaves dof_edge unset)
__global__ void k_dof_morton(MeshView M, const int32_t* __restrict__ dof_vert, const int32_t* __restrict__ dof_edge,
                             int p2, int64_t m, unsigned long long* __restrict__ keys) {
    const int64_t total = M.nv + (p2 ? M.ne : 0);
    for (int64_t node = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; node < total;
         node += (int64_t)gridDim.x * blockDim.x) {
        const int32_t dof = node < M.nv ? dof_vert[node] : dof_edge[node - M.nv];
        if (dof < 0 || dof >= m) continue;
        int g[3];
        if (M.explicit_mesh) {
            double x[3];
            if (node < M.nv) {
                for (int k = 0; k < 3; ++k) x[k] = M.coords[3 * node + k];
            } else {
                const int32_t a = M.edge_v[2 * (node - M.nv)], b = M.edge_v[2 * (node - M.nv) + 1];
                for (int k = 0; k < 3; ++k) x[k] = 0.5 * (M.coords[3 * (int64_t)a + k] + M.coords[3 * (int64_t)b + k]);
            }
            for (int k = 0; k < 3; ++k) g[k] = (int)fmin(fmax((x[k] - M.bb_lo[k]) * M.bb_scale[k], 0.0), 2097151.0);
        } else {
            brick_node_grid2(M.b, node, M.nv, g);
        }
        keys[dof] = spread3((unsigned)g[0]) | spread3((unsigned)g[1]) << 1 | spread3((unsigned)g[2]) << 2;
    }
}

}  // namespace

int dof_locality_order(Context* c, const int32_t** order) {
    *order = nullptr;
    const MeshView& M = c->mesh;
    if (M.nbatch || c->legacy_numbering || (c->fe != TF_P1IF && c->fe != TF_P2IF) || c->n_dofs <= 0) return TF_OK;
    if (!M.explicit_mesh && 2 * (int64_t)std::max({M.b.n1, M.b.n2, M.b.n3}) + 1 >= (1 << 21)) return TF_OK;
    const int64_t m = c->n_dofs;
    if (c->dof_order_version != c->dof_version) {
        TF_TRY(ensure(c, c->order_keys, (size_t)(2 * m)));
        TF_TRY(ensure(c, c->dof_order, (size_t)(2 * m)));
        unsigned long long* kin = c->order_keys.p;
        int32_t* rin = c->dof_order.p + m;
        const int p2 = c->fe == TF_P2IF;
        k_order_init<<<grid_for(c, m), kBlock, 0, c->stream>>>(m, kin, rin);
        k_dof_morton<<<grid_for(c, M.nv + (p2 ? M.ne : 0)), kBlock, 0, c->stream>>>(M, c->dof_vert.p,
                                                                                   p2 ? c->dof_edge.p : nullptr, p2, m,
                                                                                   kin);
        c->launches += 2;
        TF_CUDA(c, cudaGetLastError());
        size_t bytes = 0;
        TF_CUDA(c, cub::DeviceRadixSort::SortPairs(nullptr, bytes, kin, kin + m, rin, c->dof_order.p, (int)m, 0, 63,
                                                  c->stream));
        TF_TRY(ensure(c, c->order_tmp, bytes > 0 ? bytes : 1));
        TF_CUDA(c, cub::DeviceRadixSort::SortPairs(c->order_tmp.p, bytes, kin, kin + m, rin, c->dof_order.p, (int)m, 0,
                                                  63, c->stream));
        c->launches += 4;  // the radix sort's passes
        c->dof_order_version = c->dof_version;
    }
    *order = c->dof_order.p;
    return TF_OK;
}

}  // namespace tf
