// Cut classification and interface DOF numbering.
//
// IdxDescCL::DistributeDOFs (misc/problem.cpp:283-336) walks the tets in
// triangulation order and gives every vertex (and, for P2, edge) of an active
// tet the next number on first touch.  Here that serial walk becomes three
// data-parallel steps with the same result:
//   1. classify: one thread per tet evaluates distance() on its 10 level-set
//      values (geom/subtriangulation.tpp:38-46) and writes an activity flag;
//      the active tets are compacted in tet order by a device-wide scan;
//   2. first touch: each active tet r offers the key r*nloc + slot to each of
//      its vertices/edges with atomicMin -- the minimum key is exactly the
//      position of the first touch in the reference's walk;
//   3. ranking: the keys are unique, so a scan over the key space turns every
//      owned key into its DOF number.
#include <climits>
#include <cstring>

#include "tf_internal.cuh"

namespace tf {

__device__ inline void set_status(int* st, int code, int64_t where) {
    if (atomicCAS(st, 0, code) == 0) st[1] = (int)where;
}

// The distance test on the IEEE-754 bit patterns, with integer operations
// only: GB300 issues FP64 compares on its narrow FP64 pipe, and ten values per
// tet made classification FP64-bound.  For a double with bits b and
// magnitude bits m = b & 0x7ff..f: sign(d) (misc/utils.h:810-813) is 0 for
// m == 0 (+-0) and for NaN (m > 0x7ff0..0, where both comparisons of sign()
// are false), else -1 or +1 by the sign bit; for non-NaN values |a| < |c| iff
// m_a < m_c, so min |f| is the minimum of the m.
struct DistTest {
    unsigned long long dmag;  // magnitude bits of dist (when dist >= 0)
    int dmag_ok;              // dist >= 0: min |f| <= dist is dmag compare
    int mixed_active;         // 0 <= dist: a tet with a sign change is active
};

__global__ void k_classify(MeshView M, const double* __restrict__ lsv, const double* __restrict__ lse, DistTest D,
                           int32_t* __restrict__ flags, int* __restrict__ status) {
    const long long* bv = reinterpret_cast<const long long*>(lsv);
    const long long* be = reinterpret_cast<const long long*>(lse);
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < M.nt; t += (int64_t)gridDim.x * blockDim.x) {
        int32_t v[4], e[6];
        mesh_tet(M, t, v, e);
        long long f[10];
        for (int k = 0; k < 4; ++k) f[k] = __ldg(bv + v[k]);
        for (int k = 0; k < 6; ++k) f[4 + k] = __ldg(be + e[k]);
        int sum = 0, zeros = 0;
        unsigned long long mn = ~0ull;
        for (int k = 0; k < 10; ++k) {
            const unsigned long long m = (unsigned long long)f[k] & 0x7fffffffffffffffull;
            const bool zero = m == 0ull, nan = m > 0x7ff0000000000000ull;
            sum += (zero || nan) ? 0 : (f[k] < 0 ? -1 : 1);
            zeros += zero;
            mn = m < mn ? m : mn;
        }
        int active;
        if (sum == 10 || sum == -10) {
            active = D.dmag_ok && mn <= D.dmag;  // distance() = min |f| <= dist
        } else {
            if (zeros) set_status(status, TF_ERR_ZERO_NODE, t);
            active = D.mixed_active;  // distance() = 0 <= dist
        }
        flags[t] = active;
    }
}

__global__ void k_compact(int64_t n, const int32_t* __restrict__ flags, const int32_t* __restrict__ pos,
                          int32_t* __restrict__ out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        if (flags[t]) out[pos[t]] = (int32_t)t;
}

__global__ void k_fill_i32(int32_t* p, int64_t n, int32_t v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

__global__ void k_first_touch(MeshView M, int64_t n_active, const int32_t* __restrict__ active, int p2,
                              int32_t* __restrict__ kv, int32_t* __restrict__ ke) {
    const int nl = p2 ? 10 : 4;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_active; r += (int64_t)gridDim.x * blockDim.x) {
        int32_t v[4], e[6];
        mesh_tet(M, active[r], v, p2 ? e : nullptr);
        const int32_t base = (int32_t)(r * nl);
        for (int s = 0; s < 4; ++s) atomicMin(&kv[v[s]], base + s);
        if (p2)
            for (int s = 0; s < 6; ++s) atomicMin(&ke[e[s]], base + 4 + s);
    }
}

__global__ void k_mark_owned(int64_t n, const int32_t* __restrict__ keys, int32_t* __restrict__ owned) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t k = keys[i];
        if (k != INT_MAX) owned[k] = 1;
    }
}

__global__ void k_assign(int64_t n, const int32_t* __restrict__ keys, const int32_t* __restrict__ rank,
                         int32_t* __restrict__ dof) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t k = keys[i];
        dof[i] = k != INT_MAX ? rank[k] : -1;
    }
}

__global__ void k_loc2glo(MeshView M, int64_t n_active, const int32_t* __restrict__ active, int p2,
                          const int32_t* __restrict__ dv, const int32_t* __restrict__ de, int32_t* __restrict__ l2g) {
    const int nl = p2 ? 10 : 4;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_active; r += (int64_t)gridDim.x * blockDim.x) {
        int32_t v[4], e[6];
        mesh_tet(M, active[r], v, p2 ? e : nullptr);
        for (int s = 0; s < 4; ++s) l2g[r * nl + s] = dv[v[s]];
        if (p2)
            for (int s = 0; s < 6; ++s) l2g[r * nl + 4 + s] = de[e[s]];
    }
}

// active tets -> compacted list (tet order); flags must hold 0/1 per tet
int compact_active(Context* c, int64_t* n_active) {
    const int64_t nt = c->mesh.nt;
    TF_TRY(ensure(c, c->owner, (size_t)nt + 1));  // reused as scan output
    TF_TRY(exclusive_scan_i32_to_i32(c, (const int32_t*)c->scratch.p, c->owner.p, nt, n_active));
    TF_TRY(ensure(c, c->active, (size_t)(*n_active > 0 ? *n_active : 1)));
    k_compact<<<grid_for(c, nt), kBlock, 0, c->stream>>>(nt, (const int32_t*)c->scratch.p, c->owner.p, c->active.p);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    return TF_OK;
}

int number_from_active(Context* c, int p2) {
    const MeshView& M = c->mesh;
    const int nl = p2 ? 10 : 4;
    const int64_t na = c->n_active;
    if (na * nl >= INT_MAX) return set_err(c, TF_ERR_CAPACITY, "too many active tets for 32-bit DOF keys");
    TimedLaunch tl(c, TF_K_NUMBER);
    TF_TRY(ensure(c, c->keys_v, (size_t)M.nv));
    TF_TRY(ensure(c, c->dof_vert, (size_t)M.nv));
    k_fill_i32<<<grid_for(c, M.nv), kBlock, 0, c->stream>>>(c->keys_v.p, M.nv, INT_MAX);
    ++c->launches;
    if (p2) {
        TF_TRY(ensure(c, c->keys_e, (size_t)M.ne));
        TF_TRY(ensure(c, c->dof_edge, (size_t)M.ne));
        k_fill_i32<<<grid_for(c, M.ne), kBlock, 0, c->stream>>>(c->keys_e.p, M.ne, INT_MAX);
        ++c->launches;
    }
    if (na > 0) {
        k_first_touch<<<grid_for(c, na), kBlock, 0, c->stream>>>(M, na, c->active.p, p2, c->keys_v.p, c->keys_e.p);
        ++c->launches;
    }
    const int64_t nkeys = na * nl;
    TF_TRY(ensure(c, c->owner, (size_t)nkeys + 1));
    TF_CUDA(c, cudaMemsetAsync(c->owner.p, 0, sizeof(int32_t) * (size_t)(nkeys + 1), c->stream));
    k_mark_owned<<<grid_for(c, M.nv), kBlock, 0, c->stream>>>(M.nv, c->keys_v.p, c->owner.p);
    ++c->launches;
    if (p2) {
        k_mark_owned<<<grid_for(c, M.ne), kBlock, 0, c->stream>>>(M.ne, c->keys_e.p, c->owner.p);
        ++c->launches;
    }
    TF_TRY(ensure(c, c->loc2glo, (size_t)(nkeys > 0 ? nkeys : 1) + 1));  // scan output, then loc2glo
    int64_t ndofs = 0;
    TF_TRY(exclusive_scan_i32_to_i32(c, c->owner.p, c->loc2glo.p, nkeys, &ndofs));
    k_assign<<<grid_for(c, M.nv), kBlock, 0, c->stream>>>(M.nv, c->keys_v.p, c->loc2glo.p, c->dof_vert.p);
    ++c->launches;
    if (p2) {
        k_assign<<<grid_for(c, M.ne), kBlock, 0, c->stream>>>(M.ne, c->keys_e.p, c->loc2glo.p, c->dof_edge.p);
        ++c->launches;
    }
    if (na > 0) {
        k_loc2glo<<<grid_for(c, na), kBlock, 0, c->stream>>>(M, na, c->active.p, p2, c->dof_vert.p,
                                                              p2 ? c->dof_edge.p : nullptr, c->loc2glo.p);
        ++c->launches;
    }
    TF_CUDA(c, cudaGetLastError());
    c->n_dofs = ndofs;
    c->fe = p2 ? TF_P2IF : TF_P1IF;
    ++c->dof_version;
    return TF_OK;
}

int distribute_dofs(Context* c, int fe, double dist) {
    if (!c->has_mesh || !c->has_ls) return set_err(c, TF_ERR_BAD_INPUT, "distribute_dofs: mesh and level set required");
    if (fe != TF_P1IF && fe != TF_P2IF) return set_err(c, TF_ERR_BAD_INPUT, "distribute_dofs: fe must be TF_P1IF or TF_P2IF");
    const MeshView& M = c->mesh;
    c->fe = 0;
    c->legacy_numbering = false;
    TF_TRY(ensure(c, c->scratch, (size_t)M.nt * sizeof(int32_t)));
    TF_CUDA(c, cudaMemsetAsync(c->status.p, 0, 4 * sizeof(int), c->stream));
    {
        TimedLaunch tl(c, TF_K_CLASSIFY);
        DistTest D;
        D.dmag_ok = dist >= 0.;
        D.dmag = 0;
        if (D.dmag_ok) {
            std::memcpy(&D.dmag, &dist, sizeof(double));
            D.dmag &= 0x7fffffffffffffffull;
        }
        D.mixed_active = 0. <= dist;
        k_classify<<<grid_for(c, M.nt), kBlock, 0, c->stream>>>(M, c->ls_vert.p, c->ls_edge.p, D,
                                                                  (int32_t*)c->scratch.p, c->status.p);
        ++c->launches;
        TF_CUDA(c, cudaGetLastError());
        int st = 0;
        TF_TRY(sync_status(c, &st));
        if (st != 0)
            return set_err(c, st, "distance: level set is exactly zero at a node of a cut tet (tet " +
                                      std::to_string(c->h_status[1]) + ")");
        TF_TRY(compact_active(c, &c->n_active));
    }
    return number_from_active(c, fe == TF_P2IF);
}

}  // namespace tf
