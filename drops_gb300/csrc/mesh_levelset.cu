// Mesh (implicit Kuhn brick) and level-set evaluation.
//
// This translation unit is compiled with -fmad=false: every product and sum
// rounds separately, so vertex coordinates and level-set values equal the
// reference's host arithmetic bit for bit (BrickBuilderCL::build_ser_impl,
// geom/builder.cpp:112-118; LSInit / LinearLSInit, surfactant/surfactant.cpp:733-758;
// Sphere::dist / Torus::dist, surfactant/Surface.hpp:71,130).  Exact values
// matter: the sign of every level-set value decides cut classification and
// the patch topology.
#include "tf_internal.cuh"

namespace tf {

// Brick geometry of n1 x n2 x n3 cubes spanned by e1, e2, e3 from orig;
// returns false when the ids would not fit 32 bits.
static bool make_brick(const double orig[3], const double e1[3], const double e2[3], const double e3[3], int n1,
                       int n2, int n3, Brick& B, int64_t& nv, int64_t& ne, int64_t& nt) {
    B = Brick{};
    B.n1 = n1; B.n2 = n2; B.n3 = n3;
    for (int k = 0; k < 3; ++k) {
        B.orig[k] = orig[k];
        B.o1[k] = (1.0 / (double)n1) * e1[k];
        B.o2[k] = (1.0 / (double)n2) * e2[k];
        B.o3[k] = (1.0 / (double)n3) * e3[k];
    }
    static const int dir[7][3] = {{0, 0, 1}, {0, 1, 0}, {1, 0, 0}, {0, 1, 1}, {1, 0, 1}, {1, 1, 0}, {1, 1, 1}};
    B.eoff[0] = 0;
    for (int t = 0; t < 7; ++t)
        B.eoff[t + 1] = B.eoff[t] + (int64_t)(n3 + 1 - dir[t][0]) * (n2 + 1 - dir[t][1]) * (n1 + 1 - dir[t][2]);
    nv = (int64_t)(n1 + 1) * (n2 + 1) * (n3 + 1);
    ne = B.eoff[7];
    nt = (int64_t)6 * n1 * n2 * n3;
    return nv <= INT32_MAX && ne <= INT32_MAX && nt <= ((int64_t)1 << 40);
}

int mesh_set_brick(Context* c, const double orig[3], const double e1[3], const double e2[3], const double e3[3],
                   int n1, int n2, int n3) {
    if (n1 < 1 || n2 < 1 || n3 < 1) return set_err(c, TF_ERR_BAD_INPUT, "brick: n1, n2, n3 must be >= 1");
    MeshView& M = c->mesh;
    M = MeshView{};
    M.explicit_mesh = 0;
    if (!make_brick(orig, e1, e2, e3, n1, n2, n3, M.b, M.nv, M.ne, M.nt))
        return set_err(c, TF_ERR_CAPACITY, "brick too large for 32-bit vertex/edge ids");
    c->has_mesh = true;
    c->has_ls = false;
    c->has_wind = false;
    c->fe = 0;
    c->batch_count = 0;
    return TF_OK;
}

// A batch of independent bricks numbered one after the other: instance i owns
// vertices [v0_i, v0_{i+1}), edges [e0_i, e0_{i+1}) and tets [t0_i, t0_{i+1}),
// and inside its ranges it is numbered exactly as tf_mesh_brick numbers it.
int mesh_set_brick_batch(Context* c, int count, const int32_t* n, const double* orig, const double* axes) {
    if (count < 1 || !n || !orig || !axes) return set_err(c, TF_ERR_BAD_INPUT, "brick batch: count and arrays required");
    std::vector<BatchBrick> tab((size_t)count);
    std::vector<int64_t> ts(count + 1), vs(count + 1), es(count + 1);
    ts[0] = vs[0] = es[0] = 0;
    for (int i = 0; i < count; ++i) {
        if (n[3 * i] < 1 || n[3 * i + 1] < 1 || n[3 * i + 2] < 1)
            return set_err(c, TF_ERR_BAD_INPUT, "brick batch: n1, n2, n3 must be >= 1");
        int64_t nv, ne, nt;
        if (!make_brick(orig + 3 * i, axes + 9 * i, axes + 9 * i + 3, axes + 9 * i + 6, n[3 * i], n[3 * i + 1],
                        n[3 * i + 2], tab[i].b, nv, ne, nt))
            return set_err(c, TF_ERR_CAPACITY, "brick batch: instance too large");
        tab[i].v0 = vs[i];
        tab[i].e0 = es[i];
        tab[i].t0 = ts[i];
        vs[i + 1] = vs[i] + nv;
        es[i + 1] = es[i] + ne;
        ts[i + 1] = ts[i] + nt;
    }
    if (vs[count] > INT32_MAX || es[count] > INT32_MAX || ts[count] > INT32_MAX)
        return set_err(c, TF_ERR_CAPACITY, "brick batch: more than 2^31 vertices, edges or tets in total");
    TF_TRY(ensure(c, c->batch_tab, (size_t)count));
    TF_TRY(ensure(c, c->batch_start, (size_t)3 * (count + 1)));
    TF_CUDA(c, cudaMemcpyAsync(c->batch_tab.p, tab.data(), sizeof(BatchBrick) * count, cudaMemcpyHostToDevice, c->stream));
    TF_CUDA(c, cudaMemcpyAsync(c->batch_start.p, ts.data(), sizeof(int64_t) * (count + 1), cudaMemcpyHostToDevice, c->stream));
    TF_CUDA(c, cudaMemcpyAsync(c->batch_start.p + (count + 1), vs.data(), sizeof(int64_t) * (count + 1),
                               cudaMemcpyHostToDevice, c->stream));
    TF_CUDA(c, cudaMemcpyAsync(c->batch_start.p + 2 * (count + 1), es.data(), sizeof(int64_t) * (count + 1),
                               cudaMemcpyHostToDevice, c->stream));
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    MeshView& M = c->mesh;
    M = MeshView{};
    M.explicit_mesh = 0;
    M.nbatch = count;
    M.nv = vs[count];
    M.ne = es[count];
    M.nt = ts[count];
    M.batch = c->batch_tab.p;
    M.tstart = c->batch_start.p;
    M.vstart = c->batch_start.p + (count + 1);
    M.estart = c->batch_start.p + 2 * (count + 1);
    c->batch_count = count;
    c->h_batch_tstart = ts;
    c->h_batch_vstart = vs;
    c->h_batch_estart = es;
    c->batch_dof_version = -1;
    c->has_mesh = true;
    c->has_ls = false;
    c->has_wind = false;
    c->fe = 0;
    return TF_OK;
}

__device__ inline void brick_edge(const Brick& B, int64_t e, int64_t v0, int32_t& a, int32_t& b) {
    int cls = 0;
    while (cls < 6 && e >= B.eoff[cls + 1]) ++cls;
    const int d3 = (cls == 2 || cls == 4 || cls == 5 || cls == 6) ? 1 : 0;
    const int d2 = (cls == 1 || cls == 3 || cls == 5 || cls == 6) ? 1 : 0;
    const int d1 = (cls == 0 || cls == 3 || cls == 4 || cls == 6) ? 1 : 0;
    int64_t k = e - B.eoff[cls];
    const int w1 = B.n1 + 1 - d1, w2 = B.n2 + 1 - d2;
    const int i1 = (int)(k % w1);
    k /= w1;
    const int i2 = (int)(k % w2);
    const int i3 = (int)(k / w2);
    a = (int32_t)(v0 + ((int64_t)i3 * (B.n2 + 1) + i2) * (B.n1 + 1) + i1);
    b = (int32_t)(v0 + ((int64_t)(i3 + d3) * (B.n2 + 1) + i2 + d2) * (B.n1 + 1) + i1 + d1);
}

// endpoints of edge e
__device__ inline void mesh_edge(const MeshView& M, int64_t e, int32_t& a, int32_t& b) {
    if (M.explicit_mesh) {
        a = M.edge_v[2 * e];
        b = M.edge_v[2 * e + 1];
        return;
    }
    if (M.nbatch) {
        const BatchBrick& I = M.batch[batch_find(M.estart, M.nbatch, e)];
        brick_edge(I.b, e - I.e0, I.v0, a, b);
        return;
    }
    brick_edge(M.b, e, 0, a, b);
}

struct LsPar {
    int kind;
    double p[16];
};

__device__ inline double nrm3(double a, double b, double c) { return sqrt(a * a + b * b + c * c); }

__device__ double ls_value(const LsPar& P, const double x[3]) {
    switch (P.kind) {
        case TF_LS_SPHERE:
            return nrm3(x[0] - P.p[0], x[1] - P.p[1], x[2] - P.p[2]) - P.p[3];
        case TF_LS_TORUS: {
            const int ax = (int)P.p[2];
            const int a0 = (ax + 1) % 3, a1 = (ax + 2) % 3;
            const double rho = sqrt(x[a0] * x[a0] + x[a1] * x[a1]) - P.p[0];
            return sqrt(rho * rho + x[ax] * x[ax]) - P.p[1];
        }
        case TF_LS_ELLIPSOID: {
            const double d0 = x[0] - P.p[0], d1 = x[1] - P.p[1], d2 = x[2] - P.p[2];
            const double* R = P.p + 6;
            double y[3];
            for (int i = 0; i < 3; ++i) y[i] = (R[i] * d0 + R[3 + i] * d1) + R[6 + i] * d2;
            return nrm3(y[0] / P.p[3], y[1] / P.p[4], y[2] / P.p[5]) - 1.0;
        }
        case TF_LS_PLANE:
            return ((P.p[0] * x[0] + P.p[1] * x[1]) + P.p[2] * x[2]) - P.p[3];
    }
    return nan("");
}

// tab != nullptr: per-instance parameters of a brick batch
__global__ void k_ls_vertices(MeshView M, LsPar P, const LsPar* __restrict__ tab, double* __restrict__ lsv) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < M.nv; v += (int64_t)gridDim.x * blockDim.x) {
        double x[3];
        mesh_coord(M, (int32_t)v, x);
        lsv[v] = ls_value(tab ? tab[batch_find(M.vstart, M.nbatch, v)] : P, x);
    }
}

__global__ void k_ls_edges(MeshView M, LsPar P, const LsPar* __restrict__ tab, int p2, const double* __restrict__ lsv,
                           double* __restrict__ lse) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < M.ne; e += (int64_t)gridDim.x * blockDim.x) {
        int32_t a, b;
        mesh_edge(M, e, a, b);
        if (!p2) {
            lse[e] = 0.5 * (lsv[a] + lsv[b]);
        } else {
            double xa[3], xb[3], m[3];
            mesh_coord(M, a, xa);
            mesh_coord(M, b, xb);
            for (int k = 0; k < 3; ++k) m[k] = 0.5 * (xa[k] + xb[k]);
            lse[e] = ls_value(tab ? tab[batch_find(M.estart, M.nbatch, e)] : P, m);
        }
    }
}

static int ls_need(int kind) {
    return kind == TF_LS_SPHERE ? 4 : kind == TF_LS_TORUS ? 3 : kind == TF_LS_ELLIPSOID ? 15 : kind == TF_LS_PLANE ? 4 : -1;
}

// count == 0: one parameter set for the whole mesh; count == number of batch
// instances: par holds count consecutive sets of npar values.
int levelset_analytic(Context* c, int kind, const double* par, int npar, int p2, int count) {
    if (!c->has_mesh) return set_err(c, TF_ERR_BAD_INPUT, "levelset: no mesh");
    const int need = ls_need(kind);
    if (need < 0 || !par || npar < need) return set_err(c, TF_ERR_BAD_INPUT, "levelset: bad kind or parameters");
    if (count != 0 && count != c->batch_count)
        return set_err(c, TF_ERR_BAD_INPUT, "levelset: one parameter set per batch instance required");
    LsPar P{};
    P.kind = kind;
    for (int i = 0; i < need && i < 16; ++i) P.p[i] = par[i];
    const LsPar* tab = nullptr;
    if (count > 0) {
        std::vector<LsPar> h((size_t)count);
        for (int j = 0; j < count; ++j) {
            h[j] = LsPar{};
            h[j].kind = kind;
            for (int i = 0; i < need; ++i) h[j].p[i] = par[(size_t)j * npar + i];
        }
        TF_TRY(ensure(c, c->batch_ls, sizeof(LsPar) * count));
        TF_CUDA(c, cudaMemcpyAsync(c->batch_ls.p, h.data(), sizeof(LsPar) * count, cudaMemcpyHostToDevice, c->stream));
        TF_CUDA(c, cudaStreamSynchronize(c->stream));
        tab = (const LsPar*)c->batch_ls.p;
    }
    TF_TRY(ensure(c, c->ls_vert, (size_t)c->mesh.nv));
    TF_TRY(ensure(c, c->ls_edge, (size_t)c->mesh.ne));
    {
        TimedLaunch tl(c, TF_K_LEVELSET);
        k_ls_vertices<<<grid_for(c, c->mesh.nv), kBlock, 0, c->stream>>>(c->mesh, P, tab, c->ls_vert.p);
        k_ls_edges<<<grid_for(c, c->mesh.ne), kBlock, 0, c->stream>>>(c->mesh, P, tab, p2, c->ls_vert.p, c->ls_edge.p);
        c->launches += 2;
    }
    TF_CUDA(c, cudaGetLastError());
    c->has_ls = true;
    ++c->ls_version;
    c->fe = 0;
    return TF_OK;
}

int levelset_p1_edges(Context* c) {
    LsPar P{};
    P.kind = -1;
    k_ls_edges<<<grid_for(c, c->mesh.ne), kBlock, 0, c->stream>>>(c->mesh, P, nullptr, 0, c->ls_vert.p, c->ls_edge.p);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    return TF_OK;
}

__global__ void k_mesh_materialise(MeshView M, double* coords, int32_t* tet_v, int32_t* tet_e, int32_t* edge_v) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (coords)
        for (int64_t v = i0; v < M.nv; v += stride) {
            double x[3];
            mesh_coord(M, (int32_t)v, x);
            coords[3 * v] = x[0];
            coords[3 * v + 1] = x[1];
            coords[3 * v + 2] = x[2];
        }
    if (tet_v || tet_e)
        for (int64_t t = i0; t < M.nt; t += stride) {
            int32_t v[4], e[6];
            mesh_tet(M, t, v, e);
            if (tet_v)
                for (int k = 0; k < 4; ++k) tet_v[4 * t + k] = v[k];
            if (tet_e)
                for (int k = 0; k < 6; ++k) tet_e[6 * t + k] = e[k];
        }
    if (edge_v)
        for (int64_t e = i0; e < M.ne; e += stride) {
            int32_t a, b;
            mesh_edge(M, e, a, b);
            edge_v[2 * e] = a;
            edge_v[2 * e + 1] = b;
        }
}

int mesh_materialise(Context* c, double* coords, int32_t* tet_v, int32_t* tet_e, int32_t* edge_v) {
    k_mesh_materialise<<<grid_for(c, c->mesh.nt), kBlock, 0, c->stream>>>(c->mesh, coords, tet_v, tet_e, edge_v);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    return TF_OK;
}

}  // namespace tf
