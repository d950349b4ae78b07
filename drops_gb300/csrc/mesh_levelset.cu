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

int mesh_set_brick(Context* c, const double orig[3], const double e1[3], const double e2[3], const double e3[3],
                   int n1, int n2, int n3) {
    if (n1 < 1 || n2 < 1 || n3 < 1) return set_err(c, TF_ERR_BAD_INPUT, "brick: n1, n2, n3 must be >= 1");
    MeshView& M = c->mesh;
    M = MeshView{};
    M.explicit_mesh = 0;
    M.n1 = n1; M.n2 = n2; M.n3 = n3;
    for (int k = 0; k < 3; ++k) {
        M.orig[k] = orig[k];
        M.o1[k] = (1.0 / (double)n1) * e1[k];
        M.o2[k] = (1.0 / (double)n2) * e2[k];
        M.o3[k] = (1.0 / (double)n3) * e3[k];
    }
    static const int dir[7][3] = {{0, 0, 1}, {0, 1, 0}, {1, 0, 0}, {0, 1, 1}, {1, 0, 1}, {1, 1, 0}, {1, 1, 1}};
    M.eoff[0] = 0;
    for (int t = 0; t < 7; ++t)
        M.eoff[t + 1] = M.eoff[t] + (int64_t)(n3 + 1 - dir[t][0]) * (n2 + 1 - dir[t][1]) * (n1 + 1 - dir[t][2]);
    M.nv = (int64_t)(n1 + 1) * (n2 + 1) * (n3 + 1);
    M.ne = M.eoff[7];
    M.nt = (int64_t)6 * n1 * n2 * n3;
    if (M.nv > INT32_MAX || M.ne > INT32_MAX || M.nt > ((int64_t)1 << 40))
        return set_err(c, TF_ERR_CAPACITY, "brick too large for 32-bit vertex/edge ids");
    c->has_mesh = true;
    c->has_ls = false;
    c->fe = 0;
    return TF_OK;
}

// endpoints of edge e
__device__ inline void mesh_edge(const MeshView& M, int64_t e, int32_t& a, int32_t& b) {
    if (M.explicit_mesh) {
        a = M.edge_v[2 * e];
        b = M.edge_v[2 * e + 1];
        return;
    }
    int cls = 0;
    while (cls < 6 && e >= M.eoff[cls + 1]) ++cls;
    const int d3 = (cls == 2 || cls == 4 || cls == 5 || cls == 6) ? 1 : 0;
    const int d2 = (cls == 1 || cls == 3 || cls == 5 || cls == 6) ? 1 : 0;
    const int d1 = (cls == 0 || cls == 3 || cls == 4 || cls == 6) ? 1 : 0;
    int64_t k = e - M.eoff[cls];
    const int w1 = M.n1 + 1 - d1, w2 = M.n2 + 1 - d2;
    const int i1 = (int)(k % w1);
    k /= w1;
    const int i2 = (int)(k % w2);
    const int i3 = (int)(k / w2);
    a = (int32_t)(((int64_t)i3 * (M.n2 + 1) + i2) * (M.n1 + 1) + i1);
    b = (int32_t)(((int64_t)(i3 + d3) * (M.n2 + 1) + i2 + d2) * (M.n1 + 1) + i1 + d1);
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

__global__ void k_ls_vertices(MeshView M, LsPar P, double* __restrict__ lsv) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < M.nv; v += (int64_t)gridDim.x * blockDim.x) {
        double x[3];
        mesh_coord(M, (int32_t)v, x);
        lsv[v] = ls_value(P, x);
    }
}

__global__ void k_ls_edges(MeshView M, LsPar P, int p2, const double* __restrict__ lsv, double* __restrict__ lse) {
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
            lse[e] = ls_value(P, m);
        }
    }
}

int levelset_analytic(Context* c, int kind, const double* par, int npar, int p2) {
    if (!c->has_mesh) return set_err(c, TF_ERR_BAD_INPUT, "levelset: no mesh");
    const int need = kind == TF_LS_SPHERE ? 4 : kind == TF_LS_TORUS ? 3 : kind == TF_LS_ELLIPSOID ? 15 : kind == TF_LS_PLANE ? 4 : -1;
    if (need < 0 || !par || npar < need) return set_err(c, TF_ERR_BAD_INPUT, "levelset: bad kind or parameters");
    LsPar P{};
    P.kind = kind;
    for (int i = 0; i < need && i < 16; ++i) P.p[i] = par[i];
    TF_TRY(ensure(c, c->ls_vert, (size_t)c->mesh.nv));
    TF_TRY(ensure(c, c->ls_edge, (size_t)c->mesh.ne));
    {
        TimedLaunch tl(c, TF_K_LEVELSET);
        k_ls_vertices<<<grid_for(c, c->mesh.nv), kBlock, 0, c->stream>>>(c->mesh, P, c->ls_vert.p);
        k_ls_edges<<<grid_for(c, c->mesh.ne), kBlock, 0, c->stream>>>(c->mesh, P, p2, c->ls_vert.p, c->ls_edge.p);
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
    k_ls_edges<<<grid_for(c, c->mesh.ne), kBlock, 0, c->stream>>>(c->mesh, P, 0, c->ls_vert.p, c->ls_edge.p);
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
